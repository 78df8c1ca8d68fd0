"""Free-running statistics of a scenario and a two-sample band test.

The GPU path draws from Philox4x32-10; the reference draws from a Kokkos
XorShift1024 pool.  Their free-running results cannot agree bit for bit, so
they are compared as distributions: each side runs the same scenario under
32 seeds, and every summary statistic (per-compartment occupancy, per-
compartment mean particle mass, live count, cumulative births, the liquid
concentration per compartment) must agree within a 99 % family-wise band
(Welch two-sample t interval, Bonferroni over the statistics compared).
"""
from __future__ import annotations

import dataclasses

import numpy as np
from scipy import stats as sst

N_SEEDS = 32


def summary(parts: dict, C: np.ndarray, n_c: int, n_init: int, next_id: int) -> np.ndarray:
    """Vector of statistics of one finished run."""
    live = parts["status"] == 0
    pos = parts["pos"][live].astype(np.int64)
    mass = np.asarray(parts["state"][0][live], dtype=np.float64)
    counts = np.bincount(pos, minlength=n_c).astype(np.float64)
    n_live = counts.sum()
    occupancy = counts / max(n_live, 1.0)
    mass_sum = np.bincount(pos, weights=mass, minlength=n_c)
    mean_mass = np.divide(mass_sum, counts, out=np.zeros(n_c), where=counts > 0)
    births = float(next_id - n_init)
    return np.concatenate([occupancy, mean_mass, [n_live, births], C[:, 0]])


def seeded(scen, seed: int):
    return dataclasses.replace(scen, seed=seed)


def band_test(a: np.ndarray, b: np.ndarray, alpha: float = 0.01):
    """a, b: [n_seeds, n_stats].  Returns (ok, worst ratio |diff|/halfwidth,
    index of the worst statistic)."""
    na, nb = a.shape[0], b.shape[0]
    ma, mb = a.mean(0), b.mean(0)
    va, vb = a.var(0, ddof=1), b.var(0, ddof=1)
    se = np.sqrt(va / na + vb / nb)
    # Welch-Satterthwaite degrees of freedom
    num = (va / na + vb / nb) ** 2
    den = (va / na) ** 2 / (na - 1) + (vb / nb) ** 2 / (nb - 1)
    dof = np.divide(num, den, out=np.full_like(num, na + nb - 2.0), where=den > 0)
    m = a.shape[1]
    t = sst.t.ppf(1.0 - alpha / (2.0 * m), dof)
    half = t * se
    diff = np.abs(ma - mb)
    scale = np.maximum(np.abs(ma), np.abs(mb))
    # statistics with no spread on either side must agree to rounding
    half = np.where(se > 0, half, 1e-12 * scale)
    ratio = np.divide(diff, half, out=np.zeros_like(diff), where=half > 0)
    ratio = np.where((half == 0) & (diff > 0), np.inf, ratio)
    worst = int(np.argmax(ratio))
    return bool(np.all(ratio <= 1.0)), float(ratio[worst]), worst
