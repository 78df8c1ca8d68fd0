"""Synthetic compartment networks (the CMA flow maps the hot path consumes).

The reference reads flow maps from CFD through rcmtool (external Rust crate,
pinned ``v1.4`` in subprojects/rcmtool.wrap) and derives, per compartment,
the neighbour table, the total outgoing flow (``diag_transition``), the
cumulative probability of each destination given a departure, and the
transition matrix (documentation/pages/03_cma.md, "Transition Matrix" and
"Cumulative probability").  Those derivations are restated here from the
published method:

* ``T[i, j] = F(i -> j)`` off the diagonal and ``T[j, j] = -sum_k F(j -> k)``;
* ``P(I_j | L) = F(i, j) / sum_k F(i, k)``, accumulated in neighbour order.

Two seeded generators supply the flows:

* :func:`ring_network` -- a ring with extra random exchange links;
* :func:`lattice_vortex` -- a cubic lattice whose face flows are the discrete
  curl of an azimuthal vector potential (a toroidal recirculation cell), so
  every compartment's inflow equals its outflow to rounding.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Network:
    n_c: int
    volume: np.ndarray  # float64 [n_c], m^3
    src: np.ndarray  # int64 [n_links] flow origin
    dst: np.ndarray  # int64 [n_links] flow destination
    flow: np.ndarray  # float64 [n_links], m^3/s, > 0
    meta: dict = field(default_factory=dict)

    # derived (filled by finalize)
    out_flow: np.ndarray | None = None
    K: int = 1
    neighbors: np.ndarray | None = None  # uint32 [n_c, K]
    cdf: np.ndarray | None = None  # float64 [n_c, K]
    in_ptr: np.ndarray | None = None  # uint32 [n_c+1]
    in_idx: np.ndarray | None = None  # uint32 [nnz]
    in_flow: np.ndarray | None = None  # float64 [nnz]

    @property
    def total_volume(self) -> float:
        return float(self.volume.sum())

    def finalize(self) -> "Network":
        n = self.n_c
        order = np.lexsort((self.dst, self.src))
        src, dst, flow = self.src[order], self.dst[order], self.flow[order]
        out_flow = np.zeros(n, dtype=np.float64)
        np.add.at(out_flow, src, flow)
        counts = np.bincount(src, minlength=n)
        K = max(1, int(counts.max()) if len(counts) else 1)
        neighbors = np.zeros((n, K), dtype=np.uint32)
        cdf = np.ones((n, K), dtype=np.float64)
        start = 0
        for i in range(n):
            c = int(counts[i])
            if c == 0:
                neighbors[i, :] = i
                continue
            d = dst[start:start + c]
            f = flow[start:start + c]
            run = np.cumsum(f)  # sequential: its last value is the out-flow
            acc = run / run[-1]
            neighbors[i, :c] = d
            neighbors[i, c:] = d[-1]
            cdf[i, :c] = acc
            cdf[i, c:] = 1.0
            start += c
        # incoming CSR by destination column (transition matrix columns)
        order_in = np.lexsort((src, dst))
        isrc, idst, iflow = src[order_in], dst[order_in], flow[order_in]
        in_counts = np.bincount(idst, minlength=n)
        in_ptr = np.zeros(n + 1, dtype=np.uint32)
        in_ptr[1:] = np.cumsum(in_counts)
        self.out_flow = out_flow
        self.K = K
        self.neighbors = np.ascontiguousarray(neighbors)
        self.cdf = np.ascontiguousarray(cdf)
        self.in_ptr = in_ptr
        self.in_idx = isrc.astype(np.uint32)
        self.in_flow = iflow.astype(np.float64)
        return self

    def divergence(self) -> np.ndarray:
        """Inflow minus outflow per compartment (zero for a closed, balanced map)."""
        d = np.zeros(self.n_c)
        np.add.at(d, self.dst, self.flow)
        np.subtract.at(d, self.src, self.flow)
        return d

    def max_courant(self, dt: float) -> float:
        """max_i dt * Q_out(i) / V(i): the move probability bound and the
        explicit-Euler stability number of the liquid step."""
        return float(np.max(dt * self.out_flow / self.volume))

    def transition_dense(self) -> np.ndarray:
        T = np.zeros((self.n_c, self.n_c))
        np.add.at(T, (self.src, self.dst), self.flow)
        T[np.arange(self.n_c), np.arange(self.n_c)] -= self.out_flow
        return T


def _lognormal(rng: np.random.Generator, median: float, sigma: float, size):
    return median * np.exp(sigma * rng.standard_normal(size))


def ring_network(n_c: int = 10, extra_links: int = 2, median_flow: float = 1e-3,
                 sigma: float = 0.5, v_lo: float = 0.5e-3, v_hi: float = 2e-3,
                 seed: int = 42, max_courant: float | None = None,
                 dt: float | None = None) -> Network:
    """Ring of ``n_c`` compartments plus ``extra_links`` random outgoing
    exchange links per compartment.

    The ring carries one lognormal circulation; each random link i->j carries
    a lognormal flow and is balanced by the same flow j->i, so inflow equals
    outflow everywhere and a uniform field is a steady state of the liquid
    step.  With ``max_courant`` and ``dt`` given, all flows are scaled down
    (never up) so that ``dt * Q_out / V <= max_courant``.
    """
    rng = np.random.default_rng(seed)
    volume = rng.uniform(v_lo, v_hi, size=n_c)
    links: dict[tuple[int, int], float] = {}

    def add(a, b, f):
        links[(a, b)] = links.get((a, b), 0.0) + f

    if n_c > 1:
        q_ring = float(_lognormal(rng, median_flow, sigma, 1)[0])
        for i in range(n_c):
            add(i, (i + 1) % n_c, q_ring)
        for i in range(n_c):
            choices = [j for j in range(n_c) if j != i]
            k = min(extra_links, len(choices))
            targets = rng.choice(choices, size=k, replace=False)
            for j in targets:
                f = float(_lognormal(rng, median_flow, sigma, 1)[0])
                add(i, int(j), f)
                add(int(j), i, f)
    src = np.array([a for a, _ in links], dtype=np.int64)
    dst = np.array([b for _, b in links], dtype=np.int64)
    flow = np.array([links[k] for k in links], dtype=np.float64)
    net = Network(n_c, volume, src, dst, flow,
                  meta={"kind": "ring", "seed": seed, "extra_links": extra_links,
                        "median_flow": median_flow, "sigma": sigma, "flow_scale": 1.0})
    net.finalize()
    if max_courant is not None and dt is not None and n_c > 1:
        cmax = net.max_courant(dt)
        if cmax > max_courant:
            scale = max_courant / cmax
            net.flow = net.flow * scale
            net.meta["flow_scale"] = scale
            net.finalize()
    return net


def lattice_vortex(n: int = 8, side: float = 1.0, peak_velocity: float = 0.5,
                   noise: float = 0.1, seed: int = 1, max_courant: float | None = None,
                   dt: float | None = None) -> Network:
    """``n^3`` cubic lattice in a cube of edge ``side`` (m) with a toroidal
    recirculation: face flows are the discrete curl (Stokes circulation) of
    the vector potential ``A = psi(r, z) e_theta``,
    ``psi = sin(pi r / R) sin(pi z / H)`` for ``r < R`` (R = side/2, H = side),
    scaled so the fastest face velocity equals ``peak_velocity``.  The noise
    multiplies each edge value of A by ``exp(noise * N(0,1))`` (lognormal),
    which keeps every compartment exactly balanced.  Compartment index is
    ``i + n*j + n*n*k`` for cell (i, j, k) with k vertical."""
    rng = np.random.default_rng(seed)
    h = side / n
    R = side / 2.0
    H = side
    xc = yc = side / 2.0

    def psi(x, y, z):
        r = np.sqrt((x - xc) ** 2 + (y - yc) ** 2)
        val = np.where(r < R, np.sin(np.pi * r / R) * np.sin(np.pi * z / H), 0.0)
        return val, r

    def ax_ay(x, y, z):
        p, r = psi(x, y, z)
        rs = np.where(r > 0, r, 1.0)
        return -p * (y - yc) / rs, p * (x - xc) / rs

    g = np.arange(n + 1) * h  # node coordinates
    m = np.arange(n) * h + h / 2  # edge midpoints
    # A_x on x-edges: midpoint x, node y, node z -> shape (n, n+1, n+1)
    X, Y, Z = np.meshgrid(m, g, g, indexing="ij")
    Ax, _ = ax_ay(X, Y, Z)
    # A_y on y-edges: node x, midpoint y, node z -> shape (n+1, n, n+1)
    X, Y, Z = np.meshgrid(g, m, g, indexing="ij")
    _, Ay = ax_ay(X, Y, Z)
    Ax = Ax * np.exp(noise * rng.standard_normal(Ax.shape))
    Ay = Ay * np.exp(noise * rng.standard_normal(Ay.shape))
    Ax *= h
    Ay *= h
    # face fluxes (positive along +axis), from the circulation of A (A_z = 0)
    # x-faces at node x index a (0..n), cell span j,k: flux = Ay(a, j, k) - Ay(a, j, k+1)
    fx = Ay[:, :, :-1] - Ay[:, :, 1:]  # (n+1, n, n)
    # y-faces at node y index b: flux = Ax(i, b, k+1) - Ax(i, b, k)
    fy = Ax[:, :, 1:] - Ax[:, :, :-1]  # (n, n+1, n)
    # z-faces at node z index c: flux = Ax(i, j, c) - Ax(i, j+1, c) + Ay(i+1, j, c) - Ay(i, j, c)
    fz = (Ax[:, :-1, :] - Ax[:, 1:, :]) + (Ay[1:, :, :] - Ay[:-1, :, :])  # (n, n, n+1)
    # walls carry no flux (psi = 0 on every boundary edge); drop them
    fx, fy, fz = fx[1:-1], fy[:, 1:-1], fz[:, :, 1:-1]
    vmax = max(np.abs(fx).max(initial=0.0), np.abs(fy).max(initial=0.0), np.abs(fz).max(initial=0.0)) / (h * h)
    scale = peak_velocity / vmax if vmax > 0 else 0.0  # n <= 2: no interior recirculation
    fx, fy, fz = fx * scale, fy * scale, fz * scale

    def cid(i, j, k):
        return i + n * j + n * n * k

    src, dst, flow = [], [], []
    I, J, Kk = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    for axis, f in ((0, fx), (1, fy), (2, fz)):
        if axis == 0:
            a = cid(I[:-1], J[:-1], Kk[:-1]); b = cid(I[1:], J[1:], Kk[1:])
        elif axis == 1:
            a = cid(I[:, :-1], J[:, :-1], Kk[:, :-1]); b = cid(I[:, 1:], J[:, 1:], Kk[:, 1:])
        else:
            a = cid(I[:, :, :-1], J[:, :, :-1], Kk[:, :, :-1]); b = cid(I[:, :, 1:], J[:, :, 1:], Kk[:, :, 1:])
        a, b, f = a.ravel(), b.ravel(), f.ravel()
        pos = f > 0
        neg = f < 0
        src.append(a[pos]); dst.append(b[pos]); flow.append(f[pos])
        src.append(b[neg]); dst.append(a[neg]); flow.append(-f[neg])
    src = np.concatenate(src).astype(np.int64)
    dst = np.concatenate(dst).astype(np.int64)
    flow = np.concatenate(flow).astype(np.float64)
    volume = np.full(n ** 3, h ** 3)
    net = Network(n ** 3, volume, src, dst, flow,
                  meta={"kind": "lattice_vortex", "n": n, "side": side, "seed": seed,
                        "peak_velocity": peak_velocity, "noise": noise, "flow_scale": 1.0})
    net.finalize()
    if max_courant is not None and dt is not None and len(net.flow):
        cmax = net.max_courant(dt)
        if cmax > max_courant:
            net.flow = net.flow * (max_courant / cmax)
            net.meta["flow_scale"] = max_courant / cmax
            net.finalize()
    return net


def single_compartment(volume: float = 1e-3) -> Network:
    """0-D reactor: one compartment, no internal flows (move disabled)."""
    net = Network(1, np.array([volume]), np.zeros(0, np.int64), np.zeros(0, np.int64),
                  np.zeros(0), meta={"kind": "0d"})
    return net.finalize()
