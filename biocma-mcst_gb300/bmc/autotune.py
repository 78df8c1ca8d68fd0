"""Launch-shape autotuner for the cycle kernel.

The cycle kernel has seven instantiated shapes per model: five that stream
particles through registers (256 threads with 1, 2 or 4 particles per
thread, 512 x 2 and 1024 x 1, each compiled for its own register budget)
and two that stage 1024-slot tiles in shared memory through the copy
engine (256 or 512 consumer threads plus a producer warp), with a free
choice of resident blocks per SM.  The autotuner times each candidate
on the live scenario (or batch) for a few steps -- every timed step is a
real step of the simulation, so tuning doubles as warm-up -- and keeps the
fastest.  Results are remembered per workload key (compartment-count
bucket, particle-count bucket, n_var, precision, batch size) for the life
of the process.
"""
from __future__ import annotations

import math
import time

from ._lib import BmcError

# (threads, particles per thread, blocks per SM; 0 = as many as fit).  288 and
# 544 threads are the tile-staging kernel (256 / 512 consumers + 1 producer warp).
CANDIDATES = [(256, 1, 0), (256, 2, 0), (256, 4, 0), (512, 2, 0), (1024, 1, 0), (288, 4, 0), (544, 2, 0)]

_cache: dict = {}


def _bucket(x: float) -> int:
    return int(math.log2(max(x, 1)))


def workload_key(n_c: int, n_particles: int, n_var: int, f64: bool, n_scen: int = 1):
    return (_bucket(n_c), _bucket(n_particles), n_var, bool(f64), _bucket(n_scen))


def tune_scenario(g, steps: int = 4, candidates=CANDIDATES):
    """Pick the fastest shape for a GpuScenario; returns (shape, timings)."""
    key = workload_key(g.scen.net.n_c, g.scen.n_particles, g.scen.model.n_var, g.scen.model.f64)
    if key in _cache:
        g.set_shape(*_cache[key])
        return _cache[key], {}
    timings = {}
    for shape in candidates:
        try:
            g.set_shape(*shape)
            g.run(1)  # graph capture for this shape
            _, ms = g.run_timed(steps)
        except BmcError:  # shape does not fit this scenario (shared memory)
            continue
        timings[shape] = ms / steps
    best = min(timings, key=timings.get)
    g.set_shape(*best)
    _cache[key] = best
    return best, timings


def tune_batch(b, dt: float, steps: int = 3, candidates=CANDIDATES):
    """Pick the fastest shape for a GpuBatch (host wall time around
    synchronised runs of `steps` steps)."""
    members = b.members
    n_c = max(m.scen.net.n_c for m in members)
    n_p = sum(m.scen.n_particles for m in members)
    m0 = members[0].scen.model
    key = workload_key(n_c, n_p, m0.n_var, m0.f64, len(members))
    if key in _cache:
        b.set_shape(*_cache[key])
        return _cache[key], {}
    timings = {}
    for shape in candidates:
        try:
            b.set_shape(*shape)
            b.run(1, dt)
            b.synchronize()
            t0 = time.perf_counter()
            b.run(steps, dt)
            b.synchronize()
        except BmcError:  # shape does not fit these scenarios (shared memory)
            continue
        timings[shape] = (time.perf_counter() - t0) * 1e3 / steps
    best = min(timings, key=timings.get)
    b.set_shape(*best)
    _cache[key] = best
    return best, timings
