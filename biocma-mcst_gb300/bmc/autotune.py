"""Launch-shape autotuner for the cycle kernel.

The cycle kernel has five instantiated shapes per model (256 threads with
1, 2 or 4 particles per thread, 512 x 2 and 1024 x 1, each compiled for
its own register budget) and a free choice of resident blocks per SM.  The autotuner times each candidate
on the live scenario (or batch) for a few steps -- every timed step is a
real step of the simulation, so tuning doubles as warm-up -- and keeps the
fastest.  Results are remembered per workload key (compartment-count
bucket, particle-count bucket, n_var, precision, batch size) for the life
of the process.
"""
from __future__ import annotations

import math
import time

# (threads per block, particles per thread, resident blocks per SM; 0 = max)
CANDIDATES = [(256, 1, 0), (256, 2, 0), (256, 4, 0), (512, 2, 0), (1024, 1, 0)]

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
        g.set_shape(*shape)
        g.run(1)  # graph capture for this shape
        _, ms = g.run_timed(steps)
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
        b.set_shape(*shape)
        b.run(1, dt)
        b.synchronize()
        t0 = time.perf_counter()
        b.run(steps, dt)
        b.synchronize()
        timings[shape] = (time.perf_counter() - t0) * 1e3 / steps
    best = min(timings, key=timings.get)
    b.set_shape(*best)
    _cache[key] = best
    return best, timings
