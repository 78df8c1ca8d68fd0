"""Serving: continuous batching of reactor-scenario requests on one GPU.

Requests arrive over time (each: a scenario and a number of steps).  The
server admits them in arrival order while their device memory fits the HBM
budget and a batch slot is free, keeps every admitted scenario's particle
and liquid state resident on the device, and advances all admitted
scenarios together, chunk after chunk, with one batched launch sequence per
step (libbmc's slot batch: built once, its captured step replayed, empty
slots skipped on the device).  A scenario carries a step limit, so it stops
exactly at its requested step count inside a chunk; finished scenarios give
their slot and memory back between chunks.  While a chunk runs on the GPU
the host admits new requests (their initialisation uses their own streams)
and they take their slots as soon as the chunk ends, so admission overlaps
device work.

Latency of a request = completion time - arrival time.  Particle-steps
are counted from live particles: for every completed request, its step
count times the mean of its live particles at admission and at completion
(births between the two are counted half).
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import scenarios
from .sim import GpuBatch, GpuScenario


def scenario_bytes(scen) -> int:
    """Device memory a scenario takes (libbmc's arenas, to within a few KiB)."""
    cap = (scen.capacity + 1023) // 1024 * 1024
    fsz = scen.model.itemsize
    nv = scen.model.n_var
    per_slot = 2 * nv * fsz + 4 + 1 + 4 + 4 + 4 + 4 + 4 + 4 + 4
    n_c, K, ns = scen.net.n_c, scen.net.K, scen.n_species
    n_acc = 1 if scen.model.separable else scen.model.n_ctb
    domain = n_c * (8 * K + 5 * 8 + 64 + 8 * ns * 4 + 16 * n_acc) + len(scen.net.flow) * 12 + (n_c + 1) * 4
    return cap * per_slot + cap // 32 * 4 + 5 * (cap // 1024) * 4 + domain + 64 * 1024


@dataclass
class Request:
    rid: int
    arrival: float  # s, relative to the start of the run
    scen: object
    steps: int
    admitted: float | None = None
    finished: float | None = None
    result: dict = field(default_factory=dict)

    @property
    def latency(self) -> float | None:
        return None if self.finished is None else self.finished - self.arrival

    @property
    def particle_steps(self) -> float:
        return float(self.scen.n_particles) * self.steps


def poisson_requests(rate: float, duration: float, seed: int = 5, steps_lo: int = 100,
                     steps_hi: int = 10000, particle_scale: float = 1.0) -> list[Request]:
    """Poisson arrivals at `rate` per second over `duration` seconds; sizes as
    the batched workload, step counts log-uniform on [steps_lo, steps_hi]."""
    rng = np.random.default_rng(seed)
    t, reqs, k = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        sc = scenarios.batch_scenario(k, seed=seed, steps_lo=steps_lo, steps_hi=steps_hi,
                                      particle_scale=particle_scale)
        reqs.append(Request(k, t, sc, sc.n_steps))
        k += 1
    return reqs


class Server:
    """Continuous batching over a fixed-slot batch (libbmc's
    bmc_batch_create_slots): an admitted scenario takes a free slot, a
    finished one gives it back; the batch and its captured step are built
    once, empty slots cost nothing on the device."""

    def __init__(self, hbm_budget: float = 160e9, chunk_steps: int = 32, dt: float = 0.1,
                 shape: tuple | None = None, max_chunk_ms: float = 60.0, slots: int = 512):
        self.budget = hbm_budget
        self.chunk_steps = chunk_steps
        self.dt = dt
        self.shape = shape
        self.max_chunk_ms = max_chunk_ms
        self.n_slots = slots
        self.used = 0
        self.log = []

    def serve(self, requests: list[Request], clock=time.perf_counter, sleep=time.sleep,
              max_wall: float | None = None, on_finish=None) -> dict:
        """Serve `requests` until all are done (or `max_wall` seconds have
        passed); `on_finish(request, gpu_scenario)` runs before a finished
        scenario is released."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        t0 = clock()
        i = 0
        pending: deque = deque()
        active: list = []  # [request, GpuScenario, bytes, steps done, slot]
        joining: list = []  # admitted while a chunk ran: slot set after it
        free = list(range(self.n_slots - 1, -1, -1))
        batch = None
        step_ms = 1.0
        busy = 0.0
        steps_done = 0.0
        running = False

        def admit():
            nonlocal batch
            while pending and free:
                r = pending[0]
                need = scenario_bytes(r.scen)
                if self.used + need > self.budget:
                    if not active and not joining and not running:
                        raise RuntimeError(f"request {r.rid} needs {need} B, more than the HBM budget")
                    break
                pending.popleft()
                g = GpuScenario(r.scen)
                g.set_step_limit(r.steps)
                r.admitted = clock() - t0
                if batch is None:
                    batch = GpuBatch.slots(self.n_slots, r.scen.model)
                    if self.shape:
                        batch.set_shape(*self.shape)
                joining.append([r, g, need, 0, free.pop()])
                self.used += need

        while True:
            now = clock() - t0
            if max_wall is not None and now > max_wall:
                break
            while i < len(reqs) and reqs[i].arrival <= now:
                pending.append(reqs[i])
                i += 1
            admit()
            for a in joining:  # the batch is idle here: slots can change
                batch.set_slot(a[4], a[1])
                active.append(a)
            joining.clear()
            if not active:
                if i >= len(reqs) and not pending:
                    break
                nxt = reqs[i].arrival if i < len(reqs) else now
                sleep(max(0.0, min(0.01, nxt - now)))
                continue
            # chunk length: bounded wall time per chunk so arrivals are admitted promptly
            members = list(active)
            remaining = [a[0].steps - a[3] for a in members]
            chunk = max(1, min(self.chunk_steps, max(remaining), int(self.max_chunk_ms / max(step_ms, 1e-3))))
            tc = clock()
            batch.run(chunk, self.dt)
            running = True
            # admission overlaps the chunk on the GPU (new scenarios take
            # their slots once it is done)
            now = clock() - t0
            while i < len(reqs) and reqs[i].arrival <= now:
                pending.append(reqs[i])
                i += 1
            admit()
            batch.synchronize()
            running = False
            el = clock() - tc
            busy += el
            step_ms = 1e3 * el / chunk
            done_at = clock() - t0
            retired = set()
            for a in members:
                r, g, need, st, slot = a
                adv = min(chunk, r.steps - st)
                a[3] = st + adv
                if a[3] >= r.steps:
                    r.finished = done_at
                    r.result = g.stats()
                    alive_end = r.result["n_used"] - r.result["inactive"]
                    steps_done += 0.5 * (float(r.scen.n_particles) + float(alive_end)) * r.steps
                    if on_finish is not None:
                        on_finish(r, g)
                    batch.set_slot(slot, None)
                    g.close()
                    self.used -= need
                    free.append(slot)
                    retired.add(id(a))
            active = [a for a in active if id(a) not in retired]
        wall = clock() - t0
        for a in active + joining:
            if batch is not None:
                batch.set_slot(a[4], None)
            a[1].close()
        if batch is not None:
            batch.close()
        done = [r for r in reqs if r.finished is not None]
        lat = np.array([r.latency for r in done]) if done else np.array([np.nan])
        return {
            "requests": len(reqs), "completed": len(done), "wall_s": wall, "gpu_busy_s": busy,
            "utilisation": busy / wall if wall > 0 else 0.0,
            "particle_steps": steps_done, "particle_steps_per_s": steps_done / wall if wall > 0 else 0.0,
            "latency_p50_s": float(np.nanpercentile(lat, 50)), "latency_p99_s": float(np.nanpercentile(lat, 99)),
            "latency_mean_s": float(np.nanmean(lat)), "slots": self.n_slots,
        }
