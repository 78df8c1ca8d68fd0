"""Serving loop logic on the CPU: admission by HBM budget, continuous batching,
exact step counts, retirement, latency bookkeeping.  The device scenario and
batch are replaced by fakes that record what the server asks of them; the
GPU tests (test_gpu_serve.py) check the results themselves.
"""
import pytest

from bmc import serve


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-4)


class World:
    """Shared state of the fakes: live scenarios, batches, a clock."""

    def __init__(self, clock, step_cost=1e-3):
        self.clock = clock
        self.step_cost = step_cost
        self.live = set()
        self.max_live_bytes = 0
        self.batches = []


def make_fakes(world, budget_probe):
    class FakeScenario:
        def __init__(self, scen):
            self.scen = scen
            self.limit = None
            self.steps = 0
            world.live.add(self)
            budget_probe()

        def set_step_limit(self, n):
            self.limit = n

        def stats(self):
            # one birth per step, nothing removed
            return {"step": self.steps, "n_used": self.scen.n_particles + self.steps, "inactive": 0}

        def close(self):
            world.live.discard(self)

    class FakeBatch:
        def __init__(self, capacity):
            self.members = [None] * capacity

        @classmethod
        def slots(cls, capacity, model):
            return cls(capacity)

        def set_slot(self, slot, g):
            assert (g is None) != (self.members[slot] is None)  # fill an empty slot or empty a full one
            self.members[slot] = g

        def set_shape(self, *a):
            pass

        def run(self, n, dt):
            live = [m for m in self.members if m is not None]
            world.batches.append(len(live))
            for m in live:
                m.steps = min(m.limit, m.steps + n)
            world.clock.t += n * world.step_cost

        def synchronize(self):
            pass

        def close(self):
            assert all(m is None for m in self.members)

    return FakeScenario, FakeBatch


def requests(n, steps):
    from bmc import scenarios

    out = []
    for k in range(n):
        sc = scenarios.batch_scenario(k, seed=3, particle_scale=0.01, steps_lo=steps[0], steps_hi=steps[1])
        out.append(serve.Request(k, 0.02 * k, sc, sc.n_steps))
    return out


def test_every_request_runs_exactly_its_steps(monkeypatch):
    clock = FakeClock()
    world = World(clock)
    FS, FB = make_fakes(world, lambda: None)
    monkeypatch.setattr(serve, "GpuScenario", FS)
    monkeypatch.setattr(serve, "GpuBatch", FB)
    reqs = requests(12, (50, 400))
    out = serve.Server(hbm_budget=1e12, chunk_steps=32).serve(reqs, clock=clock, sleep=clock.sleep)
    assert out["completed"] == 12
    for r in reqs:
        assert r.result["step"] == r.steps
        assert r.finished >= r.arrival and r.latency >= 0
    assert not world.live  # every scenario released
    # counted from live particles: the mean of the counts at admission and completion
    assert out["particle_steps"] == pytest.approx(sum((r.scen.n_particles + 0.5 * r.steps) * r.steps for r in reqs))
    assert 0.0 < out["utilisation"] <= 1.0
    assert max(world.batches) > 1  # scenarios shared launches


def test_admission_never_exceeds_budget(monkeypatch):
    clock = FakeClock()
    world = World(clock)
    reqs = requests(10, (100, 200))
    sizes = sorted(serve.scenario_bytes(r.scen) for r in reqs)
    budget = sizes[-1] + sizes[-2]  # at most two of the largest at once
    srv = serve.Server(hbm_budget=budget, chunk_steps=16)

    def probe():
        assert srv.used <= budget

    FS, FB = make_fakes(world, probe)
    monkeypatch.setattr(serve, "GpuScenario", FS)
    monkeypatch.setattr(serve, "GpuBatch", FB)
    out = srv.serve(reqs, clock=clock, sleep=clock.sleep)
    assert out["completed"] == 10
    assert srv.used == 0


def test_request_larger_than_budget_is_refused(monkeypatch):
    clock = FakeClock()
    world = World(clock)
    FS, FB = make_fakes(world, lambda: None)
    monkeypatch.setattr(serve, "GpuScenario", FS)
    monkeypatch.setattr(serve, "GpuBatch", FB)
    reqs = requests(1, (10, 20))
    with pytest.raises(RuntimeError, match="HBM budget"):
        serve.Server(hbm_budget=1000).serve(reqs, clock=clock, sleep=clock.sleep)


def test_arrivals_after_start_are_admitted_while_running(monkeypatch):
    clock = FakeClock()
    world = World(clock, step_cost=5e-3)
    FS, FB = make_fakes(world, lambda: None)
    monkeypatch.setattr(serve, "GpuScenario", FS)
    monkeypatch.setattr(serve, "GpuBatch", FB)
    reqs = requests(6, (300, 300))
    for k, r in enumerate(reqs):
        r.arrival = 0.3 * k  # later requests arrive while earlier ones run
    out = serve.Server(hbm_budget=1e12, chunk_steps=20).serve(reqs, clock=clock, sleep=clock.sleep)
    assert out["completed"] == 6
    # a request admitted before the previous one finished shared its launches
    overlapped = sum(1 for a, b in zip(reqs, reqs[1:]) if b.admitted < a.finished)
    assert overlapped >= 1


def test_slots_bound_the_batch(monkeypatch):
    clock = FakeClock()
    world = World(clock)
    FS, FB = make_fakes(world, lambda: None)
    monkeypatch.setattr(serve, "GpuScenario", FS)
    monkeypatch.setattr(serve, "GpuBatch", FB)
    reqs = requests(7, (40, 80))
    out = serve.Server(hbm_budget=1e12, chunk_steps=16, slots=2).serve(reqs, clock=clock, sleep=clock.sleep)
    assert out["completed"] == 7 and out["slots"] == 2
    assert max(world.batches) <= 2
    assert not world.live
