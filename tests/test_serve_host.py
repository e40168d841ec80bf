"""Host logic of the served form (CPU only): admission by memory budget,
first-come first-served order, continuous batching at quantum boundaries,
latency accounting.  A fake backend stands in for the GPU."""
import pytest

from fluidsim_gb300 import serve


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-3)


class FakeBackend:
    """Each instance needs `mem` bytes; a batch step of k steps takes k ms."""

    def __init__(self, clock, mem):
        self.clock, self.mem = clock, mem
        self.alive = set()
        self.batches = []

    def prepare(self, r):
        return r.rid, self.mem[r.rid], 1000

    def create(self, rid):
        assert rid not in self.alive
        self.alive.add(rid)
        return rid

    def batch(self, instances):
        backend = self

        class B:
            def __init__(self):
                backend.batches.append(tuple(instances))

            def step(self, k):
                backend.clock.t += 1e-3 * k

            def sync(self):
                pass

            def close(self):
                pass

        return B()

    def result(self, inst):
        return {"rid": inst}

    def destroy(self, inst):
        self.alive.remove(inst)


def _reqs(arrivals, steps):
    return [serve.Request(i, a, None, None, s) for i, (a, s) in enumerate(zip(arrivals, steps))]


def test_budget_limits_concurrency_and_order_is_fcfs():
    clock = FakeClock()
    be = FakeBackend(clock, mem={0: 60, 1: 60, 2: 30, 3: 10})
    srv = serve.Server(budget_bytes=100, backend=be, quantum=5, keep_results=True)
    reqs = _reqs([0, 0, 0, 0], [20, 10, 10, 10])
    out = srv.run(reqs, clock=clock, sleep=clock.sleep)
    assert out["requests"] == 4 and not be.alive
    admits = [rid for ev, rid, _ in srv.log if ev == "admit"]
    assert admits == [0, 1, 2, 3]  # first come, first served (no skipping ahead)
    # 0 and 1 never run together (60 + 60 > 100); 1 waits for 0
    assert all(not ({0, 1} <= set(b)) for b in be.batches)
    for r in reqs:
        assert r.result == {"rid": r.rid} and r.done_at >= r.arrival


def test_oversized_request_runs_alone():
    clock = FakeClock()
    be = FakeBackend(clock, mem={0: 500, 1: 10})
    out = serve.Server(budget_bytes=100, backend=be, quantum=4).run(_reqs([0, 0], [8, 8]), clock=clock,
                                                                   sleep=clock.sleep)
    assert out["requests"] == 2
    assert all(len(b) == 1 for b in be.batches)


def test_late_arrival_joins_running_batch():
    clock = FakeClock()
    be = FakeBackend(clock, mem={0: 10, 1: 10})
    srv = serve.Server(budget_bytes=100, backend=be, quantum=5)
    reqs = _reqs([0.0, 0.012], [40, 10])
    out = srv.run(reqs, clock=clock, sleep=clock.sleep)
    assert (0, 1) in be.batches  # request 1 was admitted while 0 was running
    assert reqs[1].done_at < reqs[0].done_at
    assert out["p99_latency_s"] >= out["p50_latency_s"] > 0


def test_work_accounting():
    clock = FakeClock()
    be = FakeBackend(clock, mem={0: 1, 1: 1, 2: 1})
    out = serve.Server(budget_bytes=10, backend=be, quantum=7).run(_reqs([0, 0.001, 0.002], [13, 5, 9]),
                                                                  clock=clock, sleep=clock.sleep)
    assert out["particle_updates"] == 1000 * (13 + 5 + 9)


def test_work_budget_bounds_concurrency():
    """max_particles caps the particles of the running batch (1000 per request
    here): at most two run together, the rest wait in arrival order."""
    clock = FakeClock()
    be = FakeBackend(clock, mem={k: 1 for k in range(5)})
    srv = serve.Server(budget_bytes=10 ** 9, backend=be, quantum=5, max_particles=2500)
    out = srv.run(_reqs([0, 0, 0, 0, 0], [10, 20, 10, 10, 10]), clock=clock, sleep=clock.sleep)
    assert out["requests"] == 5 and not be.alive
    assert max(len(b) for b in be.batches) == 2
    admits = [rid for ev, rid, _ in srv.log if ev == "admit"]
    assert admits == [0, 1, 2, 3, 4]
