"""Host logic of the served form (CPU only): admission by memory budget,
first-come first-served order, continuous batching at quantum boundaries,
latency accounting, and per-request failures injected on the host (failed
admission, an instance's error flag, cancellation).  A fake backend stands in
for the GPU."""
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
    """Each instance needs `mem` bytes; a batch step of k steps takes k ms.
    fail_create: request ids whose instance creation raises (like an allocation
    failure); flag_after: request id -> steps after which its instance reports
    an error status (like its particles leaving the grid)."""

    def __init__(self, clock, mem, fail_create=(), flag_after=None):
        self.clock, self.mem = clock, mem
        self.fail_create = set(fail_create)
        self.flag_after = dict(flag_after or {})
        self.steps_done = {}
        self.alive = set()
        self.batches = []

    def prepare(self, r):
        return r.rid, self.mem[r.rid], 1000

    def create(self, rid):
        assert rid not in self.alive
        if rid in self.fail_create:
            raise RuntimeError("out of device memory")
        self.alive.add(rid)
        self.steps_done[rid] = 0
        return rid

    def batch(self, instances):
        backend = self

        class B:
            def __init__(self):
                self.instances = list(instances)
                backend.batches.append(tuple(instances))

            def step(self, k):
                backend.clock.t += 1e-3 * k
                for rid in instances:
                    backend.steps_done[rid] += k

            def sync(self):
                pass

            def close(self):
                pass

        return B()

    def result(self, inst):
        return {"rid": inst}

    def member_status(self, batch):
        return [5 if rid in self.flag_after and self.steps_done[rid] >= self.flag_after[rid] else 0
                for rid in batch.instances]

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


def test_admission_failure_fails_that_request_only():
    clock = FakeClock()
    be = FakeBackend(clock, mem={0: 1, 1: 1, 2: 1}, fail_create={1})
    srv = serve.Server(budget_bytes=10, backend=be, quantum=5, keep_results=True)
    reqs = _reqs([0, 0, 0], [10, 10, 10])
    out = srv.run(reqs, clock=clock, sleep=clock.sleep)
    assert out["requests"] == 3 and out["failed"] == 1 and not be.alive
    assert reqs[1].error.startswith("admission failed") and not reqs[1].result
    assert reqs[0].result == {"rid": 0} and reqs[2].result == {"rid": 2}
    assert out["particle_updates"] == 1000 * 20


def test_instance_error_evicts_only_that_member():
    """Request 1's instance reports an error after 10 steps: it is evicted at
    that quantum boundary; 0 and 2 finish all their steps."""
    clock = FakeClock()
    be = FakeBackend(clock, mem={0: 1, 1: 1, 2: 1}, flag_after={1: 10})
    srv = serve.Server(budget_bytes=10, backend=be, quantum=5, keep_results=True)
    reqs = _reqs([0, 0, 0], [30, 30, 30])
    out = srv.run(reqs, clock=clock, sleep=clock.sleep)
    assert out["failed"] == 1 and reqs[1].error == "instance error 5" and not be.alive
    assert ("failed", 1, reqs[1].done_at) in srv.log
    assert reqs[0].result and reqs[2].result and not reqs[0].error
    assert out["particle_updates"] == 1000 * (30 + 5 + 30)  # 1's erroring quantum does not count
    assert all(1 not in b for b in be.batches[-1:])


def test_cancellation_of_waiting_and_running_requests():
    """1 is cancelled while it waits (behind 0 for memory); 0 is cancelled
    while it runs, after 10 of its 40 steps; 2 is unaffected."""
    clock = FakeClock()
    be = FakeBackend(clock, mem={0: 60, 1: 60, 2: 1})
    srv = serve.Server(budget_bytes=100, backend=be, quantum=5, keep_results=True)
    reqs = _reqs([0, 0, 0], [40, 10, 10])
    srv.cancel(1)
    status = be.member_status

    def member_status(batch):
        if be.steps_done.get(0, 0) >= 10:
            srv.cancel(0)
        return status(batch)

    be.member_status = member_status
    out = srv.run(reqs, clock=clock, sleep=clock.sleep)
    assert reqs[1].error == "cancelled" and reqs[0].error == "cancelled" and out["failed"] == 2
    assert be.steps_done[0] < 40 and 1 not in be.steps_done
    assert reqs[2].result == {"rid": 2} and not be.alive


def test_admission_overlaps_the_running_quantum():
    """A request that arrives while a quantum runs is created between the
    quantum's launch and the wait for it (its creation overlaps the GPU work),
    and joins the batch at the next quantum, not the running one."""
    clock = FakeClock()
    be = FakeBackend(clock, mem={0: 10, 1: 10})
    calls = []
    create, member_status, batch = be.create, be.member_status, be.batch

    def rec_create(rid):
        calls.append(("create", rid))
        return create(rid)

    def rec_status(b):
        calls.append(("status", tuple(b.instances)))
        return member_status(b)

    def rec_batch(instances):
        b = batch(instances)
        step = b.step

        def rec_step(k):
            calls.append(("step", tuple(b.instances)))
            step(k)

        b.step = rec_step
        return b

    be.create, be.member_status, be.batch = rec_create, rec_status, rec_batch
    reqs = _reqs([0.0, 0.003], [40, 10])
    out = serve.Server(budget_bytes=100, backend=be, quantum=5).run(reqs, clock=clock, sleep=clock.sleep)
    assert out["requests"] == 2 and not be.alive
    k = calls.index(("create", 1))
    # created right after a quantum of request 0 alone was launched, before its wait
    assert calls[k - 1] == ("step", (0,)) and calls[k + 1] == ("status", (0,))
    # and stepped with 0 from the next quantum on
    assert ("step", (0, 1)) in calls[k + 1:]
