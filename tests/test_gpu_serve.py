"""Served form on the GPU: requests admitted while others run produce the
same results as when each runs alone (bit for bit: a member of a batch runs
the same kernels on its own data)."""
import numpy as np
import pytest

from fluidsim_gb300 import serve

pytestmark = pytest.mark.gpu


def _stream():
    return serve.poisson_stream(5, rate=400.0, seed=11, fluid_range=(2000, 9000), solid_range=(200, 900),
                                steps_range=(8, 30))


def test_served_results_equal_solo():
    mixed = _stream()
    out = serve.Server(budget_bytes=2 ** 36, quantum=3, keep_results=True).run(mixed)
    # requests joined and left the live batch while it ran
    assert out["requests"] == 5 and out["batch_rebuilds"] + out["batch_joins"] >= 2 and out["batch_leaves"] >= 1
    solo = _stream()
    serve.serve_one_by_one(solo, keep_results=True)
    for a, b in zip(mixed, solo):
        assert a.result.keys() == b.result.keys()
        for k in a.result:
            assert np.array_equal(a.result[k], b.result[k]), (a.rid, k)


def test_budget_admits_one_at_a_time():
    reqs = _stream()[:3]
    srv = serve.Server(budget_bytes=1, quantum=4)  # every request alone
    out = srv.run(reqs)
    assert out["requests"] == 3
    assert out["batch_rebuilds"] == 3


def test_instance_error_evicts_only_that_request():
    reqs = _stream()
    bad = reqs[2].rid
    be = serve.GpuBackend(0)
    create = be.create

    def create_flagged(prepared):
        inst = create(prepared)
        if prepared is flagged["data"]:
            x = inst.get("fluid_pos")
            x[0] = [50.0, 50.0, 50.0]
            inst.set("fluid_pos", x)
        return inst

    flagged = {"data": None}
    prepare = be.prepare

    def prepare_mark(r):
        out = prepare(r)
        if r.rid == bad:
            flagged["data"] = out[0]
        return out

    be.prepare, be.create = prepare_mark, create_flagged
    out = serve.Server(budget_bytes=2 ** 36, backend=be, quantum=3, keep_results=True).run(reqs)
    assert out["failed"] == 1 and reqs[2].error.startswith("instance error")
    solo = _stream()
    serve.serve_one_by_one(solo, keep_results=True)
    for a, b in zip(reqs, solo):
        if a.rid == bad:
            continue
        for k in a.result:
            assert np.array_equal(a.result[k], b.result[k]), (a.rid, k)
