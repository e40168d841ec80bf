"""The device case generator (fsim_create_case) against the host generator
(fsim_case_generate + fsim_create): the same particles in the same order,
bit for bit, and the same trajectory."""
import time

import numpy as np
import pytest

from fluidsim_gb300 import api, cases

pytestmark = pytest.mark.gpu

FIELDS = ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "solid_ref_pos",
          "solid_type", "virt_pos")


def _compare(spec, steps=0):
    cfg, case = spec
    host_cfg, pa = cases.make(spec)
    a = api.Simulation(host_cfg, pa, device=0)
    b = api.Simulation.from_case(cfg, case, device=0)
    assert a.n == b.n
    for s in (a, b):
        s.step(steps)
        s.sync()
    for f in FIELDS:
        if f.startswith("solid") and a.n["solid"] == 0:
            continue
        assert np.array_equal(a.get(f), b.get(f)), f
    a.close()
    b.close()


@pytest.mark.parametrize("spec", [
    cases.tiny_box(),
    cases.tiny_box(jitter=0.02, seed=99, with_solid=False, viscid=False),
    cases.small_dam_break(jitter=0.01, seed=5),
    cases.small_dam_break(jitter=0.01, seed=5, precision=api.PRECISION_MIXED),
])
def test_device_case_equals_host_case(spec):
    _compare(spec, steps=0)
    _compare(spec, steps=3)


def test_device_case_4m_bitexact_and_counts():
    spec = cases.fsi_4m_jitter(precision=api.PRECISION_FP32)
    cfg, case = spec
    t0 = time.perf_counter()
    host_cfg, pa = cases.make(spec)
    t_host = time.perf_counter() - t0
    assert api.case_counts(case) == (pa.n_fluid, pa.n_solid, pa.n_virt) == (4194304, 27000, 912600)
    a = api.Simulation(host_cfg, pa, device=0)
    t0 = time.perf_counter()
    b = api.Simulation.from_case(cfg, case, device=0)
    t_dev = time.perf_counter() - t0
    print("host generate %.2f s, device create %.2f s" % (t_host, t_dev))
    for f in FIELDS:
        assert np.array_equal(a.get(f), b.get(f)), f
    a.close()
    b.close()


def test_device_case_solid_below_floor_and_outside_tank():
    cfg, case = cases.tiny_box(jitter=0.015, seed=123)
    case.solid_fixed_layers = 3
    case.solid_lo[2] = -2
    case.solid_n[2] = 30
    _compare((cfg, case), steps=2)
