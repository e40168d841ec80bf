"""Binary snapshots: an instance restored from a snapshot continues bit for
bit like the original (both precision forms), and snapshots round-trip
through files."""
import numpy as np
import pytest

from fluidsim_gb300 import api, cases

pytestmark = pytest.mark.gpu

FIELDS = ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "solid_PK1", "virt_p",
          "solid_normal")


def _state(sim):
    return {f: sim.get(f) for f in FIELDS}


@pytest.mark.parametrize("precision", [api.PRECISION_FP32, api.PRECISION_MIXED])
def test_resume_is_bit_exact(precision):
    cfg, pa = cases.make(cases.small_dam_break(jitter=0.01, seed=21, precision=precision))
    a = api.Simulation(cfg, pa, device=0)
    a.step(7)
    snap = a.snapshot(step=7)
    a.step(5)
    a.sync()
    want = _state(a)
    b = api.Simulation.from_snapshot(snap, device=0)
    assert b.snapshot_step == 7 and b.n == a.n
    b.step(5)
    b.sync()
    for f, w in want.items():
        assert np.array_equal(b.get(f), w), f
    a.close()
    b.close()


def test_snapshot_file_round_trip(tmp_path):
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=4))
    a = api.Simulation(cfg, pa, device=0)
    a.step(3)
    path = tmp_path / "state.fsnap"
    a.snapshot_write(str(path), step=3)
    b = api.Simulation.from_snapshot_file(str(path), device=0)
    assert b.snapshot_step == 3
    for f in ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "virt_pos"):
        assert np.array_equal(a.get(f), b.get(f)), f
    # the same bytes again from the restored instance
    assert np.array_equal(a.snapshot(step=3), b.snapshot(step=3))
    a.close()
    b.close()


def test_corrupt_snapshots_are_rejected():
    cfg, pa = cases.make(cases.tiny_box())
    with api.Simulation(cfg, pa, device=0) as a:
        snap = a.snapshot()
    with pytest.raises(api.FsimError):
        api.Simulation.from_snapshot(snap[:-16], device=0)  # truncated
    bad = snap.copy()
    bad[100:104] = 0xFF  # counts no longer match the size
    with pytest.raises(api.FsimError):
        api.Simulation.from_snapshot(bad, device=0)
