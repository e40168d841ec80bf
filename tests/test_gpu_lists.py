"""Fluid neighbour lists (cfg.neighbor_skin > 0, the default), plain and mixed form.

The list sweep must see exactly the pairs the reference's cell walk sees:
every pair within the impact distance, in neighbouring cells.  These tests
check that property directly (list entries within R against the cell-walk
neighbour counts, bit for bit, while particles move fast enough to force
rebuilds), check the list path against the cell-walk sweep of the same
library (skin 0) per phase and over steps, and check the bookkeeping around
it: rebuilds after positions are set, snapshots taken between rebuilds, and
the cell-coordinate check where a cell side is within FP32 rounding of the
impact distance.
"""
import numpy as np
import pytest

from conftest import nerr
from fluidsim_gb300 import api, cases

pytestmark = pytest.mark.gpu

# Summation order differs between the list sweep (list-grid rows) and the
# cell-walk sweep (impact-grid rows): FP32 rounding differences only.
TOL_RATE = 2e-4   # per-phase rates (sums of ~80 pair terms with cancellation)
TOL_STATE = 1e-5  # positions, velocities, densities after a few steps
# wall pressure: the nearest fluid particle's EOS pressure, p ~ (rho/rho0)^7,
# which scales a density rounding difference by gamma c0^2 rho0 / max|p|
TOL_STATE_P = 5e-5


FORMS = [api.PRECISION_FP32, api.PRECISION_MIXED]


def _moving_dam(skin, vx=3.0, precision=api.PRECISION_FP32):
    """The jittered small dam break with a uniform extra velocity: at 3 m/s a
    particle moves the rebuild allowance (about 0.05 R = 1.3 mm) in about four
    steps, so a few dozen steps rebuild the lists several times."""
    cfg, pa = cases.make(cases.small_dam_break(keep=True, jitter=0.01, seed=13, precision=precision))
    cfg.neighbor_skin = skin
    vel = pa.fluid_vel.copy()
    vel[:, 0] += vx
    pa = api.ParticleArrays(pa.fluid_pos, vel, pa.fluid_rho, pa.fluid_p, pa.solid_pos, pa.solid_vel,
                            pa.solid_ref_pos, pa.solid_type, pa.virt_pos)
    return cfg, pa


def test_list_forms():
    cfg, pa = cases.make(cases.tiny_box())
    with api.Simulation(cfg, pa, device=0) as sim:
        st = sim.list_stats()
        assert st["enabled"] == 1 and st["builds"] == 0 and st["capacity"] > 100 and st["check"] == 0
        sim.step(2)
        assert sim.list_stats()["builds"] == 1  # the first step builds; nothing has moved since
    cfg.neighbor_skin = 0.0
    with api.Simulation(cfg, pa, device=0) as sim:
        assert sim.list_stats()["enabled"] == 0
        with pytest.raises(api.FsimError):
            sim.list_counts()
    cfg, pa = cases.make(cases.tiny_box(precision=api.PRECISION_MIXED))
    with api.Simulation(cfg, pa, device=0) as sim:
        st = sim.list_stats()  # the mixed form always compares cell coordinates
        assert st["enabled"] == 1 and st["check"] == 1
        sim.step(2)
        assert sim.list_stats()["builds"] == 1


@pytest.mark.parametrize("precision", FORMS)
def test_lists_hold_every_pair_while_moving(precision):
    """After every cell phase the list entries within R are exactly the
    cell walk's pairs (fluid, solid and wall counts per particle), through
    several rebuilds."""
    cfg, pa = _moving_dam(0.1, precision=precision)
    sim = api.Simulation(cfg, pa, device=0)
    for step in range(24):
        sim.phase(api.PHASE_CELL)
        got, want = sim.list_counts(), sim.neighbor_counts()
        assert np.array_equal(got, want), step
        for ph in (api.PHASE_COUPLE, api.PHASE_VIRT, api.PHASE_FLUID, api.PHASE_SOLID):
            sim.phase(ph)
    sim.sync()
    builds = sim.list_stats()["builds"]
    print("list builds in 24 steps:", builds)
    assert builds >= 4
    sim.close()


@pytest.mark.parametrize("precision", FORMS)
def test_lists_match_cell_walk_per_phase(precision):
    cfg, pa = _moving_dam(0.1, precision=precision)
    a = api.Simulation(cfg, pa, device=0)
    cfg0, _ = _moving_dam(0.0, precision=precision)
    b = api.Simulation(cfg0, pa, device=0)
    for step in range(3):
        for ph in range(5):
            a.phase(ph)
            b.phase(ph)
        a.sync()
        b.sync()
        for f in ("fluid_drho_dt", "fluid_du_dt"):
            e = nerr(a.get(f), b.get(f).astype(np.float64))
            print("step %d %-14s lists vs cell walk %.3g" % (step, f, e))
            assert e <= TOL_RATE, (step, f, e)
        for f in ("fluid_cell_id", "solid_cell_id", "virt_cell_id"):
            assert np.array_equal(a.get(f), b.get(f)), f
    a.close()
    b.close()


@pytest.mark.parametrize("precision", FORMS)
def test_lists_match_cell_walk_over_steps(precision):
    """30 steps with rebuilds: the list path stays within FP32 rounding of the
    cell-walk path (and the solid, which sees the fluid through the per-step
    cell index, too)."""
    cfg, pa = _moving_dam(0.1, precision=precision)
    cfg0, _ = _moving_dam(0.0, precision=precision)
    with api.Simulation(cfg, pa, device=0) as a, api.Simulation(cfg0, pa, device=0) as b:
        a.step(30)
        b.step(30)
        a.sync()
        b.sync()
        assert a.list_stats()["builds"] >= 5
        for f in ("fluid_pos", "fluid_vel", "fluid_rho", "solid_pos", "solid_vel", "virt_p"):
            e = nerr(a.get(f), b.get(f).astype(np.float64))
            print("30 steps %-10s lists vs cell walk %.3g" % (f, e))
            assert e <= (TOL_STATE_P if f == "virt_p" else TOL_STATE), (f, e)


@pytest.mark.parametrize("precision", FORMS)
def test_positions_set_after_the_cell_phase_reach_the_walks(precision):
    """The wall and coupling walks test positions in the per-step index's
    order (a copy the cell phase writes): positions written from the host
    after the cell phase must reach that copy, so the walls and the solid's
    pressure see them exactly as the cell walk (skin 0) does."""
    cfg, pa = _moving_dam(0.1, vx=0.0, precision=precision)
    cfg0, _ = _moving_dam(0.0, vx=0.0, precision=precision)
    a = api.Simulation(cfg, pa, device=0)
    b = api.Simulation(cfg0, pa, device=0)
    shifted = pa.fluid_pos.copy()
    shifted[:, 1] += 0.2 * cfg.particle_diameter  # along gravity: the walls' hydrostatic pressure moves
    for sim in (a, b):
        sim.phase(api.PHASE_CELL)
        sim.set("fluid_pos", shifted)  # both walk the index of the unshifted positions
        sim.phase(api.PHASE_COUPLE)
        sim.phase(api.PHASE_VIRT)
    a.sync()
    b.sync()
    # the nearest fluid particle is order-independent: the walls agree bit for bit
    for f in ("virt_rho", "virt_p", "virt_vel"):
        assert np.array_equal(a.get(f), b.get(f)), f
    # the Shepard sums follow each index's order within a cell: rounding only
    e = nerr(a.get("solid_p"), b.get("solid_p").astype(np.float64))
    assert e <= 1e-6, e
    # and the walls did see the shift
    with api.Simulation(cfg0, pa, device=0) as c:
        c.phase(api.PHASE_CELL)
        c.phase(api.PHASE_COUPLE)
        c.phase(api.PHASE_VIRT)
        c.sync()
        assert not np.array_equal(c.get("virt_p"), b.get("virt_p"))
    a.close()
    b.close()


@pytest.mark.parametrize("precision", FORMS)
def test_set_positions_counts_as_displacement(precision):
    """Positions written from the host move particles like a step does: a
    shift beyond the rebuild allowance (about 0.05 R = 0.13 dx) rebuilds the
    lists at the next step, a shift well within it does not, and either way
    the lists hold every pair."""
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=2, precision=precision))
    with api.Simulation(cfg, pa, device=0) as sim:
        sim.step(3)
        b0 = sim.list_stats()["builds"]
        pos = sim.get("fluid_pos")
        pos[:, 1] += 0.01 * cfg.particle_diameter
        sim.set("fluid_pos", pos)
        sim.step(1)
        assert sim.list_stats()["builds"] == b0
        pos = sim.get("fluid_pos")
        pos[:, 1] += 0.3 * cfg.particle_diameter
        sim.set("fluid_pos", pos)
        sim.step(1)
        assert sim.list_stats()["builds"] == b0 + 1
        sim.phase(api.PHASE_CELL)
        assert np.array_equal(sim.list_counts(), sim.neighbor_counts())


@pytest.mark.parametrize("precision", FORMS)
def test_snapshot_between_rebuilds_resumes_bit_exact(precision):
    cfg, pa = _moving_dam(0.1, precision=precision)
    a = api.Simulation(cfg, pa, device=0)
    a.step(6)
    builds = a.list_stats()["builds"]
    snap = a.snapshot(step=6)
    a.step(14)
    a.sync()
    assert a.list_stats()["builds"] > builds  # the continuation rebuilds
    b = api.Simulation.from_snapshot(snap, device=0)
    assert b.list_stats()["builds"] == builds
    b.step(14)
    b.sync()
    for f in ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "virt_p"):
        assert np.array_equal(a.get(f), b.get(f)), f
    assert a.list_stats()["builds"] == b.list_stats()["builds"]
    a.close()
    b.close()


def test_cell_coordinate_check_where_a_side_is_near_r():
    """Ensemble member 25 has a y cell side within FP32 rounding of the impact
    distance: its lists also compare cell coordinates, and its pair set and
    rates match the cell walk."""
    cfg, case = cases.ensemble(64, 2024)[25]
    cfg.keep_derivatives = 1
    cfg, pa = cases.make((cfg, case))
    a = api.Simulation(cfg, pa, device=0)
    assert a.list_stats()["check"] == 1
    cfg.neighbor_skin = 0.0
    b = api.Simulation(cfg, pa, device=0)
    for step in range(2):
        for ph in range(5):
            a.phase(ph)
            b.phase(ph)
            if ph == api.PHASE_CELL:
                want = b.neighbor_counts()
                assert np.array_equal(a.neighbor_counts(), want)
                # the lists hold every cell-walk pair; pairs within R in cells two
                # apart (rounding) are in them too and the sweep's check drops them
                assert (a.list_counts() >= want).all()
        a.sync()
        b.sync()
        for f in ("fluid_drho_dt", "fluid_du_dt"):
            e = nerr(a.get(f), b.get(f).astype(np.float64))
            print("member 25 step %d %-14s %.3g" % (step, f, e))
            assert e <= TOL_RATE, (step, f, e)
    a.close()
    b.close()
