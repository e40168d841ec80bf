"""CUDA path vs the CPU oracle, through the C ABI.

Bit-exact: cell indices, per-cell membership sets (the cell-sorted
permutation) and per-particle neighbour counts.  Floating point: per-phase
outputs against the FP32 and FP64 oracles and trajectories against the FP64
oracle, as normalised max error |gpu - oracle|_inf / |oracle|_inf per field.
"""
import numpy as np
import pytest

from conftest import nerr, target_200_steps
from fluidsim_gb300 import api, cases
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

# Tolerances (normalised max error, per field).
# The plain form computes in FP32 like the reference, and some outputs of that
# formulation are ill-conditioned in FP32 whatever the kernel does (the Green
# strain of a solid at rest is a cancellation F^T F - I of ~1e-7, the Tait EOS
# (rho/rho0)^7 - 1 near rho0).  So every check is two-sided:
#   err(gpu, fp64) <= FP32_FACTOR * err(fp32 oracle, fp64) + TOL
# i.e. the CUDA path is as accurate as an FP32 restatement of the reference,
# and exact-ish where FP32 is well-conditioned.  On these cases the solid is at
# rest or falling freely, so its stress is FP32 round-off and its check here is
# loose by nature; tests/test_gpu_contact.py checks the stress of a deformed
# solid, and the coupling with fluid and solid in contact, to 1e-4.
TOL_PHASE = 5e-5        # one phase
FP32_FACTOR = 2.0
TRAJ_FP32_FACTOR = 3.0  # chaotic trajectories: rounding differences grow, so a wider factor


@pytest.fixture(scope="module")
def dam():
    return cases.make(cases.small_dam_break(keep=True, jitter=0.01, seed=7))


def _gpu_oracles(cfg, pa):
    return api.Simulation(cfg, pa, device=0), orc.OracleSim(cfg, pa, "f32"), orc.OracleSim(cfg, pa, "f64")


def test_cell_ids_and_membership_bitexact(dam):
    cfg, pa = dam
    sim = api.Simulation(cfg, pa, device=0)
    sim.phase(api.PHASE_CELL)
    d = sim.derived()
    for name, pos in (("fluid", pa.fluid_pos), ("solid", pa.solid_pos), ("virt", pa.virt_pos)):
        got = sim.get(name + "_cell_id")
        want = orc.cell_ids(d, pos)
        assert np.array_equal(got, want), name
        # the cell-sorted permutation: cell c holds exactly the ids whose cell is c
        start, ids = sim.cells({"fluid": 0, "solid": 1, "virt": 2}[name])
        assert start[0] == 0 and start[-1] == len(pos)
        counts = np.bincount(want, minlength=d.cell_number_total)
        assert np.array_equal(np.diff(start), counts)
        assert np.array_equal(np.sort(ids), np.arange(len(pos)))
        cell_of_slot = np.repeat(np.arange(d.cell_number_total), counts)
        assert np.array_equal(want[ids], cell_of_slot)
    sim.close()


def test_neighbor_counts_bitexact(dam):
    cfg, pa = dam
    sim = api.Simulation(cfg, pa, device=0)
    ref = orc.OracleSim(cfg, pa, "f64")
    sim.phase(api.PHASE_CELL)
    ref.phase(api.PHASE_CELL)
    got, want = sim.neighbor_counts(), ref.neighbor_counts()
    assert np.array_equal(got, want)
    # every fluid particle sees fluid and the block corner sees walls; the
    # plate starts 0.4 m away from the fluid, so fluid-solid counts are 0 here
    assert want[:, 0].min() > 0 and want[:, 2].sum() > 0
    sim.close()


def test_phases_match_oracle(dam):
    cfg, pa = dam
    sim, r32, r64 = _gpu_oracles(cfg, pa)
    checks = {
        api.PHASE_COUPLE: ["solid_normal", "solid_p"],
        api.PHASE_VIRT: ["virt_rho", "virt_p", "virt_vel", "virt_normal"],
        api.PHASE_FLUID: ["fluid_drho_dt", "fluid_du_dt", "fluid_pos", "fluid_vel", "fluid_rho", "fluid_p"],
        api.PHASE_SOLID: ["solid_F", "solid_PK1", "solid_Linv", "solid_du_dt", "solid_couple_dudt", "solid_pos",
                          "solid_vel"],
    }
    for step in range(2):
        for ph in (api.PHASE_CELL, api.PHASE_COUPLE, api.PHASE_VIRT, api.PHASE_FLUID, api.PHASE_SOLID):
            sim.phase(ph)
            r32.phase(ph)
            r64.phase(ph)
            sim.sync()
            for f in checks.get(ph, []):
                g, want = sim.get(f), r64.get(f)
                e_gpu, e_f32 = nerr(g, want), nerr(r32.get(f), want)
                print("step %d %-18s gpu %.3g  fp32-oracle %.3g" % (step, f, e_gpu, e_f32))
                assert e_gpu <= FP32_FACTOR * e_f32 + TOL_PHASE, (step, f, e_gpu, e_f32)
    sim.close()


def test_one_step_graph_matches_phases(dam):
    """fsim_step (CUDA graph) equals the phase-by-phase calls bit for bit."""
    cfg, pa = dam
    a = api.Simulation(cfg, pa, device=0)
    b = api.Simulation(cfg, pa, device=0)
    for _ in range(3):
        a.step(1)
        for ph in range(5):
            b.phase(ph)
    a.sync()
    b.sync()
    for f in ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "virt_p", "solid_F"):
        assert np.array_equal(a.get(f), b.get(f)), f
    a.close()
    b.close()


def test_sweep_shapes_bit_identical(dam):
    """The autotuner's first step sweeps with each of the three launch shapes
    (twice) in place of one sweep; a handle stepped by phases keeps shape 0.
    The states agree bit for bit, and the tuner has picked one shape from
    three timed ones."""
    cfg, pa = dam
    a = api.Simulation(cfg, pa, device=0)
    b = api.Simulation(cfg, pa, device=0)
    assert a.sweep_tuning()[0] == -1
    a.step(5)
    for _ in range(5):
        for ph in range(5):
            b.phase(ph)
    a.sync()
    b.sync()
    chosen, ms = a.sweep_tuning()
    assert chosen in (0, 1, 2) and all(t > 0 for t in ms)
    for f in ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "virt_p"):
        assert np.array_equal(a.get(f), b.get(f)), f
    a.close()
    b.close()


def _plate_touching_fluid(speed):
    """tiny_box with the plate moved to one particle spacing from the fluid
    block (inside the impact distance), moving at `speed` along x."""
    cfg, pa = cases.make(cases.tiny_box())
    shift = pa.solid_pos[:, 0].min() - pa.fluid_pos[:, 0].max() - cfg.particle_diameter
    sp, sr, sv = pa.solid_pos.copy(), pa.solid_ref_pos.copy(), np.zeros_like(pa.solid_vel)
    sp[:, 0] -= shift
    sr[:, 0] -= shift
    sv[:, 0] = speed
    return cfg, api.ParticleArrays(pa.fluid_pos, pa.fluid_vel, pa.fluid_rho, pa.fluid_p, sp, sv, sr,
                                   pa.solid_type, pa.virt_pos)


@pytest.mark.parametrize("bypass", [False, True])
def test_solid_fluid_lists_equal_full_walk(bypass):
    """Solid sub-steps after the first walk a per-lane list of the fluid
    candidates that the first recorded; the results equal the full 27-cell
    walk of every sub-step bit for bit.  With `bypass` the plate moves more
    than 0.1 R per sub-step, so later sub-steps fall back to the walk."""
    cfg, pa = _plate_touching_fluid(0.0)
    steps = 6
    if bypass:
        # 0.75 of the allowed displacement (0.1 R) per sub-step: sub-step 1
        # walks the list, sub-steps 2 and 3 walk the cells; one step
        R = float(np.sqrt(api.derive(cfg).impact_distance_square))
        cfg, pa = _plate_touching_fluid(-0.75 * 0.1 * R / (cfg.dt / cfg.solid_sub_step))
        steps = 1
    full = api.Config.from_buffer_copy(cfg)
    full.solid_full_walk = 1
    out = []
    for c in (cfg, full):
        with api.Simulation(c, pa, device=0) as s:
            s.step(steps)
            s.sync()
            out.append({f: s.get(f) for f in ("solid_pos", "solid_vel", "fluid_pos", "fluid_vel", "fluid_p")})
    for f in out[0]:
        assert np.all(np.isfinite(out[0][f])), f
        assert np.array_equal(out[0][f], out[1][f]), f
    if not bypass:  # the plate's free particles (type 0) felt the fluid
        assert np.any(out[0]["solid_vel"][pa.solid_type == 0, 0] != 0.0)


def test_deterministic_repeat(dam):
    cfg, pa = dam
    outs = []
    for _ in range(2):
        s = api.Simulation(cfg, pa, device=0)
        s.step(5)
        s.sync()
        outs.append((s.get("fluid_pos"), s.get("fluid_rho"), s.get("solid_pos")))
        s.close()
    for x, y in zip(*outs):
        assert np.array_equal(x, y)


def test_1_and_200_steps_vs_fp64():
    """Per-field error after 1 and 200 steps.  Fluid fields and solid
    positions meet the accuracy target (1e-3, or 1.5x the FP32 oracle's error
    where that exceeds it); every field stays within 3x the FP32 oracle's own
    error plus 5e-5."""
    cfg, pa = cases.make(cases.small_dam_break(jitter=0.01, seed=11))
    sim = api.Simulation(cfg, pa, device=0)
    r64 = orc.OracleSim(cfg, pa, "f64")
    r32 = orc.OracleSim(cfg, pa, "f32")
    fields = ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "solid_PK1")
    for n in (1, 199):
        sim.step(n)
        r64.step(n)
        r32.step(n)
        sim.sync()
        for f in fields:
            want = r64.get(f)
            e_gpu, e_f32 = nerr(sim.get(f), want), nerr(r32.get(f), want)
            print("after %3d more steps %-10s gpu %.3g  fp32-oracle %.3g" % (n, f, e_gpu, e_f32))
            if f.startswith("fluid") or f == "solid_pos":
                assert e_gpu < target_200_steps(e_f32), (f, e_gpu, e_f32)
            # no field worse than the FP32 restatement's own error allows
            assert e_gpu <= TRAJ_FP32_FACTOR * e_f32 + TOL_PHASE, (f, e_gpu, e_f32)
    sim.close()
