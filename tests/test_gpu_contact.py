"""Fluid-solid coupling and solid stress against the CPU oracle, with fluid
and solid in contact and the solid deformed.

Reference: fluidSolidCalculate (src/fluid.cu:71-119), solidFluidCouple
(src/solid.cu:81-117), the Shepard solid pressure and normal of
solidCoupleUpdate (src/solid.cu:262-328), solidStressCalculation and
solidSolidForce (src/solid.cu:27-36,119-157).

Cases (tests/parity_cases.py): a plate one spacing from a fluid block, at
rest and moving into it at 0.5 m/s; the 32,000-particle dam break with its
plate inside the impact distance of the fluid; an elastic cube under an
affine 2-4 % stretch and 4 % shear with a linear velocity field.
"""
import numpy as np
import pytest

import parity_cases as pc
from conftest import nerr, target_200_steps
from fluidsim_gb300 import api
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

# Per phase: err(gpu, fp64) <= FP32_FACTOR * err(fp32 oracle, fp64) + TOL_PHASE
# (normalised max error).  Every field checked below is O(1) relative to its
# own scale here (contact pressure, traction, O(strain) stress), so a wrong
# term is an O(1) error and fails by orders of magnitude.
FP32_FACTOR = 2.0
TOL_PHASE = 5e-5
TRAJ_FP32_FACTOR = 3.0     # other fields after 200 steps: within 3x the FP32 restatement's error
TOL_STRESS = 1e-4          # deformed solid, one sub-step: F, PK1, du/dt vs FP64
TOL_F_ANALYTIC = 1e-5      # deformed solid: F equals the prescribed affine map

CONTACT_FIELDS = {
    api.PHASE_COUPLE: ["solid_normal", "solid_p"],
    api.PHASE_FLUID: ["fluid_drho_dt", "fluid_du_dt", "fluid_vel", "fluid_rho", "fluid_p"],
    api.PHASE_SOLID: ["solid_couple_dudt", "solid_du_dt", "solid_PK1", "solid_pos", "solid_vel"],
}


def _contact_case(name):
    if name == "plate_rest":
        return pc.plate_touching_fluid(0.0)
    if name == "plate_impact":
        return pc.plate_touching_fluid(-0.5)
    return pc.dam_gate_near()


def _run_phases(cfg, pa, steps, fields, check):
    sim = api.Simulation(cfg, pa, device=0)
    r32, r64 = orc.OracleSim(cfg, pa, "f32"), orc.OracleSim(cfg, pa, "f64")
    seen = {}
    for step in range(steps):
        for ph in range(5):
            for s in (sim, r32, r64):
                s.phase(ph)
            sim.sync()
            if ph == api.PHASE_CELL:
                got, want = sim.neighbor_counts(), r64.neighbor_counts()
                assert np.array_equal(got, want), "neighbour counts"
                seen.setdefault("fluid_solid_pairs", int(want[:, 1].sum()))
            for f in fields.get(ph, []):
                want = r64.get(f)
                g = sim.get(f)
                e_gpu, e_f32 = nerr(g, want), nerr(r32.get(f), want)
                seen[f] = max(seen.get(f, 0.0), float(np.abs(want).max()))
                print("step %d %-18s |fp64| %.3g  gpu %.3g  fp32-oracle %.3g" % (step, f, np.abs(want).max(), e_gpu,
                                                                                  e_f32))
                check(f, e_gpu, e_f32)
    sim.close()
    return seen


@pytest.mark.parametrize("name", ["plate_rest", "plate_impact", "dam_gate"])
def test_contact_phases_match_oracle(name):
    cfg, pa = _contact_case(name)

    def check(f, e_gpu, e_f32):
        assert e_gpu <= FP32_FACTOR * e_f32 + TOL_PHASE, (f, e_gpu, e_f32)

    seen = _run_phases(cfg, pa, 2, CONTACT_FIELDS, check)
    # the coupling terms are live: fluid-solid pairs exist, the Shepard
    # pressure and the traction are far from zero
    assert seen["fluid_solid_pairs"] > 0
    assert seen["solid_p"] > 100.0 and seen["solid_couple_dudt"] > 1.0, seen


@pytest.mark.parametrize("name", ["plate_impact", "dam_gate"])
def test_contact_200_steps_vs_fp64(name):
    cfg, pa = _contact_case(name)
    sim = api.Simulation(cfg, pa, device=0)
    r32, r64 = orc.OracleSim(cfg, pa, "f32"), orc.OracleSim(cfg, pa, "f64")
    for s in (sim, r32, r64):
        s.step(200)
    sim.sync()
    for f in ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "solid_p",
              "solid_couple_dudt", "solid_PK1"):
        want = r64.get(f)
        e_gpu, e_f32 = nerr(sim.get(f), want), nerr(r32.get(f), want)
        print("200 steps %-18s |fp64| %.3g  gpu %.3g  fp32-oracle %.3g" % (f, np.abs(want).max(), e_gpu, e_f32))
        if f.startswith("fluid") or f == "solid_pos":
            assert e_gpu < target_200_steps(e_f32), (f, e_gpu, e_f32)
        assert e_gpu <= TRAJ_FP32_FACTOR * e_f32 + TOL_PHASE, (f, e_gpu, e_f32)
    assert np.abs(r64.get("solid_couple_dudt")).max() > 1.0
    sim.close()


def test_deformed_solid_one_substep():
    """One sub-step on a prescribed affine deformation: F equals the map, and
    F, the first Piola-Kirchhoff stress P = F S and the stress-divergence plus
    artificial-viscosity acceleration match FP64 to 1e-4."""
    cfg, pa = pc.deformed_block(sub_steps=1)
    sim = api.Simulation(cfg, pa, device=0)
    r32, r64 = orc.OracleSim(cfg, pa, "f32"), orc.OracleSim(cfg, pa, "f64")
    for ph in range(5):
        for s in (sim, r32, r64):
            s.phase(ph)
    sim.sync()
    F = sim.get("solid_F").reshape(-1, 3, 3)
    assert np.abs(F - pc.A_DEFORM).max() < TOL_F_ANALYTIC
    for f in ("solid_F", "solid_PK1", "solid_du_dt", "solid_vel"):
        want = r64.get(f)
        e_gpu, e_f32 = nerr(sim.get(f), want), nerr(r32.get(f), want)
        print("deformed %-12s |fp64| %.3g  gpu %.3g  fp32-oracle %.3g" % (f, np.abs(want).max(), e_gpu, e_f32))
        assert e_gpu < TOL_STRESS, (f, e_gpu)
    assert np.abs(r64.get("solid_PK1")).max() > 1e4  # O(strain * E): well conditioned
    sim.close()


def test_deformed_solid_20_steps():
    cfg, pa = pc.deformed_block(sub_steps=4)
    sim = api.Simulation(cfg, pa, device=0)
    r32, r64 = orc.OracleSim(cfg, pa, "f32"), orc.OracleSim(cfg, pa, "f64")
    for s in (sim, r32, r64):
        s.step(20)
    sim.sync()
    for f in ("solid_F", "solid_PK1", "solid_du_dt", "solid_vel", "solid_pos"):
        want = r64.get(f)
        e_gpu, e_f32 = nerr(sim.get(f), want), nerr(r32.get(f), want)
        print("deformed 20 steps %-12s gpu %.3g  fp32-oracle %.3g" % (f, e_gpu, e_f32))
        assert e_gpu <= TRAJ_FP32_FACTOR * e_f32 + TOL_STRESS, (f, e_gpu, e_f32)
    sim.close()
