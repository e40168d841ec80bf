"""The mixed-precision form against the FP64 oracle, and the FP64
conservation sums against sums of the fields.

The mixed form stores fluid positions as cell + FP32 offset and density as
delta = rho/rho0 - 1, gathers neighbour density/pressure as FP16 deviations
from per-cell FP32 references, compensates the density-rate sum and forms the
solid's L^-1 in FP64.  It is checked with the same per-field policy as the
FP32 form (normalised max error |gpu - fp64|_inf / |fp64|_inf)."""
import numpy as np
import pytest

from conftest import nerr, target_200_steps
from fluidsim_gb300 import api, cases
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TRAJ_FP32_FACTOR = 3.0  # every field: within 3x the FP32 oracle's error plus TOL_FLOOR
TOL_FLOOR = 5e-5


def test_mixed_field_round_trip():
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=5, precision=api.PRECISION_MIXED))
    sim = api.Simulation(cfg, pa, device=0)
    # offsets are exact to ~1e-9 m; the absolute FP32 position is recovered to 1 ulp
    assert np.abs(sim.get("fluid_pos") - pa.fluid_pos).max() <= 1e-7
    assert np.array_equal(sim.get("fluid_rho"), pa.fluid_rho)
    assert np.abs(sim.get("virt_pos") - pa.virt_pos).max() <= 1e-7
    # pressure is the EOS of the density (the generator's hydrostatic p is consistent with it)
    assert nerr(sim.get("fluid_p"), pa.fluid_p) < 1e-4
    # setting positions/density round-trips the same way
    x = sim.get("fluid_pos").copy()
    x[:, 1] += 1e-4
    sim.set("fluid_pos", x)
    assert np.abs(sim.get("fluid_pos") - x).max() <= 1e-7
    with pytest.raises(api.FsimError):
        sim.set("fluid_p", pa.fluid_p)  # pressure follows from density
    sim.phase(api.PHASE_CELL)
    # the mixed form's pair set (offsets shifted by whole cells) is the FP32
    # form's up to pairs within rounding of the impact distance
    cfg_plain = api.Config.from_buffer_copy(cfg)
    cfg_plain.precision = api.PRECISION_FP32
    with api.Simulation(cfg_plain, pa, device=0) as plain:
        plain.set("fluid_pos", x)
        plain.phase(api.PHASE_CELL)
        got, want = sim.neighbor_counts(), plain.neighbor_counts()
    assert (got[:, 0] > 0).all() and (got != want).any(axis=1).mean() < 1e-3
    sim.close()


def test_mixed_1_and_200_steps_vs_fp64():
    cfg, pa = cases.make(cases.small_dam_break(jitter=0.01, seed=11, precision=api.PRECISION_MIXED))
    cfg_plain = api.Config.from_buffer_copy(cfg)
    cfg_plain.precision = api.PRECISION_FP32
    mixed = api.Simulation(cfg, pa, device=0)
    plain = api.Simulation(cfg_plain, pa, device=0)
    r64 = orc.OracleSim(cfg_plain, pa, "f64")
    r32 = orc.OracleSim(cfg_plain, pa, "f32")
    fields = ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "solid_PK1")
    for n in (1, 199):
        for s in (mixed, plain, r64, r32):
            s.step(n)
        mixed.sync()
        plain.sync()
        for f in fields:
            want = r64.get(f)
            e_m, e_p, e_32 = nerr(mixed.get(f), want), nerr(plain.get(f), want), nerr(r32.get(f), want)
            print("after %3d more steps %-10s mixed %.3g  plain %.3g  fp32-oracle %.3g" % (n, f, e_m, e_p, e_32))
            if f.startswith("fluid") or f == "solid_pos":
                assert e_m < target_200_steps(e_32), (f, e_m, e_32)
            else:
                assert e_m <= TRAJ_FP32_FACTOR * e_32 + TOL_FLOOR, (f, e_m, e_32)
    mixed.close()
    plain.close()


def test_mixed_batch_equals_standalone():
    specs = [
        cases.tiny_box(jitter=0.01, seed=1, precision=api.PRECISION_MIXED),
        cases.tiny_box(jitter=0.02, seed=2, with_solid=False, viscid=False, fluid=(8, 6, 9),
                       precision=api.PRECISION_MIXED),
        cases.tiny_box(jitter=0.01, seed=3, fluid=(14, 12, 10), tank=(30, 18, 16), precision=api.PRECISION_MIXED),
    ]
    members = [cases.make(s) for s in specs]
    fields = ("fluid_pos", "fluid_vel", "fluid_rho", "virt_p", "solid_pos", "solid_PK1")
    alone = []
    for cfg, pa in members:
        with api.Simulation(cfg, pa, device=0) as s:
            s.step(5)
            s.sync()
            alone.append({f: s.get(f) for f in fields if not (f.startswith("solid") and s.n["solid"] == 0)})
    sims = [api.Simulation(cfg, pa, device=0) for cfg, pa in members]
    with api.Batch(sims) as b:
        b.step(5)
        b.sync()
        for k, s in enumerate(sims):
            for f, a in alone[k].items():
                assert np.array_equal(a, s.get(f)), (k, f)
    # a batch takes one precision form
    cfg, pa = cases.make(cases.tiny_box())
    plain = api.Simulation(cfg, pa, device=0)
    with pytest.raises(api.FsimError):
        api.Batch([sims[0], plain])
    for s in sims + [plain]:
        s.close()


def test_mixed_deterministic():
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=9, precision=api.PRECISION_MIXED))
    outs = []
    for _ in range(2):
        with api.Simulation(cfg, pa, device=0) as s:
            s.step(20)
            s.sync()
            outs.append((s.get("fluid_pos"), s.get("fluid_rho"), s.get("solid_pos")))
    for x, y in zip(*outs):
        assert np.array_equal(x, y)


def _numpy_conservation(sim, cfg, d):
    vol = float(d.particle_volume)
    g = np.array([0.0, -float(cfg.gravity), 0.0])
    x, u, rho = (sim.get(f).astype(np.float64) for f in ("fluid_pos", "fluid_vel", "fluid_rho"))
    mf = cfg.fluid_density * vol
    out = {"fluid_mass": mf * len(x), "momentum": mf * u.sum(0), "kinetic_energy": 0.5 * mf * (u * u).sum(),
           "potential_energy": -mf * (x @ g).sum(), "fluid_density_excess": ((rho - cfg.fluid_density) * vol).sum()}
    if sim.n["solid"]:
        ms = cfg.solid_density * vol
        xs, us = sim.get("solid_pos").astype(np.float64), sim.get("solid_vel").astype(np.float64)
        out["solid_mass"] = ms * len(xs)
        out["momentum"] = out["momentum"] + ms * us.sum(0)
        out["kinetic_energy"] += 0.5 * ms * (us * us).sum()
        out["potential_energy"] += -ms * (xs @ g).sum()
    return out


@pytest.mark.parametrize("precision", [api.PRECISION_FP32, api.PRECISION_MIXED])
def test_conservation_sums(precision):
    cfg, pa = cases.make(cases.small_dam_break(jitter=0.01, seed=3, precision=precision))
    sim = api.Simulation(cfg, pa, device=0)
    sim.step(30)
    sim.sync()
    c = sim.conservation()
    want = _numpy_conservation(sim, cfg, sim.derived())
    assert c["fluid_mass"] == pytest.approx(want["fluid_mass"], rel=1e-12)
    assert c["solid_mass"] == pytest.approx(want["solid_mass"], rel=1e-12)
    mom = np.array([c["momentum_x"], c["momentum_y"], c["momentum_z"]])
    scale = np.abs(want["momentum"]).max()
    assert np.abs(mom - want["momentum"]).max() <= 1e-6 * scale
    assert c["kinetic_energy"] == pytest.approx(want["kinetic_energy"], rel=1e-6)
    assert c["potential_energy"] == pytest.approx(want["potential_energy"], rel=1e-6)
    assert c["fluid_density_excess"] == pytest.approx(want["fluid_density_excess"], rel=1e-4)
    # the compressed column stores elastic energy; the loaded plate strain energy
    assert c["fluid_elastic_energy"] > 0.0 and c["solid_strain_energy"] > 0.0
    sim.close()
