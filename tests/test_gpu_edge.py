"""Edge cases of the CUDA path: empty and one-species instances, a single
particle, positions exactly on cell boundaries, and an input the cell hash
flags (a particle outside the grid).  Compared with the FP64 oracle where
there is something to compare."""
import numpy as np
import pytest

from conftest import nerr
from fluidsim_gb300 import api, cases
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

E3 = np.zeros((0, 3), np.float32)
E1 = np.zeros(0, np.float32)


def _split(pa, fluid=True, solid=True, virt=True):
    """A copy of a particle set keeping only the chosen species."""
    return api.ParticleArrays(
        pa.fluid_pos if fluid else E3, pa.fluid_vel if fluid else E3, pa.fluid_rho if fluid else E1,
        pa.fluid_p if fluid else E1, pa.solid_pos if solid else E3, pa.solid_vel if solid else E3,
        pa.solid_ref_pos if solid else E3, pa.solid_type if solid else np.zeros(0, np.int32),
        pa.virt_pos if virt else E3)


FORMS = [api.PRECISION_FP32, api.PRECISION_MIXED]


def _vs_oracle(cfg, pa, steps, fields, tol=2e-4):
    """The parity policy of the main tests: err(gpu, fp64) <= 2 err(fp32 oracle, fp64) + tol
    (the oracles restate the plain method; a mixed-form instance is held to it too)."""
    sim = api.Simulation(cfg, pa, device=0)
    plain = api.Config.from_buffer_copy(cfg)
    plain.precision = api.PRECISION_FP32
    ref = orc.OracleSim(plain, pa, "f64")
    r32 = orc.OracleSim(plain, pa, "f32")
    for s in (sim, ref, r32):
        s.step(steps)
    sim.sync()
    for f in fields:
        want = ref.get(f)
        e, e32 = nerr(sim.get(f), want), nerr(r32.get(f), want)
        assert e <= 2.0 * e32 + tol, (f, e, e32)
    sim.close()


@pytest.mark.parametrize("precision", FORMS)
def test_empty_instance(precision):
    cfg, _ = cases.tiny_box(precision=precision)
    pa = api.ParticleArrays(E3, E3, E1, E1, E3, E3, E3, np.zeros(0, np.int32), E3)
    with api.Simulation(cfg, pa, device=0) as sim:
        assert sim.n == {"fluid": 0, "solid": 0, "virt": 0}
        sim.step(3)
        sim.sync()
        assert sim.get("fluid_pos").shape == (0, 3)
        c = sim.conservation()
        assert all(v == 0.0 for v in c.values())


@pytest.mark.parametrize("precision", FORMS)
def test_fluid_only_no_walls(precision):
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=2, precision=precision))
    _vs_oracle(cfg, _split(pa, solid=False, virt=False), 3, ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p"))


@pytest.mark.parametrize("precision", FORMS)
def test_solid_and_walls_without_fluid(precision):
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=3, precision=precision))
    _vs_oracle(cfg, _split(pa, fluid=False), 3, ("solid_pos",), tol=1e-5)


def test_single_fluid_particle_falls_freely():
    cfg, _ = cases.tiny_box()
    pa = api.ParticleArrays([[0.1, 0.1, 0.08]], [[0, 0, 0]], [cfg.fluid_density], [0.0], E3, E3, E3,
                            np.zeros(0, np.int32), E3)
    with api.Simulation(cfg, pa, device=0) as sim:
        sim.step(10)
        sim.sync()
        v = sim.get("fluid_vel")[0]
        assert v[0] == 0 and v[2] == 0
        assert v[1] == pytest.approx(-cfg.gravity * cfg.dt * 10, rel=1e-5)
        assert sim.get("fluid_rho")[0] == pytest.approx(cfg.fluid_density, rel=1e-6)


def test_positions_on_cell_boundaries_bitexact_cells():
    """Particles placed exactly on the FP32 cell boundaries (cell_min + k *
    interval, and one ulp either side): cell ids and membership match the
    oracle's FP32 cell index bit for bit."""
    cfg, pa = cases.make(cases.tiny_box())
    d = api.derive(cfg)
    rng = np.random.default_rng(0)
    pts = []
    for _ in range(300):
        p = []
        for a in range(3):
            k = rng.integers(1, d.cell_number[a] - 1)
            edge = np.float32(d.cell_min[a]) + np.float32(k) * np.float32(d.interval[a])
            p.append(np.nextafter(edge, np.float32(rng.choice([-1e9, 1e9]))) if rng.random() < 0.5 else edge)
        pts.append(p)
    pts = np.asarray(pts, np.float32)
    fl = api.ParticleArrays(pts, np.zeros_like(pts), np.full(len(pts), cfg.fluid_density, np.float32),
                            np.zeros(len(pts), np.float32), E3, E3, E3, np.zeros(0, np.int32), pa.virt_pos)
    with api.Simulation(cfg, fl, device=0) as sim:
        sim.phase(api.PHASE_CELL)
        assert np.array_equal(sim.get("fluid_cell_id"), orc.cell_ids(sim.derived(), pts))
        ref = orc.OracleSim(cfg, fl, "f64")
        ref.phase(api.PHASE_CELL)
        assert np.array_equal(sim.neighbor_counts(), ref.neighbor_counts())


def test_particle_outside_the_grid_is_reported():
    cfg, pa = cases.make(cases.tiny_box())
    pos = pa.fluid_pos.copy()
    pos[5] = [40.0, -3.0, 7.0]
    bad = api.ParticleArrays(pos, pa.fluid_vel, pa.fluid_rho, pa.fluid_p, pa.solid_pos, pa.solid_vel,
                             pa.solid_ref_pos, pa.solid_type, pa.virt_pos)
    with api.Simulation(cfg, bad, device=0) as sim:
        sim.step(1)
        with pytest.raises(api.FsimError) as ei:
            sim.sync()
        assert ei.value.status == api.ENUMERIC
        sim.step(1)  # clamped into the domain by the update: the next step is clean
        sim.sync()
