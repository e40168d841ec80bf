"""Checks of the oracle itself, on the CPU: independent restatements of the
cell index, exact lattice neighbour counts, FP32-vs-FP64 agreement and the
antisymmetry (momentum conservation) of the fluid pair forces."""
import os

import numpy as np
import pytest

from conftest import nerr
from fluidsim_gb300 import api, cases
from oracle import oracle as orc


def test_cell_ids_match_numpy_float32():
    cfg, pa = cases.make(cases.small_dam_break(jitter=0.01, seed=1))
    d = api.derive(cfg)
    got = orc.cell_ids(d, pa.fluid_pos)
    p = pa.fluid_pos.astype(np.float32)
    cmin = np.array(d.cell_min[:], np.float32)
    inv = np.array(d.interval_inv[:], np.float32)
    idx = ((p - cmin) * inv).astype(np.int32)  # float32 ops, truncation toward zero
    n = d.cell_number
    want = idx[:, 0] * n[1] * n[2] + idx[:, 1] * n[2] + idx[:, 2]
    assert np.array_equal(got, want)


def _lattice_count(r2_over_dx2):
    k = np.arange(-4, 5)
    a, b, c = np.meshgrid(k, k, k, indexing="ij")
    return int(((a * a + b * b + c * c) < r2_over_dx2).sum())


def test_lattice_neighbor_counts():
    """On the unjittered lattice an interior fluid particle sees exactly the
    lattice points within 2h = 2.6 dx: 81 including itself."""
    cfg, pa = cases.make(cases.small_dam_break())
    o = orc.OracleSim(cfg, pa)
    o.phase(api.PHASE_CELL)
    cnt = o.neighbor_counts()
    x = pa.fluid_pos
    inner = ((x[:, 0] > 0.035) & (x[:, 0] < 0.365) & (x[:, 1] > 0.035) & (x[:, 1] < 0.165) &
             (x[:, 2] > 0.035) & (x[:, 2] < 0.365))
    assert inner.sum() > 1000
    assert _lattice_count(6.76) == 81
    assert np.all(cnt[inner, 0] == 81)
    assert np.all(cnt[inner, 1] == 0) and np.all(cnt[inner, 2] == 0)
    # a corner particle: fluid + walls fill its neighbourhood like the lattice
    corner = np.argmin(np.abs(x - 0.005).sum(1))
    assert cnt[corner, 0] + cnt[corner, 2] == 81


@pytest.mark.parametrize("phase_fields", [
    (api.PHASE_COUPLE, ["solid_normal"]),
    (api.PHASE_VIRT, ["virt_rho", "virt_p", "virt_normal"]),
    (api.PHASE_FLUID, ["fluid_drho_dt", "fluid_du_dt", "fluid_rho", "fluid_pos"]),
])
def test_fp32_oracle_agrees_with_fp64(phase_fields):
    phase, fields = phase_fields
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=2))
    a, b = orc.OracleSim(cfg, pa, "f32"), orc.OracleSim(cfg, pa, "f64")
    for ph in range(phase + 1):
        a.phase(ph)
        b.phase(ph)
    for f in fields:
        assert nerr(a.get(f), b.get(f)) < 1e-4, f


def test_fluid_pair_forces_conserve_momentum():
    """sum_i rho_i du_i/dt = 0 for fluid-fluid pairs (pressure and viscous
    terms are antisymmetric), here with random velocities to exercise the
    Riemann limiter and the viscosity."""
    cfg, case = cases.tiny_box(jitter=0.05, seed=4, with_solid=False)
    case.virt_layers = 0
    cfg.gravity = 0.0
    cfg, pa = cases.make((cfg, case))
    rng = np.random.default_rng(0)
    pa.fluid_vel[:] = rng.uniform(-0.2, 0.2, pa.fluid_vel.shape).astype(np.float32)
    rho0 = pa.fluid_rho.astype(np.float64).copy()
    o = orc.OracleSim(cfg, pa, "f64")
    o.phase(api.PHASE_CELL)
    o.phase(api.PHASE_FLUID)
    a = o.get("fluid_du_dt")
    mom = (rho0[:, None] * a).sum(0)
    scale = np.abs(rho0[:, None] * a).sum(0)
    assert np.all(np.abs(mom) <= 1e-10 * scale)
    assert np.abs(a).max() > 0


def test_oracle_deterministic_across_threads():
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=3))
    outs = []
    for t in (1, 4):
        o = orc.OracleSim(cfg, pa, "f64", threads=t)
        o.step(3)
        outs.append(o.get("fluid_pos"))
    orc.load("f64").orc_set_threads(os.cpu_count() or 1)
    assert np.array_equal(outs[0], outs[1])


def test_oracle_probe_defaults_and_rest_state():
    """At rest every velocity is 0; a point with no particle in range or
    outside the grid reads (0, 0, 0, 0, rho0); inside the column the Shepard
    density lies between the smallest and largest particle density."""
    cfg, pa = cases.make(cases.tiny_box())
    s = orc.OracleSim(cfg, pa, "f64")
    s.phase(0)
    lo, hi = pa.fluid_pos.min(0), pa.fluid_pos.max(0)
    pts = np.vstack([(lo + hi) / 2, [0.2, 0.14, 0.14], [-3.0, 0.0, 0.0]])
    out = s.probe(pts)
    assert np.all(out[:, :3] == 0)
    assert np.array_equal(out[2], [0, 0, 0, 0, cfg.fluid_density])
    assert pa.fluid_rho.min() <= out[0, 4] <= pa.fluid_rho.max()
    assert out[0, 3] > 0
