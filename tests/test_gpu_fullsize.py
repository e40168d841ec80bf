"""The CUDA path at the full size of the 4M FSI case (4,194,304 fluid +
27,000 solid + 912,600 wall particles, +-0.01 dx jitter), through checks that
do not grow with the size: bit-exact cell ids, cell membership and neighbour
counts against the oracle, one and 20 steps against the FP64 oracle,
repeatability and exact mass conservation."""
import os

import numpy as np
import pytest

from conftest import TARGET_FP32_FACTOR, nerr
from fluidsim_gb300 import api, cases
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def big():
    return cases.make(cases.fsi_4m_jitter(precision=api.PRECISION_FP32))


def test_full_size_cells_membership_and_counts_bitexact(big):
    cfg, pa = big
    sim = api.Simulation(cfg, pa, device=0)
    sim.phase(api.PHASE_CELL)
    d = sim.derived()
    for k, (name, pos) in enumerate((("fluid", pa.fluid_pos), ("solid", pa.solid_pos), ("virt", pa.virt_pos))):
        want = orc.cell_ids(d, pos)
        assert np.array_equal(sim.get(name + "_cell_id"), want), name
        start, ids = sim.cells(k)
        counts = np.bincount(want, minlength=d.cell_number_total)
        assert np.array_equal(np.diff(start), counts), name
        assert np.array_equal(want[ids], np.repeat(np.arange(d.cell_number_total), counts)), name
    ref = orc.OracleSim(cfg, pa, "f64", threads=THREADS)
    ref.phase(api.PHASE_CELL)
    got, want = sim.neighbor_counts(), ref.neighbor_counts()
    assert np.array_equal(got, want)
    assert 60 < want[:, 0].mean() < 100  # ~81 in-range fluid neighbours on the lattice
    sim.close()
    ref.close()


def test_full_size_1_and_20_steps_vs_fp64(big):
    """After one full step fluid fields are within 1e-4 (normalised max
    error); after 20 steps within 1e-3 (or 1.5x the FP32 oracle's error where
    that is larger).  Every field stays within 2x (one
    step) or 3x (20 steps) the FP32 restatement's own error plus 5e-5."""
    cfg, pa = big
    sim = api.Simulation(cfg, pa, device=0)
    r64 = orc.OracleSim(cfg, pa, "f64", threads=THREADS)
    r32 = orc.OracleSim(cfg, pa, "f32", threads=THREADS)
    for n, tol, factor in ((1, 1e-4, 2.0), (19, 1e-3, 3.0)):
        sim.step(n)
        r64.step(n)
        r32.step(n)
        sim.sync()
        for f in ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "virt_p"):
            want = r64.get(f)
            e_gpu, e_32 = nerr(sim.get(f), want), nerr(r32.get(f), want)
            print("after %2d more steps %-10s gpu %.3g  fp32-oracle %.3g" % (n, f, e_gpu, e_32))
            if f.startswith("fluid") or f in ("solid_pos", "virt_p"):
                assert e_gpu < max(tol, TARGET_FP32_FACTOR * e_32), (f, e_gpu, e_32)
            assert e_gpu <= factor * e_32 + 5e-5, (f, e_gpu, e_32)
    sim.close()


def test_full_size_repeatable_and_mass_exact(big):
    cfg, pa = big
    outs = []
    for _ in range(2):
        with api.Simulation(cfg, pa, device=0) as s:
            c0 = s.conservation()
            s.step(5)
            s.sync()
            c1 = s.conservation()
            outs.append((s.get("fluid_pos"), s.get("fluid_vel"), s.get("fluid_rho"), s.get("solid_pos"),
                         c1["momentum_x"], c1["kinetic_energy"]))
            assert c1["fluid_mass"] == c0["fluid_mass"] and c1["solid_mass"] == c0["solid_mass"]
    for x, y in zip(*outs):
        assert np.array_equal(x, y)
