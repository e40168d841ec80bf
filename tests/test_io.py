""".dat particle files and the case generator (CPU only)."""
import glob
import json
import os

import numpy as np
import pytest

from fluidsim_gb300 import api, cases

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "counts_*.json"))))
def test_count_reader_matches_reference(path, tmp_path):
    """Counts and the count/row mismatch error as the reference's readers
    report them (fixtures from {Fluid,Solid,Virtual}Properties::readNumber)."""
    with open(path) as f:
        g = json.load(f)
    for fn, text in g["files"].items():
        (tmp_path / fn).write_text(text)
    if g["count_error"]:
        with pytest.raises(api.FsimError) as e:
            api.read_dat(str(tmp_path))
        assert e.value.status == api.EINVAL
        assert "mismatch" in str(e.value)
    else:
        pa = api.read_dat(str(tmp_path))
        assert (pa.n_fluid, pa.n_solid, pa.n_virt) == (g["n_fluid"], g["n_solid"], g["n_virt"])


def test_dat_round_trip(tmp_path):
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=5))
    pa.write_dat(str(tmp_path))
    pb = api.read_dat(str(tmp_path))
    for k in ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "solid_ref_pos",
              "solid_type", "virt_pos", "virt_type"):
        assert np.array_equal(getattr(pa, k), getattr(pb, k)), k


def test_dat_row_layout(tmp_path):
    (tmp_path / "fluid_particle.dat").write_text("1\n1 2 3 4 5 6 7 8\n")
    (tmp_path / "solid_particle.dat").write_text("1\n1 2 3 4 5 6 7 8 9 1\n")
    (tmp_path / "virt_particle.dat").write_text("1\n-1 -2 -3 0\n")
    pa = api.read_dat(str(tmp_path))
    assert pa.fluid_pos.tolist() == [[1, 2, 3]] and pa.fluid_vel.tolist() == [[4, 5, 6]]
    assert pa.fluid_rho.tolist() == [7] and pa.fluid_p.tolist() == [8]
    assert pa.solid_pos.tolist() == [[1, 2, 3]] and pa.solid_vel.tolist() == [[4, 5, 6]]
    assert pa.solid_ref_pos.tolist() == [[7, 8, 9]] and pa.solid_type.tolist() == [1]
    assert pa.virt_pos.tolist() == [[-1, -2, -3]]


def test_dat_errors(tmp_path):
    with pytest.raises(api.FsimError) as e:
        api.read_dat(str(tmp_path / "nowhere"))
    assert e.value.status == api.EIO
    (tmp_path / "fluid_particle.dat").write_text("1\n1 2 x 4 5 6 7 8\n")
    (tmp_path / "solid_particle.dat").write_text("0\n")
    (tmp_path / "virt_particle.dat").write_text("0\n")
    with pytest.raises(api.FsimError) as e:
        api.read_dat(str(tmp_path))
    assert e.value.status == api.EINVAL


def test_small_dam_break_counts():
    cfg, pa = cases.make(cases.small_dam_break())
    assert pa.n_fluid == 40 * 20 * 40
    assert pa.n_solid == 4 * 20 * 40 + 4 * 3 * 40
    assert int((pa.solid_type == 1).sum()) == 480
    # closed tank 160x40x80 with 3 wall layers, minus the 480 plate cells in the floor
    assert pa.n_virt == 166 * 46 * 86 - 160 * 40 * 80 - 480
    # FIXED plate particles are exactly the ones below the floor
    assert np.array_equal(pa.solid_type == 1, pa.solid_pos[:, 1] < 0)
    assert np.array_equal(pa.solid_pos, pa.solid_ref_pos)


def test_fsi_4m_counts():
    cfg, pa = cases.make(cases.fsi_4m())
    assert (pa.n_fluid, pa.n_solid, pa.n_virt) == (4194304, 27000, 912600)
    d = api.derive(cfg)
    assert tuple(d.cell_number) == (203, 55, 55)


def test_hydrostatic_start():
    cfg, pa = cases.make(cases.small_dam_break())
    H = 20 * 0.01
    p = 1000.0 * 9.81 * (H - pa.fluid_pos[:, 1].astype(np.float64))
    assert np.allclose(pa.fluid_p, p, rtol=1e-6, atol=1e-3)
    rho = 1000.0 * (p * 7.0 / (1000.0 * 30.0 ** 2) + 1.0) ** (1.0 / 7.0)
    assert np.allclose(pa.fluid_rho, rho, rtol=1e-7)


def test_jitter_bounded_and_seeded():
    _, a = cases.make(cases.tiny_box(jitter=0.01, seed=9))
    _, b = cases.make(cases.tiny_box(jitter=0.01, seed=9))
    _, c = cases.make(cases.tiny_box(jitter=0.01, seed=10))
    _, z = cases.make(cases.tiny_box())
    assert np.array_equal(a.fluid_pos, b.fluid_pos)
    assert not np.array_equal(a.fluid_pos, c.fluid_pos)
    assert np.abs(a.fluid_pos - z.fluid_pos).max() <= 0.01 * 0.01 * 1.0001
    assert np.array_equal(a.virt_pos, z.virt_pos)  # walls are not jittered


@pytest.mark.parametrize("spec", [
    cases.tiny_box(), cases.tiny_box(with_solid=False), cases.small_dam_break(),
    cases.tiny_box(fluid=(30, 20, 30)),  # fluid block larger than the tank: clipped
])
def test_case_counts_match_host_generator(spec):
    """The per-row interval logic of the device generator counts the same
    particles as the host generator's site loop."""
    cfg, case = spec
    _, pa = cases.make(spec)
    assert api.case_counts(case) == (pa.n_fluid, pa.n_solid, pa.n_virt)


def test_case_counts_with_solid_below_the_floor_and_outside():
    """Fixed layers below the floor, and a solid block reaching out of the tank."""
    cfg, case = cases.tiny_box()
    case.solid_fixed_layers = 3
    case.solid_lo[2] = -2
    case.solid_n[2] = 30
    _, pa = cases.make((cfg, case))
    assert api.case_counts(case) == (pa.n_fluid, pa.n_solid, pa.n_virt)
