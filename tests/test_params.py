"""input.ini parsing and FP32 parameter derivation vs the reference itself.

The fixtures tests/golden/params_*.json were produced by the reference's own
host sources (src/config.cpp, src/kernel.cpp, src/properties.cpp,
src/domain.cpp, src/physics.cpp, src/sim_time.cpp) compiled unmodified
(tests/golden/make_golden.py).  Everything is compared bit for bit in FP32.
"""
import glob
import json
import os

import numpy as np
import pytest

from fluidsim_gb300 import api
from oracle import oracle as orc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = sorted(os.path.basename(p)[7:-5] for p in glob.glob(os.path.join(GOLD, "params_*.json")))

RAW_FLOAT = ["gravity", "min_pressure", "fluid_sound_speed", "fluid_density", "gamma", "viscosity",
             "solid_density", "youngs_modulus", "poisson_ratio", "arti_vis_alpha", "arti_vis_beta",
             "xmin", "ymin", "zmin", "xmax", "ymax", "zmax", "dt", "smoothing_length", "particle_diameter",
             "impact_length_hsml_ratio"]
RAW_INT = ["is_viscid", "istart", "iend", "solid_sub_step", "result_interval", "sort_every_step", "thread_num"]
DERIVED = {  # fsim_derived field -> fixture key
    "smoothing_length_square": "smoothing_length_square",
    "smoothing_length_inverse": "smoothing_length_inverse",
    "smoothing_length_inverse_square": "smoothing_length_inverse_square",
    "impact_distance_square": "impact_distance_square",
    "particle_volume": "particle_volume",
    "kernel_coefficient_1": "kernel_coefficient_1",
    "kernel_coefficient_2": "kernel_coefficient_2",
    "kernel_differential": "kernel_differential",
    "coefficient_p2rho": "coefficient_p2rho",
    "coefficient_rho2p": "coefficient_rho2p",
    "gamma_inv": "gamma_inv",
    "reference_density_inverse": "reference_density_inverse",
    "min_density": "min_density",
    "max_density": "max_density",
    "lambda_": "lambda",
    "shear_modulus": "shear_modulus",
    "bulk_modulus": "bulk_modulus",
    "solid_sound_speed": "solid_sound_speed",
}


def _load(name):
    with open(os.path.join(GOLD, "params_%s.json" % name)) as f:
        g = json.load(f)
    with open(os.path.join(GOLD, "ini", name + ".ini")) as f:
        text = f.read()
    return g, text


def _f32(v):
    return np.float32(float(v))


def test_fixtures_present():
    assert {"small_dam_break", "fsi_4m", "quirks", "defaults_only", "missing_kernel"} <= set(NAMES)


@pytest.mark.parametrize("name", NAMES)
def test_ini_matches_reference(name):
    g, text = _load(name)
    if g["read_error"]:
        with pytest.raises(api.FsimError) as e:
            api.config_from_ini_text(text)
        assert e.value.status == api.EINVAL
        assert g["messages"][0] in str(e.value)
        return
    cfg = api.config_from_ini_text(text)
    for k in RAW_FLOAT:
        assert _f32(getattr(cfg, k)) == _f32(g[k]), k
    for k in RAW_INT:
        assert getattr(cfg, k) == g[k], k


@pytest.mark.parametrize("name", [n for n in NAMES if n not in ("missing_kernel", "missing_time", "flat_domain")])
@pytest.mark.parametrize("impl", ["library", "oracle"])
def test_derivation_matches_reference_bitexact(name, impl):
    g, text = _load(name)
    cfg = api.config_from_ini_text(text)
    d = api.derive(cfg) if impl == "library" else orc.derive(cfg, api.Derived)
    for field, key in DERIVED.items():
        assert _f32(getattr(d, field)) == _f32(g[key]), field
    assert _f32(d.gravity_vec[1]) == _f32(g["gravity_vec_y"])
    for i in range(3):
        assert _f32(d.cell_min[i]) == _f32(g["cell_min_%d" % i])
        assert _f32(d.cell_max[i]) == _f32(g["cell_max_%d" % i])
        assert _f32(d.interval[i]) == _f32(g["interval_%d" % i])
        assert _f32(d.interval_inv[i]) == _f32(g["interval_inv_%d" % i])
        assert d.cell_number[i] == g["cell_number_%d" % i]
    assert d.cell_number_total == g["cell_number_total"]


def test_quirk_bool_followed_by_section_reads_true():
    """`is_viscid = false` directly followed by a `[section]` line continues the
    value ("false\\n[solid]"), which the reference's bool reader takes as true."""
    g, text = _load("quirks")
    assert g["is_viscid"] == 1
    assert api.config_from_ini_text(text).is_viscid == 1


def test_defaults_are_the_reference_defaults():
    g, text = _load("defaults_only")
    cfg = api.config_from_ini_text(text)
    dflt = api.default_config()
    for k in RAW_FLOAT + RAW_INT:
        if k not in text:
            assert _f32(getattr(dflt, k)) == _f32(g[k]), k
            assert _f32(getattr(cfg, k)) == _f32(g[k]), k


def test_ini_from_file_equals_text(tmp_path):
    g, text = _load("small_dam_break")
    p = tmp_path / "input.ini"
    p.write_text(text)
    a, b = api.config_from_ini(str(p)), api.config_from_ini_text(text)
    assert a.as_dict() == b.as_dict()
    with pytest.raises(api.FsimError) as e:
        api.config_from_ini(str(tmp_path / "missing.ini"))
    assert e.value.status == api.EIO


def test_extension_keys_ignored_by_reference_semantics():
    g, text = _load("small_dam_break")
    cfg = api.config_from_ini_text(text + "\n[gb300]\ngb300_precision = mixed\ngb300_keep_derivatives = yes\n")
    assert cfg.precision == api.PRECISION_MIXED and cfg.keep_derivatives == 1
    cfg = api.config_from_ini_text(text + "\n[gb300]\ngb300_solid_fused = yes\n")
    assert cfg.solid_fused == 1 and cfg.precision == api.PRECISION_FP32
    assert api.config_from_ini_text(text).solid_full_walk == 0
    walk = api.config_from_ini_text(text + "\n[gb300]\ngb300_solid_full_walk = yes\n")
    assert walk.solid_full_walk == 1 and walk.solid_fused == 0
    base = api.config_from_ini_text(text)
    for k in RAW_FLOAT + RAW_INT:
        assert getattr(cfg, k) == getattr(base, k)
