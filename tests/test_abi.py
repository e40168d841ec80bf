"""The C ABI library loads and exports every entry point include/*.h declares.

CPU only: no call here reaches a GPU (argument checks fail before any CUDA
call)."""
import ctypes as C
import glob
import os
import re

import pytest

from fluidsim_gb300 import api, cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(fsim_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported():
    lib = api.load()
    decl = declared_functions()
    assert len(decl) >= 25
    for name in sorted(decl):
        assert hasattr(lib, name), name
    assert set(api.EXPORTED) <= decl


def test_library_is_the_in_tree_build():
    assert os.path.exists(api.LIB_PATH)
    assert api.LIB_PATH.startswith(os.path.join(ROOT, "fluidsim_gb300"))


def test_status_strings():
    lib = api.load()
    assert lib.fsim_status_string(api.OK) == b"FSIM_OK"
    assert lib.fsim_status_string(api.ETIMEOUT) == b"FSIM_ETIMEOUT"
    assert lib.fsim_status_string(99) == b"FSIM_UNKNOWN"


def test_field_widths():
    lib = api.load()
    widths = {"fluid_pos": 3, "fluid_rho": 1, "solid_F": 9, "solid_PK1": 9, "virt_normal": 3, "solid_cell_id": 1}
    for k, w in widths.items():
        assert lib.fsim_field_width(api.FIELDS[k]) == w
    assert lib.fsim_field_width(999) == 0


def test_create_rejects_bad_arguments_before_touching_a_gpu():
    lib = api.load()
    cfg, pa = cases.make(cases.tiny_box())
    h = C.c_void_p()
    p = pa.struct()
    p.n_fluid = -1
    assert lib.fsim_create(C.byref(cfg), C.byref(p), 0, C.byref(h)) == api.EINVAL
    assert not h.value
    p = pa.struct()
    cfg2 = api.Config.from_buffer_copy(cfg)
    cfg2.solid_sub_step = 0
    assert lib.fsim_create(C.byref(cfg2), C.byref(p), 0, C.byref(h)) == api.EINVAL
    assert lib.fsim_create(None, C.byref(p), 0, C.byref(h)) == api.EINVAL
    assert lib.fsim_step(None, 1) == api.EINVAL
    assert lib.fsim_destroy(None) == api.OK


def test_derive_rejects_degenerate_kernel():
    cfg = api.default_config()
    with pytest.raises(api.FsimError):
        api.derive(cfg)  # smoothing_length = 0


def test_snapshot_header_is_checked_before_any_device_work():
    """Garbage and short inputs are rejected as FSIM_EIO without a GPU."""
    lib = api.load()
    h, step = C.c_void_p(), C.c_longlong()
    for data in (b"", b"FSIMSNP1", b"x" * 4096):
        buf = C.create_string_buffer(data, len(data) or 1)
        assert lib.fsim_snapshot_load(buf, len(data), 0, C.byref(h), C.byref(step)) == api.EIO
        assert not h.value
