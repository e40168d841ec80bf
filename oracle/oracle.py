"""ctypes loader of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
use this module, as the checker the CUDA path is compared against.  It restates
the reference algorithm (see oracle.c for the file:line of every phase).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

FIELD_WIDTH = {0: 3, 1: 3, 2: 1, 3: 1, 4: 1, 5: 3, 6: 1,
               10: 3, 11: 3, 12: 3, 13: 1, 14: 3, 15: 1, 16: 3, 17: 3, 18: 9, 19: 9, 20: 9, 21: 1,
               30: 3, 31: 3, 32: 3, 33: 1, 34: 1, 35: 1}
FIELD_IDS = {
    "fluid_pos": 0, "fluid_vel": 1, "fluid_rho": 2, "fluid_p": 3, "fluid_drho_dt": 4, "fluid_du_dt": 5,
    "fluid_cell_id": 6,
    "solid_pos": 10, "solid_vel": 11, "solid_ref_pos": 12, "solid_type": 13, "solid_normal": 14, "solid_p": 15,
    "solid_du_dt": 16, "solid_couple_dudt": 17, "solid_F": 18, "solid_PK1": 19, "solid_Linv": 20,
    "solid_cell_id": 21,
    "virt_pos": 30, "virt_normal": 31, "virt_vel": 32, "virt_p": 33, "virt_rho": 34, "virt_cell_id": 35,
}

_libs = {}


def load(precision="f64"):
    if precision in _libs:
        return _libs[precision]
    path = _build.oracle_lib_path(precision)
    if not os.path.exists(path):
        _build.build_oracle()
    lib = C.CDLL(path)
    V, I, P = C.c_void_p, C.c_int, C.c_void_p
    lib.orc_derive.argtypes = [V, V]
    lib.orc_derive.restype = None
    lib.orc_cell_of.argtypes = [V, C.c_float, C.c_float, C.c_float]
    lib.orc_cell_of.restype = I
    lib.orc_cell_ids.argtypes = [V, I, P, P]
    lib.orc_cell_ids.restype = None
    lib.orc_create.argtypes = [V, I, P, P, P, P, I, P, P, P, P, I, P]
    lib.orc_create.restype = V
    lib.orc_destroy.argtypes = [V]
    lib.orc_phase.argtypes = [V, I]
    lib.orc_step.argtypes = [V, I]
    lib.orc_get.argtypes = [V, I, P]
    lib.orc_get.restype = I
    lib.orc_set.argtypes = [V, I, P]
    lib.orc_set.restype = I
    lib.orc_neighbor_counts.argtypes = [V, P]
    lib.orc_probe.argtypes = [V, I, P, P]
    lib.orc_set_threads.argtypes = [I]
    lib.orc_real_bytes.restype = I
    _libs[precision] = lib
    return lib


def derive(cfg, derived_struct_type, precision="f64"):
    """Oracle's FP32 derivation into a structure laid out like fsim_derived."""
    d = derived_struct_type()
    load(precision).orc_derive(C.addressof(cfg), C.addressof(d))
    return d


def cell_ids(derived, pos, precision="f64"):
    """FP32 cell index of every position (src/pair.cu:8-24)."""
    p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    out = np.empty(len(p), np.int32)
    if len(p):
        load(precision).orc_cell_ids(C.addressof(derived), len(p), p.ctypes.data, out.ctypes.data)
    return out


class OracleSim:
    """The oracle simulation of one instance; fields come back as float64 arrays in input order."""

    def __init__(self, cfg, particles, precision="f64", threads=0):
        self.lib = load(precision)
        if threads:
            self.lib.orc_set_threads(threads)
        pa = particles
        self._keep = pa  # arrays must outlive the create call only, but keep them for clarity
        self.n = {"fluid": pa.n_fluid, "solid": pa.n_solid, "virt": pa.n_virt}
        ptr = lambda a: a.ctypes.data if a.size else None
        self.s = self.lib.orc_create(C.addressof(cfg), pa.n_fluid, ptr(pa.fluid_pos), ptr(pa.fluid_vel),
                                     ptr(pa.fluid_rho), ptr(pa.fluid_p), pa.n_solid, ptr(pa.solid_pos),
                                     ptr(pa.solid_vel), ptr(pa.solid_ref_pos), ptr(pa.solid_type), pa.n_virt,
                                     ptr(pa.virt_pos))

    def close(self):
        if self.s:
            self.lib.orc_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def phase(self, p):
        self.lib.orc_phase(self.s, p)

    def step(self, n=1):
        self.lib.orc_step(self.s, n)

    def get(self, name):
        fid = FIELD_IDS[name]
        w = FIELD_WIDTH[fid]
        n = self.n["fluid"] if fid < 10 else self.n["solid"] if fid < 30 else self.n["virt"]
        out = np.empty(n * w, np.float64)
        if n:
            self.lib.orc_get(self.s, fid, out.ctypes.data)
        return out.reshape(n, w) if w > 1 else out

    def set(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        if self.lib.orc_set(self.s, FIELD_IDS[name], a.ctypes.data):
            raise ValueError("field %s not settable" % name)

    def probe(self, points):
        """(n, 5) array: Shepard-averaged u, v, w, p, rho at each point."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        out = np.empty((len(pts), 5), np.float64)
        if len(pts):
            self.lib.orc_probe(self.s, len(pts), pts.ctypes.data, out.ctypes.data)
        return out

    def neighbor_counts(self):
        out = np.empty((self.n["fluid"], 3), np.int32)
        if self.n["fluid"]:
            self.lib.orc_neighbor_counts(self.s, out.ctypes.data)
        return out
