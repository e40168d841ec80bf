"""ctypes loader of the reference build (test infrastructure only).

The reference build is the reference's own CUDA kernels (src/pair.cu,
src/fluid.cu, src/virt.cu, src/solid.cu, unmodified; compiled by
oracle/build.py into ``_ref/refcuda_{release,precise}.fatbin``) driven by the
host program refcuda/ref_harness.cpp, which restates the reference's
initialisation and step loop (src/sim.cu:153-302, src/calculation.cu:20-35).
Only tests/ and bench.py's reference arm use it: it is the checker the CUDA
path is compared with and the reference throughput it is measured beside.

Fields come back in input order (the reference never reorders particles):
float32 arrays, (n, 3) for vectors and (n, 9) row-major for matrices (as the
library's fields),
int32 for cell ids.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

FIELD_IDS = {
    "fluid_pos": 0, "fluid_vel": 1, "fluid_rho": 2, "fluid_p": 3, "fluid_drho_dt": 4, "fluid_du_dt": 5,
    "fluid_cell_id": 6,
    "solid_pos": 10, "solid_vel": 11, "solid_ref_pos": 12, "solid_type": 13, "solid_normal": 14, "solid_p": 15,
    "solid_du_dt": 16, "solid_couple_dudt": 17, "solid_F": 18, "solid_PK1": 19, "solid_Linv": 20,
    "solid_cell_id": 21,
    "virt_pos": 30, "virt_normal": 31, "virt_vel": 32, "virt_p": 33, "virt_rho": 34, "virt_cell_id": 35,
    "fluid_color": 40,
}
WIDTH = {0: 3, 1: 3, 5: 3, 10: 3, 11: 3, 12: 3, 14: 3, 16: 3, 17: 3, 18: 9, 19: 9, 20: 9, 30: 3, 31: 3, 32: 3}
INT_FIELDS = {6, 13, 21, 35}
SPECIES = {"fluid": 0, "solid": 1, "virt": 2}

_lib = None


def image_path(variant="release"):
    return _build.refcuda_image_path(variant)


def available(variant="release"):
    """True when the device image and the harness library both exist."""
    return os.path.exists(image_path(variant)) and os.path.exists(_build.harness_lib_path())


def load():
    global _lib
    if _lib is not None:
        return _lib
    path = _build.harness_lib_path()
    if not os.path.exists(path):
        _build.build_harness()
    lib = C.CDLL(path)
    V, I = C.c_void_p, C.c_int
    lib.ref_last_error.restype = C.c_char_p
    lib.ref_layout.argtypes = [V, I]
    lib.ref_layout.restype = I
    lib.ref_create.argtypes = [C.c_char_p, V, V, V, I, C.POINTER(V)]
    lib.ref_create.restype = I
    lib.ref_destroy.argtypes = [V]
    lib.ref_phase.argtypes = [V, I]
    lib.ref_phase.restype = I
    lib.ref_step.argtypes = [V, I]
    lib.ref_step.restype = I
    lib.ref_time_steps.argtypes = [V, I, C.POINTER(C.c_float)]
    lib.ref_time_steps.restype = I
    lib.ref_get.argtypes = [V, I, V]
    lib.ref_get.restype = I
    lib.ref_list_cells.argtypes = [V, I, V]
    lib.ref_list_cells.restype = I
    _lib = lib
    return lib


def layout():
    """Byte offsets of the harness's mirror of the reference's structs."""
    a = (C.c_longlong * 64)()
    n = load().ref_layout(a, 64)
    return list(a[:n])


class RefBuildError(RuntimeError):
    pass


class RefBuildSim:
    """One run of the reference build on the current CUDA device."""

    def __init__(self, cfg, particles, variant="release", device=0):
        from fluidsim_gb300 import api

        self.lib = load()
        path = image_path(variant)
        if not os.path.exists(path):
            raise RefBuildError("reference device image %s is missing" % path)
        pa = particles
        self.n = {"fluid": pa.n_fluid, "solid": pa.n_solid, "virt": pa.n_virt}
        self._derived = api.derive(cfg)
        self._particles = pa
        self._view = pa.struct()
        self.h = C.c_void_p()
        rc = self.lib.ref_create(path.encode(), C.addressof(cfg), C.addressof(self._derived), C.addressof(self._view),
                                 device, C.byref(self.h))
        if rc:
            msg = self.lib.ref_last_error().decode()
            self.close()
            raise RefBuildError("ref_create: " + msg)

    def _check(self, rc, what):
        if rc:
            raise RefBuildError("%s: %s" % (what, self.lib.ref_last_error().decode()))

    def close(self):
        if self.h:
            self.lib.ref_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def phase(self, p):
        self._check(self.lib.ref_phase(self.h, p), "ref_phase")

    def step(self, n=1):
        self._check(self.lib.ref_step(self.h, n), "ref_step")

    def time_steps(self, n):
        ms = C.c_float()
        self._check(self.lib.ref_time_steps(self.h, n, C.byref(ms)), "ref_time_steps")
        return ms.value

    def get(self, name):
        fid = FIELD_IDS[name]
        w = WIDTH.get(fid, 1)
        n = self.n["fluid"] if fid < 10 or fid == 40 else self.n["solid"] if fid < 30 else self.n["virt"]
        out = np.empty(n * w, np.int32 if fid in INT_FIELDS else np.float32)
        if n:
            self._check(self.lib.ref_get(self.h, fid, out.ctypes.data), "ref_get")
        return out.reshape(n, w) if w > 1 else out

    def list_cells(self, species):
        """Cell whose linked list holds each particle (-1 none, -2 several)."""
        n = self.n[species]
        out = np.empty(n, np.int32)
        if n:
            self._check(self.lib.ref_list_cells(self.h, SPECIES[species], out.ctypes.data), "ref_list_cells")
        return out
