"""ctypes binding of the C ABI in include/fluidsim.h.

This is the Python face of the library: tests and bench.py drive the CUDA path
through exactly the entry points a C, C++ or FFI caller would use.  There is no
fallback: if ``_build/libfluidsim.so`` is missing, loading raises.
"""
import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libfluidsim.so")

# status codes
OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, ENUMERIC, EIO = range(7)
PRECISION_FP32, PRECISION_MIXED = 0, 1
CONSERVATION_N = 10
CONSERVATION_KEYS = ("fluid_mass", "solid_mass", "momentum_x", "momentum_y", "momentum_z", "kinetic_energy",
                     "potential_energy", "fluid_elastic_energy", "fluid_density_excess", "solid_strain_energy")
PHASE_CELL, PHASE_COUPLE, PHASE_VIRT, PHASE_FLUID, PHASE_SOLID = range(5)

FIELDS = {
    "fluid_pos": 0, "fluid_vel": 1, "fluid_rho": 2, "fluid_p": 3, "fluid_drho_dt": 4, "fluid_du_dt": 5,
    "fluid_cell_id": 6,
    "solid_pos": 10, "solid_vel": 11, "solid_ref_pos": 12, "solid_type": 13, "solid_normal": 14, "solid_p": 15,
    "solid_du_dt": 16, "solid_couple_dudt": 17, "solid_F": 18, "solid_PK1": 19, "solid_Linv": 20,
    "solid_cell_id": 21,
    "virt_pos": 30, "virt_normal": 31, "virt_vel": 32, "virt_p": 33, "virt_rho": 34, "virt_cell_id": 35,
}
INT_FIELDS = {"fluid_cell_id", "solid_cell_id", "virt_cell_id", "solid_type"}


class Config(C.Structure):
    _fields_ = [
        ("gravity", C.c_float),
        ("is_viscid", C.c_int),
        ("min_pressure", C.c_float), ("fluid_sound_speed", C.c_float), ("fluid_density", C.c_float),
        ("gamma", C.c_float), ("viscosity", C.c_float),
        ("solid_density", C.c_float), ("youngs_modulus", C.c_float), ("poisson_ratio", C.c_float),
        ("arti_vis_alpha", C.c_float), ("arti_vis_beta", C.c_float),
        ("xmin", C.c_float), ("ymin", C.c_float), ("zmin", C.c_float),
        ("xmax", C.c_float), ("ymax", C.c_float), ("zmax", C.c_float),
        ("dt", C.c_float),
        ("istart", C.c_int), ("iend", C.c_int), ("solid_sub_step", C.c_int), ("result_interval", C.c_int),
        ("sort_every_step", C.c_int),
        ("smoothing_length", C.c_float), ("particle_diameter", C.c_float),
        ("impact_length_hsml_ratio", C.c_float),
        ("thread_num", C.c_int),
        ("precision", C.c_int),
        ("keep_derivatives", C.c_int),
        ("solid_fused", C.c_int),
        ("solid_full_walk", C.c_int),
        ("barrier_wait_polls", C.c_int),
        ("neighbor_skin", C.c_float),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Derived(C.Structure):
    _fields_ = [
        ("smoothing_length_square", C.c_float), ("smoothing_length_inverse", C.c_float),
        ("smoothing_length_inverse_square", C.c_float),
        ("impact_distance_square", C.c_float), ("particle_volume", C.c_float),
        ("kernel_coefficient_1", C.c_float), ("kernel_coefficient_2", C.c_float),
        ("kernel_differential", C.c_float),
        ("coefficient_p2rho", C.c_float), ("coefficient_rho2p", C.c_float), ("gamma_inv", C.c_float),
        ("reference_density_inverse", C.c_float),
        ("min_density", C.c_float), ("max_density", C.c_float),
        ("lambda_", C.c_float), ("shear_modulus", C.c_float), ("bulk_modulus", C.c_float),
        ("solid_sound_speed", C.c_float),
        ("gravity_vec", C.c_float * 3),
        ("cell_min", C.c_float * 3), ("cell_max", C.c_float * 3), ("interval", C.c_float * 3),
        ("interval_inv", C.c_float * 3),
        ("cell_number", C.c_int * 3),
        ("cell_number_total", C.c_int),
    ]


class Particles(C.Structure):
    _fields_ = [
        ("n_fluid", C.c_int),
        ("fluid_pos", C.POINTER(C.c_float)), ("fluid_vel", C.POINTER(C.c_float)),
        ("fluid_rho", C.POINTER(C.c_float)), ("fluid_p", C.POINTER(C.c_float)),
        ("n_solid", C.c_int),
        ("solid_pos", C.POINTER(C.c_float)), ("solid_vel", C.POINTER(C.c_float)),
        ("solid_ref_pos", C.POINTER(C.c_float)), ("solid_type", C.POINTER(C.c_int)),
        ("n_virt", C.c_int),
        ("virt_pos", C.POINTER(C.c_float)), ("virt_type", C.POINTER(C.c_int)),
    ]


class Case(C.Structure):
    _fields_ = [
        ("dx", C.c_float),
        ("tank_n", C.c_int * 3),
        ("fluid_n", C.c_int * 3),
        ("solid_lo", C.c_int * 3),
        ("solid_n", C.c_int * 3),
        ("solid_fixed_layers", C.c_int),
        ("virt_layers", C.c_int),
        ("hydrostatic", C.c_int),
        ("jitter", C.c_float),
        ("seed", C.c_uint64),
    ]


_lib = None


def load():
    """Load libfluidsim.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("native library %s is missing: run `python -c \"import __graft_entry__ as g; g.build()\"`"
                           % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    sig = {
        "fsim_status_string": (C.c_char_p, [C.c_int]),
        "fsim_last_error": (C.c_char_p, []),
        "fsim_config_defaults": (C.c_int, [C.POINTER(Config)]),
        "fsim_config_from_ini": (C.c_int, [C.c_char_p, C.POINTER(Config)]),
        "fsim_config_from_ini_text": (C.c_int, [C.c_char_p, C.POINTER(Config)]),
        "fsim_derive": (C.c_int, [C.POINTER(Config), C.POINTER(Derived)]),
        "fsim_particles_read": (C.c_int, [C.c_char_p, C.POINTER(P)]),
        "fsim_particles_view": (C.c_int, [P, C.POINTER(Particles)]),
        "fsim_particles_free": (C.c_int, [P]),
        "fsim_particles_write": (C.c_int, [C.c_char_p, C.POINTER(Particles)]),
        "fsim_case_generate": (C.c_int, [C.POINTER(Case), C.POINTER(Config), C.POINTER(P)]),
        "fsim_create": (C.c_int, [C.POINTER(Config), C.POINTER(Particles), C.c_int, C.POINTER(P)]),
        "fsim_destroy": (C.c_int, [P]),
        "fsim_step": (C.c_int, [P, C.c_int]),
        "fsim_sync": (C.c_int, [P]),
        "fsim_run_phase": (C.c_int, [P, C.c_int]),
        "fsim_field_width": (C.c_int, [C.c_int]),
        "fsim_get_field": (C.c_int, [P, C.c_int, P, C.c_size_t]),
        "fsim_set_field": (C.c_int, [P, C.c_int, P, C.c_size_t]),
        "fsim_neighbor_counts": (C.c_int, [P, P, C.c_size_t]),
        "fsim_list_stats": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int)]),
        "fsim_list_counts": (C.c_int, [P, P, C.c_size_t]),
        "fsim_get_cells": (C.c_int, [P, C.c_int, P, C.c_size_t, P, C.c_size_t]),
        "fsim_write_vtk": (C.c_int, [P, C.c_char_p, C.c_int]),
        "fsim_time_steps": (C.c_int, [P, C.c_int, C.POINTER(C.c_float)]),
        "fsim_time_sweep": (C.c_int, [P, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "fsim_launches_per_step": (C.c_int, [P, C.POINTER(C.c_int)]),
        "fsim_conservation": (C.c_int, [P, C.POINTER(C.c_double), C.c_int]),
        "fsim_measure_fp32_peak": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
        "fsim_sweep_tuning": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_float), C.c_int]),
        "fsim_snapshot_bytes": (C.c_int, [P, C.POINTER(C.c_size_t)]),
        "fsim_probe": (C.c_int, [P, P, C.c_int, P]),
        "fsim_write_vtk_binary": (C.c_int, [P, C.c_char_p, C.c_int]),
        "fsim_batch_sync_members": (C.c_int, [P, P, C.c_int]),
        "fsim_create_case": (C.c_int, [P, P, C.c_int, C.POINTER(P)]),
        "fsim_case_counts": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "fsim_get_fields": (C.c_int, [P, C.c_int, P, P, P]),
        "fsim_batch_add": (C.c_int, [P, P]),
        "fsim_time_phases": (C.c_int, [P, C.c_int, C.POINTER(C.c_float), C.c_int]),
        "fsim_batch_remove": (C.c_int, [P, P]),
        "fsim_set_fields": (C.c_int, [P, C.c_int, P, P, P]),
        "fsim_snapshot_save": (C.c_int, [P, C.c_longlong, P, C.c_size_t]),
        "fsim_snapshot_load": (C.c_int, [P, C.c_size_t, C.c_int, C.POINTER(P), C.POINTER(C.c_longlong)]),
        "fsim_snapshot_write": (C.c_int, [P, C.c_longlong, C.c_char_p]),
        "fsim_snapshot_read": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(P), C.POINTER(C.c_longlong)]),
        "fsim_batch_sweep_tuning": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_float), C.c_int]),
        "fsim_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(P)]),
        "fsim_host_free": (C.c_int, [P]),
        "fsim_counts": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "fsim_get_derived": (C.c_int, [P, C.POINTER(Derived)]),
        "fsim_cell_sort_noalloc": (C.c_int, [C.POINTER(Derived), P, C.c_int, P, P, P]),
        "fsim_batch_create": (C.c_int, [C.POINTER(P), C.c_int, C.POINTER(P)]),
        "fsim_batch_step": (C.c_int, [P, C.c_int]),
        "fsim_batch_sync": (C.c_int, [P]),
        "fsim_batch_time_steps": (C.c_int, [P, C.c_int, C.POINTER(C.c_float)]),
        "fsim_batch_launches_per_step": (C.c_int, [P, C.POINTER(C.c_int)]),
        "fsim_batch_destroy": (C.c_int, [P]),
        "fsim_estimate_bytes": (C.c_int, [C.POINTER(Config), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_size_t)]),
        "fsim_device_bytes": (C.c_int, [P, C.POINTER(C.c_size_t)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


EXPORTED = [
    "fsim_status_string", "fsim_last_error", "fsim_config_defaults", "fsim_config_from_ini",
    "fsim_config_from_ini_text", "fsim_derive", "fsim_particles_read", "fsim_particles_view",
    "fsim_particles_free", "fsim_particles_write", "fsim_case_generate", "fsim_create", "fsim_destroy",
    "fsim_step", "fsim_sync", "fsim_run_phase", "fsim_field_width", "fsim_get_field", "fsim_set_field",
    "fsim_neighbor_counts", "fsim_get_cells", "fsim_write_vtk", "fsim_time_steps", "fsim_time_sweep",
    "fsim_launches_per_step", "fsim_host_alloc", "fsim_host_free", "fsim_counts", "fsim_get_derived",
    "fsim_cell_sort_noalloc", "fsim_batch_create", "fsim_batch_step", "fsim_batch_sync", "fsim_batch_time_steps",
    "fsim_batch_launches_per_step", "fsim_batch_destroy", "fsim_estimate_bytes", "fsim_device_bytes",
    "fsim_conservation",
    "fsim_measure_fp32_peak", "fsim_sweep_tuning", "fsim_batch_sweep_tuning", "fsim_snapshot_bytes",
    "fsim_snapshot_save", "fsim_snapshot_load", "fsim_snapshot_write", "fsim_snapshot_read", "fsim_probe",
    "fsim_write_vtk_binary", "fsim_batch_sync_members", "fsim_create_case", "fsim_case_counts",
    "fsim_get_fields", "fsim_set_fields", "fsim_batch_add", "fsim_batch_remove",
    "fsim_time_phases", "fsim_list_stats", "fsim_list_counts",
]
SWEEP_SHAPES = ((4, 48), (4, 32), (8, 32))  # (warps per block, list capacity) per shape index


class FsimError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (load().fsim_status_string(status).decode(), msg))
        self.status = status


def check(status):
    if status != OK:
        raise FsimError(status, load().fsim_last_error().decode(errors="replace"))


# ------------------------------------------------------------------ config
def default_config():
    cfg = Config()
    check(load().fsim_config_defaults(C.byref(cfg)))
    return cfg


def config_from_ini_text(text):
    cfg = Config()
    check(load().fsim_config_from_ini_text(text.encode(), C.byref(cfg)))
    return cfg


def config_from_ini(path):
    cfg = Config()
    check(load().fsim_config_from_ini(os.fsencode(path), C.byref(cfg)))
    return cfg


def estimate_bytes(cfg, n_fluid, n_solid, n_virt):
    out = C.c_size_t()
    check(load().fsim_estimate_bytes(C.byref(cfg), n_fluid, n_solid, n_virt, C.byref(out)))
    return out.value


def _tuning(fn, handle):
    chosen = C.c_int()
    ms = (C.c_float * len(SWEEP_SHAPES))()
    check(fn(handle, C.byref(chosen), ms, len(SWEEP_SHAPES)))
    return chosen.value, list(ms)


def case_counts(case):
    """(n_fluid, n_solid, n_virt) of a lattice case, without generating it."""
    nf, ns, nv = C.c_int(), C.c_int(), C.c_int()
    check(load().fsim_case_counts(C.byref(case), C.byref(nf), C.byref(ns), C.byref(nv)))
    return nf.value, ns.value, nv.value


def measure_fp32_peak(device=0):
    """FP32 FMA throughput of the device in TFLOP/s (fsim_measure_fp32_peak)."""
    out = C.c_double()
    check(load().fsim_measure_fp32_peak(device, C.byref(out)))
    return out.value


def derive(cfg):
    d = Derived()
    check(load().fsim_derive(C.byref(cfg), C.byref(d)))
    return d


# --------------------------------------------------------------- particles
def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class ParticleArrays:
    """Host particle arrays (input order) as contiguous numpy arrays."""

    def __init__(self, fluid_pos, fluid_vel, fluid_rho, fluid_p, solid_pos, solid_vel, solid_ref_pos, solid_type,
                 virt_pos, virt_type=None):
        f32 = lambda a, w: np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, w))
        self.fluid_pos, self.fluid_vel = f32(fluid_pos, 3), f32(fluid_vel, 3)
        self.fluid_rho, self.fluid_p = f32(fluid_rho, 1).ravel(), f32(fluid_p, 1).ravel()
        self.solid_pos, self.solid_vel, self.solid_ref_pos = f32(solid_pos, 3), f32(solid_vel, 3), f32(solid_ref_pos, 3)
        self.solid_type = np.ascontiguousarray(np.asarray(solid_type, dtype=np.int32).ravel())
        self.virt_pos = f32(virt_pos, 3)
        vt = np.zeros(len(self.virt_pos), np.int32) if virt_type is None else virt_type
        self.virt_type = np.ascontiguousarray(np.asarray(vt, dtype=np.int32).ravel())

    @property
    def n_fluid(self):
        return len(self.fluid_rho)

    @property
    def n_solid(self):
        return len(self.solid_type)

    @property
    def n_virt(self):
        return len(self.virt_pos)

    def struct(self):
        p = Particles()
        p.n_fluid, p.n_solid, p.n_virt = self.n_fluid, self.n_solid, self.n_virt
        p.fluid_pos, p.fluid_vel = _fptr(self.fluid_pos), _fptr(self.fluid_vel)
        p.fluid_rho, p.fluid_p = _fptr(self.fluid_rho), _fptr(self.fluid_p)
        p.solid_pos, p.solid_vel, p.solid_ref_pos = _fptr(self.solid_pos), _fptr(self.solid_vel), _fptr(
            self.solid_ref_pos)
        p.solid_type = _iptr(self.solid_type)
        p.virt_pos, p.virt_type = _fptr(self.virt_pos), _iptr(self.virt_type)
        return p

    @staticmethod
    def from_set(handle):
        lib = load()
        v = Particles()
        check(lib.fsim_particles_view(handle, C.byref(v)))

        def arr(ptr, n, w, dt):
            if n == 0:
                return np.zeros((0, w), dt)
            return np.ctypeslib.as_array(ptr, shape=(n * w,)).reshape(n, w).astype(dt, copy=True)

        pa = ParticleArrays(arr(v.fluid_pos, v.n_fluid, 3, np.float32), arr(v.fluid_vel, v.n_fluid, 3, np.float32),
                            arr(v.fluid_rho, v.n_fluid, 1, np.float32), arr(v.fluid_p, v.n_fluid, 1, np.float32),
                            arr(v.solid_pos, v.n_solid, 3, np.float32), arr(v.solid_vel, v.n_solid, 3, np.float32),
                            arr(v.solid_ref_pos, v.n_solid, 3, np.float32),
                            arr(v.solid_type, v.n_solid, 1, np.int32),
                            arr(v.virt_pos, v.n_virt, 3, np.float32), arr(v.virt_type, v.n_virt, 1, np.int32))
        return pa

    def write_dat(self, data_dir):
        check(load().fsim_particles_write(os.fsencode(data_dir), C.byref(self.struct())))


def read_dat(data_dir):
    lib = load()
    h = C.c_void_p()
    check(lib.fsim_particles_read(os.fsencode(data_dir), C.byref(h)))
    try:
        return ParticleArrays.from_set(h)
    finally:
        lib.fsim_particles_free(h)


def generate_case(case, cfg):
    lib = load()
    h = C.c_void_p()
    check(lib.fsim_case_generate(C.byref(case), C.byref(cfg), C.byref(h)))
    try:
        return ParticleArrays.from_set(h)
    finally:
        lib.fsim_particles_free(h)


# -------------------------------------------------------------- simulation
class Simulation:
    """One instance on one GPU, owned through an fsim_handle."""

    def __init__(self, cfg, particles, device=-1):
        self.lib = load()
        self.cfg = cfg
        self.particles = particles
        self.h = C.c_void_p()
        check(self.lib.fsim_create(C.byref(cfg), C.byref(particles.struct()), device, C.byref(self.h)))
        self._set_counts()
        self.snapshot_step = None

    def _set_counts(self):
        nf, ns, nv = C.c_int(), C.c_int(), C.c_int()
        check(self.lib.fsim_counts(self.h, C.byref(nf), C.byref(ns), C.byref(nv)))
        self.n = {"fluid": nf.value, "solid": ns.value, "virt": nv.value}

    @classmethod
    def _from_handle(cls, h, step):
        self = cls.__new__(cls)
        self.lib, self.h, self.cfg, self.particles = load(), h, None, None
        self._set_counts()
        self.snapshot_step = step
        return self

    @classmethod
    def from_case(cls, cfg, case, device=-1):
        """Generate a lattice case on the device (fsim_create_case)."""
        h = C.c_void_p()
        check(load().fsim_create_case(C.byref(cfg), C.byref(case), device, C.byref(h)))
        self = cls._from_handle(h, None)
        self.cfg = cfg
        return self

    @classmethod
    def from_snapshot(cls, data, device=-1):
        """Restore an instance from fsim_snapshot_save bytes (a bytes object or uint8 array)."""
        buf = np.frombuffer(data, np.uint8) if not isinstance(data, np.ndarray) else data
        h, step = C.c_void_p(), C.c_longlong()
        check(load().fsim_snapshot_load(buf.ctypes.data, buf.nbytes, device, C.byref(h), C.byref(step)))
        return cls._from_handle(h, step.value)

    @classmethod
    def from_snapshot_file(cls, path, device=-1):
        h, step = C.c_void_p(), C.c_longlong()
        check(load().fsim_snapshot_read(os.fsencode(path), device, C.byref(h), C.byref(step)))
        return cls._from_handle(h, step.value)

    def probe(self, points):
        """(n, 5) float32: Shepard-averaged u, v, w, p, rho at each point (fsim_probe)."""
        pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        out = np.empty((len(pts), 5), np.float32)
        check(self.lib.fsim_probe(self.h, pts.ctypes.data, len(pts), out.ctypes.data))
        return out

    def snapshot(self, step=0):
        """The instance's state as snapshot bytes (numpy uint8 array)."""
        n = C.c_size_t()
        check(self.lib.fsim_snapshot_bytes(self.h, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        check(self.lib.fsim_snapshot_save(self.h, step, buf.ctypes.data, buf.nbytes))
        return buf

    def snapshot_write(self, path, step=0):
        check(self.lib.fsim_snapshot_write(self.h, step, os.fsencode(path)))

    def close(self):
        if self.h:
            self.lib.fsim_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def step(self, n=1):
        check(self.lib.fsim_step(self.h, n))

    def sync(self):
        check(self.lib.fsim_sync(self.h))

    def phase(self, p):
        check(self.lib.fsim_run_phase(self.h, p))

    def _count(self, field_id):
        return self.n["fluid"] if field_id < 10 else self.n["solid"] if field_id < 30 else self.n["virt"]

    def get(self, name, out=None):
        fid = FIELDS[name]
        w = self.lib.fsim_field_width(fid)
        n = self._count(fid)
        dt = np.int32 if name in INT_FIELDS else np.float32
        if out is None:
            out = np.empty((n, w) if w > 1 else (n,), dt)
        check(self.lib.fsim_get_field(self.h, fid, out.ctypes.data, out.nbytes))
        return out

    def set(self, name, values):
        fid = FIELDS[name]
        a = np.ascontiguousarray(values, dtype=np.float32)
        check(self.lib.fsim_set_field(self.h, fid, a.ctypes.data, a.nbytes))

    def set_ptr(self, name, ptr, nbytes):
        check(self.lib.fsim_set_field(self.h, FIELDS[name], ptr, nbytes))

    def get_ptr(self, name, ptr, nbytes):
        check(self.lib.fsim_get_field(self.h, FIELDS[name], ptr, nbytes))

    def get_many_ptr(self, names, ptrs, nbytes):
        """fsim_get_fields: several fields into host pointers, one synchronisation."""
        n = len(names)
        ids = (C.c_int * n)(*[FIELDS[k] for k in names])
        dst = (C.c_void_p * n)(*[p.value if isinstance(p, C.c_void_p) else p for p in ptrs])
        nb = (C.c_size_t * n)(*nbytes)
        check(self.lib.fsim_get_fields(self.h, n, ids, dst, nb))

    def set_many_ptr(self, names, ptrs, nbytes):
        """fsim_set_fields: several fields from host pointers."""
        n = len(names)
        ids = (C.c_int * n)(*[FIELDS[k] for k in names])
        src = (C.c_void_p * n)(*[p.value if isinstance(p, C.c_void_p) else p for p in ptrs])
        nb = (C.c_size_t * n)(*nbytes)
        check(self.lib.fsim_set_fields(self.h, n, ids, src, nb))

    def neighbor_counts(self):
        out = np.empty((self.n["fluid"], 3), np.int32)
        check(self.lib.fsim_neighbor_counts(self.h, out.ctypes.data, out.nbytes))
        return out

    def list_counts(self):
        """Neighbour-list entries within the impact distance per fluid particle."""
        out = np.empty((self.n["fluid"], 3), np.int32)
        check(self.lib.fsim_list_counts(self.h, out.ctypes.data, out.nbytes))
        return out

    def list_stats(self):
        """{"enabled", "builds", "capacity", "check"} of the fluid neighbour lists."""
        v = [C.c_int() for _ in range(4)]
        check(self.lib.fsim_list_stats(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("enabled", "builds", "capacity", "check"), (x.value for x in v)))

    def cells(self, species):
        d = self.derived()
        start = np.empty(d.cell_number_total + 1, np.int32)
        n = [self.n["fluid"], self.n["solid"], self.n["virt"]][species]
        ids = np.empty(n, np.int32)
        check(self.lib.fsim_get_cells(self.h, species, start.ctypes.data, start.nbytes, ids.ctypes.data, ids.nbytes))
        return start, ids

    def derived(self):
        d = Derived()
        check(self.lib.fsim_get_derived(self.h, C.byref(d)))
        return d

    def write_vtk(self, out_dir, file_step, binary=False):
        fn = self.lib.fsim_write_vtk_binary if binary else self.lib.fsim_write_vtk
        check(fn(self.h, os.fsencode(out_dir), file_step))

    def time_steps(self, n):
        ms = C.c_float()
        check(self.lib.fsim_time_steps(self.h, n, C.byref(ms)))
        return ms.value

    def time_sweep(self, n):
        tot, sw = C.c_float(), C.c_float()
        check(self.lib.fsim_time_sweep(self.h, n, C.byref(tot), C.byref(sw)))
        return tot.value, sw.value

    def launches_per_step(self):
        n = C.c_int()
        check(self.lib.fsim_launches_per_step(self.h, C.byref(n)))
        return n.value

    def time_phases(self, n):
        """Device ms per phase over n launch-by-launch steps (fsim_time_phases)."""
        ms = (C.c_float * 5)()
        check(self.lib.fsim_time_phases(self.h, n, ms, 5))
        return dict(zip(("cell", "couple", "virt", "fluid", "solid"), list(ms)))

    def sweep_tuning(self):
        """(chosen shape or -1, [ms per shape]) of the sweep autotuner."""
        return _tuning(self.lib.fsim_sweep_tuning, self.h)

    def device_bytes(self):
        """Device memory the instance's own arrays hold (fsim_device_bytes)."""
        out = C.c_size_t()
        check(self.lib.fsim_device_bytes(self.h, C.byref(out)))
        return out.value

    def conservation(self):
        """FP64 conservation totals (fsim_conservation) as a dict."""
        out = (C.c_double * CONSERVATION_N)()
        check(self.lib.fsim_conservation(self.h, out, CONSERVATION_N))
        return dict(zip(CONSERVATION_KEYS, list(out)))


class PinnedBuffer:
    """Page-locked host memory from fsim_host_alloc, viewed as a numpy array."""

    def __init__(self, shape, dtype=np.float32):
        self.lib = load()
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = C.c_void_p()
        check(self.lib.fsim_host_alloc(self.nbytes, C.byref(self.ptr)))
        buf = (C.c_char * self.nbytes).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self.lib.fsim_host_free(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch:
    """Several Simulations advanced in lockstep by batched launches (fsim_batch_*)."""

    def __init__(self, sims):
        self.lib = load()
        self.sims = list(sims)
        arr = (C.c_void_p * len(self.sims))(*[sm.h.value for sm in self.sims])
        self.b = C.c_void_p()
        check(self.lib.fsim_batch_create(arr, len(self.sims), C.byref(self.b)))

    def step(self, n=1):
        check(self.lib.fsim_batch_step(self.b, n))

    def sync(self):
        check(self.lib.fsim_batch_sync(self.b))

    def time_steps(self, n):
        ms = C.c_float()
        check(self.lib.fsim_batch_time_steps(self.b, n, C.byref(ms)))
        return ms.value

    def launches_per_step(self):
        n = C.c_int()
        check(self.lib.fsim_batch_launches_per_step(self.b, C.byref(n)))
        return n.value

    def add(self, sim):
        """Admit a standalone Simulation into the live batch."""
        check(self.lib.fsim_batch_add(self.b, sim.h))
        self.sims.append(sim)

    def remove(self, sim):
        """Let a member leave; it continues standalone."""
        check(self.lib.fsim_batch_remove(self.b, sim.h))
        self.sims.remove(sim)

    def sync_members(self):
        """Wait for the batch; the status code of every member (OK, or ENUMERIC
        for a member whose particles left the grid)."""
        st = np.empty(len(self.sims), np.int32)
        check(self.lib.fsim_batch_sync_members(self.b, st.ctypes.data, len(st)))
        return [int(x) for x in st]

    def sweep_tuning(self):
        """(chosen shape or -1, [ms per shape]) of the batch's sweep autotuner."""
        return _tuning(self.lib.fsim_batch_sweep_tuning, self.b)

    def close(self):
        if self.b:
            self.lib.fsim_batch_destroy(self.b)
            self.b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
