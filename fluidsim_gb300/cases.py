"""Benchmark and test cases: dam breaks with an elastic gate or cube.

Coordinates follow the reference: y is vertical and gravity points along -y
(src/physics.cpp:12-15).  The kernel is the reference's truncated Gaussian with
impact_length_hsml_ratio = 2 (config/input.ini:40 of the reference).

* ``small_dam_break``  — 160x40x80 tank at dx = 0.01 (1.6 x 0.4 x 0.8 m), a
  40x20x40 fluid block (32,000 particles) with hydrostatic density, a 4x20x40
  plate (3,200 free particles) at x = 0.8 m continued 3 layers into the floor
  as FIXED solid (480), 3 layers of wall particles; rho0 1000, c0 30, gamma 7,
  mu 1e-3 (viscous), solid rho 1100, E 1e6, nu 0.4; dt 1e-4, 4 solid
  sub-steps.
* ``fsi_4m``  — 512x128x128 tank at dx = 0.005 (2.56 x 0.64 x 0.64 m), a
  256x128x128 fluid column (4,194,304 particles), a free 30^3 elastic cube
  (27,000) on the floor at x = 1.68 m, centred in z; solid rho 1200, E 5e6,
  nu 0.3; dt 5e-5, 4 sub-steps; 912,600 wall particles.
* ``fsi_4m_jitter``  — ``fsi_4m`` with uniform +-0.01 dx position jitter
  (seed 12345).
* ``tiny_box`` — a few thousand particles for fast tests.
"""
import math

from . import api


def _config(dx, tank, h_ratio=1.3, c0=30.0, rho0=1000.0, gamma=7.0, mu=1e-3, viscid=True, rho_s=1100.0, E=1e6,
            nu=0.4, dt=1e-4, sub=4, steps=2000, precision=api.PRECISION_FP32, keep=False):
    cfg = api.default_config()
    cfg.gravity = 9.81
    cfg.is_viscid = 1 if viscid else 0
    cfg.fluid_sound_speed = c0
    cfg.fluid_density = rho0
    cfg.gamma = gamma
    cfg.viscosity = mu
    cfg.solid_density = rho_s
    cfg.youngs_modulus = E
    cfg.poisson_ratio = nu
    cfg.xmin = cfg.ymin = cfg.zmin = 0.0
    cfg.xmax, cfg.ymax, cfg.zmax = tank[0] * dx, tank[1] * dx, tank[2] * dx
    cfg.dt = dt
    cfg.istart = 0
    cfg.iend = steps
    cfg.solid_sub_step = sub
    cfg.result_interval = steps + 1
    cfg.smoothing_length = h_ratio * dx
    cfg.particle_diameter = dx
    cfg.impact_length_hsml_ratio = 2.0
    cfg.precision = precision
    cfg.keep_derivatives = 1 if keep else 0
    return cfg


def _case(dx, tank, fluid, solid_lo, solid_n, fixed_layers, virt_layers=3, hydrostatic=True, jitter=0.0, seed=0):
    c = api.Case()
    c.dx = dx
    for k in range(3):
        c.tank_n[k] = tank[k]
        c.fluid_n[k] = fluid[k]
        c.solid_lo[k] = solid_lo[k]
        c.solid_n[k] = solid_n[k]
    c.solid_fixed_layers = fixed_layers
    c.virt_layers = virt_layers
    c.hydrostatic = 1 if hydrostatic else 0
    c.jitter = jitter
    c.seed = seed
    return c


def small_dam_break(keep=False, jitter=0.0, seed=0, precision=api.PRECISION_FP32):
    dx, tank = 0.01, (160, 40, 80)
    cfg = _config(dx, tank, keep=keep, precision=precision)
    case = _case(dx, tank, (40, 20, 40), (80, 0, 0), (4, 20, 40), 3, jitter=jitter, seed=seed)
    return cfg, case


def fsi_4m(keep=False, jitter=0.0, seed=0, precision=api.PRECISION_FP32):
    dx, tank = 0.005, (512, 128, 128)
    cfg = _config(dx, tank, rho_s=1200.0, E=5e6, nu=0.3, dt=5e-5, sub=4, steps=1000, keep=keep,
                  precision=precision)
    case = _case(dx, tank, (256, 128, 128), (336, 0, 49), (30, 30, 30), 0, jitter=jitter, seed=seed)
    return cfg, case


def fsi_4m_jitter(keep=False, precision=api.PRECISION_MIXED):
    return fsi_4m(keep=keep, jitter=0.01, seed=12345, precision=precision)


def tiny_box(keep=False, jitter=0.0, seed=0, with_solid=True, viscid=True, fluid=(12, 10, 12), tank=(24, 16, 16),
             precision=api.PRECISION_FP32):
    dx = 0.01
    cfg = _config(dx, tank, viscid=viscid, keep=keep, precision=precision)
    solid_n = (2, 8, 8) if with_solid else (0, 0, 0)
    case = _case(dx, tank, fluid, (16, 0, 4), solid_n, 2 if with_solid else 0, jitter=jitter, seed=seed)
    return cfg, case


def make(cfg_case):
    """Generate the particles of a (config, case) pair."""
    cfg, case = cfg_case
    return cfg, api.generate_case(case, cfg)


def _solid_substeps(cfg, base=4):
    """Solid sub-steps for stability: the explicit TLSPH step must stay below
    about 0.25 h / c_s (c_s from the bulk modulus); never fewer than `base`."""
    E, nu, rho = cfg.youngs_modulus, cfg.poisson_ratio, cfg.solid_density
    cs = math.sqrt(E / (3.0 * (1.0 - 2.0 * nu)) / rho)
    limit = 0.25 * cfg.smoothing_length / cs
    return max(base, int(math.ceil(cfg.dt / limit)))


def ensemble_member(rng, dx=0.01, n_range=(8000, 250000), steps=500):
    """One dam-break instance of the batched ensemble: fluid count log-uniform
    in n_range (random block dims), plate E log-uniform in [1e5, 1e7] Pa, nu
    uniform in [0.3, 0.45], gate x uniform in [0.6, 1.0] m; tank 1.6 m long and
    0.8 m wide, tall enough for the column."""
    target = math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))
    gate = int(round(rng.uniform(0.6, 1.0) / dx))
    nz = int(rng.integers(30, 81))
    nx = int(rng.integers(max(10, gate // 3), gate - 2 + 1))
    ny = max(4, int(round(target / (nx * nz))))
    tank = (int(round(1.6 / dx)), max(int(round(0.4 / dx)), ny + 10), int(round(0.8 / dx)))
    E = math.exp(rng.uniform(math.log(1e5), math.log(1e7)))
    nu = float(rng.uniform(0.3, 0.45))
    cfg = _config(dx, tank, rho_s=1100.0, E=E, nu=nu, dt=1e-4, sub=4, steps=steps)
    cfg.solid_sub_step = _solid_substeps(cfg)
    case = _case(dx, tank, (nx, ny, nz), (gate, 0, 0), (4, min(20, tank[1] - 1), min(40, tank[2])), 3)
    return cfg, case


def ensemble(n=64, seed=2024, **kw):
    """The batched-ensemble workload: n independent instances (seeded)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    return [ensemble_member(rng, **kw) for _ in range(n)]
