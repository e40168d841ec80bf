"""Small cases for the parity tests: fluid and solid in contact, and an
elastic block under a prescribed affine deformation.

* ``plate_touching_fluid(speed)`` — ``tiny_box`` (12x10x12 fluid, a 2x8x8
  plate continued 2 layers into the floor as FIXED solid) with the plate moved
  to one particle spacing from the fluid block, inside the impact distance
  2h = 2.6 dx, moving along x at ``speed`` (negative: into the fluid).
* ``dam_gate_near(gate_x)`` — the 32,000-particle dam break with its plate at
  x = gate_x (0.41 m: the plate's first particles sit two spacings from the
  fluid block's last ones, inside the impact distance).
* ``deformed_block(...)`` — a free 6x6x6 elastic cube away from walls and
  fluid whose current positions are x = c + A (X - c) for its reference
  positions X, with velocities v = B (X - c): a 2-4 % stretch plus 4 % shear
  and a linear velocity field.  With the kernel-correction matrix the SPH
  deformation gradient of an affine map is exactly A for every particle, so
  F, the Green strain and the stresses are O(strain) and well conditioned in
  FP32.
"""
import numpy as np

from fluidsim_gb300 import api, cases

A_DEFORM = np.array([[1.040, 0.040, 0.000],
                     [0.000, 0.980, 0.040],
                     [0.020, 0.000, 1.030]])
B_VELOCITY = np.array([[0.20, -0.10, 0.00],
                       [0.05, 0.10, -0.15],
                       [0.00, 0.10, -0.05]])


def plate_touching_fluid(speed, keep=True):
    cfg, pa = cases.make(cases.tiny_box(keep=keep))
    shift = pa.solid_pos[:, 0].min() - pa.fluid_pos[:, 0].max() - cfg.particle_diameter
    sp, sr, sv = pa.solid_pos.copy(), pa.solid_ref_pos.copy(), np.zeros_like(pa.solid_vel)
    sp[:, 0] -= shift
    sr[:, 0] -= shift
    sv[:, 0] = np.where(pa.solid_type == 0, speed, 0.0)
    return cfg, api.ParticleArrays(pa.fluid_pos, pa.fluid_vel, pa.fluid_rho, pa.fluid_p, sp, sv, sr,
                                   pa.solid_type, pa.virt_pos)


def dam_gate_near(gate_x=0.41, keep=True, jitter=0.01, seed=5):
    cfg, case = cases.small_dam_break(keep=keep, jitter=jitter, seed=seed)
    case.solid_lo[0] = int(round(gate_x / case.dx))
    return cases.make((cfg, case))


def deformed_block(sub_steps=1, keep=True, A=A_DEFORM, B=B_VELOCITY):
    dx, tank = 0.01, (24, 16, 16)
    cfg = cases._config(dx, tank, keep=keep, rho_s=1100.0, E=1e6, nu=0.4)
    cfg.solid_sub_step = sub_steps
    case = cases._case(dx, tank, (4, 4, 4), (12, 5, 5), (6, 6, 6), 0)
    cfg, pa = cases.make((cfg, case))
    X = pa.solid_ref_pos.astype(np.float64)
    c = X.mean(axis=0)
    x = c + (X - c) @ A.T
    v = (X - c) @ B.T
    return cfg, api.ParticleArrays(pa.fluid_pos, pa.fluid_vel, pa.fluid_rho, pa.fluid_p, x.astype(np.float32),
                                   v.astype(np.float32), pa.solid_ref_pos, pa.solid_type, pa.virt_pos)
