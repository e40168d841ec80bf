"""CPU checks of the reference build's host side and of the power of the
stress checks.

* The harness's mirror of the reference's Parameter / Data_Pointer / Cell
  layouts equals the reference headers' own (include/parameter.h:17-49,
  include/data_pointer.cuh:7-47, include/cell.cuh:11-20), compared through
  oracle/_ref/ref_layout (built from the reference headers where the
  reference checkout exists).
* The harness library loads and exports its entry points (no GPU call).
* A stress computed in the wrong order (P = S F instead of F S) or with the
  wrong sign of the coupling traction differs from the FP64 oracle by at
  least ten times the tolerances of tests/test_gpu_contact.py: those checks
  can fail.  The mistakes are planted in a CPU copy of the oracle's output.
"""
import os
import subprocess

import numpy as np
import pytest

import parity_cases as pc
from conftest import nerr
from oracle import build as obuild
from oracle import oracle as orc
from oracle import refbuild

ENTRY_POINTS = ["ref_last_error", "ref_layout", "ref_create", "ref_destroy", "ref_phase", "ref_step",
                "ref_time_steps", "ref_get", "ref_list_cells"]


def test_harness_exports():
    obuild.build_harness()
    lib = refbuild.load()
    for name in ENTRY_POINTS:
        assert hasattr(lib, name), name


@pytest.mark.skipif(not os.path.exists(obuild.ref_layout_path()),
                    reason="reference layout probe not built (needs the reference checkout)")
def test_mirror_layout_matches_reference_headers():
    out = subprocess.run([obuild.ref_layout_path()], capture_output=True, text=True, check=True).stdout.split("\n")
    theirs = [int(x) for x in out if x.strip() and x.strip().lstrip("-").isdigit()]
    assert refbuild.layout() == theirs


def _pk1(F, lam, mu):
    E = 0.5 * (np.einsum("nki,nkj->nij", F, F) - np.eye(3))
    S = 2.0 * mu * E + lam * np.trace(E, axis1=1, axis2=2)[:, None, None] * np.eye(3)
    return F @ S, S


def test_planted_stress_mistakes_fail_the_bound():
    from fluidsim_gb300 import api

    cfg, pa = pc.deformed_block(sub_steps=1)
    r64 = orc.OracleSim(cfg, pa, "f64")
    for ph in range(5):
        r64.phase(ph)
    d = api.derive(cfg)
    F = r64.get("solid_F").reshape(-1, 3, 3)
    P_oracle = r64.get("solid_PK1").reshape(-1, 3, 3)
    P, S = _pk1(F, d.lambda_, d.shear_modulus)
    assert nerr(P, P_oracle) < 1e-9  # P = F S with the oracle's own F
    from test_gpu_contact import TOL_STRESS

    assert nerr(S @ F, P_oracle) > 10 * TOL_STRESS            # wrong order
    assert nerr(np.transpose(P, (0, 2, 1)), P_oracle) > 10 * TOL_STRESS  # transposed
    assert nerr(F @ (2.0 * S), P_oracle) > 10 * TOL_STRESS     # doubled shear and bulk terms


def test_planted_coupling_sign_fails_the_bound():
    cfg, pa = pc.plate_touching_fluid(-0.5)
    r64 = orc.OracleSim(cfg, pa, "f64")
    for ph in range(5):
        r64.phase(ph)
    c = r64.get("solid_couple_dudt")
    from test_gpu_contact import TOL_PHASE

    assert np.abs(c).max() > 1.0
    assert nerr(-c, c) > 100 * TOL_PHASE
