"""Point probes (fsim_probe) against the oracle's restatement of the
reference's probe (both forms)."""
import numpy as np
import pytest

from conftest import nerr
from fluidsim_gb300 import api, cases
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _points(pa, rng):
    lo, hi = pa.fluid_pos.min(0), pa.fluid_pos.max(0)
    inside = rng.uniform(lo, hi, size=(200, 3))
    near_plate = pa.solid_pos[rng.integers(0, len(pa.solid_pos), 40)] + rng.normal(0, 0.004, size=(40, 3))
    empty = np.array([[1.5, 0.35, 0.7], [1.2, 0.3, 0.1]])           # in the tank, away from everything
    outside = np.array([[-5.0, 0.1, 0.1], [0.5, 9.0, 0.2]])         # outside the cell grid
    return np.vstack([inside, near_plate, empty, outside]).astype(np.float32)


@pytest.mark.parametrize("precision", [api.PRECISION_FP32, api.PRECISION_MIXED])
def test_probe_matches_oracle(precision):
    cfg, pa = cases.make(cases.small_dam_break(jitter=0.01, seed=17, precision=precision))
    cfg_plain = api.Config.from_buffer_copy(cfg)
    cfg_plain.precision = api.PRECISION_FP32
    sim = api.Simulation(cfg, pa, device=0)
    ref = orc.OracleSim(cfg_plain, pa, "f64")
    r32 = orc.OracleSim(cfg_plain, pa, "f32")
    sim.step(5)
    ref.step(5)
    r32.step(5)
    pts = _points(pa, np.random.default_rng(3))
    got, want, w32 = sim.probe(pts), ref.probe(pts.astype(np.float64)), r32.probe(pts.astype(np.float64))
    # no particle in range / outside the grid: exactly (0, 0, 0, 0, rho0)
    for k in range(len(pts) - 4, len(pts)):
        assert np.array_equal(got[k], [0, 0, 0, 0, cfg.fluid_density]), k
        assert np.array_equal(want[k], [0, 0, 0, 0, cfg.fluid_density]), k
    # probes near the plate average solid velocities, whose FP32 error is set by
    # the conditioning of the stress (as for the solid_vel field): two-sided bound
    names = ("u", "v", "w", "p", "rho")
    for c, name in enumerate(names):
        e, e32 = nerr(got[:, c], want[:, c]), nerr(w32[:, c], want[:, c])
        print("%-3s gpu %.3g  fp32-oracle %.3g" % (name, e, e32))
        assert e <= 3.0 * e32 + 1e-3, (name, e, e32)
    sim.close()


def test_probe_needs_cells():
    cfg, pa = cases.make(cases.tiny_box())
    with api.Simulation(cfg, pa, device=0) as sim:
        with pytest.raises(api.FsimError):
            sim.probe([[0.1, 0.05, 0.05]])
        sim.step(1)
        assert sim.probe(np.zeros((0, 3))).shape == (0, 5)
