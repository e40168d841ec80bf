"""fsim_estimate_bytes, which the server's admission control trusts, bounds
the device memory an instance really holds (fsim_device_bytes) for every
form: plain and mixed precision, neighbour lists or the cell walk, with and
without kept derivatives, with and without a solid, after steps have run
(the lists and the solid's per-lane lists exist from creation)."""
import pytest

from fluidsim_gb300 import api, cases

pytestmark = pytest.mark.gpu


def _forms():
    for precision in (api.PRECISION_FP32, api.PRECISION_MIXED):
        for skin in (0.15, 0.0):
            for keep in (False, True):
                yield precision, skin, keep


@pytest.mark.parametrize("precision,skin,keep", list(_forms()))
def test_estimate_bounds_the_allocation(precision, skin, keep):
    for spec in (cases.small_dam_break(keep=keep, precision=precision),
                 cases.tiny_box(keep=keep, with_solid=False, precision=precision)):
        cfg, pa = cases.make(spec)
        cfg.neighbor_skin = skin
        est = api.estimate_bytes(cfg, pa.n_fluid, pa.n_solid, pa.n_virt)
        with api.Simulation(cfg, pa, device=0) as sim:
            sim.step(2)
            sim.sync()
            held = sim.device_bytes()
        print("precision %d skin %.2f keep %d: %d particles, estimate %.1f MB, held %.1f MB" % (
            precision, skin, keep, pa.n_fluid + pa.n_solid + pa.n_virt, est / 1e6, held / 1e6))
        assert held <= est, (held, est)
        # an upper estimate, not a wild one
        assert est <= 1.6 * held + (8 << 20), (held, est)
