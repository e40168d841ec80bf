"""Batched instances (fsim_batch_*): every member's result equals its
standalone result bit for bit, whatever else is in the batch."""
import numpy as np
import pytest

from fluidsim_gb300 import api, cases

pytestmark = pytest.mark.gpu

FIELDS = ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "solid_PK1", "virt_p",
          "solid_normal")


def _members():
    """Instances that differ in size, viscosity, solid and sub-steps."""
    specs = [
        cases.tiny_box(jitter=0.01, seed=1),
        cases.tiny_box(jitter=0.02, seed=2, with_solid=False, viscid=False, fluid=(8, 6, 9)),
        cases.tiny_box(jitter=0.01, seed=3, fluid=(14, 12, 10), tank=(30, 18, 16)),
    ]
    specs[2][0].solid_sub_step = 6
    specs[2][0].youngs_modulus = 3e5
    return [cases.make(s) for s in specs]


def _fields(sim):
    out = {}
    for f in FIELDS:
        if f.startswith("solid") and sim.n["solid"] == 0:
            continue
        out[f] = sim.get(f)
    return out


@pytest.mark.parametrize("steps", [1, 7])
def test_batch_members_equal_standalone(steps):
    members = _members()
    alone = []
    for cfg, pa in members:
        with api.Simulation(cfg, pa, device=0) as s:
            s.step(steps)
            s.sync()
            alone.append(_fields(s))
    sims = [api.Simulation(cfg, pa, device=0) for cfg, pa in members]
    with api.Batch(sims) as b:
        b.step(steps)
        b.sync()
        # 20 launches outside the solid sub-steps: the neighbour-list decision,
        # the list-grid sort (work only on a rebuild), the per-step cell index,
        # the list build, coupling, walls and the sweep; 3 per solid sub-step
        assert b.launches_per_step() <= 20 + 3 * 6
        batched = [_fields(s) for s in sims]
    for k, (a, c) in enumerate(zip(alone, batched)):
        for f in a:
            assert np.array_equal(a[f], c[f]), (k, f)
    # dissolved: the members continue standalone
    for s in sims:
        s.step(1)
        s.sync()
        s.close()


def test_large_batch_uses_the_item_array_sweep_and_equals_standalone():
    """A plain-form batch larger than the sweep's by-value parameter block (72
    instances) reads its items from global memory: the same results as each
    member alone, bit for bit."""
    members = [cases.make(cases.tiny_box(jitter=0.01, seed=100 + k, fluid=(8 + k % 5, 10, 8))) for k in range(80)]
    alone = []
    for cfg, pa in members:
        with api.Simulation(cfg, pa, device=0) as s:
            s.step(4)
            s.sync()
            alone.append({f: s.get(f) for f in ("fluid_pos", "fluid_vel", "fluid_p", "solid_pos")})
    sims = [api.Simulation(cfg, pa, device=0) for cfg, pa in members]
    with api.Batch(sims) as b:
        b.step(4)
        b.sync()
        for k, s in enumerate(sims):
            for f, want in alone[k].items():
                assert np.array_equal(s.get(f), want), (k, f)
    for s in sims:
        s.close()


def test_batch_rejects_misuse():
    (cfg, pa), = _members()[:1]
    s = api.Simulation(cfg, pa, device=0)
    with api.Batch([s]) as b:
        with pytest.raises(api.FsimError):
            s.step(1)  # members are stepped through the batch
        with pytest.raises(api.FsimError):
            api.Batch([s])  # already in a batch
        b.step(2)
        assert np.isfinite(s.get("fluid_pos")).all()  # getters wait for the batch
    s.close()


def test_batch_after_phase_calls_normalises_parity():
    """A member whose buffers were left at the other parity by phase calls
    joins the batch and still matches its standalone continuation."""
    (cfg, pa), = _members()[:1]
    ref = api.Simulation(cfg, pa, device=0)
    s = api.Simulation(cfg, pa, device=0)
    # a lone cell phase leaves both fluid and solid at the other buffer
    ref.phase(api.PHASE_CELL)
    s.phase(api.PHASE_CELL)
    ref.step(3)
    ref.sync()
    with api.Batch([s]) as b:
        b.step(3)
        b.sync()
    for f in ("fluid_pos", "fluid_vel", "solid_pos"):
        assert np.array_equal(ref.get(f), s.get(f)), f
    ref.close()
    s.close()


def test_member_status_is_per_instance():
    """A member whose particle leaves the cell grid (moved far outside: the
    cell hash clamps it and sets that instance's flag) reports ENUMERIC; the
    other members report OK."""
    sims = [api.Simulation(cfg, pa, device=0) for cfg, pa in _members()]
    x = sims[1].get("fluid_pos")
    x[0] = [50.0, 50.0, 50.0]
    sims[1].set("fluid_pos", x)
    with api.Batch(sims) as b:
        b.step(1)
        assert b.sync_members() == [api.OK, api.ENUMERIC, api.OK]
        b.step(1)
        assert b.sync_members() == [api.OK, api.OK, api.OK]  # clamped back into the domain
    for s in sims:
        s.close()


def test_fused_solid_launch_matches_standalone_and_oracle_policy():
    """solid_fused: all solid sub-steps of a step in one persistent cooperative
    launch.  Batch members still equal their standalone runs bit for bit, and
    the state stays within the FP32 parity policy of the per-phase launches."""
    members = _members()
    for cfg, _ in members:
        cfg.solid_fused = 1
    alone = []
    for cfg, pa in members:
        with api.Simulation(cfg, pa, device=0) as s:
            s.step(7)
            s.sync()
            alone.append(_fields(s))
    sims = [api.Simulation(cfg, pa, device=0) for cfg, pa in members]
    with api.Batch(sims) as b:
        b.step(7)
        b.sync()
        assert b.launches_per_step() <= 22  # the solid sub-steps are one launch (plus its slot pass)
        batched = [_fields(s) for s in sims]
    for k, (a, c) in enumerate(zip(alone, batched)):
        for f in a:
            assert np.array_equal(a[f], c[f]), (k, f)
    # against the per-phase launches: the same physics up to FP32 rounding
    cfg, pa = members[0]
    ref_cfg = api.Config.from_buffer_copy(cfg)
    ref_cfg.solid_fused = 0
    with api.Simulation(ref_cfg, pa, device=0) as r:
        r.step(7)
        r.sync()
        for f in ("solid_pos", "fluid_pos", "fluid_rho"):
            assert np.allclose(r.get(f), alone[0][f], rtol=1e-5, atol=1e-7), f
    # a batch takes one solid launch form
    plain = api.Simulation(ref_cfg, pa, device=0)
    with pytest.raises(api.FsimError):
        api.Batch([sims[0], plain])
    for s in sims + [plain]:
        s.close()


def test_add_and_remove_members_of_a_live_batch():
    """Members join and leave a live batch; every member's trajectory still
    equals its standalone run bit for bit."""
    members = _members()
    ref = []
    for cfg, pa in members:
        with api.Simulation(cfg, pa, device=0) as s:
            s.step(9)
            s.sync()
            ref.append(_fields(s))
    sims = [api.Simulation(cfg, pa, device=0) for cfg, pa in members]
    b = api.Batch(sims[:1])
    b.step(3)
    sims[1].step(3)        # standalone for a while, then joins
    b.add(sims[1])
    b.step(3)
    b.add(sims[2])         # joins fresh: 3 batched steps, then 6 alone
    b.remove(sims[0])      # leaves after 6 steps, continues alone
    sims[0].step(3)
    b.step(3)
    b.remove(sims[1])
    b.remove(sims[2])
    assert b.launches_per_step() == 0  # empty batch
    b.step(1)
    sims[2].step(6)
    b.close()
    for s in sims:
        s.sync()
    for k, s in enumerate(sims):
        got = _fields(s)
        for f, want in ref[k].items():
            assert np.array_equal(got[f], want), (k, f)
        s.close()


def test_fused_barrier_wait_runs_out_then_recovers():
    """The fused solid kernel's grid barrier gives up after a bounded wait.
    With the wait limited to one poll (gb300_barrier_wait_polls = 1) a CTA
    that is not the last to arrive gives up at once: the kernel returns, the
    instance's flag reports FSIM_ETIMEOUT, and the context stays usable — a
    handle with the default limit then steps normally and equals the
    per-phase launches up to FP32 rounding."""
    cfg, pa = cases.make(cases.small_dam_break())
    short = api.Config.from_buffer_copy(cfg)
    short.solid_fused = 1
    short.barrier_wait_polls = 1
    seen = None
    with api.Simulation(short, pa, device=0) as s:
        for _ in range(10):  # a CTA arriving within ~100 ns of the last one does not time out
            s.step(1)
            try:
                s.sync()
            except api.FsimError as e:
                seen = e
                break
    assert seen is not None and seen.status == api.ETIMEOUT, seen
    fused = api.Config.from_buffer_copy(cfg)
    fused.solid_fused = 1
    with api.Simulation(fused, pa, device=0) as a, api.Simulation(cfg, pa, device=0) as b:
        a.step(3)
        b.step(3)
        a.sync()
        b.sync()
        for f in ("solid_pos", "solid_vel", "fluid_pos"):
            assert np.allclose(a.get(f), b.get(f), rtol=1e-5, atol=1e-7), f
