"""The learned surrogate end to end on the GPU.

* Training data comes from the batched plain solver (an ensemble of seeded
  dx = 0.02 dam breaks); the network is trained by the library's own forward,
  backward and Adam kernels.
* Gain over the method without it: on held-out members, the trained network's
  one-jump error (mean squared normalised residual over the K = 10 step jump)
  is well below that of the constant-acceleration prior alone (the surrogate
  with its output set to zero).
* On-policy samples pair the states a judged learned rollout visits with the
  plain method's continuation from them.
* A rollout of the config-1 dam break with the plain-step fallback keeps its
  accounting (every jump accepted or undone), stays finite, and never accepts
  a jump whose density moved by more than the judge's tolerance.
* A jump after an accepted one reuses the fluid grid its judge built: that
  grid is exactly the re-bin of the current positions.
* Jumps judged on the device (conditional graph node) that all fall back
  reproduce the plain method bit for bit; an edge-buffer overflow falls back
  on the device and the host grows the buffer.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    from warp_sph_gpt_gb300.batch import Ensemble
    from warp_sph_gpt_gb300.generate import config_batch_member
    from warp_sph_gpt_gb300.surrogate import Network, SurrogateConfig, evaluate, fit_scales, generate, train

    members = [config_batch_member(1000 + i) for i in range(8)]
    ens = Ensemble(members)
    s = ens.solv
    cfg = SurrogateConfig(radius=float(s.support), dt=float(s.dt), rho0=float(s.rho0))
    ts = generate(ens, 400, cfg)
    train_ids, val_ids = list(range(6)), [6, 7]
    fit_scales(ts, cfg, train_ids, "cuda")
    net = Network(cfg, "cuda", seed=0)
    prior = evaluate(net, ts, val_ids, zero=True)
    hist = train(net, ts, train_ids, iters=800, lr=2e-3)
    val = evaluate(net, ts, val_ids)
    return dict(net=net, ts=ts, prior=prior, val=val, hist=hist, cfg=cfg)


def test_trained_network_beats_the_prior_on_held_out_members(trained):
    prior, val = trained["prior"], trained["val"]
    print(f"held-out one-jump loss: prior {prior:.4f}, trained {val:.4f}; training {trained['hist'][::2]}")
    assert np.isfinite(val)
    assert 0.5 < prior < 2.0  # output scales are the prior's RMS residual
    assert val < 0.6 * prior


def test_on_policy_samples_pair_rollout_states_with_plain_targets(trained):
    """collect_on_policy: one sample per jump window of each case, the target is
    the plain continuation, and training on them keeps the loss finite."""
    from warp_sph_gpt_gb300.batch import Case
    from warp_sph_gpt_gb300.generate import config_batch_member
    from warp_sph_gpt_gb300.surrogate import collect_on_policy, train

    picks = [m for m in (config_batch_member(1000 + i) for i in range(1, 12)) if len(m[1])][:2]
    cases = [Case(*m) for m in picks]
    samples = collect_on_policy(trained["net"], cases, 100)
    assert len(samples) == 10 * len(cases)
    for sets, x_t, v_t in samples:
        assert x_t.shape == v_t.shape == (sets.P.n + sets.D.n, 3)
        assert torch.isfinite(x_t).all() and torch.isfinite(v_t).all()
    hist = train(trained["net"], trained["ts"], list(range(6)), iters=50, lr=1e-4, extra=samples, log_every=10)
    assert all(np.isfinite(h[1]) for h in hist)


def test_rollout_with_fallback_respects_the_judge(trained):
    from warp_sph_gpt_gb300.batch import Case
    from warp_sph_gpt_gb300.generate import config_small
    from warp_sph_gpt_gb300.surrogate import LearnedRollout

    case = Case(config_small())
    ro = LearnedRollout(case, trained["net"])
    stats = ro.run(0, 200)
    torch.cuda.synchronize()
    assert stats["jumps"] > 0
    assert stats["plain_steps"] + stats["learned_steps"] == 200
    assert stats["learned_steps"] == trained["cfg"].substeps * (stats["jumps"] - stats["fallbacks"])
    assert torch.isfinite(case.P.pos).all() and torch.isfinite(case.D.pos).all()
    assert int(ro.g.status()) == 0


def test_jump_after_an_accepted_one_reuses_a_current_grid(trained):
    """After an accepted jump the fluid grid (cell starts and slot order) is
    exactly the one a re-bin of the current positions builds, so the next jump
    may skip that re-bin.  (Two whole rollouts are not compared bit for bit:
    the edge pass combines partial receiver sums across CTAs with atomics.)"""
    import ctypes as C

    from warp_sph_gpt_gb300 import _lib
    from warp_sph_gpt_gb300.batch import Case
    from warp_sph_gpt_gb300.engine import KIND_SPH
    from warp_sph_gpt_gb300.generate import config_small
    from warp_sph_gpt_gb300.surrogate import LearnedRollout

    case = Case(config_small())
    ro = LearnedRollout(case, trained["net"])
    step = 0
    while step < 200:
        ro.run(step, 10)
        step += 10
        if ro.last_accepted and step >= 30:
            break
    assert ro.last_accepted and ro.stats["jumps"] - ro.stats["fallbacks"] >= 2
    torch.cuda.synchronize()
    b = case.grids[0].buffers
    order, start = b["order"].clone(), b["cell_start"].clone()
    ctx = ro.ctx
    _lib.check(ctx.lib.sphdem_grid_build(C.byref(ctx.ctx), KIND_SPH, C.byref(ctx.params), ctx.stream), "grid")
    torch.cuda.synchronize()
    assert torch.equal(order, b["order"]) and torch.equal(start, b["cell_start"])


def test_device_judged_fallbacks_reproduce_the_plain_method(trained):
    """With a judge that rejects every jump, each jump is undone on the device
    and its steps replayed plain inside the rollout graph (conditional node):
    the rollout then equals the plain method bit for bit, and the accounting
    counts every jump as a fallback."""
    import dataclasses

    from warp_sph_gpt_gb300.batch import Case
    from warp_sph_gpt_gb300.generate import config_small
    from warp_sph_gpt_gb300.surrogate import LearnedRollout, Network

    base = trained["net"]
    net = Network(dataclasses.replace(base.cfg, tol=-1.0), "cuda", theta=base.theta.cpu().numpy())
    plain = Case(config_small())
    plain.run(0, 100)
    case = Case(config_small())
    ro = LearnedRollout(case, net)
    stats = ro.run(0, 100)
    torch.cuda.synchronize()
    assert stats["jumps"] == 10 and stats["fallbacks"] == 10 and stats["learned_steps"] == 0
    assert stats["plain_steps"] == 100
    for a, b in ((plain.P.pos, case.P.pos), (plain.P.vel, case.P.vel), (plain.D.pos, case.D.pos),
                 (plain.D.vel, case.D.vel), (plain.D.omega, case.D.omega)):
        np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    np.testing.assert_array_equal(plain.D.contact_dem_offset_old.cpu().numpy(),
                                  case.D.contact_dem_offset_old.cpu().numpy())


@pytest.mark.parametrize("native", [True, False])
def test_position_judge_alone_forces_the_plain_method(trained, native):
    """The position term of the judge: with a density tolerance no jump can
    exceed but a correction bound below any correction the network makes,
    every jump falls back (device-judged and host-judged), the rollout equals
    the plain method bit for bit, and with the bound far above the largest
    correction no jump falls back on its account."""
    import dataclasses

    from warp_sph_gpt_gb300.batch import Case
    from warp_sph_gpt_gb300.generate import config_small
    from warp_sph_gpt_gb300.surrogate import LearnedRollout, Network

    base = trained["net"]
    plain = Case(config_small())
    plain.run(0, 100)
    net = Network(dataclasses.replace(base.cfg, tol=1e9, pos_tol=1e-30), "cuda", theta=base.theta.cpu().numpy())
    case = Case(config_small())
    ro = LearnedRollout(case, net)
    ro.native = native
    stats = ro.run(0, 100)
    torch.cuda.synchronize()
    assert stats["jumps"] == 10 and stats["fallbacks"] == 10 and stats["learned_steps"] == 0
    for a, b in ((plain.P.pos, case.P.pos), (plain.P.vel, case.P.vel), (plain.D.pos, case.D.pos)):
        np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    net2 = Network(dataclasses.replace(base.cfg, tol=1e9, pos_tol=1e9), "cuda", theta=base.theta.cpu().numpy())
    ro2 = LearnedRollout(Case(config_small()), net2)
    ro2.native = native
    stats2 = ro2.run(0, 100)
    assert stats2["fallbacks"] == 0 and 0.0 < stats2["max_pos_accepted"] < 1e-2


def test_device_judged_rollout_recovers_from_an_edge_capacity_overflow(trained):
    """A graph that outgrows its edge buffer flags it; the device judge then
    falls back (the plain method runs those steps), and the host grows the
    buffer from the graph's own edge count and re-captures: later jumps are
    accepted again and the accounting stays whole."""
    from warp_sph_gpt_gb300.batch import Case
    from warp_sph_gpt_gb300.generate import config_small
    from warp_sph_gpt_gb300.surrogate import LearnedRollout

    case = Case(config_small())
    ro = LearnedRollout(case, trained["net"])
    ro.run(0, 10)  # the host-judged first jump
    ro.g._alloc_edges(2000)  # far below the ~400k edges of the config-1 graph
    ro.jump.net = ro.g._net(ro.net)
    fb0 = ro.stats["fallbacks"]
    ro.run(10, 60)
    assert ro.stats["fallbacks"] - fb0 == 6  # every jump of the overflowing chunk fell back
    assert ro.g.capacity >= ro.g.n_edges()
    stats = ro.run(70, 100)
    torch.cuda.synchronize()
    assert stats["jumps"] - stats["fallbacks"] >= 5  # accepted again
    assert stats["plain_steps"] + stats["learned_steps"] == 170
    assert torch.isfinite(case.P.pos).all() and int(ro.g.status()) == 0
