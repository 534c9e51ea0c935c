"""Host side of batched ensembles and the launch autotuner (no GPU).

* Ensemble concatenation: member slices, per-set instance ids, grid instance
  counts, rejection of members with different solver controls.
* The autotuner picks the fastest candidate, caches it by case key and reads
  the cache back without timing again; candidates keep the porosity
  implementation that supports instance-keyed grids.
"""
import numpy as np
import pytest
import torch

from warp_sph_gpt_gb300 import autotune as AT
from warp_sph_gpt_gb300.batch import Ensemble
from warp_sph_gpt_gb300.generate import config_batch_member


def test_ensemble_concatenation_on_host():
    ids = [0, 3, 5]
    members = [config_batch_member(i) for i in ids]
    ens = Ensemble(members, device="cpu")
    assert ens.ninst == 3
    from warp_sph_gpt_gb300.generate import build_case

    for k, (gen, pos, rad) in enumerate(members):
        P, B, D, W = build_case(gen, pos, rad, device="cpu")
        for kind, part in (("sph", P), ("bnd", B), ("dem", D), ("dembnd", W)):
            assert ens.counts[kind][k] == part.n
            np.testing.assert_array_equal(ens.member(k, kind, "pos").numpy(), part.pos.numpy())
    for g, kind in zip(ens.grids, ("sph", "bnd", "dem", "dembnd")):
        assert g.ninst == 3
        inst = g.inst.numpy()
        assert inst.dtype == np.int32 and len(inst) == sum(ens.counts[kind])
        assert (np.diff(inst) >= 0).all()
        np.testing.assert_array_equal(np.bincount(inst, minlength=3), ens.counts[kind])
    assert ens.n_units == sum(ens.counts["sph"]) + sum(ens.counts["dem"])


def test_ensemble_rejects_mixed_solver_controls():
    a = config_batch_member(0)
    gen_b, pos_b, rad_b = config_batch_member(1)
    gen_b.dt = gen_b.dt * 2
    with pytest.raises(ValueError, match="dt"):
        Ensemble([a, (gen_b, pos_b, rad_b)], device="cpu")
    with pytest.raises(ValueError):
        Ensemble([], device="cpu")


def test_autotune_picks_fastest_and_caches(tmp_path):
    cost = {(1.0, 128, 0): 5.0, (1.0, 256, 0): 4.0, (0.75, 128, 0): 3.5, (0.75, 256, 0): 6.0,
            (1.0, 128, 1): 7.0, (1.0, 256, 1): 8.0, (0.75, 128, 1): 9.0, (0.75, 256, 1): 9.5}
    calls = []

    def timer(make_case, cfg):
        calls.append(cfg)
        return cost[(cfg["cell_factor"], cfg["block_sph"], cfg["porosity_variant"])]

    path = tmp_path / "tune.json"
    best = AT.autotune(None, "case-A", ninst=1, timer=timer, cache_path=path)
    assert (best["cell_factor"], best["block_sph"], best["porosity_variant"]) == (0.75, 128, 0)
    assert best["ms_per_step"] == 3.5 and len(calls) == 8
    again = AT.autotune(None, "case-A", ninst=1, timer=timer, cache_path=path)
    assert again == best and len(calls) == 8  # served from the cache
    multi = list(AT.candidates(ninst=4))
    assert multi and all(c["porosity_variant"] == 0 for c in multi)
    AT.autotune(None, "case-B", ninst=4, timer=timer, cache_path=path)
    import json

    assert set(json.loads(path.read_text())) == {"case-A", "case-B"}


def test_neighbour_capacity():
    """Neighbour-record capacity per particle and kind.  Member slots: 1.25 x
    a full support ball + 8, a multiple of 8.  Walk masks: 1.25 x the slots of
    a walk over cells spanning 2 s + c per axis, + 64 bits, in 32-bit words.
    An explicit request wins; too large a buffer means none."""
    import math

    from warp_sph_gpt_gb300._lib import NBR_MASKS, NBR_SLOTS
    from warp_sph_gpt_gb300.engine import NBR_BYTES_MAX, neighbour_capacity

    dx = 0.005
    s = 2.6 * dx
    cap = neighbour_capacity(792_000, s, dx ** 3)
    ball = 4.0 / 3.0 * math.pi * 2.6 ** 3  # 73.6 particles
    assert cap == neighbour_capacity(792_000, s, dx ** 3, fmt=NBR_SLOTS)
    assert cap % 8 == 0 and 1.25 * ball + 8 <= cap < 1.25 * ball + 16
    words = neighbour_capacity(792_000, s, dx ** 3, fmt=NBR_MASKS)
    walked = (3 * 2.6) ** 3  # cell = support: 474.6 slots
    assert words == math.ceil((1.25 * walked + 64) / 32) == 21
    half = neighbour_capacity(792_000, s, dx ** 3, cell=0.5 * s, fmt=NBR_MASKS)  # finer cells, shorter walk
    assert half == math.ceil((1.25 * (2.5 * 2.6) ** 3 + 64) / 32) < words
    for fmt in (NBR_SLOTS, NBR_MASKS):
        assert neighbour_capacity(1000, s, dx ** 3, request=16, fmt=fmt) == 16
        assert neighbour_capacity(1000, s, dx ** 3, request=0, fmt=fmt) == 0
    n_big = NBR_BYTES_MAX // (4 * (2 * cap + 2)) + 1
    assert neighbour_capacity(n_big, s, dx ** 3) == 0


def test_rollout_accounting():
    """Host bookkeeping of a device-judged chunk: steps, the largest accepted
    judge value from its float bits, kernel counts, and the CSR parity."""
    import numpy as np

    from warp_sph_gpt_gb300.surrogate import rollout_accounting

    stats = dict(jumps=0, fallbacks=0, plain_steps=0, learned_steps=0, max_dev_accepted=0.0, jump_kernels=0)
    bits = int(np.array(0.0075, np.float32).view(np.int32))
    odd = rollout_accounting(stats, [50, 2, bits, 0], 9, 2000, 400)
    assert stats == dict(jumps=50, fallbacks=2, plain_steps=68, learned_steps=432,
                         max_dev_accepted=float(np.float32(0.0075)), jump_kernels=2000 + 16)
    assert odd is False  # 68 plain steps
    assert rollout_accounting(stats, [3, 0, 0, 0], 9, -1, -1) is True and stats["plain_steps"] == 71


def test_domain_box_leaves_out_non_finite_positions():
    """A NaN or Inf position does not poison the grid box (it bins to a face
    cell on the device, which flags it); the box spans the finite points."""
    from types import SimpleNamespace

    from warp_sph_gpt_gb300.engine import StepContext
    from warp_sph_gpt_gb300.struct import BNDptl, SPHptl

    P, B = SPHptl(3, "cpu"), BNDptl(2, "cpu")
    P.pos.copy_(torch.tensor([[0.0, 1.0, 2.0], [float("nan"), 5.0, 1.0], [3.0, -1.0, float("inf")]]))
    B.pos.copy_(torch.tensor([[-1.0, 0.5, 0.0], [0.5, 0.5, 0.5]]))
    ctx = SimpleNamespace(box=None, sets=[P, B])  # the box logic alone (a context pins host memory)
    lo, hi = StepContext._domain(ctx)
    assert lo == [-1.0, 0.5, 0.0]
    assert hi[:2] == [0.5, 1.0] and hi[2] == pytest.approx(2.0 + 0.5 * 2.0)
    P.pos.fill_(float("nan"))
    B.pos.fill_(float("nan"))
    ctx.box = None
    lo, hi = StepContext._domain(ctx)
    assert all(np.isfinite(lo)) and all(np.isfinite(hi))


def test_porosity_frame_edge():
    """Frame blocks of the tensor-core porosity pass hold >= 4 tiles of 128 at
    the mean particle volume, edge 2..8 cells, and depend only on the cell
    width and the particle volume."""
    from warp_sph_gpt_gb300.engine import porosity_frame

    dx = 0.005
    assert porosity_frame(2.6 * dx, dx ** 3) == 4    # cell = support 2h = 2.6 dx: 17.6 particles per cell
    assert porosity_frame(0.052, 0.02 ** 3) == 4     # config 1
    assert porosity_frame(1.0, 1e-3) == 2            # 1000 per cell: the minimum edge
    assert porosity_frame(0.01, 0.01 ** 3) == 8      # one per cell: capped
    assert porosity_frame(0.0, 1.0) == 4 and porosity_frame(1.0, 0.0) == 4
    for f in (porosity_frame(c, v) for c in (0.01, 0.013, 0.05) for v in (1e-7, 1e-6, 1e-5)):
        assert 2 <= f <= 8
