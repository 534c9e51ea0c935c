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
