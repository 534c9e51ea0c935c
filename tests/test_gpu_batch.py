"""Batched ensembles and launch tuning on the GPU.

* An ensemble of dam breaks of uneven sizes (instance-keyed grids, one launch
  per phase, one CUDA graph per step) evolves every member bit for bit as the
  member run alone: same neighbour traversal order (world-anchored lattice,
  members keep their particle order), same kernels.
* Launch tuning (cell width factor, block size, porosity implementation,
  thread or warp per particle) does not change results beyond summation
  order: every configuration agrees with the default within the whole-step
  tolerance, and neighbour sets are equal.
"""
import numpy as np
import pytest
import torch

from warp_sph_gpt_gb300.batch import Case, Ensemble
from warp_sph_gpt_gb300.generate import config_batch_member

pytestmark = pytest.mark.gpu


def _members(ids):
    return [config_batch_member(i) for i in ids]


def test_ensemble_members_evolve_exactly_as_alone():
    ids = [0, 3, 5, 11]
    members = _members(ids)
    ens = Ensemble(members)
    assert len(set(ens.counts["sph"])) > 1  # uneven sizes
    ens.run(0, 25)
    torch.cuda.synchronize()
    for k, (gen, pos, rad) in enumerate(members):
        alone = Case(gen, pos, rad)
        alone.run(0, 25)
        torch.cuda.synchronize()
        for kind, part in (("sph", alone.P), ("dem", alone.D)):
            for field in ("pos", "vel"):
                np.testing.assert_array_equal(ens.member(k, kind, field).cpu().numpy(),
                                              getattr(part, field).cpu().numpy(), err_msg=f"member {k} {kind}.{field}")
        np.testing.assert_array_equal(ens.member(k, "sph", "rho").cpu().numpy(), alone.P.rho.cpu().numpy())
        np.testing.assert_array_equal(ens.member(k, "bnd", "rho").cpu().numpy(), alone.B.rho.cpu().numpy())


@pytest.mark.parametrize("cell_factor,block,variant,lanes", [(0.75, 256, 0, 1), (1.0, 64, 1, 1), (0.75, 128, 1, 1),
                                                               (1.0, 128, 0, 32), (0.75, 256, 1, 32)])
def test_tuning_does_not_change_results(cell_factor, block, variant, lanes):
    gen, pos, rad = config_batch_member(5)
    ref = Case(gen, pos, rad)
    ref.run(0, 10)
    alt = Case(gen, pos, rad, cell_factor=cell_factor)
    alt.tune({"block_sph": block, "porosity_variant": variant, "lanes_sph": lanes})
    alt.run(0, 10)
    torch.cuda.synchronize()
    for part_a, part_b in ((ref.P, alt.P), (ref.D, alt.D)):
        a, b = part_a.pos.cpu().numpy(), part_b.pos.cpu().numpy()
        assert np.abs(a - b).max() < 1e-3 * 0.02
    np.testing.assert_array_equal(ref.D.contact_dem_offset_old.cpu().numpy(), alt.D.contact_dem_offset_old.cpu().numpy())
    if cell_factor == 1.0 and lanes == 1:  # same cells and order: only the porosity implementation differs
        np.testing.assert_array_equal(ref.P.rho.cpu().numpy(), alt.P.rho.cpu().numpy())


def test_snapshot_restore_replays_bit_for_bit():
    gen, pos, rad = config_batch_member(7)
    case = Case(gen, pos, rad)
    case.run(0, 5)
    snap = case.snapshot()
    case.run(5, 30)
    first = (case.P.pos.clone(), case.P.vel.clone(), case.D.pos.clone(), case.D.omega.clone())
    case.restore(snap)
    case.run(5, 30)
    torch.cuda.synchronize()
    for a, b in zip(first, (case.P.pos, case.P.vel, case.D.pos, case.D.omega)):
        np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())


@pytest.mark.parametrize("fmt,nbr_cap", [(0, 0), (0, 16), (1, -1), (1, 4), (1, 12)])
def test_neighbour_lists_give_identical_steps(fmt, nbr_cap):
    """Forces from the density pass's neighbour records equal the cell walk
    bit for bit (same members, same order), against the default (member
    slots, default capacity): records off (0); member slots so few that most
    particles overflow and walk (16); walk masks at their default capacity;
    masks so short that nearly every particle walks (4 words = 128 walked
    slots); and masks where walks of either kind overflow for some particles
    only (12)."""
    gen, _, _ = config_batch_member(4)
    xs = np.arange(0.04, gen.fluid_width - 0.03, 0.07)
    zs = np.arange(0.026, gen.fluid_height - 0.03, 0.07)
    pos = np.array([(x, 0.2, z) for x in xs for z in zs])
    rad = np.full(len(pos), 0.025)
    ref = Case(gen, pos, rad)
    ref.run(0, 25)
    alt = Case(gen, pos, rad)
    alt.tune({"nbr_cap": nbr_cap, "nbr_format": fmt})
    alt.run(0, 25)
    torch.cuda.synchronize()
    from warp_sph_gpt_gb300.engine import context_for

    params = [context_for(c.P, c.B, c.D, c.W, tuple(c.grids)).params for c in (ref, alt)]
    assert params[0].nbr_cap >= 64 and params[0].nbr_format == 0
    assert params[1].nbr_format == fmt and (params[1].nbr_cap == nbr_cap if nbr_cap >= 0 else params[1].nbr_cap >= 16)
    for part_a, part_b in ((ref.P, alt.P), (ref.D, alt.D)):
        for field in ("pos", "vel"):
            np.testing.assert_array_equal(getattr(part_a, field).cpu().numpy(), getattr(part_b, field).cpu().numpy())
    np.testing.assert_array_equal(ref.P.acc.cpu().numpy(), alt.P.acc.cpu().numpy())
    np.testing.assert_array_equal(ref.P.pgf.cpu().numpy(), alt.P.pgf.cpu().numpy())


def test_batch_member_step_matches_oracle():
    """A member's coupled step inside a batched state against the oracle run on
    that member alone: fields within max(1e-5, 2.5 x the FP32 oracle's own error)
    of FP64, contact CSR bit-exact against the FP32 oracle (as in
    tests/test_gpu_step_parity.py)."""
    from oracle.oracle import HostState
    from test_gpu_step_parity import _compare_csr, _compare_step
    from warp_sph_gpt_gb300.generate import build_case

    ids = [3, 7, 11]
    members = _members(ids)
    ens = Ensemble(members)
    k = 1  # the middle member: particles before and after it in every set
    gen, pos, rad = members[k]
    P, B, D, W = build_case(gen, pos, rad, device="cpu")
    assert D.n > 0
    h64, h32 = HostState(P, B, D, W), HostState(P, B, D, W)
    ens.step(0)
    torch.cuda.synchronize()
    h64.sphdem_onestep(ens.solv, 0, ens.scales, p="f64")
    h32.sphdem_onestep(ens.solv, 0, ens.scales, p="f32")

    class View:  # the member's slice of every field, in the struct's names
        pass

    views = {}
    for kind, part in (("sph", ens.P), ("bnd", ens.B), ("dem", ens.D)):
        v = View()
        for name, _ in type(part)._fields:
            setattr(v, name, ens.member(k, kind, name))
        views[kind] = v
    _compare_step(ens.solv, views["sph"], views["bnd"], views["dem"], h32, h64)
    # the member's contact CSR: rows k of the batched CSR, neighbour ids relative to its first sphere
    o = ens.offsets
    for kind, wkey in (("dem", "dem"), ("bnd", "dembnd")):
        off = getattr(ens.D, f"contact_{kind}_offset_old").cpu().numpy()
        ids_all = getattr(ens.D, f"contact_{kind}_id_old").cpu().numpy()
        rows = off[o["dem"][k]:o["dem"][k + 1] + 1]
        ref = h32.side(kind, "old")
        np.testing.assert_array_equal(rows - rows[0], ref["offset"], err_msg=f"{kind} offsets")
        np.testing.assert_array_equal(ids_all[rows[0]:rows[-1]] - o[wkey][k], ref["id"], err_msg=f"{kind} ids")
