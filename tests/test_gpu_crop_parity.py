"""Parity at the benchmark's resolutions, and of the hot-path kernels' own
member sets.

* Cropped copies of the large (dx = 0.005, h = 0.0065, coupling h = 0.08, DEM
  R ~ U[0.01, 0.03]) and scaled (dx = 0.01, R = 0.025 jittered) dam breaks
  (tests/helpers.py): whole coupled steps against the FP64 oracle (fields) and
  the FP32 oracle (contact CSR, bit-exact) with spheres of unequal radius
  pressed into each other and into the walls, then all eleven neighbour
  relations bit-exact on the final state.  Tolerances as in
  tests/test_gpu_step_parity.py; the per-field errors are printed.
* The member sets that the production kernels decide -- the density pass's
  recorded lists, the members the force pass sums over, the porosity pass's
  near list -- digested from the kernels' own buffers right after a step and
  compared bit for bit with the FP32 oracle's relations on the step's start
  state (kernel/KERNEL_rho.py:45-82, kernel/KERNEL_force.py:40,57,
  kernel/KERNEL_SPHDEM_interaction.py:87-88), at dx = 0.04, on config 1 and on
  the large crop.
* The porosity normaliser decides no membership: it sums a clamped Wendland
  weight that is exactly 0 from q = 2 on.  Fluid particles placed at
  2 h (1 -+ 2^-23) from a subject give the oracle's porosity within 1e-5.
"""
import numpy as np
import pytest
import torch

from helpers import config_large_crop, config_scaled_crop, field_err, scene
from oracle.oracle import HostState
from test_gpu_step_parity import FIELD_FACTOR, _compare_csr, _err, _np, _record
from warp_sph_gpt_gb300 import SPHDEM_OneStep, dem_search_scales
from warp_sph_gpt_gb300.kernels import member_digest, neighbour_digest

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5
RELATIONS = ["SPH_SPH_SUPPORT", "SPH_BND_SUPPORT", "BND_SPH_SUPPORT", "BND_BND_SUPPORT", "SPH_SPH_FORCE",
             "SPH_BND_FORCE", "SPH_SPH_LEN", "SPH_DEM_2H", "DEM_SPH_2H", "DEM_DEM_2H", "SPH_DEM_REACT"]
# hot-path member set -> the reference relation it must equal
MEMBER_RELATIONS = (("DENSITY_FLUID", "SPH_SPH_SUPPORT"), ("DENSITY_WALL", "SPH_BND_SUPPORT"),
                    ("FORCE_FLUID", "SPH_SPH_FORCE"), ("FORCE_WALL", "SPH_BND_FORCE"),
                    ("POROSITY_NEAR", "SPH_DEM_2H"))


def _case(make, lanes, fmt=0):
    from warp_sph_gpt_gb300.batch import Case

    gen, pos, rad = make()
    c = Case(gen, pos, rad)
    c.tune({"lanes_sph": lanes, "nbr_format": fmt})
    return c


def _field_errors(s, P, B, D, h32, h64):
    """{field: (err(gpu, f64), err(f32 oracle, f64))}, field-normalised;
    pressure normalised by the bulk modulus."""
    bulk = s.rho0 * s.c0 ** 2
    out = {}
    groups = (("sph", P, ("rho", "pres", "acc", "pos", "vel", "porosity", "pgf", "acc_dem", "flt")),
              ("bnd", B, ("rho", "pres")),
              ("dem", D, ("force", "torque", "pos", "vel", "omega", "flt_s", "porosity", "drag", "pressure_force")))
    for group, obj, names in groups:
        for name in names:
            floor = bulk if name == "pres" else 0.0
            r64 = getattr(h64, group)[name]
            out[f"{group}.{name}"] = (_err(_np(getattr(obj, name)), r64, floor),
                                      _err(getattr(h32, group)[name], r64, floor))
    return out


def _check_members(s, scales, P, B, D, W, grids, start: HostState):
    """Every hot-path member set of the step just run equals the FP32 oracle's
    relation on the step's start state (start)."""
    for members, rel in MEMBER_RELATIONS:
        radius = 2.0 * scales[2] if rel == "SPH_DEM_2H" else s.support
        got_c, got_h = member_digest(members, P, B, D, W, tuple(grids))
        ref_c, ref_h = start.neighbour_digest(rel, radius)
        got_c, got_h = _np(got_c), _np(got_h).view(np.uint64)
        if members == "POROSITY_NEAR":
            np.testing.assert_array_equal(got_c, (ref_c > 0).astype(np.int32), err_msg=members)
        else:
            np.testing.assert_array_equal(got_c, ref_c, err_msg=members)
            np.testing.assert_array_equal(got_h, ref_h, err_msg=members)
        assert ref_c.sum() > 0, members


@pytest.mark.parametrize("which,fmt", [("large", 0), ("scaled", 0), ("large", 1)])
def test_cropped_benchmark_steps_match_oracle(which, fmt):
    """Three coupled steps of a cropped benchmark dam break (one thread per
    particle and neighbour records -- member slots (0) or walk masks (1) -- as
    at 800k): fields within max(1e-5,
    2.5 x the FP32 oracle's own error) of FP64, contact CSR bit-exact, the
    kernels' member sets bit-exact every step, all relations at the end."""
    c = _case(config_large_crop if which == "large" else config_scaled_crop, 1, fmt)
    s, P, B, D, W, grids, scales = c.solv, c.P, c.B, c.D, c.W, c.grids, c.scales
    assert D.radius.min() < D.radius.max() or which == "scaled"
    worst = {}
    contacts = [0, 0]
    for step in range(3):
        h64 = HostState(P, B, D, W)
        h32 = HostState(P, B, D, W)
        start = HostState(P, B, D, W)
        SPHDEM_OneStep(s, P, B, D, W, *grids, step, scales)
        torch.cuda.synchronize()
        _check_members(s, scales, P, B, D, W, grids, start)
        h64.sphdem_onestep(s, step, scales, p="f64")
        h32.sphdem_onestep(s, step, scales, p="f32")
        errs = _field_errors(s, P, B, D, h32, h64)
        _record({"case": f"crop-{which}-{fmt}", "step": step, "field": k, "gpu": v[0], "fp32_oracle": v[1]}
                for k, v in errs.items())
        bad = {k: v for k, v in errs.items() if not v[0] <= max(FIELD_TOL, FIELD_FACTOR * v[1])}
        assert not bad, f"step {step}: fields beyond max({FIELD_TOL}, {FIELD_FACTOR} x FP32-oracle error): {bad}"
        for k, v in errs.items():
            worst[k] = max(worst.get(k, (0.0, 0.0)), v)
        _compare_csr(D, h32)
        contacts[0] += int(D.contact_dem_offset_old[-1])
        contacts[1] += int(D.contact_bnd_offset_old[-1])
    assert contacts[0] > 0 and contacts[1] > 0, "the crop must exercise both contact kinds"
    print(f"\n[{which} crop] per-field err(gpu, f64) / err(f32 oracle, f64), worst of 3 steps:")
    for k, (g, r) in sorted(worst.items()):
        print(f"  {k:20s} {g:.3e} {r:.3e} ratio {g / r if r > 0 else float('nan'):.2f}")
    host = HostState(P, B, D, W)
    for rel in RELATIONS:
        radius = s.support if "SUPPORT" in rel or "FORCE" in rel else 2.0 * scales[2]
        got_c, got_h = neighbour_digest(rel, radius, P, B, D, grids[:3] + [None])
        ref_c, ref_h = host.neighbour_digest(rel, radius)
        np.testing.assert_array_equal(_np(got_c), ref_c, err_msg=rel)
        np.testing.assert_array_equal(_np(got_h).view(np.uint64), ref_h, err_msg=rel)


@pytest.mark.parametrize("fmt", [0, 1])
def test_member_sets_at_dx004_and_config1(fmt):
    """The hot-path member sets on the dx = 0.04 test scene (after two steps,
    off the lattice) and on config 1 (the reference's input files), with
    member-slot (0) and walk-mask (1) records."""
    from warp_sph_gpt_gb300.batch import Case
    from warp_sph_gpt_gb300.engine import context_for
    from warp_sph_gpt_gb300.generate import config_small

    s, P, B, D, W, grids = scene(dem_nx=3, dem_ny=2, dem_origin_x=0.1, dem_origin_y=0.1, dem_spacing=0.05,
                                 dem_origin_z=0.2)
    scales = dem_search_scales(D, W)
    context_for(P, B, D, W, tuple(grids)).tuning["nbr_format"] = fmt
    for step in range(3):
        start = HostState(P, B, D, W)
        SPHDEM_OneStep(s, P, B, D, W, *grids, step, scales)
        torch.cuda.synchronize()
        if step >= 2:
            _check_members(s, scales, P, B, D, W, grids, start)
    c = Case(config_small())
    c.tune({"lanes_sph": 1, "nbr_format": fmt})
    for step in range(2):
        start = HostState(c.P, c.B, c.D, c.W)
        c.step(step)
        torch.cuda.synchronize()
        _check_members(c.solv, c.scales, c.P, c.B, c.D, c.W, c.grids, start)


@pytest.mark.parametrize("fmt,cap", [(0, 8), (1, 4)])
def test_member_lists_overflow_walk_the_same_members(fmt, cap):
    """With a record capacity far below the member counts (8 slots) or the
    walk lengths (4 mask words = 128 slots) every particle walks its cells in
    the force pass; the members are the same."""
    from warp_sph_gpt_gb300.engine import context_for

    s, P, B, D, W, grids = scene(dem_nx=3, dem_ny=2, dem_origin_x=0.1, dem_origin_y=0.1, dem_spacing=0.05,
                                 dem_origin_z=0.2)
    scales = dem_search_scales(D, W)
    context_for(P, B, D, W, tuple(grids)).tuning.update({"nbr_cap": cap, "nbr_format": fmt})
    for step in range(2):
        start = HostState(P, B, D, W)
        SPHDEM_OneStep(s, P, B, D, W, *grids, step, scales)
        torch.cuda.synchronize()
    _check_members(s, scales, P, B, D, W, grids, start)


def test_porosity_normaliser_at_the_support_boundary():
    """Fluid placed at 2 h_c (1 - 2^-23) and 2 h_c (1 + 2^-23) around subjects
    near a sphere: the clamped-weight normaliser (no membership test) gives
    the FP64 oracle's porosity within 1e-5, as it does with those particles
    moved well inside and well outside the ball."""
    from warp_sph_gpt_gb300.batch import Case

    gen, pos, rad = config_scaled_crop()
    c = Case(gen, pos, rad)
    s, P, B, D, W, grids, scales = c.solv, c.P, c.B, c.D, c.W, c.grids, c.scales
    h_c = float(scales[3])
    assert h_c > 0
    x = P.pos.cpu().numpy().astype(np.float64)
    dpos = D.pos.cpu().numpy().astype(np.float64)
    near = np.where(np.linalg.norm(x[:, None, :] - dpos[None, :, :], axis=2).min(1) < 2 * h_c)[0]
    rng = np.random.default_rng(3)
    subjects = rng.choice(near, 6, replace=False)
    others = np.setdiff1d(np.arange(P.n), subjects)
    movers = rng.choice(others, 48, replace=False)
    for k, j in enumerate(movers):
        i = subjects[k % len(subjects)]
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        f = 1.0 - 2.0 ** -23 if k % 2 == 0 else 1.0 + 2.0 ** -23
        x[j] = x[i] + 2.0 * h_c * f * u
    P.pos.copy_(torch.as_tensor(x.astype(np.float32), device=P.pos.device))
    # the exact float distances straddle the support as intended for most movers
    xf = x.astype(np.float32)
    d = np.array([np.float32(np.sqrt(np.float32(((xf[j] - xf[subjects[k % 6]]) ** 2).sum())))
                  for k, j in enumerate(movers)])
    assert (d < np.float32(2 * h_c)).sum() >= 8 and (d >= np.float32(2 * h_c)).sum() >= 8
    h64 = HostState(P, B, D, W)
    h32 = HostState(P, B, D, W)
    c.step(0)
    torch.cuda.synchronize()
    h64.sphdem_onestep(s, 0, scales, p="f64")
    h32.sphdem_onestep(s, 0, scales, p="f32")
    got = _np(P.porosity)
    assert field_err(got, h64.sph["porosity"]) <= max(FIELD_TOL, FIELD_FACTOR * field_err(h32.sph["porosity"],
                                                                              h64.sph["porosity"]))
    assert np.abs(got[subjects] - h64.sph["porosity"][subjects]).max() < FIELD_TOL


def test_tensor_core_porosity_is_canonical():
    """The tensor-core normaliser (porosity_variant 2, the default) against the
    direct one (0) on the large crop: the same porosity within FP32 summation
    order; a rerun from the same state reproduces it bit for bit; and a
    different frame-block edge (other tiles, other centres) stays within the
    same tolerance."""
    import warp_sph_gpt_gb300.engine as E

    runs = {}
    for tag, variant, frame in (("mma", 2, None), ("again", 2, None), ("direct", 0, None), ("frame3", 2, 3)):
        c = _case(config_large_crop, 1)
        ctx = E.context_for(c.P, c.B, c.D, c.W, tuple(c.grids))
        ctx.tuning["porosity_variant"] = variant
        orig = E.porosity_frame
        if frame is not None:
            E.porosity_frame = lambda cell, vol: frame
        try:
            c.step(0)
        finally:
            E.porosity_frame = orig
        torch.cuda.synchronize()
        runs[tag] = (_np(c.P.porosity).copy(), int(ctx.ctl[6]))
    ref, n_near = runs["mma"]
    assert n_near > 1000
    np.testing.assert_array_equal(runs["again"][0], ref)
    assert np.abs(runs["direct"][0] - ref).max() < 2e-6
    assert np.abs(runs["frame3"][0] - ref).max() < 2e-6
    assert runs["direct"][1] == n_near == runs["frame3"][1]
