"""Failures made on the host, reported by the step's status bits.

The reference raises OverflowError when the directed contact count does not
fit the CSR (source/Simulation.py:153-154) and FloatingPointError on a
non-finite state (output/frame_writer.py:58-62).  Here the device ORs
SPHDEM_FLAG_* bits into the control block and the host maps them to the same
exceptions at its status check.  Each failure is made on the host -- a CSR
allocated too small for the contacts the spheres have, a NaN written into a
position, a barrier wait that nothing will end -- and after each the GPU runs
a normal step on a fresh state with the oracle's results.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from helpers import field_err, scene
from oracle.oracle import HostState
from warp_sph_gpt_gb300 import SPHDEM_OneStep, _lib, dem_search_scales
from warp_sph_gpt_gb300.engine import context_for
from warp_sph_gpt_gb300.simulation import check_status

pytestmark = pytest.mark.gpu


def _pressed_scene(capacity_dem=None, capacity_bnd=None):
    s, P, B, D, W, grids = scene(dem_nx=3, dem_ny=2, dem_origin_x=0.1, dem_origin_y=0.1, dem_spacing=0.05,
                                 dem_origin_z=0.2)
    if capacity_dem is not None or capacity_bnd is not None:
        D._init_contacts(D.n, D.pos.device, capacity_dem, capacity_bnd)  # before any context exists
    D.pos[:, 2] = 0.015  # into the floor wall spheres
    D.pos[:, 0] -= 0.004 * torch.arange(D.n, dtype=torch.float32, device=D.pos.device)  # into each other
    return s, P, B, D, W, grids


def _healthy_step():
    """A normal coupled step on a fresh state equals the FP32 oracle's CSR and
    stays within the FP64 oracle's fields: the GPU and the library are fine."""
    s, P, B, D, W, grids = _pressed_scene()
    scales = dem_search_scales(D, W)
    h32 = HostState(P, B, D, W)
    SPHDEM_OneStep(s, P, B, D, W, *grids, 0, scales)
    torch.cuda.synchronize()
    check_status(P)
    h32.sphdem_onestep(s, 0, scales, p="f32")
    ref = h32.side("dem", "old")
    np.testing.assert_array_equal(D.contact_dem_offset_old.cpu().numpy(), ref["offset"])
    np.testing.assert_array_equal(D.contact_dem_id_old.cpu().numpy(), ref["id"])
    assert int(ref["offset"][-1]) > 0
    assert np.isfinite(P.pos.cpu().numpy()).all()
    assert field_err(P.rho.cpu().numpy(), h32.sph["rho"]) < 1e-5


@pytest.mark.parametrize("kind", ["dem", "bnd"])
def test_contact_csr_overflow_raises_overflow_error(kind):
    caps = dict(capacity_dem=1) if kind == "dem" else dict(capacity_bnd=2)
    s, P, B, D, W, grids = _pressed_scene(**caps)
    scales = dem_search_scales(D, W)
    SPHDEM_OneStep(s, P, B, D, W, *grids, 0, scales)
    torch.cuda.synchronize()
    ctl = D._ctl.cpu().numpy()
    flag = _lib.FLAG_CSR_DEM_OVERFLOW if kind == "dem" else _lib.FLAG_CSR_BND_OVERFLOW
    assert ctl[3] & flag
    assert ctl[4 if kind == "dem" else 5] > (1 if kind == "dem" else 2)  # the true count was still taken
    with pytest.raises(OverflowError):
        check_status(P)
    assert int(D._ctl[3]) == 0  # the status was consumed
    _healthy_step()


def test_nonfinite_position_raises_floating_point_error():
    s, P, B, D, W, grids = _pressed_scene()
    scales = dem_search_scales(D, W)
    P.pos[17, 1] = float("nan")
    SPHDEM_OneStep(s, P, B, D, W, *grids, 0, scales)
    torch.cuda.synchronize()
    assert int(D._ctl[3]) & _lib.FLAG_NONFINITE
    with pytest.raises(FloatingPointError):
        check_status(P)
    _healthy_step()


@pytest.mark.parametrize("polls", [0, 64])
def test_bounded_wait_times_out_and_reports(polls):
    """A barrier wait that nothing ends gives up after its poll limit, flags
    SPHDEM_FLAG_TIMEOUT, and the step status check raises for it."""
    s, P, B, D, W, grids = _pressed_scene()
    ctx = context_for(P, B, D, W, tuple(grids))
    ctx._fill()
    rc = ctx.lib.sphdem_wait_selftest(C.c_void_p(D._ctl.data_ptr()), polls, ctx.stream)
    _lib.check(rc, "wait self-test")
    torch.cuda.synchronize()
    assert int(D._ctl[3]) & _lib.FLAG_TIMEOUT
    with pytest.raises(RuntimeError, match="timed out"):
        check_status(P)
    assert ctx.lib.sphdem_wait_selftest(C.c_void_p(D._ctl.data_ptr()), -1, ctx.stream) == 2
    _healthy_step()
