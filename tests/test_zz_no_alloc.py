"""The allocation-free contact rebuild against the regular one.

``sphdem_contacts_noalloc`` serves callers that cannot allocate device memory
(their GPU memory belongs to another framework's pool, or their time loop must
not allocate): it keeps the per-row contact counts in a fixed array inside the
library.  Called through the C ABI on one copy of a state, it must give the
same contact CSR, tangential history, force and torque as the regular entry
points (caller scratch) on an identical copy -- on two calls in a row, so a
second call also proves that the first call's leftovers in the shared array do
no harm.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from helpers import field_err, scene
from warp_sph_gpt_gb300 import _lib, dem_search_scales
from warp_sph_gpt_gb300 import kernels as K
from warp_sph_gpt_gb300.engine import context_for

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _case():
    s, P, B, D, DB, grids = scene(dem_nx=3, dem_ny=2, dem_origin_x=0.1, dem_origin_y=0.1, dem_spacing=0.05,
                                  dem_origin_z=0.2)
    g = torch.Generator(device="cpu").manual_seed(7)
    # press the spheres into each other and into the floor wall spheres
    D.pos[:, 2] = 0.015
    D.pos[:, 0] -= 0.004 * torch.arange(D.n, dtype=torch.float32).to(D.pos.device)
    D.vel.copy_((torch.rand(D.vel.shape, generator=g) - 0.5).to(D.vel.device) * 0.1)
    D.omega.copy_((torch.rand(D.omega.shape, generator=g) - 0.5).to(D.omega.device))
    for grid, part in ((grids[2], D), (grids[3], DB)):
        grid.build(part.pos, grid.radius)
    return s, D, DB, grids


def _noalloc(D, DB, grids, radius_max, bnd_radius_max, g, dt, which):
    ctx = context_for(None, None, D, DB, (None, None, grids[2], grids[3]))
    ctx.prepare(rebuild_moving=True)
    rc = ctx.lib.sphdem_contacts_noalloc(C.byref(ctx.ctx), radius_max, bnd_radius_max, g, dt, which, ctx.stream)
    _lib.check(rc, "sphdem_contacts_noalloc")
    if which & 1:
        D._flip("dem")
    if which & 2:
        D._flip("bnd")


def _same_contacts(Dg, Dr):
    for kind in ("dem", "bnd"):
        np.testing.assert_array_equal(getattr(Dg, f"contact_{kind}_offset_old").cpu().numpy(),
                                      getattr(Dr, f"contact_{kind}_offset_old").cpu().numpy())
        np.testing.assert_array_equal(getattr(Dg, f"contact_{kind}_id_old").cpu().numpy(),
                                      getattr(Dr, f"contact_{kind}_id_old").cpu().numpy())
        assert field_err(getattr(Dg, f"tang_{kind}_old").cpu().numpy(),
                         getattr(Dr, f"tang_{kind}_old").cpu().numpy()) < TOL
    for name in ("force", "torque"):
        assert field_err(getattr(Dg, name).cpu().numpy(), getattr(Dr, name).cpu().numpy()) < TOL


def test_no_alloc_contacts_match_regular_entry_points():
    """Separate calls per contact kind (which = 1, then 2) on one copy and the
    fused call (which = 3: both count passes and both halves of the shared
    array in one kernel) on a third copy, each against the regular entry
    points on an identical copy."""
    s, D1, W1, g1 = _case()
    _, D2, W2, g2 = _case()
    _, D3, W3, g3 = _case()
    scales = dem_search_scales(D1, W1)
    for call in range(2):
        K.force_dem(D1, g1[2], scales[0], s.g, s.dt)
        K.bc_dem(D1, W1, g1[3], scales[1], s.dt)
        _noalloc(D2, W2, g2, scales[0], 0.0, s.g, s.dt, 1)
        _noalloc(D2, W2, g2, 0.0, scales[1], 0.0, s.dt, 2)
        _noalloc(D3, W3, g3, scales[0], scales[1], s.g, s.dt, 3)
        torch.cuda.synchronize()
        _same_contacts(D2, D1)
        _same_contacts(D3, D1)
        assert int(D1.contact_dem_offset_old[-1]) > 0 and int(D1.contact_bnd_offset_old[-1]) > 0, call


def test_no_alloc_rejects_too_many_spheres():
    s, D, DB, grids = _case()
    ctx = context_for(None, None, D, DB, (None, None, grids[2], grids[3]))
    ctx.prepare(rebuild_moving=True)
    big = _lib.CtxT()
    C.memmove(C.byref(big), C.byref(ctx.ctx), C.sizeof(big))
    big.dem.n = 65537  # one more than SPHDEM_NOALLOC_MAX_DEM; rejected before any launch
    rc = ctx.lib.sphdem_contacts_noalloc(C.byref(big), 0.025, 0.01, 9.81, 1e-4, 3, ctx.stream)
    assert rc == 2
    assert b"SPHDEM_NOALLOC_MAX_DEM" in ctx.lib.sphdem_last_error()
