"""Single-kernel entry points with the reference kernels' names and arguments.

Each function runs one reference kernel (kernel/*.py) on the GPU: grids passed
as ``HashGrid`` objects or their ``.id``; struct fields read and written in
place.  ``launch(kernel, dim, inputs)`` mirrors ``wp.launch`` for these
callables.  The DEM contact entry points ``force_dem`` / ``bc_dem`` perform the
whole count -> scan -> fill -> swap sequence that the reference spreads over
Kernel_count_*, wp.utils.array_scan, two allocations and a swap
(source/Simulation.py:142-203), and return nothing; ``contact_count`` reads
the resulting edge count.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .engine import context_for


def _f32(x) -> float:
    return float(C.c_float(float(x)).value)


def _ctx(sph=None, bnd=None, dem=None, dembnd=None, grids=(None, None, None, None), wall_key=None,
         light=False):
    ctx = context_for(sph, bnd, dem, dembnd, grids)
    if light:
        ctx._fill()
        ctx._fill_grids()
        return ctx
    ctx.prepare(rebuild_moving=True, wall_key=wall_key)
    ctx.refresh()
    return ctx


def _call(fn, ctx, *args, what=""):
    _lib.check(fn(C.byref(ctx.ctx), *args, ctx.stream), what or fn.__name__)


# -- SPH ----------------------------------------------------------------------
def Kernel_shepard_sph(P_sph, P_bnd, grid_sph, grid_bnd, support, h):
    """Shepard filter P_sph.flt (kernel/KERNEL_rho.py:6-40)."""
    ctx = _ctx(P_sph, P_bnd, grids=(grid_sph, grid_bnd, None, None), wall_key=(_f32(support), _f32(h)))
    _call(ctx.lib.sphdem_shepard_sph, ctx, support, h)


def Kernel_density_sph(P_sph, P_bnd, grid_sph, grid_bnd, support, h):
    """Filtered fluid density P_sph.rho (kernel/KERNEL_rho.py:45-82)."""
    ctx = _ctx(P_sph, P_bnd, grids=(grid_sph, grid_bnd, None, None), wall_key=(_f32(support), _f32(h)))
    _call(ctx.lib.sphdem_density_sph, ctx, support, h)


def Kernel_density_bnd(P_sph, P_bnd, grid_sph, grid_bnd, support, h):
    """Raw wall density P_bnd.rho (kernel/KERNEL_rho.py:87-126)."""
    ctx = _ctx(P_sph, P_bnd, grids=(grid_sph, grid_bnd, None, None), wall_key=(_f32(support), _f32(h)))
    _call(ctx.lib.sphdem_density_bnd, ctx, support, h)


def Kernel_pres_sph(P_sph, rho0, c0, gamma):
    """Tait pressure of fluid particles (kernel/KERNEL_pres.py:6-23)."""
    ctx = _ctx(P_sph, light=True)
    _call(ctx.lib.sphdem_pres_sph, ctx, rho0, c0, gamma)


def Kernel_pres_bnd(P_bnd, rho0, c0, gamma):
    """Tait pressure of wall particles (kernel/KERNEL_pres.py:26-45)."""
    ctx = _ctx(bnd=P_bnd, light=True)
    _call(ctx.lib.sphdem_pres_bnd, ctx, rho0, c0, gamma)


def Kernel_force_sph(P_sph, P_bnd, grid_sph, grid_bnd, support, h, mu, g):
    """Pressure + Morris viscosity + gravity into P_sph.acc (kernel/KERNEL_force.py:7-71)."""
    ctx = _ctx(P_sph, P_bnd, grids=(grid_sph, grid_bnd, None, None), wall_key=(_f32(support), _f32(h)))
    _call(ctx.lib.sphdem_force_sph, ctx, support, h, mu, g)


def Kernel_step_sph(P_sph, dt):
    """Semi-implicit Euler of fluid particles (kernel/KERNEL_step.py:6-22)."""
    ctx = _ctx(P_sph, light=True)
    _call(ctx.lib.sphdem_step_sph, ctx, dt)


# -- DEM ----------------------------------------------------------------------
def force_dem(P_dem, grid_dem, radius_max, g, dt) -> None:
    """DEM-DEM contacts: count, scan, fill (Kernel_force_dem,
    kernel/KERNEL_DEM_force.py:77-135) and swap of the CSR sides."""
    ctx = _ctx(dem=P_dem, grids=(None, None, grid_dem, None))
    _call(ctx.lib.sphdem_force_dem, ctx, radius_max, g, dt)
    P_dem._flip("dem")
    ctx.post_status()


def bc_dem(P_dem, P_dem_bnd, grid_dem_bnd, radius_max, dt) -> None:
    """DEM-wall contacts: count, scan, fill (Kernel_bc_dem,
    kernel/KERNEL_DEM_BC.py:27-84) and swap; adds to force and torque."""
    ctx = _ctx(dem=P_dem, dembnd=P_dem_bnd, grids=(None, None, None, grid_dem_bnd))
    _call(ctx.lib.sphdem_bc_dem, ctx, radius_max, dt)
    P_dem._flip("bnd")
    ctx.post_status()


def contact_count(P_dem, kind: str = "dem") -> int:
    """Directed edge count E of the readable CSR side (synchronises)."""
    return int(getattr(P_dem, f"contact_{kind}_offset_old")[-1].item())


def Kernel_step_dem(P_dem, dt):
    """DEM translation and rotation update (kernel/KERNEL_DEM_step.py:6-30)."""
    ctx = _ctx(dem=P_dem, light=True)
    _call(ctx.lib.sphdem_step_dem, ctx, dt)


# -- coupling -----------------------------------------------------------------
def Kernel_prep_sphdem(P_sph, P_bnd, P_dem, grid_sph, grid_bnd, grid_dem, support, h, sph_support, sph_h,
                       eps_min, eps_max):
    """Porosity and -grad p at fluid particles
    (kernel/KERNEL_SPHDEM_interaction.py:43-115)."""
    ctx = _ctx(P_sph, P_bnd, P_dem, None, grids=(grid_sph, grid_bnd, grid_dem, None),
               wall_key=(_f32(sph_support), _f32(sph_h)))
    _call(ctx.lib.sphdem_prep_sphdem, ctx, support, h, sph_support, sph_h, eps_min, eps_max)


def Kernel_interaction_dem(P_sph, P_dem, grid_sph, grid_dem, mu, eps_min, eps_max, dt):
    """Fluid interpolation, pressure force and semi-implicit drag on DEM
    (kernel/KERNEL_SPHDEM_interaction.py:118-187)."""
    ctx = _ctx(P_sph, None, P_dem, None, grids=(grid_sph, None, grid_dem, None))
    _call(ctx.lib.sphdem_interaction_dem, ctx, mu, eps_min, eps_max, dt)


def Kernel_interaction_sph(P_sph, P_dem, grid_sph, grid_dem, support):
    """Drag reaction on the fluid (kernel/KERNEL_SPHDEM_interaction.py:190-226)."""
    ctx = _ctx(P_sph, None, P_dem, None, grids=(grid_sph, None, grid_dem, None))
    _call(ctx.lib.sphdem_interaction_sph, ctx, support)


# -- point evaluations ----------------------------------------------------------
def wendland(r: torch.Tensor, h: float):
    """W and dW/dr of the 3D Wendland C2 kernel (kernel/Kernel_KNL.py:7-41)."""
    lib = _lib.load()
    r = r.contiguous().to(torch.float32)
    w = torch.empty_like(r)
    dw = torch.empty_like(r)
    _lib.check(lib.sphdem_wendland(r.data_ptr(), r.numel(), h, w.data_ptr(), dw.data_ptr(),
                                   C.c_void_p(torch.cuda.current_stream(r.device).cuda_stream)), "wendland")
    return w, dw


def DEM_drag_beta(eps, rho, mu, diameter, speed) -> torch.Tensor:
    """beta/(1-eps) of the Ergun / Wen-Yu law, elementwise
    (kernel/KERNEL_SPHDEM_interaction.py:11-40)."""
    eps = torch.as_tensor(eps, dtype=torch.float32, device="cuda").contiguous()
    args = [torch.broadcast_to(torch.as_tensor(x, dtype=torch.float32, device=eps.device), eps.shape).contiguous()
            for x in (rho, mu, diameter, speed)]
    out = torch.empty_like(eps)
    lib = _lib.load()
    _lib.check(lib.sphdem_drag_beta(eps.data_ptr(), *(a.data_ptr() for a in args), eps.numel(), out.data_ptr(),
                                    C.c_void_p(torch.cuda.current_stream(eps.device).cuda_stream)), "drag_beta")
    return out


# -- verification / diagnostics -------------------------------------------------------
def neighbour_digest(relation: str, radius: float, P_sph=None, P_bnd=None, P_dem=None,
                     grids=(None, None, None, None)):
    """(count, hash) per subject of one neighbour relation (SPHDEM_REL_*)."""
    rel = _lib.REL[relation]
    ctx = _ctx(P_sph, P_bnd, P_dem, None, grids=grids)
    subj = {2: P_bnd, 3: P_bnd, 8: P_dem, 9: P_dem}.get(rel, P_sph)
    count = torch.zeros(subj.n, dtype=torch.int32, device=subj.device)
    hsh = torch.zeros(subj.n, dtype=torch.int64, device=subj.device)
    _lib.check(ctx.lib.sphdem_neighbour_digest(C.byref(ctx.ctx), rel, radius, count.data_ptr(), hsh.data_ptr(),
                                               ctx.stream), "neighbour_digest")
    return count, hsh


def member_digest(which: str, P_sph, P_bnd=None, P_dem=None, P_dem_bnd=None, grids=(None, None, None, None)):
    """(count, hash) per fluid particle of the member set one hot-path kernel
    decided in the last step (SPHDEM_MEMBERS_*: the density pass's recorded
    lists, the force pass's members, the porosity pass's near list).  Reads
    the step's working copies as they are: call it right after a step with the
    structs and grids of that step (the same four structs and four grids, so
    the same context), before anything re-bins them."""
    ctx = context_for(P_sph, P_bnd, P_dem, P_dem_bnd, grids)  # the step's own context and buffers
    ctx._fill()
    count = torch.zeros(P_sph.n, dtype=torch.int32, device=P_sph.device)
    hsh = torch.zeros(P_sph.n, dtype=torch.int64, device=P_sph.device)
    _lib.check(ctx.lib.sphdem_member_digest(C.byref(ctx.ctx), C.byref(ctx.params), _lib.MEMBERS[which],
                                            count.data_ptr(), hsh.data_ptr(), ctx.stream), "member_digest")
    return count, hsh


def diagnostics(P_sph, P_dem=None, g: float = 9.81) -> torch.Tensor:
    """FP64 totals: fluid mass, DEM mass, momentum xyz, translational and
    rotational kinetic energy, potential energy m g z (no reference counterpart)."""
    ctx = _ctx(P_sph, None, P_dem, None, light=True)
    out = torch.zeros(8, dtype=torch.float64, device=P_sph.device)
    _lib.check(ctx.lib.sphdem_diagnostics(C.byref(ctx.ctx), g, out.data_ptr(), ctx.stream), "diagnostics")
    return out


_SUBJECTS = {Kernel_shepard_sph: 0, Kernel_density_sph: 0, Kernel_density_bnd: 1, Kernel_pres_sph: 0,
             Kernel_pres_bnd: 0, Kernel_force_sph: 0, Kernel_step_sph: 0, Kernel_step_dem: 0,
             Kernel_prep_sphdem: 0, Kernel_interaction_dem: 1, Kernel_interaction_sph: 0}


def launch(kernel, dim: int, inputs) -> None:
    """``wp.launch`` for the entry points above: ``dim`` must equal the subject
    count the reference would launch (it is checked, not used)."""
    inputs = list(inputs)
    subject = inputs[_SUBJECTS.get(kernel, 0)]
    if hasattr(subject, "n") and int(dim) != subject.n:
        raise ValueError(f"{kernel.__name__}: dim {dim} != subject count {subject.n}")
    kernel(*inputs)
