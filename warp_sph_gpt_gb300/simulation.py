"""Step API: ``SPH_OneStep`` and ``SPHDEM_OneStep`` (source/Simulation.py:17-221)
and the forward driver ``run_forward`` (main.py:38-98).

Same signatures, same in-place semantics and the same ordering contract as the
reference; the arithmetic runs in libsphdem (hand-written sm_103a kernels).
Moving grids (fluid, DEM) are re-binned from the current positions inside
every step, fixed grids (walls) when their ``build`` was called, so a caller
that follows the reference contract -- rebuild moving grids each step, fixed
grids once -- gets exactly its semantics.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .engine import context_for
from .input_reader import dem_search_scales, validate_dem_particles


def _shepard_due(solv, step: int) -> bool:
    return step == 0 or (solv.shepard_step > 0 and step % solv.shepard_step == 0)


def SPH_OneStep(solv, P_sph, P_bnd, grid_sph, grid_bnd, step: int, integrate: bool = True) -> None:
    """One WCSPH step: [Shepard] -> density -> Tait pressure -> force ->
    [symplectic Euler] (source/Simulation.py:17-99).  Writes P_sph.flt (on
    Shepard steps), rho, pres, acc (and vel, pos when integrate); P_bnd.rho,
    P_bnd.pres."""
    ctx = context_for(P_sph, P_bnd, None, None, (grid_sph, grid_bnd, None, None))
    ctx.set_params(solv)
    ctx.poll_status()
    ctx.prepare(rebuild_moving=True, wall_key=(float(C.c_float(solv.support).value),
                                               float(C.c_float(solv.h).value)))
    _lib.check(ctx.lib.sphdem_sph_onestep(C.byref(ctx.ctx), C.byref(ctx.params), int(step), int(bool(integrate)),
                                          ctx.stream), "SPH_OneStep")


def SPHDEM_OneStep(solv, P_sph, P_bnd, P_dem, P_dem_bnd, grid_sph, grid_bnd, grid_dem, grid_dem_bnd, step: int,
                   search_scales=None) -> None:
    """One coupled step at a common time level (source/Simulation.py:102-221):
    SPH fields and forces -> DEM-DEM and DEM-wall contacts with CSR history
    rebuild and swap -> porosity and -grad p -> fluid-to-DEM pressure and drag
    -> drag reaction on the fluid -> SPH and DEM integration.  The moving grids
    are re-binned inside the step; the step is replayed from the same CUDA
    graph as run_steps (one per Shepard cadence variant)."""
    run_steps(solv, P_sph, P_bnd, grid_sph, grid_bnd, P_dem, P_dem_bnd, grid_dem, grid_dem_bnd, first_step=step,
              n_steps=1, search_scales=search_scales)


def run_steps(solv, P_sph, P_bnd, grid_sph, grid_bnd, P_dem=None, P_dem_bnd=None, grid_dem=None,
              grid_dem_bnd=None, first_step: int = 0, n_steps: int = 1, search_scales=None) -> None:
    """``n_steps`` consecutive steps of run_forward's loop body (main.py:84-91)
    -- moving-grid rebuild plus one step -- replayed from CUDA graphs (one per
    Shepard cadence variant).  Equivalent to calling the step API in a loop."""
    coupled = P_dem is not None
    if coupled:
        scales = dem_search_scales(P_dem, P_dem_bnd) if search_scales is None else search_scales
        ctx = context_for(P_sph, P_bnd, P_dem, P_dem_bnd, (grid_sph, grid_bnd, grid_dem, grid_dem_bnd))
        ctx.set_params(solv, scales)
    else:
        ctx = context_for(P_sph, P_bnd, None, None, (grid_sph, grid_bnd, None, None))
        ctx.set_params(solv)
    ctx.poll_status()
    ctx.prepare(rebuild_moving=False, wall_key=(float(C.c_float(solv.support).value),
                                                float(C.c_float(solv.h).value)))
    _lib.check(ctx.lib.sphdem_run(C.byref(ctx.ctx), C.byref(ctx.params), int(first_step), int(n_steps),
                                  int(coupled), ctx.stream), "run_steps")
    if coupled:
        if n_steps % 2:
            P_dem._flip("dem")
            P_dem._flip("bnd")
        ctx.post_status()


def check_status(P) -> None:
    """Blocking check of the device status bits of every context of P."""
    for ctx in P.__dict__.get("_sphdem_contexts", {}).values():
        ctx.check_status()


def run_forward(solv, P_sph, P_bnd, grid_sph, grid_bnd, P_dem=None, P_dem_bnd=None, grid_dem=None,
                grid_dem_bnd=None, on_frame=None, use_graphs: bool = True) -> None:
    """Forward SPH or coupled SPH-DEM run (main.py:38-98).

    Fixed grids are built once, moving grids every step.  ``on_frame(step)`` is
    called for the initial state, every ``output_step`` steps and for the final
    state, with the device state current (file output is the caller's)."""
    print(f"\n[forward] {solv.n_steps} step \t\t (t={solv.n_steps * solv.dt:.3f} s\tdt={solv.dt:.1e} s)\n")
    grid_bnd.build(P_bnd.pos, solv.support)
    coupled = solv.dem_enable and P_dem is not None
    if solv.dem_enable and not coupled:
        raise ValueError("DEM is enabled: provide DEM particles, boundaries and coupling grids")
    scales = None
    if coupled:
        scales = validate_dem_particles(solv, P_dem, P_dem_bnd)
        grid_dem_bnd.build(P_dem_bnd.pos, max(2.0 * scales[1], solv.support))
    grid_sph.build(P_sph.pos, solv.support)
    if coupled:
        grid_dem.build(P_dem.pos, max(2.0 * scales[0], 2.0 * scales[2]))
    if on_frame is not None and solv.output_step > 0:
        on_frame(0)
    step = 0
    chunk = solv.output_step if solv.output_step > 0 else solv.n_steps
    while step < solv.n_steps:
        n = min(chunk - step % chunk if chunk else solv.n_steps, solv.n_steps - step)
        if use_graphs:
            run_steps(solv, P_sph, P_bnd, grid_sph, grid_bnd, P_dem if coupled else None,
                      P_dem_bnd if coupled else None, grid_dem, grid_dem_bnd, first_step=step, n_steps=n,
                      search_scales=scales)
        else:
            for s in range(step, step + n):
                if coupled:
                    SPHDEM_OneStep(solv, P_sph, P_bnd, P_dem, P_dem_bnd, grid_sph, grid_bnd, grid_dem,
                                   grid_dem_bnd, s, scales)
                else:
                    SPH_OneStep(solv, P_sph, P_bnd, grid_sph, grid_bnd, s)
        step += n
        if on_frame is not None and solv.output_step > 0 and (step % solv.output_step == 0
                                                             or step == solv.n_steps):
            on_frame(step)
            print(f"[output] step {step:>6d} / {solv.n_steps}\t t={step * solv.dt:.4f} s")
    torch.cuda.current_stream().synchronize()
    for P in (P_sph, P_dem):
        if P is not None:
            check_status(P)
