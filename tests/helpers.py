"""Test fixtures restating the reference's own (tests/test_dem.py:40-146)."""
from __future__ import annotations

import numpy as np
import torch

from warp_sph_gpt_gb300 import HashGrid
from warp_sph_gpt_gb300.generate import CoupledGenerationConfig, DamPtlGeneration, DEMPtlGeneration
from warp_sph_gpt_gb300.kernels import bc_dem, contact_count, force_dem


def gen_config(**kwargs) -> CoupledGenerationConfig:
    """The compact dam break of tests/test_dem.py:52-56 (dx = 0.04)."""
    settings = dict(dx=0.04, h=0.052, support=0.104, tank_width=0.8, tank_height=0.8, tank_depth=0.32,
                    fluid_width=0.4, fluid_height=0.4, fluid_depth=0.32, dem_nx=2, dem_ny=1, dem_nz=1,
                    dem_origin_y=0.16, dem_origin_z=0.60, grid_slice=32)
    settings.update(kwargs)
    return CoupledGenerationConfig(device="cuda", **settings)


def scene(device="cuda", **kwargs):
    """solv, fluid, wall, DEM, DEM wall and four grids built at the initial
    positions (tests/test_dem.py:40-66)."""
    solv = gen_config(**kwargs)
    P, B = DamPtlGeneration(solv).build(device)
    D, DB = DEMPtlGeneration(solv).build(device)
    grids = [HashGrid(32, 32, 32) for _ in range(4)]
    for grid, part, radius in zip(grids, (P, B, D, DB),
                                  (solv.support, solv.support, solv.dem_support, 2 * solv.dem_bnd_radius)):
        grid.build(part.pos, radius)
    return solv, P, B, D, DB, grids


def run_force_dem(D, grid, radius_max, g, dt) -> int:
    force_dem(D, grid, radius_max, g, dt)
    return contact_count(D, "dem")


def run_bc_dem(D, DB, grid, radius_max, dt) -> int:
    bc_dem(D, DB, grid, radius_max, dt)
    return contact_count(D, "bnd")


def contact_history(D, kind, subject, neighbour) -> np.ndarray:
    """One history by stable pair ids (tests/test_dem.py:75-83)."""
    offsets = getattr(D, f"contact_{kind}_offset_old").cpu().numpy()
    ids = getattr(D, f"contact_{kind}_id_old").cpu().numpy()
    tang = getattr(D, f"tang_{kind}_old").cpu().numpy()
    for k in range(int(offsets[subject]), int(offsets[subject + 1])):
        if int(ids[k]) == neighbour:
            return tang[k]
    raise KeyError((kind, subject, neighbour))


def assign(t: torch.Tensor, values) -> None:
    t.copy_(torch.as_tensor(np.asarray(values, dtype=np.float32), device=t.device))


def field_err(got, ref) -> float:
    """max |got - ref| / max |ref|: the field-normalised error.  Pointwise
    relative error is not meaningful for the Tait pressure near rest, where
    B((rho/rho0)^7 - 1) cancels."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = max(np.abs(ref).max(), 1e-30) if ref.size else 1.0
    return float(np.abs(got - ref).max() / scale) if ref.size else 0.0
