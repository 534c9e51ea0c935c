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


# ---------------------------------------------------------------------------
# cropped copies of the benchmark dam breaks: the benchmark's resolution,
# smoothing and coupling lengths and DEM size distribution in a tank small
# enough for the CPU oracle to finish a step in about a second
# ---------------------------------------------------------------------------
def _pressed(pos, rad, tank, wall_r):
    """Deterministic contacts: sphere 0 sits 2 mm into the floor wall spheres,
    sphere 1 is moved 2 mm into sphere 0, sphere 2 presses 1.5 mm into the
    x = 0 wall.  Radii stay as sampled (unequal)."""
    pos = pos.copy()
    pos[0, 2] = rad[0] - 0.002
    d = pos[1] - pos[0]
    d[2] = 0.0
    d = d / max(np.linalg.norm(d), 1e-9)
    pos[1] = pos[0] + d * (rad[0] + rad[1] - 0.002)
    pos[1, 2] = max(pos[1, 2], rad[1] - 0.001)
    pos[2, 0] = rad[2] - 0.0015
    for k in range(3):
        pos[k, 0] = min(max(pos[k, 0], -wall_r), tank[0] + wall_r)
        pos[k, 1] = min(max(pos[k, 1], rad[k]), tank[1] - rad[k])
    return pos


def config_large_crop(seed: int = 0, n_dem: int = 12):
    """The large dam break's parameters (dx = 0.005, h = 0.0065, coupling
    h = 0.08, DEM R ~ U[0.01, 0.03] at rho 2500 placed by seeded rejection
    sampling, wall spheres r = 0.005 at spacing 0.01, dt = 2.5e-5) in a
    0.5 x 0.12 x 0.3 m tank with a 0.35 x 0.12 x 0.1 m fluid block (33,600
    fluid particles).  Spheres are sampled over the first 0.2 m of the tank
    across the water surface (z in [0.04, 0.2]), so some are submerged and the
    far end of the block has no sphere within its coupling reach; three are
    pressed into each other and into the walls."""
    from warp_sph_gpt_gb300.generate import CoupledGenerationConfig, _rejection_sample

    gen = CoupledGenerationConfig(device="cpu", dx=0.005, h=0.0065, dt=2.5e-5, tank_width=0.5, tank_depth=0.12,
                                  tank_height=0.3, fluid_width=0.35, fluid_depth=0.12, fluid_height=0.1,
                                  dem_radius=0.03, dem_bnd_radius=0.005, dem_bnd_spacing=0.01, dem_nx=1,
                                  dem_ny=1, dem_nz=1, dem_origin_x=0.1, dem_origin_y=0.06, dem_origin_z=0.2)
    rng = np.random.default_rng(seed)
    pos, rad = _rejection_sample(rng, n_dem, (0.0, 0.2), (0.0, gen.tank_depth), (0.04, 0.2),
                                 lambda r: r.uniform(0.01, 0.03))
    return gen, _pressed(pos, rad, (gen.tank_width, gen.tank_depth), gen.dem_bnd_radius), rad


def config_scaled_crop(seed: int = 0):
    """The scaled dam break's parameters (dx = 0.01, h = 0.013, coupling h =
    0.08, R = 0.025 spheres on a lattice at spacing 0.065 jittered by
    U(+-0.005) from default_rng(seed), wall spheres r = 0.005, dt = 5e-5) in a
    0.4 x 0.2 x 0.4 m tank with a 0.25 x 0.2 x 0.15 m fluid block (7,500
    fluid particles); a 4 x 2 x 2 lattice from (0.05, 0.05, 0.1) straddles the
    water surface, and three spheres are pressed into each other and into the
    walls."""
    from warp_sph_gpt_gb300.generate import CoupledGenerationConfig, DEMPtlGeneration

    gen = CoupledGenerationConfig(device="cpu", dx=0.01, h=0.013, dt=5.0e-5, tank_width=0.4, tank_depth=0.2,
                                  tank_height=0.4, fluid_width=0.25, fluid_depth=0.2, fluid_height=0.15,
                                  dem_nx=4, dem_ny=2, dem_nz=2, dem_origin_x=0.05, dem_origin_y=0.05,
                                  dem_origin_z=0.1, dem_bnd_radius=0.005, dem_bnd_spacing=0.01)
    base = DEMPtlGeneration(gen).dem_particle()
    rng = np.random.default_rng(seed)
    pos = base + rng.uniform(-0.005, 0.005, size=base.shape)
    rad = np.full(len(pos), gen.dem_radius)
    return gen, _pressed(pos, rad, (gen.tank_width, gen.tank_depth), gen.dem_bnd_radius), None
