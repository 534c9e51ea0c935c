"""Initial-condition generators (restating input_gen/: config.py, gen_ptl.py,
gen_dem.py, generate.py) plus the seeded scaled / batched dam-break cases.

The lattice generators follow the reference rules exactly -- same meshgrid
order, same integer shell masks, same float32 rounding, same ``%.9g`` writer
-- so the four config-1 input files they write are byte-identical to the
reference's ``input_file/input_{SPH,BND,DEM,DEMBND}.txt``.  The scaled cases
(dx = 0.01; the 800k / 4.8M tank; the 64-instance ensemble) use the same rules
with seeded jitter or rejection sampling from ``numpy.random.default_rng``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, fields
from pathlib import Path

import numpy as np
import torch

from .config import Solv
from .input_reader import INPUT_FIELDS, column_indices
from .struct import BNDptl, DEMBNDptl, DEMptl, SPHptl


@dataclass
class GenerationConfig:
    """Geometry and material presets (input_gen/config.py:11-352)."""

    device: str = "cpu"
    dx: float = 0.04
    tank_width: float = 2.0
    tank_height: float = 1.0
    tank_depth: float = 0.4
    fluid_width: float = 0.5
    fluid_height: float = 0.5
    fluid_depth: float = 0.4
    fluid_origin_x: float = 0.0
    fluid_origin_y: float = 0.0
    fluid_origin_z: float = 0.0
    bnd_layer: int = 3
    h: float | None = None
    support: float | None = None
    rho0: float = 1.0
    gamma: float = 7.0
    c0: float = 31.3209
    mu: float = 0.05
    g: float = 9.81
    h_factor: float = 1.3
    shepard_step: int = 20
    dt: float = 2.0e-3
    n_steps: int = 5000
    output_step: int = 100
    gif_save: bool = True
    output_dir: str = "result/3d"
    animation_dir: str = "animation/3d"
    grid_slice: int = 64
    dem_enable: bool = False
    dem_radius: float = 0.025
    dem_rho: float = 2500.0
    dem_K: float = 2.0e4
    dem_eta: float = 4.0
    dem_mu: float = 0.3
    dem_inertia_factor: float = 0.4
    dem_nx: int = 5
    dem_ny: int = 2
    dem_nz: int = 2
    dem_spacing: float = 0.065
    dem_origin_x: float = 0.12
    dem_origin_y: float = 0.1675
    dem_origin_z: float = 0.62
    dem_vel_x: float = 0.0
    dem_vel_y: float = 0.0
    dem_vel_z: float = 0.0
    dem_omega_x: float = 0.0
    dem_omega_y: float = 0.0
    dem_omega_z: float = 0.0
    dem_bnd_radius: float = 0.01
    dem_bnd_rho: float = 2500.0
    dem_bnd_spacing: float = 0.02
    dem_h: float = 0.08
    dem_porosity_min: float = 0.05
    dem_porosity_max: float = 1.0
    dem_dt_safety: float = 0.1

    def __post_init__(self) -> None:
        if self.h is None:
            self.h = self.h_factor * self.dx
        if self.support is None:
            self.support = 2.0 * self.h

    @property
    def dem_volume(self) -> float:
        return (4.0 / 3.0) * math.pi * self.dem_radius ** 3

    @property
    def dem_mass(self) -> float:
        return self.dem_rho * self.dem_volume

    @property
    def dem_inertia(self) -> float:
        return self.dem_inertia_factor * self.dem_mass * self.dem_radius ** 2

    @property
    def dem_bnd_volume(self) -> float:
        return (4.0 / 3.0) * math.pi * self.dem_bnd_radius ** 3

    @property
    def dem_bnd_mass(self) -> float:
        return self.dem_bnd_rho * self.dem_bnd_volume

    @property
    def dem_bnd_inertia(self) -> float:
        return self.dem_inertia_factor * self.dem_bnd_mass * self.dem_bnd_radius ** 2

    @property
    def dem_support(self) -> float:
        return 2.0 * self.dem_h

    def validate_sph(self) -> None:
        """3D SPH domain, lattice, material and time step (input_gen/config.py:230-267)."""
        for name in ("dx", "h", "support", "tank_width", "tank_height", "tank_depth", "fluid_width",
                     "fluid_height", "fluid_depth", "rho0", "c0", "gamma", "dt"):
            value = getattr(self, name)
            if not math.isfinite(value) or value <= 0.0:
                raise ValueError(f"{name} must be finite and positive")
        if not math.isclose(self.support, 2.0 * self.h):
            raise ValueError("Wendland support must equal 2*h")
        if self.dt > 0.25 * self.h / self.c0:
            raise ValueError("dt exceeds the initial SPH acoustic limit 0.25*h/c0")
        for name in ("g", "mu"):
            if not math.isfinite(getattr(self, name)) or getattr(self, name) < 0.0:
                raise ValueError(f"{name} must be finite and nonnegative")
        for name in ("bnd_layer", "grid_slice"):
            if not isinstance(getattr(self, name), int) or getattr(self, name) < 1:
                raise ValueError(f"{name} must be a positive integer")
        for name in ("n_steps", "output_step", "shepard_step"):
            if not isinstance(getattr(self, name), int) or getattr(self, name) < 0:
                raise ValueError(f"{name} must be a nonnegative integer")
        for name in ("tank_width", "tank_height", "tank_depth"):
            cells = getattr(self, name) / self.dx
            if not math.isclose(cells, round(cells), abs_tol=1.0e-8):
                raise ValueError(f"{name} must be an integer multiple of dx")
        for axis, extent, tank in (("x", self.fluid_width, self.tank_width), ("y", self.fluid_depth, self.tank_depth),
                                   ("z", self.fluid_height, self.tank_height)):
            origin = getattr(self, "fluid_origin_" + axis)
            if (not math.isfinite(origin) or origin < 0.0 or origin + extent > tank + 1.0e-12
                    or round(extent / self.dx) < 1):
                raise ValueError(f"initial fluid block must fit the tank along {axis}")

    def validate_dem(self) -> None:
        """DEM material, spacing, porosity bounds and contact time step
        (input_gen/config.py:304-352)."""
        if not self.dem_enable:
            return
        for name in ("dem_radius", "dem_rho", "dem_K", "dem_inertia_factor", "dem_bnd_radius", "dem_bnd_rho",
                     "dem_bnd_spacing", "dem_h", "dem_dt_safety", "dt"):
            value = getattr(self, name)
            if not math.isfinite(value) or value <= 0.0:
                raise ValueError(f"{name} must be finite and positive")
        if (not math.isfinite(self.dem_eta) or not math.isfinite(self.dem_mu) or self.dem_eta < 0.0
                or self.dem_mu < 0.0):
            raise ValueError("dem_eta and dem_mu must be nonnegative")
        if any(not isinstance(n, int) or n < 1 for n in (self.dem_nx, self.dem_ny, self.dem_nz)):
            raise ValueError("dem_nx, dem_ny and dem_nz must be positive integers")
        if not math.isfinite(self.dem_spacing) or self.dem_spacing < 2.0 * self.dem_radius:
            raise ValueError("initial DEM particles must not overlap")
        if self.dem_bnd_spacing > 2.0 * self.dem_bnd_radius:
            raise ValueError("DEM boundary spacing must not exceed the boundary diameter")
        if self.dem_bnd_spacing / math.sqrt(2.0) >= self.dem_radius + self.dem_bnd_radius:
            raise ValueError("DEM boundary pores must be smaller than the moving spheres")
        for name in ("dem_origin_x", "dem_origin_y", "dem_origin_z", "dem_vel_x", "dem_vel_y", "dem_vel_z",
                     "dem_omega_x", "dem_omega_y", "dem_omega_z"):
            if not math.isfinite(getattr(self, name)):
                raise ValueError(f"{name} must be finite")
        if not 0.0 < self.dem_porosity_min <= self.dem_porosity_max <= 1.0:
            raise ValueError("DEM porosity bounds must satisfy 0 < min <= max <= 1")
        mass_eff = 0.5 * self.dem_mass
        dt_contact = self.dem_dt_safety * min(math.sqrt(mass_eff / self.dem_K), mass_eff / max(self.dem_eta, 1.0e-20))
        if self.dt > dt_contact:
            raise ValueError(f"dt exceeds DEM contact limit {dt_contact:.6g} s")


@dataclass
class CoupledGenerationConfig(GenerationConfig):
    """The 3D SPH-DEM example defaults (input_gen/config.py:355-363)."""

    dx: float = 0.02
    rho0: float = 1000.0
    dt: float = 1.0e-4
    n_steps: int = 9000
    output_step: int = 90
    dem_enable: bool = True


def _f32(a) -> np.ndarray:
    return np.asarray(a, dtype=np.float32)


class DamPtlGeneration:
    """Fluid block and 3-layer dummy walls (input_gen/gen_ptl.py:7-101)."""

    def __init__(self, solv: GenerationConfig) -> None:
        self.solv = solv
        self.dx = solv.dx
        self.bnd_layer = solv.bnd_layer

    def fluid_particle(self) -> np.ndarray:
        s, dx = self.solv, self.dx
        n_x, n_y, n_z = (int(round(s.fluid_width / dx)), int(round(s.fluid_depth / dx)),
                         int(round(s.fluid_height / dx)))
        gx, gy, gz = np.meshgrid(s.fluid_origin_x + np.arange(n_x) * dx, s.fluid_origin_y + np.arange(n_y) * dx,
                                 s.fluid_origin_z + np.arange(n_z) * dx, indexing="ij")
        return np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)

    def boundary_particle(self) -> np.ndarray:
        """Bottom, left, right, front and back walls; every edge/corner once."""
        s, dx, bnd = self.solv, self.dx, self.bnd_layer
        nx, ny, nz = (int(round(s.tank_width / dx)), int(round(s.tank_depth / dx)), int(round(s.tank_height / dx)))
        gx, gy, gz = np.meshgrid(np.arange(-bnd, nx + bnd), np.arange(-bnd, ny + bnd), np.arange(-bnd, nz + bnd),
                                 indexing="ij")
        wall = (gz < 0) | (gx < 0) | (gx >= nx) | (gy < 0) | (gy >= ny)
        return np.stack([gx[wall], gy[wall], gz[wall]], axis=1) * dx

    def build(self, device=None) -> tuple[SPHptl, BNDptl]:
        s = self.solv
        s.validate_sph()
        dev = device or s.device
        fluid, wall = self.fluid_particle(), self.boundary_particle()
        mass = s.rho0 * s.dx ** 3
        sph = SPHptl(len(fluid), dev)
        sph.pos = torch.as_tensor(_f32(fluid), device=dev)
        sph.rho_raw.fill_(s.rho0)
        sph.rho.fill_(s.rho0)
        sph.m.fill_(mass)
        sph.porosity.fill_(1.0)
        bnd = BNDptl(len(wall), dev)
        bnd.pos = torch.as_tensor(_f32(wall), device=dev)
        bnd.rho_raw.fill_(s.rho0)
        bnd.rho.fill_(s.rho0)
        bnd.m.fill_(mass)
        return sph, bnd


class DEMPtlGeneration:
    """Moving DEM lattice and fixed wall spheres (input_gen/gen_dem.py:8-125)."""

    def __init__(self, solv: GenerationConfig) -> None:
        self.solv = solv

    def dem_particle(self) -> np.ndarray:
        s = self.solv
        gx, gy, gz = np.meshgrid(s.dem_origin_x + np.arange(s.dem_nx) * s.dem_spacing,
                                 s.dem_origin_y + np.arange(s.dem_ny) * s.dem_spacing,
                                 s.dem_origin_z + np.arange(s.dem_nz) * s.dem_spacing, indexing="ij")
        pos = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)
        _check_inside(pos, np.full(len(pos), s.dem_radius), s)
        return pos

    def boundary_particle(self) -> np.ndarray:
        """Wall sphere centres one radius outside the tank, spacing <= dem_bnd_spacing."""
        s = self.solv
        r = s.dem_bnd_radius
        nx = int(np.ceil((s.tank_width + 2.0 * r) / s.dem_bnd_spacing))
        ny = int(np.ceil((s.tank_depth + 2.0 * r) / s.dem_bnd_spacing))
        nz = int(np.ceil((s.tank_height + r) / s.dem_bnd_spacing))
        x = np.linspace(-r, s.tank_width + r, nx + 1)
        y = np.linspace(-r, s.tank_depth + r, ny + 1)
        z = np.linspace(-r, s.tank_height, nz + 1)
        gx, gy, gz = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
        wall = (gz == 0) | (gx == 0) | (gx == nx) | (gy == 0) | (gy == ny)
        return np.stack([x[gx[wall]], y[gy[wall]], z[gz[wall]]], axis=1)

    def build(self, device=None, positions=None, radii=None) -> tuple[DEMptl, DEMBNDptl]:
        s = self.solv
        s.validate_dem()
        dev = device or s.device
        dem_pos = self.dem_particle() if positions is None else np.asarray(positions, dtype=np.float64)
        wall_pos = self.boundary_particle()
        nd, nw = len(dem_pos), len(wall_pos)
        rad = np.full(nd, s.dem_radius) if radii is None else np.asarray(radii, dtype=np.float64)
        vol = (4.0 / 3.0) * math.pi * rad ** 3
        mass = s.dem_rho * vol
        dem = DEMptl(nd, dev)
        dem.pos = torch.as_tensor(_f32(dem_pos), device=dev)
        dem.radius = torch.as_tensor(_f32(rad), device=dev)
        dem.rho.fill_(s.dem_rho)
        dem.m = torch.as_tensor(_f32(mass), device=dev)
        dem.volume = torch.as_tensor(_f32(vol), device=dev)
        dem.inertia = torch.as_tensor(_f32(s.dem_inertia_factor * mass * rad ** 2), device=dev)
        for key, value in (("K", s.dem_K), ("eta", s.dem_eta), ("mu", s.dem_mu), ("h", s.dem_h)):
            getattr(dem, key).fill_(value)
        dem.vel[:] = torch.tensor([s.dem_vel_x, s.dem_vel_y, s.dem_vel_z], dtype=torch.float32)
        dem.omega[:] = torch.tensor([s.dem_omega_x, s.dem_omega_y, s.dem_omega_z], dtype=torch.float32)
        dem.porosity.fill_(1.0)
        wall = DEMBNDptl(nw, dev)
        wall.pos = torch.as_tensor(_f32(wall_pos), device=dev)
        for key, value in (("radius", s.dem_bnd_radius), ("rho", s.dem_bnd_rho), ("m", s.dem_bnd_mass),
                           ("volume", s.dem_bnd_volume), ("inertia", s.dem_bnd_inertia), ("K", s.dem_K),
                           ("eta", s.dem_eta), ("mu", s.dem_mu)):
            getattr(wall, key).fill_(value)
        return dem, wall


def _check_inside(pos: np.ndarray, radius: np.ndarray, s: GenerationConfig) -> None:
    """Sphere extents against the five closed tank sides (input_gen/gen_dem.py:38-44)."""
    if len(pos) and ((pos[:, 0] - radius).min() < 0.0 or (pos[:, 0] + radius).max() > s.tank_width
                     or (pos[:, 1] - radius).min() < 0.0 or (pos[:, 1] + radius).max() > s.tank_depth
                     or (pos[:, 2] - radius).min() < 0.0):
        raise ValueError("initial DEM spheres must lie inside the tank walls")


def write_particle_file(path: str | Path, kind: str, particle) -> Path:
    """Input fields only, numeric-ID header, ``%.9g`` tab separated
    (input_gen/generate.py:20-31): nine significant digits round-trip float32."""
    destination = Path(path)
    destination.parent.mkdir(parents=True, exist_ok=True)
    n = particle.pos.shape[0]
    columns = [getattr(particle, name).detach().cpu().numpy().reshape(n, width)
               for name, width in INPUT_FIELDS[kind]]
    header = "\t".join(str(i) for ids in column_indices(kind).values() for i in ids)
    np.savetxt(destination, np.concatenate(columns, axis=1) if columns else np.zeros((0, 0)), fmt="%.9g",
               delimiter="\t", header=header, comments="", encoding="utf-8")
    return destination


def generate_files(output_dir: str | Path, coupled: CoupledGenerationConfig | None = None,
                   dem_positions=None, dem_radii=None) -> dict[str, Path]:
    """The four WCSPH-DEM input files of one configuration (input_gen/generate.py:34-45)."""
    coupled = CoupledGenerationConfig(device="cpu") if coupled is None else coupled
    parts = dict(zip(("SPH", "BND"), DamPtlGeneration(coupled).build("cpu")))
    parts.update(zip(("DEM", "DEMBND"), DEMPtlGeneration(coupled).build("cpu", dem_positions, dem_radii)))
    return {kind: write_particle_file(Path(output_dir) / f"input_{kind}.txt", kind, p) for kind, p in parts.items()}


def solver_config(gen: GenerationConfig, **overrides) -> Solv:
    """Runtime Solv carrying the generator's solver fields."""
    values = {f.name: getattr(gen, f.name) for f in fields(Solv) if hasattr(gen, f.name)}
    values.update(overrides)
    return Solv(**values)


# ---------------------------------------------------------------------------
# seeded benchmark configurations
# ---------------------------------------------------------------------------
def config_small() -> CoupledGenerationConfig:
    """Config 1: the reference's own input files (12,500 / 48,336 / 20 / 14,688)."""
    return CoupledGenerationConfig(device="cpu", h=0.026)


def config_scaled(seed: int = 0):
    """Config 2: dx = 0.01, h = 0.013, 160 DEM (10x4x4, spacing 0.065, first
    centre (0.12, 0.1025, 0.62)) each jittered by U(+-0.005) from
    default_rng(seed); wall spheres r = 0.005; dt = 5e-5."""
    gen = CoupledGenerationConfig(device="cpu", dx=0.01, h=0.013, dt=5.0e-5, dem_nx=10, dem_ny=4, dem_nz=4,
                                  dem_origin_x=0.12, dem_origin_y=0.1025, dem_origin_z=0.62,
                                  dem_bnd_radius=0.005, dem_bnd_spacing=0.01)
    base = DEMPtlGeneration(gen).dem_particle()
    rng = np.random.default_rng(seed)
    pos = base + rng.uniform(-0.005, 0.005, size=base.shape)
    return gen, pos, None


def config_large(fluid_width: float = 1.0, seed: int = 0, n_dem: int = 2000):
    """Config 3: tank 4 x 0.8 x 1.5, fluid 1.0 (or subsampled x-extent) x 0.8 x
    0.75 at dx = 0.005 (h = 0.0065), n_dem spheres R ~ U[0.01, 0.03], rho 2500,
    placed without overlap by rejection sampling in the upper half of the tank
    (z in [0.75, 1.5]) with default_rng(seed); wall spheres r = 0.005 at
    spacing 0.01; dt = 2.5e-5.  fluid_width = 0.167 gives the 792,000-particle
    variant (33 columns)."""
    gen = CoupledGenerationConfig(device="cpu", dx=0.005, h=0.0065, dt=2.5e-5, tank_width=4.0, tank_depth=0.8,
                                  tank_height=1.5, fluid_width=fluid_width, fluid_depth=0.8, fluid_height=0.75,
                                  dem_radius=0.03, dem_bnd_radius=0.005, dem_bnd_spacing=0.01, dem_nx=1,
                                  dem_ny=1, dem_nz=1, dem_origin_x=0.5, dem_origin_y=0.4, dem_origin_z=1.0)
    rng = np.random.default_rng(seed)
    pos, rad = _rejection_sample(rng, n_dem, (0.0, gen.tank_width), (0.0, gen.tank_depth), (0.75, 1.5),
                                 lambda r: r.uniform(0.01, 0.03))
    return gen, pos, rad


def _rejection_sample(rng, n, xr, yr, zr, radius_fn, max_tries: int = 2_000_000):
    """Non-overlapping spheres inside a box (seeded, deterministic)."""
    cell = 0.06
    buckets: dict[tuple, list[int]] = {}
    pos, rad = [], []
    tries = 0
    while len(pos) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"rejection sampling placed only {len(pos)} of {n} spheres")
        r = float(radius_fn(rng))
        p = np.array([rng.uniform(xr[0] + r, xr[1] - r), rng.uniform(yr[0] + r, yr[1] - r),
                      rng.uniform(zr[0] + r, zr[1] - r)])
        key = tuple((p // cell).astype(int))
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for k in buckets.get((key[0] + dx, key[1] + dy, key[2] + dz), ()):
                        if np.linalg.norm(pos[k] - p) < rad[k] + r:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            buckets.setdefault(key, []).append(len(pos))
            pos.append(p)
            rad.append(r)
    return np.array(pos), np.array(rad)


def config_batch_member(i: int):
    """Config 4 member i: dx = 0.02 in the 2 x 0.4 x 1 tank, fluid x-length
    U[0.3, 0.7] and height U[0.3, 0.6] (default_rng(i)), DEM count U{0..40},
    R = 0.025, non-overlapping above the water; dt = 1e-4."""
    rng = np.random.default_rng(i)
    width = float(rng.uniform(0.3, 0.7))
    height = float(rng.uniform(0.3, 0.6))
    n_dem = int(rng.integers(0, 41))
    width = round(width / 0.02) * 0.02
    height = round(height / 0.02) * 0.02
    gen = CoupledGenerationConfig(device="cpu", h=0.026, fluid_width=width, fluid_height=height)
    if n_dem:
        pos, rad = _rejection_sample(rng, n_dem, (0.0, gen.tank_width), (0.0, gen.tank_depth),
                                     (height + 0.05, gen.tank_height), lambda r: 0.025)
    else:
        pos, rad = np.zeros((0, 3)), np.zeros(0)
    return gen, pos, rad


def build_case(gen: GenerationConfig, dem_positions=None, dem_radii=None, device="cuda"):
    """SPHptl, BNDptl, DEMptl, DEMBNDptl of one generated case on ``device``."""
    sph, bnd = DamPtlGeneration(gen).build(device)
    dem, wall = DEMPtlGeneration(gen).build(device, dem_positions, dem_radii)
    return sph, bnd, dem, wall
