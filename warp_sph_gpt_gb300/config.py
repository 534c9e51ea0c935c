"""Solver controls (``Solv``), restating input/Config.py:11-93 and the SPH-DEM
defaults of input/Config_SPH_DEM.py:6-15.

``BaseSolv`` carries the shared defaults of input/Config.py; ``Solv`` is the
coupled WCSPH-DEM configuration the step path uses.  Geometry and particle
properties are not here: they come from the input files (input_reader).
The 2D EISPH controls of the base class are kept as plain fields for
configuration compatibility; the EISPH solver itself is not part of this
package.
"""
from __future__ import annotations

import math
from dataclasses import dataclass


@dataclass
class BaseSolv:
    # Input files are resolved relative to the working directory, or absolute.
    input_dir: str = "input_file"
    device: str = "cuda:0"

    # Hydrodynamic solver / material.
    h: float = 0.052
    rho0: float = 1.0
    c0: float = 31.3209
    gamma: float = 7.0
    mu: float = 0.05
    g: float = 9.81
    nu: float = 0.01
    shepard_step: int = 20
    grid_slice: int = 64

    # Fixed time stepping.
    dt: float = 2.0e-3
    n_steps: int = 5000

    # Coupling controls; K, eta, mu, h belong to the DEM particle arrays.
    dem_enable: bool = False
    dem_porosity_min: float = 0.05
    dem_porosity_max: float = 1.0
    dem_dt_safety: float = 0.1

    # Output controls.
    output_step: int = 100
    gif_save: bool = True
    gif_fps: int = 20
    output_dir: str = "result/3d"
    animation_dir: str = "animation/3d"
    animation_path: str = "animation/lid_driven_cavity.gif"

    @property
    def support(self) -> float:
        """The Wendland kernel has support 2*h (input/Config.py:40-43)."""
        return 2.0 * self.h

    def _validate_common(self) -> None:
        for name in ("h", "rho0", "dt"):
            value = getattr(self, name)
            if not math.isfinite(value) or value <= 0.0:
                raise ValueError(f"{name} must be finite and positive")
        for name in ("n_steps", "output_step", "shepard_step"):
            value = getattr(self, name)
            if type(value) is not int or value < 0:
                raise ValueError(f"{name} must be a nonnegative integer")
        for name in ("grid_slice", "gif_fps"):
            value = getattr(self, name)
            if type(value) is not int or value < 1:
                raise ValueError(f"{name} must be a positive integer")

    def validate_sph(self) -> None:
        """Solver settings; particle data is validated by input_reader
        (input/Config.py:59-72)."""
        self._validate_common()
        for name in ("c0", "gamma"):
            value = getattr(self, name)
            if not math.isfinite(value) or value <= 0.0:
                raise ValueError(f"{name} must be finite and positive")
        for name in ("mu", "g"):
            value = getattr(self, name)
            if not math.isfinite(value) or value < 0.0:
                raise ValueError(f"{name} must be finite and nonnegative")
        if self.dt > 0.25 * self.h / self.c0:
            raise ValueError("dt exceeds the initial SPH acoustic limit 0.25*h/c0")
        self.validate_dem()

    def validate_dem(self) -> None:
        """Coupling controls (input/Config.py:74-81)."""
        if not self.dem_enable:
            return
        if not 0.0 < self.dem_porosity_min <= self.dem_porosity_max <= 1.0:
            raise ValueError("DEM porosity bounds must satisfy 0 < min <= max <= 1")
        if not math.isfinite(self.dem_dt_safety) or self.dem_dt_safety <= 0.0:
            raise ValueError("dem_dt_safety must be finite and positive")


@dataclass
class Solv(BaseSolv):
    """Shared configuration with the SPH-DEM defaults (input/Config_SPH_DEM.py:6-15)."""

    h: float = 0.026
    rho0: float = 1000.0
    dt: float = 1.0e-4
    n_steps: int = 9000
    output_step: int = 90
    dem_enable: bool = True
