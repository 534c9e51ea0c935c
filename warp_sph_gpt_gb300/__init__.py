"""GB300-native WCSPH-DEM time step of hojin9908/Warp_SPH_GPT.

Drop-in for the reference's step path: ``SPHDEM_OneStep`` / ``SPH_OneStep``
(source/Simulation.py), the ``SPHptl``/``BNDptl``/``DEMptl``/``DEMBNDptl``
field layout (input/struct.py), ``input_parser`` and the particle text format
(input/input_reader.py), ``Solv`` (input/Config*.py), and ``HashGrid`` in place
of ``wp.HashGrid``.  All arithmetic runs in libsphdem.so, hand-written CUDA for
sm_103a, on PyTorch-owned device buffers; importing the package does not load
the library, the first step does (and fails loudly without it).
"""
from .config import BaseSolv, Solv
from .grid import HashGrid
from .input_reader import (INPUT_FIELDS, column_indices, dem_search_scales, input_parser, load_sph_particles,
                           validate_dem_particles)
from .simulation import SPH_OneStep, SPHDEM_OneStep, check_status, run_forward, run_steps
from .struct import BNDptl, DEMBNDptl, DEMptl, SPHptl

__all__ = ["BaseSolv", "Solv", "HashGrid", "INPUT_FIELDS", "column_indices", "dem_search_scales", "input_parser",
           "load_sph_particles", "validate_dem_particles", "SPH_OneStep", "SPHDEM_OneStep", "check_status",
           "run_forward", "run_steps", "SPHptl", "BNDptl", "DEMptl", "DEMBNDptl"]
