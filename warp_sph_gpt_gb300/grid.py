"""``HashGrid``: drop-in for ``wp.HashGrid`` (main.py:117-122, 66-87).

The reference bins points into a 64^3 *hashed* bucket table whose cell width is
the ``radius`` given to ``build``; every kernel then filters the candidates of a
query with its own distance predicate, so results depend only on the
predicates.  This grid is a dense cell box instead (no aliasing), built on the
GPU by a stable counting sort (``csrc/grid.cu``).  ``build`` records the
points and the cell width; the device work runs when a step or kernel next
needs the grid, on the stream of that call, so the per-step rebuild of
run_forward costs no extra synchronisation and can be captured in a graph.

Geometry: the lattice is anchored at the world origin (cell of x is
floor(x / radius)); the box is chosen once, from the bounding box of every
particle set of the first step that uses the grid plus a margin, and clamps at
its faces (a point outside lands in a face cell; nothing is ever missed).
"""
from __future__ import annotations

import itertools
import math
import weakref

import torch

from . import _lib

_REGISTRY: "weakref.WeakValueDictionary[int, HashGrid]" = weakref.WeakValueDictionary()
_IDS = itertools.count(1)

# Cells per instance are capped; wider cells only add candidates.
MAX_CELLS = 1 << 26


class HashGrid:
    """Neighbour grid with the ``wp.HashGrid`` call surface.

    ``dim_x, dim_y, dim_z`` are accepted for signature compatibility (the
    reference's bucket counts); the dense box is sized from the domain."""

    def __init__(self, dim_x: int = 64, dim_y: int = 64, dim_z: int = 64, device=None):
        self.dims = (int(dim_x), int(dim_y), int(dim_z))
        self.device = device
        self.points = None
        self.radius = None
        self.dirty = False
        self.built_for = None  # (data_ptr, n, radius, key) of the last device build
        self.geometry = None  # (lo[3], dim[3], cell) once resolved
        self.ninst = 1
        self.inst = None  # optional per-point instance ids (batched ensembles)
        self.buffers = None
        # cell width = radius * cell_factor; neighbour sets do not depend on it
        # (only the candidate count does), so it is a tuning parameter
        self.cell_factor = 1.0
        self.id = next(_IDS)
        _REGISTRY[self.id] = self

    @staticmethod
    def from_id(gid) -> "HashGrid":
        if isinstance(gid, HashGrid):
            return gid
        try:
            return _REGISTRY[int(gid)]
        except KeyError as exc:
            raise ValueError(f"unknown grid id {gid}") from exc

    def build(self, points: torch.Tensor, radius: float) -> None:
        """Record a (re)build over ``points`` with cell width ``radius``."""
        if not (radius > 0.0) or not math.isfinite(radius):
            raise ValueError("HashGrid.build: radius must be finite and positive")
        self.points = points
        if self.radius is not None and float(radius) != self.radius:
            self.geometry = None
        self.radius = float(radius)
        self.dirty = True

    # -- device side -----------------------------------------------------------
    def ensure_geometry(self, box_lo, box_hi, n: int, device) -> None:
        """Fix the cell box the first time (or after a radius change)."""
        if self.geometry is not None:
            return
        cell = float(torch.tensor(self.radius * self.cell_factor, dtype=torch.float32).item())
        while True:
            inv = float(torch.tensor(1.0 / cell, dtype=torch.float32).item())
            lo, dim = [], []
            for d in range(3):
                a = math.floor(box_lo[d] * inv) - 2
                b = math.floor(box_hi[d] * inv) + 2
                lo.append(int(a))
                dim.append(int(b - a + 1))
            if dim[0] * dim[1] * dim[2] <= MAX_CELLS:
                break
            cell *= 1.25
        self.geometry = (lo, dim, cell, inv)
        self._alloc(n, device)

    def _alloc(self, n: int, device) -> None:
        lo, dim, cell, inv = self.geometry
        ncl = dim[0] * dim[1] * dim[2]
        ncell = ncl * self.ninst
        lib = _lib.load()
        scratch = int(lib.sphdem_scan_scratch(ncell))
        i32 = dict(dtype=torch.int32, device=device)
        self.buffers = dict(cell_start=torch.zeros(ncell + 1, **i32), order=torch.zeros(max(n, 1), **i32),
                            key=torch.zeros(max(n, 1), **i32), cursor=torch.zeros(ncell, **i32),
                            block_sums=torch.zeros(scratch, **i32))
        self.nalloc = n

    def fill(self, g: "_lib.GridT", n: int) -> None:
        """Write this grid into a ctypes sphdem_grid_t."""
        lo, dim, cell, inv = self.geometry
        if self.nalloc < n:
            self._alloc(n, self.buffers["order"].device)
        for d in range(3):
            g.lo[d] = lo[d]
            g.dim[d] = dim[d]
        g.cell = cell
        g.inv_cell = inv
        g.ncell_local = dim[0] * dim[1] * dim[2]
        g.ninst = self.ninst
        g.n = n
        b = self.buffers
        g.cell_start = _lib.iptr(b["cell_start"])
        g.order = _lib.iptr(b["order"])
        g.key = _lib.iptr(b["key"])
        g.cursor = _lib.iptr(b["cursor"])
        g.block_sums = _lib.iptr(b["block_sums"])
        g.inst = _lib.iptr(self.inst) if self.inst is not None else _lib.c_int_p()

    def sorted_order(self) -> torch.Tensor:
        """Slot -> point index of the last device build (for tests)."""
        return self.buffers["order"][: self.nalloc]

    def cell_keys(self) -> torch.Tensor:
        """Cell key of each point of the last device build (for tests)."""
        return self.buffers["key"][: self.nalloc]


def empty_grid() -> HashGrid:
    g = HashGrid()
    g.radius = 1.0
    return g
