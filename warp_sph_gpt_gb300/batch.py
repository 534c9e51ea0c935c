"""Batched ensembles: many independent dam breaks advanced as one state.

The members (each an initial configuration of the same tank and solver
controls, e.g. the 64 seeded dam breaks of ``generate.config_batch_member``)
are concatenated into one flattened ``SPHptl``/``BNDptl``/``DEMptl``/
``DEMBNDptl`` state with a per-particle instance id.  Every grid then keys its
cells by (instance, cell), so neighbour searches never cross members, and each
phase of the step is one kernel launch over all members; the whole step is
replayed from one CUDA graph.  A member's particles keep their relative order
and the cell lattice is anchored at the world origin, so every member
evolves bit for bit as it would alone (tests/test_gpu_batch.py).
"""
from __future__ import annotations

import numpy as np
import torch

from .generate import build_case, solver_config
from .grid import HashGrid
from .input_reader import dem_search_scales
from .simulation import SPHDEM_OneStep, run_steps
from .struct import BNDptl, DEMBNDptl, DEMptl, SPHptl

TUNING_KEYS = ("block_sph", "porosity_variant", "lanes_sph", "nbr_cap", "nbr_format")
_SOLVER_FIELDS = ("h", "support", "rho0", "c0", "gamma", "mu", "g", "dt", "shepard_step", "dem_porosity_min",
                  "dem_porosity_max")


def _concat(kind, parts, device):
    n = sum(p.n for p in parts)
    out = kind(n, device=device) if kind is not DEMptl else DEMptl(n, device=device)
    for name, _ in kind._fields:
        setattr(out, name, torch.cat([getattr(p, name) for p in parts]).to(device).contiguous())
    return out


class _Runner:
    def tune(self, tuning: dict) -> None:
        """Launch tuning of this state's context (results are unaffected)."""
        from .engine import context_for

        ctx = context_for(self.P, self.B, self.D, self.W, tuple(self.grids))
        ctx.tuning.update({k: int(v) for k, v in tuning.items() if k in TUNING_KEYS})

    @property
    def n_units(self) -> int:
        """Moving particles (fluid + DEM)."""
        return self.P.n + self.D.n

    def run(self, first_step: int, n_steps: int) -> None:
        """Advance n_steps steps (CUDA-graph replay of run_forward's loop body)."""
        run_steps(self.solv, self.P, self.B, self.grids[0], self.grids[1], self.D, self.W, self.grids[2],
                  self.grids[3], first_step=first_step, n_steps=n_steps, search_scales=self.scales)

    def step(self, step: int) -> None:
        """One coupled step through the step API."""
        SPHDEM_OneStep(self.solv, self.P, self.B, self.D, self.W, *self.grids, step, self.scales)

    def snapshot(self) -> dict:
        """Device copy of the whole dynamic state (every particle field, both
        contact CSR sides, the control block and the host parity mirror)."""
        snap = {}
        for key, part in (("P", self.P), ("B", self.B), ("D", self.D), ("W", self.W)):
            for name, _ in part._fields:
                snap[(key, name)] = getattr(part, name).clone()
        for kind, ck in self.D._kinds.items():
            for si, side in enumerate(ck.sides):
                for a in type(side).__slots__:
                    snap[("csr", kind, si, a)] = getattr(side, a).clone()
        snap["ctl"] = self.D._ctl.clone()
        snap["old"] = dict(self.D._old)
        return snap

    def restore(self, snap: dict) -> None:
        """Copy a snapshot back in place (buffers keep their addresses, so
        contexts and captured graphs stay valid)."""
        for key, part in (("P", self.P), ("B", self.B), ("D", self.D), ("W", self.W)):
            for name, _ in part._fields:
                getattr(part, name).copy_(snap[(key, name)])
        for kind, ck in self.D._kinds.items():
            for si, side in enumerate(ck.sides):
                for a in type(side).__slots__:
                    getattr(side, a).copy_(snap[("csr", kind, si, a)])
        self.D._ctl.copy_(snap["ctl"])
        self.D._old.update(snap["old"])

    def _make_grids(self, inst=None, cell_factor: float = 1.0) -> None:
        s, sc = self.solv, self.scales
        self.grids = [HashGrid() for _ in range(4)]
        radii = (s.support, s.support, max(2.0 * sc[0], 2.0 * sc[2]), max(2.0 * sc[1], s.support))
        for g, part, key, r in zip(self.grids, (self.P, self.B, self.D, self.W), ("sph", "bnd", "dem", "dembnd"),
                                   radii):
            if inst is not None:
                g.ninst = self.ninst
                g.inst = inst[key]
            if key in ("sph", "bnd"):
                g.cell_factor = cell_factor
            g.build(part.pos, r)


class Case(_Runner):
    """One generated dam break on the GPU (generation config, DEM centres, radii)."""

    def __init__(self, gen, dem_positions=None, dem_radii=None, device="cuda", cell_factor: float = 1.0):
        self.device = torch.device(device)
        self.P, self.B, self.D, self.W = build_case(gen, dem_positions, dem_radii, device=self.device)
        self.solv = solver_config(gen, device=str(device))
        self.scales = dem_search_scales(self.D, self.W)
        self.ninst = 1
        self._make_grids(None, cell_factor)


class Ensemble(_Runner):
    """``members``: list of (generation config, DEM centres or None, DEM radii or None)."""

    def __init__(self, members, device="cuda", cell_factor: float = 1.0):
        if not members:
            raise ValueError("an ensemble needs at least one member")
        gens = [m[0] for m in members]
        for f in _SOLVER_FIELDS:
            vals = {float(getattr(g, f)) for g in gens}
            if len(vals) != 1:
                raise ValueError(f"ensemble members must share solver control {f!r}")
        cases = [build_case(g, pos, rad, device="cpu") for g, pos, rad in members]
        self.device = torch.device(device)
        self.solv = solver_config(gens[0], device=str(device))
        self.ninst = len(members)
        self.counts = {k: [c[i].n for c in cases] for i, k in enumerate(("sph", "bnd", "dem", "dembnd"))}
        self.P = _concat(SPHptl, [c[0] for c in cases], self.device)
        self.B = _concat(BNDptl, [c[1] for c in cases], self.device)
        self.D = _concat(DEMptl, [c[2] for c in cases], self.device)
        self.W = _concat(DEMBNDptl, [c[3] for c in cases], self.device)
        self.offsets = {k: np.concatenate([[0], np.cumsum(v)]) for k, v in self.counts.items()}
        inst = {k: torch.repeat_interleave(torch.arange(self.ninst, dtype=torch.int32),
                                           torch.tensor(v)).to(self.device).contiguous()
                for k, v in self.counts.items()}
        self.scales = dem_search_scales(self.D, self.W)
        self._make_grids(inst, cell_factor)

    def member(self, k: int, kind: str = "sph", field: str = "pos") -> torch.Tensor:
        """View of one member's field (e.g. member(3, "dem", "vel"))."""
        o = self.offsets[kind]
        part = {"sph": self.P, "bnd": self.B, "dem": self.D, "dembnd": self.W}[kind]
        return getattr(part, field)[int(o[k]):int(o[k + 1])]
