"""Particle structures: the reference's Warp structs as torch tensors.

Field names, dtypes and shapes follow ``input/struct.py:3-104``.  A Warp
``array(dtype=float)`` becomes a float32 tensor ``[n]``; ``array(dtype=vec3)``
becomes a contiguous float32 tensor ``[n, 3]`` (byte-identical layout).

Contact history (``DEMptl``).  The reference keeps, per contact kind, an old
(readable) and a new (writable) CSR side and swaps them after every rebuild,
reallocating the id / tangent arrays to the exact edge count E each time
(source/Simulation.py:142-203).  Here each side is a fixed-capacity buffer
set; ``contact_dem_id_old`` and friends are views of exactly ``offset[-1]``
elements (reading that length synchronises with the device), so shapes match
the reference while the step itself never synchronises and can be replayed
from a CUDA graph.  The index of the readable side lives in the device control
block ``_ctl`` and is mirrored on the host.
"""
from __future__ import annotations

import torch

VEC3 = 3


def _zeros(n: int, width: int, device, dtype=torch.float32) -> torch.Tensor:
    shape = (n, width) if width > 1 else (n,)
    return torch.zeros(shape, dtype=dtype, device=device)


class _Particles:
    """Common SoA container.  ``_fields`` lists (name, width) in struct order."""

    _fields: tuple = ()

    def __init__(self, n: int = 0, device="cpu"):
        for name, width in self._fields:
            object.__setattr__(self, name, _zeros(n, width, device))

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    @property
    def device(self) -> torch.device:
        return self.pos.device

    def field_names(self) -> tuple:
        return tuple(name for name, _ in self._fields)

    def to(self, device) -> "_Particles":
        out = type(self).__new__(type(self))
        for name in self.field_names():
            object.__setattr__(out, name, getattr(self, name).to(device).contiguous())
        return out

    def __repr__(self) -> str:
        return f"{type(self).__name__}(n={self.n}, device={self.device})"


class SPHptl(_Particles):
    """Fluid particles (input/struct.py:3-21)."""

    _fields = (("pos", VEC3), ("vel", VEC3), ("rho_raw", 1), ("rho", 1), ("pres", 1), ("acc", VEC3),
               ("m", 1), ("flt", 1), ("porosity", 1), ("pgf", VEC3), ("acc_dem", VEC3))


class BNDptl(_Particles):
    """Dummy wall particles (input/struct.py:23-36)."""

    _fields = (("pos", VEC3), ("vel", VEC3), ("rho_raw", 1), ("rho", 1), ("pres", 1), ("acc", VEC3),
               ("m", 1))


class DEMBNDptl(_Particles):
    """Fixed DEM wall spheres (input/struct.py:85-104)."""

    _fields = (("pos", VEC3), ("vel", VEC3), ("omega", VEC3), ("radius", 1), ("rho", 1), ("m", 1),
               ("volume", 1), ("inertia", 1), ("K", 1), ("eta", 1), ("mu", 1))


# Default per-row contact capacities of the fixed CSR buffers.  A moving sphere
# rarely touches more than a dozen equal spheres; wall-sphere lattices give at
# most ~100 overlaps in a corner for the configurations here.  Exceeding a
# capacity raises a device status bit that the step API turns into
# OverflowError (the reference raises OverflowError only for int32 overflow).
ROW_CAPACITY_DEM = 64
ROW_CAPACITY_BND = 256


class _CsrSide:
    __slots__ = ("offset", "id", "tang", "tang64")

    def __init__(self, n: int, capacity: int, device):
        self.offset = torch.zeros(n + 1, dtype=torch.int32, device=device)
        self.id = torch.zeros(capacity, dtype=torch.int32, device=device)
        self.tang = torch.zeros((capacity, 3), dtype=torch.float32, device=device)
        self.tang64 = torch.zeros((capacity, 3), dtype=torch.float64, device=device)

    @property
    def capacity(self) -> int:
        return int(self.id.shape[0])

    def edges(self) -> int:
        return int(self.offset[-1].item())


class _ContactKind:
    """Both CSR sides of one contact kind ('dem' or 'bnd')."""

    def __init__(self, n: int, capacity: int, device):
        self.sides = [_CsrSide(n, capacity, device), _CsrSide(n, capacity, device)]


class DEMptl(_Particles):
    """Moving DEM spheres (input/struct.py:39-82), CSR fields as exact views."""

    _fields = (("pos", VEC3), ("vel", VEC3), ("acc", VEC3), ("force", VEC3), ("omega", VEC3),
               ("torque", VEC3), ("radius", 1), ("rho", 1), ("m", 1), ("volume", 1), ("inertia", 1),
               ("K", 1), ("eta", 1), ("mu", 1), ("h", 1), ("flt_s", 1), ("porosity", 1), ("drag", VEC3),
               ("pressure_force", VEC3))
    _csr_names = ("contact_dem_offset_old", "contact_dem_id_old", "tang_dem_old", "contact_dem_offset_new",
                  "contact_dem_id_new", "tang_dem_new", "contact_bnd_offset_old", "contact_bnd_id_old",
                  "tang_bnd_old", "contact_bnd_offset_new", "contact_bnd_id_new", "tang_bnd_new")

    def __init__(self, n: int = 0, device="cpu", capacity_dem: int | None = None,
                 capacity_bnd: int | None = None):
        super().__init__(n, device)
        self._init_contacts(n, device, capacity_dem, capacity_bnd)

    def _init_contacts(self, n, device, capacity_dem=None, capacity_bnd=None):
        if capacity_dem is None:
            capacity_dem = n * min(max(n - 1, 0), ROW_CAPACITY_DEM)
        if capacity_bnd is None:
            capacity_bnd = n * ROW_CAPACITY_BND
        object.__setattr__(self, "_kinds", {"dem": _ContactKind(n, capacity_dem, device),
                                            "bnd": _ContactKind(n, capacity_bnd, device)})
        # device control block (sphdem_ctl_t): [1] readable DEM-DEM side,
        # [2] readable DEM-wall side, [3] status bits, [4]/[5] last edge counts
        object.__setattr__(self, "_ctl", torch.zeros(16, dtype=torch.int32, device=device))
        object.__setattr__(self, "_old", {"dem": 0, "bnd": 0})

    # -- CSR side bookkeeping -------------------------------------------------
    def _side(self, kind: str, which: str) -> _CsrSide:
        old = self._old[kind]
        return self._kinds[kind].sides[old if which == "old" else 1 - old]

    def _flip(self, kind: str) -> None:
        """Host mirror of the device-side swap (source/Simulation.py:166-171)."""
        self._old[kind] = 1 - self._old[kind]

    def contact_capacity(self, kind: str) -> int:
        return self._kinds[kind].sides[0].capacity

    @staticmethod
    def _parse(name: str):
        parts = name.split("_")
        if name.startswith("contact_"):
            return parts[1], parts[2], parts[3]  # kind, offset|id, old|new
        return parts[1], "tang", parts[2]

    def __getattr__(self, name):
        if name in DEMptl._csr_names:
            kind, what, which = self._parse(name)
            side = self._side(kind, which)
            if what == "offset":
                return side.offset
            e = side.edges()
            return side.id[:e] if what == "id" else side.tang[:e]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in DEMptl._csr_names:
            kind, what, which = self._parse(name)
            side = self._side(kind, which)
            value = torch.as_tensor(value, device=side.offset.device)
            if what == "offset":
                side.offset.copy_(value.to(torch.int32))
            else:
                dst = side.id if what == "id" else side.tang
                k = int(value.shape[0])
                if k > dst.shape[0]:
                    raise OverflowError(f"{name}: {k} edges exceed the CSR capacity {dst.shape[0]}")
                dst[:k].copy_(value.to(dst.dtype).reshape(dst[:k].shape))
            return
        object.__setattr__(self, name, value)

    def field_names(self) -> tuple:
        return tuple(name for name, _ in self._fields) + self._csr_names

    def to(self, device) -> "DEMptl":
        out = DEMptl.__new__(DEMptl)
        for name, _ in self._fields:
            object.__setattr__(out, name, getattr(self, name).to(device).contiguous())
        object.__setattr__(out, "_kinds", {})
        for kind, ck in self._kinds.items():
            nk = _ContactKind.__new__(_ContactKind)
            nk.sides = []
            for s in ck.sides:
                ns = _CsrSide.__new__(_CsrSide)
                for a in _CsrSide.__slots__:
                    setattr(ns, a, getattr(s, a).to(device))
                nk.sides.append(ns)
            out._kinds[kind] = nk
        object.__setattr__(out, "_ctl", self._ctl.to(device))
        object.__setattr__(out, "_old", dict(self._old))
        return out


STRUCTURES = {"SPH": SPHptl, "BND": BNDptl, "DEM": DEMptl, "DEMBND": DEMBNDptl}
