"""Execution context: binds particle structs and grids to libsphdem.

A ``StepContext`` owns the sorted working copies, the scan scratch of the grids
and the ctypes ``sphdem_ctx_t`` that points at every tensor; it is cached per
(structs, grids) combination on the fluid (or DEM) struct.  Every call
enqueues work on torch's current CUDA stream; nothing here synchronises the
host except the explicit status checks and the exact-length CSR views.
"""
from __future__ import annotations

import ctypes as C
import math
import weakref

import torch

from . import _lib
from .grid import HashGrid, empty_grid
from .struct import BNDptl, DEMBNDptl, DEMptl, SPHptl

KIND_SPH, KIND_BND, KIND_DEM, KIND_DEMBND = 0, 1, 2, 3
NBR_BYTES_MAX = 16 << 30  # neighbour records above this size are not kept (the force pass walks cells)


def neighbour_capacity(n: int, support: float, mean_volume: float, request: int = -1, cell: float = 0.0,
                       fmt: int = _lib.NBR_SLOTS) -> int:
    """Per-particle capacity of each kind's density -> force neighbour record
    (``request`` >= 0 sets it; 0 = none).  Member slots (NBR_SLOTS): 1.25 x
    the particles a full support ball holds at the mean particle volume, + 8,
    rounded up to a multiple of 8.  Walk masks (NBR_MASKS): 32-bit words for
    1.25 x the slots one walk visits -- the cells overlapping [p - s, p + s]
    span 2 s + c per axis on average (s = support, c = cell width, the support
    when 0) -- + 64 bits.  0 when the (2 cap + 2) n words exceed
    NBR_BYTES_MAX.  A
    particle whose record overflows has its force pass walk its cells (same
    results)."""
    cap = max(0, int(request))
    if request < 0 and mean_volume > 0.0:
        ball = 4.0 / 3.0 * math.pi * support ** 3 / mean_volume
        if fmt == _lib.NBR_MASKS:
            c = cell if cell > 0.0 else support
            walked = (2.0 * support + c) ** 3 / mean_volume
            cap = math.ceil((1.25 * walked + 64.0) / 32.0)
        else:
            cap = 8 * math.ceil((1.25 * ball + 8.0) / 8.0)
    return 0 if (2 * cap + 2) * n * 4 > NBR_BYTES_MAX else cap


def porosity_frame(cell: float, mean_volume: float) -> int:
    """Frame-block edge F (in fluid-grid cells) of the tensor-core porosity
    pass: its subject tiles are the listed particles of world-anchored blocks
    of F^3 cells, centred on the block.  The smallest F >= 2 whose block holds
    at least four full tiles of 128 at the mean particle volume (so tiles are
    mostly full), at most 8 (so |x - centre| stays below ~h).  Depends only on
    the cell width and the particle volume: every member of a batched state
    and the same case alone get the same blocks."""
    if not (cell > 0.0 and mean_volume > 0.0):
        return 4
    per_cell = cell ** 3 / mean_volume
    f = 2
    while f < 8 and f ** 3 * per_cell < 4 * 128:
        f += 1
    return f


def _require_cuda(t: torch.Tensor, name: str) -> None:
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor: the GB300 step has no CPU path")
    if t.dtype not in (torch.float32, torch.int32, torch.float64) or not t.is_contiguous():
        raise RuntimeError(f"{name} must be a contiguous float32/int32 tensor")


class StepContext:
    def __init__(self, sph, bnd, dem, dembnd, grids, device):
        self.device = torch.device(device)
        self.lib = _lib.load()
        self.sets = [sph if sph is not None else SPHptl(0, self.device),
                     bnd if bnd is not None else BNDptl(0, self.device),
                     dem if dem is not None else DEMptl(0, self.device),
                     dembnd if dembnd is not None else DEMBNDptl(0, self.device)]
        self.has = [x is not None for x in (sph, bnd, dem, dembnd)]
        self.grids = [g if g is not None else empty_grid() for g in grids]
        self.ctl = self.sets[2]._ctl if dem is not None else torch.zeros(16, dtype=torch.int32,
                                                                          device=self.device)
        self.ctx = _lib.CtxT()
        self.params = _lib.ParamsT()
        self.box = None
        self.wall_key = None
        self.built = [False] * 4
        self._sig = None
        self._status_host = torch.zeros(16, dtype=torch.int32, pin_memory=True)
        self._status_event = None
        # launch tuning (results do not depend on it): see autotune.py
        self.tuning = {"block_sph": 0, "porosity_variant": 2, "lanes_sph": 1, "nbr_cap": -1,
                       "nbr_format": _lib.NBR_SLOTS}
        self._nbr_key = None
        self._nbr_cap = 0
        self._mean_vol = 0.0
        self._pkey = None
        self._alloc_work()
        addr = C.addressof(self.ctx)
        weakref.finalize(self, _release, self.lib, addr)

    # -- buffers ---------------------------------------------------------------
    def _alloc_work(self) -> None:
        ns, nb, nd = self.sets[0].n, self.sets[1].n, self.sets[2].n
        f = dict(dtype=torch.float32, device=self.device)
        i = dict(dtype=torch.int32, device=self.device)
        self.work = dict(
            f_posm=torch.zeros((ns, 4), **f), f_vel=torch.zeros((ns, 4), **f), f_rp=torch.zeros((ns, 4), **f),
            f_vprev=torch.zeros(ns, **f), f_posv=torch.zeros((ns, 4), **f), f_pgf=torch.zeros((ns, 4), **f),
            near_list=torch.zeros(ns, **i), b_posm=torch.zeros((nb, 4), **f), b_vel=torch.zeros((nb, 4), **f),
            b_rp=torch.zeros((nb, 4), **f), b_vprev=torch.zeros(nb, **f), b_self=torch.zeros(nb, **f),
            dem_count=torch.zeros(2 * (nd + 1), **i), dem_aux=torch.zeros((nd, 4), **f),
            f_posq=torch.zeros((ns, 4), **f), nbr=torch.zeros(1, **i))

    def _neighbour_lists(self, solv, request: int = -1, fmt: int = _lib.NBR_SLOTS) -> int:
        """Neighbour-record capacity (neighbour_capacity at the smaller of the
        fluid and wall mean particle volumes m / rho0 and the fluid-grid cell
        width) and buffer, allocated once per (support, rho0, cell, request,
        format)."""
        P, B = self.sets[0], self.sets[1]
        g = self.grids[0]
        cell = float(g.radius) * float(g.cell_factor) if g.radius else 0.0
        key = (float(solv.support), float(solv.rho0), cell, int(request), int(fmt))
        if P.n == 0 or key == self._nbr_key:
            return self._nbr_cap
        vol = float(P.m.double().mean().item()) / key[1]  # host syncs once per key
        self._mean_vol = vol
        if B is not None and B.n > 0:
            vol = min(vol, float(B.m.double().mean().item()) / key[1])
        cap = neighbour_capacity(P.n, key[0], vol if request < 0 else 0.0, request, cell, fmt)
        self.work["nbr"] = (torch.zeros((2 * cap + 2) * P.n, dtype=torch.int32, device=self.device) if cap
                            else torch.zeros(1, dtype=torch.int32, device=self.device))
        self._nbr_key, self._nbr_cap = key, cap
        self._sig = None  # pointers changed
        return cap

    def _porosity_scratch(self) -> None:
        """Scratch of the tensor-core porosity pass (work.pfb, ptiles, ppart,
        pflag), sized by the library for the fluid grid geometry and the frame
        edge; allocated once per geometry.  Coupled contexts with spheres only."""
        P, D = self.sets[0], self.sets[2]
        if P.n == 0 or D.n == 0 or self.grids[0].geometry is None:
            return
        frame = porosity_frame(self.grids[0].geometry[2], self._mean_vol)
        key = (frame, tuple(self.grids[0].geometry[0]), tuple(self.grids[0].geometry[1]), self.grids[0].ninst, P.n)
        if key != self._pkey:
            out = (C.c_int64 * 4)()
            _lib.check(self.lib.sphdem_porosity_scratch(C.byref(self.ctx), frame, out), "porosity scratch")
            i32 = dict(dtype=torch.int32, device=self.device)
            self.work.update(pfb=torch.zeros(max(1, out[0]), **i32), ptiles=torch.zeros(max(1, out[1]), **i32),
                             ppart=torch.zeros(max(1, out[2]), dtype=torch.float32, device=self.device),
                             pflag=torch.zeros(max(1, out[3]), **i32))
            self._pwords, self._pframe, self._pkey = int(out[0]), frame, key
            self._sig = None  # pointers changed
            self._fill()
        self.ctx.work.pfb_words = self._pwords
        self.ctx.work.pframe = self._pframe

    def _domain(self):
        """Union bounding box of all particle sets (one host sync, once).
        Non-finite positions are left out of the box: they bin to a face cell
        and the device flags them (SPHDEM_FLAG_NONFINITE -> FloatingPointError
        at the status check)."""
        if self.box is None:
            los, his = [], []
            for s in self.sets:
                if s.n > 0:
                    ok = torch.isfinite(s.pos).all(dim=1, keepdim=True)
                    inf = torch.full_like(s.pos, float("inf"))
                    los.append(torch.where(ok, s.pos, inf).amin(0))
                    his.append(torch.where(ok, s.pos, -inf).amax(0))
            lo_hi = (torch.stack(los).amin(0), torch.stack(his).amax(0)) if los else None
            if lo_hi is not None and not bool(torch.isfinite(lo_hi[0]).all() & torch.isfinite(lo_hi[1]).all()):
                los = []  # no finite position at all
            if not los:
                lo = [0.0, 0.0, 0.0]
                hi = [1.0, 1.0, 1.0]
            else:
                lo = lo_hi[0].tolist()
                hi = lo_hi[1].tolist()
            # open top: leave room above for splashes (points beyond still bin correctly)
            hi[2] = hi[2] + 0.5 * max(hi[2] - lo[2], 1e-6)
            self.box = (lo, hi)
        return self.box

    # -- ctypes structure --------------------------------------------------------
    def _signature(self):
        sig = []
        for s in self.sets:
            for name in s.field_names():
                if name.startswith(("contact_", "tang_")):
                    continue
                sig.append(getattr(s, name).data_ptr())
        return tuple(sig)

    def _fill(self) -> None:
        sig = self._signature()
        if sig == self._sig:
            return
        sph, bnd, dem, dembnd = self.sets
        P = self.ctx.sph
        for name in SPHptl._fields:
            t = getattr(sph, name[0])
            if sph.n:
                _require_cuda(t, f"SPHptl.{name[0]}")
            setattr(P, name[0], _lib.fptr(t))
        P.n = sph.n
        B = self.ctx.bnd
        for name, _ in BNDptl._fields:
            t = getattr(bnd, name)
            if bnd.n:
                _require_cuda(t, f"BNDptl.{name}")
            setattr(B, name, _lib.fptr(t))
        B.n = bnd.n
        D = self.ctx.dem
        for name, _ in DEMptl._fields:
            t = getattr(dem, name)
            if dem.n:
                _require_cuda(t, f"DEMptl.{name}")
            setattr(D, name, _lib.fptr(t))
        for kind, arr in (("dem", D.csr_dem), ("bnd", D.csr_bnd)):
            for k, side in enumerate(dem._kinds[kind].sides):
                arr[k].offset = _lib.iptr(side.offset)
                arr[k].id = _lib.iptr(side.id)
                arr[k].tang = _lib.fptr(side.tang)
                arr[k].tang64 = _lib.dptr(side.tang64)
                arr[k].capacity = side.capacity
        D.n = dem.n
        W = self.ctx.dembnd
        for name, _ in DEMBNDptl._fields:
            t = getattr(dembnd, name)
            if dembnd.n:
                _require_cuda(t, f"DEMBNDptl.{name}")
            setattr(W, name, _lib.fptr(t))
        W.n = dembnd.n
        w = self.ctx.work
        for name, t in self.work.items():
            setattr(w, name, _lib.iptr(t) if t.dtype == torch.int32 else _lib.fptr(t))
        self.ctx.ctl = self.ctl.data_ptr()
        self._sig = sig

    def _fill_grids(self) -> None:
        lo, hi = self._domain()
        for k, (g, s) in enumerate(zip(self.grids, self.sets)):
            g.ensure_geometry(lo, hi, s.n, self.device)
            g.fill(getattr(self.ctx, ("grid_sph", "grid_bnd", "grid_dem", "grid_dembnd")[k]), s.n)

    def set_params(self, solv, scales=None) -> None:
        p = self.params
        p.h = solv.h
        p.support = solv.support
        p.rho0 = solv.rho0
        p.c0 = solv.c0
        p.gamma = solv.gamma
        p.mu = solv.mu
        p.g = solv.g
        p.dt = solv.dt
        p.shepard_step = int(solv.shepard_step)
        p.porosity_min = getattr(solv, "dem_porosity_min", 0.05)
        p.porosity_max = getattr(solv, "dem_porosity_max", 1.0)
        if scales is not None:
            p.radius_max, p.boundary_radius_max, p.h_max, p.h_uniform = (float(x) for x in scales)
        p.block_sph = int(self.tuning.get("block_sph", 0))
        p.porosity_variant = int(self.tuning.get("porosity_variant", 0))
        p.lanes_sph = int(self.tuning.get("lanes_sph", 1))
        fmt = int(self.tuning.get("nbr_format", _lib.NBR_SLOTS))
        p.nbr_cap = self._neighbour_lists(solv, int(self.tuning.get("nbr_cap", -1)), fmt)
        p.nbr_format = fmt

    @property
    def stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    # -- grids -------------------------------------------------------------------
    def prepare(self, rebuild_moving=True, wall_key=None) -> None:
        """Pointers, grid geometry, and device builds of stale grids.
        wall_key = (support, h) of the wall self-density cache."""
        self._fill()
        self._fill_grids()
        self._porosity_scratch()
        sph, bnd, dem, dembnd = self.sets
        st = self.stream
        for kind in (KIND_BND, KIND_DEMBND, KIND_SPH, KIND_DEM):
            g = self.grids[kind]
            s = self.sets[kind]
            if self.has[kind] and g.points is not None and g.points.data_ptr() != s.pos.data_ptr() and s.n:
                raise ValueError("a grid must be built on the positions of its particle struct")
            moving = kind in (KIND_SPH, KIND_DEM)
            need = not self.built[kind] or g.dirty or (moving and rebuild_moving)
            if kind == KIND_BND and wall_key is not None and wall_key != self.wall_key:
                need = True
            if not need:
                continue
            params = self.params
            if kind == KIND_BND and wall_key is not None:
                params = _lib.ParamsT()
                C.memmove(C.byref(params), C.byref(self.params), C.sizeof(params))
                params.support, params.h = wall_key
                self.wall_key = wall_key
            _lib.check(self.lib.sphdem_grid_build(C.byref(self.ctx), kind, C.byref(params), st),
                       f"grid build (kind {kind})")
            g.dirty = False
            self.built[kind] = True

    def refresh(self) -> None:
        _lib.check(self.lib.sphdem_refresh_sorted(C.byref(self.ctx), self.stream), "refresh sorted copies")

    # -- status ------------------------------------------------------------------
    def poll_status(self) -> None:
        """Raise for device flags of an earlier step if its copy has landed."""
        ev = self._status_event
        if ev is not None and ev.query():
            self._raise_for(int(self._status_host[3]))

    def post_status(self) -> None:
        self._status_host.copy_(self.ctl, non_blocking=True)
        if self._status_event is None:
            self._status_event = torch.cuda.Event()
        self._status_event.record()

    def check_status(self) -> None:
        """Blocking check of the device status bits."""
        self._raise_for(int(self.ctl[3].item()))

    def _raise_for(self, flags: int) -> None:
        if flags & (_lib.FLAG_CSR_DEM_OVERFLOW | _lib.FLAG_CSR_BND_OVERFLOW):
            self.ctl[3] = 0
            raise OverflowError("directed contact count exceeded the CSR capacity "
                                f"(status 0x{flags:x}); allocate DEMptl with a larger capacity")
        if flags & _lib.FLAG_TIMEOUT:
            self.ctl[3] = 0
            raise RuntimeError("a bounded device-side wait timed out (status 0x%x); the step is void" % flags)
        if flags & _lib.FLAG_NONFINITE:
            self.ctl[3] = 0
            raise FloatingPointError("non-finite particle position met while binning")


def _release(lib, addr):
    try:
        lib.sphdem_release(C.c_void_p(addr))
    except Exception:
        pass


def context_for(sph=None, bnd=None, dem=None, dembnd=None, grids=(None, None, None, None)) -> StepContext:
    """Cached context for this combination of structs and grids."""
    grids = tuple(HashGrid.from_id(g) if g is not None else None for g in grids)
    owner = next(x for x in (sph, dem, bnd, dembnd) if x is not None)
    key = tuple(id(x) if x is not None else 0 for x in (sph, bnd, dem, dembnd) + grids)
    cache = owner.__dict__.setdefault("_sphdem_contexts", {})
    ctx = cache.get(key)
    if ctx is None:
        ctx = StepContext(sph, bnd, dem, dembnd, grids, owner.pos.device)
        cache[key] = ctx
    return ctx
