"""ctypes binding of the CPU oracle (oracle/sphdem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() (the
oracle its step is compared with), and by bench.py's CPU-baseline leg.  The
product never imports it.

``HostState`` holds numpy copies of the four particle structs (same field
layout as include/sphdem.h) plus both sides of each contact CSR, and runs the
oracle's restatement of the reference kernels on them.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_dp = C.POINTER(C.c_double)


class _Sph(C.Structure):
    _fields_ = [(n, _fp) for n in ("pos", "vel", "rho_raw", "rho", "pres", "acc", "m", "flt", "porosity", "pgf",
                                   "acc_dem")] + [("n", C.c_int32)]


class _Bnd(C.Structure):
    _fields_ = [(n, _fp) for n in ("pos", "vel", "rho_raw", "rho", "pres", "acc", "m")] + [("n", C.c_int32)]


class _Csr(C.Structure):
    _fields_ = [("offset", _ip), ("id", _ip), ("tang", _fp), ("tang64", _dp), ("capacity", C.c_int64)]


class _Dem(C.Structure):
    _fields_ = ([(n, _fp) for n in ("pos", "vel", "acc", "force", "omega", "torque", "radius", "rho", "m",
                                    "volume", "inertia", "K", "eta", "mu", "h")]
                + [("csr_dem", _Csr * 2), ("csr_bnd", _Csr * 2)]
                + [(n, _fp) for n in ("flt_s", "porosity", "drag", "pressure_force")] + [("n", C.c_int32)])


class _DemBnd(C.Structure):
    _fields_ = [(n, _fp) for n in ("pos", "vel", "omega", "radius", "rho", "m", "volume", "inertia", "K", "eta",
                                   "mu")] + [("n", C.c_int32)]


class _Params(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("h", "support", "rho0", "c0", "gamma", "mu", "g", "dt")] + [
        ("shepard_step", C.c_int32)] + [(n, C.c_float) for n in (
            "porosity_min", "porosity_max", "radius_max", "boundary_radius_max", "h_max", "h_uniform")] + [
        ("block_sph", C.c_int32), ("porosity_variant", C.c_int32), ("lanes_sph", C.c_int32),
        ("pad_params", C.c_int32)]


SPH_FIELDS = (("pos", 3), ("vel", 3), ("rho_raw", 1), ("rho", 1), ("pres", 1), ("acc", 3), ("m", 1), ("flt", 1),
              ("porosity", 1), ("pgf", 3), ("acc_dem", 3))
BND_FIELDS = (("pos", 3), ("vel", 3), ("rho_raw", 1), ("rho", 1), ("pres", 1), ("acc", 3), ("m", 1))
DEM_FIELDS = (("pos", 3), ("vel", 3), ("acc", 3), ("force", 3), ("omega", 3), ("torque", 3), ("radius", 1),
              ("rho", 1), ("m", 1), ("volume", 1), ("inertia", 1), ("K", 1), ("eta", 1), ("mu", 1), ("h", 1),
              ("flt_s", 1), ("porosity", 1), ("drag", 3), ("pressure_force", 3))
DEMBND_FIELDS = (("pos", 3), ("vel", 3), ("omega", 3), ("radius", 1), ("rho", 1), ("m", 1), ("volume", 1),
                 ("inertia", 1), ("K", 1), ("eta", 1), ("mu", 1))

REL = dict(SPH_SPH_SUPPORT=0, SPH_BND_SUPPORT=1, BND_SPH_SUPPORT=2, BND_BND_SUPPORT=3, SPH_SPH_FORCE=4,
           SPH_BND_FORCE=5, SPH_SPH_LEN=6, SPH_DEM_2H=7, DEM_SPH_2H=8, DEM_DEM_2H=9, SPH_DEM_REACT=10)


def build() -> None:
    """Compile both oracle builds with gcc (no CUDA needed)."""
    BUILD.mkdir(parents=True, exist_ok=True)
    src = HERE / "sphdem_oracle.c"
    hdr = ROOT / "include" / "sphdem.h"
    for tag, real in (("f32", "float"), ("f64", "double")):
        out = BUILD / f"liboracle_{tag}.so"
        if out.exists() and out.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime):
            continue
        tmp = out.with_suffix(".so.tmp")
        subprocess.run([os.environ.get("CC", "gcc"), "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
                        "-fno-fast-math", f"-I{ROOT / 'include'}", f"-DORACLE_REAL={real}", str(src), "-o",
                        str(tmp), "-lpthread", "-lm"], check=True)
        os.replace(tmp, out)


_LIBS: dict[str, C.CDLL] = {}


def lib(precision: str = "f32") -> C.CDLL:
    if precision not in _LIBS:
        build()
        L = C.CDLL(str(BUILD / f"liboracle_{precision}.so"))
        L.oracle_force_dem.restype = C.c_int64
        L.oracle_bc_dem.restype = C.c_int64
        L.oracle_set_threads.restype = C.c_int
        L.oracle_set_threads(os.cpu_count() or 1)
        for name in ("oracle_shepard_sph", "oracle_density_sph", "oracle_density_bnd", "oracle_force_sph",
                     "oracle_prep_sphdem", "oracle_interaction_dem", "oracle_interaction_sph"):
            getattr(L, name).restype = None
        _LIBS[precision] = L
    return _LIBS[precision]


def set_threads(n: int) -> None:
    for p in ("f32", "f64"):
        lib(p).oracle_set_threads(int(n))


def set_subject_stride(stride: int) -> None:
    """Timing samples only: process every stride-th subject (results incomplete)."""
    for p in ("f32", "f64"):
        lib(p).oracle_set_subject_stride(int(stride))


def _np(t, width):
    """numpy float32 copy of a torch tensor / array with shape [n, width] or [n]
    (always a copy: two states made from the same CPU tensors must not share
    memory)."""
    if hasattr(t, "detach"):
        t = t.detach().cpu().numpy()
    a = np.array(t, dtype=np.float32, order="C", copy=True)
    return a.reshape(-1, width) if width > 1 else a.reshape(-1)


def _ptr(a, kind=_fp):
    return a.ctypes.data_as(kind)


class HostState:
    """Host copy of one SPH-DEM state, driven by the oracle."""

    def __init__(self, sph=None, bnd=None, dem=None, dembnd=None):
        self.sph = {k: _np(getattr(sph, k), w) for k, w in SPH_FIELDS} if sph is not None else \
            {k: np.zeros((0, w) if w > 1 else 0, np.float32) for k, w in SPH_FIELDS}
        self.bnd = {k: _np(getattr(bnd, k), w) for k, w in BND_FIELDS} if bnd is not None else \
            {k: np.zeros((0, w) if w > 1 else 0, np.float32) for k, w in BND_FIELDS}
        self.dem = {k: _np(getattr(dem, k), w) for k, w in DEM_FIELDS} if dem is not None else \
            {k: np.zeros((0, w) if w > 1 else 0, np.float32) for k, w in DEM_FIELDS}
        self.dembnd = {k: _np(getattr(dembnd, k), w) for k, w in DEMBND_FIELDS} if dembnd is not None else \
            {k: np.zeros((0, w) if w > 1 else 0, np.float32) for k, w in DEMBND_FIELDS}
        nd = len(self.dem["pos"])
        self.csr = {}
        self.old = {"dem": 0, "bnd": 0}
        for kind in ("dem", "bnd"):
            sides = []
            if dem is not None:
                for which in ("old", "new"):
                    off = getattr(dem, f"contact_{kind}_offset_{which}").detach().cpu().numpy().astype(np.int32)
                    ids = getattr(dem, f"contact_{kind}_id_{which}").detach().cpu().numpy().astype(np.int32)
                    tang = _np(getattr(dem, f"tang_{kind}_{which}"), 3)
                    cap = max(dem.contact_capacity(kind), len(ids))
                    side = dict(offset=off.copy(), id=np.zeros(cap, np.int32), tang=np.zeros((cap, 3), np.float32))
                    side["id"][:len(ids)] = ids
                    side["tang"][:len(ids)] = tang
                    sides.append(side)
            else:
                for _ in range(2):
                    sides.append(dict(offset=np.zeros(nd + 1, np.int32), id=np.zeros(0, np.int32),
                                      tang=np.zeros((0, 3), np.float32)))
            self.csr[kind] = sides

    # -- ctypes views ----------------------------------------------------------
    def _sph_t(self):
        s = _Sph(*[_ptr(self.sph[k]) for k, _ in SPH_FIELDS], len(self.sph["pos"]))
        return s

    def _bnd_t(self):
        return _Bnd(*[_ptr(self.bnd[k]) for k, _ in BND_FIELDS], len(self.bnd["pos"]))

    def _dem_t(self):
        d = _Dem()
        for k, _ in DEM_FIELDS:
            setattr(d, k, _ptr(self.dem[k]))
        for kind, arr in (("dem", d.csr_dem), ("bnd", d.csr_bnd)):
            for i, side in enumerate(self.csr[kind]):
                arr[i].offset = _ptr(side["offset"], _ip)
                arr[i].id = _ptr(side["id"], _ip)
                arr[i].tang = _ptr(side["tang"])
                arr[i].tang64 = _dp()
                arr[i].capacity = len(side["id"])
        d.n = len(self.dem["pos"])
        return d

    def _dembnd_t(self):
        return _DemBnd(*[_ptr(self.dembnd[k]) for k, _ in DEMBND_FIELDS], len(self.dembnd["pos"]))

    # -- contact views (reference field names) --------------------------------
    def side(self, kind: str, which: str = "old") -> dict:
        o = self.old[kind]
        s = self.csr[kind][o if which == "old" else 1 - o]
        e = int(s["offset"][-1])
        return dict(offset=s["offset"], id=s["id"][:e], tang=s["tang"][:e])

    # -- kernels ---------------------------------------------------------------
    def shepard(self, support, h, p="f32"):
        lib(p).oracle_shepard_sph(C.byref(self._sph_t()), C.byref(self._bnd_t()), C.c_float(support), C.c_float(h))

    def density_sph(self, support, h, p="f32"):
        lib(p).oracle_density_sph(C.byref(self._sph_t()), C.byref(self._bnd_t()), C.c_float(support), C.c_float(h))

    def density_bnd(self, support, h, p="f32"):
        lib(p).oracle_density_bnd(C.byref(self._sph_t()), C.byref(self._bnd_t()), C.c_float(support), C.c_float(h))

    def pres(self, rho0, c0, gamma, p="f32"):
        lib(p).oracle_pres_sph(C.byref(self._sph_t()), C.c_float(rho0), C.c_float(c0), C.c_float(gamma))
        lib(p).oracle_pres_bnd(C.byref(self._bnd_t()), C.c_float(rho0), C.c_float(c0), C.c_float(gamma))

    def force_sph(self, support, h, mu, g, p="f32"):
        lib(p).oracle_force_sph(C.byref(self._sph_t()), C.byref(self._bnd_t()), C.c_float(support), C.c_float(h),
                                C.c_float(mu), C.c_float(g))

    def step_sph(self, dt, p="f32"):
        lib(p).oracle_step_sph(C.byref(self._sph_t()), C.c_float(dt))

    def force_dem(self, radius_max, g, dt, p="f32") -> int:
        """Count, scan, fill and swap (the reference's run_force_dem sequence)."""
        self._ensure_capacity("dem")
        e = lib(p).oracle_force_dem(C.byref(self._dem_t()), self.old["dem"], C.c_float(radius_max), C.c_float(g),
                                    C.c_float(dt))
        if e < 0:
            raise OverflowError("oracle DEM-DEM CSR capacity exceeded")
        self.old["dem"] = 1 - self.old["dem"]
        return int(e)

    def bc_dem(self, radius_max, dt, p="f32") -> int:
        self._ensure_capacity("bnd")
        e = lib(p).oracle_bc_dem(C.byref(self._dem_t()), C.byref(self._dembnd_t()), self.old["bnd"],
                                 C.c_float(radius_max), C.c_float(dt))
        if e < 0:
            raise OverflowError("oracle DEM-wall CSR capacity exceeded")
        self.old["bnd"] = 1 - self.old["bnd"]
        return int(e)

    def _ensure_capacity(self, kind):
        nd = len(self.dem["pos"])
        nn = nd if kind == "dem" else len(self.dembnd["pos"])
        cap = nd * max(min(nn, 512), 1)
        for side in self.csr[kind]:
            if len(side["id"]) < cap:
                ids = np.zeros(cap, np.int32)
                tang = np.zeros((cap, 3), np.float32)
                ids[:len(side["id"])] = side["id"]
                tang[:len(side["tang"])] = side["tang"]
                side["id"], side["tang"] = ids, tang

    def step_dem(self, dt, p="f32"):
        lib(p).oracle_step_dem(C.byref(self._dem_t()), C.c_float(dt))

    def prep_sphdem(self, support, h, sph_support, sph_h, eps_min, eps_max, p="f32"):
        lib(p).oracle_prep_sphdem(C.byref(self._sph_t()), C.byref(self._bnd_t()), C.byref(self._dem_t()),
                                  *(C.c_float(x) for x in (support, h, sph_support, sph_h, eps_min, eps_max)))

    def interaction_dem(self, mu, eps_min, eps_max, dt, p="f32"):
        lib(p).oracle_interaction_dem(C.byref(self._sph_t()), C.byref(self._dem_t()),
                                      *(C.c_float(x) for x in (mu, eps_min, eps_max, dt)))

    def interaction_sph(self, support, p="f32"):
        lib(p).oracle_interaction_sph(C.byref(self._sph_t()), C.byref(self._dem_t()), C.c_float(support))

    @staticmethod
    def params(solv, scales=None) -> _Params:
        q = _Params()
        q.h, q.support, q.rho0, q.c0, q.gamma = solv.h, solv.support, solv.rho0, solv.c0, solv.gamma
        q.mu, q.g, q.dt, q.shepard_step = solv.mu, solv.g, solv.dt, int(solv.shepard_step)
        q.porosity_min, q.porosity_max = solv.dem_porosity_min, solv.dem_porosity_max
        if scales is not None:
            q.radius_max, q.boundary_radius_max, q.h_max, q.h_uniform = scales
        return q

    def sph_onestep(self, solv, step, integrate=True, p="f32"):
        lib(p).oracle_sph_onestep(C.byref(self._sph_t()), C.byref(self._bnd_t()), C.byref(self.params(solv)),
                                  int(step), int(bool(integrate)))

    def sphdem_onestep(self, solv, step, scales, p="f32"):
        for kind in ("dem", "bnd"):
            self._ensure_capacity(kind)
        od = C.c_int(self.old["dem"])
        ob = C.c_int(self.old["bnd"])
        rc = lib(p).oracle_sphdem_onestep(C.byref(self._sph_t()), C.byref(self._bnd_t()), C.byref(self._dem_t()),
                                          C.byref(self._dembnd_t()), C.byref(self.params(solv, scales)), int(step),
                                          C.byref(od), C.byref(ob))
        if rc:
            raise OverflowError("oracle CSR capacity exceeded")
        self.old["dem"], self.old["bnd"] = od.value, ob.value

    def neighbour_digest(self, relation: str, radius: float, p="f32"):
        rel = REL[relation]
        nsub = {2: len(self.bnd["pos"]), 3: len(self.bnd["pos"]), 8: len(self.dem["pos"]),
                9: len(self.dem["pos"])}.get(rel, len(self.sph["pos"]))
        count = np.zeros(nsub, np.int32)
        hsh = np.zeros(nsub, np.uint64)
        lib(p).oracle_neighbour_digest(C.byref(self._sph_t()), C.byref(self._bnd_t()), C.byref(self._dem_t()), rel,
                                       C.c_float(radius), _ptr(count, _ip), hsh.ctypes.data_as(C.POINTER(C.c_uint64)))
        return count, hsh

    def diagnostics(self, g, p="f64") -> np.ndarray:
        out = np.zeros(8, np.float64)
        lib(p).oracle_diagnostics(C.byref(self._sph_t()), C.byref(self._dem_t()), C.c_float(g), _ptr(out, _dp))
        return out


def wendland(r: np.ndarray, h: float, p="f64"):
    r = np.ascontiguousarray(r, dtype=np.float32)
    w = np.zeros(len(r))
    dw = np.zeros(len(r))
    lib(p).oracle_wendland(_ptr(r), len(r), C.c_float(h), _ptr(w, _dp), _ptr(dw, _dp))
    return w, dw


def drag_beta(eps, rho, mu, d, speed, p="f64") -> np.ndarray:
    arrs = [np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float32), np.shape(eps)), dtype=np.float32)
            for x in (eps, rho, mu, d, speed)]
    out = np.zeros(len(arrs[0]))
    lib(p).oracle_drag_beta(*(_ptr(a) for a in arrs), len(arrs[0]), _ptr(out, _dp))
    return out
