"""ctypes binding of libsphdem.so (include/sphdem.h, include/sphdem_mpnn.h).

The structures below mirror the C ABI field for field; ``check_layout`` compares
their sizes with the library's own ``sizeof`` values at load time.  Loading
fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .build import LIB

c_float_p = C.POINTER(C.c_float)
c_int_p = C.POINTER(C.c_int32)
c_double_p = C.POINTER(C.c_double)
c_u64_p = C.POINTER(C.c_uint64)


class SphT(C.Structure):
    _fields_ = [(n, c_float_p) for n in ("pos", "vel", "rho_raw", "rho", "pres", "acc", "m", "flt",
                                         "porosity", "pgf", "acc_dem")] + [("n", C.c_int32)]


class BndT(C.Structure):
    _fields_ = [(n, c_float_p) for n in ("pos", "vel", "rho_raw", "rho", "pres", "acc", "m")] + [
        ("n", C.c_int32)]


class CsrT(C.Structure):
    _fields_ = [("offset", c_int_p), ("id", c_int_p), ("tang", c_float_p), ("tang64", c_double_p),
                ("capacity", C.c_int64)]


class DemT(C.Structure):
    _fields_ = ([(n, c_float_p) for n in ("pos", "vel", "acc", "force", "omega", "torque", "radius", "rho",
                                          "m", "volume", "inertia", "K", "eta", "mu", "h")]
                + [("csr_dem", CsrT * 2), ("csr_bnd", CsrT * 2)]
                + [(n, c_float_p) for n in ("flt_s", "porosity", "drag", "pressure_force")]
                + [("n", C.c_int32)])


class DemBndT(C.Structure):
    _fields_ = [(n, c_float_p) for n in ("pos", "vel", "omega", "radius", "rho", "m", "volume", "inertia",
                                         "K", "eta", "mu")] + [("n", C.c_int32)]


class GridT(C.Structure):
    _fields_ = [("lo", C.c_int32 * 3), ("cell", C.c_float), ("inv_cell", C.c_float), ("dim", C.c_int32 * 3),
                ("ncell_local", C.c_int32), ("ninst", C.c_int32), ("n", C.c_int32),
                ("cell_start", c_int_p), ("order", c_int_p), ("key", c_int_p), ("cursor", c_int_p),
                ("block_sums", c_int_p), ("inst", c_int_p)]


class CtlT(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("step", "old_dem", "old_bnd", "status", "e_dem", "e_bnd",
                                         "n_near", "near_next", "n_ptiles", "n_pfb", "n_pchunks")] + [("pad", C.c_int32 * 5)]


class WorkT(C.Structure):
    _fields_ = [("f_posm", c_float_p), ("f_vel", c_float_p), ("f_rp", c_float_p), ("f_vprev", c_float_p),
                ("f_posv", c_float_p), ("f_pgf", c_float_p), ("near_list", c_int_p),
                ("b_posm", c_float_p), ("b_vel", c_float_p), ("b_rp", c_float_p), ("b_vprev", c_float_p),
                ("b_self", c_float_p), ("dem_count", c_int_p), ("dem_aux", c_float_p), ("f_posq", c_float_p),
                ("nbr", c_int_p), ("pfb", c_int_p), ("ptiles", c_int_p), ("ppart", c_float_p), ("pflag", c_int_p),
                ("pfb_words", C.c_int64), ("pframe", C.c_int32), ("pad_work", C.c_int32)]


class ParamsT(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("h", "support", "rho0", "c0", "gamma", "mu", "g", "dt")] + [
        ("shepard_step", C.c_int32)] + [(n, C.c_float) for n in (
            "porosity_min", "porosity_max", "radius_max", "boundary_radius_max", "h_max", "h_uniform")] + [
        ("block_sph", C.c_int32), ("porosity_variant", C.c_int32), ("lanes_sph", C.c_int32),
        ("nbr_cap", C.c_int32), ("nbr_format", C.c_int32)]


class CtxT(C.Structure):
    _fields_ = [("sph", SphT), ("bnd", BndT), ("dem", DemT), ("dembnd", DemBndT), ("grid_sph", GridT),
                ("grid_bnd", GridT), ("grid_dem", GridT), ("grid_dembnd", GridT), ("work", WorkT),
                ("ctl", C.c_void_p)]


c_u16_p = C.POINTER(C.c_uint16)


class MpnnNodesT(C.Structure):
    _fields_ = ([(n, c_float_p) for n in ("f_pos", "f_vel", "f_acc", "f_rho", "f_por")] + [("n_fluid", C.c_int32)]
                + [(n, c_float_p) for n in ("d_pos", "d_vel", "d_acc", "d_rad")] + [("n_dem", C.c_int32)]
                + [(n, c_float_p) for n in ("b_pos", "b_rho")] + [("n_wall", C.c_int32)]
                + [(n, c_float_p) for n in ("w_pos", "w_rad")] + [("n_dem_wall", C.c_int32)]
                + [(n, C.c_float) for n in ("rho0", "inv_vscale", "inv_ascale", "inv_radius")]
                + [(n, c_float_p) for n in ("node_pos3", "node_pos4", "node_vel4")] + [("x", c_u16_p)])


class MpnnNetT(C.Structure):
    _fields_ = ([(n, C.c_int32) for n in ("n_nodes", "n_recv", "edge_capacity", "pad0")]
                + [(n, C.c_float) for n in ("inv_radius", "inv_vscale", "inv_norm", "pad1")]
                + [("node_pos4", c_float_p), ("node_vel4", c_float_p), ("x", c_u16_p), ("offset", c_int_p),
                   ("sender", c_int_p), ("receiver", c_int_p), ("theta", c_float_p), ("packed", c_u16_p),
                   ("z0", c_float_p), ("h0", c_u16_p), ("agg", c_float_p), ("h1", c_u16_p), ("z2", c_float_p),
                   ("h2", c_u16_p), ("h3", c_u16_p), ("out", c_float_p), ("status", c_int_p),
                   ("active", c_int_p), ("active_list", c_int_p)])


class MpnnGradT(C.Structure):
    _fields_ = [("d_out", c_float_p), ("g2", c_float_p), ("d_h2", c_float_p), ("d_h1", c_float_p),
                ("d_h0", c_float_p), ("bf_a", c_u16_p), ("bf_b", c_u16_p), ("partial", c_float_p),
                ("grad", c_float_p)]


class JumpT(C.Structure):
    _fields_ = [("nodes", MpnnNodesT), ("net", MpnnNetT), ("node_grid", GridT), ("scan_scratch", c_int_p),
                ("graph_ctl", C.c_void_p), ("radius", C.c_float), ("substeps", C.c_int32), ("scale", C.c_float * 4),
                ("keep", c_float_p), ("dev", c_float_p), ("judge", C.c_int32), ("pos_tol", C.c_float)]


_MIRRORS = (SphT, BndT, CsrT, DemT, DemBndT, GridT, CtlT, WorkT, ParamsT, CtxT, MpnnNodesT, MpnnNetT, MpnnGradT,
            JumpT)

# Flags and codes of include/sphdem.h
FLAG_CSR_DEM_OVERFLOW = 0x1
FLAG_CSR_BND_OVERFLOW = 0x2
FLAG_NONFINITE = 0x4
FLAG_TIMEOUT = 0x10
ABI_VERSION = 11
NBR_SLOTS, NBR_MASKS = 0, 1  # sphdem_params_t.nbr_format
PHASES = ("grid_sph", "grid_dem", "density", "wall_density", "force", "contacts", "porosity", "exchange",
          "react_integrate", "dem_step")
POROSITY_SLABS = 8
MEMBERS = dict(DENSITY_FLUID=0, DENSITY_WALL=1, FORCE_FLUID=2, FORCE_WALL=3, POROSITY_NEAR=4)
REL = dict(SPH_SPH_SUPPORT=0, SPH_BND_SUPPORT=1, BND_SPH_SUPPORT=2, BND_BND_SUPPORT=3, SPH_SPH_FORCE=4,
           SPH_BND_FORCE=5, SPH_SPH_LEN=6, SPH_DEM_2H=7, DEM_SPH_2H=8, DEM_DEM_2H=9, SPH_DEM_REACT=10)

_lib = None

_SIGNATURES = {
    "sphdem_abi_version": ([], C.c_int),
    "sphdem_last_error": ([], C.c_char_p),
    "sphdem_scan_scratch": ([C.c_int64], C.c_int64),
    "sphdem_struct_sizes": ([C.POINTER(C.c_int64), C.c_int], C.c_int),
    "sphdem_grid_build": ([C.c_void_p, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_refresh_sorted": ([C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_sph_onestep": ([C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p], C.c_int),
    "sphdem_sphdem_onestep": ([C.c_void_p, C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "sphdem_run": ([C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p], C.c_int),
    "sphdem_release": ([C.c_void_p], C.c_int),
    "sphdem_graph_kernels": ([C.c_void_p, C.c_int], C.c_int),
    "sphdem_profile_step": ([C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_shepard_sph": ([C.c_void_p, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "sphdem_density_sph": ([C.c_void_p, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "sphdem_density_bnd": ([C.c_void_p, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "sphdem_pres_sph": ([C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "sphdem_pres_bnd": ([C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "sphdem_force_sph": ([C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "sphdem_step_sph": ([C.c_void_p, C.c_float, C.c_void_p], C.c_int),
    "sphdem_force_dem": ([C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "sphdem_bc_dem": ([C.c_void_p, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "sphdem_step_dem": ([C.c_void_p, C.c_float, C.c_void_p], C.c_int),
    "sphdem_contacts_noalloc": ([C.c_void_p] + [C.c_float] * 4 + [C.c_int, C.c_void_p], C.c_int),
    "sphdem_prep_sphdem": ([C.c_void_p] + [C.c_float] * 6 + [C.c_void_p], C.c_int),
    "sphdem_interaction_dem": ([C.c_void_p] + [C.c_float] * 4 + [C.c_void_p], C.c_int),
    "sphdem_interaction_sph": ([C.c_void_p, C.c_float, C.c_void_p], C.c_int),
    "sphdem_wendland": ([C.c_void_p, C.c_int32, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_drag_beta": ([C.c_void_p] * 5 + [C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_neighbour_digest": ([C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p],
                                C.c_int),
    "sphdem_wait_selftest": ([C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "sphdem_porosity_scratch": ([C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "sphdem_member_digest": ([C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_diagnostics": ([C.c_void_p, C.c_float, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_format_f32": ([C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_int32], C.c_int64),
    "sphdem_format_i32": ([C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_int32], C.c_int64),
    # include/sphdem_mpnn.h
    "sphdem_mpnn_partial_floats": ([], C.c_int64),
    "sphdem_mpnn_pack": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_mpnn_nodes": ([C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_mpnn_graph": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_float] + [C.c_void_p] * 3
                          + [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_mpnn_forward": ([C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "sphdem_mpnn_backward": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_mpnn_loss": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_mpnn_edge_loss": ([C.c_void_p] * 3 + [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_float,
                                                   C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_mpnn_adam": ([C.c_void_p] * 4 + [C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32,
                                             C.c_void_p], C.c_int),
    "sphdem_mpnn_apply": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                           C.c_int32, C.c_void_p, C.c_int32, C.c_float] + [C.c_void_p] * 5, C.c_int),
    "sphdem_mpnn_maxdev": ([C.c_void_p, C.c_void_p, C.c_float, C.c_int32, C.c_float, C.c_void_p, C.c_void_p],
                           C.c_int),
    "sphdem_mpnn_gemm": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                          C.c_void_p], C.c_int),
    "sphdem_jump": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int32, C.c_void_p], C.c_int),
    "sphdem_rollout": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_int32, C.c_void_p,
                        C.c_void_p], C.c_int),
    "sphdem_rollout_kernels": ([C.c_void_p, C.c_int, C.c_int, C.c_int32, C.c_int], C.c_int64),
    "sphdem_jump_undo": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sphdem_jump_kernels": ([C.c_void_p, C.c_int], C.c_int),
    "sphdem_mpnn_wgrad": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                           C.c_void_p], C.c_int),
}

# Symbols declared in include/*.h (checked by the CPU test suite).
EXPORTED = tuple(_SIGNATURES)


class SphdemError(RuntimeError):
    """A libsphdem call returned a non-zero status."""


def library_path() -> Path:
    return LIB


def load(path: Path | None = None):
    """Load libsphdem.so once, bind signatures and check the ABI layout."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the GB300 path has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.sphdem_abi_version() != ABI_VERSION:
        raise RuntimeError(f"libsphdem ABI {lib.sphdem_abi_version()} != binding {ABI_VERSION}")
    check_layout(lib)
    if path is None:
        _lib = lib
    return lib


def check_layout(lib) -> None:
    sizes = (C.c_int64 * 16)()
    n = lib.sphdem_struct_sizes(sizes, 16)
    if n != len(_MIRRORS):
        raise RuntimeError(f"libsphdem reports {n} ABI structs, binding has {len(_MIRRORS)}")
    for k, mirror in enumerate(_MIRRORS[:n]):
        if C.sizeof(mirror) != sizes[k]:
            raise RuntimeError(f"ctypes mirror {mirror.__name__} has size {C.sizeof(mirror)}, "
                               f"library says {sizes[k]}")


def check(rc: int, what: str) -> None:
    if rc != 0:
        msg = _lib.sphdem_last_error().decode() if _lib is not None else ""
        raise SphdemError(f"{what} failed with status {rc}: {msg}")


def fptr(t):
    """float* of a contiguous float32 tensor (or NULL for None)."""
    return C.cast(t.data_ptr(), c_float_p) if t is not None else c_float_p()


def iptr(t):
    return C.cast(t.data_ptr(), c_int_p) if t is not None else c_int_p()


def dptr(t):
    return C.cast(t.data_ptr(), c_double_p) if t is not None else c_double_p()
