"""Numeric-header particle text format (restates input/input_reader.py:1-184).

Each file has a whitespace-separated header of integer column IDs and one
particle per row.  IDs restart at 1 for each particle kind, follow the field
order of ``INPUT_FIELDS`` and expand vec3 fields as x/y/z; computed fields have
no IDs and the columns may come in any order.  Files are initial conditions,
not checkpoints.  Validation errors are ``ValueError`` with ``path:line``.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from .struct import STRUCTURES

# (field, scalar-column count) in the documented order (input/input_reader.py:18-30).
INPUT_FIELDS = {
    "SPH": (("pos", 3), ("vel", 3), ("rho", 1), ("m", 1)),
    "BND": (("pos", 3), ("vel", 3), ("rho", 1), ("m", 1)),
    "DEM": (("pos", 3), ("vel", 3), ("omega", 3), ("radius", 1), ("rho", 1), ("m", 1), ("inertia", 1),
            ("K", 1), ("eta", 1), ("mu", 1), ("h", 1)),
    "DEMBND": (("pos", 3), ("vel", 3), ("omega", 3), ("radius", 1), ("rho", 1), ("m", 1), ("inertia", 1),
               ("K", 1), ("eta", 1), ("mu", 1)),
}
_F32_MAX = float(np.finfo(np.float32).max)


def column_indices(kind: str) -> dict[str, tuple[int, ...]]:
    """Documented numeric IDs of each input field (input/input_reader.py:36-45)."""
    if kind not in INPUT_FIELDS:
        raise ValueError(f"unknown particle kind {kind!r}; choose {tuple(INPUT_FIELDS)}")
    index = 1
    result = {}
    for field, width in INPUT_FIELDS[kind]:
        result[field] = tuple(range(index, index + width))
        index += width
    return result


def _parse_rows(path: Path, lines: list[str], width: int) -> np.ndarray:
    """Rows as float64 [n, width]; the first offending line is reported."""
    if not lines:
        return np.zeros((0, width), dtype=np.float64)
    try:
        tokens = " ".join(lines).split()
        if len(tokens) == width * len(lines) and all(len(l.split()) == width for l in lines):
            data = np.array(tokens, dtype=np.float64).reshape(len(lines), width)
            bad = ~np.isfinite(data).all(axis=1) | (np.abs(data) > _F32_MAX).any(axis=1)
            if not bad.any():
                return data
    except ValueError:
        pass
    # Slow path: find the first bad line exactly as the reference reports it.
    rows = []
    for line_number, line in enumerate(lines, 2):
        toks = line.split()
        if len(toks) != width:
            raise ValueError(f"{path}:{line_number}: expected {width} values, got {len(toks)}")
        try:
            row = [float(t) for t in toks]
        except ValueError as exc:
            raise ValueError(f"{path}:{line_number}: invalid numeric value") from exc
        if not np.isfinite(row).all() or np.any(np.abs(row) > _F32_MAX):
            raise ValueError(f"{path}:{line_number}: values must be finite float32 numbers")
        rows.append(row)
    return np.asarray(rows, dtype=np.float64).reshape(-1, width)


def read_table(path: str | Path, kind: str) -> dict[str, np.ndarray]:
    """Parse and validate one particle file (input/input_reader.py:48-95)."""
    path = Path(path)
    columns = column_indices(kind)
    required = {i for ids in columns.values() for i in ids}
    text = path.read_text(encoding="utf-8-sig")
    lines = text.splitlines()
    first = lines[0] if lines else ""
    try:
        header = [int(token) for token in first.split()]
    except ValueError as exc:
        raise ValueError(f"{path}:1: header must contain integer column IDs") from exc
    if not header or len(header) != len(set(header)):
        raise ValueError(f"{path}:1: empty header or duplicate column IDs")
    if set(header) != required:
        raise ValueError(f"{path}:1: missing IDs {sorted(required - set(header))}; "
                         f"unknown IDs {sorted(set(header) - required)}")
    data = _parse_rows(path, lines[1:], len(header))
    result = {}
    for field, ids in columns.items():
        values = data[:, [header.index(i) for i in ids]]
        result[field] = values[:, 0] if len(ids) == 1 else values
    for field in ("rho", "m", "radius", "inertia", "K", "h"):
        if field in result and np.any(result[field].astype(np.float32) <= 0.0):
            raise ValueError(f"{path}: {field} must be positive in float32")
    for field in ("eta", "mu"):
        if field in result and np.any(result[field] < 0.0):
            raise ValueError(f"{path}: {field} must be nonnegative")
    if "radius" in result:
        volume = (4.0 / 3.0) * np.pi * result["radius"] ** 3
        if not np.allclose(result["m"], result["rho"] * volume, rtol=1e-5, atol=0.0):
            raise ValueError(f"{path}: sphere mass must equal rho*(4/3)*pi*radius^3")
        if np.any(volume.astype(np.float32) <= 0) or not np.isfinite(volume.astype(np.float32)).all():
            raise ValueError(f"{path}: derived sphere volume is outside float32 range")
    return result


def input_parser(file_path: str | Path, kind: str | None = None, device: str = "cpu"):
    """Read ``input_<kind>.txt`` into a fully allocated particle struct
    (input/input_reader.py:98-134).  ``kind`` is SPH, BND, DEM or DEMBND and
    is inferred from the file name when omitted.  Header-only files give empty
    structs.  Post-load initialisation: rho_raw = rho, porosity = 1, DEM
    volume = (4/3) pi R^3, and empty contact CSR with zero offsets."""
    path = Path(file_path)
    kind = path.stem.removeprefix("input_") if kind is None else kind
    data = read_table(path, kind)
    n = len(data["pos"])
    particle = STRUCTURES[kind](n, device=device)
    for name, values in data.items():
        setattr(particle, name, torch.as_tensor(np.ascontiguousarray(values), dtype=torch.float32,
                                                device=device))
    if kind in ("SPH", "BND"):
        particle.rho_raw = particle.rho.clone()
    if kind in ("SPH", "DEM"):
        particle.porosity.fill_(1.0)
    if kind in ("DEM", "DEMBND"):
        volume = (4.0 / 3.0) * np.pi * data["radius"] ** 3
        particle.volume = torch.as_tensor(volume, dtype=torch.float32, device=device)
    return particle


def input_directory(solv) -> Path:
    return Path(solv.input_dir)


def dem_search_scales(dem, boundary) -> tuple[float, float, float, float]:
    """Search maxima (Rmax, Rbnd_max, hmax, common h or 0); cache once per run
    (input/input_reader.py:163-168)."""
    h = dem.h.detach().cpu().numpy()
    rb = boundary.radius.detach().cpu().numpy() if boundary is not None else np.zeros(0, np.float32)
    return (float(dem.radius.detach().cpu().numpy().max()),
            float(rb.max()) if rb.shape[0] else 0.0,
            float(h.max()), float(h[0]) if np.all(h == h[0]) else 0.0)


def validate_dem_particles(solv, dem, boundary) -> tuple[float, float, float, float]:
    """Contact dt check from the loaded materials, then the search scales
    (input/input_reader.py:142-160).  The conservative reduced mass min(m)/2
    bounds every moving pair."""
    solv.validate_dem()
    if dem.pos.shape[0] == 0:
        raise ValueError("DEM enabled but input_DEM.txt contains no particles")
    mass = dem.m.detach().cpu().numpy().astype(float)
    stiffness = dem.K.detach().cpu().numpy().astype(float)
    damping = dem.eta.detach().cpu().numpy().astype(float)
    m_eff = 0.5 * mass.min()
    limit = solv.dem_dt_safety * min(np.sqrt(m_eff / stiffness.max()),
                                     m_eff / max(float(damping.max()), 1e-20))
    if solv.dt > limit:
        raise ValueError(f"dt exceeds loaded DEM contact limit {limit:.6g} s")
    return dem_search_scales(dem, boundary)


def load_sph_particles(solv):
    """Read the two or four WCSPH particle files selected by dem_enable
    (input/input_reader.py:171-184)."""
    solv.validate_sph()
    directory = input_directory(solv)
    sph, bnd = (input_parser(directory / f"input_{kind}.txt", kind, solv.device) for kind in ("SPH", "BND"))
    if sph.pos.shape[0] == 0:
        raise ValueError("input_SPH.txt must contain fluid particles")
    dem = dem_bnd = None
    if solv.dem_enable:
        dem, dem_bnd = (input_parser(directory / f"input_{kind}.txt", kind, solv.device)
                        for kind in ("DEM", "DEMBND"))
        validate_dem_particles(solv, dem, dem_bnd)
    return sph, bnd, dem, dem_bnd
