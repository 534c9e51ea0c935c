"""Frame output: VTK XML PolyData frames and ParaView collections.

Same files as the reference's writer (output/output.py:113-207,
output/frame_writer.py:9-87): one ASCII ``.vtp`` per frame with the fluid and
the dummy wall stacked (``sph_XXXXXX.vtp``) and, for coupled runs, the moving
and fixed DEM spheres (``dem_XXXXXX.vtp``), tied into ``sph.pvd`` /
``dem.pvd`` time series.  Byte-identical text (tests/test_output.py).

GB300 side: ``FrameWriter.write_frame`` does not stall the step loop.  It
snapshots the frame's fields device-to-device on the step stream (HBM speed),
orders their copy into pinned host buffers on a side CUDA stream, and returns;
a host thread waits for that copy, checks the fields are finite, formats the
arrays with the library's multi-threaded "%.6g" formatter and writes the
files.  A
small ring of pinned buffers bounds the frames in flight.  A non-finite field
raises ``FloatingPointError`` (as the reference does) at the next
``write_frame`` or at ``finalize``, and that frame's files are not written.
The reference's optional GIF (matplotlib) is not produced.
"""
from __future__ import annotations

import ctypes as C
import os
import queue
import threading

import numpy as np
import torch

from . import _lib

SPH_TYPE, BND_TYPE, DEM_TYPE, DEM_BND_TYPE = 1, 0, 2, 3  # output/output.py:9-12

_SPH_FIELDS = ("pos", "vel", "rho", "pres", "m", "porosity", "pgf", "acc_dem", "acc")
_BND_FIELDS = ("pos", "vel", "rho", "pres", "m", "acc")
_DEM_FIELDS = ("pos", "vel", "omega", "radius", "rho", "m", "volume", "inertia", "acc", "force", "torque", "drag",
               "pressure_force", "porosity")
_DEMBND_FIELDS = ("pos", "vel", "omega", "radius", "rho", "m", "volume", "inertia")
# fields checked for finite values before a frame is written (frame_writer.py:48-62)
_CHECK = {"sph": ("pos", "vel", "acc", "rho"), "bnd": ("pos", "vel", "acc", "rho"),
          "dem": ("pos", "vel", "acc", "rho"), "dembnd": ("pos", "vel", "rho")}


def _fmt(a: np.ndarray, per_line: int, integer: bool) -> bytes:
    lib = _lib.load()
    a = np.ascontiguousarray(a, dtype=np.int32 if integer else np.float32)
    fn = lib.sphdem_format_i32 if integer else lib.sphdem_format_f32
    n = a.size
    cap = 16 * n + 16  # "%.6g" of a float or "%d" of an int32 plus a separator fits 16 bytes
    buf = C.create_string_buffer(cap)
    got = fn(a.ctypes.data, n, per_line, buf, cap, 0)
    if got < 0:
        raise RuntimeError("frame formatting failed")
    return buf.raw[:got]


_VERTS: dict = {}


def _verts(n: int) -> bytes:
    """Connectivity and offsets text of n vertex cells (the same every frame)."""
    if n not in _VERTS:
        _VERTS.clear()
        _VERTS[n] = (_fmt(np.arange(n, dtype=np.int32), 20, True), _fmt(np.arange(1, n + 1, dtype=np.int32), 20, True))
    return _VERTS[n]


def fmt_float(a, per_line: int = 6) -> str:
    """output/output.py:16-19 with the native formatter."""
    return _fmt(np.asarray(a), per_line, False).decode()


def fmt_int(a, per_line: int = 20) -> str:
    """output/output.py:22-25 with the native formatter."""
    return _fmt(np.asarray(a), per_line, True).decode()


def sph_dataset(sph: dict, bnd: dict) -> dict:
    """Fluid then dummy-boundary points (output/output.py:28-62)."""
    n_sph, n_bnd = len(sph["pos"]), len(bnd["pos"])
    return {
        "pos": np.vstack([sph["pos"], bnd["pos"]]),
        "vel": np.vstack([sph["vel"], bnd["vel"]]),
        "rho": np.concatenate([sph["rho"], bnd["rho"]]),
        "pres": np.concatenate([sph["pres"], bnd["pres"]]),
        "m": np.concatenate([sph["m"], bnd["m"]]),
        "porosity": np.concatenate([sph["porosity"], np.ones(n_bnd, np.float32)]),
        "pgf": np.vstack([sph["pgf"], np.zeros((n_bnd, 3), np.float32)]),
        "acc_dem": np.vstack([sph["acc_dem"], np.zeros((n_bnd, 3), np.float32)]),
        "type": np.concatenate([np.full(n_sph, SPH_TYPE, np.int32), np.full(n_bnd, BND_TYPE, np.int32)]),
    }


def dem_dataset(dem: dict, wall: dict) -> dict:
    """Moving then fixed DEM spheres (output/output.py:85-110)."""
    n_bnd = len(wall["pos"])
    d = {k: np.concatenate([dem[k], wall[k]]) for k in ("pos", "vel", "omega", "radius", "rho", "m", "volume",
                                                         "inertia")}
    for k in ("acc", "force", "torque"):
        d[k] = np.vstack([dem[k], np.zeros((n_bnd, 3), np.float32)])
    d["type"] = np.concatenate([np.full(len(dem["pos"]), DEM_TYPE, np.int32), np.full(n_bnd, DEM_BND_TYPE, np.int32)])
    for k in ("drag", "pressure_force"):
        d[k] = np.vstack([dem[k], np.zeros((n_bnd, 3), np.float32)])
    d["porosity"] = np.concatenate([dem["porosity"], np.ones(n_bnd, np.float32)])
    return d


def vtp_bytes(d: dict, scalar: str) -> bytes:
    """One VTK XML PolyData file (output/output.py:113-176), vertex per point."""
    n = d["pos"].shape[0]
    parts = [b'<?xml version="1.0"?>\n', b'<VTKFile type="PolyData" version="0.1" byte_order="LittleEndian">\n',
             b'  <PolyData>\n',
             f'    <Piece NumberOfPoints="{n}" NumberOfVerts="{n}" '
             'NumberOfLines="0" NumberOfStrips="0" NumberOfPolys="0">\n'.encode(),
             b'      <Points>\n',
             b'        <DataArray type="Float32" Name="Points" NumberOfComponents="3" format="ascii">\n',
             _fmt(d["pos"], 6, False), b"\n", b'        </DataArray>\n', b'      </Points>\n', b'      <Verts>\n',
             b'        <DataArray type="Int32" Name="connectivity" format="ascii">\n',
             _verts(n)[0], b"\n", b'        </DataArray>\n',
             b'        <DataArray type="Int32" Name="offsets" format="ascii">\n',
             _verts(n)[1], b"\n", b'        </DataArray>\n',
             b'      </Verts>\n', f'      <PointData Scalars="{scalar}" Vectors="vel">\n'.encode()]
    for key, values in d.items():
        if key == "pos":
            continue
        integer = key == "type"
        components = ' NumberOfComponents="3"' if values.ndim == 2 else ""
        parts.append(f'        <DataArray type="{"Int32" if integer else "Float32"}" Name="{key}"{components} '
                     'format="ascii">\n'.encode())
        parts += [_fmt(values, 20 if integer else 6, integer), b"\n", b'        </DataArray>\n']
    parts += [b'      </PointData>\n', b'    </Piece>\n', b'  </PolyData>\n', b'</VTKFile>\n']
    return b"".join(parts)


def pvd_bytes(frames) -> bytes:
    """The ParaView collection (output/output.py:179-207)."""
    out = ['<?xml version="1.0"?>\n', '<VTKFile type="Collection" version="0.1" byte_order="LittleEndian">\n',
           '  <Collection>\n']
    out += [f'    <DataSet timestep="{t:.9g}" group="" part="0" file="{fname}"/>\n' for fname, t in frames]
    out += ['  </Collection>\n', '</VTKFile>\n']
    return "".join(out).encode()


def save_pvd(frames, out_dir: str, name: str = "ptl") -> str:
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, f"{name}.pvd")
    with open(path, "wb") as f:
        f.write(pvd_bytes(frames))
    return path


class _Slot:
    """Device staging and pinned host copies of every field one frame needs."""

    def __init__(self, parts):
        self.host, self.dev = {}, {}
        for kind, part, names in parts:
            for name in names:
                t = getattr(part, name)
                self.host[(kind, name)] = torch.empty(t.shape, dtype=t.dtype, pin_memory=t.is_cuda)
                if t.is_cuda:
                    self.dev[(kind, name)] = torch.empty_like(t)
        self.event = None

    def arrays(self, kind, names):
        return {n: self.host[(kind, n)].numpy() for n in names}


class FrameWriter:
    """Drop-in for output/frame_writer.py:FrameWriter (VTP/PVD part)."""

    def __init__(self, solv, P_sph, P_bnd, P_dem=None, P_dem_bnd=None, slots: int = 2, out_dir: str | None = None):
        if (P_dem is None) != (P_dem_bnd is None):
            raise ValueError("provide both moving and fixed DEM particles")
        self.solv = solv
        self.out_dir = out_dir or solv.output_dir
        self.coupled = P_dem is not None
        self.parts = [("sph", P_sph, _SPH_FIELDS), ("bnd", P_bnd, _BND_FIELDS)]
        if self.coupled:
            self.parts += [("dem", P_dem, _DEM_FIELDS), ("dembnd", P_dem_bnd, _DEMBND_FIELDS)]
        self.cuda = P_sph.pos.is_cuda
        self.stream = torch.cuda.Stream(device=P_sph.pos.device) if self.cuda else None
        self.free: queue.Queue = queue.Queue()
        for _ in range(max(1, slots)):
            self.free.put(_Slot(self.parts))
        self.jobs: queue.Queue = queue.Queue()
        self.error: BaseException | None = None
        self.frames: list[tuple[str, float]] = []
        self.dem_frames: list[tuple[str, float]] = []
        self.thread = threading.Thread(target=self._work, daemon=True)
        self.thread.start()

    # -- step-loop side ------------------------------------------------------------
    def write_frame(self, step: int) -> None:
        """Queue one frame of the state after `step` steps (step 0 = initial)."""
        self._raise()
        slot = self.free.get()  # blocks only when every buffer is in flight
        t = step * self.solv.dt
        if self.cuda:
            # device-to-device snapshot on the step stream (fast, so the run goes
            # on at once), then the host copy on the side stream
            main = torch.cuda.current_stream(self.stream.device)
            for kind, part, names in self.parts:
                for name in names:
                    slot.dev[(kind, name)].copy_(getattr(part, name), non_blocking=True)
            self.stream.wait_stream(main)
            with torch.cuda.stream(self.stream):
                for key, dev in slot.dev.items():
                    slot.host[key].copy_(dev, non_blocking=True)
                slot.event = torch.cuda.Event()
                slot.event.record(self.stream)
        else:
            for kind, part, names in self.parts:
                for name in names:
                    slot.host[(kind, name)].copy_(getattr(part, name))
        fname = f"sph_{step:06d}.vtp"
        dname = f"dem_{step:06d}.vtp" if self.coupled else None
        self.frames.append((fname, t))
        if self.coupled:
            self.dem_frames.append((dname, t))
        self.jobs.put((slot, step, fname, dname))

    def finalize(self) -> None:
        """Wait for the queued frames, then write the PVD collections."""
        self.jobs.put(None)
        self.thread.join()
        self._raise()
        if self.frames:
            save_pvd(self.frames, self.out_dir, "sph")
        if self.dem_frames:
            save_pvd(self.dem_frames, self.out_dir, "dem")

    # -- writer thread -------------------------------------------------------------
    def _work(self) -> None:
        while True:
            job = self.jobs.get()
            if job is None:
                return
            slot, step, fname, dname = job
            try:
                if slot.event is not None:
                    slot.event.synchronize()
                if self.error is None:
                    self._write(slot, step, fname, dname)
            except BaseException as exc:  # surfaced on the step-loop side
                if self.error is None:
                    self.error = exc
            finally:
                self.free.put(slot)

    def _write(self, slot, step, fname, dname) -> None:
        for kind, names in _CHECK.items():
            if kind in ("dem", "dembnd") and not self.coupled:
                continue
            for name in names:
                if not np.isfinite(slot.host[(kind, name)].numpy()).all():
                    raise FloatingPointError(f"non-finite {name} at step {step}")
        os.makedirs(self.out_dir, exist_ok=True)
        d = sph_dataset(slot.arrays("sph", _SPH_FIELDS), slot.arrays("bnd", _BND_FIELDS))
        with open(os.path.join(self.out_dir, fname), "wb") as f:
            f.write(vtp_bytes(d, "pres"))
        if self.coupled:
            d = dem_dataset(slot.arrays("dem", _DEM_FIELDS), slot.arrays("dembnd", _DEMBND_FIELDS))
            with open(os.path.join(self.out_dir, dname), "wb") as f:
                f.write(vtp_bytes(d, "radius"))

    def _raise(self) -> None:
        if self.error is not None:
            err, self.error = self.error, None
            raise err
