"""Frame output (VTK XML PolyData + ParaView collections), no GPU.

* The native multi-threaded "%.6g" / "%d" formatter gives exactly the text of
  the reference's _fmt_float / _fmt_int (restated in oracle/vtp_oracle.py),
  whatever the thread count.
* FrameWriter writes the reference's files byte for byte (fluid + wall frame,
  DEM frame, both collections) and, like the reference, refuses a frame whose
  state is not finite.
"""
import ctypes as C
import os

import numpy as np
import pytest
import torch

from oracle import vtp_oracle as VO


@pytest.fixture(scope="module")
def lib():
    from warp_sph_gpt_gb300 import _lib, build

    build.build_cuda()
    return _lib.load()


def test_formatter_matches_reference_text(lib):
    from warp_sph_gpt_gb300 import output as O

    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.normal(0, 1, 5000), rng.normal(0, 1e-9, 50), rng.normal(0, 1e9, 50),
                           [0.0, -0.0, 1.0, -1.0, 123456789.0, 1e-40, 3.4e38, 0.1, 2.5e-5]]).astype(np.float32)
    for per_line in (6, 1, 7):
        assert O.fmt_float(vals, per_line) == VO.fmt_float(vals, per_line)
    ints = rng.integers(-10 ** 9, 10 ** 9, 9001).astype(np.int32)
    assert O.fmt_int(ints) == VO.fmt_int(ints)
    assert O.fmt_float(np.zeros(0, np.float32)) == VO.fmt_float(np.zeros(0))
    # thread count does not change the text
    a = np.ascontiguousarray(vals)
    n = a.size
    size = lib.sphdem_format_f32(a.ctypes.data, n, 6, None, 0, 1)
    outs = []
    for threads in (1, 3, 16):
        buf = C.create_string_buffer(size)
        assert lib.sphdem_format_f32(a.ctypes.data, n, 6, buf, size, threads) == size
        outs.append(buf.raw)
    assert outs[0] == outs[1] == outs[2]
    assert lib.sphdem_format_f32(a.ctypes.data, n, 6, C.create_string_buffer(10), 10, 1) == -1


def _small_case():
    from warp_sph_gpt_gb300.generate import CoupledGenerationConfig, build_case

    gen = CoupledGenerationConfig(device="cpu", dx=0.04, h=0.052, dem_nx=2, dem_ny=1, dem_nz=1)
    return gen, build_case(gen, device="cpu")


def _host(part, names):
    return {n: getattr(part, n).numpy().copy() for n in names}


def test_frame_writer_writes_reference_files(tmp_path):
    from warp_sph_gpt_gb300.config import Solv
    from warp_sph_gpt_gb300.output import FrameWriter

    gen, (P, B, D, W) = _small_case()
    rng = np.random.default_rng(1)
    for part in (P, B, D):
        part.vel.copy_(torch.tensor(rng.normal(0, 0.1, part.vel.shape), dtype=torch.float32))
    P.pres.copy_(torch.tensor(rng.normal(0, 50, P.pres.shape), dtype=torch.float32))
    solv = Solv(dt=1e-4)
    w = FrameWriter(solv, P, B, D, W, out_dir=str(tmp_path))
    w.write_frame(0)
    expect0 = (VO.vtp_text(VO.sph_dataset(_host(P, ("pos", "vel", "rho", "pres", "m", "porosity", "pgf", "acc_dem")),
                                          _host(B, ("pos", "vel", "rho", "pres", "m"))), "pres"),
               VO.vtp_text(VO.dem_dataset(_host(D, ("pos", "vel", "omega", "radius", "rho", "m", "volume", "inertia",
                                                    "acc", "force", "torque", "drag", "pressure_force",
                                                    "porosity")),
                                          _host(W, ("pos", "vel", "omega", "radius", "rho", "m", "volume",
                                                    "inertia"))), "radius"))
    P.pos.add_(0.001)  # the next frame sees the new state
    w.write_frame(90)
    w.finalize()
    assert (tmp_path / "sph_000000.vtp").read_text() == expect0[0]
    assert (tmp_path / "dem_000000.vtp").read_text() == expect0[1]
    assert (tmp_path / "sph_000090.vtp").exists() and (tmp_path / "dem_000090.vtp").exists()
    assert (tmp_path / "sph.pvd").read_text() == VO.pvd_text([("sph_000000.vtp", 0.0), ("sph_000090.vtp", 90 * 1e-4)])
    assert (tmp_path / "dem.pvd").read_text() == VO.pvd_text([("dem_000000.vtp", 0.0), ("dem_000090.vtp", 90 * 1e-4)])


def test_frame_writer_refuses_non_finite_state(tmp_path):
    from warp_sph_gpt_gb300.config import Solv
    from warp_sph_gpt_gb300.output import FrameWriter

    gen, (P, B, D, W) = _small_case()
    P.vel[3, 1] = float("nan")
    w = FrameWriter(Solv(dt=1e-4), P, B, out_dir=str(tmp_path))
    w.write_frame(7)
    with pytest.raises(FloatingPointError, match="vel at step 7"):
        w.finalize()
    assert not (tmp_path / "sph_000007.vtp").exists()
