"""Frame output from device state: the asynchronous writer (pinned copies on a
side stream, ordered after the step stream) writes the frame of the state at
the moment write_frame was called, even though the run continues meanwhile."""
import numpy as np
import pytest
import torch

from oracle import vtp_oracle as VO

pytestmark = pytest.mark.gpu


def test_async_frames_capture_the_state_at_the_call(tmp_path):
    from warp_sph_gpt_gb300.batch import Case
    from warp_sph_gpt_gb300.generate import config_batch_member
    from warp_sph_gpt_gb300.output import FrameWriter

    case = Case(*config_batch_member(5))
    case.run(0, 5)
    w = FrameWriter(case.solv, case.P, case.B, case.D, case.W, out_dir=str(tmp_path))
    host = lambda part, names: {n: getattr(part, n).cpu().numpy() for n in names}
    expect = VO.vtp_text(VO.sph_dataset(host(case.P, ("pos", "vel", "rho", "pres", "m", "porosity", "pgf", "acc_dem")),
                                        host(case.B, ("pos", "vel", "rho", "pres", "m"))), "pres")
    w.write_frame(5)
    case.run(5, 20)  # queued at once: the frame must still be the state at step 5
    w.write_frame(25)
    w.finalize()
    assert (tmp_path / "sph_000005.vtp").read_text() == expect
    assert (tmp_path / "sph_000025.vtp").read_text() != expect
    assert (tmp_path / "sph.pvd").exists() and (tmp_path / "dem.pvd").exists()
