"""Multi-step behaviour on the GPU.

* 100-step rollout of config 1 (the reference's own input files, regenerated
  byte-identically) against the FP32 oracle.  Stated tolerance: after 100
  steps every fluid and DEM position within 1e-3 dx (2e-5 m) of the oracle's,
  densities within 1e-4 relative (field-normalised), contact CSR identical.
  Both sides are FP32 with different summation orders, so trajectories
  separate slowly; this bounds that drift.
* CUDA-graph replay (run_steps / run_forward) gives bit-identical states to
  calling SPHDEM_OneStep step by step.
* FP64 diagnostics: total mass exact, momentum and energy match the oracle.
"""
import tempfile

import numpy as np
import pytest
import torch

from oracle.oracle import HostState
from warp_sph_gpt_gb300 import HashGrid, SPHDEM_OneStep, dem_search_scales, load_sph_particles, run_forward, run_steps
from warp_sph_gpt_gb300.generate import build_case, config_small, generate_files, solver_config
from warp_sph_gpt_gb300.kernels import diagnostics

pytestmark = pytest.mark.gpu


def _grids(solv, P, B, D, W, scales):
    g = [HashGrid(64, 64, 64) for _ in range(4)]
    g[0].build(P.pos, solv.support)
    g[1].build(B.pos, solv.support)
    g[2].build(D.pos, max(2 * scales[0], 2 * scales[2]))
    g[3].build(W.pos, max(2 * scales[1], solv.support))
    return g


def test_config1_100_step_rollout_against_oracle():
    gen = config_small()
    with tempfile.TemporaryDirectory() as d:
        generate_files(d, gen)
        solv = solver_config(gen, device="cuda", input_dir=d, n_steps=100)
        P, B, D, W = load_sph_particles(solv)
    scales = dem_search_scales(D, W)
    host = HostState(P, B, D, W)
    grids = _grids(solv, P, B, D, W, scales)
    run_steps(solv, P, B, grids[0], grids[1], D, W, grids[2], grids[3], first_step=0, n_steps=100,
              search_scales=scales)
    for step in range(100):
        host.sphdem_onestep(solv, step, scales, p="f32")
    torch.cuda.synchronize()
    dx = 0.02
    assert np.abs(P.pos.cpu().numpy() - host.sph["pos"]).max() < 1e-3 * dx
    assert np.abs(D.pos.cpu().numpy() - host.dem["pos"]).max() < 1e-3 * dx
    rho = P.rho.cpu().numpy().astype(np.float64)
    assert np.abs(rho - host.sph["rho"]).max() / np.abs(host.sph["rho"]).max() < 1e-4
    for kind in ("dem", "bnd"):
        np.testing.assert_array_equal(getattr(D, f"contact_{kind}_offset_old").cpu().numpy(),
                                      host.side(kind)["offset"])
    assert P.pos.cpu().numpy()[:, 0].max() > 0.48  # the front (initially x = 0.48) has started to move


def test_graph_replay_equals_step_api():
    gen, pos, rad = config_small(), None, None
    s = solver_config(gen)
    states = [build_case(gen, device="cuda") for _ in range(2)]
    scales = dem_search_scales(states[0][2], states[0][3])
    ga = _grids(s, *states[0], scales)
    gb = _grids(s, *states[1], scales)
    P, B, D, W = states[0]
    run_steps(s, P, B, ga[0], ga[1], D, W, ga[2], ga[3], first_step=0, n_steps=25, search_scales=scales)
    P2, B2, D2, W2 = states[1]
    for step in range(25):
        SPHDEM_OneStep(s, P2, B2, D2, W2, *gb, step, scales)
    torch.cuda.synchronize()
    for a, b in ((P, P2), (D, D2)):
        for name in ("pos", "vel", "acc"):
            np.testing.assert_array_equal(getattr(a, name).cpu().numpy(), getattr(b, name).cpu().numpy())
    np.testing.assert_array_equal(D.contact_dem_id_old.cpu().numpy(), D2.contact_dem_id_old.cpu().numpy())


def test_run_forward_frames_and_diagnostics():
    gen = config_small()
    s = solver_config(gen, n_steps=30, output_step=10)
    P, B, D, W = build_case(gen, device="cuda")
    host = HostState(P, B, D, W)
    d0 = diagnostics(P, D, s.g).cpu().numpy()
    np.testing.assert_allclose(d0, host.diagnostics(s.g), rtol=1e-12, atol=1e-9)
    frames = []
    run_forward(s, P, B, *[HashGrid() for _ in range(2)], D, W, *[HashGrid() for _ in range(2)],
                on_frame=frames.append)
    assert frames == [0, 10, 20, 30]
    d1 = diagnostics(P, D, s.g).cpu().numpy()
    assert d1[0] == d0[0] and d1[1] == d0[1]  # mass is conserved exactly
    assert d1[7] < d0[7]  # potential energy falls as the column collapses
    np.testing.assert_allclose(d1, HostState(P, B, D, W).diagnostics(s.g), rtol=1e-9, atol=1e-9)
