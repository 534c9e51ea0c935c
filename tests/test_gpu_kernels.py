"""Each GPU kernel against the FP64 oracle on identical inputs.

The state is advanced a few coupled steps (positions off the lattice, wet DEM
spheres), copied to the host, then one kernel runs on both sides.  Fields
must agree within 1e-5 (field-normalised max|gpu - ref| / max|ref|) against
the FP64 oracle; the integrators, which round every operation as the
reference does, must agree bit for bit with the FP32 oracle; contact CSR
(offsets, ids) bit for bit.  Known-answer tests of the reference
(tests/test_3d.py:36-53, tests/test_dem.py:494-513) are checked on the GPU's
Wendland and drag-law code.
"""
import numpy as np
import pytest
import torch

from helpers import field_err, scene
from oracle.oracle import HostState
from oracle import oracle as O
from warp_sph_gpt_gb300 import SPHDEM_OneStep, dem_search_scales
from warp_sph_gpt_gb300 import kernels as K

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _np(t):
    return t.detach().cpu().numpy()


@pytest.fixture
def wet():
    s, P, B, D, DB, grids = scene(dem_nx=3, dem_ny=2, dem_origin_x=0.1, dem_origin_y=0.1, dem_spacing=0.05,
                                  dem_origin_z=0.2)
    scales = dem_search_scales(D, DB)
    for step in range(3):
        SPHDEM_OneStep(s, P, B, D, DB, *grids, step, scales)
    torch.cuda.synchronize()
    return s, P, B, D, DB, grids, scales


def test_shepard_density_pressure(wet):
    s, P, B, D, DB, grids, _ = wet
    h = HostState(P, B, D, DB)
    K.Kernel_shepard_sph(P, B, grids[0], grids[1], s.support, s.h)
    h.shepard(s.support, s.h, p="f64")
    assert field_err(_np(P.flt), h.sph["flt"]) < TOL
    h = HostState(P, B, D, DB)
    K.Kernel_density_sph(P, B, grids[0], grids[1], s.support, s.h)
    K.Kernel_density_bnd(P, B, grids[0], grids[1], s.support, s.h)
    h.density_sph(s.support, s.h, p="f64")
    h.density_bnd(s.support, s.h, p="f64")
    assert field_err(_np(P.rho), h.sph["rho"]) < TOL
    assert field_err(_np(B.rho), h.bnd["rho"]) < TOL
    h = HostState(P, B, D, DB)
    K.Kernel_pres_sph(P, s.rho0, s.c0, s.gamma)
    K.Kernel_pres_bnd(B, s.rho0, s.c0, s.gamma)
    h.pres(s.rho0, s.c0, s.gamma, p="f64")
    bulk = s.rho0 * s.c0 ** 2
    for got, ref in ((P.pres, h.sph["pres"]), (B.pres, h.bnd["pres"])):
        got = _np(got).astype(np.float64)
        # pointwise: the expm1/log1p form keeps relative accuracy near rest
        assert np.all(np.abs(got - ref) <= TOL * np.abs(ref) + 1e-9 * bulk)


def test_force_and_pressure_gradient(wet):
    s, P, B, D, DB, grids, scales = wet
    h = HostState(P, B, D, DB)
    K.Kernel_force_sph(P, B, grids[0], grids[1], s.support, s.h, s.mu, s.g)
    h.force_sph(s.support, s.h, s.mu, s.g, p="f64")
    assert field_err(_np(P.acc), h.sph["acc"]) < TOL
    h = HostState(P, B, D, DB)
    K.Kernel_prep_sphdem(P, B, D, grids[0], grids[1], grids[2], 2 * scales[2], scales[3], s.support, s.h,
                         s.dem_porosity_min, s.dem_porosity_max)
    h.prep_sphdem(2 * scales[2], scales[3], s.support, s.h, s.dem_porosity_min, s.dem_porosity_max, p="f64")
    assert field_err(_np(P.pgf), h.sph["pgf"]) < TOL
    assert field_err(_np(P.porosity), h.sph["porosity"]) < TOL
    assert h.sph["porosity"].min() < 0.99  # the wet spheres do lower the fluid fraction


def test_heterogeneous_h_porosity(wet):
    """Per-neighbour normalisation when DEM h differs (h_uniform = 0,
    kernel/KERNEL_SPHDEM_interaction.py:89-95; tests/test_input_reader.py:205-253)."""
    s, P, B, D, DB, grids, _ = wet
    D.h.copy_(torch.linspace(0.04, 0.10, D.n, device=D.h.device))
    h = HostState(P, B, D, DB)
    K.Kernel_prep_sphdem(P, B, D, grids[0], grids[1], grids[2], 0.2, 0.0, s.support, s.h, s.dem_porosity_min,
                         s.dem_porosity_max)
    h.prep_sphdem(0.2, 0.0, s.support, s.h, s.dem_porosity_min, s.dem_porosity_max, p="f64")
    assert field_err(_np(P.porosity), h.sph["porosity"]) < TOL
    assert h.sph["porosity"].min() < 0.99


def test_interaction_dem_and_sph(wet):
    s, P, B, D, DB, grids, scales = wet
    h = HostState(P, B, D, DB)
    K.Kernel_interaction_dem(P, D, grids[0], grids[2], s.mu, s.dem_porosity_min, s.dem_porosity_max, s.dt)
    h.interaction_dem(s.mu, s.dem_porosity_min, s.dem_porosity_max, s.dt, p="f64")
    for name in ("flt_s", "porosity", "drag", "pressure_force", "force"):
        assert field_err(_np(getattr(D, name)), h.dem[name]) < TOL, name
    assert np.abs(h.dem["drag"]).max() > 0
    h = HostState(P, B, D, DB)
    K.Kernel_interaction_sph(P, D, grids[0], grids[2], 2 * scales[2])
    h.interaction_sph(2 * scales[2], p="f64")
    assert field_err(_np(P.acc_dem), h.sph["acc_dem"]) < TOL
    assert field_err(_np(P.acc), h.sph["acc"]) < TOL
    assert np.abs(h.sph["acc_dem"]).max() > 0


def test_dem_contacts_against_oracle(wet):
    s, P, B, D, DB, grids, scales = wet
    # push the spheres into each other and into the floor
    D.pos[:, 2] = 0.015
    D.vel.copy_(torch.randn_like(D.vel) * 0.05)
    D.omega.copy_(torch.randn_like(D.omega))
    grids[2].build(D.pos, s.dem_support)
    for rep in range(3):
        h32 = HostState(P, B, D, DB)
        h64 = HostState(P, B, D, DB)
        K.force_dem(D, grids[2], scales[0], s.g, s.dt)
        K.bc_dem(D, DB, grids[3], scales[1], s.dt)
        for h, p in ((h32, "f32"), (h64, "f64")):
            h.force_dem(scales[0], s.g, s.dt, p=p)
            h.bc_dem(scales[1], s.dt, p=p)
        for kind in ("dem", "bnd"):
            ref = h32.side(kind)
            np.testing.assert_array_equal(_np(getattr(D, f"contact_{kind}_offset_old")), ref["offset"])
            np.testing.assert_array_equal(_np(getattr(D, f"contact_{kind}_id_old")), ref["id"])
            assert field_err(_np(getattr(D, f"tang_{kind}_old")), h64.side(kind)["tang"]) < TOL
        assert int(D.contact_bnd_offset_old[-1]) > 0 and int(D.contact_dem_offset_old[-1]) > 0
        assert field_err(_np(D.force), h64.dem["force"]) < TOL
        assert field_err(_np(D.torque), h64.dem["torque"]) < TOL


def test_integrators_bit_exact(wet):
    s, P, B, D, DB, grids, _ = wet
    h = HostState(P, B, D, DB)
    K.Kernel_step_sph(P, s.dt)
    K.Kernel_step_dem(D, s.dt)
    h.step_sph(s.dt, p="f32")
    h.step_dem(s.dt, p="f32")
    for name in ("pos", "vel"):
        np.testing.assert_array_equal(_np(getattr(P, name)), h.sph[name])
    for name in ("pos", "vel", "acc", "omega"):
        np.testing.assert_array_equal(_np(getattr(D, name)), h.dem[name])


def test_wendland_normalisation_and_derivative():
    """tests/test_3d.py:36-53 on the GPU's Wendland: integral of W over the ball
    is 1 to 6 places, dW/dr matches finite differences, W(2h) = dW(0) = dW(2h) = 0."""
    h = 0.08
    r = torch.linspace(0.0, 2.0 * h, 4001, dtype=torch.float32, device="cuda")
    w, dw = K.wendland(r, h)
    rr, values, slopes = _np(r).astype(float), _np(w), _np(dw)
    integrand = 4.0 * np.pi * rr ** 2 * values
    assert abs(np.sum(0.5 * (integrand[:-1] + integrand[1:]) * np.diff(rr)) - 1.0) < 5e-7
    numerical = np.gradient(values.astype(float), rr)
    np.testing.assert_allclose(slopes[50:-50:100], numerical[50:-50:100], rtol=0.002)
    assert values[-1] == 0.0 and slopes[0] == 0.0 and slopes[-1] == 0.0
    ref_w, ref_dw = O.wendland(_np(r), h)
    assert field_err(values, ref_w) < 1e-6 and field_err(slopes, ref_dw) < 1e-6


def test_drag_branches_and_stokes_limit():
    """Ergun, Wen-Yu Re <= / > 1000 and the zero-speed Stokes limit 18 mu/d^2
    (tests/test_dem.py:494-513), on the GPU's drag law."""
    eps = np.array([0.5, 0.8, 0.9, 1.0, 1.0], np.float32)
    speed = np.array([0.2, 0.1, 0.2, 2.0, 0.0], np.float32)
    got = _np(K.DEM_drag_beta(eps, 1000.0, 0.05, 0.05, speed))
    expected = []
    for e, v in zip(eps.astype(float), speed.astype(float)):
        if e <= 0.80000002:
            expected.append(150 * (1 - e) / e * 0.05 / 0.05 ** 2 + 1.75 * 1000 * v / 0.05)
        elif v == 0:
            expected.append(18 * 0.05 / 0.05 ** 2)
        else:
            re = 1000 * v
            cd = 24 / re * (1 + 0.15 * re ** 0.687) if re <= 1000 else 0.44
            expected.append(0.75 * cd * 1000 * v / 0.05 * e ** -1.65)
    np.testing.assert_allclose(got, expected, rtol=2e-6)
    np.testing.assert_allclose(got, O.drag_beta(eps, 1000.0, 0.05, 0.05, speed), rtol=2e-6)
