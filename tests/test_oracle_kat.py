"""The CPU oracle against the reference's own known-answer tests (no GPU).

Each test restates one analytic check of the reference's suite
(tests/test_dem.py, tests/test_3d.py, tests/test_input_reader.py) on the
oracle, which pins the oracle to the reference before it is used to judge the
GPU path.  States come from the project's restatement of input_gen on CPU
tensors; the FP32 oracle build has the reference's rounding.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle.oracle import HostState
from warp_sph_gpt_gb300.generate import CoupledGenerationConfig, DamPtlGeneration, DEMPtlGeneration


def scene(**kwargs):
    settings = dict(dx=0.04, h=0.052, support=0.104, tank_width=0.8, tank_height=0.8, tank_depth=0.32,
                    fluid_width=0.4, fluid_height=0.4, fluid_depth=0.32, dem_nx=2, dem_ny=1, dem_nz=1,
                    dem_origin_y=0.16, dem_origin_z=0.60, grid_slice=32)
    settings.update(kwargs)
    s = CoupledGenerationConfig(device="cpu", **settings)
    P, B = DamPtlGeneration(s).build("cpu")
    D, DB = DEMPtlGeneration(s).build("cpu")
    return s, HostState(P, B, D, DB)


def hist(h, kind, a, b):
    side = h.side(kind)
    for k in range(int(side["offset"][a]), int(side["offset"][a + 1])):
        if int(side["id"][k]) == b:
            return side["tang"][k]
    raise KeyError((kind, a, b))


def test_wendland_volume_normalisation_and_derivative():
    """tests/test_3d.py:36-53."""
    h = 0.08
    r = np.linspace(0.0, 2.0 * h, 4001, dtype=np.float32)
    for p in ("f32", "f64"):
        w, dw = O.wendland(r, h, p)
        integrand = 4.0 * np.pi * r.astype(float) ** 2 * w
        assert abs(np.sum(0.5 * (integrand[:-1] + integrand[1:]) * np.diff(r.astype(float))) - 1.0) < 5e-7
        np.testing.assert_allclose(dw[50:-50:100], np.gradient(w, r.astype(float))[50:-50:100], rtol=0.002)
        assert w[-1] == 0.0 and dw[0] == 0.0 and dw[-1] == 0.0


def test_drag_branches_and_stokes_limit():
    """tests/test_dem.py:494-513 (Ergun, Wen-Yu Re <= / > 1000, Stokes limit)."""
    eps = np.array([0.5, 0.8, 0.9, 1.0, 1.0], np.float32)
    speed = np.array([0.2, 0.1, 0.2, 2.0, 0.0], np.float32)
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
    for p in ("f32", "f64"):
        np.testing.assert_allclose(O.drag_beta(eps, 1000.0, 0.05, 0.05, speed, p), expected, rtol=2e-6)


def test_normal_contact_release_and_fresh_recontact():
    """tests/test_dem.py:386-416."""
    s, h = scene(dem_nx=2, dem_ny=1)
    h.dem["pos"][:] = [[0.2, 0.16, 0.6], [0.249, 0.16, 0.6]]
    h.dem["vel"][:] = [[1, 0, 0], [-1, 0, 0]]
    h.force_dem(s.dem_radius, 0.0, s.dt)
    expected = s.dem_K * 0.001 + s.dem_eta * 2
    np.testing.assert_allclose(h.dem["force"], [[-expected, 0, 0], [expected, 0, 0]], rtol=2e-5, atol=0.01)
    np.testing.assert_allclose(h.dem["force"].sum(axis=0), 0, atol=1e-6)
    h.dem["pos"][:] = [[0.2, 0.16, 0.6], [1.5, 0.16, 0.6]]
    assert h.force_dem(s.dem_radius, 0.0, s.dt) == 0
    np.testing.assert_array_equal(h.dem["force"], 0)
    h.dem["pos"][:] = [[0.2, 0.16, 0.6], [0.249, 0.16, 0.6]]
    h.dem["vel"][:] = [[0, 0, 0], [0, 0.01, 0]]
    h.force_dem(s.dem_radius, 0.0, s.dt)
    assert abs(float(hist(h, "dem", 0, 1)[1]) - 0.01 * s.dt) < 1e-8


def test_friction_history_torque_spin_and_coulomb_limit():
    """tests/test_dem.py:418-444."""
    s, h = scene(dem_nx=2, dem_ny=1)
    h.dem["pos"][:] = [[0.2, 0.16, 0.6], [0.249, 0.16, 0.6]]
    h.dem["vel"][:] = [[0, 0, 0], [0, 0.01, 0]]
    for count in (1, 2):
        h.force_dem(s.dem_radius, 0.0, s.dt)
        tangential = s.dem_K * 0.01 * s.dt * count + s.dem_eta * 0.01
        assert abs(float(h.dem["force"][0, 1]) - tangential) < 1e-5
        assert abs(float(hist(h, "dem", 0, 1)[1]) - count * 0.01 * s.dt) < 1e-8
    torque = h.dem["torque"].copy()
    np.testing.assert_allclose(torque[:, 2], 0.0245 * tangential, rtol=1e-5)
    h.step_dem(s.dt)
    np.testing.assert_allclose(h.dem["omega"][:, 2], torque[:, 2] / s.dem_inertia * s.dt, rtol=1e-5)
    h.dem["vel"][:] = [[0, 0, 0], [0, 10, 0]]
    h.dem["omega"][:] = 0
    h.dem["pos"][:] = [[0.2, 0.16, 0.6], [0.249, 0.16, 0.6]]
    h.force_dem(s.dem_radius, 0.0, s.dt)
    assert abs(float(h.dem["force"][0, 1]) - s.dem_mu * s.dem_K * 0.001) < 0.01


def test_csr_lifecycle_0_2_6_2_0_2():
    """tests/test_dem.py:199-286: exact counts, rows, survivor history."""
    s, h = scene(dem_nx=3)
    assert h.force_dem(s.dem_radius, 0.0, s.dt) == 0
    pair = [[0.200, 0.16, 0.60], [0.249, 0.16, 0.60], [0.600, 0.16, 0.60]]
    h.dem["pos"][:] = pair
    h.dem["vel"][:] = [[0, 0, 0], [0, 0.01, 0], [0, 0, 0]]
    assert h.force_dem(s.dem_radius, 0.0, s.dt) == 2
    first = hist(h, "dem", 0, 1).copy()
    h.dem["pos"][:] = [0.3, 0.16, 0.6]
    assert h.force_dem(s.dem_radius, 0.0, s.dt) == 6
    side = h.side("dem")
    np.testing.assert_array_equal(np.diff(side["offset"]), [2, 2, 2])
    for a in range(3):
        assert set(side["id"][side["offset"][a]:side["offset"][a + 1]]) == {0, 1, 2} - {a}
    h.dem["pos"][:] = pair
    assert h.force_dem(s.dem_radius, 0.0, s.dt) == 2
    np.testing.assert_allclose(hist(h, "dem", 0, 1), 3.0 * first, rtol=1e-6, atol=1e-9)
    h.dem["pos"][:] = [[0.1, 0.16, 0.60], [0.4, 0.16, 0.60], [0.7, 0.16, 0.60]]
    assert h.force_dem(s.dem_radius, 0.0, s.dt) == 0
    h.dem["pos"][:] = pair
    assert h.force_dem(s.dem_radius, 0.0, s.dt) == 2
    np.testing.assert_allclose(hist(h, "dem", 0, 1), first, rtol=1e-6, atol=1e-9)


def test_row_replacement_keeps_survivor():
    """tests/test_dem.py:320-357."""
    s, h = scene(dem_nx=4)
    first = np.array([[0.300, 0.16, 0.600], [0.349, 0.16, 0.600], [0.251, 0.16, 0.600], [0.600, 0.16, 0.700]],
                     np.float32)
    h.dem["pos"][:] = first
    h.dem["vel"][:] = [[0, 0, 0], [0, 0, 0], [0, 0.01, 0], [0.01, 0, 0]]
    assert h.force_dem(s.dem_radius, 0.0, s.dt) == 4
    t02 = hist(h, "dem", 0, 2).copy()
    second = first.copy()
    second[1] = [0.600, 0.16, 0.600]
    second[3] = [0.300, 0.16, 0.649]
    h.dem["pos"][:] = second
    assert h.force_dem(s.dem_radius, 0.0, s.dt) == 4
    side = h.side("dem")
    assert set(side["id"][side["offset"][0]:side["offset"][1]]) == {2, 3}
    np.testing.assert_allclose(hist(h, "dem", 0, 2), 2.0 * t02, rtol=1e-6, atol=1e-9)


def test_oblique_contact_and_three_axis_translation():
    """tests/test_3d.py:104-121."""
    s, h = scene(dem_nx=2)
    n = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    pos = np.array([[0.2, 0.12, 0.6], [0.2, 0.12, 0.6] + 0.049 * n], np.float32)
    h.dem["pos"][:] = pos
    h.dem["vel"][:] = np.array([n, -n], np.float32)
    h.force_dem(s.dem_radius, 0.0, s.dt)
    np.testing.assert_allclose(h.dem["force"][0], -(s.dem_K * 0.001 + 2 * s.dem_eta) * n, rtol=5e-5, atol=0.002)
    np.testing.assert_allclose(h.dem["force"].sum(axis=0), 0.0, atol=1e-5)
    velocity = h.dem["vel"] + h.dem["force"] / s.dem_mass * s.dt
    h.step_dem(s.dt)
    np.testing.assert_allclose(h.dem["pos"], pos + velocity * s.dt, atol=1e-7)


def test_transverse_slip_x_torque():
    """tests/test_3d.py:123-138."""
    s, h = scene(dem_nx=2)
    h.dem["pos"][:] = [[0.2, 0.10, 0.6], [0.2, 0.149, 0.6]]
    h.dem["vel"][:] = [[0, 0, 0], [0, 0, 0.01]]
    h.force_dem(s.dem_radius, 0.0, s.dt)
    tangential = s.dem_K * 0.01 * s.dt + s.dem_eta * 0.01
    np.testing.assert_allclose(h.dem["torque"][:, 0], 0.0245 * tangential, rtol=1e-5)


@pytest.mark.parametrize("back", [False, True])
def test_front_and_back_wall_contacts(back):
    """tests/test_3d.py:140-158."""
    s, h = scene(dem_nx=1)
    sign = -1.0 if back else 1.0
    h.dem["pos"][:] = [0.4, s.tank_depth - 0.02 if back else 0.02, 0.4]
    h.dem["vel"][:] = [0.1, -sign * 0.2, 0.0]
    wall = h.dembnd["pos"].copy()
    assert h.bc_dem(s.dem_bnd_radius, s.dt) > 0
    assert sign * h.dem["force"][0, 1] > 0
    assert np.linalg.norm(h.dem["torque"][0]) > 0
    np.testing.assert_array_equal(h.dembnd["pos"], wall)


def test_floor_wall_contact_history_release_and_recontact():
    """tests/test_dem.py:446-492."""
    s, h = scene(dem_nx=1, dem_ny=1)
    h.dem["pos"][:] = [[0.4, 0.16, 0.020]]
    h.dem["vel"][:] = [0.1, 0.0, -0.2]
    n = h.bc_dem(s.dem_bnd_radius, s.dt)
    assert n > 0
    nb = int(h.side("bnd")["id"][0])
    first = hist(h, "bnd", 0, nb).copy()
    assert np.linalg.norm(first) > 0 and h.dem["force"][0, 2] > 0
    h.dem["pos"][:] = [0.4, 0.16, 0.8]
    assert h.bc_dem(s.dem_bnd_radius, s.dt) == 0
    h.dem["pos"][:] = [[0.4, 0.16, 0.020]]
    h.dem["vel"][:] = [0.1, 0.0, -0.2]
    h.dem["omega"][:] = 0
    h.dem["force"][:] = 0
    h.dem["torque"][:] = 0
    h.bc_dem(s.dem_bnd_radius, s.dt)
    np.testing.assert_allclose(hist(h, "bnd", 0, nb), first, rtol=1e-6, atol=1e-9)


def test_gravity_along_negative_z():
    """tests/test_3d.py:87-102."""
    s, h = scene()
    h.force_sph(s.support, s.h, s.mu, s.g)
    exp = np.zeros_like(h.sph["acc"])
    exp[:, 2] = -s.g
    np.testing.assert_allclose(h.sph["acc"], exp, rtol=1e-7)
    h.force_dem(s.dem_radius, s.g, s.dt)
    exp = np.zeros_like(h.dem["force"])
    exp[:, 2] = -s.dem_mass * s.g
    np.testing.assert_allclose(h.dem["force"], exp, rtol=1e-7)


def test_buoyancy_bounded_drag_weighted_reaction_and_dry_reset():
    """tests/test_dem.py:515-556."""
    s, h = scene(dem_nx=1, dem_ny=1)
    h.dem["pos"][:] = [0.24, 0.24, 0.16]
    h.sph["vel"][:] = [0.2, 0, 0]
    h.sph["pgf"][:] = [0, 0, s.rho0 * s.g]
    h.sph["porosity"][:] = 0.7
    h.interaction_dem(s.mu, s.dem_porosity_min, s.dem_porosity_max, s.dt)
    np.testing.assert_allclose(h.dem["pressure_force"][0], [0, 0, s.dem_volume * s.rho0 * s.g], rtol=2e-6)
    assert h.dem["drag"][0, 0] > 0 and h.dem["drag"][0, 0] / s.dem_mass * s.dt < 0.2
    h.sph["acc"][:] = [1.0, 0.0, -s.g]
    acc0 = h.sph["acc"].copy()
    h.interaction_sph(s.dem_support)
    reaction = np.sum(h.sph["m"][:, None] * h.sph["porosity"][:, None] * h.sph["acc_dem"], axis=0)
    np.testing.assert_allclose(reaction, -h.dem["drag"].sum(axis=0), rtol=3e-6, atol=1e-5)
    np.testing.assert_allclose(h.sph["acc"], acc0 + h.sph["acc_dem"], rtol=1e-6)
    h.dem["pos"][:] = [0.24, 0.16, 2.0]
    h.interaction_dem(s.mu, s.dem_porosity_min, s.dem_porosity_max, s.dt)
    for f in ("drag", "pressure_force", "flt_s"):
        np.testing.assert_array_equal(h.dem[f], 0)
    prev = h.sph["acc"].copy()
    h.interaction_sph(s.dem_support)
    np.testing.assert_array_equal(h.sph["acc_dem"], 0.0)
    np.testing.assert_array_equal(h.sph["acc"], prev)


def test_hydrostatic_pressure_gradient_sign():
    """tests/test_dem.py:558-572 and the xyz gradient of tests/test_3d.py:160-172."""
    for gradient in (np.array([0.0, 0.0, -1000.0 * 9.81]), np.array([400.0, -900.0, 700.0])):
        s, h = scene(dem_nx=1)
        for part in (h.sph, h.bnd):
            part["pres"][:] = (10000.0 + part["pos"] @ gradient).astype(np.float32)
        h.prep_sphdem(s.dem_support, s.dem_h, s.support, s.h, s.dem_porosity_min, s.dem_porosity_max)
        centre = np.argmin(np.linalg.norm(h.sph["pos"] - [0.24 if gradient[0] == 0 else 0.2, 0.16 if gradient[0] == 0
                                                          else 0.2, 0.24 if gradient[0] == 0 else 0.16], axis=1))
        np.testing.assert_allclose(h.sph["pgf"][centre], -gradient, rtol=0.06, atol=0.02)


def test_heterogeneous_h_porosity_against_numpy_brute_force():
    """tests/test_input_reader.py:205-253: per-neighbour normalisation, rtol 2e-6."""
    s, h = scene(dem_nx=2, dem_ny=1, dem_origin_z=0.2)
    h.dem["h"][:] = [0.04, 0.10]
    h.sph["vel"][:] = [0.5, -0.2, 0.3]
    h.prep_sphdem(0.2, 0.0, s.support, s.h, s.dem_porosity_min, s.dem_porosity_max, p="f64")
    pos, centres = h.sph["pos"].astype(float), h.dem["pos"].astype(float)
    vol = (h.sph["m"] / h.sph["rho"]).astype(float)
    sample = np.arange(0, len(pos), 17)
    solid = np.zeros(len(sample))

    def weight(d, hh):
        q = d / hh
        return np.where(q < 2, 21 / (16 * np.pi * hh ** 3) * (1 - q / 2) ** 4 * (1 + 2 * q), 0)

    for b, hb in enumerate(h.dem["h"].astype(float)):
        norm = (weight(np.linalg.norm(pos[sample, None] - pos[None], axis=2), hb) * vol[None]).sum(axis=1)
        solid += h.dem["volume"][b] * weight(np.linalg.norm(pos[sample] - centres[b], axis=1), hb) / (norm + 1e-20)
    np.testing.assert_allclose(h.sph["porosity"][sample], np.clip(1 - solid, s.dem_porosity_min, s.dem_porosity_max),
                               rtol=2e-6, atol=2e-6)
    assert h.sph["porosity"].min() < 0.99


def test_dry_free_fall_matches_sph_only():
    """tests/test_dem.py:574-597 on the oracle: coupled step with far DEM ==
    SPH-only step, and free fall of the DEM."""
    s, h = scene(dem_origin_z=1.5)
    _, h0 = scene(dem_origin_z=1.5)
    from warp_sph_gpt_gb300 import dem_search_scales

    P = type("P", (), {})
    scales = (s.dem_radius, s.dem_bnd_radius, s.dem_h, s.dem_h)
    z0 = h.dem["pos"][:, 2].copy()
    for step in range(5):
        h0.sph_onestep(s, step, True)
        h.sphdem_onestep(s, step, scales)
    np.testing.assert_array_equal(h.sph["pos"], h0.sph["pos"])
    np.testing.assert_array_equal(h.sph["vel"], h0.sph["vel"])
    np.testing.assert_allclose(h.dem["vel"][:, 2], -5 * s.g * s.dt, rtol=1e-6)
    np.testing.assert_allclose(h.dem["pos"][:, 2], z0 - s.g * s.dt ** 2 * 15, atol=5e-7)


def test_neighbour_digest_on_lattice():
    """On the unperturbed dx = 0.04 lattice, the fluid-fluid relation with
    support 0.104 (< 2.6 dx) counts the lattice points within 2.6 lattice
    spacings of an interior particle: 81 (self included)."""
    s, h = scene()
    count, _ = h.neighbour_digest("SPH_SPH_SUPPORT", s.support)
    lattice = np.array([(i, j, k) for i in range(-3, 4) for j in range(-3, 4) for k in range(-3, 4)])
    expected = int((np.linalg.norm(lattice, axis=1) * 0.04 < 0.104).sum())
    assert count.max() == expected == 81
    force, _ = h.neighbour_digest("SPH_SPH_FORCE", s.support)
    np.testing.assert_array_equal(force, count - 1)  # only the particle itself is excluded


def test_host_states_do_not_share_memory_with_cpu_tensors():
    """Two oracle states made from the same CPU structs are independent copies."""
    import torch

    from oracle.oracle import HostState
    from warp_sph_gpt_gb300.struct import SPHptl

    P = SPHptl(4, "cpu")
    P.pos.copy_(torch.arange(12, dtype=torch.float32).reshape(4, 3))
    a, b = HostState(P), HostState(P)
    a.sph["pos"][0, 0] = 99.0
    assert b.sph["pos"][0, 0] == 0.0 and float(P.pos[0, 0]) == 0.0
