"""Particle text format, initialisation and generators (no GPU).

Restates the reference's tests/test_input_reader.py:53-164 and
tests/test_3d.py:55-85, and pins the generator to the reference's own config-1
input files through tests/golden/input_files.json (SHA-256 of each file).
"""
import hashlib
import json
import tempfile
from dataclasses import fields
from pathlib import Path

import numpy as np
import pytest
import torch

from warp_sph_gpt_gb300 import BaseSolv, Solv, column_indices, input_parser, load_sph_particles
from warp_sph_gpt_gb300.generate import (CoupledGenerationConfig, DamPtlGeneration, DEMPtlGeneration, config_batch_member,
                                         config_large, config_scaled, config_small, generate_files, solver_config,
                                         write_particle_file)
from warp_sph_gpt_gb300.input_reader import INPUT_FIELDS, dem_search_scales, validate_dem_particles

GOLDEN = json.loads((Path(__file__).parent / "golden" / "input_files.json").read_text())


@pytest.fixture(scope="module")
def small_files():
    gen = CoupledGenerationConfig(device="cpu", dx=0.04, h=0.052, tank_width=0.8, tank_height=0.8, tank_depth=0.32,
                                  fluid_width=0.4, fluid_height=0.4, fluid_depth=0.32, dem_nx=2, dem_ny=1, dem_nz=1,
                                  dem_origin_y=0.16, dem_origin_z=0.2)
    with tempfile.TemporaryDirectory() as d:
        yield gen, generate_files(d, gen), Path(d)


def test_generator_writes_the_reference_input_files_byte_for_byte():
    """Config 1 (the reference's input_file/*) from the project's generator."""
    with tempfile.TemporaryDirectory() as d:
        for kind, path in generate_files(d, config_small()).items():
            data = path.read_bytes()
            assert hashlib.sha256(data).hexdigest() == GOLDEN[kind]["sha256"], kind
            assert len(data.decode().splitlines()) - 1 == GOLDEN[kind]["rows"]


def test_documented_column_ids_and_solver_only_config():
    """tests/test_input_reader.py:53-65."""
    assert column_indices("SPH") == {"pos": (1, 2, 3), "vel": (4, 5, 6), "rho": (7,), "m": (8,)}
    assert column_indices("DEM")["K"] == (14,)
    assert column_indices("DEM")["h"] == (17,)
    banned = {"dx", "bnd_layer", "dem_K", "dem_eta", "dem_mu", "dem_h", "dem_radius", "dem_mass", "tank_width"}
    for config in (BaseSolv, Solv):
        assert not banned.intersection(f.name for f in fields(config))
    for kind in INPUT_FIELDS:
        assert not {"pres", "acc", "volume", "flt", "porosity"}.intersection(column_indices(kind))
    with pytest.raises(ValueError):
        column_indices("NOPE")


def test_files_match_generated_structs(small_files):
    """tests/test_input_reader.py:67-83 (file round trip of every field)."""
    gen, paths, d = small_files
    generated = dict(zip(("SPH", "BND"), DamPtlGeneration(gen).build("cpu")))
    generated.update(zip(("DEM", "DEMBND"), DEMPtlGeneration(gen).build("cpu")))
    solv = solver_config(gen, device="cpu", input_dir=str(d))
    loaded = dict(zip(("SPH", "BND", "DEM", "DEMBND"), load_sph_particles(solv)))
    for kind, part in loaded.items():
        for name in part.field_names():
            np.testing.assert_allclose(getattr(part, name).numpy(), getattr(generated[kind], name).numpy(),
                                       rtol=2e-7, atol=0, err_msg=f"{kind}.{name}")


def test_reordered_columns_dispatch_by_id(small_files):
    """tests/test_input_reader.py:84-96."""
    gen, paths, _ = small_files
    for kind, source in paths.items():
        with tempfile.TemporaryDirectory() as d:
            lines = source.read_text().splitlines()
            path = Path(d) / source.name
            path.write_text(" ".join(reversed(lines[0].split())) + "\n" + " ".join(reversed(lines[1].split())) + "\n")
            got, want = input_parser(path), input_parser(source)
            for name, _ in INPUT_FIELDS[kind]:
                np.testing.assert_array_equal(getattr(got, name).numpy()[0], getattr(want, name).numpy()[0])


@pytest.mark.parametrize("text", [
    "", "1 1 2 3 4 5 6 7\n0 0 0 0 0 0 1000 0.001\n", "1 2 3 4 5 6 7 99\n0 0 0 0 0 0 1000 0.001\n",
    "1.0 2 3 4 5 6 7 8\n0 0 0 0 0 0 1000 0.001\n", "1 2 3 4 5 6 7 8\n0 0\n", "1 2 3 4 5 6 7 8\n\n",
    "1 2 3 4 5 6 7 8\n0 0 0 0 0 0 nan 0.001\n", "1 2 3 4 5 6 7 8\n0 0 0 0 0 0 inf 0.001\n",
    "1 2 3 4 5 6 7 8\n0 0 0 0 0 0 1e100 0.001\n", "1 2 3 4 5 6 7 8\n0 0 0 0 0 0 -1 0.001\n",
    "1 2 3 4 5 6 7 8\n0 0 0 0 0 0 1000 1e-100\n", "1 2 3 4 5 6 7 8\n0 0 0 0 0 0 oops 0.001\n"])
def test_invalid_input_is_rejected(text):
    """tests/test_input_reader.py:98-113."""
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "input_SPH.txt"
        path.write_text(text)
        with pytest.raises(ValueError):
            input_parser(path)


def test_error_reports_path_and_line():
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "input_SPH.txt"
        path.write_text("1 2 3 4 5 6 7 8\n0 0 0 0 0 0 1000 0.001\n0 0 0 0 0 0 oops 0.001\n")
        with pytest.raises(ValueError, match=r"input_SPH.txt:3: invalid numeric value"):
            input_parser(path)


def test_empty_boundary_and_zero_contact_buffers(small_files):
    """tests/test_input_reader.py:115-128."""
    gen, paths, _ = small_files
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "input_DEMBND.txt"
        path.write_text(" ".join(str(i) for i in range(1, 17)) + "\n")
        boundary = input_parser(path)
        assert boundary.pos.shape[0] == 0
        dem = input_parser(paths["DEM"])
        solv = solver_config(gen, device="cpu")
        assert validate_dem_particles(solv, dem, boundary)[1] == 0
        for kind in ("dem", "bnd"):
            for side in ("old", "new"):
                assert getattr(dem, f"contact_{kind}_id_{side}").numel() == 0
                np.testing.assert_array_equal(getattr(dem, f"contact_{kind}_offset_{side}").numpy(), 0)


def test_post_load_initialisation(small_files):
    """input/input_reader.py:113-133: rho_raw = rho, porosity = 1, volume."""
    _, paths, _ = small_files
    sph = input_parser(paths["SPH"])
    np.testing.assert_array_equal(sph.rho_raw.numpy(), sph.rho.numpy())
    np.testing.assert_array_equal(sph.porosity.numpy(), 1.0)
    dem = input_parser(paths["DEM"])
    np.testing.assert_allclose(dem.volume.numpy(), 4.0 / 3.0 * np.pi * dem.radius.numpy().astype(float) ** 3,
                               rtol=1e-6)
    np.testing.assert_array_equal(dem.porosity.numpy(), 1.0)


def test_loaded_materials_control_contact_dt_and_search_extents(small_files):
    """tests/test_input_reader.py:147-164."""
    gen, paths, d = small_files
    solv = solver_config(gen, device="cpu", input_dir=str(d))
    _, _, dem, boundary = load_sph_particles(solv)
    dem.h = torch.tensor([0.04, 0.12])
    dem.K = torch.tensor([2e4, 8e4])
    dem.eta = torch.tensor([4.0, 7.0])
    dem.mu = torch.tensor([0.1, 0.6])
    with tempfile.TemporaryDirectory() as d2:
        loaded = input_parser(write_particle_file(Path(d2) / "input_DEM.txt", "DEM", dem))
        for name in ("K", "eta", "mu", "h"):
            np.testing.assert_array_equal(getattr(loaded, name).numpy(), getattr(dem, name).numpy())
        scales = dem_search_scales(loaded, boundary)
        assert abs(scales[2] - 0.12) < 1e-7 and scales[3] == 0.0
        solv.dt = 0.5
        with pytest.raises(ValueError, match="loaded DEM contact limit"):
            validate_dem_particles(solv, loaded, boundary)


def test_volume_mass_and_five_wall_geometry():
    """tests/test_3d.py:55-85."""
    s = CoupledGenerationConfig(device="cpu")
    fluid = DamPtlGeneration(s).fluid_particle()
    sph_wall = DamPtlGeneration(s).boundary_particle()
    dem = DEMPtlGeneration(s).dem_particle()
    dem_wall = DEMPtlGeneration(s).boundary_particle()
    assert abs(len(fluid) * s.rho0 * s.dx ** 3 - 100.0) < 1e-9 and len(dem) == 20
    assert abs(np.ptp(fluid[:, 1]) + s.dx - s.fluid_depth) < 1e-9
    for wall in (sph_wall, dem_wall):
        assert len(wall) == len(np.unique(wall, axis=0))
        assert all(wall[:, a].min() < 0.0 for a in range(3))
        interior = (wall[:, 0] > 0) & (wall[:, 0] < s.tank_width) & (wall[:, 1] > 0) & (wall[:, 1] < s.tank_depth)
        assert np.all(wall[interior, 2] < 0.0)
    with pytest.raises(ValueError):
        DEMPtlGeneration(CoupledGenerationConfig(dem_origin_y=0.39)).dem_particle()
    with pytest.raises(ValueError):
        CoupledGenerationConfig(dt=1.0e-3).validate_dem()


def test_scaled_configuration_counts():
    """dx = 0.01: 100,000 fluid, 180,456 dummy, 160 jittered DEM, 57,368 wall spheres."""
    gen, pos, rad = config_scaled(seed=0)
    assert len(DamPtlGeneration(gen).fluid_particle()) == 100_000
    assert len(DamPtlGeneration(gen).boundary_particle()) == 180_456
    assert len(DEMPtlGeneration(gen).boundary_particle()) == 57_368
    base = DEMPtlGeneration(gen).dem_particle()
    assert pos.shape == (160, 3) and np.abs(pos - base).max() <= 0.005


def test_large_configuration_counts_and_non_overlap():
    """Tank 4 x 0.8 x 1.5 at dx = 0.005: 792,000 fluid in the 0.167 m variant,
    2,157,576 dummy, 2,000 non-overlapping DEM in the upper half, 178,528 wall spheres."""
    gen, pos, rad = config_large(fluid_width=0.167, seed=0, n_dem=2000)
    assert len(DamPtlGeneration(gen).fluid_particle()) == 792_000
    assert len(DamPtlGeneration(gen).boundary_particle()) == 2_157_576
    assert len(DEMPtlGeneration(gen).boundary_particle()) == 178_528
    assert pos.shape == (2000, 3) and rad.min() >= 0.01 and rad.max() <= 0.03
    assert (pos[:, 2] - rad).min() >= 0.75 and (pos[:, 2] + rad).max() <= 1.5
    from scipy.spatial import cKDTree
    pairs = cKDTree(pos).query_pairs(0.06, output_type="ndarray")
    d = np.linalg.norm(pos[pairs[:, 0]] - pos[pairs[:, 1]], axis=1)
    assert np.all(d >= rad[pairs[:, 0]] + rad[pairs[:, 1]])


def test_batch_member_ranges():
    """Config 4 members: fluid x-length in [0.3, 0.7], height in [0.3, 0.6],
    0..40 spheres of R = 0.025 above the water, none overlapping."""
    for i in range(8):
        gen, pos, rad = config_batch_member(i)
        assert 0.3 - 0.02 <= gen.fluid_width <= 0.7 + 0.02 and 0.3 - 0.02 <= gen.fluid_height <= 0.6 + 0.02
        assert 0 <= len(pos) <= 40
        if len(pos):
            assert (pos[:, 2] - 0.025).min() >= gen.fluid_height
