"""Oracle of the reference's frame files (test infrastructure only).

A plain-Python restatement of the reference writer's text output
(output/output.py:16-25 _fmt_float / _fmt_int, :113-176 _save_vtp,
:179-207 save_pvd; point-data sets of gather_state :28-62 and save_dem_vtk
:85-110), used by the tests to check the native formatter and the
asynchronous writer byte for byte.  It takes host numpy arrays, so it runs
without Warp.
"""
from __future__ import annotations

import numpy as np

SPH_TYPE, BND_TYPE, DEM_TYPE, DEM_BND_TYPE = 1, 0, 2, 3


def fmt_float(a, per_line: int = 6) -> str:
    v = ["%.6g" % x for x in np.asarray(a, dtype=np.float64).ravel()]
    return "\n".join(" ".join(v[i:i + per_line]) for i in range(0, len(v), per_line))


def fmt_int(a, per_line: int = 20) -> str:
    v = ["%d" % x for x in np.asarray(a).ravel()]
    return "\n".join(" ".join(v[i:i + per_line]) for i in range(0, len(v), per_line))


def sph_dataset(sph: dict, bnd: dict) -> dict:
    """gather_state: fluid then dummy boundary, placeholders on the boundary."""
    n_sph, n_bnd = len(sph["pos"]), len(bnd["pos"])
    return {
        "pos": np.vstack([sph["pos"], bnd["pos"]]),
        "vel": np.vstack([sph["vel"], bnd["vel"]]),
        "rho": np.concatenate([sph["rho"], bnd["rho"]]),
        "pres": np.concatenate([sph["pres"], bnd["pres"]]),
        "m": np.concatenate([sph["m"], bnd["m"]]),
        "porosity": np.concatenate([sph["porosity"], np.ones(n_bnd)]),
        "pgf": np.vstack([sph["pgf"], np.zeros((n_bnd, 3))]),
        "acc_dem": np.vstack([sph["acc_dem"], np.zeros((n_bnd, 3))]),
        "type": np.concatenate([np.full(n_sph, SPH_TYPE, dtype=np.int32), np.full(n_bnd, BND_TYPE, dtype=np.int32)]),
    }


def dem_dataset(dem: dict, wall: dict) -> dict:
    """save_dem_vtk: moving spheres then fixed wall spheres."""
    n_dem, n_bnd = len(dem["pos"]), len(wall["pos"])
    d = {}
    for key in ("pos", "vel", "omega", "radius", "rho", "m", "volume", "inertia"):
        d[key] = np.concatenate([dem[key], wall[key]])
    for key in ("acc", "force", "torque"):
        d[key] = np.vstack([dem[key], np.zeros((n_bnd, 3))])
    d["type"] = np.concatenate([np.full(n_dem, DEM_TYPE, dtype=np.int32), np.full(n_bnd, DEM_BND_TYPE, dtype=np.int32)])
    for key in ("drag", "pressure_force"):
        d[key] = np.vstack([dem[key], np.zeros((n_bnd, 3))])
    d["porosity"] = np.concatenate([dem["porosity"], np.ones(n_bnd)])
    return d


def vtp_text(d: dict, scalar: str) -> str:
    n = d["pos"].shape[0]
    out = ['<?xml version="1.0"?>\n', '<VTKFile type="PolyData" version="0.1" byte_order="LittleEndian">\n',
           '  <PolyData>\n',
           f'    <Piece NumberOfPoints="{n}" NumberOfVerts="{n}" '
           'NumberOfLines="0" NumberOfStrips="0" NumberOfPolys="0">\n',
           '      <Points>\n',
           '        <DataArray type="Float32" Name="Points" NumberOfComponents="3" format="ascii">\n',
           fmt_float(d["pos"]) + "\n", '        </DataArray>\n', '      </Points>\n', '      <Verts>\n',
           '        <DataArray type="Int32" Name="connectivity" format="ascii">\n', fmt_int(np.arange(n)) + "\n",
           '        </DataArray>\n', '        <DataArray type="Int32" Name="offsets" format="ascii">\n',
           fmt_int(np.arange(1, n + 1)) + "\n", '        </DataArray>\n', '      </Verts>\n',
           f'      <PointData Scalars="{scalar}" Vectors="vel">\n']
    for key, values in d.items():
        if key == "pos":
            continue
        dtype = "Int32" if key == "type" else "Float32"
        components = ' NumberOfComponents="3"' if values.ndim == 2 else ""
        out.append(f'        <DataArray type="{dtype}" Name="{key}"{components} format="ascii">\n')
        out.append((fmt_int(values) if key == "type" else fmt_float(values)) + "\n")
        out.append('        </DataArray>\n')
    out += ['      </PointData>\n', '    </Piece>\n', '  </PolyData>\n', '</VTKFile>\n']
    return "".join(out)


def pvd_text(frames) -> str:
    out = ['<?xml version="1.0"?>\n', '<VTKFile type="Collection" version="0.1" byte_order="LittleEndian">\n',
           '  <Collection>\n']
    for fname, t in frames:
        out.append(f'    <DataSet timestep="{t:.9g}" group="" part="0" file="{fname}"/>\n')
    out += ['  </Collection>\n', '</VTKFile>\n']
    return "".join(out)
