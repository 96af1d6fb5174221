"""Writes tests/golden/mc_reference.npz: the reference's RunMarchingCubesOnSdf (its own shader and
tables, compiled by oracle/hlsl_ref) on the grids of tests/mc_cases.py and on the SDF of a skinned
head mesh, with the inputs.

    python tests/golden/make_mc_golden.py
"""
import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parent.parent))

import mc_cases  # noqa: E402
import oracle  # noqa: E402
from oracle import hlsl_ref  # noqa: E402


def head_case():
    from tressfx_gb300.synthetic import head_mesh
    m = head_mesh(1500)
    v = m.vertices.reshape(-1, 8)[:, :3]
    lo, hi = v.min(0), v.max(0)
    cell = float(np.float32((hi[0] - lo[0]) / 20.0))
    pad = 3 * cell
    dims = tuple(int((hi[k] - lo[k] + 2 * pad) / cell) + 1 for k in range(3))
    g = mc_cases.grid(lo - pad, cell, dims)
    words = oracle.sdf_build(g, m.vertices, m.indices)
    return g, words.view(np.float32).reshape(dims[2], dims[1], dims[0])


def main() -> None:
    if not hlsl_ref.available():
        raise SystemExit("the reference tree is not available")
    l = hlsl_ref.lib()
    edge, tri = np.zeros(256, np.int32), np.zeros(4096, np.int32)
    l.tfxr_mc_tables(edge.ctypes.data, tri.ctypes.data)
    cases = {"sphere_plane": mc_cases.sphere_plane() + (0.0, 1 << 16),
             "noise": mc_cases.noise() + (0.1, 1 << 14),
             "noise_overflow": mc_cases.noise() + (0.1, 1500),
             "head": head_case() + (0.0, 1 << 16)}
    out = {}
    for name, (g, sdf, iso_cells, maxv) in cases.items():
        sdf = np.ascontiguousarray(sdf, np.float32)
        iso = np.float32(np.float32(g.cell_size) * np.float32(iso_cells))
        buf = np.zeros((maxv, 8), np.float32)
        cnt = np.zeros(1, np.int32)
        gp = oracle.sdf_params(g)
        l.tfxr_marching_cubes(sdf.view(np.uint32).ctypes.data, sdf.size, C.addressof(gp), float(iso), edge.ctypes.data,
                              tri.ctypes.data, maxv, buf.ctypes.data, cnt.ctypes.data)
        used = min(int(cnt[0]), maxv)
        out[f"{name}/sdf"] = sdf
        out[f"{name}/grid"] = np.array([*g.origin[:3], g.cell_size], np.float32)
        out[f"{name}/dims"] = np.array([g.num_cells_x, g.num_cells_y, g.num_cells_z], np.int32)
        out[f"{name}/iso_cells"] = np.float32(iso_cells)
        out[f"{name}/max_vertices"] = np.int32(maxv)
        out[f"{name}/counter"] = np.int32(cnt[0])
        out[f"{name}/positions"] = buf[:used, :3].copy()
        print(name, "counter", int(cnt[0]), "dims", g.num_cells_x, g.num_cells_y, g.num_cells_z)
    np.savez_compressed(HERE / "mc_reference.npz", **out)


if __name__ == "__main__":
    main()
