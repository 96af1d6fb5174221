"""SDF marching cubes (TressFXSDFMarchingCubes / RunMarchingCubesOnSdf, TressFXMarchingCubes.hlsl:147-280).

Pins, on the CPU:
  * the oracle's extraction with the reference's own tables is bit-identical to the reference's shader
    compiled as C++ (where the reference tree is present);
  * the library's tables equal the oracle's independently written generator, use every crossing edge,
    and give a closed, consistently wound surface across cubes;
  * the oracle with the library's tables puts the same vertices in every cube as the reference's shader
    did on the committed golden grids (the triangulations differ, the iso-vertices do not).
On the GPU, through the C ABI: the CUDA extraction equals the oracle bit for bit (positions, normals,
counter, zeroed tail), with the default tables, with caller tables, and when the buffer overflows.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import mc_cases
import oracle
from oracle import hlsl_ref
from oracle.mc_tables import EDGES, tables

GOLDEN = Path(__file__).resolve().parent / "golden" / "mc_reference.npz"
CASES = ("sphere_plane", "noise", "noise_overflow", "head")


def same(a: np.ndarray, b: np.ndarray) -> bool:
    """Bit-identical, except that any NaN equals any NaN: a degenerate triangle's normal is
    0 * (1 / sqrt(0)) = NaN, whose payload the hardware chooses (x86, Arm and the GPU differ)."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return a.shape == b.shape and np.array_equal(na, nb) and np.array_equal(a.view(np.uint32)[~na], b.view(np.uint32)[~nb])


def golden_case(name):
    z = np.load(GOLDEN)
    gv, dims = z[f"{name}/grid"], z[f"{name}/dims"]
    g = mc_cases.grid(gv[:3], float(gv[3]), dims)
    iso = np.float32(np.float32(g.cell_size) * z[f"{name}/iso_cells"])
    return (g, z[f"{name}/sdf"], float(z[f"{name}/iso_cells"]), iso, int(z[f"{name}/max_vertices"]),
            int(z[f"{name}/counter"]), z[f"{name}/positions"])


# ------------------------------------------------------------------------------------------- tables
def test_library_tables_equal_oracle_generator(built_lib):
    e = np.zeros(256, np.int32)
    t = np.zeros(4096, np.int32)
    assert built_lib.tfx_mc_default_tables(e.ctypes.data, t.ctypes.data) == 0
    e2, t2 = tables()
    assert np.array_equal(e, e2) and np.array_equal(t, t2)


def test_tables_use_every_crossing_edge():
    e, t = tables()
    t = t.reshape(256, 16)
    for cfg in range(256):
        used = t[cfg][t[cfg] >= 0]
        assert len(used) % 3 == 0 and len(used) <= 15
        crossing = {k for k, (a, b) in enumerate(EDGES) if ((cfg >> a) & 1) != ((cfg >> b) & 1)}
        assert set(used.tolist()) == crossing, cfg
        assert e[cfg] == sum(1 << k for k in crossing)
        for tri in used.reshape(-1, 3):
            assert len(set(tri.tolist())) == 3


def _grid_edge_id(x, y, z, e, dims):
    """Global id of cube (x, y, z)'s edge e: (lower corner, axis)."""
    from oracle.mc_tables import CORNERS
    a, b = EDGES[e]
    pa, pb = np.array(CORNERS[a]), np.array(CORNERS[b])
    lo = np.minimum(pa, pb) + (x, y, z)
    axis = int(np.argmax(np.abs(pb - pa)))
    X, Y, _ = dims
    return ((int(lo[2]) * (Y + 1) + int(lo[1])) * (X + 1) + int(lo[0])) * 3 + axis


def test_tables_give_closed_consistently_wound_surface():
    """On noise (every ambiguous face occurs) inside a +1 border, every mesh edge joins exactly two
    triangles, once in each direction."""
    e, t = tables()
    t = t.reshape(256, 16)
    rng = np.random.default_rng(11)
    X = Y = Z = 9
    s = rng.standard_normal((Z, Y, X)).astype(np.float32)
    s[0], s[-1], s[:, 0], s[:, -1], s[:, :, 0], s[:, :, -1] = 1, 1, 1, 1, 1, 1
    g = mc_cases.grid((0, 0, 0), 1.0, (X, Y, Z))
    cfg = mc_cases.configs(g, s, 0.0).reshape(Z, Y, X)
    directed = {}
    ambiguous = 0
    for z in range(Z - 1):
        for y in range(Y - 1):
            for x in range(X - 1):
                c = cfg[z, y, x]
                row = t[c][t[c] >= 0].reshape(-1, 3)
                ambiguous += len(row) >= 3
                for tri in row:
                    ids = [_grid_edge_id(x, y, z, int(k), (X, Y, Z)) for k in tri]
                    for i in range(3):
                        key = (ids[i], ids[(i + 1) % 3])
                        directed[key] = directed.get(key, 0) + 1
    assert ambiguous > 0 and directed
    for (a, b), n in directed.items():
        assert n == 1, (a, b, n)
        assert directed.get((b, a)) == 1, (a, b)


# ------------------------------------------------------------------------------------------- oracle pins
@pytest.mark.skipif(not hlsl_ref.available(), reason="needs the reference's shader sources")
@pytest.mark.parametrize("name", CASES)
def test_oracle_equals_reference_shader(name):
    g, sdf, _, iso, maxv, _, _ = golden_case(name)
    l = hlsl_ref.lib()
    edge, tri = np.zeros(256, np.int32), np.zeros(4096, np.int32)
    l.tfxr_mc_tables(edge.ctypes.data, tri.ctypes.data)
    sdf = np.ascontiguousarray(sdf, np.float32)
    for mv in (maxv, 700):
        buf = np.zeros((mv, 8), np.float32)
        cnt = np.zeros(1, np.int32)
        gp = oracle.sdf_params(g)
        l.tfxr_marching_cubes(sdf.view(np.uint32).ctypes.data, sdf.size, C.addressof(gp), float(iso), edge.ctypes.data,
                              tri.ctypes.data, mv, buf.ctypes.data, cnt.ctypes.data)
        out, c = oracle.marching_cubes(g, sdf, iso, edge, tri, mv)
        assert c == int(cnt[0])
        assert same(out, buf)


@pytest.mark.parametrize("name", CASES)
def test_oracle_cube_vertices_equal_reference_golden(name):
    g, sdf, _, iso, maxv, counter, positions = golden_case(name)
    e, t = tables()
    out, c = oracle.marching_cubes(g, sdf, iso, e, t, maxv)
    assert c == counter
    cfg = mc_cases.configs(g, sdf, iso)
    counts = mc_cases.vertex_counts(t, e)
    w = mc_cases.written_vertices(cfg, counts, maxv)
    assert w == len(positions) or (counter >= maxv and w <= len(positions))
    ref = mc_cases.cube_vertex_sets(cfg, counts, positions, w)
    ours = mc_cases.cube_vertex_sets(cfg, counts, out, w)
    assert np.array_equal(ref, ours)
    assert not out[w:].any()


# ------------------------------------------------------------------------------------------- CUDA
def _run_cuda(ctx, g, sdf, iso_cells, maxv, tables_=None):
    import torch
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.api import SDFMarchingCubes
    dev = torch.from_numpy(np.ascontiguousarray(sdf, np.float32).reshape(-1)).cuda()
    mc = SDFMarchingCubes(ctx, maxv, dev.numel())
    try:
        if tables_ is not None:
            mc.set_tables(*tables_)
        mc.set_iso_level(iso_cells)
        sg = A.SdfGrid()
        for k in range(3):
            sg.origin[k] = g.origin[k]
        sg.cell_size = g.cell_size
        sg.num_cells_x, sg.num_cells_y, sg.num_cells_z = g.num_cells_x, g.num_cells_y, g.num_cells_z
        torch.cuda.synchronize()
        mc.run(dev.data_ptr(), sg)
        return mc.read()
    finally:
        mc.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_cuda_equals_oracle_and_reference_golden(ctx, name):
    g, sdf, iso_cells, iso, maxv, counter, positions = golden_case(name)
    e, t = tables()
    got, c = _run_cuda(ctx, g, sdf, iso_cells, maxv)
    want, cw = oracle.marching_cubes(g, sdf, iso, e, t, maxv)
    assert c == cw == counter
    assert same(got, want)
    cfg = mc_cases.configs(g, sdf, iso)
    counts = mc_cases.vertex_counts(t, e)
    w = mc_cases.written_vertices(cfg, counts, maxv)
    assert np.array_equal(mc_cases.cube_vertex_sets(cfg, counts, positions, w),
                          mc_cases.cube_vertex_sets(cfg, counts, got, w))


def _scrambled_tables():
    """The default tables with every triangle's corners rotated, the triangle order reversed, and
    configurations 1..7 given a fourth (unterminated-triangle) entry: a count not divisible by 3."""
    e, t = tables()
    t = t.reshape(256, 16).copy()
    for cfg in range(256):
        row = t[cfg][t[cfg] >= 0].reshape(-1, 3)
        row = np.roll(row[::-1], 1, axis=1).reshape(-1)
        t[cfg, :] = -1
        t[cfg, :len(row)] = row
        if 1 <= cfg <= 7:
            t[cfg, len(row)] = row[0]
    return e, t


@pytest.mark.gpu
@pytest.mark.parametrize("maxv", [1 << 14, 3001, 0])
def test_cuda_caller_tables_and_overflow(ctx, maxv):
    g, sdf = mc_cases.noise((17, 9, 14), seed=8)
    e, t = _scrambled_tables()
    got, c = _run_cuda(ctx, g, sdf, 0.25, maxv, (e, t))
    want, cw = oracle.marching_cubes(g, sdf, np.float32(np.float32(g.cell_size) * np.float32(0.25)), e, t, maxv)
    assert c == cw
    assert same(got, want)


@pytest.mark.gpu
def test_cuda_bad_tables_rejected(ctx, built_lib):
    from tressfx_gb300._capi import TfxError
    from tressfx_gb300.api import SDFMarchingCubes
    mc = SDFMarchingCubes(ctx, 1024, 4096)
    try:
        e, t = tables()
        t = t.copy()
        t[40] = 12
        with pytest.raises(TfxError):
            mc.set_tables(e, t)
    finally:
        mc.close()


@pytest.mark.gpu
def test_cuda_update_from_sdf_object_and_shrinking_surface(ctx):
    """tfx_mc_update on a tfx_sdf built from a mesh; a second update on a smaller surface leaves the
    rest of the buffer zero, as InitializeMCVertices does."""
    import torch
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.api import SDFCollision, SDFMarchingCubes
    from tressfx_gb300.synthetic import head_mesh
    m = head_mesh(3000)
    v = m.vertices.reshape(-1, 8)[:, :3]
    lo, hi = v.min(0), v.max(0)
    cell = float(np.float32((hi[0] - lo[0]) / 40.0))
    pad = 3 * cell
    dims = tuple(int((hi[k] - lo[k] + 2 * pad) / cell) + 1 for k in range(3))
    g = mc_cases.grid(lo - pad, cell, dims)
    cells = dims[0] * dims[1] * dims[2]
    sg = A.SdfGrid()
    for k in range(3):
        sg.origin[k] = g.origin[k]
    sg.cell_size, sg.num_cells_x, sg.num_cells_y, sg.num_cells_z = g.cell_size, *dims
    verts = torch.from_numpy(np.ascontiguousarray(m.vertices, np.float32).reshape(-1)).cuda()
    idx = torch.from_numpy(np.ascontiguousarray(m.indices, np.uint32).view(np.int32).reshape(-1)).cuda()
    sdf = SDFCollision(ctx, cells)
    mc = SDFMarchingCubes(ctx, 1 << 17, cells)
    try:
        sdf.set_mesh_device(verts.data_ptr(), len(v), idx.data_ptr(), len(m.indices.reshape(-1)) // 3)
        sdf.update(sg)
        words = sdf.read(cells)
        assert np.array_equal(words, oracle.sdf_build(g, m.vertices, m.indices))
        e, t = tables()
        for iso_cells in (1.5, 0.0):
            mc.set_iso_level(iso_cells)
            mc.update(sdf, sg)
            got, c = mc.read()
            iso = np.float32(np.float32(cell) * np.float32(iso_cells))
            want, cw = oracle.marching_cubes(g, words.view(np.float32), iso, e, t, 1 << 17)
            assert c == cw and c > 1000
            assert same(got, want), iso_cells
    finally:
        mc.close()
        sdf.close()


@pytest.mark.gpu
def test_cuda_full_size_grid_128(ctx):
    """A 128^3 grid (the sample's largest SDF): bit-identical to the oracle."""
    g, sdf = mc_cases.sphere_plane((128, 128, 128), (-0.2, -0.1, 0.0), 0.01)
    e, t = tables()
    got, c = _run_cuda(ctx, g, sdf, 0.0, 1 << 18)
    want, cw = oracle.marching_cubes(g, sdf, np.float32(0.0), e, t, 1 << 18)
    assert c == cw and c > 10000
    assert same(got, want)
