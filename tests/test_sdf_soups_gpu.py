"""The SDF build on meshes that are not smooth closed surfaces: random triangle soups, the same far from
the origin, slivers, duplicated and coplanar overlapping triangles (ties of the atomicMin), tiny
triangles, a fine grid over a dense mesh, soups large enough that the construct's warps take chunks
of several triangles (each lane making one triangle's job), and Construct alone on words already near
its result -- each grid bit for bit against the oracle."""
import numpy as np
import pytest

import oracle


def _grid(lo, cell, dims):
    from tressfx_gb300 import _capi as A
    g = A.SdfGrid()
    for k in range(3):
        g.origin[k] = float(lo[k])
    g.cell_size = float(cell)
    g.num_cells_x, g.num_cells_y, g.num_cells_z = dims
    return g


def _soup(kind, rng):
    n = 600
    if kind in ("random", "far"):
        a = rng.uniform(-0.1, 0.1, (n, 3))
        tri = a[:, None, :] + rng.normal(0, 0.02, (n, 3, 3))
        if kind == "far":
            tri += np.array([50.0, -30.0, 20.0])
    elif kind == "sliver":
        a = rng.uniform(-0.1, 0.1, (n, 3))
        d = rng.normal(0, 0.03, (n, 3))
        t = rng.uniform(0, 1, n)
        third = a + t[:, None] * d + rng.normal(0, 1e-7, (n, 3))   # almost on the first edge
        tri = np.stack([a, a + d, third], 1)
    elif kind == "ties":
        a = rng.uniform(-0.1, 0.1, (n // 3, 3))
        base = a[:, None, :] + rng.normal(0, 0.02, (n // 3, 3, 3))
        shifted = base.copy()
        shifted[:, 2] = base[:, 0] + 0.5 * (base[:, 2] - base[:, 0])   # coplanar, overlapping
        tri = np.concatenate([base, base, shifted])                     # exact duplicates too
    elif kind == "tiny":
        a = rng.uniform(-0.1, 0.1, (n, 3))
        tri = a[:, None, :] + rng.normal(0, 1e-4, (n, 3, 3))
    else:
        raise ValueError(kind)
    tri = tri.astype(np.float32)
    verts = np.zeros((3 * len(tri), 8), np.float32)
    verts[:, :3] = tri.reshape(-1, 3)
    return verts, np.arange(3 * len(tri), dtype=np.uint32).reshape(-1, 3)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["random", "far", "sliver", "ties", "tiny"])
def test_construct_on_triangle_soups(ctx, kind):
    torch = pytest.importorskip("torch")
    from tressfx_gb300.api import SDFCollision
    rng = np.random.default_rng({"random": 1, "far": 2, "sliver": 3, "ties": 4, "tiny": 5}[kind])
    verts, idx = _soup(kind, rng)
    p = verts[:, :3]
    lo = p.min(0) - 0.02
    cell = np.float32((p.max(0) - p.min(0)).max() / 40.0)
    dims = tuple(int(x) for x in np.ceil((p.max(0) + 0.02 - lo) / cell) + 1)
    g = _grid(lo, cell, dims)
    cells = dims[0] * dims[1] * dims[2]
    dv = torch.from_numpy(verts.reshape(-1)).cuda()
    di = torch.from_numpy(idx.view(np.int32).reshape(-1)).cuda()
    sdf = SDFCollision(ctx, cells)
    try:
        sdf.set_mesh_device(dv.data_ptr(), len(verts), di.data_ptr(), len(idx))
        torch.cuda.synchronize()
        sdf.update(g)
        got = sdf.read(cells)
        want = oracle.sdf_build(g, verts, idx.reshape(-1))
        assert np.array_equal(got, want), f"{int((got != want).sum())} of {cells} cells differ"
    finally:
        sdf.close()


@pytest.mark.gpu
def test_construct_fine_grid_dense_mesh(ctx):
    torch = pytest.importorskip("torch")
    from tressfx_gb300.api import SDFCollision
    from tressfx_gb300.synthetic import head_mesh
    m = head_mesh(30000)
    verts = np.ascontiguousarray(m.vertices, np.float32).reshape(-1, 8)
    idx = np.ascontiguousarray(m.indices, np.uint32).reshape(-1, 3)
    p = verts[:, :3]
    lo = p.min(0) - 0.01
    cell = np.float32((p.max(0) - p.min(0)).max() / 110.0)
    dims = tuple(int(x) for x in np.ceil((p.max(0) + 0.01 - lo) / cell) + 1)
    g = _grid(lo, cell, dims)
    cells = dims[0] * dims[1] * dims[2]
    dv = torch.from_numpy(verts.reshape(-1)).cuda()
    di = torch.from_numpy(idx.view(np.int32).reshape(-1)).cuda()
    sdf = SDFCollision(ctx, cells)
    try:
        sdf.set_mesh_device(dv.data_ptr(), len(verts), di.data_ptr(), len(idx))
        torch.cuda.synchronize()
        sdf.update(g)
        assert np.array_equal(sdf.read(cells), oracle.sdf_build(g, verts, idx.reshape(-1)))
    finally:
        sdf.close()


@pytest.mark.gpu
@pytest.mark.parametrize("ntri", [70000, 480000])
def test_construct_large_soup_in_chunks(ctx, ntri):
    """A launch over this many triangles hands each warp chunks of several consecutive triangles (on
    152 SMs: 4 a chunk at 70,000, 32 at 480,000); the soup mixes small triangles, exact duplicates,
    coplanar overlaps and slivers, and its triangle count is not a multiple of the chunk."""
    torch = pytest.importorskip("torch")
    from tressfx_gb300.api import SDFCollision
    rng = np.random.default_rng(ntri)
    total = ntri - 3
    ns, nd = total // 2, total // 8
    a = rng.uniform(-0.1, 0.1, (ns, 3))
    small = a[:, None, :] + rng.normal(0, 0.002, (ns, 3, 3))
    dup = small[rng.integers(0, ns, nd)]                               # exact duplicates
    cop = dup.copy()
    cop[:, 2] = dup[:, 0] + 0.5 * (dup[:, 2] - dup[:, 0])              # coplanar, overlapping
    b = rng.uniform(-0.1, 0.1, (total - ns - 2 * nd, 3))
    d = rng.normal(0, 0.003, b.shape)
    sliver = np.stack([b, b + d, b + rng.uniform(0, 1, (len(b), 1)) * d + rng.normal(0, 1e-7, b.shape)], 1)
    tri = np.concatenate([small, dup, sliver, cop]).astype(np.float32)
    assert len(tri) == total
    verts = np.zeros((3 * len(tri), 8), np.float32)
    verts[:, :3] = tri.reshape(-1, 3)
    idx = np.arange(3 * len(tri), dtype=np.uint32).reshape(-1, 3)
    p = verts[:, :3]
    lo = p.min(0) - 0.01
    cell = np.float32((p.max(0) - p.min(0)).max() / 96.0)
    dims = tuple(int(x) for x in np.ceil((p.max(0) + 0.01 - lo) / cell) + 1)
    g = _grid(lo, cell, dims)
    cells = dims[0] * dims[1] * dims[2]
    dv = torch.from_numpy(verts.reshape(-1)).cuda()
    di = torch.from_numpy(idx.view(np.int32).reshape(-1)).cuda()
    sdf = SDFCollision(ctx, cells)
    try:
        sdf.set_mesh_device(dv.data_ptr(), len(verts), di.data_ptr(), len(idx))
        torch.cuda.synchronize()
        sdf.update(g)
        got = sdf.read(cells)
        want = oracle.sdf_build(g, verts, idx.reshape(-1))
        assert np.array_equal(got, want), f"{int((got != want).sum())} of {cells} cells differ"
    finally:
        sdf.close()


def _flip(f32: np.ndarray) -> np.ndarray:
    u = f32.view(np.uint32)
    return ((u << np.uint32(1)) | (u >> np.uint32(31))).astype(np.uint32)


def _unflip(w: np.ndarray) -> np.ndarray:
    return ((w >> np.uint32(1)) | (w << np.uint32(31))).astype(np.uint32)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["random", "ties", "tiny", "far"])
def test_construct_from_words_near_its_result(ctx, kind):
    """Construct alone on words that already sit within a few ulps of the result, with either sign:
    every pair's word lies close to a cell's current word, the case in which skipping pairs that
    cannot lower a word is hardest to get right.  The grid must still be the reference's
    atomicMin of every pair into those words."""
    torch = pytest.importorskip("torch")
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.api import SDFCollision
    rng = np.random.default_rng({"random": 11, "ties": 12, "tiny": 13, "far": 14}[kind])
    verts, idx = _soup(kind, rng)
    p = verts[:, :3]
    lo = p.min(0) - 0.02
    cell = np.float32((p.max(0) - p.min(0)).max() / 40.0)
    dims = tuple(int(x) for x in np.ceil((p.max(0) + 0.02 - lo) / cell) + 1)
    g = _grid(lo, cell, dims)
    cells = dims[0] * dims[1] * dims[2]
    result = _flip(np.full(cells, 1e10, np.float32))
    oracle.sdf_construct(g, result, verts, idx.reshape(-1))
    mag = _unflip(result) & np.uint32(0x7FFFFFFF)
    step = rng.integers(-3, 4, cells)
    mag = np.clip(mag.astype(np.int64) + step, 0, 0x7F7FFFFF).astype(np.uint32)
    sign = rng.integers(0, 2, cells).astype(np.uint32) << np.uint32(31)
    start = _flip((mag | sign).view(np.float32))
    want = start.copy()
    oracle.sdf_construct(g, want, verts, idx.reshape(-1))
    assert int((want != start).sum()) > 0
    dv = torch.from_numpy(verts.reshape(-1)).cuda()
    di = torch.from_numpy(idx.view(np.int32).reshape(-1)).cuda()
    sdf = SDFCollision(ctx, cells)
    try:
        sdf.set_mesh_device(dv.data_ptr(), len(verts), di.data_ptr(), len(idx))
        sdf.write(start)
        torch.cuda.synchronize()
        sdf.dispatch(A.K_SDF_CONSTRUCT, g)
        got = sdf.read(cells)
        assert np.array_equal(got, want), f"{int((got != want).sum())} of {cells} cells differ"
    finally:
        sdf.close()
