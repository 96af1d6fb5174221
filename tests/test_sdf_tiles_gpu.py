"""The batched SDF build, in both forms (TFX_BATCH_SDF_FORM 1: triangles binned into 8x8x4-cell tiles
with exact pair culling; 0: one warp per triangle), bit for bit against the oracle's
Initialize + Construct + Finalize on meshes chosen to break a culled construct: random soups, the
same far from the origin, slivers, exact duplicates and coplanar overlaps (ties), tiny triangles,
degenerate triangles (a point, a segment), triangles outside the grid (their boxes clamp to its
border), huge triangles next to small ones (the per-SDF big list), a fine grid over a dense mesh, and
several SDFs of different sizes (none a multiple of 8 cells) in one batch."""
import ctypes as C

import numpy as np
import pytest

import oracle
from tressfx_gb300 import _capi as A
from tressfx_gb300.api import Batch, CollisionMesh, HairObject, SDFCollision, default_settings
from tressfx_gb300.synthetic import build_asset, grow_strands, head_mesh, sample_on_ellipsoid

pytestmark = pytest.mark.gpu


def _grid(lo, cell, dims):
    g = A.SdfGrid()
    for k in range(3):
        g.origin[k] = float(lo[k])
    g.cell_size = float(cell)
    g.num_cells_x, g.num_cells_y, g.num_cells_z = (int(d) for d in dims)
    return g


def _soup(kind, rng, n=600):
    if kind in ("random", "far"):
        a = rng.uniform(-0.1, 0.1, (n, 3))
        tri = a[:, None, :] + rng.normal(0, 0.02, (n, 3, 3))
        if kind == "far":
            tri += np.array([50.0, -30.0, 20.0])
    elif kind == "sliver":
        a = rng.uniform(-0.1, 0.1, (n, 3))
        d = rng.normal(0, 0.03, (n, 3))
        t = rng.uniform(0, 1, n)
        tri = np.stack([a, a + d, a + t[:, None] * d + rng.normal(0, 1e-7, (n, 3))], 1)
    elif kind == "ties":
        a = rng.uniform(-0.1, 0.1, (n // 3, 3))
        base = a[:, None, :] + rng.normal(0, 0.02, (n // 3, 3, 3))
        shifted = base.copy()
        shifted[:, 2] = base[:, 0] + 0.5 * (base[:, 2] - base[:, 0])
        tri = np.concatenate([base, base, shifted])
    elif kind == "tiny":
        a = rng.uniform(-0.1, 0.1, (n, 3))
        tri = a[:, None, :] + rng.normal(0, 1e-4, (n, 3, 3))
    elif kind == "degenerate":
        a = rng.uniform(-0.1, 0.1, (n, 3))
        d = rng.normal(0, 0.03, (n, 3))
        point = np.stack([a, a, a], 1)[: n // 3]
        segment = np.stack([a, a + d, a + 0.5 * d], 1)[n // 3: 2 * n // 3]      # collinear
        normal = a[2 * n // 3:, None, :] + rng.normal(0, 0.02, (n - 2 * n // 3, 3, 3))
        tri = np.concatenate([point, segment, normal])
    elif kind == "huge":
        a = rng.uniform(-0.1, 0.1, (n, 3))
        tri = a[:, None, :] + rng.normal(0, 0.01, (n, 3, 3))
        big = rng.uniform(-0.12, 0.12, (12, 3, 3))                             # boxes over most of the grid
        tri = np.concatenate([tri, big])
    else:
        raise ValueError(kind)
    tri = tri.astype(np.float32)
    verts = np.zeros((3 * len(tri), 8), np.float32)
    verts[:, :3] = tri.reshape(-1, 3)
    verts[:, 3] = 1.0
    return verts, np.arange(3 * len(tri), dtype=np.uint32)


def _grid_around(verts, cells_x, pad=0.02):
    p = verts[:, :3]
    lo = p.min(0) - pad
    cell = np.float32((p.max(0) - p.min(0)).max() / cells_x)
    dims = tuple(int(x) for x in np.ceil((p.max(0) + pad - lo) / cell) + 1)
    return _grid(lo, cell, dims)


def _tiny_hair_asset(rng):
    roots, normals = sample_on_ellipsoid((0.0, 0.0, 0.0), (0.05, 0.05, 0.05), 64, rng)
    return build_asset(grow_strands(roots, normals, 8, 0.004, 10.0, rng))


def _batched_grids(ctx, meshes, grids, form):
    """One batch with one SDF per mesh (static skinning) and a small hair object on each; one frame;
    returns each SDF's grid as uint32 (the floats' bits)."""
    rng = np.random.default_rng(0)
    batch = Batch(ctx)
    keep = []
    try:
        for verts, idx in meshes:
            skin = np.zeros((len(verts), 8), np.float32)
            skin[:, 4] = 1.0
            m = CollisionMesh(ctx, verts, idx, skin)
            g = grids[len(keep)]
            s = SDFCollision(ctx, g.num_cells_x * g.num_cells_y * g.num_cells_z)
            h = HairObject(ctx, _tiny_hair_asset(rng))
            si = batch.add_sdf(s, m, (g.num_cells_x, g.num_cells_y, g.num_cells_z))
            batch.add_hair(h, si)
            keep.append((m, s, h))
        batch.build()
        batch.set_option(batch.SDF_FORM, form)
        assert batch.get_option(batch.SDF_FORM) == form
        eye = np.eye(4, dtype=np.float32).reshape(1, 16)
        for i, ((m, s, h), g) in enumerate(zip(keep, grids)):
            h.update_simulation_parameters(default_settings(), 1 / 60)
            h.update_bone_matrices(eye)
            batch.set_hair_constants(i, h.current_params(), h.num_bones, h.cpu_local_iterations)
            batch.set_sdf_frame(i, g, 0.5 * g.cell_size)
            batch.set_mesh_bones(i, np.tile(eye, (3, 1)))
        batch.run()
        batch.synchronize()
        # the grids, and the skinned vertices they were built from (the oracle's input)
        return [(s.read(g.num_cells_x * g.num_cells_y * g.num_cells_z).view(np.uint32), m.read_skinned().reshape(-1, 8))
                for (m, s, h), g in zip(keep, grids)]
    finally:
        batch.close()
        for m, s, h in keep:
            h.close()
            s.close()
            m.close()


def _want(g, verts, idx):
    return oracle.sdf_build(g, verts, idx)   # Initialize + Construct + Finalize: the floats' bits


def _check(got, want, what):
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, f"{what}: {len(bad)} of {len(want)} cells differ (first {bad[:5].tolist()})"


@pytest.mark.parametrize("form", [1, 0])
@pytest.mark.parametrize("kind", ["random", "far", "sliver", "ties", "tiny", "degenerate", "huge"])
def test_batched_construct_on_soups(ctx, kind, form):
    rng = np.random.default_rng({"random": 1, "far": 2, "sliver": 3, "ties": 4, "tiny": 5, "degenerate": 6,
                                 "huge": 7}[kind])
    verts, idx = _soup(kind, rng)
    g = _grid_around(verts, 37)
    got, skinned = _batched_grids(ctx, [(verts, idx)], [g], form)[0]
    want = _want(g, skinned, idx)
    _check(got, want, f"{kind}, form {form}")
    assert (want.view(np.float32) < 1e10).sum() > 500


def test_batched_construct_triangles_outside_the_grid(ctx):
    """Boxes of triangles beyond the grid clamp to its border cells (the reference's clamp)."""
    rng = np.random.default_rng(8)
    verts, idx = _soup("random", rng, 300)
    g = _grid_around(verts, 30)
    out = verts.copy()
    out[:, 0] += 0.5                                       # every triangle beyond +x
    out2 = verts.copy()
    out2[:, 1] -= 0.5                                      # and beyond -y
    allv = np.concatenate([verts, out, out2])
    alli = np.arange(3 * (len(allv) // 3), dtype=np.uint32)
    for form in (1, 0):
        got, skinned = _batched_grids(ctx, [(allv, alli)], [g], form)[0]
        _check(got, _want(g, skinned, alli), f"outside, form {form}")


def test_batched_construct_fine_grid_dense_mesh(ctx):
    m = head_mesh(30000)
    verts = np.ascontiguousarray(m.vertices, np.float32).reshape(-1, 8)
    idx = np.ascontiguousarray(m.indices, np.uint32).reshape(-1)
    g = _grid_around(verts, 110, pad=0.01)
    got, skinned = _batched_grids(ctx, [(verts, idx)], [g], 1)[0]
    _check(got, _want(g, skinned, idx), "dense head, 110 cells")


def test_batched_construct_several_sdfs(ctx):
    rng = np.random.default_rng(9)
    meshes, grids = [], []
    for k, (kind, cells) in enumerate([("random", 21), ("tiny", 45), ("ties", 33), ("huge", 18)]):
        verts, idx = _soup(kind, rng, 400)
        verts[:, :3] += np.float32(k)                      # apart from each other
        meshes.append((verts, idx))
        grids.append(_grid_around(verts, cells))
    got = _batched_grids(ctx, meshes, grids, 1)
    for k, ((verts, idx), g) in enumerate(zip(meshes, grids)):
        _check(got[k][0], _want(g, got[k][1], idx), f"SDF {k}")
