"""tfx_sdf_build_static, the SDF build for callers that may not allocate device memory once they run
(an engine with a GPU memory budget fixed at start-up, or a frame recorded for replay): its scratch is
a static device array, so the call allocates nothing.

Checked through the C ABI against tfx_sdf_update (the entry point with an allocated grid) and against
the oracle, bit for bit, on two calls in a row with different poses and grids.  The grid's cell count
is not a multiple of four, so the finalize's scalar tail runs.  Free device memory is the same before
and after further calls.

Named to be collected last, so it also runs after every other GPU test in one process."""
import ctypes as C

import numpy as np
import pytest

import oracle
from tressfx_gb300 import _capi as A
from tressfx_gb300.api import CollisionMesh, SDFCollision, grid_from_bbox
from tressfx_gb300.synthetic import head_mesh, pose_bones

pytestmark = pytest.mark.gpu

STATIC_MAX_CELLS = 2097152   # TFX_SDF_STATIC_MAX_CELLS


def _grids():
    m = head_mesh(6000)
    p = m.vertices[:, :3]
    c = (p.min(0) + p.max(0)) / 2
    r = float(np.linalg.norm(p - c, axis=1).max())
    g0, _, _ = grid_from_bbox(c - r, c + r, 34)
    g0.num_cells_x, g0.num_cells_y, g0.num_cells_z = 37, 41, 39   # 59,163 cells: 3 past a multiple of 4
    for k in range(3):                                             # the mesh's box, two cells of margin
        g0.origin[k] = float(np.float32(c[k] - r) - np.float32(2.0) * np.float32(g0.cell_size))
    g1 = A.SdfGrid()
    C.memmove(C.byref(g1), C.byref(g0), C.sizeof(A.SdfGrid))
    g1.origin[0] = g0.origin[0] + 3.0 * g0.cell_size   # the grid follows the moved mesh
    g1.origin[1] = g0.origin[1] - 2.0 * g0.cell_size
    return m, c, g0, g1


def _static_build(ctx, mesh, g, out_ptr):
    st = A.lib().tfx_sdf_build_static(ctx.handle, C.byref(g), C.c_void_p(mesh.skinned_ptr), mesh.num_vertices,
                                      C.c_void_p(mesh.index_ptr), mesh.num_triangles, out_ptr)
    assert st == 0, A.lib().tfx_last_error()


def test_static_build_matches_allocating_build_and_oracle_twice(ctx):
    m, pivot, g0, g1 = _grids()
    cells = g0.num_cells_x * g0.num_cells_y * g0.num_cells_z
    assert cells % 4 != 0 and cells <= STATIC_MAX_CELLS
    mesh = CollisionMesh(ctx, m.vertices, m.indices, m.skinning)
    ref = SDFCollision(ctx, cells)
    ref.bind_mesh(mesh)
    out = SDFCollision(ctx, cells)        # only its device buffer is used, as the caller's output
    out_ptr = C.c_void_p()
    assert A.lib().tfx_sdf_get_buffer(out.handle, C.byref(out_ptr), None) == 0

    poses = [((0.0, 0.0, 0.0), g0), ((0.2, -0.35, 0.5), g1)]
    for call, (angles, g) in enumerate(poses):
        mesh.skin(pose_bones(pivot, angles))
        _static_build(ctx, mesh, g, out_ptr)
        ref.update(g)
        got = out.read(cells)
        want = ref.read(cells)
        assert np.array_equal(got, want), f"call {call}: {int((got != want).sum())} cells differ from tfx_sdf_update"
        skinned = mesh.read_skinned().reshape(-1, 8)
        floats = oracle.sdf_build(g, skinned, m.indices)   # Initialize + Construct + Finalize: the floats' bits
        assert np.array_equal(got.view(np.uint32), floats), \
            f"call {call}: {int((got.view(np.uint32) != floats).sum())} cells differ from the oracle"
        assert (want.view(np.float32) < 1e10).sum() > 1000, "the mesh must reach into the grid"
    mesh.close()
    ref.close()
    out.close()


def test_static_build_allocates_nothing(ctx):
    torch = pytest.importorskip("torch")
    m, pivot, g0, _ = _grids()
    cells = g0.num_cells_x * g0.num_cells_y * g0.num_cells_z
    mesh = CollisionMesh(ctx, m.vertices, m.indices, m.skinning)
    out = SDFCollision(ctx, cells)
    out_ptr = C.c_void_p()
    assert A.lib().tfx_sdf_get_buffer(out.handle, C.byref(out_ptr), None) == 0
    mesh.skin(pose_bones(pivot, (0.1, 0.2, -0.3)))
    _static_build(ctx, mesh, g0, out_ptr)   # loads the kernels' module if it is not loaded yet
    ctx.synchronize()
    first = out.read(cells)
    torch.cuda.mem_get_info(ctx.device)
    free_before, _ = torch.cuda.mem_get_info(ctx.device)
    for _ in range(3):
        _static_build(ctx, mesh, g0, out_ptr)
    ctx.synchronize()
    free_after, _ = torch.cuda.mem_get_info(ctx.device)
    assert free_after == free_before, f"free device memory moved by {free_before - free_after} bytes"
    assert np.array_equal(out.read(cells), first)
    mesh.close()
    out.close()


def test_static_build_rejects_grids_beyond_its_scratch(ctx):
    _, _, g0, _ = _grids()
    g = A.SdfGrid()
    C.memmove(C.byref(g), C.byref(g0), C.sizeof(A.SdfGrid))
    g.num_cells_x, g.num_cells_y, g.num_cells_z = 129, 128, 128
    dummy = C.c_void_p(256)   # never dereferenced: the size check comes first
    st = A.lib().tfx_sdf_build_static(ctx.handle, C.byref(g), dummy, 3, dummy, 1, dummy)
    assert st == 8  # TFX_ERR_SIZE
    assert b"exceeds the static scratch" in A.lib().tfx_last_error()
