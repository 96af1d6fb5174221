"""Host-side logic of the C ABI (no device): the local-iteration split and reset frames of the
constant block (its every word, wind included, is pinned to the reference's own code by
test_consts_pin.py), the double-buffered blocks, SDF grid sizing, and argument validation."""
import ctypes as C
import math

import numpy as np
import pytest

from tressfx_gb300 import _capi as A
from tressfx_gb300.api import SimConstants, default_settings, fill_sim_params, grid_from_bbox


def f32(x):
    return np.float32(x)


@pytest.mark.parametrize("n,expect_gpu,expect_cpu", [(16, 1, 3), (32, 1, 3), (64, 3, 1)])
def test_local_iteration_split(built_lib, n, expect_gpu, expect_cpu):
    s = default_settings()
    s.local_constraints_iterations = 3
    p = A.SimParams()
    cpu = fill_sim_params(p, s, 1 / 60, n, 2, 5)
    assert (p.sim_ints[1], cpu) == (expect_gpu, expect_cpu)
    assert tuple(p.counts[:3]) == (64 // n, 2, n)
    assert p.clamp_position_delta == 20.0 and p.sim_ints[2] == 0
    assert p.reset_positions == 0.0


def test_reset_on_first_two_frames(built_lib):
    s = default_settings()
    for frame, want in [(0, 1.0), (1, 1.0), (2, 0.0)]:
        p = A.SimParams()
        fill_sim_params(p, s, 1 / 60, 16, 0, frame)
        assert p.reset_positions == want


def test_sim_constants_double_buffer(built_lib):
    """m_SimCB[frame % 2]: bone matrices and the reset flag live in the slot of the current frame."""
    sc = SimConstants(16, 0)
    assert sc.sim_cb[0].reset_positions == 1.0
    sc.update_bone_matrices(np.arange(16, dtype=np.float32))
    assert sc.sim_cb[0].bones_view()[0, 5] == 5.0 and sc.sim_cb[1].bones_view()[0, 5] == 0.0
    sc.increase_simulation_frame()
    assert sc.frame == 1 and sc.sim_cb[0].reset_positions == 0.0
    assert sc.current_params() is sc.sim_cb[1]


def test_sdf_grid_sizing_reference_rule(built_lib):
    bmin, bmax = (-0.1, 1.45, -0.12), (0.1, 1.75, 0.1)
    g, pad, alloc = grid_from_bbox(bmin, bmax, 50)
    cell = (f32(bmax[0]) - f32(bmin[0])) / f32(50)
    assert g.cell_size == cell
    extra = int(f32(0.8) * f32(50))
    assert extra == 40 and pad == np.float32(extra * cell)
    lo = np.float32(bmin) - np.float32(pad)
    hi = np.float32(bmax) + np.float32(pad)
    assert g.num_cells_x == int((hi[0] - lo[0]) / cell)
    assert g.num_cells_y == int((hi[1] - lo[1]) / cell)
    assert g.num_cells_z == int((hi[2] - lo[2]) / cell)
    assert tuple(np.float32(g.origin[:3])) == tuple(lo)
    assert alloc == int(f32(1.4) * g.num_cells_x * g.num_cells_y * g.num_cells_z)


def _desc(G=64, n=16, F=0):
    return A.HairDesc(G, n, F, 0)


def test_validate_rejects_bad_inputs(built_lib):
    lib = A.lib()
    skin = np.zeros((64, 8), dtype=np.float32)
    skin[:, 4] = 1.0
    assert lib.tfx_hair_validate(C.byref(_desc()), skin.ctypes.data) == A.TFX_OK
    for n in (2, 5, 12, 128):
        assert lib.tfx_hair_validate(C.byref(_desc(n=n)), skin.ctypes.data) == A.TFX_ERR_VERTS_PER_STRAND
    assert lib.tfx_hair_validate(C.byref(_desc(G=0)), skin.ctypes.data) == A.TFX_ERR_INVALID_ARGUMENT
    assert lib.tfx_hair_validate(C.byref(_desc(G=2**27, n=64)), skin.ctypes.data) == A.TFX_ERR_SIZE
    bad = skin.copy()
    bad[3, 0] = 512.0
    assert lib.tfx_hair_validate(C.byref(_desc()), bad.ctypes.data) == A.TFX_ERR_BONE_INDEX
    assert b"512" in lib.tfx_last_error()
    bad = skin.copy()
    bad[3, 4] = 0.0
    assert lib.tfx_hair_validate(C.byref(_desc()), bad.ctypes.data) == A.TFX_ERR_BONE_WEIGHTS
    # an unused slot (weight 0) may carry any index, as the shader never reads it
    ok = skin.copy()
    ok[:, 1] = 9999.0
    assert lib.tfx_hair_validate(C.byref(_desc()), ok.ctypes.data) == A.TFX_OK
    # only guide strands are read: with F = 1 the follow strands' skinning is ignored
    sk2 = np.zeros((128, 8), dtype=np.float32)
    sk2[0::2, 4] = 1.0
    assert lib.tfx_hair_validate(C.byref(_desc(F=1)), sk2.ctypes.data) == A.TFX_OK
    assert lib.tfx_hair_validate(None, skin.ctypes.data) == A.TFX_ERR_INVALID_ARGUMENT


def test_create_without_device_fails_cleanly(built_lib):
    """On a machine without a CUDA device, context creation reports TFX_ERR_NO_DEVICE (no crash)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = C.c_void_p()
    assert A.lib().tfx_context_create(0, C.byref(h)) == A.TFX_ERR_NO_DEVICE
    assert not h.value
