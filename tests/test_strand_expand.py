"""Strand quad expansion (GetExpandedTressFXVert / GetExpandedTressFXShadowVert of TressFXStrands.hlsl):
the oracle against the reference shader compiled as C++ (where the reference is mounted), and the
CUDA kernel against the oracle on the GPU, bit for bit, for both forms, thin tips on and off, and
tangents that degenerate the screen-space right vector."""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from oracle import hlsl_ref


def case(seed: int, n: int = 16, strands: int = 200):
    rng = np.random.default_rng(seed)
    pos = np.zeros((strands * n, 4), np.float32)
    pos[:, :3] = rng.normal(0, 0.1, (strands * n, 3)) + np.array([0.0, 1.6, 0.0])
    pos[:, 3] = 1.0
    tan = np.zeros_like(pos)
    t = rng.normal(size=(strands * n, 3))
    tan[:, :3] = t / np.linalg.norm(t, axis=1, keepdims=True)
    eye = np.array([0.3, 1.7, 1.2], np.float32)
    d = pos[:7, :3] - eye   # tangents along the view direction: right = 0
    tan[:7, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    tan[7:9, :3] = 0.0
    f, a, zn, zf = 1.0 / math.tan(0.5), 16 / 9, 0.05, 50.0
    P = np.array([[f / a, 0, 0, 0], [0, f, 0, 0], [0, 0, zf / (zn - zf), zn * zf / (zn - zf)], [0, 0, -1, 0]])
    V = np.eye(4)
    V[:3, 3] = -eye
    vp = (P @ V).astype(np.float32).reshape(16)
    fp = np.array([0.4, 0.3, 0.2, 1.0, 0.9, 0.8, 0.7, 1.0, 0.35, 1.0, 0.25, 0.0012], np.float32)
    return pos, tan, n, fp, eye, np.array([1920.0, 1080.0], np.float32), vp


def run_oracle(pos, tan, n, fp, eye, win, vp, thin, shadow):
    ip = np.array([n, thin], np.int32)
    out = np.zeros((2 * len(pos), 16), np.float32)
    lib = oracle.lib()
    lib.tfxo_expand_strands.argtypes = [C.c_void_p] * 2 + [C.c_int64] + [C.c_void_p] * 5 + [C.c_int, C.c_void_p]
    r = lib.tfxo_expand_strands(pos.ctypes.data, tan.ctypes.data, len(pos), fp.ctypes.data, ip.ctypes.data,
                                eye.ctypes.data, win.ctypes.data, vp.ctypes.data, shadow, out.ctypes.data)
    assert r == 0
    return out


@pytest.mark.skipif(not hlsl_ref.available(), reason="reference shader sources not mounted")
@pytest.mark.parametrize("thin,shadow", [(0, 0), (1, 0), (1, 1)])
def test_oracle_expansion_equals_reference(oracle_lib, thin, shadow):
    pos, tan, n, fp, eye, win, vp = case(3)
    want = np.zeros((2 * len(pos), 16), np.float32)
    ip = np.array([n, thin], np.int32)
    hlsl_ref.lib().tfxr_expand_strands(pos.ctypes.data, tan.ctypes.data, len(pos), fp.ctypes.data, ip.ctypes.data,
                                       eye.ctypes.data, win.ctypes.data, vp.ctypes.data, shadow, want.ctypes.data)
    got = run_oracle(pos, tan, n, fp, eye, win, vp, thin, shadow)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.isfinite(got).all() and np.abs(got[:, :4]).max() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("thin,shadow", [(0, 0), (1, 0), (1, 1)])
def test_cuda_expansion_equals_oracle(ctx, thin, shadow):
    torch = pytest.importorskip("torch")
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.api import HairObject
    pos, tan, n, fp, eye, win, vp = case(5)

    class Asset:
        pass
    a = Asset()
    a.num_guide_strands, a.verts_per_strand, a.follow_per_guide = len(pos) // n, n, 0
    a.positions, a.tangents = pos.copy(), tan.copy()
    a.rest_lengths = np.zeros(len(pos), np.float32)
    a.follow_root_offsets = np.zeros((len(pos) // n, 4), np.float32)
    sk = np.zeros((len(pos) // n, 8), np.float32)
    sk[:, 4] = 1.0
    a.bone_skinning = sk
    h = HairObject(ctx, a)
    h.write(A.BUF_TANGENTS, tan)
    p = A.StrandParams()
    for k in range(4):
        p.mat_base_color[k], p.mat_tip_color[k] = float(fp[k]), float(fp[4 + k])
    p.tip_percentage, p.strand_uv_tiling_factor, p.fiber_ratio, p.fiber_radius = (float(x) for x in fp[8:12])
    p.num_vertices_per_strand, p.enable_thin_tip = n, thin
    out = torch.zeros((2 * len(pos), 16), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    f3 = (C.c_float * 3)(*eye)
    f2 = (C.c_float * 2)(*win)
    f16 = (C.c_float * 16)(*vp)
    assert A.lib().tfx_hair_expand_strands(h.handle, C.byref(p), f3, f2, f16, shadow, out.data_ptr()) == 0
    ctx.synchronize()
    got = out.cpu().numpy()
    want = run_oracle(pos, tan, n, fp, eye, win, vp, thin, shadow)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    h.close()
