"""CollideHairVerticesWithSdf, the mixed forward / backward difference collide of
TressFXSDFCollision.hlsl:599-715: the oracle against the reference shader compiled as C++ (where the
reference is mounted), and the CUDA kernel against the oracle on the GPU, bit for bit."""
import ctypes as C

import numpy as np
import pytest

import oracle
from oracle import hlsl_ref


def head():
    from tressfx_gb300 import synthetic as S
    return S.scene_head(seed=31, num_guides=160, n=16, follows=2, triangles=2500, sdf_cells=28, frames=5)


@pytest.mark.skipif(not hlsl_ref.available(), reason="reference shader sources not mounted")
def test_oracle_mixed_collide_equals_reference(oracle_lib):
    from oracle.scene_driver import OraclePipeline
    from tressfx_gb300.headless import FrameInputs
    from tressfx_gb300.synthetic import margin_world
    sc = head()
    ref = hlsl_ref.RefPipeline(sc)
    ora = OraclePipeline(sc)
    for f in range(3):
        fin = FrameInputs(sc, f)
        ref.step(fin)
        ora.step(fin)
    assert np.array_equal(ref.hair[0].pos.view(np.uint32), ora.hair[0].pos.view(np.uint32))
    fin = FrameInputs(sc, 3)
    ref.skin_and_build(0, fin)
    g = fin.grids[0]
    words = ref.sdf_words[0]
    margin = 4.0 * margin_world(sc.objects[0], g)   # a wide margin, so that many vertices are projected
    before = ora.hair[0].pos.copy()
    oracle.sdf_collide_mixed(g, words, margin, ora.hair[0])
    alloc = np.zeros(max(int(np.float32(1.4) * np.float32(g.num_cells)), g.num_cells), dtype=np.uint32)
    alloc[:g.num_cells] = words
    gp = oracle.sdf_params(g)
    hlsl_ref.lib().tfxr_sdf_collide_mixed(alloc.ctypes.data, len(alloc), C.addressof(gp), margin,
                                          C.addressof(ref.hair[0]._struct))
    for key in ("pos", "prev"):
        assert np.array_equal(getattr(ref.hair[0], key).view(np.uint32), getattr(ora.hair[0], key).view(np.uint32)), key
    moved = (ora.hair[0].pos != before).any(axis=-1).sum()
    assert moved > 20, moved


@pytest.mark.gpu
def test_cuda_mixed_collide_equals_oracle(ctx):
    from oracle.scene_driver import OraclePipeline
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.headless import FrameInputs, PlainPipeline
    from tressfx_gb300.synthetic import margin_world
    sc = head()
    gpu = PlainPipeline(ctx, sc)
    ora = OraclePipeline(sc)
    try:
        for f in range(3):
            fin = gpu.step(f)
            ora.step(fin)
        fin = FrameInputs(sc, 3)
        g = fin.grids[0]
        o = sc.objects[0]
        gpu.meshes[0].skin(fin.mesh_bones[0])
        gpu.sdfs[0].update(g)
        sk = oracle.mesh_skin(o.mesh.vertices, o.mesh.skinning, fin.mesh_bones[0])
        words = oracle.sdf_build(g, sk, o.mesh.indices)
        assert np.array_equal(gpu.sdfs[0].read(g.num_cells), words)
        margin = 4.0 * margin_world(o, g)
        before = ora.hair[0].pos.copy()
        gpu.sdfs[0].collide_mixed(gpu.hair[0], g, margin)
        oracle.sdf_collide_mixed(g, words, margin, ora.hair[0])
        for buf, key in ((A.BUF_POSITIONS, "pos"), (A.BUF_POSITIONS_PREV, "prev")):
            got = gpu.hair[0].read(buf).view(np.uint32)
            want = np.ascontiguousarray(getattr(ora.hair[0], key), dtype=np.float32).reshape(got.shape).view(np.uint32)
            assert np.array_equal(got, want), key
        assert (ora.hair[0].pos != before).any(axis=-1).sum() > 20
    finally:
        gpu.close()
