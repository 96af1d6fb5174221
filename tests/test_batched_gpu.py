"""GPU parity of the batched path: one CUDA-graph launch per frame with fused persistent kernels
and the tiled SDF build, against the FP32 oracle (and the plain path), bit for bit."""
import numpy as np
import pytest

from oracle.scene_driver import OraclePipeline
from tressfx_gb300 import _capi as A
from tressfx_gb300.headless import BatchedPipeline, FrameInputs, PlainPipeline
from tressfx_gb300.synthetic import scene_batched, scene_head, scene_small

pytestmark = pytest.mark.gpu

BUFS = [(A.BUF_POSITIONS, "pos"), (A.BUF_POSITIONS_PREV, "prev"), (A.BUF_POSITIONS_PREV_PREV, "prevprev"),
        (A.BUF_TANGENTS, "tan"), (A.BUF_STRAND_LEVEL_DATA, "sld")]


def assert_same(gpu_hair, ora_hair, what):
    for buf, name in BUFS:
        g = gpu_hair.read(buf).reshape(-1).view(np.uint32)
        o = np.ascontiguousarray(getattr(ora_hair, name), dtype=np.float32).reshape(-1).view(np.uint32)
        bad = np.nonzero(g != o)[0]
        assert len(bad) == 0, f"{what}/{name}: {len(bad)} of {len(g)} words differ (first {bad[0]})"


def run_pair(ctx, sc, frames, autotune=0):
    gpu = BatchedPipeline(ctx, sc, autotune_frames=autotune)
    ora = OraclePipeline(sc)
    try:
        for f in range(frames):
            fin = gpu.step(f)
            ora.step(fin)
        for i, (h, oh) in enumerate(zip(gpu.hair, ora.hair)):
            assert_same(h, oh, f"{sc.name} object {i}")
        return gpu.batch.describe()
    finally:
        gpu.close()


def test_batched_head_with_sdf(ctx):
    sc = scene_head(seed=21, num_guides=300, n=32, follows=3, triangles=3000, sdf_cells=48, frames=6)
    desc, launches = run_pair(ctx, sc, 6)
    assert launches <= 8, desc


@pytest.mark.parametrize("n", [4, 8, 16, 32, 64])
def test_batched_every_strand_length(ctx, n):
    sc = scene_small(seed=40 + n, num_guides=77, n=n)
    sc.objects[0].settings.update(local_constraints_iterations=3, length_constraints_iterations=2, wind_magnitude=1.0)
    run_pair(ctx, sc, 8)


def test_batched_mixed_objects(ctx):
    sc = scene_batched(seed=5, num_objects=7, min_strands=64, max_strands=700, min_tris=800, max_tris=3000,
                       sdf_choices=(24, 32, 40), follows=1, frames=5)
    run_pair(ctx, sc, 5)


def test_batched_sdf_chunks_span_sdfs(ctx):
    """Meshes of 20k-40k triangles: the batch's construct hands each warp chunks of several
    consecutive triangles of the batch's list (on 152 SMs: 7 a chunk), which cross from one SDF's
    triangles into the next; every grid and the hair state against the oracle."""
    sc = scene_batched(seed=8, num_objects=4, min_strands=64, max_strands=256, min_tris=20000, max_tris=40000,
                       sdf_choices=(48, 64), frames=3)
    gpu = BatchedPipeline(ctx, sc)
    ora = OraclePipeline(sc)
    try:
        for f in range(3):
            fin = gpu.step(f)
            ora.step(fin)
        for i, g in enumerate(fin.grids):
            assert np.array_equal(gpu.sdfs[i].read(g.num_cells), ora.sdf_words[i]), f"SDF {i}"
        for i, (h, oh) in enumerate(zip(gpu.hair, ora.hair)):
            assert_same(h, oh, f"object {i}")
    finally:
        gpu.close()


@pytest.mark.parametrize("form", [0, 1, 2])
def test_batched_classes_with_and_without_follow_hairs(ctx, form):
    """A class whose objects have no follow hairs runs the follow/collide kernels specialised for
    F = 0; a class mixing objects with and without follow hairs runs the general ones.  Both, in each
    follow/collide form, against the oracle."""
    from tressfx_gb300.synthetic import build_asset
    sc = scene_batched(seed=9, num_objects=6, min_strands=64, max_strands=300, min_tris=800, max_tris=2000,
                       sdf_choices=(24, 32), verts=(16, 32), frames=4)
    rng = np.random.default_rng(90)
    for o in sc.objects[2:4]:   # two of the three n = 16 objects get two follow hairs per guide
        a = o.asset
        guides = a.positions.reshape(a.num_guide_strands, a.verts_per_strand, 4)[:, :, :3].astype(np.float64)
        o.asset = build_asset(guides, 2, tip_separation=0.5, follow_radius=0.002, rng=rng,
                              bone_skinning=a.bone_skinning.reshape(-1, 8))
    assert [o.asset.verts_per_strand for o in sc.objects] == [32, 32, 16, 16, 16, 32]
    assert [o.asset.follow_per_guide for o in sc.objects] == [0, 0, 2, 2, 0, 0]
    gpu = BatchedPipeline(ctx, sc)
    gpu.batch.set_option(gpu.batch.FOLLOW_FORM, form)
    ora = OraclePipeline(sc)
    try:
        for f in range(4):
            fin = gpu.step(f)
            ora.step(fin)
        for i, (h, oh) in enumerate(zip(gpu.hair, ora.hair)):
            assert_same(h, oh, f"form {form} object {i}")
    finally:
        gpu.close()


def test_batched_autotune_keeps_state(ctx):
    sc = scene_batched(seed=6, num_objects=4, min_strands=64, max_strands=400, min_tris=800, max_tris=2000,
                       sdf_choices=(24, 32), frames=4)
    desc, _ = run_pair(ctx, sc, 4, autotune=2)
    assert "vertices/lane" in desc


def test_batched_equals_plain_path(ctx):
    sc = scene_head(seed=22, num_guides=256, n=16, follows=2, triangles=2500, sdf_cells=40, frames=5)
    a = PlainPipeline(ctx, sc)
    b = BatchedPipeline(ctx, sc)
    try:
        for f in range(5):
            a.step(f)
            b.step(f)
        for buf, name in BUFS:
            assert np.array_equal(a.hair[0].read(buf).view(np.uint32), b.hair[0].read(buf).view(np.uint32)), name
    finally:
        a.close()
        b.close()


def test_batched_sdf_with_huge_triangles_falls_back_exactly(ctx):
    """Triangles whose cell boxes cover most of the grid overflow the (triangle, tile) list; the
    tile pass then scans every triangle and the grid is still exact."""
    import oracle
    from tressfx_gb300.synthetic import Mesh, SceneObject, Scene, build_asset, grow_strands, sample_on_ellipsoid, \
        rigid_oscillation_bones
    rng = np.random.default_rng(3)
    v = np.zeros((4 + 3 * 400, 8), dtype=np.float32)
    v[:4, :3] = [(-0.3, 1.3, -0.3), (0.3, 1.3, -0.3), (0.3, 1.9, 0.3), (-0.3, 1.9, 0.3)]
    v[4:, :3] = rng.uniform(-0.12, 0.12, size=(1200, 3)) + np.array([0.0, 1.6, 0.0])
    v[:, 3] = 1.0
    idx = [0, 1, 2, 0, 2, 3] + list(range(4, 4 + 1200))
    idx = np.array(idx, dtype=np.uint32)
    skin = np.zeros((len(v), 8), dtype=np.float32)
    skin[:, 4] = 1.0
    mesh = Mesh(v, idx, skin)
    roots, normals = sample_on_ellipsoid((0.0, 1.6, 0.0), (0.1, 0.1, 0.1), 64, rng)
    asset = build_asset(grow_strands(roots, normals, 16, 0.006, 15.0, rng))
    bones = rigid_oscillation_bones(10.0, 1.0, "y")
    st = dict(vsp_coeff=0.8, vsp_accel_threshold=1.4, local_constraint_stiffness=0.9, local_constraints_iterations=1,
              global_constraint_stiffness=0.0, global_constraints_range=0.0, length_constraints_iterations=1,
              damping=0.08, gravity_magnitude=9.8, tip_separation=0.0, wind_magnitude=0.0, wind_direction=(1, 0, 0))
    obj = SceneObject(asset, st, bones, mesh, bones, (40, 40, 40), 0.7 / 40, np.array([0.0, 1.6, 0.0]), follow_bone=0)
    sc = Scene("huge_triangles", [obj], frames=3)
    gpu = BatchedPipeline(ctx, sc)
    ora = OraclePipeline(sc)
    try:
        for f in range(3):
            fin = gpu.step(f)
            ora.step(fin)
        g = fin.grids[0]
        words = gpu.sdfs[0].read(g.num_cells)
        assert np.array_equal(words, ora.sdf_words[0])
        assert_same(gpu.hair[0], ora.hair[0], "huge triangles")
    finally:
        gpu.close()


def test_batch_rejects_bad_use(ctx):
    from tressfx_gb300.api import Batch, HairObject
    sc = scene_small(num_guides=64, n=16)
    h = HairObject(ctx, sc.objects[0].asset)
    b = Batch(ctx)
    b.add_hair(h, -1)
    with pytest.raises(A.TfxError):
        b.add_hair(h, -1)            # twice
    with pytest.raises(A.TfxError):
        b.run()                      # not built
    b.build()
    with pytest.raises(A.TfxError):
        b.run()                      # constants never set
    p = h.current_params()
    with pytest.raises(A.TfxError) as e:
        b.set_hair_constants(0, p, 1, 1)   # counts of a never-filled block are zero
    assert e.value.status == A.TFX_ERR_MISMATCH
    b.close()
    h.close()


@pytest.mark.parametrize("expanded,overlap", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_batched_options_bit_exact(ctx, expanded, overlap):
    """Corner-expanded lookups and the overlapped SDF branch change nothing in the results."""
    sc = scene_head(seed=23, num_guides=200, n=16, follows=2, triangles=2500, sdf_cells=40, frames=4)
    gpu = BatchedPipeline(ctx, sc)
    try:
        gpu.batch.set_option(gpu.batch.EXPANDED_GRIDS, expanded)
        gpu.batch.set_option(gpu.batch.OVERLAP_SDF, overlap)
        gpu.batch.set_option(gpu.batch.SDF_BLOCK, 64)
        assert (gpu.batch.get_option(gpu.batch.EXPANDED_GRIDS), gpu.batch.get_option(gpu.batch.OVERLAP_SDF)) == \
            (expanded, overlap)
        ora = OraclePipeline(sc)
        for f in range(4):
            fin = gpu.step(f)
            ora.step(fin)
        assert_same(gpu.hair[0], ora.hair[0], f"expanded={expanded} overlap={overlap}")
        with pytest.raises(Exception):
            gpu.batch.set_option(gpu.batch.SDF_BLOCK, 100)
    finally:
        gpu.close()



@pytest.mark.gpu
@pytest.mark.parametrize("follows", [2, 4, 40])
def test_batched_follow_collide_many_contacts_bit_exact(ctx, follows):
    """The follow-hair + collision kernel with a wide margin (most vertices near the scalp collide) and
    with more follow hairs than a warp has lanes: the oracle's buffers, bit for bit."""
    sc = scene_head(seed=29, num_guides=96 if follows > 31 else 300, n=16, follows=follows, triangles=2500,
                    sdf_cells=40, frames=5)
    sc.objects[0].collision_margin_cells = 5.0
    gpu = BatchedPipeline(ctx, sc)
    try:
        ora = OraclePipeline(sc)
        for f in range(5):
            fin = gpu.step(f)
            ora.step(fin)
        assert_same(gpu.hair[0], ora.hair[0], f"follows={follows}")
    finally:
        gpu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", [0, 1])
def test_batched_readback_delivers_each_frame(ctx, fmt):
    """tfx_batch_readback: the positions after each frame (float4, or packed xyz) reach host memory bit
    for bit while later frames run; bad tickets, formats and destination counts are refused."""
    from tressfx_gb300.api import PinnedArray
    sc = scene_head(seed=31, num_guides=200, n=16, follows=2, triangles=2500, sdf_cells=40, frames=6)
    sc2 = scene_small(seed=3, num_guides=100, n=8)
    sc.objects.append(sc2.objects[0])
    gpu = BatchedPipeline(ctx, sc)
    width = 4 if fmt == 0 else 3
    bufs = [[PinnedArray((h.num_vertices, width), np.float32) for h in gpu.hair] for _ in range(3)]
    try:
        tickets, want = [], []

        def check(f):
            for o in range(len(gpu.hair)):
                got = bufs[f % 3][o].array
                assert np.array_equal(got.view(np.uint32), want[f][o][:, :width].view(np.uint32)), (f, o)

        for f in range(6):
            gpu.step(f)
            tickets.append(gpu.batch.readback([b.array.ctypes.data for b in bufs[f % 3]], fmt))
            if f >= 2:
                gpu.batch.wait_readback(tickets[f - 2])
                check(f - 2)
            ctx.synchronize()
            want.append([np.ascontiguousarray(h.read(A.BUF_POSITIONS).reshape(-1, 4)) for h in gpu.hair])
        for f in (4, 5):
            gpu.batch.wait_readback(tickets[f])
            check(f)
        with pytest.raises(Exception):
            gpu.batch.wait_readback(99)
        with pytest.raises(Exception):
            gpu.batch.readback([])
        with pytest.raises(Exception):
            gpu.batch.readback([b.array.ctypes.data for b in bufs[0]], 7)
    finally:
        for side in bufs:
            for b in side:
                b.free()
        gpu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n,iters", [(4, 2), (16, 6), (32, 3), (64, 2)])
@pytest.mark.parametrize("split", [0, 1])
def test_batched_split_sweeps_bit_exact(ctx, n, iters, split):
    """The local-shape sweeps inside the strand kernel (0) or as their own launch between its two
    halves, up to four sweeps pipelined in a thread's registers and more in waves (1): the oracle's
    buffers either way, for every strand length (n = 64 runs one sweep per frame, the reference rule)."""
    sc = scene_head(seed=37, num_guides=150, n=n, follows=1, triangles=2500, sdf_cells=40, frames=4)
    sc.objects[0].settings["local_constraints_iterations"] = iters
    gpu = BatchedPipeline(ctx, sc)
    try:
        gpu.batch.set_option(gpu.batch.SPLIT_SWEEPS, split)
        assert gpu.batch.get_option(gpu.batch.SPLIT_SWEEPS) == split
        ora = OraclePipeline(sc)
        for f in range(4):
            fin = gpu.step(f)
            ora.step(fin)
        assert_same(gpu.hair[0], ora.hair[0], f"n={n} iters={iters} split={split}")
    finally:
        gpu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1, 2])
@pytest.mark.parametrize("n,follows", [(16, 0), (16, 2), (64, 0), (64, 1)])
def test_batched_follow_forms_bit_exact(ctx, form, n, follows):
    """Every form of the follow-hair + collision kernel (one vertex at a time, both lookup stages on
    per-warp queues, the gradient stage alone queued) gives the oracle's buffers, with and without
    follow hairs, on hair lying against the collision mesh."""
    sc = scene_head(seed=41 + n + follows, num_guides=180, n=n, follows=follows, triangles=2500, sdf_cells=40,
                    frames=5)
    gpu = BatchedPipeline(ctx, sc)
    try:
        gpu.batch.set_option(gpu.batch.FOLLOW_FORM, form)
        assert gpu.batch.get_option(gpu.batch.FOLLOW_FORM) == form
        ora = OraclePipeline(sc)
        for f in range(5):
            fin = gpu.step(f)
            ora.step(fin)
        assert_same(gpu.hair[0], ora.hair[0], f"form={form} n={n} follows={follows}")
        with pytest.raises(Exception):
            gpu.batch.set_option(gpu.batch.FOLLOW_FORM, 3)
    finally:
        gpu.close()
