"""A hair object colliding with several meshes in turn, each on its own SDF, as the reference's sample
applies every collision mesh to every hair object (Simulation::RunCollision, src/Simulation.cpp:106-118):
the plain path (one collide dispatch per mesh) and the batched path (tfx_batch_add_hair_collision:
the first mesh inside the follow/collide kernel, each further one as a collision level) against the
oracle, word for word over twelve frames.  The two further meshes sit where the hair hangs, so both
change the result."""
import dataclasses

import numpy as np
import pytest

from oracle.scene_driver import OraclePipeline
from tressfx_gb300 import _capi as A
from tressfx_gb300.headless import BatchedPipeline, FrameInputs, PlainPipeline
from tressfx_gb300.synthetic import HEAD_CENTER, Collider, Mesh, ellipsoid_mesh, mesh_lat_lon_for, scene_head

FRAMES = 12
BUFS = [(A.BUF_POSITIONS, "pos"), (A.BUF_POSITIONS_PREV, "prev"), (A.BUF_POSITIONS_PREV_PREV, "prevprev"),
        (A.BUF_TANGENTS, "tan"), (A.BUF_STRAND_LEVEL_DATA, "sld")]


def _ellipsoid(center, radii, triangles: int) -> Mesh:
    nl, nq = mesh_lat_lon_for(triangles)
    v, i = ellipsoid_mesh(center, radii, nl, nq)
    sk = np.zeros((len(v), 8), np.float32)
    sk[:, 0:4] = (2, 0, 0, 0)
    sk[:, 4:8] = (1, 0, 0, 0)
    return Mesh(vertices=v.astype(np.float32), indices=i.astype(np.uint32), skinning=sk)


def _scene(with_more: bool = True):
    sc = scene_head(seed=31, num_guides=1536, n=32, follows=2, triangles=3000, sdf_cells=40, frames=FRAMES)
    o = sc.objects[0]
    if with_more:
        c = np.array(HEAD_CENTER)
        for off, radii, cells in (((0.0, -0.10, 0.09), (0.07, 0.05, 0.05), 36), ((0.09, -0.06, 0.0), (0.04, 0.06, 0.05), 28)):
            m = _ellipsoid(c + np.array(off), radii, 2000)
            p = m.vertices[:, :3]
            ext = float((p.max(0) - p.min(0)).max()) + 0.04
            o.more.append(Collider(m, o.mesh_bone_fn, (cells,) * 3, ext / cells, (p.min(0) + p.max(0)) / 2,
                                   follow_bone=2, collision_margin_cells=0.5))
    return sc


def _compare(gpu, ora, what):
    for h, oh in zip(gpu.hair, ora.hair):
        for buf, name in BUFS:
            g = h.read(buf).reshape(-1).view(np.uint32)
            o = np.ascontiguousarray(getattr(oh, name), dtype=np.float32).reshape(-1).view(np.uint32)
            bad = np.nonzero(g != o)[0]
            assert len(bad) == 0, f"{what}: {name} differs in {len(bad)} of {len(g)} words (first {bad[0]})"


def test_further_meshes_change_the_result():
    """The oracle with the two further meshes differs from the oracle with the first mesh only."""
    a, b = _scene(True), _scene(False)
    oa, ob = OraclePipeline(a), OraclePipeline(b)
    for f in range(FRAMES):
        oa.step(FrameInputs(a, f))
        ob.step(FrameInputs(b, f))
    assert int((oa.hair[0].pos != ob.hair[0].pos).any(axis=1).sum()) > 200


@pytest.mark.gpu
@pytest.mark.parametrize("path", ["plain", "batched"])
def test_several_collision_meshes(ctx, path):
    sc = _scene()
    gpu = PlainPipeline(ctx, sc) if path == "plain" else BatchedPipeline(ctx, sc, autotune_frames=0)
    ora = OraclePipeline(sc)
    try:
        for f in range(FRAMES):
            if path == "plain":
                gpu.step(f)
                ora.step(FrameInputs(sc, f))
            else:
                ora.step(gpu.step(f))
            if f in (2, 7):
                _compare(gpu, ora, f"{path}, frame {f}")
        _compare(gpu, ora, f"{path}, frame {FRAMES - 1}")
    finally:
        gpu.close()


@pytest.mark.gpu
def test_batch_rejects_bad_further_collisions(ctx):
    from tressfx_gb300.api import Batch, CollisionMesh, HairObject, SDFCollision
    sc = _scene(False)
    o = sc.objects[0]
    hair = HairObject(ctx, o.asset)
    m = CollisionMesh(ctx, o.mesh.vertices, o.mesh.indices, o.mesh.skinning)
    s = SDFCollision(ctx, int(np.prod(o.sdf_dims)))
    b = Batch(ctx)
    try:
        si = b.add_sdf(s, m, o.sdf_dims)
        hi = b.add_hair(hair, -1)
        with pytest.raises(RuntimeError):
            b.add_hair_collision(hi, si)          # the object was added without an SDF
        with pytest.raises(RuntimeError):
            b.add_hair_collision(hi + 1, si)      # no such object
        with pytest.raises(RuntimeError):
            b.add_hair_collision(hi, si + 1)      # no such SDF
    finally:
        b.close()
        for x in (s, m, hair):
            x.close()


def _mixed_scene():
    """Four objects of different strand lengths (one with follow hairs); objects 0 and 2 collide with
    two further meshes, object 3 with one, object 1 with none: the levels hold different objects."""
    from tressfx_gb300.synthetic import scene_batched
    sc = scene_batched(seed=12, num_objects=4, min_strands=256, max_strands=1200, verts=(8, 16, 32, 64),
                       min_tris=1500, max_tris=3000, sdf_choices=(24, 32), follows=1, frames=FRAMES)
    for k, extra in ((0, 2), (2, 2), (3, 1)):
        o = sc.objects[k]
        c = np.asarray(o.sdf_center0) + np.array([0.0, 0.1, 0.0])   # head centre, as the scene places it
        for q in range(extra):
            off = np.array([(0.07, -0.09, 0.06), (-0.08, -0.05, 0.03)][q])
            m = _ellipsoid(c + off, (0.05, 0.05, 0.05), 1200)
            p = m.vertices[:, :3]
            ext = float((p.max(0) - p.min(0)).max()) + 0.04
            o.more.append(Collider(m, o.mesh_bone_fn, (28, 28, 28), ext / 28, (p.min(0) + p.max(0)) / 2, follow_bone=2,
                                   collision_margin_cells=0.5))
    return sc


@pytest.mark.gpu
@pytest.mark.parametrize("path", ["plain", "batched"])
def test_several_collision_meshes_mixed_classes(ctx, path):
    sc = _mixed_scene()
    gpu = PlainPipeline(ctx, sc) if path == "plain" else BatchedPipeline(ctx, sc, autotune_frames=0)
    ora = OraclePipeline(sc)
    try:
        for f in range(FRAMES):
            if path == "plain":
                gpu.step(f)
                ora.step(FrameInputs(sc, f))
            else:
                ora.step(gpu.step(f))
        _compare(gpu, ora, f"mixed classes, {path}, frame {FRAMES - 1}")
    finally:
        gpu.close()
