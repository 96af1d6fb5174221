"""Frames of the GPU paths against the FP32 oracle on real data: a slice of the reference's shipped
Ratboy asset (tests/golden/ratboy_subset.npz, loaded by the reference's own code), the mohawk slice
with the sample's mohawk settings colliding with the body slice through an SDF sized by the
reference's rule, 105 bones posed per frame.  Twelve frames (ten of them integrating), every state
buffer compared word for word, with the body's margin (0 cells) and with half a cell."""
import dataclasses

import numpy as np
import pytest

import ratboy_scene
from oracle.scene_driver import OraclePipeline
from tressfx_gb300 import _capi as A
from tressfx_gb300.headless import BatchedPipeline, FrameInputs, PlainPipeline

pytestmark = pytest.mark.gpu

FRAMES = 12
BUFS = [(A.BUF_POSITIONS, "pos"), (A.BUF_POSITIONS_PREV, "prev"), (A.BUF_POSITIONS_PREV_PREV, "prevprev"),
        (A.BUF_TANGENTS, "tan"), (A.BUF_STRAND_LEVEL_DATA, "sld")]


def _compare(gpu, ora, what):
    for h, oh in zip(gpu.hair, ora.hair):
        for buf, name in BUFS:
            g = h.read(buf).reshape(-1).view(np.uint32)
            o = np.ascontiguousarray(getattr(oh, name), dtype=np.float32).reshape(-1).view(np.uint32)
            bad = np.nonzero(g != o)[0]
            assert len(bad) == 0, f"{what}: {name} differs in {len(bad)} of {len(g)} words (first {bad[0]})"


def _contacts(sc) -> int:
    """Vertices whose final position the collision meshes changed (oracle with and without them)."""
    o = sc.objects[0]
    bare = dataclasses.replace(sc, objects=[dataclasses.replace(o, mesh=None, mesh_bone_fn=None, more=[])])
    a, b = OraclePipeline(sc), OraclePipeline(bare)
    for f in range(FRAMES):
        a.step(FrameInputs(sc, f))
        b.step(FrameInputs(bare, f))
    return int((a.hair[0].pos != b.hair[0].pos).any(axis=1).sum())


@pytest.mark.parametrize("margin,hands", [(0.0, False), (0.5, False), (0.0, True)],
                         ids=["body", "body_margin_half_cell", "body_and_hands"])
@pytest.mark.parametrize("path", ["plain", "batched"])
def test_ratboy_slice_frames(ctx, path, margin, hands):
    """With `hands`, the sample's set-up: the mohawk collides with the body (margin 0), then with each
    hand (32 cells across, margin 0.5), each on its own SDF."""
    sc = ratboy_scene.scene(FRAMES, margin_cells=margin, hands=hands)
    assert _contacts(sc) > 100
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
                _compare(gpu, ora, f"{sc.name} {path}, margin {margin}, frame {f}")
        _compare(gpu, ora, f"{sc.name} {path}, margin {margin}, frame {FRAMES - 1}")
    finally:
        gpu.close()
