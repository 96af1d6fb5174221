"""Parity on the workloads the benchmark times, at full size, over dynamic frames.

Frames 0 and 1 are reset frames (UpdateSimulationParameters sets g_ResetPositions while the
simulation frame is below 2, TressFXHairObject.cpp:433-434): the positions are the skinned rest pose
and the Verlet term never runs.  These tests run 12 frames, so 10 of them integrate, and compare every
state buffer of every object with the FP32 oracle word for word:

* the plain path (one launch per object per stage) on the head (20,000 x 32, 4 follow hairs, SDF 64^3),
  fur (200,000 x 16, SDF 128^3) and 64-object workloads;
* the batched path with the launch shapes its autotuner picks (as the benchmark runs it) on the head,
  fur and 64-object workloads.
"""
import numpy as np
import pytest

from oracle.scene_driver import OraclePipeline
from tressfx_gb300 import _capi as A
from tressfx_gb300.headless import BatchedPipeline, FrameInputs, PlainPipeline
from tressfx_gb300.synthetic import scene_batched, scene_fur, scene_head

pytestmark = pytest.mark.gpu

FRAMES = 12
BUFS = [(A.BUF_POSITIONS, "pos"), (A.BUF_POSITIONS_PREV, "prev"), (A.BUF_POSITIONS_PREV_PREV, "prevprev"),
        (A.BUF_TANGENTS, "tan"), (A.BUF_STRAND_LEVEL_DATA, "sld")]


def _scene(which):
    return {"head": scene_head, "fur": scene_fur, "batched": scene_batched}[which]()


def _compare(gpu, ora, what):
    for i, (h, oh) in enumerate(zip(gpu.hair, ora.hair)):
        for buf, name in BUFS:
            g = h.read(buf).reshape(-1).view(np.uint32)
            o = np.ascontiguousarray(getattr(oh, name), dtype=np.float32).reshape(-1).view(np.uint32)
            bad = np.nonzero(g != o)[0]
            assert len(bad) == 0, f"{what}, object {i}: {name} differs in {len(bad)} of {len(g)} words (first {bad[0]})"


def _moved(ora) -> bool:
    """Some vertex moved away from its rest position (the dynamic frames did integrate)."""
    return any(not np.array_equal(oh.pos, oh.init) for oh in ora.hair)


@pytest.mark.parametrize("which", ["head", "fur", "batched"])
def test_plain_full_size_dynamic_frames(ctx, which):
    sc = _scene(which)
    gpu = PlainPipeline(ctx, sc)
    ora = OraclePipeline(sc)
    try:
        for f in range(FRAMES):
            gpu.step(f)
            ora.step(FrameInputs(sc, f))
            if f == 2:
                _compare(gpu, ora, f"{which} plain, frame {f}")
        _compare(gpu, ora, f"{which} plain, frame {FRAMES - 1}")
        assert _moved(ora)
    finally:
        gpu.close()


@pytest.mark.parametrize("which", ["head", "fur", "batched"])
def test_batched_full_size_dynamic_frames_autotuned(ctx, which):
    sc = _scene(which)
    gpu = BatchedPipeline(ctx, sc, autotune_frames=4)
    ora = OraclePipeline(sc)
    try:
        for f in range(FRAMES):
            ora.step(gpu.step(f))
            if f == 2:
                _compare(gpu, ora, f"{which} batched, frame {f}")
        desc, _ = gpu.batch.describe()
        _compare(gpu, ora, f"{which} batched ({desc}), frame {FRAMES - 1}")
        assert _moved(ora)
    finally:
        gpu.close()


def test_batched_tiled_construct_full_size(ctx):
    """The tile-binned SDF construct (TFX_BATCH_SDF_FORM 1) on the 64-object workload: every SDF and
    every state buffer word for word against the oracle over six frames (four integrating)."""
    sc = _scene("batched")
    gpu = BatchedPipeline(ctx, sc, autotune_frames=0)
    gpu.batch.set_option(gpu.batch.SDF_FORM, 1)
    ora = OraclePipeline(sc)
    try:
        for f in range(6):
            ora.step(gpu.step(f))
        _compare(gpu, ora, "batched, tiled construct, frame 5")
        for i, s in enumerate(gpu.sdfs):
            got = s.read(int(np.prod(sc.objects[i].sdf_dims))).view(np.uint32)
            want = np.ascontiguousarray(ora.sdf_words[i]).reshape(-1)[:got.size].view(np.uint32)
            bad = np.nonzero(got != want)[0]
            assert len(bad) == 0, f"SDF {i}: {len(bad)} of {got.size} cells differ (first {bad[:5].tolist()})"
        assert _moved(ora)
    finally:
        gpu.close()
