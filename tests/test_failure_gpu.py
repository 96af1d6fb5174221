"""Failure detection without a GPU fault.

* The batched strand kernel's bounded wait for its bulk copies: with the first wait's poll limit set
  to 0 every block gives up at once, raises the device error flag, waits (with the full limit) for
  the copies still in flight, and returns.  The host must see TFX_ERR_TIMEOUT once, through
  tfx_batch_synchronize and through tfx_batch_profile_frame, and the context must stay usable: with
  the state restored and the normal limit, the same frame is bit-exact against the oracle again.
* The report-only health scan tfx_hair_count_nonfinite: NaN and infinities planted from the host are
  counted per buffer; a clean state counts zero.
"""
import numpy as np
import pytest

from oracle.scene_driver import OraclePipeline
from tressfx_gb300 import _capi as A
from tressfx_gb300.headless import BatchedPipeline, FrameInputs, PlainPipeline
from tressfx_gb300.synthetic import scene_head

pytestmark = pytest.mark.gpu

STATE = [A.BUF_POSITIONS, A.BUF_POSITIONS_PREV, A.BUF_POSITIONS_PREV_PREV, A.BUF_TANGENTS, A.BUF_STRAND_LEVEL_DATA]
DEFAULT_WAIT_POLLS = 1 << 21


def _scene():
    return scene_head(seed=31, num_guides=200, n=16, follows=2, triangles=2000, sdf_cells=32, frames=8)


def _assert_equal_to_oracle(gpu, ora, what):
    for h, oh in zip(gpu.hair, ora.hair):
        for buf, name in ((A.BUF_POSITIONS, "pos"), (A.BUF_POSITIONS_PREV, "prev"), (A.BUF_TANGENTS, "tan")):
            g = h.read(buf).view(np.uint32)
            o = np.ascontiguousarray(getattr(oh, name), dtype=np.float32).view(np.uint32)
            assert np.array_equal(g, o), f"{what}: {name} differs in {int((g != o).sum())} words"


def test_batch_timeout_is_reported_once_and_the_context_recovers(ctx):
    sc = _scene()
    gpu = BatchedPipeline(ctx, sc)
    ora = OraclePipeline(sc)
    try:
        assert gpu.batch.get_option(gpu.batch.WAIT_POLLS) == DEFAULT_WAIT_POLLS
        for f in range(3):
            ora.step(gpu.step(f))
        gpu.batch.synchronize()
        snapshot = [{b: h.read(b) for b in STATE} for h in gpu.hair]

        # frame 3 with a wait that gives up at once
        gpu.batch.set_option(gpu.batch.WAIT_POLLS, 0)
        gpu.step(3)
        with pytest.raises(A.TfxError) as err:
            gpu.batch.synchronize()
        assert err.value.status == A.TFX_ERR_TIMEOUT
        gpu.batch.synchronize()                    # reported once: the flag is cleared
        with pytest.raises(A.TfxError) as err:     # the direct-launch path reports it too
            gpu.batch.profile_frame()
        assert err.value.status == A.TFX_ERR_TIMEOUT

        # the normal limit, the state before frame 3, and frame 3 again
        gpu.batch.set_option(gpu.batch.WAIT_POLLS, DEFAULT_WAIT_POLLS)
        for h, snap in zip(gpu.hair, snapshot):
            for b, arr in snap.items():
                h.write(b, arr)
            h.frame = 3
        gpu.frame = 3
        for f in (3, 4):
            ora.step(gpu.step(f))
        gpu.batch.synchronize()
        _assert_equal_to_oracle(gpu, ora, "after recovery")
    finally:
        gpu.close()


def test_wait_polls_option_is_validated(ctx):
    sc = _scene()
    gpu = BatchedPipeline(ctx, sc)
    try:
        with pytest.raises(A.TfxError) as err:
            gpu.batch.set_option(gpu.batch.WAIT_POLLS, -1)
        assert err.value.status == A.TFX_ERR_INVALID_ARGUMENT
    finally:
        gpu.close()


def test_nonfinite_scan_counts_planted_values(ctx):
    sc = _scene()
    gpu = PlainPipeline(ctx, sc)
    try:
        for f in range(2):
            gpu.step(f)
        h = gpu.hair[0]
        assert h.count_nonfinite() == (0, 0)
        pos = h.read(A.BUF_POSITIONS)
        prev = h.read(A.BUF_POSITIONS_PREV)
        n = h.n
        pos[5 * n + 7, 0] = np.nan                  # one vertex, x
        pos[9 * n + 3, 3] = np.inf                  # one vertex, the inverse mass
        prev[2 * n + 1, 1] = -np.inf
        prev[2 * n + 2, 2] = np.nan
        prev[len(prev) - 1, :] = np.nan             # the very last vertex, every component
        h.write(A.BUF_POSITIONS, pos)
        h.write(A.BUF_POSITIONS_PREV, prev)
        want = (int((~np.isfinite(pos)).any(axis=1).sum()), int((~np.isfinite(prev)).any(axis=1).sum()))
        assert want == (2, 3)
        assert h.count_nonfinite() == want
        # report only: the buffers are unchanged by the scan
        assert np.array_equal(h.read(A.BUF_POSITIONS).view(np.uint32), pos.view(np.uint32))
        # after a frame the count still follows what is in the buffers
        gpu.step(2)
        after_pos, after_prev = h.read(A.BUF_POSITIONS), h.read(A.BUF_POSITIONS_PREV)
        assert h.count_nonfinite() == (int((~np.isfinite(after_pos)).any(axis=1).sum()),
                                       int((~np.isfinite(after_prev)).any(axis=1).sum()))
    finally:
        gpu.close()
