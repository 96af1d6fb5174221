"""The CUDA library against the golden fixtures written from the reference's own shaders (GPU)."""
import pytest

from golden_replay import GpuBackend, fixtures, load, replay

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", fixtures())
def test_cuda_matches_reference_fixture(ctx, name):
    be = GpuBackend(ctx)
    try:
        bad = replay(load(name), be)
    finally:
        be.close()
    assert not bad, f"{name}: CUDA path differs from the reference at {bad}"
