"""The oracle against the golden fixtures written from the reference's own shaders (CPU)."""
import pytest

from golden_replay import OracleBackend, fixtures, load, replay


@pytest.mark.parametrize("name", fixtures())
def test_oracle_matches_reference_fixture(oracle_lib, name):
    bad = replay(load(name), OracleBackend())
    assert not bad, f"{name}: oracle differs from the reference at {bad}"


def test_fixture_set_is_complete():
    names = fixtures()
    assert {"small_64x16", "small_64x4", "small_64x64_wind", "small_128x32_wind", "head_64x8_F1_sdf20",
            "real_ratboy_slice_sdf"} <= set(names)
