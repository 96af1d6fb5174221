"""The C++ TressFXAsset of libtressfx_host (.tfx / .tfxbone loading, GenerateFollowHairs,
ProcessAsset) against the reference's own TressFXAsset.cpp: array for array, bit for bit.

Where the reference tree is present its asset code is compiled and run beside ours
(oracle/asset_ref); everywhere, ours is checked against the committed digests of the reference's
output (tests/golden/asset_digests.json)."""
import json
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from asset_cases import CASES, build_asset_dump, digests, run_driver, write_case_files
from asset_files import strands, write_tfx, write_tfxbone

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def dump_exe(built_lib, tmp_path_factory):
    return build_asset_dump(tmp_path_factory.mktemp("asset_dump"))


@pytest.fixture(scope="module")
def ref_exe():
    from oracle.asset_ref import build as asset_ref
    try:
        return asset_ref.build()
    except RuntimeError as e:  # pragma: no cover
        pytest.skip(f"reference asset pipeline not buildable: {e}")


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_asset_matches_reference_digests(dump_exe, tmp_path, case):
    want = json.loads((HERE / "golden" / "asset_digests.json").read_text())[case[0]]
    counts, arrays = run_driver(dump_exe, tmp_path, case)
    got = digests(counts, arrays)
    assert got == want, {k: (got[k] == want[k]) for k in want}


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_asset_matches_reference_side_by_side(dump_exe, ref_exe, tmp_path, case):
    if ref_exe is None:
        pytest.skip("reference tree not present")
    c1, a1 = run_driver(dump_exe, tmp_path, case)
    c2, a2 = run_driver(ref_exe, tmp_path, case)
    assert np.array_equal(c1, c2)
    for k in a1:
        x, y = a1[k], a2[k]
        if k == "tangents":   # w is never set by the reference
            x, y = x.reshape(-1, 4)[:, :3], y.reshape(-1, 4)[:, :3]
        assert x.shape == y.shape and np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                                                     y.view(np.uint32) if y.dtype == np.float32 else y), k


def test_padding_rule_and_counts(dump_exe, tmp_path):
    """Guide strands are raised to the next multiple of 64 above the file's count (always by at
    least one strand: 128 -> 192), the made-up strands repeating the last one."""
    for num, want in ((100, 128), (128, 192), (1, 64)):
        case = (f"pad{num}", num, 8, 2, 0.0, 0.001, 9, 2)
        counts, arrays = run_driver(dump_exe, tmp_path, case)
        total_strands, total_verts, n, guides, guide_verts, F = counts
        assert guides == want and n == 8 and F == 2
        assert total_strands == guides * 3 and total_verts == total_strands * 8 and guide_verts == guides * 8
        pos = arrays["positions"].reshape(total_strands, 8, 4)
        last = pos[(num - 1) * 3]
        for g in range(num, guides):
            assert np.array_equal(pos[g * 3], last)
        # follow hairs: root offsets carry the guide index in w, follow vertices keep the guide's w
        off = arrays["follow_root_offsets"].reshape(-1, 4)
        assert np.array_equal(off[::3, :3], np.zeros((guides, 3), np.float32))
        assert np.array_equal(off[:, 3], np.repeat(np.arange(guides) * 3, 3).astype(np.float32))
        assert np.array_equal(pos[1::3, :, 3], pos[0::3, :, 3])


def test_rest_lengths_and_triangles(dump_exe, tmp_path):
    case = ("rl", 64, 16, 0, 0.0, 0.0, 3, 0)
    counts, a = run_driver(dump_exe, tmp_path, case)
    pos = a["positions"].reshape(-1, 16, 4)
    rest = a["rest_lengths"].reshape(-1, 16)
    assert np.all(rest[:, -1] == 0)
    seg = np.linalg.norm((pos[:, :-1, :3] - pos[:, 1:, :3]).astype(np.float64), axis=2)
    assert np.allclose(rest[:, :-1], seg, rtol=1e-6)
    tri = a["triangle_indices"]
    assert len(tri) == 6 * counts[0] * 15
    assert list(tri[:6]) == [0, 1, 2, 2, 1, 3]


def test_bad_files_are_rejected(dump_exe, tmp_path):
    s = strands(10, 8, 1)
    old = tmp_path / "old.tfx"
    write_tfx(old, s, version=3.0)
    r = subprocess.run([str(dump_exe), str(old), "-", "0", "0", "0", "1", str(tmp_path / "o.bin")], capture_output=True)
    assert r.returncode == 3
    bad_n = tmp_path / "n5.tfx"
    write_tfx(bad_n, strands(10, 5, 1))
    r = subprocess.run([str(dump_exe), str(bad_n), "-", "0", "0", "0", "1", str(tmp_path / "o.bin")], capture_output=True)
    assert r.returncode == 3
    good = tmp_path / "good.tfx"
    write_tfx(good, s)
    bone = tmp_path / "many.tfxbone"
    write_tfxbone(bone, 200, 2, 1)   # more strands than the asset's 64 guides
    r = subprocess.run([str(dump_exe), str(good), str(bone), "0", "0", "0", "1", str(tmp_path / "o.bin")], capture_output=True)
    assert r.returncode == 4
