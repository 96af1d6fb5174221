"""The C++ TressFXAsset and TressFXBoneSkinning of libtressfx_host (.tfx / .tfxbone / .tfxmesh
loading, GenerateFollowHairs, ProcessAsset) against the reference's own TressFXAsset.cpp and .tfxmesh
parser: array for array, bit for bit.

Where the reference tree is present its asset code is compiled and run beside ours (oracle/asset_ref,
oracle/mesh_ref), on synthetic files and on the reference's shipped Ratboy asset; ours is also checked
against the committed digests of the reference's output (tests/golden/asset_digests.json)."""
import json
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from asset_cases import CASES, REAL_ASSET_DIR, REAL_HAIR, REAL_MESHES, build_asset_dump, build_mesh_dump, \
    digests, mesh_digests, run_driver, run_mesh_driver, run_real_hair, write_case_files
from asset_files import read_dump, strands, write_tfx, write_tfxbone, write_tfxmesh

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


@pytest.fixture(scope="module")
def mesh_dump_exe(built_lib, tmp_path_factory):
    return build_mesh_dump(tmp_path_factory.mktemp("mesh_dump"))


@pytest.fixture(scope="module")
def mesh_ref_exe():
    import oracle.mesh_ref as mesh_ref
    try:
        return mesh_ref.build()
    except RuntimeError as e:  # pragma: no cover
        pytest.skip(f"reference mesh parser not buildable: {e}")


def _same(a: dict, b: dict) -> None:
    for k in a:
        x, y = a[k], b[k]
        if k == "tangents":   # w is never set by the reference
            x, y = x.reshape(-1, 4)[:, :3], y.reshape(-1, 4)[:, :3]
        assert x.shape == y.shape and np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                                                     y.view(np.uint32) if y.dtype == np.float32 else y), k


def test_real_ratboy_mohawk(dump_exe, ref_exe, tmp_path):
    """The reference's shipped hair asset (2,228 strands of 32 vertices, padded to 2,240 guides, four
    follow hairs each) through both loaders, and against the committed digests."""
    if not (REAL_ASSET_DIR / REAL_HAIR[1]).exists():
        pytest.skip("the reference's shipped asset is not present here")
    counts, arrays = run_real_hair(dump_exe, tmp_path)
    assert list(counts) == [11200, 358400, 32, 2240, 71680, 4]
    want = json.loads((HERE / "golden" / "asset_digests.json").read_text())[REAL_HAIR[0]]
    assert digests(counts, arrays) == want
    if ref_exe is not None:
        c2, a2 = run_real_hair(ref_exe, tmp_path)
        assert np.array_equal(counts, c2)
        _same(arrays, a2)


@pytest.mark.parametrize("mesh", REAL_MESHES)
def test_real_ratboy_collision_meshes(mesh_dump_exe, mesh_ref_exe, tmp_path, mesh):
    """The reference's shipped collision meshes (the body: 12,909 vertices, 25,814 triangles, 86 bones)
    through both .tfxmesh parsers, and against the committed digests."""
    if not (REAL_ASSET_DIR / mesh).exists():
        pytest.skip("the reference's shipped asset is not present here")
    counts, arrays = run_mesh_driver(mesh_dump_exe, tmp_path, REAL_ASSET_DIR / mesh)
    want = json.loads((HERE / "golden" / "asset_digests.json").read_text())[mesh]
    assert mesh_digests(counts, arrays) == want
    if mesh == "Ratboy_body.tfxmesh":
        assert list(counts[:2]) == [12909, 25814]
    if mesh_ref_exe is not None:
        c2, a2 = run_mesh_driver(mesh_ref_exe, tmp_path, REAL_ASSET_DIR / mesh)
        assert np.array_equal(counts, c2)
        _same(arrays, a2)


def test_tfxmesh_parsers_agree_on_synthetic_files(mesh_dump_exe, mesh_ref_exe, tmp_path):
    """A synthetic .tfxmesh with comments, blank lines and bone names the scene maps to ids."""
    if mesh_ref_exe is None:
        pytest.skip("reference tree not present")
    rng = np.random.default_rng(12)
    V, T = 300, 500
    verts = np.zeros((V, 8), np.float32)
    verts[:, :3] = rng.normal(size=(V, 3))
    verts[:, 4:7] = rng.normal(size=(V, 3))
    skin = np.zeros((V, 8), np.float32)
    skin[:, :4] = rng.integers(0, 5, (V, 4))
    skin[:, 4:] = rng.dirichlet(np.ones(4), V)
    idx = rng.integers(0, V, 3 * T).astype(np.uint32)
    path = tmp_path / "synthetic.tfxmesh"
    write_tfxmesh(path, verts, idx, skin, 5)
    text = path.read_text().replace("numOfVertices", "\n# a comment\n\nnumOfVertices", 1)
    path.write_text(text)
    c1, a1 = run_mesh_driver(mesh_dump_exe, tmp_path, path, "b3")
    c2, a2 = run_mesh_driver(mesh_ref_exe, tmp_path, path, "b3")
    assert np.array_equal(c1, c2) and c1[2] == 3
    _same(a1, a2)


def test_ratboy_slice_through_library_loader(dump_exe, tmp_path):
    """The slice of the shipped mohawk kept in tests/golden/ratboy_subset.npz (120 guides, real bone
    records) written back to a .tfx / .tfxbone pair and loaded by the library: every array matches what
    the reference's TressFXAsset produced from the same files (the fixture's arrays and digests)."""
    from asset_files import write_tfxbone_records
    with np.load(HERE / "golden" / "ratboy_subset.npz", allow_pickle=False) as z:
        f = {k: z[k] for k in z.files}
    F, tip, radius, seed = f["options"]
    write_tfx(tmp_path / "slice.tfx", f["raw_guides"])
    names = [bytes(x) + b"\0" for x in f["raw_bone_names"]]
    write_tfxbone_records(tmp_path / "slice.tfxbone", names, f["raw_bones"], f["raw_weights"])
    out = tmp_path / "slice.bin"
    subprocess.run([str(dump_exe), str(tmp_path / "slice.tfx"), str(tmp_path / "slice.tfxbone"), str(int(F)), repr(float(tip)),
                    repr(float(radius)), str(int(seed)), str(out)], check=True, capture_output=True)
    counts, arrays = read_dump(out)
    assert np.array_equal(counts, f["counts"])
    assert digests(counts, arrays) == json.loads(str(f["loader_digests"]))
    for k in ("positions", "follow_root_offsets", "rest_lengths", "bone_skinning"):
        assert np.array_equal(arrays[k].view(np.uint32), f[k].view(np.uint32)), k
