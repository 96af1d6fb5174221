"""Writes tests/golden/ratboy_subset.npz: a slice of the reference's shipped Ratboy asset (its mohawk
and the part of its body collision mesh around that slice), loaded by the reference's own code, for
the frame-parity tests that run where the reference tree is absent.

* Hair: 120 of the 2,228 mohawk guide strands (evenly strided over the file, so the slice spans the
  whole mohawk), written to a .tfx / .tfxbone pair and loaded by the reference's TressFXAsset
  (oracle/asset_ref, src/TressFX/TressFXAsset.cpp compiled here) with the sample's mohawk options:
  two follow hairs per guide, tip separation 2.0, radius 0.012 (src/TressFXSample.cpp:448-457,
  src/HairStrands.cpp:81).  The loader pads the 120 guides to 128.
* Bones: the sample maps bone names to engine ids through its glTF skeleton.  Here the union of the
  mohawk's and the body's bone names gets ids in order of first appearance (body first), and both
  files are rewritten with the name "b<id>" that the drivers' scene maps to <id>, so skinning keeps
  every real bone index and weight.
* Body: Ratboy_body.tfxmesh (renamed bones as above) through the reference's own .tfxmesh parser
  (oracle/mesh_ref), then the triangles with a corner within 4 cm of a vertex of the hair slice,
  re-indexed.  Follow bone: the sample's frenchHornMonster_root_JNT
  (src/TressFXSample.cpp:473-480).
* Hands: Ratboy_left_hand.tfxmesh and Ratboy_right_hand.tfxmesh whole (renamed bones as above), the
  sample's two further collision meshes (follow bones frenchHornMonster_L/R_LowerArm_JNT, 32 cells
  across, margin 0.5: src/TressFXSample.cpp:481-500).

The raw slice (guide positions, bone records, bone names) is kept too, so that a test can write the
same files again and check the library's own loader against the reference's output.

    python tests/golden/make_ratboy_golden.py
"""
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parent.parent))

from asset_cases import REAL_ASSET_DIR, digests  # noqa: E402
from asset_files import read_dump, read_mesh_dump, read_tfx_guides, read_tfxbone, write_tfx, \
    write_tfxbone_records  # noqa: E402
from oracle.asset_ref import build as asset_ref  # noqa: E402
import oracle.mesh_ref as mesh_ref  # noqa: E402

GUIDES = 120
FOLLOW, TIP, RADIUS, SEED = 2, 2.0, 0.012, 11
BODY_RADIUS = 0.04
FOLLOW_BONE = b"frenchHornMonster_root_JNT"
HANDS = (("left_hand", "Ratboy_left_hand.tfxmesh", b"frenchHornMonster_L_LowerArm_JNT"),
         ("right_hand", "Ratboy_right_hand.tfxmesh", b"frenchHornMonster_R_LowerArm_JNT"))


def mesh_bone_names(text: str) -> list[bytes]:
    lines = [ln.strip() for ln in text.splitlines()]
    i = next(k for k, ln in enumerate(lines) if ln.startswith("numOfBones"))
    nb = int(lines[i].split()[1])
    names, k = [], i + 1
    while len(names) < nb:
        if lines[k] and not lines[k].startswith("#"):
            names.append(lines[k].split()[1].encode())
        k += 1
    return names


def rename_mesh_bones(text: str, ids: dict[bytes, int]) -> str:
    out, lines = [], text.splitlines()
    i = next(k for k, ln in enumerate(lines) if ln.strip().startswith("numOfBones"))
    nb = int(lines[i].split()[1])
    out.extend(lines[:i + 1])
    k, seen = i + 1, 0
    while seen < nb:
        ln = lines[k]
        if ln.strip() and not ln.strip().startswith("#"):
            idx, name = ln.split()[:2]
            ln = f"{idx} b{ids[name.encode()]}"
            seen += 1
        out.append(ln)
        k += 1
    out.extend(lines[k:])
    return "\n".join(out) + "\n"


def main() -> None:
    exe = asset_ref.build()
    mexe = mesh_ref.build()
    if exe is None or mexe is None:
        raise SystemExit("the reference tree is not available")
    all_guides = read_tfx_guides(REAL_ASSET_DIR / "Ratboy_mohawk.tfx")
    hair_names, hair_bones, hair_weights = read_tfxbone(REAL_ASSET_DIR / "Ratboy_mohawk.tfxbone")
    body_text = (REAL_ASSET_DIR / "Ratboy_body.tfxmesh").read_text()
    body_names = mesh_bone_names(body_text)

    hand_texts = [(REAL_ASSET_DIR / f).read_text() for _, f, _ in HANDS]
    ids: dict[bytes, int] = {}
    for n in body_names + [h.rstrip(b"\0") for h in hair_names]:
        ids.setdefault(n, len(ids))
    for t in hand_texts:            # after the hair's and the body's, so their ids do not move
        for n in mesh_bone_names(t):
            ids.setdefault(n, len(ids))
    renamed_hair = [f"b{ids[h.rstrip(b'\0')]}".encode() + b"\0" for h in hair_names]

    rows = np.round(np.linspace(0, len(all_guides) - 1, GUIDES)).astype(np.int64)
    guides = all_guides[rows]
    bones, weights = hair_bones[rows], hair_weights[rows]

    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        write_tfx(d / "slice.tfx", guides)
        write_tfxbone_records(d / "slice.tfxbone", renamed_hair, bones, weights)
        import subprocess
        subprocess.run([str(exe), str(d / "slice.tfx"), str(d / "slice.tfxbone"), str(FOLLOW), repr(TIP), repr(RADIUS),
                        str(SEED), str(d / "hair.bin")], check=True, capture_output=True)
        counts, arrays = read_dump(d / "hair.bin")
        (d / "body.tfxmesh").write_text(rename_mesh_bones(body_text, ids))
        follow = f"b{ids[FOLLOW_BONE]}"
        subprocess.run([str(mexe), str(d / "body.tfxmesh"), follow, str(d / "body.bin")], check=True,
                       capture_output=True)
        mcounts, mesh = read_mesh_dump(d / "body.bin")
        hands = {}
        for (name, _, bone), text in zip(HANDS, hand_texts):
            (d / f"{name}.tfxmesh").write_text(rename_mesh_bones(text, ids))
            subprocess.run([str(mexe), str(d / f"{name}.tfxmesh"), f"b{ids[bone]}", str(d / f"{name}.bin")], check=True,
                           capture_output=True)
            hc, hm = read_mesh_dump(d / f"{name}.bin")
            hands[f"{name}_counts"] = hc
            hands[f"{name}_vertices"] = hm["bind_pose"].reshape(-1, 8)
            hands[f"{name}_indices"] = hm["indices"]
            hands[f"{name}_skinning"] = hm["skinning"].reshape(-1, 8)

    from scipy.spatial import cKDTree
    pos = arrays["positions"].reshape(-1, 4)[:, :3].astype(np.float64)
    verts = mesh["bind_pose"].reshape(-1, 8)
    tri = mesh["indices"].reshape(-1, 3)
    near = cKDTree(pos).query(verts[:, :3].astype(np.float64), distance_upper_bound=BODY_RADIUS)[0] < BODY_RADIUS
    keep = np.nonzero(near[tri].any(axis=1))[0]
    used = np.unique(tri[keep])
    remap = np.full(len(verts), -1, np.int64)
    remap[used] = np.arange(len(used))
    sub_tri = remap[tri[keep]].astype(np.uint32)

    # the reference's loader never writes the tangents' w (its value is whatever the allocation held);
    # the fixture takes 0 there, as the library's loader writes
    tangents = arrays["tangents"].reshape(-1, 4).copy()
    tangents[:, 3] = 0.0
    out = dict(
        guide_rows=rows.astype(np.int32), raw_guides=guides, raw_bones=bones.astype(np.int32),
        raw_weights=weights.astype(np.float32), raw_bone_names=np.array(renamed_hair, dtype=object).astype(bytes),
        counts=counts, positions=arrays["positions"], tangents=tangents.reshape(-1),
        follow_root_offsets=arrays["follow_root_offsets"], rest_lengths=arrays["rest_lengths"],
        bone_skinning=arrays["bone_skinning"],
        mesh_counts=mcounts, mesh_triangle_rows=keep.astype(np.int32), mesh_vertices=verts[used].copy(),
        mesh_indices=sub_tri.reshape(-1), mesh_skinning=mesh["skinning"].reshape(-1, 8)[used].copy(),
        num_bones=np.int32(len(ids)), follow_bone=np.int32(ids[FOLLOW_BONE]),
        options=np.array([FOLLOW, TIP, RADIUS, SEED], np.float64),
        loader_digests=np.array(json.dumps(digests(counts, arrays), sort_keys=True)),
        **hands,
    )
    np.savez_compressed(HERE / "ratboy_subset.npz", **out)
    print(f"hands {[int(hands[f'{n}_counts'][1]) for n, _, _ in HANDS]} triangles")
    print(f"hair {counts.tolist()}, body {len(keep)} of {len(tri)} triangles, {len(used)} vertices, "
          f"{len(ids)} bones, file {(HERE / 'ratboy_subset.npz').stat().st_size} bytes")


if __name__ == "__main__":
    main()
