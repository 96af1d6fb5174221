"""Synthetic .tfx / .tfxbone / .tfxmesh files for the asset-pipeline tests, in the reference's
formats (src/TressFX/TressFXFileFormat.h:35-61, TressFXAsset.cpp:401-480,
TressFXBoneSkinning.cpp:100-285), and readers of the asset dumps both drivers write."""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

ARRAYS = ("positions", "strand_uv", "tangents", "follow_root_offsets", "strand_types", "thickness", "rest_lengths",
          "triangle_indices", "bone_skinning")
DTYPES = (np.float32, np.float32, np.float32, np.float32, np.int32, np.float32, np.float32, np.int32, np.float32)


def strands(num: int, n: int, seed: int) -> np.ndarray:
    """[num, n, 4] random-walk strands (w = 0 for the first two vertices, else 1)."""
    rng = np.random.default_rng(seed)
    roots = rng.normal(size=(num, 3))
    roots = 0.1 * roots / np.linalg.norm(roots, axis=1, keepdims=True)
    out = np.zeros((num, n, 4), np.float32)
    d = roots / np.linalg.norm(roots, axis=1, keepdims=True)
    p = roots.copy()
    for j in range(n):
        out[:, j, :3] = p
        out[:, j, 3] = 0.0 if j < 2 else 1.0
        d = d + 0.3 * rng.normal(size=d.shape)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        p = p + 0.008 * d
    return out


def write_tfx(path: Path, s: np.ndarray, version: float = 4.0) -> None:
    num, n, _ = s.shape
    header_size = 4 * 8 + 4 * 32
    off_pos = header_size
    off_uv = off_pos + s.nbytes
    uv = np.stack([np.linspace(0, 1, num), np.linspace(1, 0, num)], 1).astype(np.float32)
    hdr = struct.pack("<fIIIIIII", version, num, n, off_pos, off_uv, 0, 0, 0) + b"\0" * (4 * 32)
    path.write_bytes(hdr + s.astype(np.float32).tobytes() + uv.tobytes())


def write_tfxbone(path: Path, num_strands: int, num_bones: int, seed: int) -> None:
    rng = np.random.default_rng(seed)
    buf = struct.pack("<i", num_bones)
    for b in range(num_bones):
        name = f"b{b}".encode() + b"\0"
        buf += struct.pack("<ii", b, len(name)) + name
    buf += struct.pack("<i", num_strands)
    for i in range(num_strands):
        idx = rng.integers(0, num_bones, 4)
        w = rng.random(4).astype(np.float32)
        w[0] += 0.1
        w[rng.random(4) < 0.3] = 0.0
        w[0] = max(w[0], 0.05)
        buf += struct.pack("<i", i)
        for k in range(4):
            buf += struct.pack("<if", int(idx[k]), float(w[k]))
    path.write_bytes(buf)


def write_tfxmesh(path: Path, vertices: np.ndarray, indices: np.ndarray, skinning: np.ndarray, num_bones: int) -> None:
    """vertices [V, 8] (pos.xyzw, normal.xyzw), indices [3T], skinning [V, 8] (bone ids, weights)."""
    lines = ["# TressFX collision mesh", f"numOfBones {num_bones}"]
    lines += [f"{b} b{b}" for b in range(num_bones)]
    lines.append("# vertex index, position, normal, bone indices, weights")
    lines.append(f"numOfVertices {len(vertices)}")
    for i, (v, s) in enumerate(zip(vertices, skinning)):
        vals = [f"{x:.9g}" for x in (*v[:3], *v[4:7])] + [str(int(b)) for b in s[:4]] + [f"{x:.9g}" for x in s[4:]]
        lines.append(" ".join([str(i)] + vals))
    tri = np.asarray(indices).reshape(-1, 3)
    lines.append(f"numOfTriangles {len(tri)}")
    lines += [f"{t} {a} {b} {c}" for t, (a, b, c) in enumerate(tri)]
    path.write_text("\n".join(lines) + "\n")


def read_dump(path: Path) -> tuple[np.ndarray, dict[str, np.ndarray]]:
    raw = path.read_bytes()
    counts = np.frombuffer(raw[:24], np.int32).copy()
    pos = 24
    out = {}
    for name, dt in zip(ARRAYS, DTYPES):
        (nb,) = struct.unpack_from("<Q", raw, pos)
        pos += 8
        out[name] = np.frombuffer(raw[pos:pos + nb], dt).copy()
        pos += nb
    return counts, out


def read_mesh_dump(path: Path) -> tuple[np.ndarray, dict[str, np.ndarray]]:
    """(vertex count, triangle count, follow bone) and the bind pose, indices and skinning a mesh
    dump holds (tests/cpp/mesh_dump.cpp, oracle/mesh_ref/driver.cpp)."""
    raw = path.read_bytes()
    counts = np.frombuffer(raw[:12], np.int32).copy()
    pos = 12
    out = {}
    for name, dt in (("bind_pose", np.float32), ("indices", np.uint32), ("skinning", np.float32)):
        (nb,) = struct.unpack_from("<Q", raw, pos)
        pos += 8
        out[name] = np.frombuffer(raw[pos:pos + nb], dt).copy()
        pos += nb
    return counts, out


def read_tfx_guides(path: Path) -> np.ndarray:
    """The guide strands [num, n, 4] of a .tfx file (TressFXAsset.cpp:401-440 reads the same header)."""
    raw = path.read_bytes()
    _, num, n, off_pos = struct.unpack_from("<fIII", raw, 0)
    return np.frombuffer(raw, np.float32, num * n * 4, off_pos).reshape(num, n, 4).copy()


def read_tfxbone(path: Path) -> tuple[list[bytes], np.ndarray, np.ndarray]:
    """Bone names (with their NUL) and per-strand (bone index [S, 4], weight [S, 4]) of a .tfxbone file
    (TressFXAsset.cpp:442-480 reads the same layout)."""
    raw = path.read_bytes()
    (nb,) = struct.unpack_from("<i", raw, 0)
    pos = 4
    names = []
    for _ in range(nb):
        _, ln = struct.unpack_from("<ii", raw, pos)
        pos += 8
        names.append(raw[pos:pos + ln])
        pos += ln
    (ns,) = struct.unpack_from("<i", raw, pos)
    pos += 4
    rec = np.frombuffer(raw, np.dtype([("strand", "<i4"), ("pairs", [("bone", "<i4"), ("weight", "<f4")], 4)]), ns, pos)
    return names, rec["pairs"]["bone"].copy(), rec["pairs"]["weight"].copy()


def write_tfxbone_records(path: Path, names: list[bytes], bones: np.ndarray, weights: np.ndarray) -> None:
    """A .tfxbone file with the given bone names and per-strand (bone index, weight) records."""
    buf = struct.pack("<i", len(names))
    for b, name in enumerate(names):
        buf += struct.pack("<ii", b, len(name)) + name
    buf += struct.pack("<i", len(bones))
    for i in range(len(bones)):
        buf += struct.pack("<i", i)
        for k in range(4):
            buf += struct.pack("<if", int(bones[i, k]), float(weights[i, k]))
    path.write_bytes(buf)
