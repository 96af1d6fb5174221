"""The asset-pipeline cases shared by the CPU test and the golden-digest generator."""
from __future__ import annotations

import hashlib
import os
import subprocess
from pathlib import Path

import numpy as np

from asset_files import read_dump, read_mesh_dump, strands, write_tfx, write_tfxbone

ROOT = Path(__file__).resolve().parent.parent

# (name, guide strands in the file, vertices per strand, follow hairs, tip separation, radius, seed, bones)
CASES = [
    ("g100_n16_f0", 100, 16, 0, 0.0, 0.0, 1, 0),
    ("g100_n16_f3", 100, 16, 3, 0.5, 0.002, 2, 3),
    ("g128_n8_f2", 128, 8, 2, 1.0, 0.004, 3, 5),
    ("g70_n32_f1", 70, 32, 1, 0.0, 0.012, 4, 2),
    ("g3_n4_f4", 3, 4, 4, 0.25, 0.001, 5, 1),
]


def write_case_files(tmp: Path, case) -> tuple[Path, str]:
    name, num, n, F, tip, radius, seed, bones = case
    tfx = tmp / f"{name}.tfx"
    write_tfx(tfx, strands(num, n, seed))
    bone = "-"
    if bones:
        p = tmp / f"{name}.tfxbone"
        write_tfxbone(p, num, bones, seed + 100)
        bone = str(p)
    return tfx, bone


def run_driver(exe: Path, tmp: Path, case) -> tuple[np.ndarray, dict[str, np.ndarray]]:
    name, num, n, F, tip, radius, seed, bones = case
    tfx, bone = write_case_files(tmp, case)
    out = tmp / f"{name}.{exe.name}.bin"
    env = dict(os.environ)
    subprocess.run([str(exe), str(tfx), bone, str(F), repr(tip), repr(radius), str(seed), str(out)], check=True, env=env,
                   capture_output=True)
    return read_dump(out)


def digests(counts: np.ndarray, arrays: dict[str, np.ndarray]) -> dict[str, str]:
    """SHA-256 per array; the w of the tangents is left out (the reference never sets it)."""
    out = {"counts": hashlib.sha256(counts.tobytes()).hexdigest()}
    for k, v in arrays.items():
        if k == "tangents":
            v = v.reshape(-1, 4)[:, :3].copy()
        out[k] = hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()
    return out


def build_asset_dump(tmp: Path) -> Path:
    """Compiles tests/cpp/asset_dump.cpp against libtressfx_host.so."""
    exe = tmp / "asset_dump"
    pkg = ROOT / "tressfx_gb300"
    subprocess.run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "asset_dump.cpp"), "-o", str(exe), f"-L{pkg}", "-ltressfx_host",
                    "-ltfxgb300", f"-Wl,-rpath,{pkg}"], check=True, capture_output=True)
    return exe


def build_mesh_dump(tmp: Path) -> Path:
    """Compiles tests/cpp/mesh_dump.cpp against libtressfx_host.so."""
    exe = tmp / "mesh_dump"
    pkg = ROOT / "tressfx_gb300"
    subprocess.run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "mesh_dump.cpp"), "-o", str(exe), f"-L{pkg}", "-ltressfx_host",
                    "-ltfxgb300", f"-Wl,-rpath,{pkg}"], check=True, capture_output=True)
    return exe


def run_mesh_driver(exe: Path, tmp: Path, mesh: Path, follow_bone: str = "b0") -> tuple[np.ndarray, dict[str, np.ndarray]]:
    out = tmp / f"{mesh.stem}.{exe.name}.bin"
    subprocess.run([str(exe), str(mesh), follow_bone, str(out)], check=True, capture_output=True)
    return read_mesh_dump(out)


# The reference's shipped asset (bin/Objects/HairAsset/Ratboy), where the reference tree is present.
REAL_ASSET_DIR = Path(os.environ.get("TFX_REFERENCE", "/root/reference")) / "bin" / "Objects" / "HairAsset" / "Ratboy"
# (name, .tfx, .tfxbone, follow hairs, tip separation, radius, seed)
REAL_HAIR = ("ratboy_mohawk_f4", "Ratboy_mohawk.tfx", "Ratboy_mohawk.tfxbone", 4, 0.5, 0.012, 7)
REAL_MESHES = ("Ratboy_body.tfxmesh", "Ratboy_left_hand.tfxmesh", "Ratboy_right_hand.tfxmesh")


def run_real_hair(exe: Path, tmp: Path) -> tuple[np.ndarray, dict[str, np.ndarray]]:
    name, tfx, bone, F, tip, radius, seed = REAL_HAIR
    out = tmp / f"{name}.{exe.name}.bin"
    subprocess.run([str(exe), str(REAL_ASSET_DIR / tfx), str(REAL_ASSET_DIR / bone), str(F), repr(tip), repr(radius),
                    str(seed), str(out)], check=True, capture_output=True)
    return read_dump(out)


def mesh_digests(counts: np.ndarray, arrays: dict[str, np.ndarray]) -> dict[str, str]:
    out = {"counts": hashlib.sha256(counts.tobytes()).hexdigest()}
    for k, v in arrays.items():
        out[k] = hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()
    return out
