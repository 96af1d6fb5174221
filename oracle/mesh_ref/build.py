"""Builds oracle/_ref/tfx_mesh_ref from the reference's own source where it lies (see __init__)."""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref" / "mesh_ref"
EXE = ORACLE / "_ref" / "tfx_mesh_ref"
REFERENCE = Path(os.environ.get("TFX_REFERENCE", "/root/reference"))
SKINNING = REFERENCE / "src" / "TressFX" / "TressFXBoneSkinning.cpp"

# (first line of the cut, first line after it) in TressFXBoneSkinning.cpp
CUTS = [("int static SuStringTokenizer(", "bool TressFXBoneSkinning::LoadTressFXCollisionMeshData("),
        ("bool TressFXBoneSkinning::LoadTressFXCollisionMeshData(", "void TressFXBoneSkinning::Initialize(")]


def available() -> bool:
    return SKINNING.exists()


def extract() -> str:
    text = SKINNING.read_text(errors="replace")
    parts = []
    for first, after in CUTS:
        a = text.index(first)
        b = text.index(after, a)
        parts.append(f"// ---- cut from {SKINNING.name}, line {text.count(chr(10), 0, a) + 1}\n" + text[a:b])
    return "\n".join(parts)


def build(verbose: bool = False, force: bool = False) -> Path | None:
    """Compiles the executable if the reference tree is present; returns its path (None without either)."""
    if not available():
        return EXE if EXE.exists() else None
    from oracle.asset_ref.build import ENGINE_SHIM
    deps = [SKINNING, HERE / "driver.cpp", Path(__file__)]
    if not force and EXE.exists() and all(EXE.stat().st_mtime > d.stat().st_mtime for d in deps):
        return EXE
    OUT.mkdir(parents=True, exist_ok=True)
    (OUT / "bone_skinning_load.inc").write_text(extract())
    # TressFXAsset.h:33 spells its include with a Windows separator: a file of that literal name
    (OUT / "Math\\\\Transform.h").write_text('#include "Math/Transform.h"\n')
    (OUT / "EngineInterface.h").write_text(ENGINE_SHIM)
    tmp = EXE.with_suffix(".tmp")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-w", f"-I{OUT}",
           f"-I{REFERENCE / 'src'}", f"-I{REFERENCE / 'src' / 'TressFX'}", str(HERE / "driver.cpp"), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the reference mesh parser failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, EXE)
    return EXE


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
