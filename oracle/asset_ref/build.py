"""Test infrastructure: compiles the reference's asset pipeline (src/TressFX/TressFXAsset.cpp and
src/Math/Vector3D.cpp, where they lie in the reference tree) with the driver beside this file into
oracle/_ref/tfx_asset_ref.  Two shim headers, written into oracle/_ref/asset_shim/, stand in for
what the sources include but cannot build on Linux:

* ``Math\\\\Transform.h`` -- TressFXAsset.h:33 spells the include path with a Windows separator; the
  shim file carries that literal name and includes ``Math/Transform.h``;
* ``EngineInterface.h`` -- the real one pulls in the D3D12 / Vulkan backends; the asset code only uses
  EI_Read / EI_Seek (the reference's own stdio macros) and EI_Scene::GetBoneIdByName, plus the C
  string / stdlib declarations the Windows headers would have brought in.

Only the compiler runs here; nothing of the reference is copied into the repository.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
SHIM = OUT / "asset_shim"
EXE = OUT / "tfx_asset_ref"
REFERENCE = Path(os.environ.get("TFX_REFERENCE", "/root/reference"))

ENGINE_SHIM = """// shim: the part of the reference's EngineInterface.h the asset loader uses
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#define EI_Read(ptr, size, pFile) fread(ptr, size, 1, pFile)
#define EI_Seek(pFile, offset) fseek(pFile, offset, SEEK_SET)
class EI_Scene {
public:
    virtual ~EI_Scene() {}
    virtual int GetBoneIdByName(int skinNumber, const char* boneName) = 0;
};
"""


def available() -> bool:
    return (REFERENCE / "src" / "TressFX" / "TressFXAsset.cpp").exists()


def build(verbose: bool = False) -> Path | None:
    """Builds tfx_asset_ref if the reference tree is present; returns its path (None without it)."""
    srcs = [REFERENCE / "src" / "TressFX" / "TressFXAsset.cpp", REFERENCE / "src" / "Math" / "Vector3D.cpp",
            HERE / "asset_ref_driver.cpp"]
    if not available():
        return EXE if EXE.exists() else None
    if EXE.exists() and all(EXE.stat().st_mtime > s.stat().st_mtime for s in srcs + [Path(__file__)]):
        return EXE
    SHIM.mkdir(parents=True, exist_ok=True)
    (SHIM / "Math\\\\Transform.h").write_text('#include "Math/Transform.h"\n')
    (SHIM / "EngineInterface.h").write_text(ENGINE_SHIM)
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-w",
           f"-I{SHIM}", f"-I{REFERENCE / 'src'}", f"-I{REFERENCE / 'src' / 'TressFX'}",
           *map(str, srcs), "-o", str(EXE)]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the reference asset pipeline failed:\n{r.stderr[-4000:]}")
    return EXE


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
