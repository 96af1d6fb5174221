"""Builds oracle/_ref/libtfx_consts_ref.so from the reference's own source where it lies.

The functions SetWindCorner, TressFXHairObject::SetWind and TressFXHairObject::UpdateSimulationParameters
are cut out of src/TressFX/TressFXHairObject.cpp by their first lines and the first lines of the
functions after them, written unchanged to oracle/_ref/consts_ref/hair_object_consts.inc, and
compiled inside driver.cpp's stand-in class.  Nothing from the reference enters the repository.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref" / "consts_ref"
LIB = ORACLE / "_ref" / "libtfx_consts_ref.so"
REFERENCE = Path(os.environ.get("TFX_REFERENCE", "/root/reference"))
HAIR_OBJECT = REFERENCE / "src" / "TressFX" / "TressFXHairObject.cpp"
MATH = [REFERENCE / "src" / "Math" / f for f in ("Vector3D.cpp", "Quaternion.cpp", "Matrix33.cpp")]

# (first line of the cut, first line after it) in TressFXHairObject.cpp
CUTS = [("static void SetWindCorner(", "void TressFXHairObject::UpdatePerObjectRenderParams("),
        ("void TressFXHairObject::UpdateSimulationParameters(", "void TressFXHairObject::UpdateRenderingParameters(")]

SHIMS = {
    # Declarations only: TressFXConstantBuffers.h's uniform-buffer template names these engine types in
    # code that the cut functions never instantiate.
    "EngineInterface.h": """#pragma once
#include <memory>
class EI_Resource { public: virtual ~EI_Resource() {} };
enum EI_ResourceState { EI_STATE_UNDEFINED, EI_STATE_COPY_DEST = 3, EI_STATE_CONSTANT_BUFFER = 8 };
struct EI_Barrier { EI_Resource* pResource; EI_ResourceState from, to; };
enum { EI_BF_UNIFORMBUFFER = 4 };
class EI_CommandContext {
public:
    void SubmitBarrier(int count, EI_Barrier* barriers);
    void UpdateBuffer(EI_Resource* res, void* data);
};
class EI_Device {
public:
    std::unique_ptr<EI_Resource> CreateBufferResource(int structSize, int count, int flags, const char* name);
};
EI_Device* GetDevice();
""",
    # the settings header includes the UI library for its rendering settings
    "imgui.h": "#pragma once\n#include <string>\n",
}


def available() -> bool:
    return HAIR_OBJECT.exists() and all(m.exists() for m in MATH)


def extract() -> str:
    text = HAIR_OBJECT.read_text(errors="replace")
    parts = []
    for first, after in CUTS:
        a = text.index(first)
        b = text.index(after, a)
        parts.append(f"// ---- cut from {HAIR_OBJECT.name}, line {text.count(chr(10), 0, a) + 1}\n" + text[a:b])
    return "\n".join(parts)


def build(verbose: bool = False, force: bool = False) -> Path | None:
    """Compiles the library if the reference tree is present; returns its path (None without either)."""
    if not available():
        return LIB if LIB.exists() else None
    deps = [HAIR_OBJECT, *MATH, HERE / "driver.cpp", Path(__file__)]
    if not force and LIB.exists() and all(LIB.stat().st_mtime > d.stat().st_mtime for d in deps):
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    (OUT / "hair_object_consts.inc").write_text(extract())
    for name, body in SHIMS.items():
        (OUT / name).write_text(body)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-w", f"-I{OUT}", f"-I{REFERENCE / 'src'}", f"-I{REFERENCE / 'src' / 'TressFX'}",
           str(HERE / "driver.cpp"), *map(str, MATH), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the reference constant code failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
