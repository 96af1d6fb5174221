"""Recipe: the reference's compute shaders -> C++ translation units (test infrastructure).

Reads the reference's HLSL files where they lie and writes mechanically rewritten copies to
oracle/_ref/ (git-ignored build output, never committed).  Only syntax the C++ compiler cannot
accept is rewritten; every expression, statement and control-flow construct is kept as written.
The rewrites, in order:

  1. `[[vk::binding(..)]]`, `: register(..)`, `[numthreads(..)]` and `: SV_*` semantics removed;
  2. `cbuffer Name { ... }` unwrapped: its members become globals of the translation unit;
  3. `groupshared`, `row_major`, `column_major` removed (storage/packing qualifiers);
  4. `inout T x` / `out T x` parameters become `T& x`;
  5. un-suffixed floating literals get an `f` (HLSL literals take float type in float context);
  6. `float4x4 name[N];` constant-buffer arrays become `HArray<float4x4, N> name;` (the shaders
     index them with a float bone index);
  7. the scalar swizzle `sharedLength[i].x` on a float array reads `sharedLength[i]`;
  8. for TressFXBoneSkinning.hlsl only the compute part (up to the "// visualization" comment) is
     kept; the vertex/pixel shaders after it are rendering code;
  9. the strand expansion unit (ref_strands) is TressFXStrands.hlsl without its #include, preceded
     by what it uses from the other files: the TRESSFX_FLOAT_EPSILON define, MatrixMult and the two
     Safe_normalize overloads of TressFXUtilities.hlsl, and the cbuffer TressFXStrandParameters of
     TressFXRendering.hlsl; `.rgb` reads `.xyz` and `(TressFXVertex)0` value-initialises.
 10. for TressFXMarchingCubes.hlsl only the compute part between `//StartHLSL` and `//EndHLSL` is
     kept; the vertex/pixel shaders after it draw the mesh.

The output is wrapped in a namespace per shader file and compiled against hlsl_shim.h.
"""
from __future__ import annotations

import os
import re
import sys
from pathlib import Path

REF = Path(os.environ.get("TFX_REFERENCE", "/root/reference"))
SHADERS = {
    "ref_sim": "src/Shaders/TressFXSimulation.hlsl",
    "ref_sdf": "src/Shaders/TressFXSDFCollision.hlsl",
    "ref_skin": "src/Shaders/TressFXBoneSkinning.hlsl",
    "ref_strands": "src/Shaders/TressFXStrands.hlsl",
    "ref_mc": "src/Shaders/TressFXMarchingCubes.hlsl",
}


def _function(text: str, signature_re: str) -> str:
    """The full text (signature + body) of the first function whose signature matches."""
    m = re.search(signature_re, text)
    if not m:
        raise ValueError(f"function {signature_re} not found")
    j = text.index("{", m.end())
    depth, k = 1, j + 1
    while depth:
        depth += {"{": 1, "}": -1}.get(text[k], 0)
        k += 1
    return text[m.start():k]


def _strands_unit() -> str:
    util = (REF / "src/Shaders/TressFXUtilities.hlsl").read_text()
    rend = (REF / "src/Shaders/TressFXRendering.hlsl").read_text()
    strands = (REF / "src/Shaders/TressFXStrands.hlsl").read_text()
    eps = re.search(r"#define\s+TRESSFX_FLOAT_EPSILON[^\n]*", util).group(0)
    m = re.search(r"\[\[vk::binding[^\n]*\]\]\s*cbuffer\s+TressFXStrandParameters[^{]*\{", rend)
    cb = _function(rend[m.start():], r"cbuffer\s+TressFXStrandParameters")
    parts = [eps, cb, _function(util, r"float4\s+MatrixMult\s*\("),
             _function(util, r"float2\s+Safe_normalize\s*\(\s*float2"),
             _function(util, r"float3\s+Safe_normalize\s*\(\s*float3"),
             re.sub(r'#include\s+"[^"]+"', "", strands)]
    s = "\n\n".join(parts)
    s = s.replace(".rgb", ".xyz").replace("(TressFXVertex)0", "TressFXVertex()")
    return s


def _unwrap_cbuffers(s: str) -> str:
    out = []
    i = 0
    pat = re.compile(r"cbuffer\s+\w+\s*\{")
    while True:
        m = pat.search(s, i)
        if not m:
            out.append(s[i:])
            break
        out.append(s[i:m.start()])
        depth, j = 1, m.end()
        while depth:
            if s[j] == "{":
                depth += 1
            elif s[j] == "}":
                depth -= 1
            j += 1
        out.append(s[m.end():j - 1])
        i = j
    return "".join(out)


FLOAT_LIT = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def translate(text: str, name: str) -> str:
    s = text
    if name == "ref_skin":
        s = s.split("// visualization")[0]
    if name == "ref_mc":
        s = s.split("//StartHLSL TressFXMarchingCubesCS")[1].split("//EndHLSL")[0]
    s = re.sub(r"\[\[vk::binding\([^)]*\)\]\]", "", s)
    s = re.sub(r":\s*register\s*\([^)]*\)", "", s)
    s = re.sub(r"^\s*\[numthreads\([^)]*\)\]\s*$", "", s, flags=re.M)
    s = re.sub(r":\s*SV_\w+", "", s)
    s = _unwrap_cbuffers(s)
    s = re.sub(r"\b(groupshared|row_major|column_major)\b", "", s)
    s = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", s)
    s = re.sub(r"\bout\s+(\w+)\s+(\w+)", r"\1& \2", s)
    s = FLOAT_LIT.sub(lambda m: m.group(1) + "f", s)
    s = re.sub(r"\bfloat4x4\s+(\w+)\s*\[([^\]]+)\]\s*;", r"HArray<float4x4, \2> \1;", s)
    s = re.sub(r"(sharedLength\[[^\]]+\])\.x\b", r"\1", s)
    return f"// generated from {SHADERS[name]} by oracle/hlsl_ref/translate.py -- do not edit\n" \
           f"namespace {name} {{\n{s}\n}}  // namespace {name}\n"


def main(out_dir: Path) -> list[Path]:
    out_dir.mkdir(parents=True, exist_ok=True)
    written = []
    for name, rel in SHADERS.items():
        src = REF / rel
        if not src.exists():
            raise FileNotFoundError(src)
        dst = out_dir / f"{name}.inc"
        text = _strands_unit() if name == "ref_strands" else src.read_text()
        dst.write_text(translate(text, name))
        written.append(dst)
    return written


if __name__ == "__main__":
    print(main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent.parent / "_ref"))
