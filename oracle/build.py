"""Build recipe of the oracle library (test infrastructure): oracle/_build/libtfx_oracle.so.

g++ with -ffp-contract=off and no fast-math, so the FP32 restatement evaluates every expression
in the reference's order with IEEE rounding on both x86-64 and AArch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libtfx_oracle.so"
SRC = HERE / "tfx_oracle.cpp"


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if not force and OUT.exists() and OUT.stat().st_mtime >= max(SRC.stat().st_mtime, Path(__file__).stat().st_mtime):
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-Wall", "-o", str(tmp), str(SRC)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, force="-f" in sys.argv))
