"""Build of the CUDA library (libtfxgb300.so) for sm_103a, in tree.

Every translation unit is compiled in parallel with nvcc (CUDA sources) or g++ (host-only C++),
then linked into ``tressfx_gb300/libtfxgb300.so``.  Floating-point flags are part of the product
contract: no FMA contraction (``-fmad=false`` on the device, ``-ffp-contract=off`` on the host),
IEEE division and square root, no flush-to-zero, so the kernels reproduce the reference
arithmetic order exactly.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD_DIR = PKG / "_build"
LIB_PATH = PKG / "libtfxgb300.so"
HOST_DIR = PKG / "host"
HOST_LIB_PATH = PKG / "libtressfx_host.so"   # the C++ host classes (include/tressfx/*.h)

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def nvcc_flags() -> list[str]:
    return [
        "-std=c++17", "-O3", "-lineinfo", ARCH,
        "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
        "--expt-relaxed-constexpr",
        f"-I{ROOT / 'include'}", f"-I{CSRC}",
    ]


def cxx_flags(cuda: Path) -> list[str]:
    return ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
            f"-I{ROOT / 'include'}", f"-I{CSRC}", f"-I{cuda / 'include'}"]


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout.strip() or r.stderr.strip()):
        print(r.stdout, r.stderr, sep="", flush=True)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every CUDA / C++ source of the library and link libtfxgb300.so. Returns its path."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD_DIR.mkdir(exist_ok=True)
    headers = _headers()
    jobs = []
    objects = []
    for src in _sources():
        obj = BUILD_DIR / (src.name + ".o")
        objects.append(obj)
        if not force and not _stale(obj, [src] + headers + [Path(__file__)]):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, *nvcc_flags(), "-c", str(src), "-o", str(obj)]
        else:
            cmd = [os.environ.get("CXX", "g++"), *cxx_flags(cuda), "-c", str(src), "-o", str(obj)]
        jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or jobs or _stale(LIB_PATH, objects):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        _run([nvcc, "-shared", ARCH, "-o", str(tmp), *map(str, objects), "-lpthread", "-ldl", "-lrt"], verbose)
        os.replace(tmp, LIB_PATH)
    build_host(verbose, force)
    return LIB_PATH


def host_sources() -> list[Path]:
    return sorted(HOST_DIR.glob("*.cpp"))


def build_host(verbose: bool = False, force: bool = False) -> Path:
    """Compile the C++ host classes into libtressfx_host.so, linked against libtfxgb300.so."""
    srcs = host_sources()
    deps = srcs + sorted(HOST_DIR.glob("*.h")) + sorted((ROOT / "include" / "tressfx").glob("*.h")) + \
        [ROOT / "include" / "tressfx_gb300.h", LIB_PATH, Path(__file__)]
    if not force and not _stale(HOST_LIB_PATH, deps):
        return HOST_LIB_PATH
    tmp = HOST_LIB_PATH.with_suffix(".so.tmp")
    _run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
          "-Wall", f"-I{ROOT / 'include'}", f"-I{HOST_DIR}", *map(str, srcs), "-o", str(tmp),
          f"-L{PKG}", "-ltfxgb300", "-Wl,-rpath,$ORIGIN"], verbose)
    os.replace(tmp, HOST_LIB_PATH)
    return HOST_LIB_PATH


if __name__ == "__main__":
    p = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(p)
