"""Build the libraries in-tree: hos_gb300/libhos_gb300.so (CUDA, sm_103a) and
hos_gb300/libhos_ref.so (the reference's C++ function-level API over it).

Each .cu translation unit is compiled by nvcc in parallel and linked into one shared
library with the static CUDA runtime; the C++ API layer (refapi/*.cpp) is compiled by the
host C++ compiler and linked against libhos_gb300.so.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
INCLUDE = PKG.parent.parent / "include"
LIB = PKG / "libhos_gb300.so"
REF_LIB = PKG / "libhos_ref.so"
REFAPI = PKG.parent / "refapi"
BUILD_DIR = PKG.parent / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -prec-div/-prec-sqrt/-ftz only change single-precision arithmetic: the FP32-bulk kernels
# divide and take square roots with the fast hardware sequences; FP64 code is unaffected.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}",
              "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build hos_gb300")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _needs_build() -> bool:
    if not LIB.exists() or not REF_LIB.exists():
        return True
    t = min(LIB.stat().st_mtime, REF_LIB.stat().st_mtime)
    deps = list(CSRC.glob("*")) + list(REFAPI.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build_refapi() -> Path:
    """Compile the reference-API layer and link it against libhos_ref.so's CUDA library."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("a C++ compiler (g++) is required to build libhos_ref.so")
    tmp = REF_LIB.with_suffix(".so.tmp")
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", f"-I{INCLUDE}", *map(str, sorted(REFAPI.glob("*.cpp"))),
           "-o", str(tmp), f"-L{PKG}", "-lhos_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"libhos_ref.so build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, REF_LIB)
    return REF_LIB


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every .cu file for sm_103a and link libhos_gb300.so; returns its path."""
    if not force and not _needs_build():
        return LIB
    BUILD_DIR.mkdir(exist_ok=True)
    exe = nvcc()

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.stem + ".o")
        cmd = [exe, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_refapi()
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
