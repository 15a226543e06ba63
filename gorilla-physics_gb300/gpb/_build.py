"""Builds libgpb.so (CUDA kernels for sm_103a + the C++ host library) in place.

Each translation unit is compiled in parallel with nvcc and linked into
``gpb/libgpb.so`` next to this file.  Objects go to ``gpb/_build/``.  No cmake:
the build must finish in a minute or two on both the x86 development host and
the Arm GPU host.
"""

from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent            # gorilla-physics_gb300/
CSRC = ROOT / "csrc"
REPO = ROOT.parent
INCLUDE = REPO / "include"
LIB = PKG / "libgpb.so"
OBJ = PKG / "_build"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")

SOURCES = ["gpb_kernels.cu", "gpb_host.cpp", "gpb_serve.cpp", "gpb_configs.cpp", "gpb_peaks.cu"]


def _compile(src: str, extra: list[str]) -> Path:
    out = OBJ / (src + ".o")
    cmd = [NVCC, "-std=c++17", "-O3", ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
           "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(CSRC / src), "-o", str(out)]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    cmd += extra
    subprocess.run(cmd, check=True)
    return out


def needs_build() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [INCLUDE / "gpb.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, extra: list[str] | None = None, verbose: bool = False) -> Path:
    """Compiles every source for sm_103a and links libgpb.so; returns its path."""
    if not force and not needs_build():
        return LIB
    OBJ.mkdir(exist_ok=True)
    extra = list(extra or [])
    if verbose:
        extra += ["-Xptxas", "-v"]
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([NVCC, "-shared", ARCH, "-o", str(tmp), *map(str, objs),
                    "-L", str(CUDA_HOME / "lib64"), "-lcudart",
                    "-Xlinker", "-rpath=" + str(CUDA_HOME / "lib64")], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
