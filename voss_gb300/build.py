"""Build ``libvoss.so`` in-tree with nvcc for sm_103a.

    python voss_gb300/build.py [--force]

Translation units compile in parallel; the link uses the shared CUDA runtime
so that the library and PyTorch share one runtime (one current device, one
set of streams).  Outputs: ``voss_gb300/libvoss.so`` and object files under
``voss_gb300/_build/`` (both git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libvoss.so"
SOURCES = ["sieve.cu", "goldbach.cu", "probe.cu", "noalloc.cu", "engine.cpp", "serve.cpp", "capi.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def cuda_lib_dir() -> str:
    return str(Path(nvcc()).resolve().parent.parent / "lib64")


def _flags() -> list[str]:
    # -ffp-contract=off: host doubles (gap moments) must not be fused into FMAs,
    # which g++ does by default on aarch64 but not on x86; the reference's
    # statistics are plain multiply-then-add.
    return ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-Wall,-ffp-contract=off",
            "-I", str(ROOT / "include"), "-I", str(CSRC)]


def _newest_input() -> float:
    files = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + \
        list(CSRC.glob("*.inc")) + list((ROOT / "include" / "voss").glob("*.h")) + [Path(__file__)]
    return max(f.stat().st_mtime for f in files)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= _newest_input():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> Path:
        obj = BUILD / (src + ".o")
        cmd = [cc, *_flags(), "-c", str(CSRC / src), "-o", str(obj)]
        if src.endswith(".cpp"):
            cmd.insert(1, "-x")
            cmd.insert(2, "cu")
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_name("libvoss.so.tmp%d" % os.getpid())
    link = [cc, *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs), "-lpthread",
            "-Xlinker", "-rpath," + cuda_lib_dir()]
    if verbose:
        print(" ".join(link), flush=True)
    subprocess.run(link, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    print(p)
