"""Builds libbiwfa_gb300.so in-tree with nvcc for sm_103a (GB300).

Every translation unit is compiled in parallel with one -gencode, then linked as one
shared library with the CUDA runtime linked statically, so the library loads without a
GPU (the CPU test suite checks its exports) and needs nothing from site-packages.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
ROOT = PKG.parent
BUILD = ROOT / "_build" / "biwfa_gb300"
LIB = PKG / "libbiwfa_gb300.so"
CLI = PKG / "align_benchmark"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "-I", str(ROOT / "include"), "-I", str(CSRC)]
SOURCES = ["biwfa_kernel.cu", "wfg_runtime.cpp", "wfa2_compat.cpp", "datagen.cpp", "noalloc.cu", "mlp_kernel.cu",
           "wfg_model.cpp", "autotune.cpp",
           "sched_kernel.cu"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str) -> Path:
    out = BUILD / (Path(src).stem + ".o")
    srcp = CSRC / src
    deps = [srcp, CSRC / "wfg_internal.h", CSRC / "wfg_context.h", ROOT / "include" / "wfa_gpu.h"]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps if d.exists()):
        return out
    lang = [] if src.endswith(".cu") else ["-x", "cu"] if src.endswith("_kernel.cpp") else []
    cmd = [nvcc_path(), *ARCH, *NVCC_FLAGS, *lang, "-c", str(srcp), "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return out


def _build_cli() -> Path:
    """The align_benchmark-compatible CLI (csrc/align_benchmark.cpp), linked to the library."""
    src = CSRC / "align_benchmark.cpp"
    deps = [src, LIB, ROOT / "include" / "wfa_gpu.h"]
    if CLI.exists() and all(CLI.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return CLI
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for the align_benchmark CLI")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"), str(src), f"-L{PKG}", "-lbiwfa_gb300",
           "-Wl,-rpath,$ORIGIN", "-o", str(CLI)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"align_benchmark build failed:\n{res.stdout}\n{res.stderr}")
    return CLI


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if not (LIB.exists() and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs)):
        cmd = [nvcc_path(), *ARCH, "-shared", "-cudart", "static", "-o", str(LIB), *map(str, objs),
               "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    _build_cli()
    if verbose:
        print(f"built {LIB} and {CLI}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
