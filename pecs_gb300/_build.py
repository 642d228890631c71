"""Builds libpecs_gb300.so (CUDA kernels + C++ host code + C ABI) in-tree.

Compiles every translation unit in parallel for sm_103a only and links a
shared library next to this file (pecs_gb300/_lib/).  No cmake, no torch
extension machinery: the product is a plain C-ABI library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIBDIR = HERE / "_lib"
LIB = LIBDIR / "libpecs_gb300.so"
INCLUDE = HERE.parent / "include"

CUDA_SOURCES = ["engine.cu", "solve.cu", "nn.cu", "front.cu"]
CXX_SOURCES = ["problem.cpp", "mf.cpp", "dense.cpp", "scaling.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources_newer_than(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link the library if any source changed; returns its path."""
    if not force and not _sources_newer_than(LIB):
        return LIB
    nvcc = _nvcc()
    obj = LIBDIR / "obj"
    obj.mkdir(parents=True, exist_ok=True)
    common = ["-O3", "-std=c++17", f"-I{INCLUDE}"]
    # host arithmetic without fused multiply-adds: g++ fuses a*b+c by default
    # in C++ on aarch64 but cannot on x86-64 without -mfma, so the host setup
    # (matrices, factors, constant right-hand sides) would round differently
    # on the two
    host = "-ffp-contract=off"
    cmds = []
    for src in CUDA_SOURCES:
        o = obj / (src + ".o")
        cmds.append([nvcc, *ARCH, *common, "-lineinfo", "-Xcompiler", f"-fPIC,{host}", "-c",
                     str(CSRC / src), "-o", str(o)])
    for src in CXX_SOURCES:
        o = obj / (src + ".o")
        cmds.append(["g++", *common, host, "-fPIC", "-c", str(CSRC / src), "-o", str(o)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(" ".join(cmd))
        return r

    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(run, cmds))
    objs = [str(obj / (s + ".o")) for s in CUDA_SOURCES + CXX_SOURCES]
    tmp = LIB.with_suffix(".so.tmp")
    run([nvcc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcublas", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
