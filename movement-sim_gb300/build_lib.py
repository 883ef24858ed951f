"""Build recipe for libmsim.so (the CUDA kernels + C ABI + C++ host code).

Compiles every translation unit under csrc/ in parallel (nvcc for .cu, g++ for
.cpp) for sm_103a only and links the shared library in place, next to this
file.  Re-running is cheap: objects newer than their sources and headers are
reused.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libmsim.so"

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [GENCODE, "-lineinfo", "-O3", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-I", str(ROOT / "include"), "-I", str(CSRC)]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-ffp-contract=off",
             "-I", str(ROOT / "include"), "-I", str(CSRC)]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmsim")


def _cuda_include(nvcc: str) -> str:
    return str(Path(nvcc).resolve().parent.parent / "include")


def _deps() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps, Path(__file__)])


def build(verbose: bool = False, extra_nvcc: list[str] | None = None) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    deps = _deps()
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if not _stale(obj, src, deps):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, *NVCC_FLAGS, *(extra_nvcc or []), "-c", str(src), "-o", str(obj)]
        else:
            cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-I", _cuda_include(nvcc), "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        jobs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, proc in jobs:
        out, _ = proc.communicate()
        if proc.returncode != 0:
            failed.append(f"--- {src.name} ---\n{out}")
        elif verbose and out.strip():
            print(out)
    if failed:
        raise RuntimeError("libmsim build failed:\n" + "\n".join(failed))
    if jobs or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, GENCODE, "-shared", "-o", str(tmp), *map(str, objs)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if res.returncode != 0:
            raise RuntimeError("libmsim link failed:\n" + res.stdout)
        os.replace(tmp, LIB)
    build_examples(verbose)
    return LIB


def build_examples(verbose: bool = False) -> None:
    """Host-only C++ programs over the façade (examples/*.cpp), linked to libmsim.so."""
    for src in sorted((PKG / "examples").glob("*.cpp")):
        exe = PKG / "examples" / src.stem
        deps = [src, LIB, *(ROOT / "include").glob("*.hpp"), *(ROOT / "include").glob("*.h")]
        if exe.exists() and all(exe.stat().st_mtime >= d.stat().st_mtime for d in deps):
            continue
        cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"), str(src),
               "-L", str(PKG), "-lmsim", f"-Wl,-rpath,{PKG}", "-pthread", "-o", str(exe)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"example {src.name} failed to build:\n" + res.stdout)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
