"""Build recipe for the oracle (test infrastructure only).

* oracle/liboracle.so  - the C restatement in msim_oracle.c (gcc, no FMA contraction)
* oracle/_ref/libref_quadtree.so - the reference's own CPU quad tree
  (shader_validation/src/main.cpp of COM8/movement-sim) compiled where it lies
  through ref_harness.cpp; built only when the reference tree is present.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libref_quadtree.so"
REFERENCE_ROOT = Path(os.environ.get("MSIM_REFERENCE_ROOT", "/root/reference"))

CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-Wall"]


def _newer(out: Path, *srcs: Path) -> bool:
    return out.exists() and all(out.stat().st_mtime >= s.stat().st_mtime for s in srcs)


def build_oracle() -> Path:
    src = HERE / "msim_oracle.c"
    if _newer(LIB, src, HERE / "msim_oracle.h", Path(__file__)):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CC", "gcc"), *CFLAGS, str(src), "-o", str(tmp), "-lm"]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout)
    os.replace(tmp, LIB)
    return LIB


def build_reference() -> Path | None:
    """Compile the reference's CPU quad tree; None when the reference is absent."""
    ref_src = REFERENCE_ROOT / "shader_validation" / "src" / "main.cpp"
    if not ref_src.exists():
        return None
    harness = HERE / "ref_harness.cpp"
    if _newer(REF_LIB, harness, ref_src, Path(__file__)):
        return REF_LIB
    REF_DIR.mkdir(exist_ok=True)
    tmp = REF_LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
           "-w", "-I", str(ref_src.parent), str(harness), "-o", str(tmp)]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference quad-tree build failed:\n" + res.stdout)
    os.replace(tmp, REF_LIB)
    return REF_LIB


def build() -> None:
    build_oracle()
    build_reference()


if __name__ == "__main__":
    build()
    print(LIB, REF_LIB if REF_LIB.exists() else "(reference absent)", file=sys.stderr)
