"""The library's host-side C++ (map loader, writer and validator, lattice generator,
reference-layout quad tree) built with AddressSanitizer and
UndefinedBehaviorSanitizer and driven by tests/cpp/host_sanitize.cpp: round trips,
rejected bad maps, truncated and mutated JSON.  The reference ships sanitizer build
types for its own C++ (cmake/sanitizer.cmake); this is the counterpart for the
host code here.  CPU only."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "movement-sim_gb300" / "csrc"


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return str(Path(nvcc).resolve().parent.parent / "include")


def test_host_code_under_asan_ubsan(tmp_path):
    exe = tmp_path / "host_sanitize"
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-ffp-contract=off", "-I", str(ROOT / "include"), "-I", str(CSRC),
           "-I", _cuda_include(), str(ROOT / "tests" / "cpp" / "host_sanitize.cpp"), str(CSRC / "msim_map.cpp"),
           str(CSRC / "msim_quadtree.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and ("asan" in r.stderr.lower() or "ubsan" in r.stderr.lower()):
        pytest.skip("sanitizer runtime not installed: " + r.stderr[-200:])
    assert r.returncode == 0, r.stderr[-3000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), (r.stdout + r.stderr)[-4000:]
