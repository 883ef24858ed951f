"""The C++ sim::Simulator façade (include/msim_simulator.hpp) used from C++."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "movement-sim_gb300"


def _build(tmp_path):
    exe = tmp_path / "simulator_client"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" /
           "simulator_client.cpp"), "-L", str(PKG), "-lmsim", f"-Wl,-rpath,{PKG}", "-pthread", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_simulator_client_builds(tmp_path):
    """The façade header and library link into a plain C++ program (no GPU needed)."""
    assert _build(tmp_path).exists()


@pytest.mark.gpu
def test_simulator_client_runs(tmp_path):
    exe = _build(tmp_path)
    log = tmp_path / "log.csv"
    r = subprocess.run([str(exe), str(log)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
    lines = log.read_text().splitlines()
    assert len(lines) > 20
    fields = lines[0].split(";")
    assert len(fields) == 5 and fields[1] == "1"
