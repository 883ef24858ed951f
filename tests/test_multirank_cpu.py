"""The multi-rank path of bench.py on CPU, world size 2 over gloo.

The path shards as independent replicas (no data-path collective): every rank runs
its own simulation and rank 0 reports N x entities x steps over the slowest rank's
time.  What needs no GPU is tested here: the barrier and max-over-ranks helpers
across two gloo ranks, and the reference arm launched under torchrun, where rank 0
alone runs and prints one JSON line and the other rank exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist

    class Args:
        pass

    w, r, _ = bench.dist_setup(Args())
    assert (w, r) == (world, rank) and dist.get_backend() == "gloo"
    bench.barrier_sync(w)
    got = bench.max_over_ranks(float(10 * rank + 3), w)
    Path(out_dir, f"rank{rank}.txt").write_text(repr(got))
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_gloo(tmp_path):
    world = 2
    port = _free_port()
    ctx = torch.multiprocessing.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        assert float((tmp_path / f"rank{r}.txt").read_text()) == 13.0  # the slowest rank's value on every rank


def test_reference_arm_under_torchrun_two_ranks():
    port = _free_port()
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference", "--config",
           "plain", "--gpus", "2", "--steps", "2", "--warmup", "3"]
    res = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout  # rank 0 alone prints
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["metric"] == "entity-steps/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_loads_only_the_oracle_and_prints_the_same_config():
    """The reference arm runs the oracle on the GPU arm's own workload and loads no
    library of the product; its config dict is the GPU arm's (nothing measured in it)."""
    code = ("import sys, json, io, contextlib; sys.path.insert(0, '.'); import bench;"
            "sys.argv = ['bench.py', '--impl', 'reference', '--config', 'neighbours', '--entities', '50000',"
            " '--lattice', '64', '--steps', '2', '--warmup', '3'];"
            "buf = io.StringIO();"
            "ctx = contextlib.redirect_stdout(buf); ctx.__enter__(); bench.main(); ctx.__exit__(None, None, None);"
            "maps = open('/proc/self/maps').read();"
            "print(json.dumps({'line': json.loads(buf.getvalue().strip().splitlines()[-1]),"
            " 'libmsim': 'libmsim' in maps, 'oracle': 'liboracle' in maps,"
            " 'pkg': any(m.startswith('movement-sim_gb300') for m in sys.modules)}))")
    res = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600,
                         env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert res.returncode == 0, res.stderr[-2000:]
    out = json.loads(res.stdout.strip().splitlines()[-1])
    assert out["oracle"] and not out["libmsim"] and not out["pkg"]
    line = out["line"]
    assert line["impl"] == "reference" and line["value"] > 0
    sys.path.insert(0, str(ROOT))
    import argparse

    import bench

    args = argparse.Namespace(config="neighbours", entities=50000, lattice=64, cap=None, ticks=None, instances=512)
    cfg = dict(bench.CONFIGS["neighbours"], entities=50000, lattice=64)
    assert line["config"] == bench.workload_config(args, cfg, 1)


def test_bench_ensemble_matches_package(msim):
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.ensemble_config(512) == msim.ensemble_config(512)
