"""Benchmark of the movement-sim per-tick path on GB300.

A step is one tick over every entity: move (random_move.comp:869-874), spatial
index rebuild (tile Morton keys, LSD radix sort, tile ranges) and the radius
neighbour query (random_move.comp:541-719 semantics).  Default workload: the
scale configuration (16,000,000 entities on a 1024 x 1024 lattice, radius 2 m,
64 neighbours kept, dt = 0.1 s, PCG32).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config scale|neighbours|plain]

One JSON line on stdout (rank 0).  Under torchrun every rank runs its own full
replica (the path is "replicas only" across GPUs: no data-path collective).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SEED = 20261203
CONFIGS = {
    # name: lattice side, entities, radius, cap, neighbours, config ticks
    "plain": dict(lattice=32, entities=10_000, radius=2.0, cap=64, neighbours=False, ticks=1000),
    "batched": dict(lattice=0, entities=0, radius=0.0, cap=0, neighbours=False, ticks=1000),
    "neighbours": dict(lattice=256, entities=1_000_000, radius=2.0, cap=64, neighbours=True, ticks=500),
    "scale": dict(lattice=1024, entities=16_000_000, radius=2.0, cap=64, neighbours=True, ticks=200),
    "adjoint": dict(lattice=128, entities=262_144, radius=0.0, cap=0, neighbours=False, ticks=2000),
}
DT = 0.1
SPEED = (1.0, 1.6)
B_STEP = 24  # algorithmic bytes per entity-step of the move (pos r/w 16, heading 4, speed 4)
ADJ_GRID = (512, 512)
ADJ_K = 100
# algorithmic bytes per entity-tick of the calibration step: forward B_step + splat
# position read 8; backward recompute B_step + splat position read 8 + reverse
# (position and adjoint read + write) 16
ADJ_FWD_BYTES = B_STEP + 8
ADJ_BWD_BYTES = B_STEP + 8 + 16


def b_nbr(k_mean: float, updates_per_tick: float = 1.0) -> float:
    """Algorithmic bytes per entity of a neighbour tick.  A tick that updates the
    index: (key, id) write 8, sort read 8 + sorted write 8, query read 8, count write
    4, 4 per kept neighbour (36 + 4k).  A tick that reuses the index: sorted-position
    write 8, query read 8, count write 4, 4 per kept neighbour (20 + 4k).  Mixed by
    the measured share of updating ticks."""
    u = min(max(updates_per_tick, 0.0), 1.0)
    return 20.0 + 16.0 * u + 4.0 * k_mean


# per-kernel algorithmic bytes per entity and launch: the per-entity figures of a
# neighbour tick (24 B move + 36 + 4 k B index and query) split over the kernels
KERNEL_BYTES = {
    "k_step": lambda k: B_STEP + 4,        # move + key write
    "k_onesweep": lambda k: 16,            # (key, id) read + write
    "k_kstart": lambda k: 4 + 20,          # sorted key read, slot read + position gather + write
                                           # (+ 4 B per key slot, added below)
    "k_mark": lambda k: 20,                # previous order 4 + old key 4 + new key 4, split write 8
    "k_merge": lambda k: 32,               # split read 8, sorted key+slot write 8, position gather 8 + write 8
                                           # (+ 4 B per key slot, added below)
    "k_query": lambda k: 12 + 4 * k,       # own pos 8 + count 4 + kept ids
    "k_gather": lambda k: 20,              # order read 4, position read 8 + write 8
    "k_move": lambda k: B_STEP + 12,       # reusing tick: move + rank read 4 + placed position write 8
    "k_permute": lambda k: 72,             # 36-byte state read + write
    "k_step_multi": lambda k: B_STEP,      # per tick
}

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per entity and launch of
# one ncu capture of the same workload at full size (third neighbour tick; 1-pass
# metrics; profiles/scale_16M_dram_traffic.md); scaled by the entities of the run
# warp instructions per entity-step of k_batch_step: smsp__inst_executed.sum of one
# ncu capture (405.8 M for 64 instances, 2,058,939 entities, 100 ticks, tuned
# schedule; profiles/batched_64_instances_k_batch_step_issue.md) over entities x ticks
NCU_BATCH_WARP_INSTR_PER_ENTITY_STEP = 1.971
# warp instructions per entity of k_query on a reused index (widened boxes):
# smsp__inst_executed.sum of one ncu capture (96.2 M for 4,000,000 entities on the
# 512 x 512 lattice, the 16 M and 1 M workloads' density;
# profiles/mid_4M_k_query_widened_ncu.md)
NCU_QUERY_WARP_INSTR_PER_ENTITY = 24.04

NCU_DRAM_BYTES_PER_ENTITY = {
    "scale": {"k_query": 26.87, "k_merge": 32.78, "k_mark": 16.91, "k_step": 27.98},
    "neighbours": {"k_query": 24.07, "k_onesweep": 6.91},
}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier_sync(world):
    try:
        import torch

        if torch.cuda.is_available():
            torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
    except ImportError:
        pass


def max_over_ranks(value: float, world: int) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"msim_clocks_{os.getpid()}_{gpu_index}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        text = self.path.read_text()
        self.path.unlink(missing_ok=True)
        for line in text.splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[4:]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for name, v in zip(names, r[3][1:]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": sorted(reasons)}


def make_sim(pkg, cfg, road_map, reuse=True):
    sim = pkg.Simulation(road_map, cfg["entities"], rng="pcg32", dt=DT, radius=cfg["radius"], cap=cfg["cap"],
                         reuse=reuse)
    sim.init_entities(SEED, placement="fraction", speed=SPEED)
    return sim


def run_ours(args, cfg, world, rank, local):
    pkg = importlib.import_module("movement-sim_gb300")
    pkg.set_device(local)  # the library's own CUDA runtime: select this rank's GPU there too
    road_map = pkg.RoadMap.lattice(cfg["lattice"], SEED)
    n = cfg["entities"]
    nbr = cfg["neighbours"]
    sim = make_sim(pkg, cfg, road_map)
    info = sim.info()
    tick = lambda k: sim.step(k, neighbours=nbr)  # noqa: E731

    # warm-up
    tick(args.warmup)
    sim.sync()
    # timed region: K steps, barrier + sync on both sides, CUDA events on the context stream
    launches0 = sim.launch_count()
    with ClockSampler(local) as clocks:
        barrier_sync(world)
        sim.timer_begin()
        if nbr:
            tick(args.steps)
        else:  # the move-only path runs many ticks per launch
            tick(args.steps)
        ms = sim.timer_end()
        sim.sync()
        barrier_sync(world)
    launches = sim.launch_count() - launches0
    ms_max = max_over_ranks(ms, world)
    value = world * n * args.steps / (ms_max / 1e3)
    # the workload's full tick count in one timed region (includes the re-orderings
    # of the state that a short window may miss)
    barrier_sync(world)
    sim.timer_begin()
    tick(cfg["ticks"])
    ms_cfg = max_over_ranks(sim.timer_end(), world)
    sim.sync()
    config_run = {"ticks": cfg["ticks"], "ms_per_step": ms_cfg / cfg["ticks"],
                  "value": world * n * cfg["ticks"] / (ms_cfg / 1e3), "unit": "entity-steps/s"}

    # mean kept neighbours of the last tick
    k_mean = 0.0
    if nbr:
        cnt, _ = sim.get_neighbours(with_idx=False)
        k_mean = float(np.minimum(cnt, cfg["cap"]).mean())

    # per-kernel times (separate profiled pass: events around every launch)
    sim.set_profiling(True)
    sim.reset_kernel_stats()
    prof_steps = max(1, min(args.steps, 50))
    tick(prof_steps)
    stats = sim.kernel_stats()
    sort = sim.sort_stats()
    sim.set_profiling(False)
    total_ms = sum(v["ms"] for v in stats.values()) or 1.0
    peak, peak_kind = peaks()
    # entries per radix pass: n for a full sort, the entries whose key changed for an
    # incremental update (every pass of an update sorts the same entries)
    sorted_per_update = sort["sorted_entries"] / sort["index_updates"] if sort["index_updates"] else float(n)
    kernels = {}
    for name, v in stats.items():
        avg = v["ms"] / v["launches"]
        if name == "k_step_multi":  # several ticks per launch
            per_launch_bytes = B_STEP * n * prof_steps / v["launches"]
        elif name == "k_onesweep":
            per_launch_bytes = KERNEL_BYTES[name](k_mean) * sorted_per_update
        else:
            per_launch_bytes = KERNEL_BYTES.get(name, lambda k: 0)(k_mean) * n
            if name in ("k_kstart", "k_merge"):  # write one word per key of the key space
                per_launch_bytes += 4 * (2 ** info["key_bits"] + 1)
        kernels[name] = {"launches": v["launches"], "avg_ms": avg, "share": v["ms"] / total_ms,
                         "algo_bytes_per_launch": per_launch_bytes,
                         "achieved_gbs": per_launch_bytes / (avg / 1e3) / 1e9 if avg > 0 else None}
    # the dominant kernel: the largest time of one launch per tick (a radix pass is one
    # of three launches per tick; the re-ordering runs once in many ticks), the unit
    # the roofline's achieved figure is taken over
    dominant = max(kernels.items(), key=lambda kv: kv[1]["avg_ms"] * min(1.0, kv[1]["launches"] / prof_steps))
    traffic = None
    per_entity = NCU_DRAM_BYTES_PER_ENTITY.get(args.config, {}).get(dominant[0])
    if per_entity is not None and not any(getattr(args, k) is not None for k in ("entities", "lattice", "cap")):
        traffic = round(per_entity * n)
    ach = dominant[1]["achieved_gbs"] or 0.0
    roofline = {"bound": "hbm", "kernel": dominant[0], "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "traffic": traffic, "peak_source": peak_kind}
    # The query is bound by instruction issue (its algorithmic bytes are a small part of
    # what it does): warp instructions per entity (ncu) x entities per launch / launch
    # time, against one warp instruction per cycle on each of the 4 schedulers of the
    # 152 SMs at the sampled SM clock.
    if dominant[0] == "k_query" and args.config in ("scale", "neighbours") and \
            not any(getattr(args, k) is not None for k in ("entities", "lattice", "cap")):
        sm_mhz = clocks.summary().get("sm_mhz") or 2070.0
        issue_peak = 152 * 4 * sm_mhz * 1e6
        inst_s = NCU_QUERY_WARP_INSTR_PER_ENTITY * n / (dominant[1]["avg_ms"] / 1e3)
        roofline["issue"] = {"bound": "issue", "achieved": round(inst_s, 1), "peak": issue_peak,
                             "unit": "warp-instructions/s", "frac": round(inst_s / issue_peak, 4),
                             "warp_instructions_per_entity": NCU_QUERY_WARP_INSTR_PER_ENTITY, "sm_mhz": sm_mhz}
    updates_per_tick = sort["index_updates"] / prof_steps if nbr else 0.0
    tick_bytes = (B_STEP + (b_nbr(k_mean, updates_per_tick) if nbr else 0.0)) * n
    tick_gbs = tick_bytes * args.steps / (ms / 1e3) / 1e9
    roofline_tick = {"achieved": round(tick_gbs, 1), "peak": peak, "unit": "GB/s", "frac": round(tick_gbs / peak, 4),
                     "algo_bytes_per_entity_step": round(tick_bytes / n, 3),
                     "index_updates_per_tick": round(updates_per_tick, 4)}

    # end to end through the C ABI with host buffers: upload the entity state from
    # pinned memory, run one tick, read the state and neighbour counts back
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(pkg, sim, cfg, n, nbr, world, min(args.steps, args.e2e_steps))
    sim.close()

    # the same timed window with the index updated on every neighbour tick
    # (MSIM_PARAM_NO_REUSE): what index reuse is worth on this workload
    reuse = None
    if nbr:
        s2 = make_sim(pkg, cfg, road_map, reuse=False)
        s2.step(args.warmup, neighbours=True)
        s2.sync()
        barrier_sync(world)
        s2.timer_begin()
        s2.step(args.steps, neighbours=True)
        ms2 = max_over_ranks(s2.timer_end(), world)
        s2.sync()
        s2.close()
        reuse = {"index_updates_per_tick": round(sort["index_updates"] / prof_steps, 4),
                 "without_reuse": {"ms_per_step": ms2 / args.steps,
                                   "value": world * n * args.steps / (ms2 / 1e3), "index_updates_per_tick": 1.0}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(cfg, budget_s=args.cpu_budget)
    return {
        "value": value, "ms_per_step": ms_max / args.steps, "clocks": clocks.summary(), "k_mean": k_mean,
        "roofline": roofline, "roofline_tick": roofline_tick, "kernels": kernels, "e2e": e2e, "cpu": cpu,
        "launches": launches, "info": info, "roads": road_map.num_roads, "config_run": config_run,
        "sorted_fraction": sorted_per_update / max(n, 1), "reuse": reuse,
    }


def run_e2e(pkg, sim, cfg, n, nbr, world, steps):
    """End to end through the C ABI with the entity state on the host (page-locked):
    every step uploads the state, runs one tick and reads back the moved state and
    the neighbour counts.  Headline path: msim_tick_host (one call; chunked upload,
    move and download overlap).  Beside it, the same round trip through the four
    separate calls (msim_set_entities, msim_step, msim_get_state, msim_get_neighbours)."""
    pos = pkg.PinnedBuffer((n, 2), np.float32)
    head = pkg.PinnedBuffer(n, np.uint32)
    rng = pkg.PinnedBuffer((n, 4), np.uint32)
    speed = pkg.PinnedBuffer(n, np.float32)
    cnt = pkg.PinnedBuffer(n, np.uint32)
    out = {"pos": pos.array, "heading": head.array, "rng": rng.array, "speed": speed.array}
    sim.get_state(out)
    L = pkg.lib()
    ctx = sim._ctx
    u32 = lambda b: b.array.ctypes.data_as(pkg._capi.u32p)  # noqa: E731
    f32 = lambda b: b.array.ctypes.data_as(pkg._capi.f32p)  # noqa: E731
    flags = pkg._capi.STEP_NEIGHBOURS if nbr else 0

    def fused():  # the state arrays are both input and output (a chunk is read before it is written)
        pkg.check(L.msim_tick_host(ctx, f32(pos), u32(head), u32(rng), f32(speed), flags, f32(pos), u32(head),
                                   u32(rng), u32(cnt) if nbr else None, None))

    def separate():
        pkg.check(L.msim_set_entities(ctx, f32(pos), u32(head), u32(rng), f32(speed)))
        pkg.check(L.msim_step(ctx, 1, flags))
        pkg.check(L.msim_get_state(ctx, f32(pos), u32(head), u32(rng), None))
        if nbr:
            pkg.check(L.msim_get_neighbours(ctx, u32(cnt), None))

    def timed(fn):
        fn()
        barrier_sync(world)
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        barrier_sync(world)
        return max_over_ranks(time.perf_counter() - t0, world)

    dt = timed(fused)
    # bytes back per step: in place (the same page-locked arrays in and out) the tick
    # downloads positions and counts and writes the headings and RNG states that change
    # into the arrays; counted here over one more tick
    h0, r0 = head.array.copy(), rng.array.copy()
    fused()
    changed_head = int(np.count_nonzero(head.array != h0))
    changed_rng = int(np.count_nonzero(np.any(rng.array != r0, axis=1)))
    dt_sep = timed(separate)
    h2d = n * (8 + 4 + 16 + 4)
    d2h = n * (8 + (4 if nbr else 0)) + 4 * changed_head + 16 * changed_rng
    for b in (pos, head, rng, speed, cnt):
        b.free()
    return {"value": world * n * steps / dt, "unit": "entity-steps/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "steps": steps, "ms_per_step": 1e3 * dt / steps,
            "path": "msim_tick_host in place: page-locked host arrays for pos, heading, rng (in and out) and speed; "
                    "positions and neighbour counts downloaded, the headings / RNG states that change "
                    f"({changed_head} / {changed_rng} per tick) written into the arrays by the move kernel",
            "separate_calls": {"value": world * n * steps / dt_sep, "ms_per_step": 1e3 * dt_sep / steps,
                               "path": "msim_set_entities + msim_step(1) + msim_get_state + msim_get_neighbours"}}


def run_batched(args, world, rank, local):
    """Batched ensemble: 512 instances (lattice side uniform 16..256, entities
    log-uniform 1e3..2e5, seed = index + SEED) advanced `steps` ticks by one
    persistent graph-captured launch, against one-at-a-time plain launches."""
    pkg = importlib.import_module("movement-sim_gb300")
    pkg.set_device(local)
    sides, ents, seeds = ensemble_config(args.instances, SEED)
    maps = [pkg.RoadMap.lattice(s, sd) for s, sd in zip(sides, seeds)]
    total = sum(ents)
    batch = pkg.Batch(maps, ents, rng="pcg32", dt=DT)
    batch.init_entities(seeds, placement="fraction", speed=SPEED)
    t_tune = time.perf_counter()
    if not args.no_tune:
        batch.tune(min(args.steps, 100), args.tune_cache)
    t_tune = time.perf_counter() - t_tune
    batch.init_entities(seeds, placement="fraction", speed=SPEED)
    batch.step(args.steps)  # warm-up: builds the graph for this tick count
    batch.sync()
    batch.init_entities(seeds, placement="fraction", speed=SPEED)
    launches0 = batch.info()["launches"]
    with ClockSampler(local) as clocks:
        barrier_sync(world)
        batch.timer_begin()
        batch.step(args.steps)
        ms = batch.timer_end()
        batch.sync()
        barrier_sync(world)
    launches = batch.info()["launches"] - launches0
    ms_max = max_over_ranks(ms, world)
    value = world * total * args.steps / (ms_max / 1e3)
    sched = batch.schedule()
    batch.close()
    # one at a time: every instance alone, its move-only launches, one after another
    sims = []
    for m, n, sd in zip(maps, ents, seeds):
        s = pkg.Simulation(m, n, rng="pcg32", dt=DT, radius=2.0, cap=0)
        s.init_entities(sd, placement="fraction", speed=SPEED)
        s.sync()
        sims.append(s)
    for s in sims[:8]:
        s.step(args.steps)
        s.sync()
    t0 = time.perf_counter()
    for s in sims:
        s.step(args.steps)
        s.sync()
    one_s = time.perf_counter() - t0
    for s in sims:
        s.close()
    one_value = total * args.steps / one_s
    peak, peak_kind = peaks()
    # per launch every entity's state is read and written once (pos 8+8, heading 4+4,
    # speed 4, rng rarely): the HBM bytes of the launch
    launch_bytes = total * 28
    gbs = launch_bytes / (ms / 1e3) / 1e9
    clk = clocks.summary()
    # The kernel keeps every entity's state in registers for all ticks of the launch,
    # so it is bound by instruction issue, not HBM: achieved = warp instructions per
    # entity-step (from an ncu capture of the kernel) x entity-steps/s, against one
    # warp instruction per cycle on each of the 4 schedulers of the 152 SMs.
    sm_mhz = clk.get("sm_mhz") or 2070.0
    issue_peak = 152 * 4 * sm_mhz * 1e6
    ipe = NCU_BATCH_WARP_INSTR_PER_ENTITY_STEP
    issue = None
    if ipe is not None:
        ach = ipe * value / world
        issue = {"bound": "issue", "kernel": "k_batch_step", "achieved": ach, "peak": issue_peak,
                 "unit": "warp-instructions/s", "frac": round(ach / issue_peak, 4),
                 "warp_instructions_per_entity_step": ipe, "sm_mhz": sm_mhz}
    return {"value": value, "ms_per_step": ms_max / args.steps, "clocks": clk, "launches": launches,
            "one_at_a_time": {"value": one_value, "unit": "entity-steps/s", "seconds": one_s,
                              "what": "each instance alone (msim_step without neighbours), synchronised one by one"},
            "speedup_vs_one_at_a_time": value / one_value, "schedule": sched, "tune_seconds": t_tune,
            "instances": len(maps), "total_entities": total, "issue": issue,
            "roofline": {"bound": "hbm", "kernel": "k_batch_step", "achieved": round(gbs, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(gbs / peak, 4), "traffic": None, "peak_source": peak_kind,
                         "note": "not the bound: the state stays in registers for all ticks of a launch (28 B "
                                 "per entity per launch); see issue"}}


def run_facade(cfg, ticks=200, warmup=5):
    """The drop-in C++ façade (sim::Simulator::tick_once, one synchronous tick per
    call with its phase times, CSV log line and pair counter) on the workload, run by
    the example program movement-sim_gb300/examples/simulator_ticks."""
    exe = ROOT / "movement-sim_gb300" / "examples" / "simulator_ticks"
    if not exe.exists():
        return {"unavailable": f"{exe.name} not built"}
    with tempfile.TemporaryDirectory() as td:
        r = subprocess.run([str(exe), str(cfg["lattice"]), str(cfg["entities"]), str(ticks), str(warmup),
                            str(Path(td) / "ticks.csv")], capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        return {"error": (r.stderr or r.stdout)[-400:]}
    out = json.loads(r.stdout.strip().splitlines()[-1])
    out["what"] = (f"sim::Simulator::tick_once x {ticks} after {warmup} warm-up ticks ({cfg['entities']} entities, "
                   f"{cfg['lattice']}x{cfg['lattice']} lattice): msim_step(1) + msim_sync + phase times + CSV log "
                   "line per tick")
    return out


def run_forms(args, world, rank, local):
    """Short runs of the two other forms, added to the default line: the batched
    ensemble (512 instances, 1,000 ticks in one launch, against one-at-a-time
    launches) and the calibration step (forward + adjoint, 2 steps after 1 warm-up)."""
    a = argparse.Namespace(**vars(args))
    a.steps, a.warmup, a.no_e2e, a.no_cpu, a.ticks, a.no_tune = CONFIGS["batched"]["ticks"], 3, True, True, None, False
    b = run_batched(a, world, rank, local)
    a.steps, a.warmup = 2, 1
    d = run_adjoint(a, world, rank, local)
    f = run_facade(CONFIGS["scale"])
    return {"facade": f,
            "batched": {"workload": "512 instances, lattice side U{16..256}, entities log-U[1e3, 2e5], "
                                    f"{b['total_entities']} entities, 1,000 ticks in one launch",
                        "value": b["value"], "unit": "entity-steps/s", "ms_per_tick": b["ms_per_step"],
                        "one_at_a_time": b["one_at_a_time"]["value"],
                        "speedup_vs_one_at_a_time": b["speedup_vs_one_at_a_time"], "issue": b["issue"],
                        "schedule": b["schedule"]},
            "adjoint": {"workload": "262,144 entities, 128x128 lattice, 2,000 ticks, 512x512 grid, K = 100",
                        "value": d["value"], "unit": "entity-steps/s (forward + backward entity-ticks)",
                        "ms_per_step": d["ms_per_step"], "forward_ms": d["forward_ms"],
                        "backward_ms": d["backward_ms"], "step_over_forward": d["step_over_forward"],
                        "roofline": d["roofline"]}}


def run_adjoint(args, world, rank, local):
    """Differentiable calibration: one step = forward (2,000 ticks of 262,144 entities
    with the density splat) + loss + the hand-written adjoint; value = entity-ticks of
    the step / its time.  Target density from hidden road factors U[0.7, 1.3]."""
    import torch

    pkg = importlib.import_module("movement-sim_gb300")
    pkg.set_device(local)
    cal = importlib.import_module("movement-sim_gb300.calibration")
    cfg = dict(CONFIGS["adjoint"])
    if args.ticks:
        cfg["ticks"] = args.ticks
    rm = pkg.RoadMap.lattice(cfg["lattice"], SEED)
    n, T = cfg["entities"], cfg["ticks"]
    G = ADJ_GRID[0] * ADJ_GRID[1]
    calib = cal.Calibration(rm, n, T, dt=DT, rng="pcg32", checkpoint_interval=ADJ_K, grid=ADJ_GRID, seed=SEED,
                            placement="fraction", speed=SPEED)
    rs = np.random.default_rng(SEED)
    hidden = torch.from_numpy(rs.uniform(0.7, 1.3, rm.num_roads).astype(np.float32)).cuda()
    target = torch.empty(G, dtype=torch.float32, device="cuda")
    calib.forward(factor=hidden, density=target)
    st = calib.initial_state()
    speed = torch.from_numpy(st["speed"].copy()).cuda()
    factor = torch.ones(rm.num_roads, dtype=torch.float32, device="cuda")
    gs = torch.empty(n, dtype=torch.float32, device="cuda")
    gf = torch.empty(rm.num_roads, dtype=torch.float32, device="cuda")

    def step():
        loss = calib.forward(speed, factor, target)
        calib.backward(gs, gf)
        return loss

    for _ in range(args.warmup):
        loss0 = step()
    phases = []
    with ClockSampler(local) as clocks:
        barrier_sync(world)
        calib.timer_begin()
        for _ in range(args.steps):
            step()
            phases.append(calib.phase_times())
        ms = calib.timer_end()
        barrier_sync(world)
    ms_max = max_over_ranks(ms, world)
    value = world * n * T * args.steps / (ms_max / 1e3)
    ph = {k: float(np.mean([p[k] for p in phases])) for k in phases[0]}
    fwd_ms = ph["forward"] + ph["loss"]
    bwd_ms = ph["backward_sweeps"] + ph["road_reduction"]
    peak, peak_kind = peaks()
    S = (T + ADJ_K - 1) // ADJ_K
    kern = {"k_adj_forward": {"launches": 1, "avg_ms": ph["forward"], "algo_bytes_per_launch": ADJ_FWD_BYTES * n * T},
            "k_adj_backward": {"launches": S, "avg_ms": ph["backward_sweeps"] / S,
                               "algo_bytes_per_launch": ADJ_BWD_BYTES * n * ADJ_K}}
    tot = sum(v["avg_ms"] * v["launches"] for v in kern.values())
    for v in kern.values():
        v["share"] = v["avg_ms"] * v["launches"] / tot
        v["achieved_gbs"] = v["algo_bytes_per_launch"] / (v["avg_ms"] / 1e3) / 1e9
    dom_name, dom = max(kern.items(), key=lambda kv: kv[1]["share"])
    roofline = {"bound": "hbm", "kernel": dom_name, "achieved": round(dom["achieved_gbs"], 1), "peak": peak,
                "unit": "GB/s", "frac": round(dom["achieved_gbs"] / peak, 4), "traffic": None,
                "peak_source": peak_kind,
                "note": f"algorithmic bytes per entity-tick: forward {ADJ_FWD_BYTES}, backward {ADJ_BWD_BYTES}"}
    # end to end through the public API with host buffers: speeds and factors from
    # pinned host memory, forward + backward, gradients and loss back to the host
    e2e = None
    if not args.no_e2e:
        hs = torch.from_numpy(st["speed"].copy()).pin_memory()
        hf = torch.ones(rm.num_roads, dtype=torch.float32).pin_memory()
        ogs = torch.empty(n, dtype=torch.float32).pin_memory()
        ogf = torch.empty(rm.num_roads, dtype=torch.float32).pin_memory()
        steps_e = max(1, min(args.steps, 3))
        barrier_sync(world)
        t0 = time.perf_counter()
        for _ in range(steps_e):
            speed.copy_(hs, non_blocking=True)
            factor.copy_(hf, non_blocking=True)
            step()
            ogs.copy_(gs)
            ogf.copy_(gf)
        barrier_sync(world)
        el = max_over_ranks(time.perf_counter() - t0, world)
        e2e = {"value": world * n * T * steps_e / el, "unit": "entity-steps/s",
               "h2d_bytes_per_step": 4 * (n + rm.num_roads), "d2h_bytes_per_step": 4 * (n + rm.num_roads) + 8,
               "steps": steps_e, "path": "pinned speeds/factors -> Calibration.forward + backward -> pinned gradients"}
    calib.close()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import oracle as orc

        cpu = cpu_adjoint(orc, orc.lattice(cfg["lattice"], SEED), args.cpu_entities or n, T, orc.cpu_count())
    return {"value": value, "ms_per_step": ms_max / args.steps, "clocks": clocks.summary(), "roofline": roofline,
            "kernels": kern, "phases_ms": ph, "forward_ms": fwd_ms, "backward_ms": bwd_ms,
            "backward_over_forward": bwd_ms / fwd_ms, "step_over_forward": (fwd_ms + bwd_ms) / fwd_ms,
            "loss": loss0, "roads": rm.num_roads, "e2e": e2e, "cpu": cpu,
            "launches": args.steps * (3 + S + 3 + 3 + 2)}


def cpu_adjoint(orc, rm, n, ticks, threads):
    """The FP64 CPU adjoint (forward, loss, reverse sweep) of the calibration
    workload: n entities over all ticks, host threads."""
    pos, head, rng, speed = orc.init_entities(rm.road_pos, n, 1, SEED, 1, SPEED[0], SPEED[1])
    state = {"pos": pos, "heading": head, "rng": rng}
    target = np.zeros(ADJ_GRID[0] * ADJ_GRID[1], np.float32)
    factor = np.ones(rm.num_roads, np.float32)
    t0 = time.perf_counter()
    orc.density_adjoint(rm, state, speed, factor, 1, DT, ticks, ADJ_GRID, target, threads=threads)
    el = time.perf_counter() - t0
    return {"value": n * ticks / el, "unit": "entity-steps/s", "cores": threads, "kind": "port",
            "sample": f"{n} entities x {ticks} ticks of the calibration step (FP64 oracle adjoint: forward, loss "
                      f"and reverse sweep), {threads} threads"}


def ensemble_config(count: int = 512, seed: int = SEED, side_range=(16, 256), entity_range=(1_000, 200_000)):
    """Instance sizes of the batched ensemble: lattice side uniform in side_range
    (inclusive), entity count log-uniform in entity_range, instance seed = index +
    seed; numpy's PCG64 generator seeded by `seed`.  (The package's ensemble_config
    gives the same lists; a CPU test checks it.)"""
    rs = np.random.default_rng(seed)
    sides = rs.integers(side_range[0], side_range[1] + 1, count)
    lo, hi = np.log(entity_range[0]), np.log(entity_range[1])
    entities = np.floor(np.exp(rs.uniform(lo, hi, count))).astype(np.int64)
    seeds = np.arange(count, dtype=np.int64) + seed
    return [int(x) for x in sides], [int(x) for x in entities], [int(x) for x in seeds]


class OracleWorkload:
    """A workload on the host cores with the oracle C restatement, built from the
    oracle's own lattice generator (nothing of the product is loaded): the entities
    of the workload, and per tick the move step and, for neighbour workloads, the
    CPU-grid query with the id lists, into arrays reused across ticks."""

    def __init__(self, orc, lattice: int, n: int, cfg: dict, threads: int, seed: int = SEED):
        self.orc, self.cfg, self.threads, self.n = orc, cfg, threads, n
        self.rm = orc.lattice(lattice, seed)
        self.state = orc.init_entities(self.rm.road_pos, n, 1, seed, 1, SPEED[0], SPEED[1])
        self.nbr = bool(cfg["neighbours"])
        if self.nbr:
            self.out = (np.empty(n, np.uint32), np.empty((n, cfg["cap"]), np.uint32) if cfg["cap"] else None)

    def ticks(self, ticks: int) -> None:
        orc, rm = self.orc, self.rm
        pos, head, rng, speed = self.state
        if not self.nbr:  # independent entities: every thread runs all ticks on its range
            orc.step(rm.road_pos, rm.road_conn, rm.connections, pos, head, rng, speed, 1, DT, ticks,
                     threads=self.threads)
            return
        for _ in range(ticks):
            orc.step(rm.road_pos, rm.road_conn, rm.connections, pos, head, rng, speed, 1, DT, 1, threads=self.threads)
            orc.neighbours(pos, self.cfg["radius"], self.cfg["cap"], threads=self.threads, with_idx=True,
                           out=self.out)

    def what(self) -> str:
        return ("oracle C restatement of random_move.comp (move" +
                (" + CPU-grid neighbour query with id lists)" if self.nbr else " only)"))


def cpu_baseline(cfg, budget_s=20.0):
    """The oracle on the full workload (same map, entities and seed as the GPU run),
    timed on the host cores for whole ticks until about budget_s seconds."""
    from oracle import oracle as orc

    threads = orc.cpu_count()
    w = OracleWorkload(orc, cfg["lattice"], cfg["entities"], cfg, threads)
    w.ticks(1)  # warm-up tick
    ticks = 0
    t0 = time.perf_counter()
    while True:
        w.ticks(1)
        ticks += 1
        el = time.perf_counter() - t0
        if el > budget_s or ticks >= cfg["ticks"]:
            break
    return {"value": cfg["entities"] * ticks / el, "unit": "entity-steps/s", "cores": threads, "kind": "port",
            "sample": f"{ticks} ticks (after 1 warm-up tick) of the full workload ({cfg['entities']} entities, "
                      f"{cfg['lattice']}x{cfg['lattice']} lattice): {w.what()}, {threads} threads"}


def run_reference(args, cfg, world, rank):
    """The reference's path on the host cores (the Vulkan shader needs a graphics
    stack that neither machine has, so it is the oracle C restatement of the shader,
    with the same threading as shader_validation): W warm-up steps, then K timed
    steps of the same workload as the GPU arm.  Loads only oracle/ libraries."""
    if rank != 0:
        return None
    from oracle import oracle as orc

    threads = orc.cpu_count()
    if args.config == "adjoint":  # each step: the FP64 calibration step (forward, loss, reverse sweep)
        n = args.cpu_entities or cfg["entities"]
        rm = orc.lattice(cfg["lattice"], SEED)
        for _ in range(min(args.warmup, 1)):
            cpu_adjoint(orc, rm, n, cfg["ticks"], threads)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r = cpu_adjoint(orc, rm, n, cfg["ticks"], threads)
        el = time.perf_counter() - t0
        return {"value": n * cfg["ticks"] * args.steps / el, "ms_per_step": el * 1e3 / args.steps,
                "threads": threads, "sample": f"each step {r['sample']}"}
    if args.config == "batched":  # each step: one move tick of every instance
        sides, ents, seeds = ensemble_config(args.instances, SEED)
        move = dict(neighbours=False)
        inst = [OracleWorkload(orc, side, n_i, move, threads, seed=sd) for side, n_i, sd in zip(sides, ents, seeds)]
        total = sum(ents)

        def run(ticks):
            for w in inst:
                w.ticks(ticks)

        run(args.warmup)
        t0 = time.perf_counter()
        run(args.steps)
        el = time.perf_counter() - t0
        return {"value": total * args.steps / el, "ms_per_step": el * 1e3 / args.steps, "threads": threads,
                "sample": f"each step one move tick of all {len(inst)} ensemble instances ({total} entities), "
                          f"instance after instance; oracle C restatement of the move step, {threads} threads"}
    w = OracleWorkload(orc, cfg["lattice"], cfg["entities"], cfg, threads)
    w.ticks(args.warmup)
    t0 = time.perf_counter()
    w.ticks(args.steps)
    el = time.perf_counter() - t0
    return {"value": cfg["entities"] * args.steps / el, "ms_per_step": el * 1e3 / args.steps, "threads": threads,
            "sample": f"each step one tick of the full workload ({cfg['entities']} entities, "
                      f"{cfg['lattice']}x{cfg['lattice']} lattice): {w.what()}, {threads} threads"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="scale")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="scale config: skip the short batched and adjoint runs added to the line")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--entities", type=int, default=None, help="override (profiling runs)")
    ap.add_argument("--lattice", type=int, default=None, help="override (profiling runs)")
    ap.add_argument("--cap", type=int, default=None, help="override (profiling runs)")
    ap.add_argument("--ticks", type=int, default=None, help="adjoint config: ticks per step (profiling runs)")
    ap.add_argument("--instances", type=int, default=512, help="batched config: number of instances")
    ap.add_argument("--tune-cache", default=None, help="batched config: tuner cache file to reuse/append")
    ap.add_argument("--no-tune", action="store_true", help="batched config: the default schedule (profiling runs)")
    ap.add_argument("--cpu-entities", type=int, default=None,
                    help="adjoint config: entities of the CPU adjoint (default: the workload's)")
    args = ap.parse_args()
    cfg = dict(CONFIGS[args.config])
    for k in ("entities", "lattice", "cap", "ticks"):
        if getattr(args, k) is not None:
            cfg[k] = getattr(args, k)
    if args.steps is None:
        args.steps = 5 if args.config == "adjoint" else cfg["ticks"]
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":  # host cores only: no process group, rank 0 alone runs
        world, rank, local = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    else:
        world, rank, local = dist_setup(args)
    config = workload_config(args, cfg, world)
    line = {"metric": "entity-steps/s", "unit": "entity-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded lattice road graph and entities)", "config": config}

    if args.impl == "reference":
        r = run_reference(args, cfg, world, rank)
        if rank == 0:
            line.update({"impl": "reference", "value": r["value"], "ms_per_step": r["ms_per_step"],
                         "cpu_baseline": {"value": r["value"], "unit": "entity-steps/s", "cores": r["threads"],
                                          "kind": "port",
                                          "sample": r["sample"] + "; the Vulkan shader itself is unavailable on "
                                                                  "this box (no graphics stack)"},
                         "e2e": {"value": r["value"], "unit": "entity-steps/s", "h2d_bytes_per_step": 0,
                                 "d2h_bytes_per_step": 0}})
            print(json.dumps(line), flush=True)
        return

    if args.config == "batched":
        r = run_batched(args, world, rank, local)
        if rank == 0:
            line.update({k: r[k] for k in ("value", "ms_per_step", "clocks", "roofline", "one_at_a_time",
                                            "speedup_vs_one_at_a_time", "issue")})
            line.update({"schedule": r["schedule"], "tune_seconds": round(r["tune_seconds"], 2),
                         "gpu_launches": r["launches"], "cpu_baseline": None, "e2e": None})
            print(json.dumps(line), flush=True)
        return
    if args.config == "adjoint":
        r = run_adjoint(args, world, rank, local)
        if rank == 0:
            line.update({k: r[k] for k in ("value", "ms_per_step", "clocks", "roofline", "e2e")})
            line.update({"cpu_baseline": r["cpu"], "gpu_launches": r["launches"], "kernels": r["kernels"],
                         "roads": r["roads"], "phases_ms": r["phases_ms"], "forward_ms": r["forward_ms"],
                         "backward_ms": r["backward_ms"], "backward_over_forward": r["backward_over_forward"],
                         "step_over_forward": r["step_over_forward"], "loss": r["loss"]})
            print(json.dumps(line), flush=True)
        return
    r = run_ours(args, cfg, world, rank, local)
    forms = None
    if args.config == "scale" and world == 1 and not args.no_forms and not any(getattr(args, k) is not None
                                                                               for k in ("entities", "lattice", "cap")):
        forms = run_forms(args, world, rank, local)
    if rank == 0:
        line.update({"value": r["value"], "ms_per_step": r["ms_per_step"], "roofline": r["roofline"],
                     "roofline_tick": r["roofline_tick"], "cpu_baseline": r["cpu"], "e2e": r["e2e"],
                     "clocks": r["clocks"], "gpu_launches": r["launches"], "config_length_run": r["config_run"],
                     "index": {"roads": r["roads"], "tiles": [r["info"]["tiles_x"], r["info"]["tiles_y"]],
                               "cell_m": round(r["info"]["cell_size"], 3), "sort_passes": r["info"]["sort_passes"],
                               "resort_interval": r["info"]["resort_interval"],
                               "mean_kept_neighbours": round(r["k_mean"], 4),
                               "sorted_fraction_per_update": round(r["sorted_fraction"], 5),
                               "reuse": r["reuse"]},
                     "kernels": {k: {kk: (round(vv, 5) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                                 for k, v in r["kernels"].items()}})
        if forms is not None:
            line["forms"] = forms
        print(json.dumps(line), flush=True)


def workload_config(args, cfg, world):
    """The workload as both arms print it (nothing measured: the same dict for the
    GPU arm and the reference arm)."""
    workload = {
        "scale": "plain+neighbours at scale: 16,000,000 entities, 1024x1024 lattice, radius 2.0 m, cap 64",
        "neighbours": "plain+neighbours: 1,000,000 entities, 256x256 lattice, radius 2.0 m, cap 64",
        "plain": "plain: 10,000 entities, 32x32 lattice, move only",
        "batched": "batched ensemble: 512 instances, lattice side U{16..256}, entities log-U[1e3, 2e5], move only",
        "adjoint": "differentiable calibration: 262,144 entities, 128x128 lattice, 2,000 ticks, 512x512 density "
                   "grid, checkpoints every 100 ticks; one step = forward + loss + adjoint",
    }[args.config]
    overrides = {k: getattr(args, k) for k in ("entities", "lattice", "cap", "ticks") if getattr(args, k) is not None}
    if overrides:
        workload += f" [profiling override {overrides}]"
    config = {"workload": workload, "entities": cfg["entities"], "lattice": cfg["lattice"], "dt_s": DT,
              "radius_m": cfg["radius"] if cfg["neighbours"] else None, "cap": cfg["cap"] if cfg["neighbours"] else None,
              "rng": "pcg32", "speed_mps": list(SPEED), "seed": SEED, "ticks_per_step": 1,
              "parallelism": f"replicas x{world}",
              "l2": "inputs larger than L2 (entity state 32 B x entities)" if cfg["entities"] * 32 > 129e6
              else "working set fits in L2 (small config)"}
    if args.config == "batched":
        _, ents, _ = ensemble_config(args.instances, SEED)
        config.update({"instances": args.instances, "entities": sum(ents), "lattice": "U{16..256}",
                       "l2": "inputs larger than L2 (28 B x total entities per launch)"})
    if args.config == "adjoint":
        config.update({"ticks_per_step": cfg["ticks"], "grid": list(ADJ_GRID), "checkpoint_interval": ADJ_K,
                       "hidden_factors": "U[0.7, 1.3] from the seed",
                       "l2": "inputs larger than L2 (checkpoints and per-segment history)"})
    return config

if __name__ == "__main__":
    main()
