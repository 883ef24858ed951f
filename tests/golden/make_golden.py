"""Generates the committed golden fixtures from the reference (run where the
reference tree is present; the fixtures travel with the repository).

* test_map.npz     - the reference's test_map.json read with Python's json module
                     and the loader rules of src/sim/Map.cpp:28-150 (numbers to
                     float32, zero-length roads skipped).
* ref_quadtree.npz - entity sets and, per entity, the collision pairs (j < i)
                     reported by the reference's own CPU quad tree
                     (shader_validation/src/main.cpp, compiled into oracle/_ref by
                     oracle/build_oracle.py).  Case 0 is the known-answer test
                     run_collision_detection_test_1 (main.cpp:1137-1199).
                     Both the distinct partner ids (from the colour writes) and
                     the raw counter increments (which count repeated visits)
                     are stored.

Usage: python tests/golden/make_golden.py   (reference tree at $MSIM_REFERENCE_ROOT,
default /root/reference, as oracle/build_oracle.py reads it)
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REFERENCE = Path(os.environ.get("MSIM_REFERENCE_ROOT", "/root/reference"))
sys.path.insert(0, str(ROOT))


def test_map() -> None:
    doc = json.loads((REFERENCE / "test_map.json").read_text())
    pos, conn = [], []
    for r in doc["roads"]:
        s = (np.float32(r["start"]["distLat"]), np.float32(r["start"]["distLong"]))
        e = (np.float32(r["end"]["distLat"]), np.float32(r["end"]["distLong"]))
        if s == e:
            continue
        pos.append([*s, *e])
        conn.append([r["connIndexStart"], r["connCountStart"], r["connIndexEnd"], r["connCountEnd"]])
    np.savez(HERE / "test_map.npz", road_pos=np.array(pos, np.float32), road_conn=np.array(conn, np.uint32),
             connections=np.array(doc["connectionRoadIndexList"], np.uint32),
             width=np.float32(doc["maxDistLat"]), height=np.float32(doc["maxDistLong"]))


def ref_quadtree() -> None:
    from oracle import build_oracle, oracle

    build_oracle.build()
    assert oracle.ref_lib() is not None, "reference quad tree could not be built"
    rs = np.random.default_rng(20261203)
    cases = []
    # 0: run_collision_detection_test_1 positions (main.cpp:1141-1190)
    W, H = np.float32(29007.4609), np.float32(16463.7656)
    p = np.array([[W / 2 - 3, 0], [W / 2 + 3, 0], [0, 0], [W / 4, 0], [W / 4 - 9, 0]], np.float32)
    cases.append((p, np.float32([W, H]), 10.0))
    # 1: uniform points, R = 10
    cases.append((rs.uniform([0, 0], [200, 150], (1000, 2)).astype(np.float32), np.float32([200, 150]), 10.0))
    # 2: points along road-like segments, R = 2
    t = rs.uniform(0, 1, 1000)
    seg = rs.integers(0, 12, 1000)
    a = rs.uniform(0, 500, (12, 2))
    b = a + rs.uniform(-60, 60, (12, 2))
    q = a[seg] + t[:, None] * (b[seg] - a[seg])
    cases.append((np.clip(q, 0, 499).astype(np.float32), np.float32([500, 500]), 2.0))
    # 3: dense clusters (many pairs, several leaf splits), R = 5
    centres = rs.uniform(20, 380, (25, 2))
    q = centres[rs.integers(0, 25, 1000)] + rs.normal(0, 4, (1000, 2))
    cases.append((np.clip(q, 0, 399).astype(np.float32), np.float32([400, 400]), 5.0))
    out = {"cases": np.int64(len(cases))}
    for k, (pos, world, radius) in enumerate(cases):
        lower, events, ids = oracle.ref_lower_sets(pos, float(world[0]), float(world[1]), radius, node_cap=10,
                                                   max_ids=256)
        assert lower.max() <= 256
        cnt, idx, _ = oracle.neighbours(pos, radius, 1024)
        for i in range(pos.shape[0]):
            mine = idx[i, : cnt[i]]
            mine = mine[mine < i]
            assert np.array_equal(mine, ids[i, : lower[i]]), f"oracle and reference disagree: case {k}, entity {i}"
        out[f"pos{k}"] = pos
        out[f"world{k}"] = world
        out[f"radius{k}"] = np.float32(radius)
        out[f"lower{k}"] = lower
        out[f"events{k}"] = events
        out[f"ids{k}"] = ids[:, : max(int(lower.max()), 1)]
    assert list(out["lower0"]) == [0, 1, 0, 0, 1]
    # the reference's own collision counter (debugData[1]) on its known-answer test
    assert list(np.cumsum(out["events0"])) == [0, 1, 1, 1, 2]
    np.savez(HERE / "ref_quadtree.npz", **out)


def ref_tree() -> None:
    """The reference's quad tree (depth 8, leaf capacity 10) after inserting 1000
    entities in id order, node and link records as uint32 words."""
    from oracle import oracle

    rs = np.random.default_rng(7)
    W, H = np.float32(300.0), np.float32(200.0)
    pos = rs.uniform([0, 0], [W, H], (1000, 2)).astype(np.float32)
    pos[500:530] = pos[499]  # a crowd on one point (the same-position rule)
    nodes, links = oracle.ref_export_tree(pos, float(W), float(H), node_cap=10)
    np.savez_compressed(HERE / "ref_tree.npz", pos=pos, world=np.float32([W, H]), nodes=nodes, links=links)


if __name__ == "__main__":
    test_map()
    ref_quadtree()
    ref_tree()
    print("fixtures written to", HERE)
