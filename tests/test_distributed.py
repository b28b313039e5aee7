"""Chunk sharding over ranks and the one host-side exchange (per-chunk
counts -> global offsets), on CPU: world size 2 with gloo, rendezvous on
127.0.0.1. The meshes come from the oracle's contouring of each chunk."""
from __future__ import annotations

import importlib
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np

from conftest import workloads

HERE = Path(__file__).resolve().parent


def _dist():
    return importlib.import_module("unnatural-planets_gb300.distributed")


def test_shards_partition_and_balance():
    W = workloads()
    _, chunks = W.chunk_set(n_planets=8, n_chunks=57, seed=3, edge_lo=8, edge_hi=64)
    sizes = [g.count for _, g in chunks]
    for world in (1, 2, 3, 4):
        parts = [_dist().shard_chunks(chunks, r, world) for r in range(world)]
        flat = sorted(c for p in parts for c in p)
        assert flat == list(range(len(chunks)))
        loads = [sum(sizes[c] for c in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)


def test_global_offsets_single_process():
    vo, io = _dist().global_offsets([0, 2, 1], [5, 7, 3], [12, 30, 6], 3)
    assert vo.tolist() == [0, 5, 8, 15] and io.tolist() == [0, 12, 18, 48]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gloo(O, tmp_path):
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()), WORLD_SIZE="2")
    procs = [subprocess.Popen([sys.executable, str(HERE / "dist_worker.py"), str(tmp_path)], env=dict(env, RANK=str(r)))
             for r in range(2)]
    for p in procs:
        assert p.wait(timeout=300) == 0
    views = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    assert views[0]["vo"] == views[1]["vo"] and views[0]["io"] == views[1]["io"]
    assert sorted(views[0]["mine"] + views[1]["mine"]) == list(range(10))
    # the same offsets from one process contouring every chunk
    W = workloads()
    planets, chunks = W.chunk_set(n_planets=4, n_chunks=10, seed=11, edge_lo=10, edge_hi=20)
    v = [0]
    i = [0]
    for p, g in chunks:
        m = O.contour_synth(planets[p], g, O.synth_points(planets[p], O.grid_positions(g)).astype(np.float32))
        v.append(v[-1] + len(m["positions"]))
        i.append(i[-1] + len(m["indices"]))
    assert views[0]["vo"] == v and views[0]["io"] == i
