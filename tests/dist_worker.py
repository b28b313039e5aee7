"""One rank of tests/test_distributed.py (CPU, gloo): contours its shard of a
small chunk set with the oracle and exchanges the per-chunk counts. Writes
its view of the global offsets as JSON. Test infrastructure."""
from __future__ import annotations

import importlib
import json
import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402
import torch.distributed as dist  # noqa: E402

from oracle import oracle as O  # noqa: E402


def main(out_dir: str):
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    dist.init_process_group("gloo")
    D = importlib.import_module("unnatural-planets_gb300.distributed")
    W = importlib.import_module("unnatural-planets_gb300.workloads")
    planets, chunks = W.chunk_set(n_planets=4, n_chunks=10, seed=11, edge_lo=10, edge_hi=20)
    mine = D.shard_chunks(chunks, rank, world)
    vc, ic = [], []
    for c in mine:
        p, g = chunks[c]
        vals = O.synth_points(planets[p], O.grid_positions(g)).astype(np.float32)
        m = O.contour_synth(planets[p], g, vals)
        vc.append(len(m["positions"]))
        ic.append(len(m["indices"]))
    vo, io = D.global_offsets(mine, vc, ic, len(chunks))
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"mine": mine, "vo": vo.tolist(), "io": io.tolist()}))
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main(sys.argv[1])
