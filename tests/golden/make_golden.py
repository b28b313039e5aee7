"""Generates tests/golden/kat.json from the oracle (run once; the outputs are
then frozen: later oracle changes that move them fail the CPU tests).

Contents: mix32 / lattice-hash / seed-key outputs, each noise type's FP64
value at fixed points, the two synthetic programs' FP64 values at fixed
points, and hand-derivable analytic cases (sphere, torus, smoothMin).
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import importlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as O  # noqa: E402

W = importlib.import_module("unnatural-planets_gb300.workloads")


def main():
    L = O.lib()
    rng = np.random.default_rng(20261203)
    mix_in = [0, 1, 2, 3, 0xFFFFFFFF, 0x9E3779B9, 12345678, 1337, 42]
    lat_in = [(0, 0, 0, 0), (1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0), (-1, -1, -1, 7), (123, -456, 789, 0xDEADBEEF),
              (2147483647, -2147483648, 5, 99)]
    pts = rng.uniform(-8, 8, size=(16, 3)).astype(np.float32)
    noise = {}
    for t in range(5):
        noise[str(t)] = O.noise(dict(type=t, seed=7), pts).tolist()
    for d in range(3):
        for op in range(7):
            noise[f"5_{d}_{op}"] = O.noise(dict(type=5, seed=7, distance=d, operation=op), pts).tolist()
    noise["fbm_simplex4"] = O.noise(dict(type=3, fractal=1, octaves=4, frequency=0.7, seed=3), pts).tolist()
    noise["ridged_perlin6"] = O.noise(dict(type=2, fractal=2, octaves=6, frequency=0.3, seed=3), pts).tolist()
    sp = rng.uniform(-1.5, 1.5, size=(32, 3)).astype(np.float32)
    out = dict(
        mix32=[[x, int(L.orc_mix32(x))] for x in mix_in],
        lattice_hash=[[*a, int(L.orc_lattice_hash(*a))] for a in lat_in],
        seed_key=[[s, int(L.orc_seed_key(s))] for s in [0, 1, 7, 42, 1337]],
        noise_points=pts.tolist(),
        noise=noise,
        synth_points=sp.tolist(),
        synth_c1=O.synth_points(W.sphere_fbm(), sp).tolist(),
        synth_c2=O.synth_points(W.torus_spheres_ridged_cellular(), sp).tolist(),
    )
    (Path(__file__).parent / "kat.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
