"""Benchmark of the planet SDF -> contour path on GB300.

Workload: the 512^3 torus + 8 spheres planet minus 6-octave ridged Perlin and
a cellular F2-F1 layer (seed 42, box [-1.6, 1.6]^3): one "step" is one fused
value + analytic-gradient sampling of the full 512^3 grid (134,217,728
samples). Also measured in the same run: the plain (value-only) kernel, the
full planet (sampling + dual contouring) in ms, and the same metric end to
end through the C ABI with pinned host output buffers.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU path (the oracle's FP32
restatement, per-sample callback, gradient by 6-tap central differences) on
the host cores; under torchrun only rank 0 runs it.

After the headline, rank 0 measures the other workloads of the path once
each ("extras" in the JSON line, each bounded to seconds):
  atlas      4096^2 texel atlas of the 512^3 planet's mesh (raster, synthetic
             coloring program, dilation 7, 8-bit) into device buffers
  adjoint    the 512^3 planet's program: value+gradient forward and the
             adjoint of L = mean(d^2) over its 25 parameters on 16,777,216
             points of its 0.05 shell
  batch      64 planets x 512 uneven chunks (1.8e8 samples): one batched
             call (graph replay) against one up_contour call per chunk
  fit        inverse fit of that program's 25 parameters, 300 Adam steps
             (lr 1e-2, octave frequencies in phase units) on 32M shell points
             plus a sign loss on the 256^3 grid; reports |theta - theta*| by
             parameter group and the SDF RMS against the FP64 oracle
  modes      reference-mode planet sphere/lakes/default, seed 0, 500^3 over
             [-2000, 2000]^3, land+water+navigation in one pass
  cpu_1t     the CPU baseline on one thread
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SDF+grad Gsamples/s at 512^3 (fused value+gradient; plain and ms/planet alongside)"
UNIT = "Gsamples/s"
CD_TAP = 1e-3  # central-difference tap distance of the CPU reference path (unit-scale planet)
# DRAM bytes (read + write) per sample of the fused grid kernel, from the ncu
# capture of the timed synth_grid_runs_kernel<1,2,1301> launch at 512^3
# (4.96 MB + 2,390.57 MB over 134,217,728 samples)
TRAFFIC_PER_SAMPLE_FUSED = 2395.53e6 / 134217728
# FP32 operations executed per sample by the fused grid kernel (FFMA x 2,
# FFMA2 x 4, FADD, FMUL per thread instruction) and its thread instructions per
# sample, from the ncu instruction counts of the same capture
EXEC_FP32_PER_SAMPLE_FUSED = 494.7
INSTR_PER_SAMPLE_FUSED = 711.1


def workload_config(grid: int, n: int) -> dict:
    """the config block of both arms' JSON lines (the same dict on both)"""
    return {"workload": f"torus+8 spheres - ridged perlin 6 oct + cellular F2-F1, seed 42, {grid}^3 over [-1.6,1.6]^3",
            "samples_per_step": grid ** 3, "parallelism": f"replicas x{n}",
            "l2": "no inputs; 2.1 GB of outputs per step (> 129 MB L2)" if grid >= 512 else "no inputs"}


def _pkg():
    return importlib.import_module("unnatural-planets_gb300")


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def _cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part", "hardware")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def _slab_groups(nz: int, slabs: int, groups: int) -> list[tuple[int, int]]:
    """`groups` runs of slabs // groups consecutive z-slabs, spread evenly over
    the grid's z extent (each run keeps every host thread busy)"""
    per = max(1, slabs // groups)
    out = []
    for k in range(groups):
        z0 = min(nz - per, int((k + 0.5) * nz / groups) - per // 2)
        out.append((max(0, z0), max(0, z0) + per))
    return out


def cpu_rate(P, grid, slabs: int, threads: int, grad: bool, groups: int = 4) -> tuple[float, float]:
    """Samples/s of the oracle's FP32 callback path over `slabs` z-slabs in
    `groups` runs spread evenly over z; returns (rate, seconds)."""
    from oracle import oracle as O
    runs = _slab_groups(int(grid.n[2]), slabs, groups)
    t = time.perf_counter()
    for z0, z1 in runs:
        if grad:
            O.synth_grid_fp32_cd(P, grid, z0, z1, CD_TAP, threads)
        else:
            O.synth_grid_fp32(P, grid, z0, z1, threads)
    dt = time.perf_counter() - t
    done = sum(z1 - z0 for z0, z1 in runs)
    return int(grid.n[0]) * int(grid.n[1]) * done / dt, dt


def cpu_planet(P, grid, threads: int) -> dict:
    """The reference's CPU flow for one planet (meshGeneration.cpp:32-44,
    updateByPosition then makeMesh): the oracle's FP32 per-sample callback
    over the whole grid on `threads` host threads, then the oracle's dual
    contouring of that grid (sequential, one thread)."""
    from oracle import oracle as O
    nz = int(grid.n[2])
    t0 = time.perf_counter()
    values = O.synth_grid_fp32(P, grid, 0, nz, threads)
    t1 = time.perf_counter()
    mesh = O.contour_synth(P, grid, values)
    t2 = time.perf_counter()
    return {"ms_per_planet": 1e3 * (t2 - t0), "sampling_ms": 1e3 * (t1 - t0), "contour_ms": 1e3 * (t2 - t1),
            "vertices": int(len(mesh["positions"])), "triangles": int(len(mesh["indices"])) // 3,
            "sample": f"the whole {grid.n[0]}x{grid.n[1]}x{nz} planet: FP32 per-sample callback on {threads} threads, "
                      "then dual contouring on one thread (FP64 Hermite normals and QEF)"}


def error_vs_fp64(up, W, planet, P, grid, d_dev, g_dev, mesh, threads: int) -> dict:
    """Error of each result against the FP64 oracle (a checker run after the
    timed regions): SDF values of both forms (d_dev holds the value-only grid,
    the last one sampled; the fused grid is sampled once more) and the fused
    gradients at 2^20 seeded grid points of the 512^3 grid, every vertex of the
    planet's mesh against the oracle's contouring of the value-only FP32 grid,
    and every covered texel of the 4096^2 atlas of that mesh."""
    import numpy as np
    import torch
    from oracle import oracle as O
    n = grid.count
    idx = np.unique(np.random.default_rng(2024).integers(0, n, size=1 << 20, dtype=np.int64))
    it = torch.from_numpy(idx).cuda()
    dv = d_dev[it].double().cpu().numpy()
    gv = torch.stack([g_dev[it], g_dev[n + it], g_dev[2 * n + it]], dim=1).double().cpu().numpy()
    # the fused form's own values at the same points: the grid is sampled once
    # more with gradients, then value-only again (the grid the mesh is checked on)
    planet.sdf_grid(grid, 1, outs=[d_dev, None, None], grad=g_dev)
    dvf = d_dev[it].double().cpu().numpy()
    planet.sdf_grid(grid, 1, outs=[d_dev, None, None])
    ref, rg = O.synth_points(P, O.grid_positions_at(grid, idx), grad=True, threads=threads)
    ev, evf = np.abs(dv - ref), np.abs(dvf - ref)
    eg = np.abs(gv - rg).max(axis=1) / np.maximum(1.0, np.abs(rg).max(axis=1))
    out = {"value": {"max": float(ev.max()), "rms": float(np.sqrt((ev ** 2).mean())), "samples": int(len(idx)), "tolerance": 1e-5,
                     "form": "value only"},
           "value_fused": {"max": float(evf.max()), "rms": float(np.sqrt((evf ** 2).mean())), "samples": int(len(idx)),
                           "tolerance": 1e-5, "form": "value + gradient"},
           "gradient": {"max_rel": float(eg.max()), "rms_rel": float(np.sqrt((eg ** 2).mean())),
                        "frac_above_1e-4": float((eg > 1e-4).mean()), "samples": int(len(idx))}}
    pos, nrm, tri = mesh
    om = O.contour_synth(P, grid, d_dev.cpu().numpy())
    step = np.array([(grid.hi[a] - grid.lo[a]) / (grid.n[a] - 1) for a in range(3)])
    same = len(pos) == len(om["positions"]) and np.array_equal(tri, om["indices"])
    if len(pos) == len(om["positions"]):
        ec = (np.abs(pos.astype(np.float64) - om["positions"]) / step).max(axis=1)
        out["vertices"] = {"max_cells": float(ec.max()), "rms_cells": float(np.sqrt((ec ** 2).mean())), "vertices": int(len(pos)),
                           "frac_above_1e-3_cell": float((ec > 1e-3).mean())}
    out["topology_bit_exact"] = bool(same)
    wh = 4096
    p2, n2, uv, i2 = W.quad_atlas(pos, nrm, tri, wh, wh)
    got = planet.texture(1, p2, n2, uv, i2, wh, wh, dilation=7, floats=True)
    want = O.texture(1, p2, n2, uv, i2, wh, wh, dilation=7, program=P, threads=threads)
    cov = want["owner"] >= 0
    tex = {"coverage_bit_exact": bool(np.array_equal(np.isnan(got["height_f"]), np.isnan(want["height_f"]))),
           "covered_texels": int(cov.sum())}
    for k in ("albedo", "special", "height"):
        a, b = got[k + "_f"][cov].astype(np.float64), want[k + "_f"][cov].astype(np.float64)
        e8 = np.abs(got[k].astype(int) - want[k].astype(int))[cov]
        tex[k] = {"max": float(np.abs(a - b).max()), "rms": float(np.sqrt(((a - b) ** 2).mean())),
                  "u8_frac_above_2": float((e8 > 2).mean())}
    out["texels"] = tex
    return out


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def _events(stream, fn, k):
    """mean CUDA-event duration (ms) of k calls of fn on stream"""
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
    torch.cuda.synchronize()
    for a, b in evs:
        a.record(stream)
        fn()
        b.record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / k


def _guard(fn):
    try:
        return fn()
    except Exception as e:  # reported in the JSON line, never hidden
        return {"error": f"{type(e).__name__}: {e}"}


def extra_atlas(up, W, planet, stream, pos0, nrm0, idx0):
    """4096^2 atlas of the 512^3 planet's mesh into device buffers"""
    import ctypes as C
    import torch
    wh = 4096
    p2, n2, uv, i2 = W.quad_atlas(pos0, nrm0, idx0, wh, wh)
    dev = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    P, N, U, I = dev(p2), dev(n2), dev(uv), dev(i2.astype("int32"))
    alb = torch.empty((wh, wh, 3), dtype=torch.uint8, device="cuda")
    spc = torch.empty((wh, wh, 2), dtype=torch.uint8, device="cuda")
    hgt = torch.empty((wh, wh), dtype=torch.uint8, device="cuda")
    m = up.abi.MeshIn(P.data_ptr(), N.data_ptr(), U.data_ptr(), I.data_ptr(), int(p2.shape[0]), int(i2.shape[0]))
    o = up.abi.TextureOut(alb.data_ptr(), spc.data_ptr(), hgt.data_ptr(), None, None, None)

    def step():
        st = planet.lib.up_texture(planet.h, up.abi.PURPOSE_LAND, C.byref(m), wh, wh, 7, C.byref(o))
        assert st == 0, st
    step()
    ms = _events(stream, step, 5)
    return {"ms": ms, "mtexels_s": wh * wh / ms / 1e3, "triangles": int(i2.shape[0]) // 3,
            "what": "4096^2: raster + synthetic coloring (3-oct value albedo, 2-oct simplex roughness, height) + dilation 7 + U8"}


def _shell(planet, n, half_width, seed):
    """n points uniform in {|d| < half_width} of planet (rejection from the
    [-1.6, 1.6]^3 box, candidates and their values on the GPU)."""
    import torch
    gen = torch.Generator(device="cuda").manual_seed(seed)
    got, have = [], 0
    while have < n:
        c = (torch.rand((1 << 25, 3), device="cuda", generator=gen) * 3.2 - 1.6).contiguous()
        d = planet.sdf_points(c, d=torch.empty(c.shape[0], device="cuda"))
        keep = c[d.abs() < half_width]
        got.append(keep)
        have += keep.shape[0]
    return torch.cat(got)[:n].contiguous()


def _morton_sorted(x):
    """the points in Morton (Z-curve) order of a 1024^3 grid over the [-1.6, 1.6]^3
    box: neighbours in space become neighbours in the array (the same set)"""
    import torch
    q = ((x + 1.6) * (1023 / 3.2)).clamp(0, 1023).to(torch.int64)

    def spread(v):
        v = (v | (v << 16)) & 0x030000FF
        v = (v | (v << 8)) & 0x0300F00F
        v = (v | (v << 4)) & 0x030C30C3
        return (v | (v << 2)) & 0x09249249
    code = spread(q[:, 0]) | (spread(q[:, 1]) << 1) | (spread(q[:, 2]) << 2)
    return x[torch.argsort(code)].contiguous()


def extra_adjoint(up, W, stream):
    """the value+adjoint configuration: the torus + 8 spheres - ridged Perlin +
    cellular planet, 16,777,216 points uniform in its 0.05 shell"""
    import torch
    P = W.torus_spheres_ridged_cellular()
    planet = up.Planet(program=P)
    planet.set_stream(stream.cuda_stream)
    n = 1 << 24
    x = _morton_sorted(_shell(planet, n, 0.05, seed=11))
    v = torch.empty(n, device="cuda")
    g = torch.empty((n, 3), device="cuda")
    nt = W.theta_count(P)
    dth = torch.empty(nt, device="cuda")
    fwd = lambda: planet.sdf_points(x, d=v, grad=g, want_grad=True)  # noqa: E731
    fwd()
    w = (2.0 / n) * v  # dL/dd of L = mean(d^2)
    bwd = lambda: planet.param_backward(x, w, dtheta=dth)  # noqa: E731
    bwd()
    f_ms, b_ms = _events(stream, fwd, 5), _events(stream, bwd, 5)
    return {"points": n, "theta": nt, "forward_ms": f_ms, "backward_ms": b_ms, "backward_gpoints_s": n / b_ms / 1e6,
            "what": "torus + 8 spheres - ridged perlin + cellular; forward value+dd/dp, backward dL/dtheta of mean(d^2) "
                    "over the 25 parameters, 16M points uniform in the 0.05 shell (Morton order, sorted once when generated)"}


def extra_batch(up, W, stream):
    import ctypes as C
    import torch
    planets, chunks = W.chunk_set()
    ctx = up.Planet(program=planets[0])
    ctx.set_stream(stream.cuda_stream)
    res = up.batch_run(ctx, planets, chunks, device=True)
    up.batch_replay(ctx, res)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        up.batch_replay(ctx, res)
    torch.cuda.synchronize()
    batch_ms = 1e3 * (time.perf_counter() - t0) / reps
    # one up_contour call per chunk into device buffers sized from the batch
    vo, io = res["vertex_offsets"], res["index_offsets"]
    ctxs = {}
    for p, _ in chunks:
        if p not in ctxs:
            ctxs[p] = up.Planet(program=planets[p])
            ctxs[p].set_stream(stream.cuda_stream)
    vmax = int(max(vo[c + 1] - vo[c] for c in range(len(chunks))))
    imax = int(max(io[c + 1] - io[c] for c in range(len(chunks))))
    pos = torch.empty((max(vmax, 1), 3), device="cuda")
    idx = torch.empty(max(imax, 1), dtype=torch.int32, device="cuda")

    def per_chunk():
        for p, g in chunks:
            m = up.abi.MeshOut(pos.data_ptr(), None, idx.data_ptr(), vmax, imax, 0, 0)
            st = ctxs[p].lib.up_contour(ctxs[p].h, 0, C.byref(g), None, C.byref(m))
            assert st in (0, up.abi.UP_ERR_EMPTY_MESH), st
    per_chunk()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    per_chunk()
    torch.cuda.synchronize()
    chunk_ms = 1e3 * (time.perf_counter() - t0)
    samples = sum(g.count for _, g in chunks)
    return {"chunks": len(chunks), "planets": len(planets), "samples": samples, "batched_ms": batch_ms,
            "per_chunk_ms": chunk_ms, "speedup": chunk_ms / batch_ms, "batched_gsamples_s": samples / batch_ms / 1e6,
            "vertices": int(vo[-1]), "triangles": int(io[-1]) // 3,
            "what": "wall time: one up_batch_run (graph replay) vs one up_contour per chunk, device outputs"}


def extra_fit(up, W, stream, steps=300):
    """inverse fit of the torus + spheres - ridged Perlin + cellular planet:
    theta* = the program's 25 parameters scaled by (1 + 0.05 U[-1,1]) from
    seed 1, theta0 = theta* scaled by (1 + 0.05 s U[-1,1]) from seed 2, with
    s the phase scale (f_min / f for octave frequencies, 1 otherwise); Adam
    moves u in theta = theta0 (1 + s u)"""
    import numpy as np
    import torch
    from oracle import oracle as O
    AG = importlib.import_module("unnatural-planets_gb300.autograd")
    P = W.torus_spheres_ridged_cellular()
    base = W.theta_of(P).astype(np.float64)
    t_star_np = (base * (1 + 0.05 * np.random.default_rng(1).uniform(-1, 1, size=base.shape))).astype(np.float32)
    t0 = (t_star_np * (1 + 0.05 * W.phase_scale(P, t_star_np) * np.random.default_rng(2).uniform(-1, 1, size=base.shape))).astype(np.float32)
    t_star = torch.from_numpy(t_star_np).cuda()
    target = up.Planet(program=P)
    target.set_stream(stream.cuda_stream)
    target.set_theta(t_star_np)
    n = 32 << 20
    x = _morton_sorted(_shell(target, n, 0.05, seed=21))
    gg = W.grid(W.GRID_C2, n=(256, 256, 256))
    xg = AG.grid_positions(gg)  # the grid kernel's sample positions
    d_star = target.sdf_points(x, d=torch.empty(n, device="cuda"))
    s_star = torch.sign(target.sdf_points(xg, d=torch.empty(xg.shape[0], device="cuda")))
    # theta = theta0 (1 + s u), Adam moves u; s: phase scale of theta0
    rel = AG.RelativeTheta(torch.tensor(t0, device="cuda"), torch.from_numpy(W.phase_scale(P, t0)).cuda())
    planet = up.Planet(program=W.torus_spheres_ridged_cellular())
    planet.set_stream(stream.cuda_stream)
    opt = torch.optim.Adam(rel.parameters(), lr=1e-2)
    err0 = float((rel().detach() - t_star).norm() / t_star.norm())

    def step():
        opt.zero_grad()
        theta = rel()
        loss = ((AG.sdf(theta, x, planet) - d_star) ** 2).mean() + torch.relu(-AG.sdf_grid(theta, gg, planet, xg) * s_star).mean()
        loss.backward()
        opt.step()
        return loss
    step()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(steps - 1):
        loss = step()
    torch.cuda.synchronize()
    ms = 1e3 * (time.perf_counter() - t) / (steps - 1)
    # final SDF against the FP64 oracle at theta* on 65536 of the shell points
    xs = x[: 1 << 16].cpu().numpy()
    theta = rel().detach()
    planet.set_theta(theta.cpu().numpy())
    fit = planet.sdf_points(xs)
    ref = O.synth_points(P, xs, theta=t_star_np.astype(np.float64))
    # relative error per parameter group (layout of workloads.theta_of)
    groups = W.theta_groups(P)

    def group_err(t):
        t = np.asarray(t, np.float64)
        return {g: float(np.linalg.norm(t[i] - t_star_np[i]) / np.linalg.norm(t_star_np[i])) for g, i in groups.items()}
    return {"steps": steps, "ms_per_step": ms, "points": n, "sign_points": int(xg.shape[0]), "loss": float(loss.detach()),
            "theta_rel_err_start": err0, "theta_rel_err_end": float((theta.detach() - t_star).norm() / t_star.norm()),
            "theta_rel_err_by_group_start": group_err(t0), "theta_rel_err_by_group_end": group_err(theta.detach().cpu().numpy()),
            "sdf_rms_vs_fp64_oracle": float(np.sqrt(np.mean((fit - ref) ** 2))),
            "what": "torus + 8 spheres - ridged perlin + cellular, 25 parameters; theta* = theta (1 + 0.05 U) seed 1, "
                    "theta0 = theta* (1 + 0.05 s U) seed 2 with s = f_min / f for octave frequencies (phase scale), 1 otherwise; "
                    "L = mean((d - d*)^2) on 32M points of the 0.05 shell (Morton order) + "
                    "mean(relu(-d sign(d*))) on 256^3 (forward through the grid kernel); Adam lr 1e-2 on u, "
                    "theta = theta0 (1 + s u); SDF RMS against the FP64 oracle at theta* on 65536 shell points"}


def extra_modes(up, stream):
    import torch
    planet = up.Planet("sphere", "lakes", "default", seed=0)
    planet.set_stream(stream.cuda_stream)
    g = up.abi.Grid.make((-2000, -2000, -2000), (2000, 2000, 2000), (500, 500, 500))
    n = g.count
    outs = [torch.empty(n, device="cuda") for _ in range(3)]
    fn = lambda: planet.sdf_grid(g, 7, outs=outs)  # noqa: E731
    fn()
    ms = _events(stream, fn, 3)
    # the land base mesh of the same planet (meshGenerateBaseLand): narrow-band
    # sampling inside up_contour, and contouring the exactly sampled grid
    import ctypes as C
    pos0, _, idx0 = planet.contour(g)
    V, I = len(pos0), len(idx0)
    pos = torch.empty((V, 3), device="cuda")
    nrm = torch.empty((V, 3), device="cuda")
    idx = torch.empty(I, dtype=torch.int32, device="cuda")
    mesh = up.abi.MeshOut(pos.data_ptr(), nrm.data_ptr(), idx.data_ptr(), V, I, 0, 0)

    def banded():
        assert planet.lib.up_contour(planet.h, 0, C.byref(g), None, C.byref(mesh)) == 0

    def full():
        planet.sdf_grid(g, 1, outs=[outs[0], None, None])
        assert planet.lib.up_contour(planet.h, 0, C.byref(g), C.c_void_p(outs[0].data_ptr()), C.byref(mesh)) == 0
    banded()
    full()
    return {"ms": ms, "gsamples_s": n / ms / 1e6, "fields": 3, "land_mesh_ms": _events(stream, banded, 3),
            "land_mesh_full_grid_ms": _events(stream, full, 3), "triangles": I // 3,
            "what": "sphere/lakes/default seed 0, 500^3 over [-2000,2000]^3: land+water+navigation in one pass (ms); "
                    "land mesh with narrow-band sampling (land_mesh_ms) and from the exactly sampled grid"}


def run_reference(args) -> None:
    ws, rank = _dist()
    if rank != 0:
        return
    up = _pkg()
    W = up.workloads
    P = W.torus_spheres_ridged_cellular()
    grid = W.grid(W.GRID_C2, n=(args.grid,) * 3)
    threads = os.cpu_count() or 1
    slabs = min(4 * threads, args.grid)
    for _ in range(args.warmup):
        cpu_rate(P, grid, 4, threads, grad=True)
    rates, secs = [], []
    for _ in range(args.steps):
        r, s = cpu_rate(P, grid, slabs, threads, grad=True)
        rates.append(r)
        secs.append(s)
    value = args.steps * slabs * args.grid * args.grid / sum(secs) / 1e9
    sample = (f"{slabs} z-slabs of {args.grid}x{args.grid} ({slabs * args.grid * args.grid} samples) per step in 4 runs spread evenly over z, "
              f"value + 6-tap central-difference gradient (h={CD_TAP})")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded planet program; no dataset)",
        "config": workload_config(args.grid, args.gpus),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample, "cpu": _cpu_model()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import numpy as np
    import torch
    import torch.distributed as dist

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl")
    up = _pkg()
    W = up.workloads
    P = W.torus_spheres_ridged_cellular()
    grid = W.grid(W.GRID_C2, n=(args.grid,) * 3)
    N = grid.count
    planet = up.Planet(program=P)
    stream = torch.cuda.current_stream()
    planet.set_stream(stream.cuda_stream)
    d = torch.empty(N, device="cuda")
    g = torch.empty(3 * N, device="cuda")

    def barrier():
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(fn, k):
        """per-step CUDA-event durations on the launching stream (ms)"""
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        barrier()
        t0 = time.perf_counter()
        for a, b in evs:
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier()
        return [a.elapsed_time(b) for a, b in evs], wall

    fused = lambda: planet.sdf_grid(grid, 1, outs=[d, None, None], grad=g)  # noqa: E731
    plain = lambda: planet.sdf_grid(grid, 1, outs=[d, None, None])  # noqa: E731
    try:
        gpu_id = "GPU-" + str(torch.cuda.get_device_properties(local).uuid).replace("GPU-", "")
    except Exception:
        gpu_id = str(local)
    # the sampler runs from warm-up to the end of the timed loops
    with Clocks(gpu_id) as clk:
        for _ in range(args.warmup):
            fused()
            plain()
        time.sleep(0.3)
        fused_ms, _ = timed(fused, args.steps)
        plain_ms, _ = timed(plain, args.steps)
    t_fused = sum(fused_ms) / len(fused_ms)
    if ws > 1:
        t = torch.tensor([t_fused], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_fused = float(t.item())
    value = ws * N / (t_fused * 1e-3) / 1e9
    t_plain = sum(plain_ms) / len(plain_ms)

    # full planet: sampling + dual contouring into device buffers
    pos0, nrm0, idx0 = planet.contour(grid)
    V, I = len(pos0), len(idx0)
    pos = torch.empty((V, 3), device="cuda")
    nrm = torch.empty((V, 3), device="cuda")
    idx = torch.empty(I, dtype=torch.int32, device="cuda")
    import ctypes as C
    mesh = up.abi.MeshOut(pos.data_ptr(), nrm.data_ptr(), idx.data_ptr(), V, I, 0, 0)

    def planet_step():
        st = planet.lib.up_contour(planet.h, 0, C.byref(grid), None, C.byref(mesh))
        assert st == 0, st
    for _ in range(max(1, args.warmup)):
        planet_step()
    planet_ms, planet_wall = timed(planet_step, args.steps)

    # the same planet from the exactly sampled full grid (as the reference's
    # marching cubes samples it): up_sdf_grid into device memory, then contour
    def planet_full_step():
        plain()
        st = planet.lib.up_contour(planet.h, 0, C.byref(grid), C.c_void_p(d.data_ptr()), C.byref(mesh))
        assert st == 0, st
    planet_full_step()
    planet_full_ms, _ = timed(planet_full_step, args.steps)

    # end to end through the C ABI with pinned host outputs (D2H inside the timed region)
    dh = torch.empty(N, pin_memory=True)
    gh = torch.empty(3 * N, pin_memory=True)
    e2e_fn = lambda: planet.sdf_grid(grid, 1, outs=[dh, None, None], grad=gh)  # noqa: E731
    e2e_fn()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_fn()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    barrier()
    if ws > 1:  # the slowest rank's time, as for the device-timed value
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())

    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return
    # roofline: FP32-pipe bound kernel; algorithmic FLOPs from the oracle's count
    flops = W.FLOPS_PER_SAMPLE_C2 * N
    achieved = flops / (t_fused * 1e-3) / 1e12
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    max_mhz = peaks.get("sm_max_mhz", 2070.0)
    fp32_peak = sms * 128 * 2 * max_mhz * 1e6 / 1e12
    # CPU baseline (rank 0, bounded samples): sampling rates over z-slabs
    # spread over the grid, and one whole planet (sampling + contouring)
    threads = os.cpu_count() or 1
    slabs = min(4 * threads, args.grid)
    cpu_grad, cpu_s = cpu_rate(P, grid, slabs, threads, grad=True)
    cpu_plain, _ = cpu_rate(P, grid, slabs, threads, grad=False)
    cpu_pl = _guard(lambda: cpu_planet(P, grid, threads))
    # error of each result against the FP64 oracle (checker, after all timing)
    errors = _guard(lambda: error_vs_fp64(up, W, planet, P, grid, d, g, (pos0, nrm0, idx0), threads))
    extras = {}
    if not args.no_extras:
        extras["atlas"] = _guard(lambda: extra_atlas(up, W, planet, stream, pos0, nrm0, idx0))
        extras["adjoint"] = _guard(lambda: extra_adjoint(up, W, stream))
        extras["batch"] = _guard(lambda: extra_batch(up, W, stream))
        extras["fit"] = _guard(lambda: extra_fit(up, W, stream))
        extras["modes"] = _guard(lambda: extra_modes(up, stream))
        extras["cpu_1t"] = _guard(lambda: {"value": cpu_rate(P, grid, 1, 1, grad=True)[0] / 1e9,
                                           "plain_value": cpu_rate(P, grid, 1, 1, grad=False)[0] / 1e9, "unit": UNIT,
                                           "sample": f"1 z-slab of {args.grid}x{args.grid}, one thread"})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_fused, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded planet program; no dataset)",
        "config": workload_config(args.grid, ws),
        "plain_gsamples_s": ws * N / (t_plain * 1e-3) / 1e9, "plain_ms": t_plain,
        "ms_per_planet": sum(planet_ms) / len(planet_ms),
        "ms_per_planet_full_grid": sum(planet_full_ms) / len(planet_full_ms),
        "planet": {"what": f"{args.grid}^3 planet mesh into device buffers: up_contour samples the grid with the narrow band "
                           "(noise evaluated where |base| <= noise bound + one grid step; the mesh is bit-identical to contouring "
                           "the full grid), then dual contouring (signs, count, scan, emit, Hermite, QEF, quads); "
                           "ms_per_planet_full_grid samples every point exactly first (up_sdf_grid) and contours those values",
                   "vertices": V, "triangles": I // 3},
        "e2e": {"value": ws * N / e2e_s / 1e9, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 16 * N,
                "what": "up_sdf_grid value+gradient into pinned host buffers"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "traffic": TRAFFIC_PER_SAMPLE_FUSED * N,
                     "traffic_source": "dram read+write of the timed synth_grid_runs_kernel<1,2,1301> launch from one ncu "
                                       f"capture of this workload at 512^3 ({TRAFFIC_PER_SAMPLE_FUSED:.2f} B/sample: writes of 16 B "
                                       "per sample and about 12 % more, no re-reads), per sample times this launch's samples",
                     "peak_source": f"nominal FP32: {sms} SMs x 128 lanes x 2 x {max_mhz:.0f} MHz (MEASURED_PEAKS.json has no FP32 figure)",
                     "flops_per_sample": W.FLOPS_PER_SAMPLE_C2,
                     "flops_definition": "value path, counted by the oracle's operation-counting FP32 scalar (FMA = 2)",
                     "value_gradient_fwd_mode": {
                         "flops_per_sample": W.FLOPS_PER_SAMPLE_C2_FWD_GRAD,
                         "achieved": W.FLOPS_PER_SAMPLE_C2_FWD_GRAD * N / (t_fused * 1e-3) / 1e12,
                         "frac": W.FLOPS_PER_SAMPLE_C2_FWD_GRAD * N / (t_fused * 1e-3) / 1e12 / fp32_peak,
                         "note": "value with dd/dp counted in sparse forward mode by the oracle: an upper bound on the gradient's "
                                 "arithmetic; the kernel's closed-form derivatives need far fewer operations, so this fraction "
                                 "overstates how busy the FP32 pipe is (exec_fp32 below is what it executes)"},
                     "exec_fp32": {"flops_per_sample": EXEC_FP32_PER_SAMPLE_FUSED,
                                   "achieved": EXEC_FP32_PER_SAMPLE_FUSED * N / (t_fused * 1e-3) / 1e12,
                                   "frac": EXEC_FP32_PER_SAMPLE_FUSED * N / (t_fused * 1e-3) / 1e12 / fp32_peak,
                                   "source": "FP32 operations the fused kernel executes per sample (FFMA and FFMA2 lanes x 2, FADD, "
                                             "FMUL), from the ncu instruction counts of this workload at 512^3 (profiles/)"},
                     "note": "the kernel is instruction-issue bound (about 82 % issue active): per sample it issues about "
                             f"{INSTR_PER_SAMPLE_FUSED:.0f} thread instructions, of which the lattice hashes and face setup of the "
                             "Perlin octaves, the cellular keys (integer min/max, bit masks), addressing and control flow are "
                             "the non-FP32 share; see profiles/",                     "hbm_view": {"algorithmic_bytes": 16 * N, "achieved_gbs": 16 * N / (t_fused * 1e-3) / 1e9,
                                  "peak_gbs": peaks.get("hbm_gbs"), "frac": (16 * N / (t_fused * 1e-3) / 1e9) / peaks["hbm_gbs"]
                                  if peaks.get("hbm_gbs") else None, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"}},
        "cpu_baseline": {"value": cpu_grad / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{slabs} z-slabs of {args.grid}x{args.grid} per leg in 4 runs spread evenly over z; "
                                   "value+gradient by 6-tap central differences",
                         "plain_value": cpu_plain / 1e9, "cpu": _cpu_model(),
                         "ms_per_planet": cpu_pl.get("ms_per_planet") if isinstance(cpu_pl, dict) else None, "planet": cpu_pl},
        "planet_speedup_vs_cpu": (cpu_pl["ms_per_planet"] / (sum(planet_ms) / len(planet_ms))) if "ms_per_planet" in cpu_pl else None,
        "error_vs_fp64": errors,
        "gpu_launches": args.steps,
        "clocks": clk.summary(),
        "extras": extras,
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def run_only(args) -> None:
    """one secondary workload alone (for profiling captures): prints its result"""
    import torch
    up = _pkg()
    W = up.workloads
    stream = torch.cuda.current_stream()
    if args.only == "atlas":
        P = W.torus_spheres_ridged_cellular()
        planet = up.Planet(program=P)
        planet.set_stream(stream.cuda_stream)
        pos0, nrm0, idx0 = planet.contour(W.grid(W.GRID_C2, n=(args.grid,) * 3))
        r = extra_atlas(up, W, planet, stream, pos0, nrm0, idx0)
    elif args.only == "adjoint":
        r = extra_adjoint(up, W, stream)
    elif args.only == "batch":
        r = extra_batch(up, W, stream)
    elif args.only == "fit":
        r = extra_fit(up, W, stream)
    else:
        r = extra_modes(up, stream)
    print(json.dumps({"only": args.only, **r}), flush=True)


def make_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--grid", type=int, default=512, help="grid edge (512 is the benchmark; smaller for profiling captures)")
    ap.add_argument("--no-extras", action="store_true", help="skip the secondary workloads (atlas, adjoint, batch, fit, modes)")
    ap.add_argument("--only", choices=["atlas", "adjoint", "batch", "fit", "modes"],
                    help="run one secondary workload alone and print its result (profiling captures)")
    return ap


def main():
    args = make_parser().parse_args()
    if args.only:
        run_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
