"""Batched uneven chunks (up_batch_run) against per-chunk contouring.

The sampled values of every chunk match the FP64 oracle (1e-5); contouring
each chunk's values alone with up_contour gives bit-identical vertices and
indices to the chunk's slice of the batch; a second call (CUDA-graph replay)
gives identical outputs."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workloads

pytestmark = pytest.mark.gpu


def test_batch_matches_per_chunk(cuda, up, O):
    W = workloads()
    planets, chunks = W.chunk_set(n_planets=5, n_chunks=24, seed=3, edge_lo=12, edge_hi=40)
    ctx = up.Planet(program=planets[0])
    res = up.batch_run(ctx, planets, chunks, values=True)
    vo, io = res["vertex_offsets"], res["index_offsets"]
    off = 0
    for c, (p, g) in enumerate(chunks):
        n = g.count
        vals = res["values"][off:off + n]
        off += n
        ref = O.synth_points(planets[p], O.grid_positions(g))
        assert np.abs(vals - ref).max() <= 1e-5
        single = up.Planet(program=planets[p])
        m = up.abi.MeshOut()
        import ctypes as C
        st = single.lib.up_contour(single.h, 0, C.byref(g), vals.ctypes.data, C.byref(m))
        if st == up.abi.UP_ERR_EMPTY_MESH:
            assert io[c + 1] == io[c]
            continue
        pos, _, idx = single.contour(g, values=vals)
        assert np.array_equal(res["indices"][io[c]:io[c + 1]], idx)
        # vertices: same QEF inputs; only the Hermite normals' evaluation kernel differs
        assert np.allclose(res["positions"][vo[c]:vo[c + 1]], pos, rtol=0, atol=1e-5)
    again = up.batch_run(ctx, planets, chunks, values=True)
    assert np.array_equal(again["indices"], res["indices"])
    assert np.array_equal(again["positions"], res["positions"])
    assert np.array_equal(again["values"], res["values"])


def test_batch_rejects_bad_chunks(cuda, up):
    W = workloads()
    planets, chunks = W.chunk_set(n_planets=2, n_chunks=3, seed=1, edge_lo=8, edge_hi=12)
    ctx = up.Planet(program=planets[0])
    chunks[1] = (7, chunks[1][1])  # planet index out of range
    with pytest.raises(up.UpError) as e:
        up.batch_run(ctx, planets, chunks)
    assert e.value.status == up.abi.UP_ERR_INVALID_ARGUMENT


def test_batch_replay_writes_live_buffers(cuda, up):
    """batch_replay reuses the output struct of batch_run: the offset arrays
    and outputs it points at must still be alive (collected garbage in
    between), and the replay reproduces the first run."""
    import gc
    W = workloads()
    planets, chunks = W.chunk_set(n_planets=3, n_chunks=12, seed=4, edge_lo=12, edge_hi=32)
    ctx = up.Planet(program=planets[0])
    res = up.batch_run(ctx, planets, chunks, values=True)
    first = {k: np.copy(res[k]) for k in ("positions", "indices", "values")}
    gc.collect()
    junk = [np.full(1024, 7, np.uint64) for _ in range(256)]  # reuse of freed memory would show up here
    for _ in range(3):
        up.batch_replay(ctx, res)
    for k in first:
        assert np.array_equal(res[k], first[k]), k
    assert all((j == 7).all() for j in junk)


@pytest.mark.parametrize("form", [1, 2])
def test_batch_narrow_band_equals_exact(cuda, up, form):
    """Without a values buffer the batch samples its chunks with the narrow
    band of contouring; the meshes equal those of the exact sampling, bit for
    bit, in each replay form. (Each call plans its own chunk list and would
    otherwise replay whichever form it timed faster; the two forms agree with
    each other to 1e-5 in the vertices, not bit for bit.)"""
    W = workloads()
    planets, chunks = W.chunk_set(n_planets=6, n_chunks=40, seed=5, edge_lo=12, edge_hi=48)
    ctx = up.Planet(program=planets[0])
    assert ctx.lib.up_debug_set_batch_form(form) == 0
    try:
        exact = up.batch_run(ctx, planets, chunks, values=True)
        banded = up.batch_run(ctx, planets, chunks, values=False)
    finally:
        ctx.lib.up_debug_set_batch_form(0)
    for k in ("positions", "indices", "vertex_offsets", "index_offsets"):
        assert np.array_equal(exact[k], banded[k]), k


def test_batch_persistent_wait_runs_out(cuda, up):
    """The persistent form replays the batch as one cooperative launch whose
    phases meet at grid-wide barriers with bounded waits. With a wait limit
    of 1 ns the waits run out: the call returns UP_ERR_TIMEOUT and the launch
    ends (no block keeps waiting). With the default limit restored the next
    replay reproduces the first run."""
    W = workloads()
    planets, chunks = W.chunk_set(n_planets=4, n_chunks=16, seed=6, edge_lo=16, edge_hi=40)
    ctx = up.Planet(program=planets[0])
    assert ctx.lib.up_debug_set_batch_form(2) == 0   # plan the persistent form whatever its speed
    try:
        res = up.batch_run(ctx, planets, chunks, values=True)
    finally:
        ctx.lib.up_debug_set_batch_form(0)
    first = {k: np.copy(res[k]) for k in ("positions", "indices", "values")}
    try:
        ctx.lib.up_debug_set_wait_limit(1)
        with pytest.raises(up.UpError) as e:
            up.batch_replay(ctx, res)
        assert e.value.status == up.abi.UP_ERR_TIMEOUT
        assert b"barrier" in ctx.lib.up_last_error(ctx.h)
    finally:
        ctx.lib.up_debug_set_wait_limit(0)
    up.batch_replay(ctx, res)
    for k in first:
        assert np.array_equal(res[k], first[k]), k


@pytest.mark.parametrize("form", [1, 2])
def test_batch_forms_equal_per_chunk(cuda, up, form):
    """Both replayed forms (the stage launches, the persistent launch) give
    the meshes of one up_contour call per chunk, bit for bit."""
    import ctypes as C
    W = workloads()
    planets, chunks = W.chunk_set(n_planets=5, n_chunks=20, seed=8, edge_lo=12, edge_hi=36)
    ctx = up.Planet(program=planets[0])
    assert ctx.lib.up_debug_set_batch_form(form) == 0
    try:
        res = up.batch_run(ctx, planets, chunks, values=True)
        up.batch_replay(ctx, res)
    finally:
        ctx.lib.up_debug_set_batch_form(0)
    vo, io = res["vertex_offsets"], res["index_offsets"]
    off = 0
    for c, (p, g) in enumerate(chunks):
        n = g.count
        vals = res["values"][off:off + n]
        off += n
        single = up.Planet(program=planets[p])
        m = up.abi.MeshOut()
        if single.lib.up_contour(single.h, 0, C.byref(g), vals.ctypes.data, C.byref(m)) == up.abi.UP_ERR_EMPTY_MESH:
            assert io[c + 1] == io[c]
            continue
        pos, _, idx = single.contour(g, values=vals)
        assert np.array_equal(res["indices"][io[c]:io[c + 1]], idx)
        assert np.allclose(res["positions"][vo[c]:vo[c + 1]], pos, rtol=0, atol=1e-5)
