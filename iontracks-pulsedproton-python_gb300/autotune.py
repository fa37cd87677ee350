"""Autotuner for the fused step's launch shape.

For one grid it times every candidate shape -- the flat kernel, and the
streaming kernel over tile rows x shared-memory stages x consumer warps x
resident CTAs per SM x planes per work item -- with CUDA events on the
launching stream, on the real buffers, and keeps the fastest. Results are
cached per (device name, no_xy, nzb, dtype, wall, deposition) in a JSON file so
a configuration is tuned once per machine.

Only shapes the library accepts are timed (``pic_resolve_shape`` checks them
against shared memory and thread limits); the register file bounds how many
CTAs of a shape can actually be resident, which the timing then shows.

Steps per launch (temporal blocking in time): when the flat kernel wins, a
segment of idle steps is also timed as one CUDA graph of per-step launches
and as cooperative launches of 32 and 256 steps (``steps_per_launch``), and
the fastest is kept. Measured on GB300 the multi-step launch wins only on
the smallest grids (24 x 24 x 206: 9.7 against 10.2 us a step) and loses on
larger ones (48 x 48 x 206: 13.9 against 13.0 us).
"""

from __future__ import annotations

import ctypes
import itertools
import json
import os
import statistics
from pathlib import Path

import numpy as np

from . import _native as N
from .engine import SHAPE_FIELDS, apply_shape, resolve_shape

CACHE = Path(os.environ.get("PIC_TUNE_CACHE", Path(__file__).resolve().parent / "_build" / "tuning.json"))
_SMEM_PER_SM = 228 * 1024


def candidate_shapes(grid, quick: bool = False) -> list[dict]:
    """Launch shapes worth timing for this grid."""
    out = [{"variant": "flat"}]
    if grid.dtype != N.PIC_F32 or grid.no_xy < 16:
        return out
    out.append({"variant": "stream"})  # the library's own default shape
    kp = grid.kpitch
    tjs = (3, 5, 7, 8, 10, 12, 15) if quick else (2, 3, 4, 5, 6, 7, 8, 10, 12, 14, 15)
    cws = (8, 12, 13, 15, 16) if quick else (4, 6, 8, 10, 12, 13, 14, 15, 16)
    planes = (4, 16, 64) if quick else (4, 8, 16, 32, 64, 128)
    stage_counts = (4, 5, 6, 8) if quick else (4, 5, 6, 8, 10, 12, 16)
    for tj, cw, ctas, stages, li in itertools.product(tjs, cws, (1, 2), stage_counts, planes):
        if tj > grid.no_xy - 2:
            continue
        smem = (2 * stages * 8 + 127) // 128 * 128 + stages * (2 * (tj + 2) * kp + 2 * ((tj + 8) & ~3)) * 4
        if ctas * (smem + 3 * 1024) > _SMEM_PER_SM:
            continue
        ipt = -(-(tj * (kp // 4)) // (cw * 32))
        # thread limits of the kernel's instantiations (2 to 4 items a thread
        # also come in wider forms, up to 17 warps, held to fewer registers)
        threads = (cw + 1) * 32
        if ipt > 6 or threads > (544, 544, 544, 544, 288, 288)[ipt - 1]:
            continue
        regs = min((96, 128, 152, 168, 168, 168)[ipt - 1], 65536 // (-(-threads // 128) * 128))
        if ctas * (cw + 1) * 32 * regs > 65536:
            continue
        out.append(dict(variant="stream", tile_rows=tj, consumer_warps=cw, ctas_per_sm=ctas, stages=stages,
                        planes_per_item=li))
    return out


def _key(grid, with_deposition: bool) -> str:
    import torch

    name = torch.cuda.get_device_name()
    return f"{name}|{grid.no_xy}|{grid.nzb}|{grid.dtype}|{grid.wall}|{int(with_deposition)}"


def load_cache() -> dict:
    try:
        return json.loads(CACHE.read_text())
    except Exception:
        return {}


def save_cache(d: dict) -> None:
    CACHE.parent.mkdir(parents=True, exist_ok=True)
    tmp = CACHE.with_suffix(".tmp")
    tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
    os.replace(tmp, CACHE)


def time_shape(engine, shape: dict, reps: int = 10, warmup: int = 2, with_deposition: bool = True) -> float:
    """Median milliseconds of one fused step with this launch shape."""
    torch = engine.torch
    g = N.PicGrid.from_buffer_copy(engine.grid)
    for k in SHAPE_FIELDS:
        setattr(g, k, 0)
    apply_shape(g, shape)
    lib = engine.lib
    st = torch.cuda.current_stream(engine.device)
    dens = engine.dens[0].data_ptr() if with_deposition else None
    cur = engine.parity
    times = []
    for r in range(warmup + reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        rc = lib.pic_step(ctypes.byref(g), engine.pos[cur].data_ptr(), engine.neg[cur].data_ptr(),
                          engine.pos[cur ^ 1].data_ptr(), engine.neg[cur ^ 1].data_ptr(), dens, None,
                          engine.tally[0].data_ptr(), engine.workspace.data_ptr(), engine.workspace.numel(),
                          st.cuda_stream)
        N.check(rc, "pic_step")
        b.record(st)
        cur ^= 1
        if r >= warmup:
            times.append((a, b))
    torch.cuda.synchronize(engine.device)
    engine.check_status()
    return statistics.median(x.elapsed_time(y) for x, y in times)


MULTI_CANDIDATES = (32, 256)
MULTI_TIMED_STEPS = 128
MULTI_MAX_CELLS = 8_000_000  # larger grids are bandwidth-bound: one launch a step


def time_segment(engine, steps_per_launch: int, n_steps: int = MULTI_TIMED_STEPS, reps: int = 3) -> float:
    """Median milliseconds per step of ``n_steps`` idle steps with the
    engine's shape and ``steps_per_launch`` (0: one CUDA graph of per-step
    launches; K: cooperative launches of up to K steps)."""
    torch = engine.torch
    lib = engine.lib
    g = N.PicGrid.from_buffer_copy(engine.grid)
    g.steps_per_launch = int(steps_per_launch)
    st = torch.cuda.current_stream(engine.device)
    off = np.zeros(n_steps + 1, dtype=np.int64)  # no tracks
    tally = torch.zeros((n_steps, 4), dtype=torch.float64, device=engine.device)
    args = (ctypes.byref(g), engine.pos[0].data_ptr(), engine.neg[0].data_ptr(), engine.pos[1].data_ptr(),
            engine.neg[1].data_ptr(), 0, n_steps, engine.xs.data_ptr(), engine.ys.data_ptr(), off.ctypes.data,
            engine.dens[0].data_ptr(), engine.dens[1].data_ptr(), 0, engine.counts.data_ptr(), tally.data_ptr(),
            engine.workspace.data_ptr(), engine.workspace.numel(), st.cuda_stream)
    graph = None
    if steps_per_launch <= 1:
        h = ctypes.c_void_p()
        N.check(lib.pic_graph_create(*args, ctypes.byref(h)), "pic_graph_create")
        graph = h.value
    times = []
    try:
        for r in range(reps + 1):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(st)
            if graph is not None:
                N.check(lib.pic_graph_launch(graph, st.cuda_stream), "pic_graph_launch")
            else:
                N.check(lib.pic_run_segment(*args), "pic_run_segment")
            b.record(st)
            if r > 0:
                times.append((a, b))
        torch.cuda.synchronize(engine.device)
    finally:
        if graph is not None:
            lib.pic_graph_destroy(graph)
    engine.check_status()
    return statistics.median(x.elapsed_time(y) for x, y in times) / n_steps


def tune_steps_per_launch(engine, verbose: bool = False):
    """``(steps_per_launch, [(K, ms per step), ...])`` for the engine's
    resolved shape: 0 unless a flat float32 grid of at most
    MULTI_MAX_CELLS cells runs faster with multi-step launches."""
    g = engine.grid
    cells = int(g.no_xy) ** 2 * int(g.kpitch)
    if resolve_shape(g)["variant"] != "flat" or g.dtype != N.PIC_F32 or cells > MULTI_MAX_CELLS:
        return 0, []
    tried = [(0, time_segment(engine, 0))]
    for k in MULTI_CANDIDATES:
        tried.append((k, time_segment(engine, k)))
    if verbose:
        for k, ms in tried:
            print(f"  steps_per_launch {k:3d}: {1e3 * ms:7.2f} us/step", flush=True)
    return min(tried, key=lambda t: t[1])[0], tried


def tune(engine, quick: bool = False, reps: int = 10, with_deposition: bool = True, use_cache: bool = True,
         verbose: bool = False) -> dict:
    """Fastest launch shape for the engine's grid (and set it on the engine).

    Returns ``{"shape": {...}, "ms": t, "tried": [(shape, ms), ...]}``.
    """
    key = _key(engine.grid, with_deposition)
    cache = load_cache() if use_cache else {}
    if key in cache:
        best = cache[key]
        apply_shape(engine.grid, best["shape"])
        return best
    tried = []
    for shape in candidate_shapes(engine.grid, quick=quick):
        g = N.PicGrid.from_buffer_copy(engine.grid)
        for k in SHAPE_FIELDS:
            setattr(g, k, 0)
        try:
            apply_shape(g, shape)
            resolve_shape(g)
        except Exception:
            continue
        ms = time_shape(engine, shape, reps=reps, with_deposition=with_deposition)
        tried.append((shape, ms))
        if verbose:
            print(f"  {ms:8.4f} ms  {shape}", flush=True)
    shape, ms = min(tried, key=lambda t: t[1])
    for k in SHAPE_FIELDS:
        setattr(engine.grid, k, 0)
    apply_shape(engine.grid, shape)
    spl, multi = tune_steps_per_launch(engine, verbose=verbose)
    if spl > 1:
        shape = dict(shape, steps_per_launch=spl)
        apply_shape(engine.grid, shape)
    best = {"shape": shape, "ms": ms, "tried": tried, "steps_per_launch": multi}
    if use_cache:
        cache[key] = {"shape": shape, "ms": ms}
        save_cache(cache)
    return best
