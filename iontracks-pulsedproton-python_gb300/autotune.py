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
"""

from __future__ import annotations

import ctypes
import itertools
import json
import os
import statistics
from pathlib import Path

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
    tjs = (3, 5, 7, 10, 12) if quick else (2, 3, 4, 5, 6, 7, 8, 10, 12, 14)
    cws = (8, 12, 16) if quick else (4, 6, 8, 10, 12, 16)
    planes = (4, 16, 64) if quick else (4, 8, 16, 32, 64, 128)
    stage_counts = (4, 5, 6, 8) if quick else (4, 5, 6, 8, 10, 12, 16)
    for tj, cw, ctas, stages, li in itertools.product(tjs, cws, (1, 2), stage_counts, planes):
        if tj > grid.no_xy - 2:
            continue
        smem = (2 * stages * 8 + 127) // 128 * 128 + stages * (2 * (tj + 2) * kp + 2 * ((tj + 8) & ~3)) * 4
        if ctas * (smem + 3 * 1024) > _SMEM_PER_SM:
            continue
        ipt = -(-(tj * (kp // 4)) // (cw * 32))
        if ipt > 6 or (cw + 1) * 32 > (544, 416, 352, 288, 288, 288)[ipt - 1]:
            continue
        regs = (96, 128, 152, 168, 168, 168)[ipt - 1]
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
    best = {"shape": shape, "ms": ms, "tried": tried}
    if use_cache:
        cache[key] = {"shape": shape, "ms": ms}
        save_cache(cache)
    for k in SHAPE_FIELDS:
        setattr(engine.grid, k, 0)
    apply_shape(engine.grid, shape)
    return best
