"""Batched runs: many independent chamber configurations on one GB300 at once.

``run_batched_b200(configs)`` returns one reference :class:`Result` per
configuration -- the same results ``run_simulation_b200`` gives for each of
them alone -- but advances all grids together (the track centres drawn on the
host one chunk of global steps ahead of the device, feeder.py): each global
step is one fused-step launch over every active grid, and the tracks of every
grid are deposited in binned tiles, one launch pair per group of up to eight
global steps (``pic_batched_segment``). The grids may differ
in every respect: size, voltage and gap (hence time step and coefficients),
dose rate, pulse length, step count, wall, seed.

``saturation_sweep_configs()`` builds the 64-configuration saturation sweep:
voltages log-spaced over 25-400 V, gaps of 0.1/0.2/0.3 cm, dose rates
log-uniform over 1-100 Gy/s, pulse lengths 100-1000 us at 50 Hz, 5 or 10 um
voxels with sampled radii 0.008-0.03 cm, seeds 1-64, the random choices drawn
from a fixed meta-seed.
"""

from __future__ import annotations

import copy
import ctypes
import os
import threading
import warnings
from concurrent.futures import ThreadPoolExecutor
from time import perf_counter
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from .config import SimulationConfig
from .engine import make_grid, nvtx_range
from .feeder import TrackFeeder
from .pulses import TrackSampler, build_track_schedule
from .state import Diagnostics, collection_efficiency

# The batched step runs 4 resident 256-thread blocks per SM (float32, 64
# registers).
# Items per block are chosen per phase for about WAVES blocks per resident
# slot on phases of at least SMALL_PHASE_ITEMS items, one block per slot
# below: few, long blocks amortise each block's set-up and reduction. Measured
# over the 64-configuration sweep (device ms of the phases with 60-64 / 40-59
# / 20-39 / 12-19 / 3-11 active grids), blocks per slot 1: 229 / 264 / 251 /
# 27.0 / 110; 2: 206 / 234 / 210 / 26.5 / 116; 4: 199 / 216 / 204 / 27.5 /
# 127; 8: 197 / 218 / 211 / 28.8 / 146; 16: 205 / 230 / 228 / 32 / 185.
BLOCKS_PER_SM = 4
WAVES = 4
WAVES_SMALL = 1
SMALL_PHASE_ITEMS = 10_000_000  # four-vector items a step (4e7 voxels)
MIN_ITEMS_PER_BLOCK = 256
MAX_ITEMS_PER_BLOCK = 1 << 16
# Phases with at most this many active grids step each grid alone with the
# single-grid kernels (pic_run_segment on its slices of the packed buffers):
# there the batched launch is bound by its per-block table and reduction work
# (23 us a step for one 53 x 53 x 208 grid), the flat step kernel is not.
SOLO_MAX_GRIDS = 2


# The streaming batched step (pic_batched_stream_*): 15 consumer warps of up to
# three k-vectors each; a grid's tile is as many rows as those fill and a
# ring stage of any grid stays under STREAM_STAGE_BYTES, so that four stages
# fit in shared memory; about STREAM_ITEMS_PER_SM items per SM and global
# step, which the CTAs take from a device-wide queue. Measured over the
# 64-configuration sweep (device ms of the phases with 60-64 / 40-59 / 20-39
# active grids): 6 items per SM 190 / 211 / 219, 3 items 179 / 197 / 195,
# 2 items 177 / 195 / 195, 1 item 176 / 198 / 197; the flat step 200 / 217 /
# 205. Fewer, longer items pay each item's two priming planes and its tally
# slot less often.
STREAM_WARPS = 15
STREAM_IPT = 3
STREAM_STAGE_BYTES = 54 * 1024
STREAM_ITEMS_PER_SM = 2
# variant="mixed" takes the streaming step on the phases whose active grids
# hold at least this many interior voxels (fields of ~0.6 GB and more, several
# times the L2), the flat step on the rest: in the same measurement the flat
# step was the faster one with 12-19 grids (3.1e7 voxels a step: 27.7 against
# 28.5 ms) and with 3-11 grids (7.8e6: 128 against 168 ms), where the
# streaming items are short and the step waits on the slowest CTA. While a
# float64 re-run runs beside the batch, "mixed" steps flat: the streaming step
# holds every SM's shared memory, so the re-run's kernels find no room beside
# it. Even so, end to end on the sweep (which re-runs one configuration in
# float64) "mixed" took 1.179-1.182 s against 1.165-1.168 s all flat, so
# "auto" is the flat step; "mixed" pays on sweeps without a re-run (7 % less
# device time without one).
STREAM_MIN_VOXELS = 40_000_000


def stream_phase(shapes, active, variant: str = "mixed", dtype: str = "float32", persistent: bool = False) -> bool:
    """Whether a phase of a batched run (grids ``active``, ``shapes[c]`` =
    (no_xy, nzb, kpitch)) takes the streaming batched step."""
    if variant == "stream":
        return True
    if variant != "mixed" or dtype != "float32" or persistent:
        return False
    vox = sum((int(shapes[c][0]) - 2) ** 2 * (int(shapes[c][1]) - 2) for c in active)
    return vox >= STREAM_MIN_VOXELS


def _stage_floats(tj: int, kp: int) -> int:
    return 2 * (tj + 2) * kp + 2 * ((tj + 8) & ~3)


def stream_tile_rows(no_xy: int, kpitch: int, warps: int = STREAM_WARPS) -> int:
    """Interior rows of a grid's tiles in the streaming batched step."""
    tj = max(1, min(int(no_xy) - 2, (STREAM_IPT * 32 * warps) // (int(kpitch) // 4)))
    while tj > 1 and _stage_floats(tj, int(kpitch)) * 4 > STREAM_STAGE_BYTES:
        tj -= 1
    return tj


def _stream_items(shapes, active, sms: int, warps: int = STREAM_WARPS):
    """The work items of one streaming batched launch over the ``active``
    grids (``shapes[c]`` = (no_xy, nzb, kpitch)): rows (grid, cj_lo, ci_lo,
    ci_hi) that cover every interior row and plane of each active grid once,
    grouped by grid, grids with the longest items first; and the tile rows of
    every grid. Items are sized for about STREAM_ITEMS_PER_SM per SM."""
    tile = np.array([stream_tile_rows(n, kp, warps) for n, _, kp in shapes], dtype=np.int32)
    act = [int(c) for c in active]
    vox = sum((shapes[c][0] - 2) ** 2 * (shapes[c][1] - 2) for c in act)
    target = max(1.0, vox / (STREAM_ITEMS_PER_SM * max(1, sms)))
    plan = []
    for c in act:
        n, nzb, _ = shapes[c]
        tj = int(tile[c])
        li = int(np.clip(np.ceil(target / (tj * (nzb - 2))), 2, n - 2))
        ranges = -(-(n - 2) // li)
        li = -(-(n - 2) // ranges)  # even split of the planes
        plan.append((tj * li * nzb, c, tj, li))
    rows = []
    for _, c, tj, li in sorted(plan, key=lambda p: (-p[0], p[1])):
        n = shapes[c][0]
        for i0 in range(1, n - 1, li):
            i1 = min(i0 + li, n - 1)
            for j0 in range(1, n - 1, tj):
                rows.append((c, j0, i0, i1))
    return np.array(rows, dtype=np.int32).reshape(-1, 4), tile


class PicBatchStream(ctypes.Structure):
    _fields_ = [
        ("n_cfgs", ctypes.c_int32),
        ("n_items", ctypes.c_int32),
        ("consumer_warps", ctypes.c_int32),
        ("stages", ctypes.c_int32),
        ("stage_floats", ctypes.c_int32),
        ("ipt", ctypes.c_int32),
        ("workspace", ctypes.c_void_p),
        ("workspace_bytes", ctypes.c_int64),
    ]


def items_per_block(total_items: int, sms: int) -> int:
    """Work items per block for a phase of ``total_items`` items."""
    waves = WAVES if int(total_items) >= SMALL_PHASE_ITEMS else WAVES_SMALL
    want = -(-int(total_items) // (waves * BLOCKS_PER_SM * max(1, sms)))
    want = -(-want // 256) * 256
    return max(MIN_ITEMS_PER_BLOCK, min(MAX_ITEMS_PER_BLOCK, want))


class PicBatchCfg(ctypes.Structure):
    _fields_ = [
        ("field_off", ctypes.c_int64),
        ("dens_off", ctypes.c_int64),
        ("counts_off", ctypes.c_int64),
        ("tally_off", ctypes.c_int64),
        ("grid", N.PicGrid),
    ]


class PicBatchLaunch(ctypes.Structure):
    _fields_ = [
        ("cfgs", ctypes.c_void_p),
        ("n_cfgs", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("blk_cfg", ctypes.c_void_p),
        ("blk_item0", ctypes.c_void_p),
        ("blk_item1", ctypes.c_void_p),
        ("n_blocks", ctypes.c_int32),
        ("index32", ctypes.c_int32),
        ("cfg_blk0", ctypes.c_void_p),
        ("cfg_nblk", ctypes.c_void_p),
        ("pos", ctypes.c_void_p * 2),
        ("neg", ctypes.c_void_p * 2),
        ("dens", ctypes.c_void_p * 2),
        ("xs", ctypes.c_void_p),
        ("ys", ctypes.c_void_p),
        ("task_cfg", ctypes.c_void_p),
        ("task_first", ctypes.c_void_p),
        ("task_prefix", ctypes.c_void_p),
        ("step_task_off", ctypes.c_void_p),
        ("step_tracks", ctypes.c_void_p),
        ("step_blocks", ctypes.c_void_p),
        ("first_step", ctypes.c_int64),
        ("n_steps", ctypes.c_int64),
        ("counts", ctypes.c_void_p),
        ("tally", ctypes.c_void_p),
        ("workspace", ctypes.c_void_p),
        ("workspace_bytes", ctypes.c_int64),
        ("dep_workspace", ctypes.c_void_p),
        ("dep_workspace_bytes", ctypes.c_int64),
        ("dep_max_tracks", ctypes.c_int64),
        ("dep_dens_bytes", ctypes.c_int64),
        ("dep_total_tiles", ctypes.c_int32),
        ("dep_max_tiles", ctypes.c_int32),
    ]


BIN_OUT = 62  # output cells per side of a binned deposition tile (pic_internal.h, kBinOut)
BIN_MAX_SLOTS = 1024  # grids the binned batched deposition takes (kBinMaxSlots)
BIN_STEPS = 8  # global steps per binned deposition launch pair (kBinSteps)


def binned_tiles(no_xy):
    """62 x 62-cell tiles of the binned deposition of grids of side no_xy."""
    return (-(-np.asarray(no_xy, dtype=np.int64) // BIN_OUT)) ** 2


def binned_eligible(grids) -> bool:
    """Whether the binned batched deposition takes these grids: at most 1024,
    each no_xy <= 4096 with truncation boxes of at most 64 cells."""
    return len(grids) <= BIN_MAX_SLOTS and all(
        int(g.no_xy) <= 4096 and 2.0 * float(g.cutoff_voxels) + 1.0 < 64.0 for g in grids)


def _align(x: int, a: int = 64) -> int:
    return (x + a - 1) // a * a


def saturation_sweep_configs(n: int = 64, meta_seed: int = 20260527, **overrides) -> list:
    """The batched saturation sweep (see the module docstring)."""
    rng = np.random.default_rng(meta_seed)
    volts = np.logspace(np.log10(25.0), np.log10(400.0), n)
    out = []
    for i in range(n):
        kw = dict(
            E_MeV_u=56.2,
            voltage_V=float(volts[i]),
            electrode_gap_cm=float(rng.choice([0.1, 0.2, 0.3])),
            dose_rate_Gy_s=float(10.0 ** rng.uniform(0.0, 2.0)),
            pulse_duration_s=float(rng.uniform(100e-6, 1000e-6)),
            repetition_rate_hz=50.0,
            grid_size_um=float(rng.choice([5.0, 10.0])),
            sampled_radius_cm=float(rng.uniform(0.008, 0.03)),
            seed=i + 1,
            max_voxels=2e9,
        )
        kw.update(overrides)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            out.append(SimulationConfig(**kw))
    return out


def _phases(total_steps: Sequence[int]):
    """Intervals [s0, s1) of global steps over which the set of active grids
    (those with s < total_steps) is constant, with that set."""
    ends = sorted(set(int(t) for t in total_steps))
    phases = []
    s0 = 0
    for e in ends:
        if e <= s0:
            continue
        active = [c for c, t in enumerate(total_steps) if t > s0]
        phases.append((s0, e, active))
        s0 = e
    return phases


DEP_TILE = 64  # cells per side of a deposition tile (pic_deposit.cuh, kDepTile)
DEP_PART_TRACKS = 32  # tracks per part of a tile (pic_deposit.cuh, kDepPartTracks)


def deposit_blocks(no_xy, tracks):
    """Blocks of the tile-form deposition of one grid's tracks in one step:
    tiles x parts, parts = one per DEP_PART_TRACKS tracks, 1 to 32
    (pic_deposit.cuh, deposit_tiles / deposit_tile_parts)."""
    tiles = (-(-np.asarray(no_xy, dtype=np.int64) // DEP_TILE)) ** 2
    parts = np.clip(-(-np.asarray(tracks, dtype=np.int64) // DEP_PART_TRACKS), 1, 32)
    return tiles * parts


def _task_tables(offsets, totals, track_base, no_xy=None):
    """The deposition tasks of every global step, in grid order within a step.

    ``offsets[c]`` = grid c's cumulative track counts per step (length
    ``totals[c] + 1``), ``track_base[c]`` = its first track in the packed
    track arrays. Returns ``(step_task_off, step_tracks, task_cfg,
    task_first, task_prefix, step_blocks)``: the tasks of step s are
    ``step_task_off[s] .. step_task_off[s + 1] - 1``, one per grid with tracks
    at s, giving the grid, its first packed track and the tracks of the step's
    earlier tasks; ``step_tracks[s]`` = all tracks of step s,
    ``step_blocks[s]`` = the blocks of its tile-form deposition (grid sizes
    ``no_xy[c]``; zeros when not given)."""
    n_cfg = len(offsets)
    S = max(totals)
    M = np.zeros((S, n_cfg), dtype=np.int64)  # tracks of grid c at global step s
    F = np.zeros((S, n_cfg), dtype=np.int64)  # first track of (s, c) in the packed arrays
    for c in range(n_cfg):
        M[: totals[c], c] = np.diff(offsets[c])
        F[: totals[c], c] = track_base[c] + offsets[c][:-1]
    s_idx, c_idx = np.nonzero(M)  # row-major: by step, then grid
    vals = M[s_idx, c_idx]
    step_task_off = np.zeros(S + 1, dtype=np.int64)
    np.cumsum(np.bincount(s_idx, minlength=S), out=step_task_off[1:])
    step_tracks = M.sum(axis=1)
    excl = np.cumsum(vals) - vals  # tracks before each task, over all steps
    t_prefix = excl - excl[step_task_off[s_idx]] if len(vals) else excl
    step_blocks = np.zeros(S, dtype=np.int64)
    if no_xy is not None and len(vals):
        np.add.at(step_blocks, s_idx, deposit_blocks(np.asarray(no_xy)[c_idx], vals))
    return step_task_off, step_tracks, c_idx.astype(np.int32), F[s_idx, c_idx], t_prefix, step_blocks


# The first chunk of global steps is sampled on the host before the device
# has anything to run; later chunks are sampled while the device runs the one
# before. Chunks start at FIRST_CHUNK_STEPS steps and double up to
# chunk_steps, so the device starts after a small first chunk (the sweep's
# all-grid phase draws ~31 000 tracks a step: 268 steps of them were ~50 ms
# of host sampling ahead of the first launch). A chunk also holds at most
# MAX_CHUNK_TRACKS tracks (one step at least), which bounds the pinned
# staging buffers the chunks are sampled into.
FIRST_CHUNK_STEPS = 16
MAX_CHUNK_TRACKS = 1 << 20


def _ramp_chunks(phases, chunk_steps: int, first: int = FIRST_CHUNK_STEPS, step_tracks=None,
                 max_tracks: int = MAX_CHUNK_TRACKS):
    """Chunks (c0, c1, phase table + phase_start) of the ``phases`` of a
    batched run: every global step once, in order, no chunk across a phase
    boundary, sizes from ``min(first, chunk_steps)`` doubling up to
    ``chunk_steps`` over the run; with ``step_tracks`` (tracks of each global
    step) a chunk of more than one step holds at most ``max_tracks``."""
    out = []
    size = max(1, min(int(first), int(chunk_steps)))
    cum = None
    if step_tracks is not None:
        cum = np.zeros(len(step_tracks) + 1, dtype=np.int64)
        np.cumsum(np.asarray(step_tracks, dtype=np.int64), out=cum[1:])
    for s0, s1, tab in phases:
        c0 = s0
        while c0 < s1:
            c1 = min(c0 + size, s1)
            if cum is not None and cum[c1] - cum[c0] > max_tracks:
                # the last step end within the budget, one step at least
                c1 = max(c0 + 1, int(np.searchsorted(cum, cum[c0] + max_tracks, side="right")) - 1)
            out.append((c0, c1, dict(tab, phase_start=s0)))
            c0 = c1
            size = min(2 * size, int(chunk_steps))
    return out


def _work_table(items, active, sms: int) -> dict:
    """Blocks of one batched launch over the ``active`` grids (``items[c]`` =
    grid c's work items): each grid gets contiguous blocks, and block b of a
    grid with nb blocks steps its items [b it / nb, (b + 1) it / nb)."""
    items = np.asarray(items, dtype=np.int64)
    act = np.asarray(active, dtype=np.int64)
    n_cfg = len(items)
    ipb = items_per_block(int(items[act].sum()), sms)
    nb = np.maximum(1, -(-items[act] // ipb))
    first = np.concatenate([[0], np.cumsum(nb)[:-1]])
    cfg_blk0 = np.zeros(n_cfg, dtype=np.int32)
    cfg_nblk = np.zeros(n_cfg, dtype=np.int32)
    cfg_blk0[act] = first
    cfg_nblk[act] = nb
    blk_cfg = np.repeat(act, nb)
    b = np.arange(int(nb.sum()), dtype=np.int64) - np.repeat(first, nb)  # block index within its grid
    it, nbr = items[blk_cfg], np.repeat(nb, nb)
    return dict(blk_cfg=blk_cfg.astype(np.int32), blk_item0=b * it // nbr, blk_item1=(b + 1) * it // nbr,
                cfg_blk0=cfg_blk0, cfg_nblk=cfg_nblk)


def run_batched_b200(
    configs: Sequence,
    rngs: Optional[Sequence[np.random.Generator]] = None,
    return_fields: bool = False,
    dtype: str = "float32",
    alpha_cm3_s: Optional[float] = None,
    chunk_steps: int = 512,
    progress: bool = False,
    persistent: bool = False,
    solo_grids: int = SOLO_MAX_GRIDS,
    variant: str = "auto",
    escalate: bool = True,
    deposit: str = "auto",
):
    """Simulate every configuration and return their Results, in order.

    Equivalent to ``[run_simulation_b200(c) for c in configs]`` (same tracks,
    same tallies to float32 rounding) but with all grids advanced together.
    The global steps run in chunks of up to ``chunk_steps`` (the first
    chunks shorter: FIRST_CHUNK_STEPS doubling, ``_ramp_chunks``), each
    sampled on the host while the device runs the one before.
    ``persistent`` runs each chunk as one
    persistent launch (``pic_batched_persistent``: deposition and step phases
    separated by device-wide barriers); otherwise (the default) each global
    step is two launches (``pic_batched_segment``). Measured on GB300 over the
    64-configuration sweep the per-step launches are faster (1.31 vs 1.44 s):
    two device-wide barriers per step cost what two launch gaps do.
    Phases with at most ``solo_grids`` active grids run each grid's chunk
    with the single-grid kernels instead (0: never). ``variant`` picks the
    fused step of the batched launches: "flat" (pic_batched_segment, neighbours
    through L1/L2), "stream" (pic_batched_stream_segment: float32, planes staged
    in a shared-memory ring, items from every grid taken from a device-wide
    queue), "mixed" (float32: the streaming step on phases whose active grids
    hold at least STREAM_MIN_VOXELS interior voxels, ``stream_phase``, except
    while a float64 re-run is in flight; the flat step on the rest, and on
    float64 and persistent runs), or "auto" (the flat step: end to end on the
    64-configuration sweep, whose configuration 6 is re-run in float64 beside
    the batch, it measured 1.165-1.168 s against 1.179-1.182 s "mixed").
    ``escalate``: a float32 configuration whose tallies come back non-finite
    is run again alone with float64 fields from the same generator state
    (run_simulation_b200's ``escalate``), and that Result takes its place.
    ``deposit`` picks the deposition of the batched launches: "binned" (every
    grid's tracks of a global step listed per 62 x 62-cell tile and summed by
    one block per tile, each cell stored once), "tiles" (a block per tile and
    32-track part, adding with atomics), or "auto" (binned where the grids
    allow it, ``binned_eligible``).
    """
    import torch

    n_cfg = len(configs)
    if rngs is not None and len(rngs) != n_cfg:
        raise ValueError(f"rngs holds {len(rngs)} generators for {n_cfg} configurations")
    if dtype not in ("float32", "float64"):
        raise ValueError(f"dtype must be 'float32' or 'float64', got {dtype!r}")
    if int(chunk_steps) < 1:
        raise ValueError("chunk_steps must be >= 1")
    if int(solo_grids) < 0:
        raise ValueError("solo_grids must be >= 0")
    if variant not in ("auto", "flat", "stream", "mixed"):
        raise ValueError(f"variant must be 'auto', 'flat', 'stream' or 'mixed', got {variant!r}")
    if deposit not in ("auto", "binned", "tiles"):
        raise ValueError(f"deposit must be 'auto', 'binned' or 'tiles', got {deposit!r}")
    if variant == "stream" and (dtype != "float32" or persistent):
        raise ValueError("the streaming batched step takes float32 batches without persistent launches")
    if not torch.cuda.is_available():
        raise RuntimeError("run_batched_b200 needs a CUDA device (a GB300); none is visible")
    lib = N.load()
    sms = N.device_info()[0]
    dev = torch.device("cuda", torch.cuda.current_device())
    if n_cfg == 0:
        return []
    tdt = torch.float32 if dtype == "float32" else torch.float64
    es = 4 if dtype == "float32" else 8
    grids = [make_grid(c, dtype, alpha_cm3_s) for c in configs]
    totals = [int(c.total_time_steps) for c in configs]

    # --- schedules of every grid, drawn on the host (same stream as the
    # reference); the track centres are drawn later, chunk by chunk, while the
    # device runs the previous chunk (feeder.py)
    rngs = rngs if rngs is not None else [np.random.default_rng(c.seed) for c in configs]
    rng_start = [copy.deepcopy(r.bit_generator.state) for r in rngs] if (escalate and dtype == "float32") else None
    offsets, samplers = [], []
    track_base = []
    base = 0
    if len(configs) > 1 and len({id(r) for r in rngs}) == len(rngs):
        # independent generators: the schedules on the host's cores at once
        # (the native draws release the interpreter)
        with ThreadPoolExecutor(max_workers=min(len(configs), os.cpu_count() or 1)) as pool:
            scheds = list(pool.map(build_track_schedule, configs, rngs))
    else:
        scheds = [build_track_schedule(c, rng) for c, rng in zip(configs, rngs)]
    for c, rng, sched in zip(configs, rngs, scheds):
        n_tr = int(sched.sum())
        samplers.append(TrackSampler(rng, c.mid_xy, c.sampling_radius, c.no_xy))
        off = np.zeros(len(sched) + 1, dtype=np.int64)
        np.cumsum(sched, out=off[1:])
        offsets.append(off)
        track_base.append(base)
        base += n_tr

    # --- packed layout
    field_off, dens_off, counts_off, tally_off = [], [], [], []
    fo = do = co = to = 0
    items = []
    for g, t in zip(grids, totals):
        n, kp = int(g.no_xy), int(g.kpitch)
        dp = (n + 3) // 4 * 4
        field_off.append(fo)
        dens_off.append(do)
        counts_off.append(co)
        tally_off.append(to)
        fo = _align(fo + n * n * kp)
        do = _align(do + n * dp)
        co = _align(co + n * n)
        to += t
        items.append(n * n * (kp // 4))
    need = 4 * fo * es + 4 * do * es + co * 4 + to * 32 + 16 * base
    free, _ = torch.cuda.mem_get_info(dev)
    if need > 0.9 * free:
        raise MemoryError(f"batch needs {need / 2**30:.2f} GiB of device memory, {free / 2**30:.2f} GiB free")

    cfg_arr = (PicBatchCfg * n_cfg)()
    for c in range(n_cfg):
        cfg_arr[c].field_off, cfg_arr[c].dens_off = field_off[c], dens_off[c]
        cfg_arr[c].counts_off, cfg_arr[c].tally_off = counts_off[c], tally_off[c]
        cfg_arr[c].grid = grids[c]
    cfg_dev = torch.frombuffer(bytearray(cfg_arr), dtype=torch.uint8).to(dev)

    kw = dict(device=dev)
    pos = [torch.zeros(max(fo, 1), dtype=tdt, **kw) for _ in range(2)]
    neg = [torch.zeros(max(fo, 1), dtype=tdt, **kw) for _ in range(2)]
    dens = [torch.zeros(max(2 * do, 2), dtype=tdt, **kw) for _ in range(2)]  # deposition pairs
    counts = torch.zeros(max(co, 1), dtype=torch.int32, **kw)
    tally = torch.zeros((max(to, 1), 4), dtype=torch.float64, **kw)
    xs_dev = torch.zeros(max(base, 1), dtype=torch.float64, device=dev)
    ys_dev = torch.zeros(max(base, 1), dtype=torch.float64, device=dev)

    # --- per global step: tasks (grid, first track, first warp), in grid
    # order within a step
    S = max(totals)
    step_task_off, step_tracks, t_cfg, t_first, t_prefix, step_blocks = _task_tables(
        offsets, totals, track_base, [int(g.no_xy) for g in grids])
    one = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a if len(a) else np.zeros(1), dtype=dt)).to(dev)
    task_cfg = one(t_cfg, np.int32)
    task_first = one(t_first, np.int64)
    task_prefix = one(t_prefix, np.int64)
    binned = deposit == "binned" or (deposit == "auto" and binned_eligible(grids))
    if binned and not binned_eligible(grids):
        raise ValueError("the binned deposition takes at most 1024 grids, each no_xy <= 4096 with cutoff < 31.5 voxels")
    dep_ws, dep_tiles, dep_max_tiles, dep_max_tracks, dep_dens_bytes = None, 0, 0, 0, 0
    if binned and not persistent:
        tiles_c = binned_tiles([int(g.no_xy) for g in grids])
        dep_tiles, dep_max_tiles = int(tiles_c.sum()), int(tiles_c.max())
        # the most tracks of BIN_STEPS consecutive global steps (one launch pair's)
        window = np.convolve(np.asarray(step_tracks, dtype=np.int64), np.ones(BIN_STEPS, dtype=np.int64))
        dep_max_tracks = int(window.max()) if len(window) else 0
        dep_dens_bytes = int(dens[0].numel()) * dens[0].element_size()
        dwb = ctypes.c_int64()
        N.check(lib.pic_batched_deposit_bytes(n_cfg, dep_tiles, dep_max_tracks, dep_dens_bytes,
                                              N.PIC_F32 if dtype == "float32" else N.PIC_F64, ctypes.byref(dwb)),
                "pic_batched_deposit_bytes")
        dep_ws = torch.zeros(int(dwb.value), dtype=torch.uint8, device=dev)

    # --- work tables, one per set of active grids
    phases = []
    max_blocks = 1
    for s0, s1, active in _phases(totals):
        wt = _work_table(items, active, sms)
        max_blocks = max(max_blocks, len(wt["blk_cfg"]))
        phases.append((s0, s1, dict(
            active=[int(c) for c in active],
            n_blocks=int(len(wt["blk_cfg"])),
            **{k: torch.from_numpy(v).to(dev) for k, v in wt.items()},
        )))
    # 32-bit offsets when every grid's fields are < 2^31 elements
    index32 = all(int(g.no_xy) <= 16383 and int(g.no_xy) ** 2 * int(g.kpitch) < 2**31 for g in grids)
    wsb = ctypes.c_int64()
    N.check(lib.pic_batched_workspace_bytes(max_blocks, n_cfg, ctypes.byref(wsb)), "pic_batched_workspace_bytes")
    workspace = torch.zeros(int(wsb.value), dtype=torch.uint8, device=dev)

    st = torch.cuda.current_stream(dev).cuda_stream
    stream_tabs = {}  # phase start -> (prepared PicBatchStream, its workspace)
    if variant in ("stream", "mixed") and dtype == "float32" and not persistent:
        shapes = [(int(g.no_xy), int(g.nzb), int(g.kpitch)) for g in grids]
        for s0, _, tab in phases:
            if solo_grids > 0 and len(tab["active"]) <= solo_grids:
                continue
            if not stream_phase(shapes, tab["active"], variant, dtype, persistent):
                continue
            items_h, tiles_h = _stream_items(shapes, tab["active"], sms)
            sb = ctypes.c_int64()
            N.check(lib.pic_batched_stream_workspace_bytes(n_cfg, len(items_h), STREAM_WARPS, ctypes.byref(sb)),
                    "pic_batched_stream_workspace_bytes")
            sws = torch.zeros(int(sb.value), dtype=torch.uint8, device=dev)
            bs = PicBatchStream()
            N.check(lib.pic_batched_stream_prepare(ctypes.addressof(cfg_arr), n_cfg, items_h.ctypes.data,
                                                   len(items_h), tiles_h.ctypes.data, STREAM_WARPS, sws.data_ptr(),
                                                   sws.numel(), st, ctypes.byref(bs)), "pic_batched_stream_prepare")
            stream_tabs[s0] = (bs, sws)
    solo_ws = None
    if solo_grids > 0 and not persistent and any(len(t["active"]) <= solo_grids for _, _, t in phases):
        need = 0
        for g in grids:  # one workspace for every solo grid: the largest any of them needs
            swb = ctypes.c_int64()
            N.check(lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(swb)), "pic_step_workspace_bytes")
            need = max(need, int(swb.value))
        solo_ws = torch.zeros(need, dtype=torch.uint8, device=dev)

    solo_graphs = []  # graph handles, freed once the run has finished

    def run_solo(c, c0, c1):
        """Grid c's global steps [c0, c1) with the single-grid kernels, on its
        slices: state of step s in buffer s & 1, deposition pairs in buffer
        s & 1 (the batched step clears the other one every step, as
        pic_run_segment expects), tallies at row tally_off + s. The chunk's
        launches are captured into one CUDA graph and replayed (small grids
        are launch-bound)."""
        fo, do2 = field_off[c] * es, 2 * dens_off[c] * es
        off = np.ascontiguousarray(offsets[c][c0 : c1 + 1])
        args = (ctypes.byref(grids[c]), pos[0].data_ptr() + fo, neg[0].data_ptr() + fo, pos[1].data_ptr() + fo,
                neg[1].data_ptr() + fo, c0 & 1, c1 - c0, xs_dev.data_ptr() + 8 * track_base[c],
                ys_dev.data_ptr() + 8 * track_base[c], off.ctypes.data, dens[0].data_ptr() + do2,
                dens[1].data_ptr() + do2, c0 & 1, counts.data_ptr() + 4 * counts_off[c],
                tally.data_ptr() + 32 * (tally_off[c] + c0), solo_ws.data_ptr(), solo_ws.numel(), st)
        h = ctypes.c_void_p()
        N.check(lib.pic_graph_create(*args, ctypes.byref(h)), "pic_graph_create")
        solo_graphs.append(h.value)
        N.check(lib.pic_graph_launch(h.value, st), "pic_graph_launch")

    sto_dev = torch.from_numpy(step_task_off).to(dev)
    stt_dev = torch.from_numpy(np.ascontiguousarray(step_tracks, dtype=np.int64)).to(dev)
    # chunks of global steps (a ramp from FIRST_CHUNK_STEPS); chunk (c0, c1)
    # needs grid c's tracks [offsets[c][min(c0, T_c)], offsets[c][min(c1, T_c)])
    chunks = _ramp_chunks(phases, int(chunk_steps), step_tracks=step_tracks)

    def jobs_of(c0, c1):
        out = []
        for c in range(n_cfg):
            a, b = offsets[c][min(c0, totals[c])], offsets[c][min(c1, totals[c])]
            out.append((samplers[c], int(b - a), int(track_base[c] + a)))
        return out

    # float64 re-runs of configurations whose float32 tallies go non-finite:
    # after every chunk the tallies are copied back on a side stream; a grid
    # found diverged is re-run at once from its starting generator state on
    # a stream of its own, beside the rest of the batch (its float64 kernels
    # are bound by the FP64 units, the batch by memory and latency)
    from .solver_b200 import run_simulation_b200

    redo, redo_threads = {}, {}

    def redo_one(c):
        bg = type(rngs[c].bit_generator)()
        bg.state = rng_start[c]
        try:
            with torch.cuda.device(dev), torch.cuda.stream(torch.cuda.Stream(device=dev)):
                redo[c] = run_simulation_b200(configs[c], rng=np.random.Generator(bg), progress=False,
                                              return_fields=return_fields, dtype="float64",
                                              alpha_cm3_s=alpha_cm3_s, escalate=False)
        except BaseException as exc:  # re-raised by the caller's thread
            redo[c] = exc

    watch = rng_start is not None and bool(chunks)
    if watch:
        tally_pin = torch.empty(tuple(tally.shape), dtype=tally.dtype, pin_memory=True)
        side = torch.cuda.Stream(device=dev)
        copy_ev = None

    def watch_tallies(final=False):
        nonlocal copy_ev
        if copy_ev is not None and (final or copy_ev.query()):
            copy_ev.synchronize()
            host = tally_pin.numpy()
            for c in range(n_cfg):
                if c not in redo_threads and not np.isfinite(host[tally_off[c] : tally_off[c] + totals[c]]).all():
                    th = threading.Thread(target=redo_one, args=(c,), daemon=True)
                    redo_threads[c] = th
                    th.start()
            copy_ev = None
        if copy_ev is None and not final:
            done = torch.cuda.Event()
            done.record(torch.cuda.current_stream(dev))
            side.wait_event(done)
            with torch.cuda.stream(side):
                tally_pin.copy_(tally, non_blocking=True)
                copy_ev = torch.cuda.Event()
                copy_ev.record(side)

    feeder = TrackFeeder(torch, dev, max((sum(n for _, n, _ in jobs_of(c0, c1)) for c0, c1, _ in chunks), default=1))
    t0 = perf_counter()
    try:
        pending = feeder.submit(jobs_of(*chunks[0][:2])) if chunks else None
        for k, (c0, c1, tab) in enumerate(chunks):
            if watch and k > 0:
                watch_tallies()
            feeder.upload(pending, xs_dev, ys_dev)
            # draw the next chunk's tracks while the device runs this one
            pending = feeder.submit(jobs_of(*chunks[k + 1][:2])) if k + 1 < len(chunks) else None
            if solo_ws is not None and len(tab["active"]) <= solo_grids:
                with nvtx_range(f"solo grids ({len(tab['active'])})"):
                    for c in tab["active"]:  # independent grids: one after the other
                        run_solo(c, c0, c1)
                if progress:
                    print(f"  global step {c1}/{S}")
                continue
            L = PicBatchLaunch()
            L.cfgs = cfg_dev.data_ptr()
            L.n_cfgs = n_cfg
            L.dtype = N.PIC_F32 if dtype == "float32" else N.PIC_F64
            L.blk_cfg = tab["blk_cfg"].data_ptr()
            L.blk_item0 = tab["blk_item0"].data_ptr()
            L.blk_item1 = tab["blk_item1"].data_ptr()
            L.n_blocks = tab["n_blocks"]
            L.index32 = int(index32)
            L.cfg_blk0 = tab["cfg_blk0"].data_ptr()
            L.cfg_nblk = tab["cfg_nblk"].data_ptr()
            L.pos[0], L.pos[1] = pos[0].data_ptr(), pos[1].data_ptr()
            L.neg[0], L.neg[1] = neg[0].data_ptr(), neg[1].data_ptr()
            L.dens[0], L.dens[1] = dens[0].data_ptr(), dens[1].data_ptr()
            L.xs, L.ys = xs_dev.data_ptr(), ys_dev.data_ptr()
            L.task_cfg, L.task_first, L.task_prefix = task_cfg.data_ptr(), task_first.data_ptr(), task_prefix.data_ptr()
            sto = np.ascontiguousarray(step_task_off[c0 : c1 + 1])
            stt = np.ascontiguousarray(step_tracks[c0:c1])
            stb = np.ascontiguousarray(step_blocks[c0:c1])
            L.step_task_off = sto.ctypes.data
            L.step_tracks = stt.ctypes.data
            L.step_blocks = stb.ctypes.data
            L.first_step, L.n_steps = c0, c1 - c0
            L.counts, L.tally = counts.data_ptr(), tally.data_ptr()
            L.workspace, L.workspace_bytes = workspace.data_ptr(), workspace.numel()
            if dep_ws is not None:
                L.dep_workspace, L.dep_workspace_bytes = dep_ws.data_ptr(), dep_ws.numel()
                L.dep_max_tracks, L.dep_total_tiles, L.dep_max_tiles = dep_max_tracks, dep_tiles, dep_max_tiles
                L.dep_dens_bytes = dep_dens_bytes
            # "mixed" steps flat while a float64 re-run is in flight: the
            # streaming step holds every SM's shared memory, the flat one
            # leaves room for the re-run's kernels beside it
            streaming = tab["phase_start"] in stream_tabs and not (
                variant == "mixed" and any(th.is_alive() for th in redo_threads.values()))
            with nvtx_range(f"batched steps ({len(tab['active'])} grids)"):
                if streaming:
                    bs = stream_tabs[tab["phase_start"]][0]
                    N.check(lib.pic_batched_stream_segment(ctypes.byref(L), ctypes.byref(bs), st),
                            "pic_batched_stream_segment")
                elif persistent:
                    N.check(lib.pic_batched_persistent(ctypes.byref(L), sto_dev.data_ptr(), stt_dev.data_ptr(), st),
                            "pic_batched_persistent")
                else:
                    N.check(lib.pic_batched_segment(ctypes.byref(L), st), "pic_batched_segment")
            if progress:
                print(f"  global step {c1}/{S}")
        torch.cuda.synchronize(dev)
        for h in solo_graphs:
            lib.pic_graph_destroy(h)
        solo_graphs.clear()
        if solo_ws is not None:
            sv = ctypes.c_int32()
            N.check(lib.pic_workspace_status(solo_ws.data_ptr(), 1, st, ctypes.byref(sv)), "pic_workspace_status")
            if sv.value != 0:
                raise RuntimeError(f"a fused-step kernel gave up on a bounded wait (code {sv.value}); "
                                   "results are invalid")
        for bs, _ in stream_tabs.values():
            sv = ctypes.c_int32()
            N.check(lib.pic_batched_stream_status(ctypes.byref(bs), 1, st, ctypes.byref(sv)), "pic_batched_stream_status")
            if sv.value != 0:
                raise RuntimeError(f"the streaming batched step gave up (status {sv.value}); results are invalid")
        if persistent and chunks:
            status = ctypes.c_int32()
            N.check(lib.pic_batched_status(ctypes.byref(L), st, ctypes.byref(status)), "pic_batched_status")
            if status.value != 0:
                raise RuntimeError(f"the persistent batched kernel gave up on a barrier (status {status.value}); "
                                   "results are invalid")
    finally:
        feeder.close()
        for th in redo_threads.values():
            th.join()
        if solo_graphs:  # an exception left graphs behind: let them finish, then free them
            try:
                torch.cuda.synchronize(dev)
            finally:
                for h in solo_graphs:
                    lib.pic_graph_destroy(h)
    elapsed = perf_counter() - t0

    # --- one Result per configuration
    tally_h = tally.cpu().numpy()
    counts_h = counts.cpu().numpy().view(np.uint32)
    results = []
    pos_h = neg_h = None
    if return_fields:
        pos_h = [pos[0].cpu().numpy(), pos[1].cpu().numpy()]
        neg_h = [neg[0].cpu().numpy(), neg[1].cpu().numpy()]
    for c, cfg in enumerate(configs):
        diag = Diagnostics(cfg)
        diag.record_block(0, tally_h[tally_off[c] : tally_off[c] + totals[c]])
        n = int(cfg.no_xy)
        diag.track_density_xy = counts_h[counts_off[c] : counts_off[c] + n * n].reshape(n, n).astype(np.float64)
        f_t = collection_efficiency(diag.injected, diag.recombined, totals[c])
        time_s = (np.arange(totals[c]) + 1) * cfg.dt
        ks = 1.0 / f_t[-1]
        if return_fields:
            lvl = totals[c] & 1
            kp = int(grids[c].kpitch)
            sl = slice(field_off[c], field_off[c] + n * n * kp)
            p = pos_h[lvl][sl].reshape(n, n, kp)[:, :, : int(cfg.no_z_with_buffer)].astype(np.float64)
            q = neg_h[lvl][sl].reshape(n, n, kp)[:, :, : int(cfg.no_z_with_buffer)].astype(np.float64)
        else:
            p = q = np.zeros((0, 0, 0))
        res = diag.build_result(cfg, time_s, f_t, ks, p, q)
        res.loop_elapsed_s = elapsed
        res.fields_dtype = dtype
        rows = tally_h[tally_off[c] : tally_off[c] + totals[c]]
        if rng_start is not None and not np.isfinite(rows).all():
            # float32 fields could not follow this configuration: its float64
            # run of the same tracks (started during the batch when the
            # divergence showed before the last chunk)
            if c not in redo:
                redo_one(c)
            if isinstance(redo[c], BaseException):
                raise redo[c]
            res = redo[c]
        results.append(res)
    return results
