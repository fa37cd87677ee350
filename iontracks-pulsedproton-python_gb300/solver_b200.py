"""``run_simulation_b200`` -- the GB300 backend behind the reference's
solver signature.

Same arguments and same :class:`Result` as the reference's drivers
(``run_simulation_numba``, pulsed_ion_chamber/solver_numba.py:237-370, and the
CUDA backend's ``max_steps`` / ``return_fields``, solver_cuda.py:645-654), so
it drops in beside them and under the reference's output writers.

How a run is driven:

* the schedule and the track centres are drawn on the host from the same
  NumPy stream as the reference (identical tracks for the same seed), one
  chunk of steps at a time on a worker thread: the next chunk's tracks are
  drawn while the device runs the current one, and copied into the pulse's
  device track buffer just before the steps that read them;
* each pulse is one segment of steps on the device (deposition + fused step
  per time step), the clearance gaps are segments without deposition; the
  library's host loop launches a segment's kernels back to back with no host
  synchronisation inside it;
* per-step tallies stay on the device and come back once, at the end, in
  float64; f(t) and k_s are formed from them as the reference forms them from
  its running totals.

The fields are float32 (``dtype="float32"``, the production mode) or float64
(the validation mode). There is no CPU fallback: without a GB300 the call
raises.
"""

from __future__ import annotations

import copy
import threading
from time import perf_counter
from typing import Optional

import numpy as np

from .engine import ChamberEngine, nvtx_range
from .feeder import TrackFeeder
from .pulses import TrackSampler, build_track_schedule
from .state import Diagnostics, collection_efficiency


def _segments(config, last_step: int):
    """Consecutive (start, stop, with_tracks) segments covering [0, last_step)."""
    segs = []
    period = int(config.pulse_period_steps)
    pulse = int(config.pulse_time_steps)
    pos = 0
    for p in range(int(config.n_pulses)):
        s0 = p * period
        s1 = min(s0 + pulse, last_step)
        if s0 >= last_step:
            break
        if pos < s0:
            segs.append((pos, s0, False))
        segs.append((s0, s1, True))
        pos = s1
    if pos < last_step:
        segs.append((pos, last_step, False))
    return segs


def run_simulation_b200(
    config,
    rng: Optional[np.random.Generator] = None,
    progress: bool = True,
    max_wall_s: Optional[float] = None,
    max_steps: Optional[int] = None,
    return_fields: bool = True,
    dtype: str = "float32",
    alpha_cm3_s: Optional[float] = None,
    chunk_steps: int = 256,
    shape: Optional[dict] = None,
    use_graphs: Optional[bool] = None,
    tune: bool = False,
    escalate: bool = True,
):
    """Simulate a pulse train on one GB300 and return the reference's Result.

    ``max_wall_s`` stops after the chunk in which that much wall time has
    passed; ``max_steps`` after a fixed number of steps. Either sets
    ``steps_completed`` and ``loop_elapsed_s`` on the Result and makes k_s
    NaN when the run did not finish (pulsed_ion_chamber/solver_cuda.py:874-891).
    ``return_fields=False`` returns empty field arrays. ``alpha_cm3_s``
    overrides the recombination coefficient. ``shape`` overrides the fused
    step's launch shape (``variant`` "flat"/"stream", ``tile_rows``, ...);
    by default the library chooses, or with ``tune=True`` the autotuner
    (timed once per grid and cached). ``use_graphs`` replays each chunk of
    ``chunk_steps`` steps from a CUDA graph captured once (every pulse has
    the same per-step track counts, so a pulse's chunks replay for every
    pulse); by default graphs are used for grids under 30 M voxels, where
    launch overhead is a visible part of a step.

    ``escalate`` (float32 runs): when the run's tallies come back non-finite,
    it is run again from the same generator state with float64 fields, and
    that Result is returned. Near the explicit scheme's stability limit for
    recombination (very high dose rates at low fields) an unstable mode grows
    by a few per cent a step during the pulse: float64 round-off never lets it
    matter, float32 round-off does, and the float32 run overflows. A
    configuration that diverges in float64 too (as in the reference) stays
    non-finite. ``Result.fields_dtype`` names the fields the result came from.
    """
    if dtype not in ("float32", "float64"):
        raise ValueError(f"dtype must be 'float32' or 'float64', got {dtype!r}")
    if int(chunk_steps) < 1:
        raise ValueError("chunk_steps must be >= 1")
    total = int(config.total_time_steps)
    last_step = total if max_steps is None else max(0, min(total, int(max_steps)))
    rng = rng if rng is not None else np.random.default_rng(config.seed)
    rng_start = copy.deepcopy(rng.bit_generator.state) if (escalate and dtype == "float32") else None
    # The schedule (one pulse's arrival draws, host cores) on a thread while
    # the engine allocates and clears its device buffers; the track buffers,
    # sized by the schedule, come after.
    drawn = {}

    def draw_schedule():
        try:
            drawn["schedule"] = build_track_schedule(config, rng)
        except BaseException as exc:  # re-raised below
            drawn["error"] = exc

    worker = threading.Thread(target=draw_schedule, daemon=True)
    worker.start()
    try:
        eng = ChamberEngine(config, dtype=dtype, alpha_cm3_s=alpha_cm3_s, max_tracks=0, shape=shape)
    finally:
        worker.join()
    if "error" in drawn:
        eng.close()
        raise drawn["error"]
    schedule = drawn["schedule"]
    sampler = TrackSampler(rng, config.mid_xy, config.sampling_radius, config.no_xy)
    pulse_steps = int(config.pulse_time_steps)
    max_pulse_tracks = int(schedule[:pulse_steps].sum())
    eng.ensure_track_capacity(max_pulse_tracks)
    torch = eng.torch
    if tune and not shape:
        from .autotune import tune as _tune

        _tune(eng, quick=True)
    if use_graphs is None:
        use_graphs = int(config.no_xy) ** 2 * int(config.no_z_with_buffer) < 30_000_000
    diagnostics = Diagnostics(config)
    report_every = max(1, total // 20)
    loop_t0 = perf_counter()
    steps_done = 0

    # The run as chunks of at most chunk_steps steps (within a pulse or an
    # idle stretch). Chunks bound the wall-clock check and the progress
    # report; the device never waits on the host inside a chunk. A chunk's
    # tracks occupy [t0, t1) of the pulse's device track buffer.
    units = []
    for s0, s1, with_tracks in _segments(config, last_step):
        offsets = np.zeros(s1 - s0 + 1, dtype=np.int64)
        if with_tracks:
            np.cumsum(schedule[s0:s1], out=offsets[1:])
        for c0 in range(0, s1 - s0, chunk_steps):
            c1 = min(c0 + chunk_steps, s1 - s0)
            units.append((s0, with_tracks, c0, c1, offsets))
    feeds = [u for u, (_, wt, c0, c1, off) in enumerate(units) if wt and off[c1] > off[c0]]
    feeder = TrackFeeder(torch, eng.device, max((int(units[u][4][units[u][3]] - units[u][4][units[u][2]])
                                                  for u in feeds), default=1))

    def submit(k):  # draw the tracks of the k-th chunk with tracks
        s0, _, c0, c1, off = units[feeds[k]]
        return feeder.submit([(sampler, off[c1] - off[c0], off[c0])])

    try:
        pending = submit(0) if feeds else None
        next_feed = 0
        for u, (s0, with_tracks, c0, c1, offsets) in enumerate(units):
            if next_feed < len(feeds) and feeds[next_feed] == u:
                feeder.upload(pending, eng.xs, eng.ys)
                next_feed += 1
                # draw the next chunk's tracks while the device runs this one
                pending = submit(next_feed) if next_feed < len(feeds) else None
            seg = offsets[c0 : c1 + 1] - offsets[c0]
            with nvtx_range("pulse steps" if with_tracks else "idle steps"):
                if use_graphs:
                    # the same chunk of every pulse (or of every idle stretch)
                    # has the same offsets; the parities complete the key
                    key = (with_tracks, c0 if with_tracks else -1, c1 - c0, eng.parity, eng.step_index & 1)
                    eng.run_segment_graphed(key, seg, track_base=int(offsets[c0]))
                else:
                    eng.run_segment(seg, track_base=int(offsets[c0]))
            steps_done = s0 + c1
            if progress and (steps_done // report_every) != ((s0 + c0) // report_every):
                print(f"  step {steps_done}/{total}")
            if max_wall_s is not None:
                torch.cuda.synchronize(eng.device)
                if perf_counter() - loop_t0 >= max_wall_s:
                    break
        torch.cuda.synchronize(eng.device)
    finally:
        feeder.close()
    loop_elapsed_s = perf_counter() - loop_t0
    eng.check_status()
    tallies = eng.tallies(steps_done)
    diagnostics.record_block(0, tallies)
    diagnostics.track_density_xy = eng.track_density_xy()
    f_t = collection_efficiency(diagnostics.injected, diagnostics.recombined, steps_done)
    time_s = (np.arange(total) + 1) * config.dt
    ks = float("nan") if steps_done < total else 1.0 / f_t[-1]
    if return_fields:
        pos, neg = eng.fields()
    else:
        pos, neg = np.zeros((0, 0, 0)), np.zeros((0, 0, 0))
    result = diagnostics.build_result(config, time_s, f_t, ks, pos, neg)
    result.fields_dtype = dtype
    if max_wall_s is not None or max_steps is not None:
        result.steps_completed = steps_done
        result.loop_elapsed_s = loop_elapsed_s
    eng.close()
    if rng_start is not None and not np.isfinite(tallies).all():
        # float32 fields could not follow this configuration: run it again,
        # same tracks, in float64
        rng.bit_generator.state = rng_start
        wide = None if not shape else {k: v for k, v in shape.items() if k != "variant"}
        return run_simulation_b200(config, rng=rng, progress=progress, max_wall_s=max_wall_s, max_steps=max_steps,
                                   return_fields=return_fields, dtype="float64", alpha_cm3_s=alpha_cm3_s,
                                   chunk_steps=chunk_steps, shape=wide, use_graphs=use_graphs, escalate=False)
    return result
