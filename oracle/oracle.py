"""FP64 CPU oracle of the reference solver's hot path.

TEST INFRASTRUCTURE ONLY: the checker the GPU path is compared against and
the CPU baseline the benchmark times. Only the test suite, the smoke check and
the benchmark's CPU-baseline leg may import this module; the product never
does.

The numerical kernels are ``pic_oracle.c`` (built by ``oracle/Makefile`` into
``oracle/_build/liboracle.so``), a float64 restatement of the reference's
kernels. This module restates the two drivers around them:

* ``mode="serial"`` -- ``run_simulation_numba`` (pulsed_ion_chamber/solver_numba.py:237-370):
  tracks deposited one at a time into both species, one Lax-Wendroff step,
  interior copied back, lateral boundary applied.
* ``mode="batched"`` -- ``run_simulation_numba_parallel``
  (pulsed_ion_chamber/solver_numba_parallel.py:526-723): a step's tracks summed
  into a 2D density, broadcast down the gap once, buffers swapped with the ring
  carried (absorbing) or mirrored (reflecting).

Track scheduling and placement are restated here too, independently of the
product package (pulsed_ion_chamber/pulses.py:39-171): the same NumPy PCG64
stream consumed in the same order.

Parity pin: tests/test_oracle.py checks this oracle against golden fixtures
produced by the reference itself (tests/golden/make_golden.py).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
RECOMBINATION_ALPHA_CM3_S = 1.60e-6

_lib = None


def build(force: bool = False) -> Path:
    """Compile liboracle.so with make (gcc, OpenMP when available)."""
    src = HERE / "pic_oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "-B" if force else "all"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        dp = ctypes.POINTER(ctypes.c_double)
        i64 = ctypes.c_int64
        d = ctypes.c_double
        L.oracle_insert_track.restype = d
        L.oracle_insert_track.argtypes = [dp, dp, d, d, i64, i64, i64, i64, d, d, d, d, d, d]
        L.oracle_accumulate_density.restype = None
        L.oracle_accumulate_density.argtypes = [dp, dp, dp, i64, i64, d, d, d]
        L.oracle_broadcast.restype = d
        L.oracle_broadcast.argtypes = [dp, dp, dp, i64, i64, i64, i64, d, d, d]
        L.oracle_lw_step.restype = None
        L.oracle_lw_step.argtypes = [dp, dp, dp, dp, i64, i64, i64, i64, d, d] + [d] * 9 + [dp]
        L.oracle_copy_back.argtypes = [dp, dp, i64, i64]
        L.oracle_apply_lateral_boundary.argtypes = [dp, i64, i64, ctypes.c_int]
        L.oracle_carry_ring.argtypes = [dp, dp, i64, i64]
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


# --------------------------------------------------------------------------
# scheduling and placement (pulsed_ion_chamber/pulses.py:39-171)
# --------------------------------------------------------------------------


def schedule(config, rng) -> np.ndarray:
    """Arrivals per step: cumulative uniforms rescaled onto the pulse and
    histogrammed into the pulse's time bins, repeated every period."""
    u = rng.random(int(config.number_of_tracks_per_pulse))
    t = np.cumsum(u)
    t /= t[-1]
    t *= config.pulse_duration_s
    counts = np.histogram(t, config.pulse_time_bins)[0].astype(np.int64)
    out = np.zeros(int(config.total_time_steps), dtype=np.int64)
    for p in range(int(config.n_pulses)):
        s0 = p * int(config.pulse_period_steps)
        out[s0 : s0 + len(counts)] += counts
    return out


class DiscSampler:
    """Rejection sampling on consecutive (u, v) pairs of the stream."""

    def __init__(self, rng, mid, radius, no_xy):
        self.rng, self.mid, self.r2, self.n = rng, mid, radius * radius, no_xy
        self.pool = np.empty((0, 2))

    def __call__(self, count):
        count = int(count)
        xs, ys = [], []
        while count > 0:
            if len(self.pool) == 0:
                self.pool = self.rng.random(2 * max(4096, 4 * count)).reshape(-1, 2)
            x = self.pool[:, 0] * self.n
            y = self.pool[:, 1] * self.n
            hit = np.flatnonzero((x - self.mid) ** 2 + (y - self.mid) ** 2 <= self.r2)[:count]
            used = int(hit[-1]) + 1 if len(hit) == count else len(self.pool)
            xs.append(x[hit])
            ys.append(y[hit])
            count -= len(hit)
            self.pool = self.pool[used:]
        if not xs:
            return np.empty(0), np.empty(0)
        return np.concatenate(xs), np.concatenate(ys)


# --------------------------------------------------------------------------
# drivers
# --------------------------------------------------------------------------


def run(config, mode: str = "serial", rng=None, max_steps=None, alpha_cm3_s=None, threads=None,
        keep_fields: bool = True, snapshot_step=None):
    """Run the reference's driver loop in float64 on the CPU.

    Returns a dict: ``f_t``, ``ks``, ``injected``, ``recombined``,
    ``n_positive``, ``n_negative`` (per step), ``track_density_xy``,
    ``positive``/``negative`` (final fields, or the fields right after step
    ``snapshot_step`` when given), ``steps``, ``wall_s``.
    """
    if mode not in ("serial", "batched"):
        raise ValueError(f"mode must be 'serial' or 'batched', got {mode!r}")
    L = lib()
    if threads is not None:
        set_threads(threads)
    rng = rng if rng is not None else np.random.default_rng(config.seed)
    sched = schedule(config, rng)
    sampler = DiscSampler(rng, config.mid_xy, config.sampling_radius, config.no_xy)

    no_xy, nzb, no_z, nze = int(config.no_xy), int(config.no_z_with_buffer), int(config.no_z), int(config.no_z_electrode)
    shape = (no_xy, no_xy, nzb)
    pos, neg, pos_next, neg_next = (np.zeros(shape) for _ in range(4))
    dens = np.zeros((no_xy, no_xy))
    (p_lat, p_zm, p_zp, p_cen), (n_lat, n_zm, n_zp, n_cen) = config.scheme_coefficients()
    alpha = RECOMBINATION_ALPHA_CM3_S if alpha_cm3_s is None else alpha_cm3_s
    alpha_dt = alpha * config.dt
    h2 = config.unit_length_cm**2
    b2 = config.track_radius_cm**2
    G = config.Gaussian_factor
    mid = config.mid_xy
    srsq = config.scoring_radius_sq
    cut = config.track_cutoff_voxels
    reflecting = 1 if config.lateral_boundary == "reflecting" else 0

    total = int(config.total_time_steps)
    last = total if max_steps is None else min(total, int(max_steps))
    injected = np.zeros(total)
    recombined = np.zeros(total)
    n_pos = np.zeros(total)
    n_neg = np.zeros(total)
    f_t = np.ones(total)
    td = np.zeros((no_xy, no_xy))
    out3 = np.zeros(3)
    I = 0.0
    R = 0.0
    snap = None
    step_wall = np.zeros(last)
    t0 = time.perf_counter()
    for step in range(last):
        ts = time.perf_counter()
        inj = 0.0
        m = int(sched[step])
        if m > 0:
            xs, ys = sampler(m)
            np.add.at(td, (xs.astype(np.int64), ys.astype(np.int64)), 1.0)
            if mode == "serial":
                for x, y in zip(xs, ys):
                    inj += L.oracle_insert_track(_p(pos), _p(neg), float(x), float(y), no_xy, nzb, no_z, nze,
                                                 h2, b2, G, mid, srsq, cut)
            else:
                dens[:] = 0.0
                xs = np.ascontiguousarray(xs)
                ys = np.ascontiguousarray(ys)
                L.oracle_accumulate_density(_p(dens), _p(xs), _p(ys), m, no_xy, h2, b2, cut)
                inj = L.oracle_broadcast(_p(pos), _p(neg), _p(dens), no_xy, nzb, no_z, nze, G, mid, srsq)
        I += inj
        L.oracle_lw_step(_p(pos), _p(neg), _p(pos_next), _p(neg_next), no_xy, nzb, nze, no_z, mid, srsq,
                         p_lat, p_zm, p_zp, p_cen, n_lat, n_zm, n_zp, n_cen, alpha_dt, _p(out3))
        R += out3[0]
        injected[step] = inj
        recombined[step] = out3[0]
        n_pos[step] = out3[1]
        n_neg[step] = out3[2]
        if mode == "serial":
            L.oracle_copy_back(_p(pos), _p(pos_next), no_xy, nzb)
            L.oracle_copy_back(_p(neg), _p(neg_next), no_xy, nzb)
            L.oracle_apply_lateral_boundary(_p(pos), no_xy, nzb, reflecting)
            L.oracle_apply_lateral_boundary(_p(neg), no_xy, nzb, reflecting)
        else:
            if reflecting:
                pos, pos_next = pos_next, pos
                neg, neg_next = neg_next, neg
                L.oracle_apply_lateral_boundary(_p(pos), no_xy, nzb, 1)
                L.oracle_apply_lateral_boundary(_p(neg), no_xy, nzb, 1)
            else:
                L.oracle_carry_ring(_p(pos_next), _p(pos), no_xy, nzb)
                L.oracle_carry_ring(_p(neg_next), _p(neg), no_xy, nzb)
                pos, pos_next = pos_next, pos
                neg, neg_next = neg_next, neg
        f_t[step] = 1.0 if I == 0.0 else (I - R) / I
        step_wall[step] = time.perf_counter() - ts
        if snapshot_step is not None and step == snapshot_step:
            snap = (pos.copy(), neg.copy())
    wall = time.perf_counter() - t0
    ks = float("nan") if last < total else 1.0 / f_t[-1]
    res = dict(f_t=f_t, ks=ks, injected=injected, recombined=recombined, n_positive=n_pos, n_negative=n_neg,
               track_density_xy=td, steps=last, wall_s=wall, step_wall_s=step_wall)
    if snap is not None:
        res["positive"], res["negative"] = snap
    elif keep_fields:
        res["positive"], res["negative"] = pos, neg
    return res


def sweep_only(config, steps: int, threads=None, seed_fields=None):
    """Time ``steps`` bare sweeps (no deposition) on a grid filled from
    ``seed_fields`` or with a smooth positive pattern; returns (wall_s, out3).
    Used as the bounded CPU-baseline sample of large grids."""
    L = lib()
    if threads is not None:
        set_threads(threads)
    no_xy, nzb, no_z, nze = int(config.no_xy), int(config.no_z_with_buffer), int(config.no_z), int(config.no_z_electrode)
    shape = (no_xy, no_xy, nzb)
    if seed_fields is None:
        pos = np.zeros(shape)
        pos[:, :, nze : nze + no_z] = 1e8
        neg = pos.copy()
    else:
        pos, neg = (np.ascontiguousarray(a, dtype=np.float64) for a in seed_fields)
    pos_next = np.zeros(shape)
    neg_next = np.zeros(shape)
    (p_lat, p_zm, p_zp, p_cen), (n_lat, n_zm, n_zp, n_cen) = config.scheme_coefficients()
    alpha_dt = RECOMBINATION_ALPHA_CM3_S * config.dt
    out3 = np.zeros(3)
    t0 = time.perf_counter()
    for _ in range(int(steps)):
        L.oracle_lw_step(_p(pos), _p(neg), _p(pos_next), _p(neg_next), no_xy, nzb, nze, no_z, config.mid_xy,
                         config.scoring_radius_sq, p_lat, p_zm, p_zp, p_cen, n_lat, n_zm, n_zp, n_cen, alpha_dt,
                         _p(out3))
        L.oracle_carry_ring(_p(pos_next), _p(pos), no_xy, nzb)
        L.oracle_carry_ring(_p(neg_next), _p(neg), no_xy, nzb)
        pos, pos_next = pos_next, pos
        neg, neg_next = neg_next, neg
    return time.perf_counter() - t0, out3.copy()


def cores_used() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1
