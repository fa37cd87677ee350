"""Track scheduling (when) and placement (where), on the host.

Both functions consume the NumPy ``Generator`` stream in exactly the order the
reference does, so the same seed gives the same tracks, bit for bit:

1. :func:`build_track_schedule` draws ``number_of_tracks_per_pulse`` uniforms
   once, turns their running sum into arrival times across the pulse and bins
   them per time step (pulsed_ion_chamber/pulses.py:39-61). The count is
   deliberately not Poisson; the same histogram repeats for every pulse.
2. :class:`TrackSampler` then rejection-samples centres uniformly in the
   sampling disc from consecutive pairs of doubles of the same stream
   (pulsed_ion_chamber/pulses.py:64-82 defines the per-track loop and
   :84-171 its block form).

The sampler's contract is the stream, not the block size: PCG64 ``random(n)``
yields the same doubles however the draws are split, so a whole pulse can be
sampled in one call and split by the schedule afterwards. That is what lets
the solver upload a pulse's tracks in one copy and replay its steps from a
captured CUDA graph.
"""

from __future__ import annotations

import numpy as np

__all__ = ["build_track_schedule", "TrackSampler", "CylinderSampler", "pulse_arrival_counts"]


def pulse_arrival_counts(config, rng: np.random.Generator) -> np.ndarray:
    """Tracks arriving in each time step of one pulse (int64, length
    ``pulse_time_steps``)."""
    n = int(config.number_of_tracks_per_pulse)
    arrival = np.cumsum(rng.random(n))
    arrival /= arrival[-1]
    arrival *= config.pulse_duration_s
    counts, _ = np.histogram(arrival, config.pulse_time_bins)
    return counts.astype(np.int64)


def build_track_schedule(config, rng: np.random.Generator) -> np.ndarray:
    """New tracks per time step over the whole run (int64, length
    ``total_time_steps``): one pulse's histogram, repeated every
    ``pulse_period_steps``."""
    schedule = np.zeros(int(config.total_time_steps), dtype=np.int64)
    counts = pulse_arrival_counts(config, rng)
    for p in range(int(config.n_pulses)):
        start = p * int(config.pulse_period_steps)
        schedule[start : start + len(counts)] += counts
    return schedule


class TrackSampler:
    """Uniform track centres inside the disc of radius ``radius`` about
    ``(mid_xy, mid_xy)``, in voxel units over ``[0, no_xy)^2``.

    Attempt ``a`` uses doubles ``2a`` and ``2a+1`` of the generator's stream:
    ``x = u * no_xy``, ``y = v * no_xy``, accepted when
    ``(x - mid)^2 + (y - mid)^2 <= radius^2``. Unused doubles are kept for the
    next call, so consecutive calls continue the stream exactly.
    """

    _MIN_DRAW = 1 << 13

    def __init__(self, rng: np.random.Generator, mid_xy, radius: float, no_xy: int):
        self.rng = rng
        self.mid_xy = mid_xy
        self.radius_sq = radius * radius
        self.no_xy = no_xy
        self._accept = min(1.0, max(0.05, np.pi * self.radius_sq / float(no_xy * no_xy)))
        self._buf = np.empty(0)
        self._pos = 0

    def _refill(self, wanted: int) -> None:
        pairs = max(self._MIN_DRAW, int(wanted / self._accept * 1.25) + 16)
        rest = self._buf[self._pos :]
        self._buf = np.concatenate([rest, self.rng.random(2 * pairs)]) if rest.size else self.rng.random(2 * pairs)
        self._pos = 0

    def sample(self, n_tracks: int):
        """``(xs, ys)`` float64 arrays of ``n_tracks`` accepted centres."""
        n_tracks = int(n_tracks)
        if n_tracks <= 0:
            return np.empty(0), np.empty(0)
        xs_out = np.empty(n_tracks)
        ys_out = np.empty(n_tracks)
        filled = 0
        while filled < n_tracks:
            if (self._buf.size - self._pos) < 2:
                self._refill(n_tracks - filled)
            n_pairs = (self._buf.size - self._pos) // 2
            block = self._buf[self._pos : self._pos + 2 * n_pairs]
            x = block[0::2] * self.no_xy
            y = block[1::2] * self.no_xy
            ok = (x - self.mid_xy) ** 2 + (y - self.mid_xy) ** 2 <= self.radius_sq
            idx = np.flatnonzero(ok)
            need = n_tracks - filled
            if idx.size >= need:
                take = idx[:need]
                used_pairs = int(take[-1]) + 1
            else:
                take = idx
                used_pairs = n_pairs
            xs_out[filled : filled + take.size] = x[take]
            ys_out[filled : filled + take.size] = y[take]
            filled += take.size
            self._pos += 2 * used_pairs
            if self._pos >= self._buf.size:
                self._buf = np.empty(0)
                self._pos = 0
        return xs_out, ys_out


# The reference's name for the same sampler.
CylinderSampler = TrackSampler
