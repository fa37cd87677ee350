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

import ctypes

import numpy as np

from . import _native as N

__all__ = ["build_track_schedule", "TrackSampler", "CylinderSampler", "pulse_arrival_counts"]


def pulse_arrival_counts(config, rng: np.random.Generator) -> np.ndarray:
    """Tracks arriving in each time step of one pulse (int64, length
    ``pulse_time_steps``)."""
    n = int(config.number_of_tracks_per_pulse)
    if n >= 1 and type(rng.bit_generator) is np.random.PCG64:
        return _arrival_counts_pcg64(config, rng, n)
    arrival = np.cumsum(rng.random(n))
    arrival /= arrival[-1]
    arrival *= config.pulse_duration_s
    # np.histogram(arrival, bins) over explicit edges counts, per bin, the
    # values in [edge_b, edge_b+1) (the last bin closed on the right) by binary
    # searches in the sorted values; arrival is already non-decreasing (a
    # running sum of non-negative draws, scaled), so the searches run on it
    # directly and the sort drops out. Same counts, without the O(n log n).
    bins = np.asarray(config.pulse_time_bins, dtype=np.float64)
    cum = np.concatenate([np.searchsorted(arrival, bins[:-1], side="left"),
                          np.searchsorted(arrival, bins[-1:], side="right")])
    return np.diff(cum).astype(np.int64)


def _pcg64_state(rng):
    d = rng.bit_generator.state
    s, inc = int(d["state"]["state"]), int(d["state"]["inc"])
    m64 = (1 << 64) - 1
    return d, np.array([s >> 64, s & m64, inc >> 64, inc & m64], dtype=np.uint64)


def _store_pcg64_state(rng, d, st) -> None:
    d["state"]["state"] = (int(st[0]) << 64) | int(st[1])
    rng.bit_generator.state = d


def _arrival_counts_pcg64(config, rng, n: int) -> np.ndarray:
    """The same counts drawn and binned natively (``pic_arrival_counts_pcg64``:
    the same doubles, the same left-to-right running sum and the same
    divide-then-multiply, each arrival binned as it is formed); the generator
    is left past the n draws."""
    lib = N.load()
    edges = np.ascontiguousarray(config.pulse_time_bins, dtype=np.float64)
    counts = np.zeros(len(edges) - 1, dtype=np.int64)
    d, st = _pcg64_state(rng)
    N.check(lib.pic_arrival_counts_pcg64(st.ctypes.data, n, float(config.pulse_duration_s), edges.ctypes.data,
                                         len(edges), counts.ctypes.data), "pic_arrival_counts_pcg64")
    _store_pcg64_state(rng, d, st)
    return counts


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

    def __init__(self, rng: np.random.Generator, mid_xy, radius: float, no_xy: int, native_rng: bool = True):
        self.rng = rng
        self.mid_xy = mid_xy
        self.radius_sq = radius * radius
        self.no_xy = no_xy
        self._accept = min(1.0, max(0.05, np.pi * self.radius_sq / float(no_xy * no_xy)))
        self._buf = np.empty(0)
        self._pos = 0
        # NumPy's PCG64 (what default_rng gives) is drawn natively from its
        # state, exactly the doubles consumed; any other bit generator is
        # drawn through NumPy in blocks and scanned natively.
        self._pcg64 = native_rng and type(rng.bit_generator) is np.random.PCG64

    def _refill(self, wanted: int) -> None:
        pairs = max(self._MIN_DRAW, int(wanted / self._accept * 1.25) + 16)
        rest = self._buf[self._pos :]
        self._buf = np.concatenate([rest, self.rng.random(2 * pairs)]) if rest.size else self.rng.random(2 * pairs)
        self._pos = 0

    def sample(self, n_tracks: int):
        """``(xs, ys)`` float64 arrays of ``n_tracks`` accepted centres.

        The doubles come from the generator here; the accept/reject scan over
        them is the library's ``pic_sample_disc`` (one pass in C, float64,
        one rounding per operation), which stops at the wanted count.
        """
        n_tracks = int(n_tracks)
        if n_tracks <= 0:
            return np.empty(0), np.empty(0)
        return self.sample_into(np.empty(n_tracks), np.empty(n_tracks))

    def sample_into(self, xs_out: np.ndarray, ys_out: np.ndarray):
        """Fill the contiguous float64 arrays ``xs_out``/``ys_out`` (equal
        lengths) with the next accepted centres -- e.g. views of pinned
        staging memory -- and return them."""
        n_tracks = len(xs_out)
        if len(ys_out) != n_tracks or xs_out.dtype != np.float64 or ys_out.dtype != np.float64:
            raise ValueError("xs_out and ys_out must be float64 arrays of equal length")
        if not (xs_out.flags.c_contiguous and ys_out.flags.c_contiguous):
            raise ValueError("xs_out and ys_out must be contiguous")
        if n_tracks == 0:
            return xs_out, ys_out
        if self._pcg64:
            return self._sample_pcg64(n_tracks, xs_out, ys_out)
        lib = N.load()
        acc, used = ctypes.c_int64(), ctypes.c_int64()
        filled = 0
        while filled < n_tracks:
            if (self._buf.size - self._pos) < 2:
                self._refill(n_tracks - filled)
            n_pairs = (self._buf.size - self._pos) // 2
            u = self._buf[self._pos :]
            N.check(lib.pic_sample_disc(u.ctypes.data, n_pairs, float(self.no_xy), float(self.mid_xy),
                                        float(self.radius_sq), n_tracks - filled,
                                        xs_out[filled:].ctypes.data, ys_out[filled:].ctypes.data,
                                        ctypes.byref(acc), ctypes.byref(used)), "pic_sample_disc")
            filled += acc.value
            self._pos += 2 * used.value
            if self._pos >= self._buf.size:
                self._buf = np.empty(0)
                self._pos = 0
        return xs_out, ys_out

    def _sample_pcg64(self, n_tracks: int, xs_out: np.ndarray, ys_out: np.ndarray):
        """Draw and scan in one native pass (``pic_sample_disc_pcg64``) from
        the generator's PCG64 state, then store the advanced state back: the
        generator ends exactly past the doubles consumed, so the next call
        (or any later draw) continues the stream."""
        lib = N.load()
        d, st = _pcg64_state(self.rng)
        acc, draws = ctypes.c_int64(), ctypes.c_int64()
        filled = 0
        while filled < n_tracks:
            # bounded calls keep the interpreter responsive; the stream is
            # continued across them through st
            max_pairs = max(1 << 16, int((n_tracks - filled) / self._accept * 1.5) + 1024)
            N.check(lib.pic_sample_disc_pcg64(st.ctypes.data, float(self.no_xy), float(self.mid_xy),
                                              float(self.radius_sq), n_tracks - filled, max_pairs,
                                              xs_out[filled:].ctypes.data, ys_out[filled:].ctypes.data,
                                              ctypes.byref(acc), ctypes.byref(draws)), "pic_sample_disc_pcg64")
            filled += acc.value
        _store_pcg64_state(self.rng, d, st)
        return xs_out, ys_out


# The reference's name for the same sampler.
CylinderSampler = TrackSampler
