"""Slab decomposition of one chamber grid over several GPUs: the plan.

A grid too large for one GPU's memory is split along i, the slowest axis of
the ``[no_xy][no_xy][kpitch]`` layout, so that every slab is one contiguous
block of each field buffer. Rank r owns planes ``[i0, i1)`` and holds
``[lo, hi) = [i0 - 1, i1 + 1)`` clipped to the grid: its own planes plus one
halo plane on each side (the 7-point stencil reaches one plane each way).
Each time step on every rank:

1. deposits the step's tracks whose widened stencil box (the truncation box
   plus one cell each way, the reach of the (density, neighbour-sum) pairs)
   meets ``[lo, hi)``: a track near a slab edge goes to both owners, and each
   adds it to its halo plane exactly as the neighbour adds it to its own;
2. steps its owned interior planes, reading the halo planes;
3. applies the lateral wall (the i-ring planes 0 and no_xy-1 live in the
   first and last slabs; the j-ring columns in every slab);
4. sends its first and last owned planes to the neighbours' halos -- one
   plane per species per neighbour per step -- and receives theirs, so that
   the next step reads the neighbours' new values.

Tallies: each rank sums its owned planes (the scored columns of planes
``[max(i0, 1), min(i1, no_xy - 1))``); the float64 partials are summed over
ranks. On GPUs the halo copies go peer to peer into the receiving GPU's own
memory before its step reads them, so every kernel reads local memory only.

This module is the host-side bookkeeping of that scheme, with no device
code: it replaces the reference's managed-memory spill for grids beyond one
GPU (pulsed_ion_chamber/solver_cuda.py:690-732), which has no multi-GPU
path of its own. tests/test_slabs.py runs it on two gloo ranks with a float64
CPU slab step and checks it against a single-grid run of the oracle.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np


@dataclass(frozen=True)
class Slab:
    """Planes of one rank: owned ``[i0, i1)``, held ``[lo, hi)``."""

    rank: int
    i0: int
    i1: int
    lo: int
    hi: int

    @property
    def planes(self) -> int:
        return self.hi - self.lo

    def local(self, i: int) -> int:
        """Local index of global plane ``i`` (which must be held)."""
        if not self.lo <= i < self.hi:
            raise IndexError(f"plane {i} is not held by rank {self.rank} ([{self.lo}, {self.hi}))")
        return i - self.lo

    def interior(self, no_xy: int) -> Tuple[int, int]:
        """Owned planes that the stencil updates: ``[max(i0, 1), min(i1, no_xy - 1))``."""
        return max(self.i0, 1), min(self.i1, no_xy - 1)


def partition(no_xy: int, world: int) -> List[Slab]:
    """Split planes ``[0, no_xy)`` into ``world`` slabs with as even a share of
    the interior planes ``[1, no_xy - 1)`` as possible; the i-ring planes go
    with the first and last slabs. Every slab owns at least one interior plane."""
    n = int(no_xy)
    world = int(world)
    if world < 1:
        raise ValueError("world must be >= 1")
    interior = n - 2
    if interior < world:
        raise ValueError(f"a {n}-plane grid has {interior} interior planes, fewer than {world} ranks")
    cuts = [1 + (interior * r) // world for r in range(world + 1)]
    cuts[0], cuts[-1] = 0, n
    return [Slab(r, cuts[r], cuts[r + 1], max(cuts[r] - 1, 0), min(cuts[r + 1] + 1, n)) for r in range(world)]


def halo_exchanges(slabs: Sequence[Slab]) -> List[Tuple[int, int, int]]:
    """The per-step plane copies ``(src_rank, dst_rank, plane)``: every rank's
    first and last owned planes to the neighbour that holds them as a halo."""
    out = []
    for a, b in zip(slabs[:-1], slabs[1:]):
        out.append((a.rank, b.rank, a.i1 - 1))  # a's last owned plane -> b's lower halo
        out.append((b.rank, a.rank, b.i0))      # b's first owned plane -> a's upper halo
    return out


def track_rows(xs: np.ndarray, cutoff_voxels: float, no_xy: int) -> Tuple[np.ndarray, np.ndarray]:
    """Rows ``[lo, hi)`` of each track's written box: the truncation box
    ``[ceil(x - cut), floor(x + cut)]`` clipped to the grid
    (pulsed_ion_chamber/solver_numba.py:86-89), widened by one row each way
    for the neighbour sums, clipped again."""
    x = np.asarray(xs, dtype=np.float64)
    lo = np.maximum(np.ceil(x - cutoff_voxels), 0.0).astype(np.int64)
    hi = np.minimum(np.floor(x + cutoff_voxels) + 1.0, float(no_xy)).astype(np.int64)
    return np.maximum(lo - 1, 0), np.minimum(hi + 1, int(no_xy))


def tracks_of(slab: Slab, xs: np.ndarray, cutoff_voxels: float, no_xy: int) -> np.ndarray:
    """Indices (ascending: the deposition order is kept) of the tracks whose
    written box meets the slab's held planes."""
    lo, hi = track_rows(xs, cutoff_voxels, no_xy)
    return np.nonzero((hi > slab.lo) & (lo < slab.hi))[0]


def slab_bytes(slab: Slab, no_xy: int, kpitch: int, elem_bytes: int = 4) -> int:
    """Field memory of one rank: two time levels of both species over its
    held planes."""
    return 4 * slab.planes * int(no_xy) * int(kpitch) * int(elem_bytes)


def ranks_needed(no_xy: int, kpitch: int, bytes_per_gpu: float, elem_bytes: int = 4, reserve: float = 0.1) -> int:
    """Fewest ranks whose slabs' fields fit ``(1 - reserve)`` of each GPU's
    memory."""
    per_plane = 4 * int(no_xy) * int(kpitch) * int(elem_bytes)
    budget = (1.0 - reserve) * float(bytes_per_gpu)
    for world in range(1, int(no_xy) - 1):
        if max(s.planes for s in partition(no_xy, world)) * per_plane <= budget:
            return world
    raise ValueError("no slab split fits: a single plane exceeds the memory budget")


def halo_bytes_per_step(no_xy: int, kpitch: int, world: int, elem_bytes: int = 4) -> int:
    """Bytes copied between GPUs per step: one plane per species per
    neighbour pair and direction."""
    return 2 * 2 * (int(world) - 1) * int(no_xy) * int(kpitch) * int(elem_bytes)


__all__ = ["Slab", "partition", "halo_exchanges", "track_rows", "tracks_of", "slab_bytes", "ranks_needed",
           "halo_bytes_per_step"]
