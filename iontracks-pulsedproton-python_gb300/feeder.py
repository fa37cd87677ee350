"""Host track sampling overlapped with the device.

The solvers draw track centres on the host from the reference's generator
(identical tracks for the same seed). Rather than drawing a whole pulse before
its first step runs, they hand the sampler a chunk at a time: a worker thread
draws chunk k+1 into pinned staging memory while the GPU runs chunk k (the
native sampler releases the interpreter lock while it runs), and each chunk
is copied to its place in the device track buffer on the solver's stream just
before the steps that read it. Every sampler is used by the worker only, in
submission order, so the stream of draws -- and the tracks -- are exactly
those of sampling up front.

Two staging slots alternate; a slot is refilled only after the copies out of
it have completed (an event recorded after them).
"""

from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor


class TrackFeeder:
    def __init__(self, torch, device, capacity: int):
        self.torch = torch
        self.device = device
        self.capacity = max(1, int(capacity))
        self._stage = [(torch.empty(self.capacity, dtype=torch.float64, pin_memory=True),
                        torch.empty(self.capacity, dtype=torch.float64, pin_memory=True)) for _ in range(2)]
        self._views = [(x.numpy(), y.numpy()) for x, y in self._stage]
        self._copied = [None, None]
        self._slot = 0
        self._pool = ThreadPoolExecutor(max_workers=1)

    def submit(self, jobs):
        """Start drawing one chunk on the worker: ``jobs`` = [(sampler, n,
        dst)], n centres from ``sampler`` for device positions [dst, dst + n).
        Returns a handle for :meth:`upload`."""
        jobs = [(s, int(n), int(d)) for s, n, d in jobs if int(n) > 0]
        total = sum(n for _, n, _ in jobs)
        if total > self.capacity:
            raise ValueError(f"chunk of {total} tracks exceeds the staging capacity {self.capacity}")
        slot = self._slot
        self._slot ^= 1
        ready = self._copied[slot]
        vx, vy = self._views[slot]

        def draw():
            if ready is not None:
                ready.synchronize()  # the copies out of this slot have finished
            parts, o = [], 0
            for sampler, n, dst in jobs:
                sampler.sample_into(vx[o : o + n], vy[o : o + n])
                parts.append((o, n, dst))
                o += n
            return parts

        return slot, self._pool.submit(draw)

    def upload(self, handle, dev_x, dev_y) -> int:
        """Wait for the chunk's draws and copy them into ``dev_x``/``dev_y``
        on the current stream (before the steps that read them). Returns the
        number of centres copied."""
        slot, fut = handle
        parts = fut.result()
        sx, sy = self._stage[slot]
        n_total = 0
        for o, n, dst in parts:
            dev_x[dst : dst + n].copy_(sx[o : o + n], non_blocking=True)
            dev_y[dst : dst + n].copy_(sy[o : o + n], non_blocking=True)
            n_total += n
        ev = self.torch.cuda.Event()
        ev.record(self.torch.cuda.current_stream(self.device))
        self._copied[slot] = ev
        return n_total

    def close(self) -> None:
        self._pool.shutdown(wait=True)
