"""The host track feeder (feeder.py) without a GPU: a stand-in for the few
torch calls it makes (pinned staging buffers become plain CPU tensors, CUDA
events become markers) drives the real class. Drawing a run chunk by chunk on
the worker thread, two staging slots alternating, gives exactly the centres
of drawing each sampler's tracks up front, each at its place in the track
buffer."""

import types

import numpy as np
import pytest
import torch

from goldens import pkg


class _Event:
    def __init__(self):
        self.recorded = self.synced = 0

    def record(self, stream=None):
        self.recorded += 1

    def synchronize(self):
        self.synced += 1


def _fake_torch(events):
    def empty(n, dtype=None, pin_memory=False):
        return torch.empty(n, dtype=dtype)

    def event():
        e = _Event()
        events.append(e)
        return e

    cuda = types.SimpleNamespace(Event=event, current_stream=lambda device=None: None)
    return types.SimpleNamespace(empty=empty, float64=torch.float64, cuda=cuda)


def test_chunked_feeding_equals_sampling_up_front():
    import importlib

    feeder_mod = importlib.import_module(pkg().__name__ + ".feeder")
    geoms = [(30, 24.0, 60), (12.5, 9.5, 25), (40, 33.0, 80)]
    counts = [[5, 0, 17, 3, 40], [0, 9, 9, 0, 1], [30, 1, 0, 22, 6]]  # per grid, per chunk
    # up front: each grid's centres in one call
    want = [pkg().TrackSampler(np.random.default_rng(10 + g), *geoms[g]).sample(sum(counts[g])) for g in range(3)]
    base = np.concatenate([[0], np.cumsum([sum(c) for c in counts])])
    total = int(base[-1])

    events = []
    samplers = [pkg().TrackSampler(np.random.default_rng(10 + g), *geoms[g]) for g in range(3)]
    chunk_total = max(sum(counts[g][k] for g in range(3)) for k in range(5))
    f = feeder_mod.TrackFeeder(_fake_torch(events), "cpu", chunk_total)
    dev_x = torch.full((total,), float("nan"), dtype=torch.float64)
    dev_y = torch.full((total,), float("nan"), dtype=torch.float64)
    done = [0, 0, 0]

    def jobs(k):
        out = []
        for g in range(3):
            out.append((samplers[g], counts[g][k], base[g] + done[g]))
            done[g] += counts[g][k]
        return out

    try:
        pending = f.submit(jobs(0))
        copied = 0
        for k in range(5):
            nxt = f.submit(jobs(k + 1)) if k + 1 < 5 else None
            copied += f.upload(pending, dev_x, dev_y)
            pending = nxt
    finally:
        f.close()
    assert copied == total
    for g in range(3):
        sl = slice(int(base[g]), int(base[g + 1]))
        assert np.array_equal(dev_x[sl].numpy(), want[g][0]) and np.array_equal(dev_y[sl].numpy(), want[g][1])
    # one event per upload; a slot's refill waited on its previous copies
    assert len(events) == 5 and all(e.recorded == 1 for e in events)
    assert sum(e.synced for e in events) == 3


def test_chunk_larger_than_staging_is_refused():
    import importlib

    feeder_mod = importlib.import_module(pkg().__name__ + ".feeder")
    s = pkg().TrackSampler(np.random.default_rng(1), 30, 24.0, 60)
    f = feeder_mod.TrackFeeder(_fake_torch([]), "cpu", 10)
    try:
        with pytest.raises(ValueError, match="exceeds the staging capacity"):
            f.submit([(s, 11, 0)])
        h = f.submit([(s, 0, 0), (s, 10, 0)])  # empty jobs are dropped
        assert f.upload(h, torch.zeros(10, dtype=torch.float64), torch.zeros(10, dtype=torch.float64)) == 10
    finally:
        f.close()
