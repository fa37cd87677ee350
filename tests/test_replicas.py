"""Multi-GPU runs are independent replicas (no data to exchange); the
processes share only the timing. These tests run the rank logic as two gloo
processes on CPU."""

import importlib
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from goldens import make_config, pkg


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rep = importlib.import_module(pkg().__name__ + ".replicas")
        pulses = importlib.import_module(pkg().__name__ + ".pulses")
        # each rank's own time and work; the job takes the slowest rank's time
        seconds = 1.0 + rank  # rank 1 is the slow one
        units = 100.0 * (rank + 1)
        rate = rep.whole_job_rate(units, seconds)
        slowest = rep.max_over_ranks(seconds)
        total = rep.sum_over_ranks(units)
        # distinct tracks per replica
        cfg = make_config("fast_dense")
        rng = np.random.default_rng(rep.replica_seed(cfg.seed, rank))
        sched = pulses.build_track_schedule(cfg, rng)
        xs, _ = pulses.TrackSampler(rng, cfg.mid_xy, cfg.sampling_radius, cfg.no_xy).sample(int(sched.sum()))
        out.put((rank, rate, slowest, total, float(xs[:8].sum())))
    finally:
        dist.destroy_process_group()


def test_two_replicas_share_only_the_timing():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, rate0, slow0, tot0, x0), (r1, rate1, slow1, tot1, x1) = res
    assert slow0 == slow1 == 2.0          # max over ranks
    assert tot0 == tot1 == 300.0           # all ranks' work
    assert rate0 == rate1 == pytest.approx(150.0)  # 300 units / 2 s
    assert x0 != x1                        # each replica its own tracks


def test_single_process_is_its_own_job():
    rep = importlib.import_module(pkg().__name__ + ".replicas")
    assert rep.max_over_ranks(3.0) == 3.0
    assert rep.whole_job_rate(10.0, 2.0) == 5.0
    assert rep.replica_seed(7, 0) == 7 and rep.replica_seed(7, 3) == 10
