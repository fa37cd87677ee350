"""Slab decomposition of one grid over several ranks (CPU, gloo).

The plan (slabs.py: partition along i, one halo plane per side, tracks to
every slab their written box meets, one plane per species per neighbour per
step) is run by a float64 slab step written here in NumPy, on gloo ranks that
exchange their halo planes with send/recv, and compared with one run of the
oracle over the whole grid: the fields bit for bit (every voxel sees the same
float64 operations in the same order), the summed tallies and k_s to 1e-12
(their sums are added in another order).
"""

from __future__ import annotations

import importlib
import os
import socket

import numpy as np
import pytest

from goldens import make_config, pkg


def _slabs():
    return importlib.import_module(pkg().__name__ + ".slabs")


# ----------------------------------------------------------------- the plan


def test_partition_owns_every_plane_once():
    S = _slabs()
    for n in (5, 8, 25, 30, 1068):
        for world in range(1, min(n - 2, 9) + 1):
            sl = S.partition(n, world)
            assert [s.rank for s in sl] == list(range(world))
            assert sl[0].i0 == 0 and sl[-1].i1 == n
            assert all(a.i1 == b.i0 for a, b in zip(sl[:-1], sl[1:]))
            for s in sl:
                a, b = s.interior(n)
                assert b > a  # every rank steps at least one plane
                assert s.lo == max(s.i0 - 1, 0) and s.hi == min(s.i1 + 1, n)
            shares = [s.interior(n)[1] - s.interior(n)[0] for s in sl]
            assert sum(shares) == n - 2 and max(shares) - min(shares) <= 1
    with pytest.raises(ValueError):
        S.partition(4, 3)


def test_halo_exchanges_fill_every_halo_from_its_owner():
    S = _slabs()
    sl = S.partition(40, 4)
    ex = S.halo_exchanges(sl)
    assert len(ex) == 2 * 3
    for src, dst, plane in ex:
        assert sl[src].i0 <= plane < sl[src].i1  # the sender owns it
        assert sl[dst].lo <= plane < sl[dst].hi and not sl[dst].i0 <= plane < sl[dst].i1  # a halo of the receiver
    halos = {(dst, plane) for _, dst, plane in ex}
    for s in sl:
        want = {p for p in (s.lo, s.hi - 1) if not s.i0 <= p < s.i1}
        assert {p for d, p in halos if d == s.rank} == want


def test_tracks_go_to_every_slab_their_box_meets():
    S = _slabs()
    rng = np.random.default_rng(3)
    n, cut = 60, 4.7
    xs = rng.uniform(0, n, 500)
    sl = S.partition(n, 3)
    lo, hi = S.track_rows(xs, cut, n)
    for t, x in enumerate(xs):
        rows = set(range(max(int(np.ceil(x - cut)) - 1, 0), min(int(np.floor(x + cut)) + 2, n)))
        assert rows == set(range(lo[t], hi[t]))
        owners = {s.rank for s in sl if t in set(S.tracks_of(s, xs, cut, n))}
        assert owners == {s.rank for s in sl if rows & set(range(s.lo, s.hi))}


def test_sizing_of_the_full_electrode_split():
    S = _slabs()
    n, kp = 1068, 408
    one = S.slab_bytes(S.partition(n, 1)[0], n, kp)
    assert one == 4 * n * n * kp * 4  # 7.45 GB of float32 fields
    assert S.ranks_needed(n, kp, 288e9) == 1
    assert S.ranks_needed(n, kp, 2e9) >= 4
    assert S.halo_bytes_per_step(n, kp, 2) == 4 * n * kp * 4  # ~7 MB a step between two GPUs


# ------------------------------------------------- the plan run on gloo ranks


def _slab_run(cfg, rank, world, send, recv):
    """The batched driver of the reference (solver_numba_parallel.py:526-723:
    deposit the step's tracks as a 2D density, broadcast it into the gap
    layers, Lax-Wendroff step with recombination, lateral wall, swap), over
    the planes this rank holds. Returns its owned fields and tally sums."""
    from oracle import oracle

    S = _slabs()
    n, nzb, no_z, nze = int(cfg.no_xy), int(cfg.no_z_with_buffer), int(cfg.no_z), int(cfg.no_z_electrode)
    slab = S.partition(n, world)[rank]
    L = oracle.lib()
    rng = np.random.default_rng(cfg.seed)
    sched = oracle.schedule(cfg, rng)
    sampler = oracle.DiscSampler(rng, cfg.mid_xy, cfg.sampling_radius, n)
    (p_lat, p_zm, p_zp, p_cen), (n_lat, n_zm, n_zp, n_cen) = cfg.scheme_coefficients()
    alpha_dt = oracle.RECOMBINATION_ALPHA_CM3_S * cfg.dt
    h2, b2, G, cut = cfg.unit_length_cm ** 2, cfg.track_radius_cm ** 2, cfg.Gaussian_factor, cfg.track_cutoff_voxels
    reflecting = cfg.lateral_boundary == "reflecting"
    shape = (slab.planes, n, nzb)
    pos, neg, pos_n, neg_n = (np.zeros(shape) for _ in range(4))
    ia, ib = slab.interior(n)
    gi = np.arange(slab.lo, slab.hi)
    di = gi.astype(np.float64) - cfg.mid_xy
    dj = np.arange(n, dtype=np.float64) - cfg.mid_xy
    inside = (di[:, None] * di[:, None] + dj[None, :] * dj[None, :]) < cfg.scoring_radius_sq
    own_i = (gi >= ia) & (gi < ib)
    own_j = (np.arange(n) >= 1) & (np.arange(n) <= n - 2)
    scored = inside & own_i[:, None] & own_j[None, :]
    tallies = np.zeros(4)  # injected, recombined, sum n+, sum n-
    A, B = ia - slab.lo, ib - slab.lo  # owned interior planes, local
    for step in range(int(cfg.total_time_steps)):
        m = int(sched[step])
        if m > 0:
            xs, ys = sampler(m)
            t = S.tracks_of(slab, xs, cut, n)
            dens = np.zeros((n, n))
            if len(t):
                x, y = np.ascontiguousarray(xs[t]), np.ascontiguousarray(ys[t])
                L.oracle_accumulate_density(oracle._p(dens), oracle._p(x), oracle._p(y), len(t), n, h2, b2, cut)
            d = dens[slab.lo:slab.hi] * G
            pos[:, :, nze:nze + no_z] += d[:, :, None]
            neg[:, :, nze:nze + no_z] += d[:, :, None]
            tallies[0] += float((d * no_z)[scored].sum())
        # the step over the owned interior planes, term for term as the oracle
        c = (slice(A, B), slice(1, n - 1), slice(1, nzb - 1))
        P, N = pos[c], neg[c]
        pkm, pkp = pos[A:B, 1:n - 1, 0:nzb - 2], pos[A:B, 1:n - 1, 2:nzb]
        nkm, nkp = neg[A:B, 1:n - 1, 0:nzb - 2], neg[A:B, 1:n - 1, 2:nzb]
        p_new = (p_zm * pkm + p_zp * pkp + p_lat * pos[A:B, 0:n - 2, 1:nzb - 1] + p_lat * pos[A:B, 2:n, 1:nzb - 1]
                 + p_lat * pos[A - 1:B - 1, 1:n - 1, 1:nzb - 1] + p_lat * pos[A + 1:B + 1, 1:n - 1, 1:nzb - 1]
                 + p_cen * P)
        n_new = (n_zm * nkp + n_zp * nkm + n_lat * neg[A:B, 0:n - 2, 1:nzb - 1] + n_lat * neg[A:B, 2:n, 1:nzb - 1]
                 + n_lat * neg[A - 1:B - 1, 1:n - 1, 1:nzb - 1] + n_lat * neg[A + 1:B + 1, 1:n - 1, 1:nzb - 1]
                 + n_cen * N)
        rec = alpha_dt * P * N
        pos_n[c] = p_new - rec
        neg_n[c] = n_new - rec
        gap = slice(nze - 1, nze - 1 + no_z)  # gap layers among k = 1 .. nzb-2
        sc = scored[A:B, 1:n - 1]
        tallies[1] += float(rec[:, :, gap][sc].sum())
        tallies[2] += float(pos_n[c][:, :, gap][sc].sum())
        tallies[3] += float(neg_n[c][:, :, gap][sc].sum())
        if reflecting:
            pos, pos_n = pos_n, pos
            neg, neg_n = neg_n, neg
            for a in (pos, neg):
                if slab.i0 == 0:
                    a[0] = a[1]
                if slab.i1 == n:
                    a[-1] = a[-2]
                a[:, 0] = a[:, 1]
                a[:, n - 1] = a[:, n - 2]
        else:
            for dst, src in ((pos_n, pos), (neg_n, neg)):
                if slab.i0 == 0:
                    dst[0] = src[0]
                if slab.i1 == n:
                    dst[-1] = src[-1]
                dst[:, 0] = src[:, 0]
                dst[:, n - 1] = src[:, n - 1]
            pos, pos_n = pos_n, pos
            neg, neg_n = neg_n, neg
        # the neighbours' new planes into this rank's halos
        for a in (pos, neg):
            if rank > 0:
                send(rank - 1, a[slab.i0 - slab.lo])
            if rank < world - 1:
                send(rank + 1, a[slab.i1 - 1 - slab.lo])
            if rank > 0:
                a[0] = recv(rank - 1, a[0].shape)
            if rank < world - 1:
                a[-1] = recv(rank + 1, a[-1].shape)
    return pos[slab.i0 - slab.lo:slab.i1 - slab.lo], neg[slab.i0 - slab.lo:slab.i1 - slab.lo], tallies


def _worker(rank, world, port, name, wall, out):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pending = []

    def send(dst, plane):
        pending.append(dist.isend(torch.from_numpy(np.ascontiguousarray(plane)), dst))

    def recv(src, shape):
        buf = torch.empty(shape, dtype=torch.float64)
        dist.recv(buf, src)
        for w in pending:
            w.wait()
        pending.clear()
        return buf.numpy()

    cfg = make_config(name, lateral_boundary=wall)
    p, q, t = _slab_run(cfg, rank, world, send, recv)
    tt = torch.from_numpy(t)
    dist.all_reduce(tt)
    np.savez(out + f".{rank}.npz", pos=p, neg=q, tallies=tt.numpy())
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("name, wall, world", [("fast_dense", "absorbing", 2), ("fast_dense", "reflecting", 3),
                                               ("rf_odd_noxy", "absorbing", 2)])
def test_slab_run_on_gloo_ranks_matches_the_oracle(tmp_path, oracle, name, wall, world):
    import torch.multiprocessing as mp

    out = str(tmp_path / "slab")
    mp.start_processes(_worker, args=(world, _free_port(), name, wall, out), nprocs=world, start_method="spawn")
    cfg = make_config(name, lateral_boundary=wall)
    ref = oracle.run(cfg, mode="batched", threads=1, keep_fields=True)
    parts = [np.load(out + f".{r}.npz") for r in range(world)]
    pos = np.concatenate([p["pos"] for p in parts])
    neg = np.concatenate([p["neg"] for p in parts])
    np.testing.assert_array_equal(pos, ref["positive"])
    np.testing.assert_array_equal(neg, ref["negative"])
    t = parts[0]["tallies"]
    assert np.array_equal(t, parts[-1]["tallies"])
    ri, rr = ref["injected"].sum(), ref["recombined"].sum()
    assert t[0] == pytest.approx(ri, rel=1e-12) and t[1] == pytest.approx(rr, rel=1e-12)
    assert t[2] == pytest.approx(ref["n_positive"].sum(), rel=1e-12)
    assert t[3] == pytest.approx(ref["n_negative"].sum(), rel=1e-12)
    ks = ri / (ri - rr)
    assert (t[0] / (t[0] - t[1])) == pytest.approx(ks, rel=1e-12) and ks == pytest.approx(ref["ks"], rel=1e-12)
