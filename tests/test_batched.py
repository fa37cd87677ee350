"""Batched runs: many configurations advanced together give each
configuration's own result (same tracks, same tallies to float32 rounding),
and the saturation-sweep definition is the documented one."""

import numpy as np
import pytest

from goldens import make_config, pkg

KS_ABS = 1e-5


def _mixed_batch(dtype_note=""):
    return [
        make_config("fast"),
        make_config("fast_dense", lateral_boundary="reflecting"),
        make_config("small_run"),
        make_config("rf_odd_noxy", scoring_region="full_grid"),
        make_config("fast_two_species"),
        make_config("aic144_dev"),
    ]


def test_saturation_sweep_definition():
    cfgs = pkg().saturation_sweep_configs()
    assert len(cfgs) == 64
    volts = [c.voltage_V for c in cfgs]
    assert volts[0] == pytest.approx(25.0) and volts[-1] == pytest.approx(400.0)
    assert all(b > a for a, b in zip(volts, volts[1:]))
    assert {c.electrode_gap_cm for c in cfgs} <= {0.1, 0.2, 0.3}
    assert all(1.0 <= c.dose_rate_Gy_s <= 100.0 for c in cfgs)
    assert all(100e-6 <= c.pulse_duration_s <= 1000e-6 for c in cfgs)
    assert {c.grid_size_um for c in cfgs} <= {5.0, 10.0}
    assert all(0.008 <= c.sampled_radius_cm <= 0.03 for c in cfgs)
    assert [c.seed for c in cfgs] == list(range(1, 65))
    sizes = [c.no_xy ** 2 * c.no_z_with_buffer for c in cfgs]
    assert max(sizes) / min(sizes) > 10  # uneven voxel counts
    again = pkg().saturation_sweep_configs()
    assert [c.number_of_tracks_per_pulse for c in again] == [c.number_of_tracks_per_pulse for c in cfgs]


def test_phases_cover_every_step_once():
    import importlib

    b = importlib.import_module(pkg().__name__ + ".batched")
    ph = b._phases([5, 3, 5, 9])
    assert ph == [(0, 3, [0, 1, 2, 3]), (3, 5, [0, 2, 3]), (5, 9, [3])]


def _ragged_schedules(rng, n):
    totals = [int(rng.integers(1, 60)) for _ in range(n)]
    offsets, base, b = [], [], 0
    for t in totals:
        sched = rng.integers(0, 5, size=t) * (rng.uniform(size=t) < 0.4)
        off = np.zeros(t + 1, dtype=np.int64)
        np.cumsum(sched, out=off[1:])
        offsets.append(off)
        base.append(b)
        b += int(off[-1])
    return offsets, totals, base


def test_deposition_tasks_of_every_global_step():
    """Per global step, one task per grid with tracks, in grid order: its
    grid, first packed track and the tracks of the step's earlier tasks."""
    import importlib

    b = importlib.import_module(pkg().__name__ + ".batched")
    rng = np.random.default_rng(9)
    for _ in range(50):
        offsets, totals, base = _ragged_schedules(rng, int(rng.integers(1, 8)))
        sizes = rng.integers(3, 300, size=len(totals))
        sto, stt, cfg, first, prefix, blocks = b._task_tables(offsets, totals, base, sizes)
        assert len(sto) == max(totals) + 1 and sto[0] == 0 and sto[-1] == len(cfg)
        for s in range(max(totals)):
            want = [(c, base[c] + offsets[c][s], offsets[c][s + 1] - offsets[c][s])
                    for c in range(len(totals)) if s < totals[c] and offsets[c][s + 1] > offsets[c][s]]
            got = range(sto[s], sto[s + 1])
            assert [(cfg[t], first[t]) for t in got] == [(c, f) for c, f, _ in want]
            assert [prefix[t] for t in got] == list(np.cumsum([0] + [m for _, _, m in want])[:-1])
            assert stt[s] == sum(m for _, _, m in want)
            tiles = lambda n: (-(-int(n) // 64)) ** 2  # noqa: E731
            assert blocks[s] == sum(tiles(sizes[c]) * min(32, max(1, -(-m // 32))) for c, _, m in want)


def test_chunks_ramp_up_and_cover_every_step_once():
    """The batched driver's chunks (CPU): every global step once, in order,
    none across a phase boundary, the first FIRST_CHUNK_STEPS long (or
    chunk_steps if shorter), then doubling up to chunk_steps."""
    b = _stream_mod()
    cfgs = pkg().saturation_sweep_configs()
    phases = b._phases([int(c.total_time_steps) for c in cfgs])
    tabs = [(s0, s1, {"active": a}) for s0, s1, a in phases]
    for chunk_steps in (1, 7, 16, 100, 512):
        chunks = b._ramp_chunks(tabs, chunk_steps)
        assert chunks[0][0] == 0 and chunks[-1][1] == phases[-1][1]
        assert all(x[1] == y[0] for x, y in zip(chunks, chunks[1:]))
        starts = {s0: s1 for s0, s1, _ in phases}
        for c0, c1, tab in chunks:
            s0 = tab["phase_start"]
            assert s0 <= c0 < c1 <= starts[s0] and 1 <= c1 - c0 <= chunk_steps
        assert chunks[0][1] - chunks[0][0] == min(b.FIRST_CHUNK_STEPS, chunk_steps, phases[0][1])
        # sizes double until chunk_steps, except where a phase ends first
        size = min(b.FIRST_CHUNK_STEPS, chunk_steps)
        for c0, c1, tab in chunks:
            assert c1 - c0 == min(size, starts[tab["phase_start"]] - c0)
            size = min(2 * size, chunk_steps)
    # with the steps' track counts: at most max_tracks a chunk (one step at
    # least), as long as the track budget allows, and still every step once
    rng = np.random.default_rng(5)
    stt = rng.integers(0, 40_000, size=phases[-1][1])
    for max_tracks in (1, 50_000, 1 << 20):
        chunks = b._ramp_chunks(tabs, 512, step_tracks=stt, max_tracks=max_tracks)
        assert chunks[0][0] == 0 and chunks[-1][1] == phases[-1][1]
        assert all(x[1] == y[0] for x, y in zip(chunks, chunks[1:]))
        for c0, c1, tab in chunks:
            n = int(stt[c0:c1].sum())
            assert c1 - c0 == 1 or n <= max_tracks
            assert c1 - c0 <= 512 and c1 <= starts[tab["phase_start"]]
            if c1 < starts[tab["phase_start"]] and c1 - c0 < 512:
                # cut by the budget or the ramp, not shorter than either allows
                assert n + int(stt[c1]) > max_tracks or c1 - c0 >= b.FIRST_CHUNK_STEPS


def test_work_tables_cover_each_active_grid_once():
    """One batched launch's blocks: every active grid's items split into
    contiguous, non-overlapping block ranges covering them exactly; inactive
    grids get no blocks."""
    import importlib

    b = importlib.import_module(pkg().__name__ + ".batched")
    rng = np.random.default_rng(4)
    for _ in range(200):
        n = int(rng.integers(1, 9))
        items = rng.integers(1, 3_000_000, size=n)
        active = sorted(rng.choice(n, size=int(rng.integers(1, n + 1)), replace=False).tolist())
        wt = b._work_table(items, active, int(rng.integers(1, 200)))
        assert wt["blk_cfg"].dtype == np.int32 and wt["cfg_blk0"].dtype == np.int32
        for c in range(n):
            b0, nb = int(wt["cfg_blk0"][c]), int(wt["cfg_nblk"][c])
            if c not in active:
                assert nb == 0
                continue
            blocks = range(b0, b0 + nb)
            assert nb >= 1 and all(wt["blk_cfg"][k] == c for k in blocks)
            i0, i1 = wt["blk_item0"][b0:b0 + nb], wt["blk_item1"][b0:b0 + nb]
            assert i0[0] == 0 and i1[-1] == items[c] and np.array_equal(i0[1:], i1[:-1])
            assert np.all(i1 > i0) or items[c] < nb
        assert len(wt["blk_cfg"]) == int(wt["cfg_nblk"].sum())


@pytest.mark.parametrize("kw, msg", [
    (dict(rngs=[np.random.default_rng(1)]), "1 generators for 2 configurations"),
    (dict(dtype="float16"), "dtype must be"),
    (dict(chunk_steps=0), "chunk_steps must be >= 1"),
    (dict(solo_grids=-1), "solo_grids must be >= 0"),
])
def test_batched_arguments_checked_before_device_work(kw, msg):
    """Inconsistent arguments are refused before any device work (and here,
    without a GPU): one generator per configuration, a known dtype, positive
    chunks."""
    with pytest.raises(ValueError, match=msg):
        pkg().run_batched_b200([make_config("fast"), make_config("small_run")], **kw)


@pytest.mark.gpu
def test_batched_matches_individual_runs():
    cfgs = _mixed_batch()
    batch = pkg().run_batched_b200(cfgs, return_fields=True)
    for cfg, got in zip(cfgs, batch):
        ref = pkg().run_simulation_b200(cfg, progress=False, use_graphs=False, shape={"variant": "flat"})
        np.testing.assert_array_equal(got.track_density_xy, ref.track_density_xy)
        assert abs(got.ks - ref.ks) <= 1e-6
        # Two float32 runs whose density atomics add in different orders (the
        # single-grid deposition spreads a track over several warps when a
        # step has few tracks) agree to float32 rounding carried through the
        # run: ~1e-6 of a tally's or a field's peak; the parity bar against the
        # float64 reference is 1e-5.
        for x, y in [(got.recombination, ref.recombination), (got.injected_positive, ref.injected_positive),
                     (got.n_positive, ref.n_positive), (got.n_negative, ref.n_negative)]:
            np.testing.assert_allclose(x, y, rtol=0, atol=1e-5 * max(np.abs(y).max(), 1e-300))
        peak = np.abs(ref.positive_array).max()
        np.testing.assert_allclose(got.positive_array, ref.positive_array, rtol=0, atol=peak * 1e-5)
        np.testing.assert_allclose(got.negative_array, ref.negative_array, rtol=0, atol=peak * 1e-5)


@pytest.mark.gpu
def test_batched_float64_matches_the_oracle(oracle):
    cfgs = _mixed_batch()
    batch = pkg().run_batched_b200(cfgs, dtype="float64")
    for cfg, got in zip(cfgs, batch):
        ref = oracle.run(cfg, mode="batched", threads=2, keep_fields=False)
        np.testing.assert_array_equal(got.track_density_xy, ref["track_density_xy"])
        assert got.ks == pytest.approx(ref["ks"], rel=1e-9)
        np.testing.assert_allclose(got.recombination, ref["recombined"], rtol=1e-9,
                                   atol=1e-9 * np.abs(ref["recombined"]).max())


@pytest.mark.gpu
def test_batched_sweep_subset_matches_the_oracle(oracle):
    """Eight configurations of the saturation sweep (uneven sizes and step
    counts), float32 batch against the float64 oracle at |dk_s| <= 1e-5."""
    cfgs = [c for c in pkg().saturation_sweep_configs() if c.no_xy ** 2 * c.no_z_with_buffer < 1.5e6][:8]
    assert len(cfgs) == 8
    batch = pkg().run_batched_b200(cfgs)
    for cfg, got in zip(cfgs, batch):
        ref = oracle.run(cfg, mode="batched", threads=8, keep_fields=False)
        np.testing.assert_array_equal(got.track_density_xy, ref["track_density_xy"])
        assert abs(got.ks - ref["ks"]) <= KS_ABS


def _check_against_sweep_fixture(results, idx, what):
    from goldens import histogram_sha256, oracle_fixture

    fx = oracle_fixture("oracle_sweep64")["configs"]
    assert len(fx) == 64
    bad = []
    for i, got in zip(idx, results):
        ref = fx[i]
        same_tracks = histogram_sha256(got.track_density_xy) == ref["track_sha256"]
        if np.isnan(ref["ks"]):
            # the reference's scheme diverges on this configuration (the
            # oracle's tallies overflow): the float32 run must not report a
            # finite k_s either
            ok = same_tracks and not np.isfinite(got.ks)
        else:
            ok = (same_tracks and abs(got.ks - ref["ks"]) <= KS_ABS
                  and abs(got.injected_positive.sum() / ref["injected_sum"] - 1.0) <= 1e-5
                  and abs(got.recombination.sum() / ref["recombined_sum"] - 1.0) <= 1e-5)
        if not ok:
            bad.append((i, got.ks, ref["ks"]))
    assert not bad, f"{what}: configurations off the float64 oracle: {bad}"


@pytest.mark.gpu
def test_whole_sweep_batched_matches_the_oracle_fixtures():
    """All 64 configurations of the saturation sweep in one float32 batched run,
    each against the float64 oracle's run of it (tests/golden/oracle_sweep64.json):
    identical tracks (histogram checksum), |dk_s| <= 1e-5, total injected and
    recombined charge within 1e-5 relative."""
    cfgs = pkg().saturation_sweep_configs()
    _check_against_sweep_fixture(pkg().run_batched_b200(cfgs), range(64), "batched")


@pytest.mark.gpu
def test_whole_sweep_plain_solves_match_the_oracle_fixtures():
    """The same 64 configurations through the plain solver, one after another."""
    cfgs = pkg().saturation_sweep_configs()
    res = [pkg().run_simulation_b200(c, progress=False, return_fields=False) for c in cfgs]
    _check_against_sweep_fixture(res, range(64), "plain")


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_persistent_launch_matches_per_step_launches(dtype):
    """The persistent form (one cooperative launch per chunk of global steps,
    device-wide barriers between the deposition and step phases) gives the
    per-step launches' results: identical tracks, k_s and tallies to the
    dtype's rounding; a chunk of 7 steps makes grids start and finish inside
    launches."""
    cfgs = _mixed_batch()
    a = pkg().run_batched_b200(cfgs, dtype=dtype, chunk_steps=7)
    b = pkg().run_batched_b200(cfgs, dtype=dtype, chunk_steps=7, persistent=True)
    tol = 1e-5 if dtype == "float32" else 1e-12
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.track_density_xy, y.track_density_xy)
        assert abs(x.ks - y.ks) <= tol
        np.testing.assert_allclose(y.recombination, x.recombination, rtol=0,
                                   atol=tol * max(np.abs(x.recombination).max(), 1e-300))


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_single_grid_phases_match_batched_launches(dtype):
    """Phases stepped grid by grid with the single-grid kernels (on the
    grids' slices of the packed buffers) against batched launches: no phase
    (solo_grids=0), the default (phases of at most two grids), and every
    phase; chunks of 7 steps hand the state over between the two paths many
    times. Identical tracks, k_s, tallies and fields to the dtype's rounding."""
    cfgs = _mixed_batch()
    runs = [pkg().run_batched_b200(cfgs, dtype=dtype, chunk_steps=7, solo_grids=k, return_fields=True)
            for k in (0, 2, len(cfgs))]
    tol = 1e-5 if dtype == "float32" else 1e-12
    for other in runs[1:]:
        for x, y in zip(runs[0], other):
            np.testing.assert_array_equal(x.track_density_xy, y.track_density_xy)
            assert abs(x.ks - y.ks) <= tol
            np.testing.assert_allclose(y.recombination, x.recombination, rtol=0,
                                       atol=tol * max(np.abs(x.recombination).max(), 1e-300))
            peak = max(np.abs(x.positive_array).max(), 1e-300)
            np.testing.assert_allclose(y.positive_array, x.positive_array, rtol=0, atol=tol * peak)
            np.testing.assert_allclose(y.negative_array, x.negative_array, rtol=0, atol=tol * peak)


def _stream_mod():
    import importlib

    return importlib.import_module(pkg().__name__ + ".batched")


def test_stream_items_cover_every_interior_voxel_once():
    """The streaming batched step's item table (CPU): for every phase of the
    64-grid sweep, each active grid's interior rows x planes are covered
    exactly once, a grid's items are consecutive, tiles fit the consumer
    threads and a ring stage, and every SM gets an item of the heavy phase."""
    B = _stream_mod()
    cfgs = pkg().saturation_sweep_configs()
    shapes = [(int(c.no_xy), int(c.no_z_with_buffer), (int(c.no_z_with_buffer) + 7) // 8 * 8) for c in cfgs]
    totals = [int(c.total_time_steps) for c in cfgs]
    for sms in (152, 7):
        for s0, s1, active in B._phases(totals):
            items, tiles = B._stream_items(shapes, active, sms)
            assert items.dtype == np.int32 and items.shape[1] == 4
            grids_seen = []
            for c in items[:, 0]:
                if not grids_seen or grids_seen[-1] != c:
                    assert c not in grids_seen, "items of a grid are not consecutive"
                    grids_seen.append(int(c))
            assert sorted(grids_seen) == sorted(active)
            for c in active:
                n, nzb, kp = shapes[c]
                tj = int(tiles[c])
                assert 1 <= tj <= n - 2 and tj * (kp // 4) <= B.STREAM_IPT * 32 * B.STREAM_WARPS
                assert B._stage_floats(tj, kp) * 4 <= B.STREAM_STAGE_BYTES
                cover = np.zeros((n, n), dtype=np.int32)  # (plane, row)
                for _, j0, i0, i1 in items[items[:, 0] == c]:
                    assert 1 <= j0 <= n - 2 and 1 <= i0 < i1 <= n - 1
                    cover[i0:i1, j0:min(j0 + tj, n - 1)] += 1
                assert (cover[1:-1, 1:-1] == 1).all() and cover[0].sum() == 0 and cover[-1].sum() == 0
                assert cover[:, 0].sum() == 0 and cover[:, -1].sum() == 0
        # the heavy first phase: about STREAM_ITEMS_PER_SM items per SM
        items, _ = B._stream_items(shapes, list(range(64)), sms)
        assert len(items) >= sms


def test_items_per_block_takes_one_block_per_slot_on_small_phases():
    """The flat batched step's work split (CPU): about WAVES blocks per
    resident slot on phases of at least SMALL_PHASE_ITEMS items, one below,
    in multiples of 256 items, within the bounds."""
    B = _stream_mod()
    slots = B.BLOCKS_PER_SM * 152
    big, small = B.SMALL_PHASE_ITEMS * 2, B.SMALL_PHASE_ITEMS // 5
    ipb_big, ipb_small = B.items_per_block(big, 152), B.items_per_block(small, 152)
    assert ipb_big % 256 == 0 and ipb_small % 256 == 0
    assert -(-big // ipb_big) <= B.WAVES * slots < -(-big // ipb_big) + slots
    assert -(-small // ipb_small) <= B.WAVES_SMALL * slots
    assert B.items_per_block(1, 152) == B.MIN_ITEMS_PER_BLOCK
    assert B.items_per_block(1 << 40, 1) == B.MAX_ITEMS_PER_BLOCK


def test_mixed_takes_the_streaming_step_on_the_heavy_phases_only():
    """variant="mixed" (CPU): the sweep's phases of many grids (above
    STREAM_MIN_VOXELS interior voxels a step) take the streaming step, those
    of a few grids the flat one; float64, persistent, variant="flat" and
    variant="auto" runs never stream, variant="stream" always does."""
    B = _stream_mod()
    cfgs = pkg().saturation_sweep_configs()
    shapes = [(int(c.no_xy), int(c.no_z_with_buffer), (int(c.no_z_with_buffer) + 7) // 8 * 8) for c in cfgs]
    totals = [int(c.total_time_steps) for c in cfgs]
    picks = [(len(a), B.stream_phase(shapes, a)) for _, _, a in B._phases(totals)]
    assert picks[0] == (64, True)
    assert all(not st for n, st in picks if n <= 19) and all(st for n, st in picks if n >= 40)
    # the choice only ever goes from streaming to flat: phases lose grids
    flags = [st for _, st in picks]
    assert flags == sorted(flags, reverse=True)
    every = list(range(64))
    assert not B.stream_phase(shapes, every, "flat")
    assert not B.stream_phase(shapes, every, "auto")
    assert not B.stream_phase(shapes, every, "mixed", dtype="float64")
    assert not B.stream_phase(shapes, every, "mixed", persistent=True)
    assert B.stream_phase(shapes, [63], "stream")


def test_stream_variant_arguments_are_checked_before_device_work():
    B = _stream_mod()
    cfg = make_config("fast")
    with pytest.raises(ValueError, match="variant"):
        B.run_batched_b200([cfg], variant="tiled")
    with pytest.raises(ValueError, match="float32"):
        B.run_batched_b200([cfg], variant="stream", dtype="float64")


@pytest.mark.gpu
@pytest.mark.parametrize("solo", [0, 2])
def test_stream_batched_step_matches_the_flat_one(solo):
    """The streaming batched step (items of every grid from a device-wide
    queue, planes staged in a shared-memory ring) against the flat batched
    step on the mixed batch (both walls, odd no_xy, the full-grid scoring
    region, two species): identical tracks, k_s and tallies within 1e-5,
    fields within 1e-5 of their peak; chunks of 7 global steps, with and
    without the single-grid tail phases."""
    cfgs = _mixed_batch()
    a = pkg().run_batched_b200(cfgs, chunk_steps=7, solo_grids=solo, variant="flat", return_fields=True)
    b = pkg().run_batched_b200(cfgs, chunk_steps=7, solo_grids=solo, variant="stream", return_fields=True)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.track_density_xy, y.track_density_xy)
        assert abs(x.ks - y.ks) <= KS_ABS
        np.testing.assert_allclose(y.recombination, x.recombination, rtol=0,
                                   atol=1e-5 * max(np.abs(x.recombination).max(), 1e-300))
        np.testing.assert_allclose(y.injected_positive, x.injected_positive, rtol=1e-5, atol=0)
        peak = max(np.abs(x.positive_array).max(), 1e-300)
        np.testing.assert_allclose(y.positive_array, x.positive_array, rtol=0, atol=1e-5 * peak)
        np.testing.assert_allclose(y.negative_array, x.negative_array, rtol=0, atol=1e-5 * peak)


@pytest.mark.gpu
def test_mixed_switches_from_the_streaming_to_the_flat_step(monkeypatch):
    """variant="mixed" with the streaming threshold set between the mixed
    batch's phases: the first phases stream, the later ones run flat (and the
    last ones solo), handing the fields, pairs and tallies across; against an
    all-flat run: identical tracks, k_s and tallies within 1e-5, fields within
    1e-5 of their peak."""
    B = _stream_mod()
    cfgs = _mixed_batch()
    shapes = [(int(c.no_xy), int(c.no_z_with_buffer), (int(c.no_z_with_buffer) + 7) // 8 * 8) for c in cfgs]
    phases = B._phases([int(c.total_time_steps) for c in cfgs])
    vox = [sum((shapes[c][0] - 2) ** 2 * (shapes[c][1] - 2) for c in a) for _, _, a in phases]
    assert len(vox) >= 3 and vox[0] > vox[1]
    monkeypatch.setattr(B, "STREAM_MIN_VOXELS", vox[1])
    assert [B.stream_phase(shapes, a) for _, _, a in phases][:3] == [True, True, False]
    a = pkg().run_batched_b200(cfgs, chunk_steps=7, variant="flat", return_fields=True)
    b = pkg().run_batched_b200(cfgs, chunk_steps=7, variant="mixed", return_fields=True)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.track_density_xy, y.track_density_xy)
        assert abs(x.ks - y.ks) <= KS_ABS
        np.testing.assert_allclose(y.recombination, x.recombination, rtol=0,
                                   atol=1e-5 * max(np.abs(x.recombination).max(), 1e-300))
        peak = max(np.abs(x.positive_array).max(), 1e-300)
        np.testing.assert_allclose(y.positive_array, x.positive_array, rtol=0, atol=1e-5 * peak)
        np.testing.assert_allclose(y.negative_array, x.negative_array, rtol=0, atol=1e-5 * peak)


@pytest.mark.gpu
def test_stream_batched_matches_the_oracle_on_sweep_grids(oracle):
    """Eight sweep configurations through the streaming batched step against
    the float64 oracle, with the streaming step forced on every phase."""
    cfgs = [c for c in pkg().saturation_sweep_configs() if c.no_xy ** 2 * c.no_z_with_buffer < 1.5e6][:8]
    batch = pkg().run_batched_b200(cfgs, variant="stream", solo_grids=0)
    for cfg, got in zip(cfgs, batch):
        ref = oracle.run(cfg, mode="batched", threads=8, keep_fields=False)
        np.testing.assert_array_equal(got.track_density_xy, ref["track_density_xy"])
        assert abs(got.ks - ref["ks"]) <= KS_ABS


@pytest.mark.gpu
def test_a_configuration_float32_cannot_follow_is_run_again_in_float64():
    """Sweep configuration 6 (32.6 V over 0.3 cm at 65 Gy/s, k_s 32.7) sits
    near the explicit scheme's recombination stability limit: an unstable mode
    grows a few per cent a step during the pulse, and float32 round-off makes it
    overflow where float64 round-off does not. The float32 call detects the
    non-finite tallies and returns the float64 run of the same tracks, within
    1e-5 of the oracle's k_s; a well-conditioned configuration stays float32."""
    from goldens import histogram_sha256, oracle_fixture

    fx = oracle_fixture("oracle_sweep64")["configs"]
    cfgs = pkg().saturation_sweep_configs()
    hard = pkg().run_simulation_b200(cfgs[6], progress=False, return_fields=False)
    assert hard.fields_dtype == "float64"
    assert abs(hard.ks - fx[6]["ks"]) <= KS_ABS
    assert histogram_sha256(hard.track_density_xy) == fx[6]["track_sha256"]
    easy = pkg().run_simulation_b200(cfgs[0], progress=False, return_fields=False)
    assert easy.fields_dtype == "float32" and abs(easy.ks - fx[0]["ks"]) <= KS_ABS
    nan = pkg().run_simulation_b200(cfgs[27], progress=False, return_fields=False)
    assert nan.fields_dtype == "float64" and not np.isfinite(nan.ks)  # as in the reference


# ------------------------------------------------ binned batched deposition


def test_binned_batched_deposition_workspace_and_arguments():
    """pic_batched_deposit_bytes: for each of 8 global steps a slot per grid,
    per-tile counts and lists and a packed pair buffer; per-track boxes and
    factors; the run's choices are checked before any device work."""
    import ctypes
    import importlib

    P = pkg()
    N = importlib.import_module(P.__name__ + "._native")
    B = importlib.import_module(P.__name__ + ".batched")
    lib = N.load()
    b = ctypes.c_int64()
    assert lib.pic_batched_deposit_bytes(64, 200, 248000, 3_300_000, N.PIC_F32, ctypes.byref(b)) == N.PIC_OK
    pad = lambda x: (x + 255) // 256 * 256  # noqa: E731
    rest = pad(8 * 200 * 4) + 8 * 200 * 4096 * 4 + pad(248000 * 8) + pad(248000 * 128 * 4) + 8 * pad(3_300_000)
    slot = (b.value - rest) // (8 * 64)
    assert 64 <= slot <= 128 and slot % 8 == 0  # one descriptor per grid and step of a launch pair
    assert lib.pic_batched_deposit_bytes(1025, 200, 10, 8, N.PIC_F32, ctypes.byref(b)) == N.PIC_E_INVALID
    assert lib.pic_batched_deposit_bytes(4, 0, 10, 8, N.PIC_F32, ctypes.byref(b)) == N.PIC_E_INVALID
    assert lib.pic_batched_deposit_bytes(4, 4, 10, 0, N.PIC_F32, ctypes.byref(b)) == N.PIC_E_INVALID
    assert lib.pic_batched_deposit_bytes(4, 4, 10, 8, 7, ctypes.byref(b)) == N.PIC_E_INVALID
    np.testing.assert_array_equal(B.binned_tiles([24, 62, 63, 124, 1068]), [1, 1, 4, 4, 324])
    grids = [type("G", (), dict(no_xy=n, cutoff_voxels=c))() for n, c in ((24, 14.1), (608, 28.3))]
    assert B.binned_eligible(grids)
    assert not B.binned_eligible(grids + [type("G", (), dict(no_xy=64, cutoff_voxels=31.6))()])
    with pytest.raises(ValueError, match="deposit"):
        B.run_batched_b200([make_config("fast")], deposit="atomic")


@pytest.mark.gpu
def test_binned_batched_deposition_matches_the_tile_form():
    """Every grid's tracks of a global step listed per tile and summed by one
    block per tile, against the tile form's atomics, on the mixed batch (both
    walls, odd no_xy, the full-grid scoring region, two species) and eight
    sweep grids: identical tracks, k_s and tallies within 1e-5, fields within
    1e-5 of their peak; chunks of 7 global steps, the single-grid tail phases
    off so that every step goes through the batched launches."""
    cfgs = _mixed_batch() + [c for c in pkg().saturation_sweep_configs()
                             if c.no_xy ** 2 * c.no_z_with_buffer < 1.5e6][:8]
    a = pkg().run_batched_b200(cfgs, chunk_steps=7, solo_grids=0, deposit="tiles", return_fields=True)
    b = pkg().run_batched_b200(cfgs, chunk_steps=7, solo_grids=0, deposit="binned", return_fields=True)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.track_density_xy, y.track_density_xy)
        assert abs(x.ks - y.ks) <= KS_ABS
        np.testing.assert_allclose(y.recombination, x.recombination, rtol=0,
                                   atol=1e-5 * max(np.abs(x.recombination).max(), 1e-300))
        np.testing.assert_allclose(y.injected_positive, x.injected_positive, rtol=1e-5, atol=0)
        peak = max(np.abs(x.positive_array).max(), 1e-300)
        np.testing.assert_allclose(y.positive_array, x.positive_array, rtol=0, atol=1e-5 * peak)
        np.testing.assert_allclose(y.negative_array, x.negative_array, rtol=0, atol=1e-5 * peak)
    # sums in a fixed order: the binned batched run repeats bit for bit
    c = pkg().run_batched_b200(cfgs, chunk_steps=7, solo_grids=0, deposit="binned", return_fields=True)
    for x, y in zip(b, c):
        assert x.ks == y.ks or (x.ks != x.ks and y.ks != y.ks)
        np.testing.assert_array_equal(x.recombination, y.recombination)
        np.testing.assert_array_equal(x.positive_array, y.positive_array)
