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
        sto, stt, cfg, first, prefix = b._task_tables(offsets, totals, base)
        assert len(sto) == max(totals) + 1 and sto[0] == 0 and sto[-1] == len(cfg)
        for s in range(max(totals)):
            want = [(c, base[c] + offsets[c][s], offsets[c][s + 1] - offsets[c][s])
                    for c in range(len(totals)) if s < totals[c] and offsets[c][s + 1] > offsets[c][s]]
            got = range(sto[s], sto[s + 1])
            assert [(cfg[t], first[t]) for t in got] == [(c, f) for c, f, _ in want]
            assert [prefix[t] for t in got] == list(np.cumsum([0] + [m for _, _, m in want])[:-1])
            assert stt[s] == sum(m for _, _, m in want)


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
