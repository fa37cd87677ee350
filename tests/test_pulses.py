"""Track scheduling and placement reproduce the reference's RNG stream bit for
bit (pulsed_ion_chamber/pulses.py:39-171), at every configuration size."""

import hashlib
import importlib

import numpy as np
import pytest

from goldens import GOLDEN, config_json, make_config, pkg

NAMES = sorted(p.stem[len("config_"):] for p in GOLDEN.glob("config_*.json"))


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_block_sampler_matches_the_per_track_sampler_on_uneven_batches():
    z = np.load(GOLDEN / "sampler.npz")
    s = pkg().TrackSampler(np.random.default_rng(11), 30, 24.0, 60)
    got = np.vstack([np.column_stack(s.sample(int(n))) for n in z["batches"]])
    np.testing.assert_array_equal(got, z["xy"])


def test_sampler_with_float_centre_and_empty_batches():
    z = np.load(GOLDEN / "sampler.npz")
    s = pkg().TrackSampler(np.random.default_rng(4), 12.5, 9.5, 25)
    got = np.vstack([np.column_stack(s.sample(n)) for n in [0, 5, 4096, 1, 0, 17]])
    np.testing.assert_array_equal(got, z["xy_odd"])


def test_sampler_stays_inside_the_disc():
    xs, ys = pkg().TrackSampler(np.random.default_rng(2), 30, 24.0, 60).sample(20_000)
    assert len(xs) == 20_000
    assert np.all((xs - 30) ** 2 + (ys - 30) ** 2 <= 24.0**2)


@pytest.mark.parametrize("name", NAMES)
def test_schedule_and_first_pulse_tracks_are_bit_identical(name):
    """Whole-pulse sampling in one call equals the reference's per-step calls:
    the property that lets a pulse be uploaded once and replayed as a graph."""
    ref = config_json(name)
    cfg = make_config(name)
    rng = np.random.default_rng(cfg.seed)
    sched = pkg().build_track_schedule(cfg, rng)
    assert _sha(sched) == ref["schedule_sha256"]
    assert int(sched.sum()) == ref["schedule_sum"]
    n_first = int(sched[: cfg.pulse_time_steps].sum())
    assert n_first == ref["first_pulse_tracks"]
    xs, ys = pkg().TrackSampler(rng, cfg.mid_xy, cfg.sampling_radius, cfg.no_xy).sample(n_first)
    assert list(xs[:8]) == ref["first_pulse_xs_head"]
    assert _sha(xs) == ref["first_pulse_xs_sha256"]
    assert _sha(ys) == ref["first_pulse_ys_sha256"]


def _numpy_disc_scan(u, scale, mid, r2, wanted):
    """The reference's array expression over the uniforms (pulses.py:84-171)."""
    x = u[0::2] * scale
    y = u[1::2] * scale
    idx = np.flatnonzero((x - mid) ** 2 + (y - mid) ** 2 <= r2)[:wanted]
    return x[idx], y[idx]


def test_native_disc_scan_equals_the_numpy_expression():
    """pic_sample_disc against the NumPy expression on the 64 sweep configs'
    disc geometries (integer and half-integer centres, radii up to the grid
    edge) and on draws landing exactly on the disc boundary."""
    import ctypes

    import importlib

    N = importlib.import_module(pkg().__name__ + "._native")
    lib = N.load()
    rng = np.random.default_rng(99)
    geoms = [(c.no_xy, c.mid_xy, c.sampling_radius) for c in pkg().saturation_sweep_configs()]
    geoms += [(25, 12.5, 9.5), (60, 30, 24.0), (7, 3.5, 3.5)]
    for no_xy, mid, rad in geoms:
        u = rng.random(2 * 5000)
        u[:8] = [0.5, 0.5, 0.0, 0.0, (mid + rad) / no_xy, mid / no_xy, 0.999999, 0.5]  # centre, corner, boundary
        for wanted in (1, 37, 10_000):
            xs, ys = np.empty(wanted), np.empty(wanted)
            acc, used = ctypes.c_int64(), ctypes.c_int64()
            N.check(lib.pic_sample_disc(u.ctypes.data, u.size // 2, float(no_xy), float(mid), float(rad * rad),
                                        wanted, xs.ctypes.data, ys.ctypes.data, ctypes.byref(acc),
                                        ctypes.byref(used)), "pic_sample_disc")
            ex, ey = _numpy_disc_scan(u, no_xy, mid, rad * rad, wanted)
            assert acc.value == len(ex)
            np.testing.assert_array_equal(xs[: acc.value], ex)
            np.testing.assert_array_equal(ys[: acc.value], ey)
            if acc.value == wanted:
                x = u[0::2] * no_xy
                y = u[1::2] * no_xy
                last = used.value - 1
                assert x[last] == ex[-1] and y[last] == ey[-1]
            else:
                assert used.value == u.size // 2


def test_arrival_counts_equal_numpy_histogram():
    """The per-step arrival histogram (drawn and binned natively for a PCG64
    generator) equals np.histogram over the same edges (pulses.py:39-61), for
    the golden configurations, the sweep and extra seeds, and leaves the
    generator where NumPy's own draws leave it."""
    cfgs = [make_config(n) for n in NAMES] + pkg().saturation_sweep_configs()
    for cfg in cfgs:
        for seed in (cfg.seed, 7):
            mine = np.random.default_rng(seed)
            a = importlib.import_module(pkg().__name__ + ".pulses").pulse_arrival_counts(cfg, mine)
            rng = np.random.default_rng(seed)
            arrival = np.cumsum(rng.random(int(cfg.number_of_tracks_per_pulse)))
            arrival /= arrival[-1]
            arrival *= cfg.pulse_duration_s
            ref, _ = np.histogram(arrival, cfg.pulse_time_bins)
            np.testing.assert_array_equal(a, ref)
            assert mine.random() == rng.random()  # the generator continues at the same point


@pytest.mark.parametrize("geom", [(60, 30, 24.0), (25, 12.5, 9.5), (95, 47.5, 43.5), (7, 3.5, 3.5)])
def test_native_pcg64_draws_equal_numpy_draws(geom):
    """The PCG64 path (doubles drawn natively from the generator's state)
    gives the same centres as drawing through NumPy, across uneven and empty
    batches, and leaves the generator exactly past the doubles consumed."""
    no_xy, mid, rad = geom
    a = pkg().TrackSampler(np.random.default_rng(5), mid, rad, no_xy)
    b = pkg().TrackSampler(np.random.default_rng(5), mid, rad, no_xy, native_rng=False)
    assert a._pcg64 and not b._pcg64
    for n in (0, 1, 3, 5000, 0, 17, 100_000, 2):
        xa, ya = a.sample(n)
        xb, yb = b.sample(n)
        np.testing.assert_array_equal(xa, xb)
        np.testing.assert_array_equal(ya, yb)
    # the generator sits where a plain NumPy draw of the consumed doubles ends
    rng = np.random.default_rng(5)
    ref = pkg().TrackSampler(np.random.default_rng(5), mid, rad, no_xy)
    xs, ys = ref.sample(1234)
    consumed = 0
    u = rng.random(10_000_000)
    x, y = u[0::2] * no_xy, u[1::2] * no_xy
    idx = np.flatnonzero((x - mid) ** 2 + (y - mid) ** 2 <= rad * rad)
    consumed = 2 * (int(idx[1233]) + 1)
    rng2 = np.random.default_rng(5)
    rng2.random(consumed)
    assert ref.rng.random() == rng2.random()


def test_other_bit_generators_take_the_numpy_draw_path():
    g = np.random.Generator(np.random.MT19937(3))
    s = pkg().TrackSampler(g, 30, 24.0, 60)
    assert not s._pcg64
    xs, ys = s.sample(1000)
    assert np.all((xs - 30) ** 2 + (ys - 30) ** 2 <= 24.0**2)


@pytest.mark.parametrize("seed", [1, 99])
def test_threaded_arrival_counts_equal_numpys_at_full_electrode_size(seed):
    """The native schedule of a 25 M-arrival pulse (draws split over the host
    cores by PCG64 jump-ahead, one running-sum pass, bins by binary search)
    against NumPy's own random + cumsum + histogram: identical counts, and
    the generator left at the same state (the next draws agree)."""
    import importlib

    P = pkg()
    pulses = importlib.import_module(P.__name__ + ".pulses")
    beam = dict(E_MeV_u=56.2, voltage_V=300.0, electrode_gap_cm=0.2, pulse_duration_s=540e-6,
                repetition_rate_hz=50.0, dose_rate_Gy_s=8.91)
    cfg = P.SimulationConfig(**dict(beam, grid_size_um=5.0, sampled_radius_cm=0.265, seed=1, max_voxels=2e9))
    n = int(cfg.number_of_tracks_per_pulse)
    assert n > 1 << 20  # the threaded path
    r_native, r_numpy = np.random.default_rng(seed), np.random.default_rng(seed)
    got = pulses.pulse_arrival_counts(cfg, r_native)
    arrival = np.cumsum(r_numpy.random(n))
    arrival /= arrival[-1]
    arrival *= cfg.pulse_duration_s
    want = np.histogram(arrival, np.asarray(cfg.pulse_time_bins, dtype=np.float64))[0]
    np.testing.assert_array_equal(got, want)
    assert r_native.bit_generator.state == r_numpy.bit_generator.state
    np.testing.assert_array_equal(r_native.random(8), r_numpy.random(8))


def test_schedules_drawn_on_threads_equal_the_sequential_ones():
    """The batched driver draws its configurations' schedules on a thread
    pool (each with its own generator; the native draws release the
    interpreter): the 64 sweep schedules and the generators' end states equal
    those of one-after-another draws."""
    from concurrent.futures import ThreadPoolExecutor

    P = pkg()
    pulses = importlib.import_module(P.__name__ + ".pulses")
    cfgs = P.saturation_sweep_configs()
    seq_rngs = [np.random.default_rng(c.seed) for c in cfgs]
    par_rngs = [np.random.default_rng(c.seed) for c in cfgs]
    seq = [pulses.build_track_schedule(c, r) for c, r in zip(cfgs, seq_rngs)]
    with ThreadPoolExecutor(max_workers=8) as pool:
        par = list(pool.map(pulses.build_track_schedule, cfgs, par_rngs))
    for a, b, ra, rb in zip(seq, par, seq_rngs, par_rngs):
        np.testing.assert_array_equal(a, b)
        assert ra.bit_generator.state == rb.bit_generator.state
