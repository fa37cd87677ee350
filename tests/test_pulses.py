"""Track scheduling and placement reproduce the reference's RNG stream bit for
bit (pulsed_ion_chamber/pulses.py:39-171), at every configuration size."""

import hashlib

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
