"""The run record (state.py) against loops restating the reference's own
bookkeeping: the track histogram (pulsed_ion_chamber/state.py:67-69, one
``int()``-floored voxel per centre), f(t) from running float64 totals
(pulsed_ion_chamber/solver_numba.py:281, :350; all ones when nothing was
injected yet or the run stopped early) and the Result's columns
(state.py:92-110). Bit-exact; no GPU."""

import importlib

import numpy as np
import pytest

from goldens import make_config, pkg


def _state():
    return importlib.import_module(pkg().__name__ + ".state")


def test_count_tracks_equals_one_floored_count_per_centre():
    cfg = make_config("fast")
    n = int(cfg.no_xy)
    rng = np.random.default_rng(3)
    xs = rng.uniform(0.0, n, size=5000)
    ys = rng.uniform(0.0, n, size=5000)
    xs[:50], ys[:50] = xs[0], ys[0]  # many centres in one voxel
    d = _state().Diagnostics(cfg)
    d.count_tracks(xs, ys)
    d.count_tracks(xs[:7], ys[:7])  # accumulates over calls
    want = np.zeros((n, n))
    for x, y in zip(np.concatenate([xs, xs[:7]]), np.concatenate([ys, ys[:7]])):
        want[int(x), int(y)] += 1.0
    assert np.array_equal(d.track_density_xy, want)
    assert d.track_density_xy.sum() == 5007


def _f_loop(injected, recombined, steps_completed):
    f = np.ones(len(injected))
    tot_i = tot_r = 0.0
    for s in range(steps_completed):
        tot_i += injected[s]
        tot_r += recombined[s]
        f[s] = 1.0 if tot_i == 0.0 else (tot_i - tot_r) / tot_i
    return f


@pytest.mark.parametrize("steps_completed", [0, 1, 37, 400])
def test_collection_efficiency_equals_running_totals(steps_completed):
    rng = np.random.default_rng(5)
    injected = rng.uniform(0.0, 1e6, size=400) * (rng.uniform(size=400) < 0.3)
    injected[:9] = 0.0  # nothing injected during the first steps
    recombined = injected * rng.uniform(0.0, 0.2, size=400) + rng.uniform(0.0, 10.0, size=400)
    recombined[:9] = 0.0
    got = _state().collection_efficiency(injected, recombined, steps_completed)
    assert np.array_equal(got, _f_loop(injected, recombined, steps_completed))
    assert np.all(got[steps_completed:] == 1.0)


def test_result_columns():
    cfg = make_config("fast")
    st = _state()
    steps = int(cfg.total_time_steps)
    d = st.Diagnostics(cfg)
    tallies = np.arange(4.0 * steps).reshape(steps, 4)
    d.record_block(0, tallies[:10])
    d.record_block(10, tallies[10:])
    d.record(3, 7.0, 8.0, 9.0, 10.0)
    r = d.build_result(cfg, np.arange(steps) * cfg.dt, np.ones(steps), 1.25, np.zeros(1), np.zeros(1))
    want = tallies.copy()
    want[3] = (7.0, 8.0, 9.0, 10.0)
    assert np.array_equal(r.injected_positive, want[:, 0])
    assert np.array_equal(r.recombination, want[:, 1])
    assert np.array_equal(r.n_positive, want[:, 2]) and np.array_equal(r.n_negative, want[:, 3])
    # one positive and one negative carrier per track: equal columns, separate arrays
    assert np.array_equal(r.injected_negative, r.injected_positive)
    assert r.injected_negative is not r.injected_positive
    assert r.ks == 1.25 and r.config is cfg and r.track_density_xy.shape == (cfg.no_xy, cfg.no_xy)
