"""Pins the FP64 CPU oracle (oracle/) to the reference solver's own outputs.

The golden fixtures were produced by running pulsed_ion_chamber's
run_simulation_numba and its kernels (tests/golden/make_golden.py). The
oracle's serial mode restates that driver in the same float64 operation
order, so on one thread it should agree to the last few ulps; its batched mode
restates run_simulation_numba_parallel, which the reference itself only
guarantees to 1e-9 against the serial one (tests/test_backends_agree.py:22).
"""

import numpy as np
import pytest

from goldens import available, run_config, run_fixture

RUNS = [
    "run_fast_base", "run_fast_reflecting", "run_fast_full_grid", "run_fast_two_species", "run_fast_nocutoff",
    "run_fast_dense", "run_fast_dense_reflect_full", "run_small_absorbing", "run_small_reflecting",
    "run_aic144_dev",
]
SERIAL_RTOL = 1e-12
BATCHED_RTOL = 1e-9


def _check(res, fx, rtol):
    np.testing.assert_array_equal(res["track_density_xy"], fx["track_density_xy"])
    for key, ref in [("injected", "injected"), ("recombined", "recombination"), ("n_positive", "n_positive"),
                     ("n_negative", "n_negative")]:
        scale = max(np.abs(fx[ref]).max(), 1e-300)
        np.testing.assert_allclose(res[key], fx[ref], rtol=rtol, atol=scale * rtol, err_msg=key)
    np.testing.assert_allclose(res["f_t"], fx["f_t"], rtol=rtol)
    assert res["ks"] == pytest.approx(float(fx["ks"]), rel=rtol)
    if "positive_array" in fx:
        peak = np.abs(fx["positive_array"]).max()
        np.testing.assert_allclose(res["positive"], fx["positive_array"], rtol=0, atol=peak * rtol)
        np.testing.assert_allclose(res["negative"], fx["negative_array"], rtol=0, atol=peak * rtol)


@pytest.mark.parametrize("name", RUNS)
def test_serial_oracle_matches_reference(oracle, name):
    if not available(name):
        pytest.skip(f"{name} fixture not generated")
    cfg, fx = run_config(name)
    res = oracle.run(cfg, mode="serial", threads=1)
    _check(res, fx, SERIAL_RTOL)


@pytest.mark.parametrize("name", RUNS)
def test_batched_oracle_matches_reference(oracle, name):
    if not available(name):
        pytest.skip(f"{name} fixture not generated")
    cfg, fx = run_config(name)
    res = oracle.run(cfg, mode="batched", threads=2)
    _check(res, fx, BATCHED_RTOL)


def test_serial_oracle_matches_reference_on_a_1622_step_column(oracle):
    """24 x 24 x 206, 22 837 tracks over 1 412 pulse steps (10 um voxels,
    r = 0.008 cm, seed 1): the small plain-method workload, whole run."""
    name = "run_column_10um_r008"
    if not available(name):
        pytest.skip("fixture not generated")
    cfg, fx = run_config(name)
    res = oracle.run(cfg, mode="batched", threads=4, keep_fields=False)
    _check(res, fx, BATCHED_RTOL)


def test_published_dev_tier_k_s(oracle):
    """The reference CLI's dev tier reports k_s = 1.0580 (tests/test_examples_cli.py:24-53)."""
    cfg, fx = run_config("run_aic144_dev")
    res = oracle.run(cfg, mode="batched", threads=2, keep_fields=False)
    assert res["ks"] == pytest.approx(1.0580, abs=1e-4)


@pytest.mark.parametrize("name", ["step_small_track_disc", "step_small_full_grid", "step_small_two_species"])
def test_kernel_level_deposit_and_sweep(oracle, name):
    """One deposit of 30 tracks and one sweep through the oracle kernels equal
    the reference kernels' outputs (tests/test_charge_conservation.py)."""
    import ctypes

    cfg, fx = run_config(name)
    L = oracle.lib()
    shape = (cfg.no_xy, cfg.no_xy, cfg.no_z_with_buffer)
    pos = np.zeros(shape)
    neg = np.zeros(shape)
    ins = 0.0
    h2, b2 = cfg.unit_length_cm**2, cfg.track_radius_cm**2
    for x, y in zip(fx["xs"], fx["ys"]):
        ins += L.oracle_insert_track(oracle._p(pos), oracle._p(neg), float(x), float(y), cfg.no_xy,
                                     cfg.no_z_with_buffer, cfg.no_z, cfg.no_z_electrode, h2, b2,
                                     cfg.Gaussian_factor, cfg.mid_xy, cfg.scoring_radius_sq, cfg.track_cutoff_voxels)
    assert ins == pytest.approx(float(fx["inserted"]), rel=1e-13)
    np.testing.assert_array_equal(pos, fx["positive"])
    dens = np.zeros((cfg.no_xy, cfg.no_xy))
    xs, ys = np.ascontiguousarray(fx["xs"]), np.ascontiguousarray(fx["ys"])
    L.oracle_accumulate_density(oracle._p(dens), oracle._p(xs), oracle._p(ys), len(xs), cfg.no_xy, h2, b2,
                                cfg.track_cutoff_voxels)
    np.testing.assert_allclose(dens, fx["total_density"], rtol=1e-13, atol=1e-300)
    pn, nn = np.zeros(shape), np.zeros(shape)
    out = np.zeros(3)
    (pl, pzm, pzp, pc), (nl, nzm, nzp, nc) = cfg.scheme_coefficients()
    oracle.set_threads(1)
    L.oracle_lw_step(oracle._p(pos), oracle._p(neg), oracle._p(pn), oracle._p(nn), cfg.no_xy, cfg.no_z_with_buffer,
                     cfg.no_z_electrode, cfg.no_z, cfg.mid_xy, cfg.scoring_radius_sq, pl, pzm, pzp, pc, nl, nzm, nzp,
                     nc, float(fx["alpha_dt"]), oracle._p(out))
    np.testing.assert_array_equal(pn, fx["positive_next"])
    np.testing.assert_array_equal(nn, fx["negative_next"])
    assert out[0] == float(fx["recombined"])
    assert out[1] == float(fx["total_positive"])
    assert out[2] == float(fx["total_negative"])
