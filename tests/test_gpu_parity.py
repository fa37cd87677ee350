"""GPU parity: run_simulation_b200 against the reference's own outputs (golden
fixtures) and against the FP64 oracle, through the C ABI on the GB300.

Tolerances, per the project's parity bar:
* track positions: identical (track_density_xy bit-equal);
* float32 fields (production): |dk_s| <= 1e-5, cumulative injected and
  recombined charge within 1e-5 relative, per-step tallies within 1e-5 of
  their peak;
* float64 fields (validation build): the same quantities within 1e-9
  relative (the remaining difference is summation order and fused
  multiply-adds).
"""

import ctypes
import importlib
import os

import numpy as np
import pytest

from goldens import available, make_config, pkg, run_config, run_fixture

pytestmark = pytest.mark.gpu

KS_ABS = 1e-5
TALLY_REL = 1e-5
F64_REL = 1e-9

RUNS = [
    "run_fast_base", "run_fast_reflecting", "run_fast_full_grid", "run_fast_two_species", "run_fast_nocutoff",
    "run_fast_dense", "run_fast_dense_reflect_full", "run_small_absorbing", "run_small_reflecting",
    "run_aic144_dev",
]


def _solver():
    return pkg().run_simulation_b200


def _check_f32(res, ks, injected, recombined, n_pos, n_neg, tracks):
    np.testing.assert_array_equal(res.track_density_xy, tracks)
    assert abs(res.ks - ks) <= KS_ABS, (res.ks, ks)
    assert res.injected_positive.sum() == pytest.approx(injected.sum(), rel=TALLY_REL)
    assert res.recombination.sum() == pytest.approx(recombined.sum(), rel=TALLY_REL)
    for got, want in [(res.injected_positive, injected), (res.recombination, recombined),
                      (res.n_positive, n_pos), (res.n_negative, n_neg)]:
        peak = np.abs(want).max()
        np.testing.assert_allclose(got, want, rtol=0, atol=TALLY_REL * peak)


@pytest.mark.parametrize("name", RUNS)
def test_float32_run_matches_reference(name):
    cfg, fx = run_config(name)
    res = _solver()(cfg, progress=False)
    _check_f32(res, float(fx["ks"]), fx["injected"], fx["recombination"], fx["n_positive"], fx["n_negative"],
               fx["track_density_xy"])
    if "positive_array" in fx:
        peak = np.abs(fx["positive_array"]).max()
        np.testing.assert_allclose(res.positive_array, fx["positive_array"], rtol=0, atol=peak * 1e-5)
        np.testing.assert_allclose(res.negative_array, fx["negative_array"], rtol=0, atol=peak * 1e-5)


@pytest.mark.parametrize("name", RUNS)
def test_float64_run_matches_reference(name):
    cfg, fx = run_config(name)
    res = _solver()(cfg, progress=False, dtype="float64")
    np.testing.assert_array_equal(res.track_density_xy, fx["track_density_xy"])
    assert res.ks == pytest.approx(float(fx["ks"]), rel=F64_REL)
    for got, key in [(res.injected_positive, "injected"), (res.recombination, "recombination"),
                     (res.n_positive, "n_positive"), (res.n_negative, "n_negative")]:
        peak = np.abs(fx[key]).max()
        np.testing.assert_allclose(got, fx[key], rtol=F64_REL, atol=F64_REL * peak, err_msg=key)
    if "positive_array" in fx:
        peak = np.abs(fx["positive_array"]).max()
        np.testing.assert_allclose(res.positive_array, fx["positive_array"], rtol=0, atol=peak * F64_REL)
        np.testing.assert_allclose(res.negative_array, fx["negative_array"], rtol=0, atol=peak * F64_REL)


def test_plain_method_column_whole_run():
    """24 x 24 x 206 at 10 um, r = 0.008 cm, seed 1: 1 622 steps, 22 837 tracks."""
    name = "run_column_10um_r008"
    if not available(name):
        pytest.skip("fixture not generated")
    cfg, fx = run_config(name)
    res = _solver()(cfg, progress=False, return_fields=False)
    _check_f32(res, float(fx["ks"]), fx["injected"], fx["recombination"], fx["n_positive"], fx["n_negative"],
               fx["track_density_xy"])


def test_published_dev_tier_k_s():
    """The reference CLI's dev tier: k_s = 1.0580 (tests/test_examples_cli.py:24-53)."""
    cfg, fx = run_config("run_aic144_dev")
    res = _solver()(cfg, progress=False, return_fields=False)
    assert res.ks == pytest.approx(1.0580, abs=1e-4)


def test_fields_mid_run_match_the_oracle(oracle):
    """The whole field, not only its tallies, at a step inside the pulse of a
    grid with many tracks per step (fields and tallies in float64 mode)."""
    cfg = make_config("rf_odd_noxy")  # odd no_xy: float centre
    k = 120
    ref = oracle.run(cfg, mode="batched", threads=4, max_steps=k + 1)
    res = _solver()(cfg, progress=False, max_steps=k + 1, dtype="float64")
    peak = np.abs(ref["positive"]).max()
    np.testing.assert_allclose(res.positive_array, ref["positive"], rtol=0, atol=peak * F64_REL)
    np.testing.assert_allclose(res.negative_array, ref["negative"], rtol=0, atol=peak * F64_REL)
    res32 = _solver()(cfg, progress=False, max_steps=k + 1)
    np.testing.assert_allclose(res32.positive_array, ref["positive"], rtol=0, atol=peak * 1e-5)


def test_max_steps_truncates_and_reports():
    cfg, _ = run_config("run_fast_dense")
    full = _solver()(cfg, progress=False)
    part = _solver()(cfg, progress=False, max_steps=5)
    assert part.steps_completed == 5
    assert part.loop_elapsed_s > 0
    assert np.isnan(part.ks)
    # float32 density sums use atomics, so two runs agree to float32
    # rounding, not bit for bit
    np.testing.assert_allclose(part.f_t[:5], full.f_t[:5], rtol=1e-7)


def test_max_wall_s_stops_and_reports():
    cfg, _ = run_config("run_fast_dense")
    res = _solver()(cfg, progress=False, max_wall_s=0.0, chunk_steps=4)
    assert res.steps_completed == 4
    assert np.isnan(res.ks)


def test_return_fields_false_drops_only_the_snapshot():
    cfg, _ = run_config("run_fast_dense")
    full = _solver()(cfg, progress=False)
    lean = _solver()(cfg, progress=False, return_fields=False)
    assert lean.positive_array.size == 0 and lean.negative_array.size == 0
    assert lean.ks == pytest.approx(full.ks, rel=1e-6)


def test_rejects_bad_dtype():
    cfg, _ = run_config("run_fast_base")
    with pytest.raises(ValueError, match="dtype"):
        _solver()(cfg, progress=False, dtype="float16")


def test_multi_pulse_run_against_the_oracle(oracle):
    """Three pulses with idle gaps between them: the pulse/idle segmenting and
    the density-buffer parity across segments."""
    cfg = make_config("fast_dense", n_pulses=3, repetition_rate_hz=20000.0)
    assert cfg.pulse_period_steps > cfg.pulse_time_steps
    ref = oracle.run(cfg, mode="batched", threads=2)
    res = _solver()(cfg, progress=False, chunk_steps=7)
    np.testing.assert_array_equal(res.track_density_xy, ref["track_density_xy"])
    assert abs(res.ks - ref["ks"]) <= KS_ABS
    res64 = _solver()(cfg, progress=False, dtype="float64", chunk_steps=5)
    assert res64.ks == pytest.approx(ref["ks"], rel=F64_REL)
    np.testing.assert_allclose(res64.recombination, ref["recombined"], rtol=F64_REL,
                               atol=F64_REL * np.abs(ref["recombined"]).max())


@pytest.mark.parametrize("name", ["step_small_track_disc", "step_small_full_grid", "step_small_two_species"])
def test_kernel_level_deposit_and_step(name):
    """pic_deposit + pic_step through the C ABI on the reference's single-step
    fixture (tests/test_charge_conservation.py): injected, recombined and the
    carrier totals, and the stepped fields."""
    import torch

    eng_mod = importlib.import_module(pkg().__name__ + ".engine")
    N = importlib.import_module(pkg().__name__ + "._native")
    cfg, fx = run_config(name)
    for dtype, tol in (("float64", 1e-12), ("float32", 1e-5)):
        eng = eng_mod.ChamberEngine(cfg, dtype=dtype, max_tracks=len(fx["xs"]))
        eng.upload_tracks(fx["xs"], fx["ys"], non_blocking=False)
        eng.run_segment(np.array([0, len(fx["xs"])]))
        torch.cuda.synchronize()
        t = eng.tallies(1)[0]
        assert t[0] == pytest.approx(float(fx["inserted"]), rel=tol)
        assert t[1] == pytest.approx(float(fx["recombined"]), rel=tol)
        assert t[2] == pytest.approx(float(fx["total_positive"]), rel=tol)
        assert t[3] == pytest.approx(float(fx["total_negative"]), rel=tol)
        pos, neg = eng.fields()
        ref_pos = fx["positive_next"].copy()
        peak = np.abs(fx["positive"]).max()
        inner = (slice(1, -1), slice(1, -1), slice(None))
        np.testing.assert_allclose(pos[inner], ref_pos[inner], rtol=0, atol=peak * tol)
        np.testing.assert_allclose(neg[inner], fx["negative_next"][inner], rtol=0, atol=peak * tol)
        # deposition pairs: (G * density, G * the four lateral neighbours' density)
        n, G = int(cfg.no_xy), float(cfg.Gaussian_factor)
        pairs = eng.dens[0].view(n, -1, 2)[:, :n].cpu().numpy().astype(np.float64)
        ref = fx["total_density"]
        np.testing.assert_allclose(pairs[..., 0] / G, ref, rtol=tol, atol=tol * ref.max())
        lat = np.zeros_like(ref)
        lat[1:] += ref[:-1]
        lat[:-1] += ref[1:]
        lat[:, 1:] += ref[:, :-1]
        lat[:, :-1] += ref[:, 1:]
        np.testing.assert_allclose(pairs[..., 1] / G, lat, rtol=tol, atol=tol * lat.max())
        eng.close()


STREAM_SHAPES = {
    "tiny_tiles": dict(variant="stream", tile_rows=3, planes_per_item=5, stages=4, consumer_warps=2),
    "mid": dict(variant="stream", tile_rows=7, planes_per_item=9, stages=6, consumer_warps=5),
    "default": dict(variant="stream"),
}
STREAM_RUNS = ["run_fast_base", "run_fast_reflecting", "run_fast_full_grid", "run_fast_two_species",
               "run_fast_dense", "run_fast_dense_reflect_full", "run_small_absorbing", "run_small_reflecting",
               "run_aic144_dev"]


@pytest.mark.parametrize("shape", sorted(STREAM_SHAPES))
@pytest.mark.parametrize("name", STREAM_RUNS)
def test_stream_variant_matches_reference(name, shape):
    """The shared-memory streaming kernel, forced on small grids with several
    tiles and work items per grid, against the reference fixtures."""
    cfg, fx = run_config(name)
    res = _solver()(cfg, progress=False, shape=STREAM_SHAPES[shape])
    _check_f32(res, float(fx["ks"]), fx["injected"], fx["recombination"], fx["n_positive"], fx["n_negative"],
               fx["track_density_xy"])
    if "positive_array" in fx:
        peak = np.abs(fx["positive_array"]).max()
        np.testing.assert_allclose(res.positive_array, fx["positive_array"], rtol=0, atol=peak * 1e-5)
        np.testing.assert_allclose(res.negative_array, fx["negative_array"], rtol=0, atol=peak * 1e-5)


MULTI_SHAPES = {"two": 2, "seven": 7, "max": 256}


@pytest.mark.parametrize("graphs", [False, True])
@pytest.mark.parametrize("spl", sorted(MULTI_SHAPES))
@pytest.mark.parametrize("name", STREAM_RUNS)
def test_multistep_launches_match_reference(name, spl, graphs):
    """Several steps per cooperative launch (steps_per_launch 2, 7 and 256:
    launches that end inside pulses and idle stretches, with and without
    CUDA graphs) against the reference fixtures, float32."""
    cfg, fx = run_config(name)
    res = _solver()(cfg, progress=False, use_graphs=graphs,
                    shape={"variant": "flat", "steps_per_launch": MULTI_SHAPES[spl]})
    _check_f32(res, float(fx["ks"]), fx["injected"], fx["recombination"], fx["n_positive"], fx["n_negative"],
               fx["track_density_xy"])
    if "positive_array" in fx:
        peak = np.abs(fx["positive_array"]).max()
        np.testing.assert_allclose(res.positive_array, fx["positive_array"], rtol=0, atol=peak * 1e-5)
        np.testing.assert_allclose(res.negative_array, fx["negative_array"], rtol=0, atol=peak * 1e-5)


@pytest.mark.parametrize("wall", ["absorbing", "reflecting"])
def test_multistep_float64_matches_the_oracle(oracle, wall):
    """Float64 fields, 5 steps per launch: k_s and the recombined tally per
    step equal the float64 oracle's to 1e-10; the tracks are identical."""
    cfg = make_config("fast_dense", lateral_boundary=wall, n_pulses=3, repetition_rate_hz=20000.0)
    res = _solver()(cfg, progress=False, dtype="float64", shape={"variant": "flat", "steps_per_launch": 5})
    ref = oracle.run(cfg, mode="batched", threads=2)
    np.testing.assert_array_equal(res.track_density_xy, ref["track_density_xy"])
    assert res.ks == pytest.approx(ref["ks"], rel=1e-10)
    np.testing.assert_allclose(res.recombination, ref["recombined"], rtol=1e-10,
                               atol=1e-10 * np.abs(ref["recombined"]).max())


LARGE_STREAM_SHAPES = {
    "default": {"variant": "stream"},
    # 12 consumer warps, 4 and 3 k-vectors a thread: the kernel's wide forms
    "wide4": {"variant": "stream", "tile_rows": 15, "consumer_warps": 12, "stages": 4},
    "wide3": {"variant": "stream", "tile_rows": 11, "consumer_warps": 12, "stages": 5},
    "wide3_15": {"variant": "stream", "tile_rows": 14, "consumer_warps": 15, "stages": 4},
    # 16 consumer warps, 2 and 3 k-vectors a thread (17-warp forms)
    "wide2_16": {"variant": "stream", "tile_rows": 10, "consumer_warps": 16, "stages": 5},
    "wide3_16": {"variant": "stream", "tile_rows": 15, "consumer_warps": 16, "stages": 4},
}


@pytest.mark.parametrize("shape", sorted(LARGE_STREAM_SHAPES))
@pytest.mark.parametrize("wall", ["absorbing", "reflecting"])
def test_stream_and_flat_agree_on_a_large_grid(wall, shape):
    """208 x 208 x 406 (5 um, r = 0.05 cm), 40 steps of the pulse at 89.1 Gy/s
    (~3 000 tracks a step): the two kernels give the same fields and tallies
    to float32 rounding."""
    cfg = make_config("column_5um_r05_d89p1", lateral_boundary=wall)
    a = _solver()(cfg, progress=False, max_steps=40, shape={"variant": "flat"})
    b = _solver()(cfg, progress=False, max_steps=40, shape=LARGE_STREAM_SHAPES[shape])
    np.testing.assert_array_equal(a.track_density_xy, b.track_density_xy)
    for x, y in [(a.recombination, b.recombination), (a.n_positive, b.n_positive), (a.injected_positive,
                                                                                     b.injected_positive)]:
        np.testing.assert_allclose(x[:40], y[:40], rtol=2e-6, atol=0)
    peak = np.abs(a.positive_array).max()
    np.testing.assert_allclose(b.positive_array, a.positive_array, rtol=0, atol=peak * 2e-6)
    np.testing.assert_allclose(b.negative_array, a.negative_array, rtol=0, atol=peak * 2e-6)


def test_stream_fields_mid_run_match_the_oracle(oracle):
    cfg = make_config("rf_odd_noxy", lateral_boundary="reflecting")
    k = 90
    ref = oracle.run(cfg, mode="batched", threads=4, max_steps=k + 1)
    res = _solver()(cfg, progress=False, max_steps=k + 1, shape=dict(variant="stream", tile_rows=4,
                                                                     planes_per_item=6))
    peak = np.abs(ref["positive"]).max()
    np.testing.assert_allclose(res.positive_array, ref["positive"], rtol=0, atol=peak * 1e-5)
    np.testing.assert_allclose(res.negative_array, ref["negative"], rtol=0, atol=peak * 1e-5)
    assert res.recombination[:k + 1].sum() == pytest.approx(ref["recombined"][:k + 1].sum(), rel=TALLY_REL)


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_graph_replay_matches_direct_launches(oracle, dtype):
    """Chunks replayed from CUDA graphs (captured once, replayed for every
    pulse and idle stretch with the same parities) give the same run as
    launching every step directly."""
    cfg = make_config("fast_dense", n_pulses=4, repetition_rate_hz=20000.0)
    a = _solver()(cfg, progress=False, use_graphs=False, chunk_steps=3, dtype=dtype)
    b = _solver()(cfg, progress=False, use_graphs=True, chunk_steps=3, dtype=dtype)
    np.testing.assert_array_equal(a.track_density_xy, b.track_density_xy)
    tol = 1e-6 if dtype == "float32" else 1e-12
    np.testing.assert_allclose(b.recombination, a.recombination, rtol=tol, atol=tol * np.abs(a.recombination).max())
    np.testing.assert_allclose(b.n_positive, a.n_positive, rtol=tol, atol=tol * np.abs(a.n_positive).max())
    assert b.ks == pytest.approx(a.ks, rel=tol)
    ref = oracle.run(cfg, mode="batched", threads=2)
    assert abs(b.ks - ref["ks"]) <= (KS_ABS if dtype == "float32" else 1e-10)


# The reference's published 5 um full-electrode run (AIC-144 chamber physics,
# 1066 x 1066 x 410 with no_z_electrode = 5 as its GPU bench builds it,
# profiling/bench_gpu.py:70-88; 4 580 steps, 24 630 400 tracks, reflecting
# wall, seed 20260527): k_s from its CUDA float64 solver,
# profiling/data/gpu_athena/gpu_5um_full_electrode.json ("gpu_ks"); its CPU
# run gives 1.1104725894530167 (cpu_5um_full_electrode.json).
PUBLISHED_FULL_ELECTRODE_KS = 1.1104725894530176


def _published_full_electrode_config():
    return make_config("aic144_full_electrode_5um", no_z_electrode=5)


def test_full_electrode_float32_matches_the_published_ks():
    """463 M voxels, the whole pulse and clearance (4 580 steps): float32
    fields within 1e-5 of the reference's published k_s (measured 3.5e-7)."""
    cfg = _published_full_electrode_config()
    assert (cfg.no_xy, cfg.no_z_with_buffer, cfg.total_time_steps) == (1066, 410, 4580)
    res = _solver()(cfg, progress=False, return_fields=False)
    assert abs(res.ks - PUBLISHED_FULL_ELECTRODE_KS) <= KS_ABS


@pytest.mark.skipif(os.environ.get("PIC_FULL_SCALE_F64") != "1",
                    reason="about 100 s of float64 on the GPU; set PIC_FULL_SCALE_F64=1")
def test_full_electrode_float64_matches_the_published_ks():
    """The same run with float64 fields: the reference's published k_s to
    float64 rounding (measured |dk_s| = 4.4e-16)."""
    res = _solver()(_published_full_electrode_config(), progress=False, return_fields=False, dtype="float64")
    assert abs(res.ks - PUBLISHED_FULL_ELECTRODE_KS) <= 1e-12


# The reference's published 10 um ladder (same chamber, sampled radius varied;
# no_z_electrode = 5; 2 194 steps): (radius cm, no_xy, k_s) from
# profiling/data/gpu_athena/ladder_10um.json -- its CPU and CUDA float64 runs
# agree on every row.
PUBLISHED_LADDER_10UM = [
    (0.014, 34, 1.101078104284521),
    (0.05, 106, 1.108750400628538),
    (0.08, 166, 1.1098094977890123),
    (0.12, 246, 1.1104074023012953),
    (0.18, 366, 1.1108197003228455),
    (0.265, 536, 1.1110811651442554),
]


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("radius, no_xy, ks", PUBLISHED_LADDER_10UM)
def test_published_10um_ladder(radius, no_xy, ks, dtype):
    cfg = make_config("aic144_full_electrode_5um", grid_size_um=10.0, sampled_radius_cm=radius, no_z_electrode=5)
    assert (cfg.no_xy, cfg.no_z_with_buffer, cfg.total_time_steps) == (no_xy, 210, 2194)
    res = _solver()(cfg, progress=False, return_fields=False, dtype=dtype)
    assert abs(res.ks - ks) <= (KS_ABS if dtype == "float32" else 1e-12)


CONFIGS1 = [(dose, seed) for dose in ("column_5um_r05_d8p91", "column_5um_r05_d89p1") for seed in (1, 2, 3, 4)]


@pytest.mark.parametrize("name, seed", CONFIGS1)
def test_plain_method_at_scale_matches_the_oracle(name, seed):
    """The plain method at scale: 5 um voxels, r = 0.05 cm (208 x 208 x 406,
    3 388 steps), 8.91 and 89.1 Gy/s, seeds 1-4, one configuration per
    launch: each float32 run against the float64 oracle's run of the same
    configuration (tests/golden/oracle_column_5um_r05.json): identical tracks,
    |dk_s| <= 1e-5, total injected and recombined charge within 1e-5."""
    from goldens import histogram_sha256, oracle_fixture

    ref = oracle_fixture("oracle_column_5um_r05")["runs"][f"{name}_seed{seed}"]
    cfg = make_config(name, seed=seed)
    assert (cfg.no_xy, cfg.no_z_with_buffer, cfg.total_time_steps) == (ref["no_xy"], ref["nzb"],
                                                                       ref["total_time_steps"])
    res = _solver()(cfg, progress=False, return_fields=False)
    assert histogram_sha256(res.track_density_xy) == ref["track_sha256"]
    assert int(res.track_density_xy.sum()) == ref["n_tracks"]
    assert abs(res.ks - ref["ks"]) <= KS_ABS
    assert res.injected_positive.sum() == pytest.approx(ref["injected_sum"], rel=TALLY_REL)
    assert res.recombination.sum() == pytest.approx(ref["recombined_sum"], rel=TALLY_REL)


def test_plain_method_at_scale_matches_the_live_oracle(oracle):
    """One of them end to end against the float64 oracle run here, in the same
    process (89.1 Gy/s, seed 1, 8.9 M tracks): the fixture's numbers are the
    oracle's."""
    cfg = make_config("column_5um_r05_d89p1")
    res = _solver()(cfg, progress=False, return_fields=False)
    ref = oracle.run(cfg, mode="batched", threads=16, keep_fields=False)
    np.testing.assert_array_equal(res.track_density_xy, ref["track_density_xy"])
    assert abs(res.ks - ref["ks"]) <= KS_ABS
    assert res.recombination.sum() == pytest.approx(ref["recombined"].sum(), rel=TALLY_REL)


def test_autotuner_chooses_steps_per_launch():
    """The autotuner times a flat float32 grid's idle steps as one CUDA graph
    of per-step launches and as cooperative launches of 32 and 256 steps, and
    keeps the fastest; the run with its choice matches the reference."""
    eng_mod = importlib.import_module(pkg().__name__ + ".engine")
    at = importlib.import_module(pkg().__name__ + ".autotune")
    cfg, fx = run_config("run_fast_dense")
    eng = eng_mod.ChamberEngine(cfg, dtype="float32")
    best = at.tune(eng, quick=True, reps=3, use_cache=False)
    tried = dict(best["steps_per_launch"])
    assert sorted(tried) == [0, 32, 256] and all(ms > 0 for ms in tried.values())
    chosen = best["shape"].get("steps_per_launch", 0)
    assert tried[chosen] == min(tried.values())
    eng.close()
    res = _solver()(cfg, progress=False, shape=best["shape"])
    _check_f32(res, float(fx["ks"]), fx["injected"], fx["recombination"], fx["n_positive"], fx["n_negative"],
               fx["track_density_xy"])


def test_bounded_waits_expire_with_a_status_and_leave_the_context_usable():
    """The kernels' two bounded waits, against partners that never come (a
    device-wide barrier one block never reaches; an mbarrier nothing arrives
    on), give up with their status codes instead of hanging; a run on the same
    context afterwards still matches the reference."""
    import torch

    N = importlib.import_module(pkg().__name__ + "._native")
    lib = N.load()
    b, m = ctypes.c_int32(-1), ctypes.c_int32(-1)
    N.check(lib.pic_selftest_waits(ctypes.byref(b), ctypes.byref(m), torch.cuda.current_stream().cuda_stream),
            "pic_selftest_waits")
    assert (b.value, m.value) == (5, 91)
    cfg, fx = run_config("run_fast_base")
    res = _solver()(cfg, progress=False)
    _check_f32(res, float(fx["ks"]), fx["injected"], fx["recombination"], fx["n_positive"], fx["n_negative"],
               fx["track_density_xy"])
