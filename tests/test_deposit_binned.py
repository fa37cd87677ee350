"""The binned tile deposition (PIC_DEPOSIT_BINNED) against the oracle's
density and against the per-track form, through pic_run_segment.

The binned form lists each track in the 62 x 62-cell tiles its box meets and
sums each tile's tracks in ascending index order as outer products of the
tracks' row and column factors; the neighbours' sum comes from the density
tile afterwards. Checked here:
* the pairs (G * density, G * the four lateral neighbours' density) equal the
  float64 oracle's density (oracle_accumulate_density, the reference's
  _accumulate_track_density_numba_parallel) to 1e-12 of the peak in float64
  and 2e-6 in float32, on grids of one tile, ragged tiles and several tiles,
  with short (rank-sorted) and long (bitonic-sorted) tile lists;
* a tile reached by more tracks than its list holds (4096) scans every track
  and gives the same pairs;
* two depositions of the same tracks give identical pairs (no atomics on the
  pairs, a fixed summation order), and the track counts equal the per-track
  form's;
* the per-tile counts are back at zero after each step;
* whole runs with the binned form match the oracle's fixtures as the other
  forms do, and repeat bit for bit;
* pic_deposit, which has no workspace, refuses BINNED.
"""

from __future__ import annotations

import ctypes
import importlib

import numpy as np
import pytest

from goldens import pkg, run_config

pytestmark = pytest.mark.gpu

BEAM = dict(E_MeV_u=56.2, voltage_V=300.0, electrode_gap_cm=0.2, pulse_duration_s=540e-6,
            repetition_rate_hz=50.0, dose_rate_Gy_s=8.91)
# (voxel um, sampled radius cm) -> no_xy: (10, 0.008) 24 (one tile), (10, 0.05)
# 108, (5, 0.03) 128 (ragged tiles), (5, 0.08) 328 (six tiles a side)
GRIDS = {"n24": (10.0, 0.008), "n108": (10.0, 0.05), "n128": (5.0, 0.03), "n328": (5.0, 0.08)}
FIXED_WORKSPACE = 152 * 32 * 4 * 8 + 256  # tally partials, counter and status of the step workspace


def _mods():
    P = pkg()
    return P, importlib.import_module(P.__name__ + ".engine"), importlib.import_module(P.__name__ + "._native")


def _config(grid):
    P, _, _ = _mods()
    um, r = GRIDS[grid]
    return P.SimulationConfig(**dict(BEAM, grid_size_um=um, sampled_radius_cm=r, seed=1, max_voxels=2e9))


def _tracks(n, m, seed, cluster=None):
    rng = np.random.default_rng(seed)
    if cluster is None:
        return rng.uniform(0.0, n, m), rng.uniform(0.0, n, m)
    cx, cy, w = cluster
    return np.clip(rng.uniform(cx - w, cx + w, m), 0, n - 1e-9), np.clip(rng.uniform(cy - w, cy + w, m), 0, n - 1e-9)


def _deposit(cfg, xs, ys, dtype, variant):
    """One segment step from zero fields: the step's pairs, the track counts
    and the workspace's per-tile count area after the step."""
    import torch

    _, E, _ = _mods()
    eng = E.ChamberEngine(cfg, dtype=dtype, max_tracks=len(xs), shape={"deposit_variant": variant})
    try:
        eng.upload_tracks(xs, ys, non_blocking=False)
        eng.run_segment(np.array([0, len(xs)]))
        torch.cuda.synchronize()
        n = int(cfg.no_xy)
        pairs = eng.dens[0].view(n, -1, 2)[:, :n].cpu().numpy().astype(np.float64)
        counts = eng.counts.cpu().numpy().copy()
        tps = (n + 61) // 62
        bins = eng.workspace[FIXED_WORKSPACE:FIXED_WORKSPACE + 4 * tps * tps].cpu().numpy().view(np.int32).copy()
        return pairs, counts, bins
    finally:
        eng.close()


def _oracle_pairs(oracle, cfg, xs, ys):
    n = int(cfg.no_xy)
    dens = np.zeros((n, n))
    L = oracle.lib()
    x, y = np.ascontiguousarray(xs), np.ascontiguousarray(ys)
    L.oracle_accumulate_density(oracle._p(dens), oracle._p(x), oracle._p(y), len(x), n, cfg.unit_length_cm ** 2,
                                cfg.track_radius_cm ** 2, cfg.track_cutoff_voxels)
    G = float(cfg.Gaussian_factor)
    lat = np.zeros_like(dens)
    lat[1:] += dens[:-1]
    lat[:-1] += dens[1:]
    lat[:, 1:] += dens[:, :-1]
    lat[:, :-1] += dens[:, 1:]
    return G * dens, G * lat


def _close(pairs, c, l, tol):
    np.testing.assert_allclose(pairs[..., 0], c, rtol=0, atol=tol * np.abs(c).max())
    np.testing.assert_allclose(pairs[..., 1], l, rtol=0, atol=tol * np.abs(l).max())


@pytest.mark.parametrize("dtype, tol", [("float64", 1e-12), ("float32", 2e-6)])
@pytest.mark.parametrize("grid, m", [("n24", 40), ("n108", 700), ("n128", 300), ("n328", 3000), ("n328", 30000)])
def test_binned_pairs_match_the_oracle(oracle, grid, m, dtype, tol):
    cfg = _config(grid)
    n = int(cfg.no_xy)
    xs, ys = _tracks(n, m, seed=m + n)
    pairs, counts, bins = _deposit(cfg, xs, ys, dtype, "binned")
    c, l = _oracle_pairs(oracle, cfg, xs, ys)
    _close(pairs, c, l, tol)
    want = np.zeros((n, n), dtype=np.int64)
    np.add.at(want, (xs.astype(np.int64), ys.astype(np.int64)), 1)
    np.testing.assert_array_equal(counts, want)
    assert not bins.any()  # every tile's count cleared by its block


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_binned_and_per_track_forms_agree(dtype):
    cfg = _config("n328")
    n = int(cfg.no_xy)
    xs, ys = _tracks(n, 5000, seed=7)
    a, ca, _ = _deposit(cfg, xs, ys, dtype, "binned")
    b, cb, _ = _deposit(cfg, xs, ys, dtype, "tracks")
    tol = 1e-12 if dtype == "float64" else 2e-6
    _close(a, b[..., 0], b[..., 1], tol)
    np.testing.assert_array_equal(ca, cb)


def test_a_tile_with_more_tracks_than_its_list_scans_them_all(oracle):
    """5000 tracks within 3 cells of one point: every tile their boxes meet
    lists more than 4096, so those tiles scan the step's tracks."""
    cfg = _config("n328")
    n = int(cfg.no_xy)
    xs, ys = _tracks(n, 5000, seed=11, cluster=(100.0, 200.0, 3.0))
    xs2, ys2 = _tracks(n, 500, seed=12)  # and tracks elsewhere, listed normally
    xs, ys = np.concatenate([xs, xs2]), np.concatenate([ys, ys2])
    pairs, _, bins = _deposit(cfg, xs, ys, "float64", "binned")
    c, l = _oracle_pairs(oracle, cfg, xs, ys)
    _close(pairs, c, l, 1e-12)
    assert not bins.any()


def test_binned_pairs_repeat_bit_for_bit():
    cfg = _config("n328")
    n = int(cfg.no_xy)
    xs, ys = _tracks(n, 20000, seed=5)
    a, _, _ = _deposit(cfg, xs, ys, "float32", "binned")
    b, _, _ = _deposit(cfg, xs, ys, "float32", "binned")
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", ["run_fast_base", "run_fast_dense", "run_fast_dense_reflect_full", "run_aic144_dev"])
def test_whole_runs_with_the_binned_form_match_the_reference(name):
    solve = pkg().run_simulation_b200
    cfg, ref = run_config(name)
    res = solve(cfg, progress=False, shape={"deposit_variant": "binned"})
    np.testing.assert_array_equal(res.track_density_xy, ref["track_density_xy"])
    assert abs(res.ks - float(ref["ks"])) <= 1e-5
    assert res.recombination.sum() == pytest.approx(ref["recombination"].sum(), rel=1e-5)
    again = solve(cfg, progress=False, shape={"deposit_variant": "binned"})
    assert again.ks == res.ks
    np.testing.assert_array_equal(again.recombination, res.recombination)


def test_pic_deposit_refuses_the_binned_form():
    import torch

    _, E, N = _mods()
    cfg = _config("n24")
    g = E.make_grid(cfg, "float32", shape={"deposit_variant": "binned"})
    n = int(cfg.no_xy)
    dens = torch.zeros((n, 2 * ((n + 3) // 4 * 4)), dtype=torch.float32, device="cuda")
    counts = torch.zeros((n, n), dtype=torch.int32, device="cuda")
    xs = torch.full((1,), 5.0, dtype=torch.float64, device="cuda")
    lib = N.load()
    rc = lib.pic_deposit(ctypes.byref(g), ctypes.c_void_p(xs.data_ptr()), ctypes.c_void_p(xs.data_ptr()), 1,
                         ctypes.c_void_p(dens.data_ptr()), ctypes.c_void_p(counts.data_ptr()), 0)
    assert rc == N.PIC_E_INVALID and b"binned deposition needs the step workspace" in lib.pic_last_error()


# ------------------------------------------- segments: eight steps per launch


def _thin_config(grid):
    """The grid's lateral size with a 0.02 cm gap (46 k-planes), so that
    float64 segments of a 328 x 328 grid stay small and quick."""
    P, _, _ = _mods()
    um, r = GRIDS[grid]
    return P.SimulationConfig(**dict(BEAM, electrode_gap_cm=0.02, voltage_V=30.0, grid_size_um=um,
                                     sampled_radius_cm=r, seed=1, max_voxels=2e9))


def _segment_tracks(n, counts, seed):
    rng = np.random.default_rng(seed)
    m = int(sum(counts))
    off = np.zeros(len(counts) + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    return rng.uniform(0.0, n, m), rng.uniform(0.0, n, m), off


def _groups(counts, steps=8, tracks=65536, span=256):
    """Launch pairs of the segment loop: greedy groups of at most `steps`
    depositing steps, `tracks` tracks and `span` steps."""
    groups, s, n = 0, 0, len(counts)
    while s < n:
        e, nd, tr = s, 0, 0
        while e < n and e - s < span:
            if counts[e] > 0 and (nd == steps or tr + counts[e] > tracks):
                break
            nd += counts[e] > 0
            tr += counts[e]
            e += 1
        groups += nd > 0
        s = e
    return groups


def _run(cfg, xs, ys, off, dtype, variant, graphed=False):
    import torch

    _, E, N = _mods()
    lib = N.load()
    eng = E.ChamberEngine(cfg, dtype=dtype, max_tracks=len(xs), tally_steps=len(off) - 1,
                          shape={"deposit_variant": variant})
    try:
        eng.upload_tracks(xs, ys, non_blocking=False)
        torch.cuda.synchronize()
        l0 = lib.pic_kernel_launches()
        if graphed:
            eng.run_segment_graphed("all", off)
        else:
            eng.run_segment(off)
        torch.cuda.synchronize()
        launches = lib.pic_kernel_launches() - l0
        n = int(cfg.no_xy)
        pos, neg = eng.fields()
        dens = [d.view(n, -1, 2)[:, :n].cpu().numpy().astype(np.float64) for d in eng.dens]
        return dict(tally=eng.tallies(len(off) - 1).copy(), pos=pos, neg=neg, dens=dens,
                    counts=eng.counts.cpu().numpy().copy(), launches=launches)
    finally:
        eng.close()


# per-step track counts: depositing and idle steps mixed, a long idle stretch,
# steps that fill a launch's eight slots and one that crosses its track limit
SEGMENT = [300, 0, 0, 500, 20, 0, 1, 700, 700, 700, 700, 700, 700, 700, 700, 700, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
           0, 0, 40000, 30000, 5, 0, 9]


@pytest.mark.parametrize("dtype, tol", [("float64", 1e-12), ("float32", 1e-6)])
def test_a_segment_deposits_up_to_eight_steps_per_launch_pair(dtype, tol):
    cfg = _thin_config("n328")
    n = int(cfg.no_xy)
    xs, ys, off = _segment_tracks(n, SEGMENT, seed=3)
    a = _run(cfg, xs, ys, off, dtype, "binned")
    b = _run(cfg, xs, ys, off, dtype, "tracks")
    for k in range(4):
        np.testing.assert_allclose(a["tally"][:, k], b["tally"][:, k], rtol=0, atol=tol * np.abs(b["tally"][:, k]).max())
    peak = np.abs(b["pos"]).max()
    np.testing.assert_allclose(a["pos"], b["pos"], rtol=0, atol=tol * peak)
    np.testing.assert_allclose(a["neg"], b["neg"], rtol=0, atol=tol * peak)
    np.testing.assert_array_equal(a["counts"], b["counts"])
    # the caller's buffers: the last step's pairs, the other one zero
    last = (len(SEGMENT) - 1) & 1
    _close(a["dens"][last], b["dens"][last][..., 0], b["dens"][last][..., 1], tol)
    assert not a["dens"][last ^ 1].any() and not b["dens"][last ^ 1].any()
    steps = len(SEGMENT)
    assert a["launches"] == steps + 2 * _groups(SEGMENT)
    assert b["launches"] == steps + sum(c > 0 for c in SEGMENT)


def test_a_segment_with_a_step_beyond_the_launch_limit_deposits_step_by_step():
    """A step of more than 65536 tracks: the segment deposits one step at a
    time, that step in two pieces (the second adds to the first)."""
    cfg = _thin_config("n328")
    n = int(cfg.no_xy)
    counts = [100, 70000, 0, 50]
    xs, ys, off = _segment_tracks(n, counts, seed=4)
    a = _run(cfg, xs, ys, off, "float64", "binned")
    b = _run(cfg, xs, ys, off, "float64", "tracks")
    np.testing.assert_allclose(a["tally"], b["tally"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(a["pos"], b["pos"], rtol=0, atol=1e-12 * np.abs(b["pos"]).max())
    assert a["launches"] == len(counts) + 2 * (1 + 2 + 1)  # two launches a piece


def test_graph_replays_of_a_binned_segment_repeat_the_direct_run_bit_for_bit():
    cfg = _thin_config("n328")
    n = int(cfg.no_xy)
    xs, ys, off = _segment_tracks(n, SEGMENT, seed=5)
    a = _run(cfg, xs, ys, off, "float32", "binned")
    g = _run(cfg, xs, ys, off, "float32", "binned", graphed=True)
    np.testing.assert_array_equal(g["tally"], a["tally"])
    np.testing.assert_array_equal(g["pos"], a["pos"])
    assert g["launches"] == a["launches"]  # a replay counts the launches captured into it


@pytest.mark.parametrize("dtype, tol", [("float64", 1e-10), ("float32", 1e-5)])
def test_the_gradients_forward_pass_deposits_in_groups_into_its_kept_slots(dtype, tol):
    """pic_adjoint_forward with the binned form deposits up to eight steps
    per launch pair straight into the slots it keeps for the reverse sweep:
    k_s and the whole gradient equal the per-track form's."""
    A = importlib.import_module(pkg().__name__ + ".adjoint")
    cfg = _config("n24")
    ks_b, g_b, _ = A.ks_and_gradient(cfg, None, dtype=dtype, shape={"deposit_variant": "binned"})
    ks_t, g_t, _ = A.ks_and_gradient(cfg, None, dtype=dtype, shape={"deposit_variant": "tracks"})
    assert ks_b == pytest.approx(ks_t, rel=tol)
    np.testing.assert_allclose(g_b, g_t, rtol=tol, atol=0)
