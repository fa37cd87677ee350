"""Generate the golden fixtures under tests/golden/ from the reference solver.

Runs ONLY in a container that has the reference checkout (default
``/root/reference``, override with ``PIC_REFERENCE_ROOT``). The reference's
package imports numba and pandas, neither of which is installed there, so the
two test-only stand-ins in ``tests/golden/_stubs`` are put first on
``sys.path``: ``numba.njit`` becomes the identity and ``prange`` becomes
``range``, so the reference kernels execute as plain Python in exactly the same
float64 arithmetic and loop order (slow, but bit-for-bit the reference's
algorithm).

Every fixture records what the reference itself produced:

* ``config_<name>.json``   -- every derived scalar of ``SimulationConfig`` for a
  list of configurations (including the large ones that are never run here),
  the pulse schedule's checksum, and a checksum of the first pulse's sampled
  track centres (bit-exact sampler pin at full size).
* ``run_<name>.npz``       -- a whole ``run_simulation_numba`` run: f_t, k_s, the
  four per-step tallies, ``track_density_xy`` and, for small grids, the final
  carrier fields.
* ``step_<name>.npz``      -- one deposit of N tracks plus one Lax-Wendroff step
  through the reference kernels (``_insert_track_numba`` and
  ``_lax_wendroff_step_numba``), with the fields before and after.
* ``sampler.npz``          -- block sampler output for uneven batch sizes.

Usage::

    python tests/golden/make_golden.py               # everything (parallel)
    python tests/golden/make_golden.py --only run_fast_base
"""

from __future__ import annotations

import argparse
import hashlib
import json
import multiprocessing as mp
import os
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE_ROOT = os.environ.get("PIC_REFERENCE_ROOT", "/root/reference")


def _import_reference():
    sys.path.insert(0, str(HERE / "_stubs"))
    sys.path.insert(0, REFERENCE_ROOT)
    import pulsed_ion_chamber.config as config_mod  # noqa: F401

    return config_mod


# --------------------------------------------------------------------------
# Configurations. Keyword dictionaries for the reference SimulationConfig.
# --------------------------------------------------------------------------

FAST = dict(
    E_MeV_u=1.0,
    voltage_V=10.0,
    electrode_gap_cm=0.02,
    pulse_duration_s=1e-6,
    dose_rate_Gy_s=1e-8,
    grid_size_um=10.0,
    sampled_radius_cm=0.01,
    buffer_radius=5,
    no_z_electrode=4,
    seed=3,
)
# A denser variant of FAST: many tracks per step so the deposition path and
# the overlap of stencils are exercised, still tiny.
FAST_DENSE = dict(FAST, pulse_duration_s=6e-6, dose_rate_Gy_s=1.0, seed=5)

TWO_SPECIES = dict(
    mu_positive_cm2_Vs=1.36,
    mu_negative_cm2_Vs=2.10,
    D_positive_cm2_s=2.82e-2,
    D_negative_cm2_s=4.35e-2,
)

SMALL = dict(
    E_MeV_u=56.2,
    voltage_V=300.0,
    electrode_gap_cm=0.2,
    pulse_duration_s=2e-6,
    repetition_rate_hz=50.0,
    dose_rate_Gy_s=8.91,
    grid_size_um=40.0,
    sampled_radius_cm=0.004,
    buffer_radius=3,
    no_z_electrode=3,
    seed=11,
)
SMALL_RUN = dict(SMALL, pulse_duration_s=4e-6)

# The AIC-144 beam and chamber physics of the reference's example CLI.
AIC144 = dict(
    E_MeV_u=56.2,
    voltage_V=300.0,
    electrode_gap_cm=0.2,
    pulse_duration_s=540e-6,
    repetition_rate_hz=50.0,
    n_pulses=1,
    rf_frequency_hz=26.26e6,
    seed=20260527,
    dose_rate_Gy_s=10.0 * 0.891,
    W_eV=33.0,
    air_density_kg_m3=1.2041,
    lateral_boundary="reflecting",
    n_clearance_separation_times=2.6,
    track_cutoff_sigmas=10.0,
    **TWO_SPECIES,
)

# The plain-method beam of the benchmark workloads: protons at 56.2 MeV/u,
# 300 V over 0.2 cm, 540 us pulses at 50 Hz, 8.91 Gy/s to air.
BEAM = dict(
    E_MeV_u=56.2,
    voltage_V=300.0,
    electrode_gap_cm=0.2,
    pulse_duration_s=540e-6,
    repetition_rate_hz=50.0,
    dose_rate_Gy_s=8.91,
)

CONFIGS = {
    "fast": FAST,
    "fast_dense": FAST_DENSE,
    "small": SMALL,
    "small_run": SMALL_RUN,
    # 10 um voxels, r = 0.008 cm, seed 1: 24 x 24 x 206, 1622 steps.
    "column_10um_r008": dict(BEAM, grid_size_um=10.0, sampled_radius_cm=0.008, seed=1),
    # 5 um voxels, r = 0.05 cm: 208 x 208 x 406.
    "column_5um_r05_d8p91": dict(BEAM, grid_size_um=5.0, sampled_radius_cm=0.05, seed=1, max_voxels=2e9),
    "column_5um_r05_d89p1": dict(BEAM, grid_size_um=5.0, sampled_radius_cm=0.05, dose_rate_Gy_s=89.1, seed=1, max_voxels=2e9),
    # 10 um voxels, r = 0.02 cm: 48 x 48 x 206 (the adjoint chamber).
    "column_10um_r02": dict(BEAM, grid_size_um=10.0, sampled_radius_cm=0.02, seed=1),
    # Full electrode at 5 um, 10 pulses: 1068 x 1068 x 406.
    "full_electrode_5um_10p": dict(
        BEAM, grid_size_um=5.0, sampled_radius_cm=0.265, n_pulses=10, seed=1, max_voxels=2e9,
        memory_budget_fraction=None,
    ),
    # The reference's published 5 um full-electrode A100 run (AIC-144 kwargs).
    "aic144_full_electrode_5um": dict(
        AIC144, grid_size_um=5.0, sampled_radius_cm=0.265, buffer_radius=3, max_voxels=2e9,
        memory_budget_fraction=None,
    ),
    # The reference CLI's dev tier.
    "aic144_dev": dict(AIC144, grid_size_um=10.0, sampled_radius_cm=0.003, buffer_radius=3),
    "aic144_archive": dict(AIC144, grid_size_um=10.0, sampled_radius_cm=0.008, buffer_radius=3),
}

# Extremes of the batched saturation sweep (10/5 um, radii 0.008-0.03 cm,
# gaps 0.1-0.3 cm, 25-400 V, 100-1000 us), pinned for the config mirror.
for _name, _kw in {
    "sweep_lo": dict(E_MeV_u=56.2, voltage_V=25.0, electrode_gap_cm=0.1, pulse_duration_s=100e-6,
                     repetition_rate_hz=50.0, dose_rate_Gy_s=1.0, grid_size_um=10.0, sampled_radius_cm=0.008, seed=1),
    "sweep_hi": dict(E_MeV_u=56.2, voltage_V=400.0, electrode_gap_cm=0.3, pulse_duration_s=1000e-6,
                     repetition_rate_hz=50.0, dose_rate_Gy_s=100.0, grid_size_um=5.0, sampled_radius_cm=0.03,
                     seed=64, max_voxels=2e9),
    "fast_two_species": dict(FAST, **TWO_SPECIES),
    "fast_nocutoff": dict(FAST, track_cutoff_sigmas=None),
    "fast_fill07": dict(FAST_DENSE, chamber_fill_fraction=0.7),
    "rf_odd_noxy": dict(E_MeV_u=56.2, voltage_V=150.0, electrode_gap_cm=0.15, pulse_duration_s=50e-6,
                        dose_rate_Gy_s=3.0, grid_size_um=10.0, sampled_radius_cm=0.0085, buffer_radius=4,
                        dt_seconds=2.0e-7, seed=9),
}.items():
    CONFIGS[_name] = _kw

DERIVED = [
    "unit_length_cm", "LET_keV_um", "track_radius_cm", "Efield_V_cm", "area_cm2",
    "mu_positive", "mu_negative", "D_positive", "D_negative", "two_carrier_species",
    "no_xy", "no_z", "no_z_with_buffer", "effective_gap_cm", "outer_radius", "mid_xy",
    "inner_radius", "inner_radius_sq", "sampling_radius", "sampling_radius_sq",
    "scoring_radius_sq", "von_neumann_dt", "dt", "courant_number",
    "slowest_mobility_cm2_Vs", "separation_time_steps", "clearance_time_steps",
    "pulse_time_steps", "pulse_period_steps", "total_time_steps", "N0",
    "Gaussian_factor", "track_sigma_cm", "track_cutoff_cm", "track_cutoff_voxels",
    "truncated_charge_fraction", "number_of_tracks_per_pulse",
]


def _sha(arr) -> str:
    import numpy as np

    return hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()


def _make_config(name):
    config_mod = _import_reference()
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return config_mod.SimulationConfig(**CONFIGS[name])


def job_config(name):
    """Derived scalars, schedule checksum and first-pulse sampler checksum."""
    import numpy as np

    _import_reference()
    from pulsed_ion_chamber.pulses import CylinderSampler, build_track_schedule

    cfg = _make_config(name)
    out = {"name": name, "kwargs": CONFIGS[name]}
    for key in DERIVED:
        v = getattr(cfg, key)
        out[key] = bool(v) if isinstance(v, (bool, np.bool_)) else (int(v) if isinstance(v, (int, np.integer)) else float(v))
    out["scheme_coefficients"] = [list(map(float, w)) for w in cfg.scheme_coefficients()]
    out["pulse_time_bins_len"] = int(len(cfg.pulse_time_bins))
    out["pulse_time_bins_sha256"] = _sha(cfg.pulse_time_bins)
    rng = np.random.default_rng(cfg.seed)
    schedule = build_track_schedule(cfg, rng)
    out["schedule_sha256"] = _sha(schedule.astype(np.int64))
    out["schedule_sum"] = int(schedule.sum())
    out["schedule_max"] = int(schedule.max())
    out["schedule_nonzero_steps"] = int((schedule > 0).sum())
    sampler = CylinderSampler(rng, cfg.mid_xy, cfg.sampling_radius, cfg.no_xy)
    n_first = int(schedule[: cfg.pulse_time_steps].sum())
    # Sample the first pulse in the per-step batches the solvers use.
    xs_parts, ys_parts = [], []
    for step in range(cfg.pulse_time_steps):
        xs, ys = sampler.sample(int(schedule[step]))
        xs_parts.append(xs)
        ys_parts.append(ys)
    xs = np.concatenate(xs_parts)
    ys = np.concatenate(ys_parts)
    assert len(xs) == n_first
    out["first_pulse_tracks"] = n_first
    out["first_pulse_xs_sha256"] = _sha(xs)
    out["first_pulse_ys_sha256"] = _sha(ys)
    out["first_pulse_xs_head"] = [float(v) for v in xs[:8]]
    out["first_pulse_ys_head"] = [float(v) for v in ys[:8]]
    (HERE / f"config_{name}.json").write_text(json.dumps(out, indent=1, sort_keys=True))
    return name


RUNS = {
    # name: (config name, overrides, store fields?)
    "run_fast_base": ("fast", {}, True),
    "run_fast_reflecting": ("fast", {"lateral_boundary": "reflecting"}, True),
    "run_fast_full_grid": ("fast", {"scoring_region": "full_grid"}, True),
    "run_fast_two_species": ("fast", TWO_SPECIES, True),
    "run_fast_nocutoff": ("fast", {"track_cutoff_sigmas": None}, False),
    "run_fast_dense": ("fast_dense", {}, True),
    "run_fast_dense_reflect_full": (
        "fast_dense",
        dict(lateral_boundary="reflecting", scoring_region="full_grid", chamber_fill_fraction=0.7, **TWO_SPECIES),
        True,
    ),
    "run_small_absorbing": ("small_run", {}, True),
    "run_small_reflecting": ("small_run", {"lateral_boundary": "reflecting"}, True),
    "run_aic144_dev": ("aic144_dev", {}, False),
    "run_column_10um_r008": ("column_10um_r008", {}, False),
}


def job_run(name):
    import numpy as np

    config_mod = _import_reference()
    from pulsed_ion_chamber.solver_numba import run_simulation_numba

    cfg_name, overrides, fields = RUNS[name]
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        cfg = config_mod.SimulationConfig(**dict(CONFIGS[cfg_name], **overrides))
    t0 = time.time()
    res = run_simulation_numba(cfg, progress=False)
    wall = time.time() - t0
    payload = dict(
        f_t=res.f_t,
        ks=np.float64(res.ks),
        time_s=res.time_s,
        injected=res.injected_positive,
        recombination=res.recombination,
        n_positive=res.n_positive,
        n_negative=res.n_negative,
        track_density_xy=res.track_density_xy,
        positive_sum=np.float64(res.positive_array.sum()),
        negative_sum=np.float64(res.negative_array.sum()),
        positive_max=np.float64(np.abs(res.positive_array).max()),
        wall_s=np.float64(wall),
    )
    if fields:
        payload["positive_array"] = res.positive_array
        payload["negative_array"] = res.negative_array
    meta = dict(config=cfg_name, overrides={k: v for k, v in overrides.items()})
    payload["meta_json"] = np.array(json.dumps(meta))
    np.savez_compressed(HERE / f"{name}.npz", **payload)
    return name


STEPS = {
    # name: (config, overrides, n_tracks)
    "step_small_track_disc": ("small", {}, 30),
    "step_small_full_grid": ("small", {"scoring_region": "full_grid"}, 30),
    "step_small_two_species": ("small", TWO_SPECIES, 30),
}


def job_step(name):
    """One deposit of N tracks plus one sweep, through the reference kernels."""
    import numpy as np

    config_mod = _import_reference()
    from pulsed_ion_chamber.constants import RECOMBINATION_ALPHA_CM3_S
    from pulsed_ion_chamber.pulses import CylinderSampler
    from pulsed_ion_chamber.solver_numba import _insert_track_numba, _lax_wendroff_step_numba
    from pulsed_ion_chamber.solver_numba_parallel import (
        _accumulate_track_density_numba_parallel,
        _build_row_index,
        _precompute_track_gaussians,
    )

    cfg_name, overrides, n_tracks = STEPS[name]
    cfg = config_mod.SimulationConfig(**dict(CONFIGS[cfg_name], **overrides))
    rng = np.random.default_rng(cfg.seed)
    sampler = CylinderSampler(rng, cfg.mid_xy, cfg.sampling_radius, cfg.no_xy)
    xs, ys = sampler.sample(n_tracks)
    shape = (cfg.no_xy, cfg.no_xy, cfg.no_z_with_buffer)
    pos = np.zeros(shape)
    neg = np.zeros(shape)
    pos_next = np.zeros(shape)
    neg_next = np.zeros(shape)
    h2 = cfg.unit_length_cm**2
    b2 = cfg.track_radius_cm**2
    inserted = 0.0
    for x, y in zip(xs, ys):
        inserted += _insert_track_numba(
            pos, neg, x, y, cfg.no_xy, cfg.no_z, cfg.no_z_electrode, h2, b2,
            cfg.Gaussian_factor, cfg.mid_xy, cfg.scoring_radius_sq, cfg.track_cutoff_voxels,
        )
    # The batched 2D density of the same tracks (dimensionless, before G).
    gi, gj, lo_i, hi_i, lo_j, hi_j = _precompute_track_gaussians(xs, ys, cfg.no_xy, h2, b2, cfg.track_cutoff_voxels)
    offsets, ids = _build_row_index(lo_i, hi_i, cfg.no_xy)
    total_density = np.zeros((cfg.no_xy, cfg.no_xy))
    _accumulate_track_density_numba_parallel(total_density, gi, gj, lo_i, lo_j, hi_j, offsets, ids, cfg.no_xy)
    (p_lat, p_zm, p_zp, p_cen), (n_lat, n_zm, n_zp, n_cen) = cfg.scheme_coefficients()
    alpha_dt = RECOMBINATION_ALPHA_CM3_S * cfg.dt
    rec, tp, tn = _lax_wendroff_step_numba(
        pos, neg, pos_next, neg_next, cfg.no_xy, cfg.no_z_with_buffer, cfg.no_z_electrode, cfg.no_z,
        cfg.mid_xy, cfg.scoring_radius_sq, p_lat, p_zm, p_zp, p_cen, n_lat, n_zm, n_zp, n_cen, alpha_dt,
    )
    np.savez_compressed(
        HERE / f"{name}.npz",
        xs=xs, ys=ys, total_density=total_density,
        positive=pos, negative=neg, positive_next=pos_next, negative_next=neg_next,
        inserted=np.float64(inserted), recombined=np.float64(rec),
        total_positive=np.float64(tp), total_negative=np.float64(tn), alpha_dt=np.float64(alpha_dt),
        meta_json=np.array(json.dumps(dict(config=cfg_name, overrides=overrides, n_tracks=n_tracks))),
    )
    return name


def job_sampler(name):
    import numpy as np

    _import_reference()
    from pulsed_ion_chamber.pulses import CylinderSampler, sample_xy_inside_cylinder

    mid_xy, radius, no_xy = 30, 24.0, 60
    batches = [7, 1, 5000, 3, 900]
    ref = np.random.default_rng(11)
    expected = np.array([sample_xy_inside_cylinder(ref, mid_xy, radius, no_xy) for _ in range(sum(batches))])
    sampler = CylinderSampler(np.random.default_rng(11), mid_xy, radius, no_xy)
    got = np.vstack([np.column_stack(sampler.sample(n)) for n in batches])
    assert np.array_equal(got, expected)
    # An odd grid with a float centre, as config.py produces (mid_xy = no_xy/2).
    s2 = CylinderSampler(np.random.default_rng(4), 12.5, 9.5, 25)
    got2 = np.vstack([np.column_stack(s2.sample(n)) for n in [0, 5, 4096, 1, 0, 17]])
    np.savez_compressed(HERE / "sampler.npz", xy=expected, batches=np.array(batches), xy_odd=got2)
    return name


def _dispatch(job):
    kind, name = job
    t0 = time.time()
    {"config": job_config, "run": job_run, "step": job_step, "sampler": job_sampler}[kind](name)
    return f"{kind}:{name} {time.time() - t0:.1f}s"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*", default=None, help="job names (e.g. run_fast_base config_small)")
    ap.add_argument("--jobs", type=int, default=os.cpu_count())
    args = ap.parse_args()
    jobs = [("sampler", "sampler")]
    jobs += [("config", n) for n in CONFIGS]
    jobs += [("step", n) for n in STEPS]
    # longest first
    jobs += [("run", n) for n in sorted(RUNS, key=lambda n: "column" not in n and "aic" not in n)]
    if args.only:
        wanted = set(args.only)
        jobs = [j for j in jobs if j[1] in wanted or f"{j[0]}_{j[1]}" in wanted]
    ctx = mp.get_context("spawn")
    with ctx.Pool(args.jobs) as pool:
        for line in pool.imap_unordered(_dispatch, jobs):
            print(line, flush=True)


if __name__ == "__main__":
    main()
