"""The package's SimulationConfig derives every scalar the kernels consume
bit-identically to the reference's SimulationConfig (pulsed_ion_chamber/config.py:180-401).

The expected values are the reference's own, recorded by
tests/golden/make_golden.py for small and full-size configurations alike."""

import math

import numpy as np
import pytest

from goldens import GOLDEN, config_json, make_config, pkg

NAMES = sorted(p.stem[len("config_"):] for p in GOLDEN.glob("config_*.json"))
SCALARS = [
    "unit_length_cm", "Efield_V_cm", "area_cm2", "mu_positive", "mu_negative", "D_positive", "D_negative",
    "two_carrier_species", "no_xy", "no_z", "no_z_with_buffer", "effective_gap_cm", "outer_radius", "mid_xy",
    "inner_radius", "inner_radius_sq", "sampling_radius", "sampling_radius_sq", "scoring_radius_sq",
    "von_neumann_dt", "dt", "courant_number", "slowest_mobility_cm2_Vs", "separation_time_steps",
    "clearance_time_steps", "pulse_time_steps", "pulse_period_steps", "total_time_steps", "N0",
    "Gaussian_factor", "track_sigma_cm", "track_cutoff_cm", "track_cutoff_voxels", "truncated_charge_fraction",
    "number_of_tracks_per_pulse",
]


def test_fixtures_present():
    assert len(NAMES) >= 10


@pytest.mark.parametrize("name", NAMES)
def test_derived_scalars_are_bit_identical(name):
    ref = config_json(name)
    cfg = make_config(name)
    for key in SCALARS:
        got = getattr(cfg, key)
        want = ref[key]
        if isinstance(want, float) and math.isnan(want):
            assert math.isnan(got), key
        else:
            assert got == want, f"{key}: {got!r} != {want!r}"
    assert [list(w) for w in cfg.scheme_coefficients()] == ref["scheme_coefficients"]
    assert len(cfg.pulse_time_bins) == ref["pulse_time_bins_len"]


@pytest.mark.parametrize("name", ["small", "aic144_dev", "column_10um_r008"])
def test_presets_reproduce_the_reference_stopping_power(name):
    """Without explicit LET/radius the 56.2 MeV/u preset is used; it must be
    the reference table's value."""
    ref = config_json(name)
    kw = dict(ref["kwargs"])
    cfg = pkg().SimulationConfig(**kw)
    assert cfg.LET_keV_um == ref["LET_keV_um"]
    assert cfg.track_radius_cm == ref["track_radius_cm"]
    assert cfg.number_of_tracks_per_pulse == ref["number_of_tracks_per_pulse"]


def test_unknown_energy_without_stopping_power_raises():
    with pytest.raises(ValueError, match="stopping-power preset"):
        pkg().SimulationConfig(E_MeV_u=123.0)


@pytest.mark.parametrize(
    "kwargs, match",
    [
        (dict(lateral_boundary="open"), "lateral_boundary"),
        (dict(scoring_region="everywhere"), "scoring_region"),
        (dict(chamber_fill_fraction=0.0), "chamber_fill_fraction"),
        (dict(grid_size_um=100.0, sampled_radius_cm=0.001, buffer_radius=2, no_z_electrode=2), "inner_radius"),
        (dict(grid_size_um=0.1, sampled_radius_cm=1.0, electrode_gap_cm=1.0), "exceeds max_voxels"),
        (dict(pulse_duration_s=1e-2, repetition_rate_hz=1000.0, n_pulses=2), "overlapping pulses"),
        (dict(dt_seconds=1.0), "von Neumann"),
        (dict(track_cutoff_sigmas=-1.0), "track_cutoff_sigmas"),
        (dict(mu_positive_cm2_Vs=-1.36), "magnitude above zero"),
    ],
)
def test_degenerate_configs_raise_like_the_reference(kwargs, match):
    base = dict(E_MeV_u=56.2, seed=0)
    base.update(kwargs)
    with pytest.raises(ValueError, match=match):
        pkg().SimulationConfig(**base)


def test_odd_grid_keeps_a_float_centre():
    cfg = make_config("rf_odd_noxy")
    assert cfg.no_xy % 2 == 1
    assert cfg.mid_xy == cfg.no_xy / 2.0
