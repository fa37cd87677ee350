"""Run configuration: the physical inputs and every scalar derived from them.

:class:`SimulationConfig` takes the same keyword fields as the reference's
``pulsed_ion_chamber.config.SimulationConfig`` (pulsed_ion_chamber/config.py:73-178)
and derives the same attributes (config.py:180-401) with the same float64
arithmetic, so that a run configured here and a run configured there drive the
kernels with bit-identical scalars. The solver never needs this class: any
object exposing those attributes works, including the reference's own config,
which is how :func:`run_simulation_b200` drops in beside ``run_simulation_numba``.

Two things differ on purpose:

* The stopping-power lookup (the reference interpolates a PSTAR table with
  pandas, pulsed_ion_chamber/stopping_power.py:18-28, and fits the track radius
  to a second table, :31-42) is host-side set-up outside the hot path. Here the
  LET and track radius are inputs: pass ``LET_keV_um`` and ``track_radius_cm``,
  or rely on :data:`STOPPING_POWER_PRESETS`, which holds the values the
  reference's tables give at the energies this project's workloads use.
* The host-RAM guard (config.py:403-436) is replaced by a device-memory check
  in the solver, because the fields live in HBM, not host RAM.

Every formula that must agree bit-for-bit with the reference is written in the
same operation order: float64 rounding depends on it.
"""

from __future__ import annotations

import warnings
from dataclasses import dataclass
from math import exp, pi, sqrt
from typing import Optional

import numpy as np

from .constants import (
    AIR_DENSITY_KG_M3,
    ION_DIFFUSION_CM2_S,
    ION_MOBILITY_CM2_VS,
    JOULE_TO_KEV,
    W_EV_PER_ION_PAIR,
)

LATERAL_BOUNDARIES = ("absorbing", "reflecting")
SCORING_REGIONS = ("track_disc", "full_grid")

# (particle, E in MeV/u) -> (LET in keV/um, Gaussian track radius b in cm),
# as pulsed_ion_chamber/stopping_power.py:18-42 evaluates them (PSTAR dry-air
# interpolation; Rossomme radius fit with its 20 um floor).
STOPPING_POWER_PRESETS = {
    ("proton", 56.2): (0.0011994843758452705, 0.002),
    ("proton", 1.0): (0.026711210613162315, 0.0030303350614661892),
}


def von_neumann_dt(ion_diff, grid_spacing_cm, ion_mobility, Efield_V_cm) -> float:
    """Largest dt on the 1/1.01 geometric ladder from 1 s at which
    ``6 s + c**2 <= 1`` for every species (s = D dt/h^2, c = mu E dt/h).

    Mirrors pulsed_ion_chamber/config.py:43-70: the same descending ladder and
    the same arithmetic, so the returned float is bit-identical.
    """
    diffs = np.atleast_1d(np.asarray(ion_diff, dtype=np.float64))
    mobilities = np.atleast_1d(np.asarray(ion_mobility, dtype=np.float64))
    if diffs.shape != mobilities.shape:
        raise ValueError(
            f"{len(diffs)} diffusion coefficients against {len(mobilities)} mobilities: "
            "ion_diff and ion_mobility need one entry per carrier species each."
        )
    h2 = grid_spacing_cm**2
    dt = 1.0
    while True:
        dt /= 1.01
        s = diffs * dt / h2
        c = mobilities * Efield_V_cm * dt / grid_spacing_cm
        if bool(np.all(6 * s + c**2 <= 1)):
            return dt


def lax_wendroff_weights(diffusion, mobility, Efield_V_cm, dt, unit_length_cm):
    """``(lateral, z_minus, z_plus, centre)`` Lax-Wendroff weights of one
    species (pulsed_ion_chamber/config.py:477-480):

    lateral = s, z_minus = s + c(c+1)/2, z_plus = s + c(c-1)/2,
    centre = 1 - c^2 - 6 s, with s = D dt/h^2 and c = mu E dt/h.
    """
    s = diffusion * dt / unit_length_cm**2
    c = mobility * Efield_V_cm * dt / unit_length_cm
    return (s, s + c * (c + 1.0) / 2.0, s + c * (c - 1.0) / 2.0, 1.0 - c * c - 6.0 * s)


@dataclass
class SimulationConfig:
    # beam / chamber
    E_MeV_u: float = 150.0
    particle: str = "proton"
    voltage_V: float = 200.0
    electrode_gap_cm: float = 0.2
    # pulse train
    pulse_duration_s: float = 540e-6
    repetition_rate_hz: float = 50.0
    dose_rate_Gy_s: float = 60.0
    n_pulses: int = 1
    n_clearance_separation_times: float = 2.0
    rf_frequency_hz: Optional[float] = None
    # grid
    grid_size_um: float = 40.0
    sampled_radius_cm: float = 0.002
    buffer_radius: int = 4
    no_z_electrode: int = 3
    max_voxels: float = 1e8
    memory_budget_fraction: Optional[float] = 0.8  # accepted for signature parity
    # carriers (None = the averaged pair)
    mu_positive_cm2_Vs: Optional[float] = None
    mu_negative_cm2_Vs: Optional[float] = None
    D_positive_cm2_s: Optional[float] = None
    D_negative_cm2_s: Optional[float] = None
    W_eV: float = W_EV_PER_ION_PAIR
    air_density_kg_m3: float = AIR_DENSITY_KG_M3
    chamber_fill_fraction: float = 1.0
    lateral_boundary: str = "absorbing"
    scoring_region: str = "track_disc"
    track_cutoff_sigmas: Optional[float] = 10.0
    dt_seconds: Optional[float] = None
    seed: Optional[int] = None
    # stopping power inputs (None = STOPPING_POWER_PRESETS)
    LET_keV_um: Optional[float] = None
    track_radius_cm: Optional[float] = None

    def __post_init__(self):
        self.unit_length_cm = self.grid_size_um * 1e-4
        self._resolve_stopping_power()
        self.Efield_V_cm = self.voltage_V / self.electrode_gap_cm
        self.area_cm2 = pi * self.sampled_radius_cm**2
        self._resolve_carriers()

        if self.lateral_boundary not in LATERAL_BOUNDARIES:
            raise ValueError(
                f"unknown lateral_boundary {self.lateral_boundary!r} (known: {', '.join(LATERAL_BOUNDARIES)})."
            )
        if self.scoring_region not in SCORING_REGIONS:
            raise ValueError(f"unknown scoring_region {self.scoring_region!r} (known: {', '.join(SCORING_REGIONS)}).")
        if isinstance(self.chamber_fill_fraction, bool) or not 0 < self.chamber_fill_fraction <= 1:
            raise ValueError(
                f"chamber_fill_fraction={self.chamber_fill_fraction!r} lies outside (0, 1]."
            )

        # grid: rounded, not truncated (config.py:210-212)
        self.no_xy = int(round(2 * self.sampled_radius_cm / self.unit_length_cm)) + 2 * self.buffer_radius
        self.no_z = int(round(self.electrode_gap_cm / self.unit_length_cm))
        self.no_z_with_buffer = 2 * self.no_z_electrode + self.no_z
        self.effective_gap_cm = self.no_z * self.unit_length_cm
        mismatch = abs(self.effective_gap_cm - self.electrode_gap_cm)
        self._gap_mismatch_relative = mismatch / self.electrode_gap_cm if self.electrode_gap_cm > 0 else 0.0
        if self._gap_mismatch_relative > 1e-3:
            warnings.warn(
                f"electrode_gap_cm={self.electrode_gap_cm:.6g} cm is not an integer multiple of "
                f"grid_size_um={self.grid_size_um:.4g} um: the simulated gap is no_z={self.no_z} voxels "
                f"= {self.effective_gap_cm:.6g} cm.",
                stacklevel=2,
            )
        if self.no_xy * self.no_xy * self.no_z > self.max_voxels:
            raise ValueError(
                f"{self.no_xy}x{self.no_xy}x{self.no_z} = {self.no_xy * self.no_xy * self.no_z:.3g} voxels "
                f"exceeds max_voxels={self.max_voxels:.3g}: use a coarser grid_size_um or a smaller "
                "sampled_radius_cm."
            )
        # continuous grid centre, a float for odd no_xy too (config.py:254-255)
        self.outer_radius = self.no_xy / 2.0
        self.mid_xy = self.outer_radius
        self.inner_radius = self.outer_radius - self.buffer_radius
        if self.inner_radius <= 0:
            raise ValueError(
                f"no sampling region left: inner_radius {self.inner_radius:.3g} is not positive "
                f"(no_xy {self.no_xy} against buffer_radius {self.buffer_radius})."
            )
        self.inner_radius_sq = self.inner_radius**2
        self.sampling_radius = self.inner_radius * self.chamber_fill_fraction
        self.sampling_radius_sq = self.sampling_radius**2
        self.scoring_radius_sq = (
            self.inner_radius_sq if self.scoring_region == "track_disc" else 2.0 * self.no_xy**2
        )

        # time step (config.py:287-307)
        self.von_neumann_dt = von_neumann_dt(
            (self.D_positive, self.D_negative),
            self.unit_length_cm,
            (self.mu_positive, self.mu_negative),
            self.Efield_V_cm,
        )
        if self.dt_seconds is None:
            self.dt = self.von_neumann_dt
        elif self.dt_seconds > self.von_neumann_dt:
            raise ValueError(
                f"unstable time step: dt_seconds {self.dt_seconds:.4g} s is above the von Neumann "
                f"bound {self.von_neumann_dt:.4g} s of this grid spacing and field."
            )
        else:
            self.dt = float(self.dt_seconds)
        self.courant_number = (
            max(self.mu_positive, self.mu_negative) * self.Efield_V_cm * self.dt / self.unit_length_cm
        )
        self.rf_cycles_per_time_step = self.dt * self.rf_frequency_hz if self.rf_frequency_hz else None
        if self.rf_cycles_per_time_step is not None and self.rf_cycles_per_time_step < 1.0:
            warnings.warn(
                f"dt ({self.dt:.3g} s) is shorter than one RF period (1/{self.rf_frequency_hz:.4g} Hz).",
                stacklevel=2,
            )

        # pulse timing (config.py:340-361)
        self.slowest_mobility_cm2_Vs = min(self.mu_positive, self.mu_negative)
        self.separation_time_steps = int(
            self.electrode_gap_cm / (2.0 * self.slowest_mobility_cm2_Vs * self.Efield_V_cm * self.dt)
        )
        self.clearance_time_steps = int(round(self.n_clearance_separation_times * self.separation_time_steps))
        self.pulse_time_bins = np.arange(0.0, self.pulse_duration_s + self.dt, self.dt)
        self.pulse_time_steps = len(self.pulse_time_bins) - 1
        self.pulse_period_steps = (
            int(round(1.0 / self.repetition_rate_hz / self.dt))
            if self.repetition_rate_hz > 0
            else self.pulse_time_steps
        )
        if self.n_pulses > 1 and self.pulse_period_steps < self.pulse_time_steps:
            raise ValueError(
                f"overlapping pulses: a pulse lasts {self.pulse_time_steps} steps but they start "
                f"every {self.pulse_period_steps} steps at this dt."
            )
        self.total_time_steps = (
            (self.n_pulses - 1) * self.pulse_period_steps + self.pulse_time_steps + self.clearance_time_steps
        )

        # Gaussian track (config.py:364-386)
        LET_eV_cm = self.LET_keV_um * 1e7
        self.N0 = LET_eV_cm / self.W_eV
        self.Gaussian_factor = self.N0 / (pi * self.track_radius_cm**2)
        self.track_sigma_cm = self.track_radius_cm / sqrt(2.0)
        if self.track_cutoff_sigmas is None:
            self.track_cutoff_voxels = float(self.no_xy)
            self.track_cutoff_cm = self.track_cutoff_voxels * self.unit_length_cm
            self.truncated_charge_fraction = 0.0
        else:
            if self.track_cutoff_sigmas <= 0:
                raise ValueError(
                    f"track_cutoff_sigmas={self.track_cutoff_sigmas!r}: give a positive number of "
                    "sigmas, or None to keep the whole Gaussian."
                )
            self.track_cutoff_cm = self.track_cutoff_sigmas * self.track_sigma_cm
            self.track_cutoff_voxels = self.track_cutoff_cm / self.unit_length_cm
            self.truncated_charge_fraction = exp(-((self.track_cutoff_cm / self.track_radius_cm) ** 2))

        # tracks per pulse from the mean dose rate (config.py:389-399,
        # stopping_power.py:45-56)
        dose_per_pulse_Gy = self.dose_rate_Gy_s / self.repetition_rate_hz
        inst_dose_rate = dose_per_pulse_Gy / self.pulse_duration_s
        LET_keV_cm = self.LET_keV_um * 1e4
        density_kg_cm3 = self.air_density_kg_m3 * 1e-6
        fluence_rate = inst_dose_rate * JOULE_TO_KEV * density_kg_cm3 / LET_keV_cm
        self.number_of_tracks_per_pulse = max(
            1, int(round(fluence_rate * self.pulse_duration_s * self.area_cm2))
        )

        voxels = self.no_xy**2 * self.no_z_with_buffer
        self.carrier_array_bytes = 4 * voxels * 8
        self.track_schedule_bytes = 2 * self.number_of_tracks_per_pulse * 8
        self.scratch_bytes = self.no_xy**2 * 8
        self.estimated_memory_bytes = max(self.track_schedule_bytes, self.carrier_array_bytes + self.scratch_bytes)

    def _resolve_stopping_power(self):
        if self.LET_keV_um is None or self.track_radius_cm is None:
            key = (self.particle, float(self.E_MeV_u))
            if key not in STOPPING_POWER_PRESETS:
                raise ValueError(
                    f"No stopping-power preset for {self.particle} at {self.E_MeV_u} MeV/u: pass "
                    "LET_keV_um= and track_radius_cm= (the values pulsed_ion_chamber.stopping_power "
                    "gives), or pass the reference's own SimulationConfig to the solver."
                )
            let, b = STOPPING_POWER_PRESETS[key]
            if self.LET_keV_um is None:
                self.LET_keV_um = let
            if self.track_radius_cm is None:
                self.track_radius_cm = b

    def _resolve_carriers(self):
        self.mu_positive = ION_MOBILITY_CM2_VS if self.mu_positive_cm2_Vs is None else self.mu_positive_cm2_Vs
        self.mu_negative = ION_MOBILITY_CM2_VS if self.mu_negative_cm2_Vs is None else self.mu_negative_cm2_Vs
        self.D_positive = ION_DIFFUSION_CM2_S if self.D_positive_cm2_s is None else self.D_positive_cm2_s
        self.D_negative = ION_DIFFUSION_CM2_S if self.D_negative_cm2_s is None else self.D_negative_cm2_s
        for name, value in (
            ("mu_positive_cm2_Vs", self.mu_positive),
            ("mu_negative_cm2_Vs", self.mu_negative),
            ("D_positive_cm2_s", self.D_positive),
            ("D_negative_cm2_s", self.D_negative),
        ):
            if value <= 0:
                raise ValueError(f"{name}={value!r}: expected a magnitude above zero (drift directions "
                                 "follow from the field and the carrier, not from this sign).")
        self.two_carrier_species = not (
            self.mu_positive == self.mu_negative and self.D_positive == self.D_negative
        )

    def scheme_coefficients(self):
        """``((lat, zm, zp, cen) positive, (lat, zm, zp, cen) negative)``;
        the negative species applies its weights to swapped z-neighbours."""
        return (
            lax_wendroff_weights(self.D_positive, self.mu_positive, self.Efield_V_cm, self.dt, self.unit_length_cm),
            lax_wendroff_weights(self.D_negative, self.mu_negative, self.Efield_V_cm, self.dt, self.unit_length_cm),
        )

    def summary(self) -> str:
        return (
            f"Grid {self.no_xy} x {self.no_xy} x {self.no_z_with_buffer} voxels "
            f"({self.unit_length_cm * 1e4:.3g} um), dt {self.dt * 1e9:.2f} ns, "
            f"{self.total_time_steps} steps, {self.number_of_tracks_per_pulse} tracks/pulse, "
            f"{self.n_pulses} pulse(s), wall {self.lateral_boundary}, scoring {self.scoring_region}"
        )
