"""GB300-native backend for the pulsed-proton ion-chamber recombination solver.

The hot path of grzanka/IonTracks-PulsedProton-Python -- the per-step
Lax-Wendroff drift-diffusion-recombination sweep and the Gaussian ion-track
deposition -- as hand-written sm_103a CUDA behind a C ABI
(``csrc/``, ``include/pic_gb300.h``), driven from Python through ctypes.

``run_simulation_b200(config)`` takes the same configuration object and
returns the same ``Result`` as the reference's ``run_simulation_numba``
(pulsed_ion_chamber/solver_numba.py:237), so it drops in beside it.
"""

from .config import SimulationConfig, STOPPING_POWER_PRESETS
from .constants import RECOMBINATION_ALPHA_CM3_S
from .pulses import CylinderSampler, TrackSampler, build_track_schedule
from .state import Diagnostics, Result

__all__ = [
    "SimulationConfig",
    "STOPPING_POWER_PRESETS",
    "RECOMBINATION_ALPHA_CM3_S",
    "Result",
    "Diagnostics",
    "TrackSampler",
    "CylinderSampler",
    "build_track_schedule",
    "run_simulation_b200",
    "run_batched_b200",
    "saturation_sweep_configs",
    "ks_b200",
    "ks_and_gradient",
    "fit_alpha",
    "fit_parameters",
    "AdjointRun",
]


def __getattr__(name):
    # The solver pulls in torch and the CUDA library; import it on first use so
    # the host-side pieces (config, pulses, state) stay importable without them.
    if name == "run_simulation_b200":
        from .solver_b200 import run_simulation_b200

        return run_simulation_b200
    if name in ("run_batched_b200", "saturation_sweep_configs"):
        from . import batched

        return getattr(batched, name)
    if name in ("ks_b200", "ks_and_gradient", "fit_alpha", "fit_parameters", "AdjointRun"):
        from . import adjoint

        return getattr(adjoint, name)
    raise AttributeError(name)
