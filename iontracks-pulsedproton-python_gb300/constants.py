"""Physical constants of ion transport in air.

The values are the published Kanai et al. (1998) carrier constants and the
recombination coefficient the reference solver uses
(pulsed_ion_chamber/constants.py:11-35). They are inputs to the physics, so
they must be the same numbers for results to agree.

``RECOMBINATION_ALPHA_CM3_S`` is read by :func:`recombination_alpha` at call
time, only as a default: pass ``alpha_cm3_s=`` to override it per run, which
is how the adjoint and the alpha fit perturb it.
"""

import sys

W_EV_PER_ION_PAIR = 34.2  # eV per ion pair in air, protons
ION_MOBILITY_CM2_VS = 1.65  # averaged carrier mobility, cm^2/(V s)
ION_DIFFUSION_CM2_S = 3.7e-2  # averaged carrier diffusion, cm^2/s
RECOMBINATION_ALPHA_CM3_S = 1.60e-6  # volume recombination coefficient, cm^3/s

ION_MOBILITY_POSITIVE_CM2_VS = 1.36
ION_MOBILITY_NEGATIVE_CM2_VS = 2.10
ION_DIFFUSION_POSITIVE_CM2_S = 2.82e-2
ION_DIFFUSION_NEGATIVE_CM2_S = 4.35e-2

AIR_DENSITY_KG_M3 = 1.225  # ISA sea level
AIR_DENSITY_20C_KG_M3 = 1.2041  # dry air, 20 degC, 101.325 kPa
JOULE_TO_KEV = 6.241e15


_REF_SOLVER = "pulsed_ion_chamber.solver_numba"
_REF_CONSTANTS = "pulsed_ion_chamber.constants"


def recombination_alpha(config=None) -> float:
    """The recombination coefficient a run uses when no ``alpha_cm3_s`` is
    given, resolved at call time.

    The reference has no alpha field on its config: each of its solvers reads
    the module constant it imported by name when the run starts
    (pulsed_ion_chamber/solver_numba.py:46, :274; solver_numba_parallel.py:100,
    :580; solver_cuda.py:99, :763), so a finite-difference study patches
    ``pulsed_ion_chamber.solver_numba.RECOMBINATION_ALPHA_CM3_S``. To give the
    same alpha as that patched solver, a configuration built by the reference
    (its class lives in ``pulsed_ion_chamber``) takes the value the loaded
    reference solver module holds when it differs from the reference's
    constant; otherwise this module's ``RECOMBINATION_ALPHA_CM3_S`` (read
    through the module, so patching it here works too)."""
    own = sys.modules[__name__].RECOMBINATION_ALPHA_CM3_S
    if config is not None and type(config).__module__.startswith("pulsed_ion_chamber"):
        solver = sys.modules.get(_REF_SOLVER)
        consts = sys.modules.get(_REF_CONSTANTS)
        patched = getattr(solver, "RECOMBINATION_ALPHA_CM3_S", None) if solver is not None else None
        default = getattr(consts, "RECOMBINATION_ALPHA_CM3_S", None) if consts is not None else None
        if patched is not None and patched != default:
            return float(patched)
    return float(own)
