"""Physical constants of ion transport in air.

The values are the published Kanai et al. (1998) carrier constants and the
recombination coefficient the reference solver uses
(pulsed_ion_chamber/constants.py:11-35). They are inputs to the physics, so
they must be the same numbers for results to agree.

``RECOMBINATION_ALPHA_CM3_S`` is read by :func:`run_simulation_b200` only as a
default: pass ``alpha_cm3_s=`` to override it per run, which is how the
adjoint and the alpha fit perturb it (the reference instead reads its module
constant at call time, pulsed_ion_chamber/solver_numba.py:46, :274).
"""

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
