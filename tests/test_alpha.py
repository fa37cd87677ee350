"""Which recombination coefficient a run uses when none is passed (CPU).

The reference has no alpha on its config: its solvers read the module
constant they imported (pulsed_ion_chamber/solver_numba.py:46, :274), and a
finite-difference study patches that solver module's constant. A reference
configuration handed to this package must then run with the patched value;
this package's own constant stays patchable the same way."""

import sys
import types

import pytest

from goldens import make_config, pkg


def _mods():
    import importlib

    name = pkg().__name__
    return importlib.import_module(name + ".constants"), importlib.import_module(name + ".engine")


class _RefConfigProxy:
    """Stands in for a configuration built by the reference: same attributes,
    class defined in the reference's config module."""

    def __init__(self, cfg):
        self.__dict__.update({k: getattr(cfg, k) for k in dir(cfg) if not k.startswith("_")})
        self._cfg = cfg

    def scheme_coefficients(self):
        return self._cfg.scheme_coefficients()


_RefConfigProxy.__module__ = "pulsed_ion_chamber.config"


@pytest.fixture
def fake_reference(monkeypatch):
    consts = types.ModuleType("pulsed_ion_chamber.constants")
    consts.RECOMBINATION_ALPHA_CM3_S = 1.60e-6
    solver = types.ModuleType("pulsed_ion_chamber.solver_numba")
    solver.RECOMBINATION_ALPHA_CM3_S = 1.60e-6
    monkeypatch.setitem(sys.modules, "pulsed_ion_chamber.constants", consts)
    monkeypatch.setitem(sys.modules, "pulsed_ion_chamber.solver_numba", solver)
    return solver


def test_default_alpha_is_the_published_constant():
    C, E = _mods()
    cfg = make_config("fast")
    assert C.recombination_alpha(cfg) == 1.60e-6
    g = E.make_grid(cfg)
    assert g.alpha_dt == 1.60e-6 * cfg.dt


def test_patching_this_package_constant_takes_effect(monkeypatch):
    C, E = _mods()
    cfg = make_config("fast")
    monkeypatch.setattr(C, "RECOMBINATION_ALPHA_CM3_S", 2.5e-6)
    assert E.make_grid(cfg).alpha_dt == 2.5e-6 * cfg.dt
    assert E.make_grid(cfg, alpha_cm3_s=1.0e-6).alpha_dt == 1.0e-6 * cfg.dt  # the keyword wins


def test_reference_config_follows_the_patched_reference_solver(fake_reference):
    C, E = _mods()
    cfg = make_config("fast")
    ref_cfg = _RefConfigProxy(cfg)
    # unpatched: the published value either way
    assert E.make_grid(ref_cfg).alpha_dt == 1.60e-6 * cfg.dt
    fake_reference.RECOMBINATION_ALPHA_CM3_S = 1.60e-6 * (1 + 1e-4)
    assert C.recombination_alpha(ref_cfg) == 1.60e-6 * (1 + 1e-4)
    assert E.make_grid(ref_cfg).alpha_dt == 1.60e-6 * (1 + 1e-4) * cfg.dt
    # this package's own configuration is not the reference's: its constant applies
    assert E.make_grid(cfg).alpha_dt == 1.60e-6 * cfg.dt
    adj = __import__("importlib").import_module(pkg().__name__ + ".adjoint")
    assert adj.base_parameters(ref_cfg)[0] == 1.60e-6 * (1 + 1e-4)
