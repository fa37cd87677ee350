"""Gradients of k_s through the hand-written adjoint (adjoint.py,
csrc/adjoint.cu) against central differences.

The derivative is taken at fixed dt, step count and tracks (the reference's
discrete dt ladder and step counts are piecewise constant in the
parameters), so the finite differences perturb the transport parameters and
the field of a copy of the configuration with everything else kept.
"""

import importlib

import numpy as np
import pytest

from goldens import make_config, pkg

REL_STEP = 1e-4  # relative step of the central differences


def _adj():
    return importlib.import_module(pkg().__name__ + ".adjoint")


def _central(fn, theta, rel=REL_STEP):
    g = np.zeros(len(theta))
    for q in range(len(theta)):
        tp, tm = theta.copy(), theta.copy()
        tp[q] = theta[q] * (1 + rel)
        tm[q] = theta[q] * (1 - rel)
        g[q] = (fn(tp) - fn(tm)) / (tp[q] - tm[q])
    return g


def test_chain_rule_from_step_numbers_to_parameters():
    """Host-side chain rule: dR/d(s+, c+, s-, c-, a) -> dk_s/dtheta equals
    finite differences of a synthetic R that is linear in the nine weights
    (random sensitivities), with the weights formed as the solver forms
    them. No GPU."""
    A = _adj()
    cfg = make_config("column_10um_r02")
    rng = np.random.default_rng(1)
    w = rng.normal(size=9)  # dR/d(lat+, zm+, zp+, cen+, lat-, zm-, zp-, cen-, a)

    def R(theta):
        pos, neg, adt, _ = A._weights(cfg, theta)
        return float(np.dot(w, list(pos) + list(neg) + [adt]))

    theta = A.base_parameters(cfg)
    # dR/ds = w_lat + w_zm + w_zp - 6 w_cen; dR/dc = (c+1/2) w_zm + (c-1/2) w_zp - 2c w_cen
    pos, neg, _, _ = A._weights(cfg, theta)
    cp, cn = pos[1] - pos[2], neg[1] - neg[2]
    gs = np.array([w[0] + w[1] + w[2] - 6 * w[3], (cp + 0.5) * w[1] + (cp - 0.5) * w[2] - 2 * cp * w[3],
                   w[4] + w[5] + w[6] - 6 * w[7], (cn + 0.5) * w[5] + (cn - 0.5) * w[6] - 2 * cn * w[7], w[8]])
    run = A.AdjointRun.__new__(A.AdjointRun)
    run.config, run.theta, run.ks, run.injected = cfg, theta, 1.0, 1.0
    got = run.chain(gs)
    want = _central(R, theta, rel=1e-6)
    # alpha * dt (~6e-13) is below the float64 resolution of this O(1)
    # synthetic R at a 1e-6 step: its derivative is checked in closed form
    want[0] = w[8] * cfg.dt
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-9 * np.abs(want[1:]).max())


def test_config_at_keeps_dt_and_steps():
    A = _adj()
    cfg = make_config("column_10um_r02")
    th = A.base_parameters(cfg)
    th[1:] *= 1.01
    c = A.config_at(cfg, th)
    assert c.dt == cfg.dt and c.total_time_steps == cfg.total_time_steps
    assert c.mu_positive == th[1] and c.voltage_V == th[5] and c.Efield_V_cm == th[5] / c.electrode_gap_cm
    assert cfg.mu_positive != c.mu_positive


@pytest.mark.gpu
@pytest.mark.parametrize("wall", ["absorbing", "reflecting"])
def test_float64_adjoint_equals_central_differences_of_the_oracle(oracle, wall):
    """Float64 fields: the adjoint gradient of k_s equals central differences
    (relative step 1e-4) of the float64 oracle to 1e-5 relative, per
    parameter, on a small pulsed column with both walls."""
    A = _adj()
    cfg = make_config("fast_dense", lateral_boundary=wall)
    theta = A.base_parameters(cfg)
    ks, grad, _ = A.ks_and_gradient(cfg, theta, checkpoint_every=5, dtype="float64")

    def ref(th):
        return oracle.run(A.config_at(cfg, th), mode="batched", alpha_cm3_s=th[0], threads=4, keep_fields=False)["ks"]

    assert ks == pytest.approx(ref(theta), rel=1e-10)
    fd = _central(ref, theta)
    np.testing.assert_allclose(grad, fd, rtol=1e-5, atol=1e-7 * np.abs(fd).max())


@pytest.mark.gpu
def test_float32_adjoint_on_the_column_chamber(oracle):
    """The 10 um, r = 0.02 cm column at 300 V (48 x 48 x 206, 1622 steps,
    142 729 tracks): float32 forward and adjoint with checkpoints every 64
    steps against central differences (relative step 1e-4) of float64
    oracle runs, to 1e-5 relative per parameter; k_s within 1e-5 of the
    oracle's."""
    A = _adj()
    cfg = make_config("column_10um_r02")
    theta = A.base_parameters(cfg)
    ks, grad, _ = A.ks_and_gradient(cfg, theta, checkpoint_every=64, dtype="float32")

    def ref(th):
        return oracle.run(A.config_at(cfg, th), mode="batched", alpha_cm3_s=th[0], threads=16, keep_fields=False)["ks"]

    assert abs(ks - ref(theta)) <= 1e-5
    fd = _central(ref, theta)
    # measured on GB300: every component within 3e-7 of the float64 differences
    for q in range(6):
        assert abs(grad[q] - fd[q]) <= 1e-5 * abs(fd[q]), (A.PARAMS[q], grad[q], fd[q])


@pytest.mark.gpu
def test_autograd_function_backward_is_the_adjoint():
    import torch

    A = _adj()
    cfg = make_config("fast_dense")
    theta = torch.tensor(A.base_parameters(cfg), dtype=torch.float64, requires_grad=True)
    ks = pkg().ks_b200(theta, cfg, checkpoint_every=4, dtype="float64")
    ks.backward()
    k2, g2, _ = A.ks_and_gradient(cfg, A.base_parameters(cfg), checkpoint_every=7, dtype="float64")
    assert float(ks.detach()) == pytest.approx(k2, rel=1e-12)
    np.testing.assert_allclose(theta.grad.numpy(), g2, rtol=1e-9)


@pytest.mark.gpu
def test_checkpoint_spacing_does_not_change_the_gradient():
    A = _adj()
    cfg = make_config("fast_dense", lateral_boundary="reflecting")
    g = [A.ks_and_gradient(cfg, None, checkpoint_every=k, dtype="float64")[1] for k in (1, 3, 1000)]
    np.testing.assert_allclose(g[0], g[1], rtol=1e-10)
    np.testing.assert_allclose(g[0], g[2], rtol=1e-10)


@pytest.mark.gpu
def test_fit_alpha_to_a_saturation_curve(oracle):
    """Fit alpha to a synthetic k_s(V) curve: the 10 um, r = 0.02 cm column
    at 8 voltages over 50-400 V, targets from the float64 oracle at alpha
    scaled by 1.3; gradient steps from the float32 adjoint recover it."""
    A = _adj()
    alpha0 = pkg().RECOMBINATION_ALPHA_CM3_S
    volts = np.linspace(50.0, 400.0, 8)
    cfgs = [make_config("column_10um_r02", voltage_V=float(v)) for v in volts]
    target = [oracle.run(c, mode="batched", alpha_cm3_s=1.3 * alpha0, threads=16, keep_fields=False)["ks"]
              for c in cfgs]
    alpha, history = A.fit_alpha(cfgs, target, alpha0, iterations=6)
    assert alpha == pytest.approx(1.3 * alpha0, rel=1e-4)
    assert history[-1][1] < 1e-6 * history[0][1]
