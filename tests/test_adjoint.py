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


# ---- binomial checkpointing (csrc/revolve.cu) -----------------------------

def _binomial_cost(l, s):
    """Fewest forward steps that reverse l steps from a stored start with s
    state slots, by exhaustive recursion over the first stored state (small
    l only): the optimum the schedule must reach."""
    from functools import lru_cache

    @lru_cache(None)
    def best(l, s):
        if l <= 1:
            return 0
        if s == 1:
            return l * (l - 1) // 2
        return min(m + best(l - m, s - 1) + best(m, s) for m in range(1, l))

    return best(l, s)


def _trace(n_steps, n_slots):
    import ctypes

    N = importlib.import_module(pkg().__name__ + "._native")
    lib = N.load()
    n_ev, adv = ctypes.c_int64(), ctypes.c_int64()
    N.check(lib.pic_revolve_trace(n_steps, n_slots, None, 0, ctypes.byref(n_ev), ctypes.byref(adv)), "trace")
    ev = np.zeros((max(n_ev.value, 1), 4), dtype=np.int64)
    N.check(lib.pic_revolve_trace(n_steps, n_slots, ev.ctypes.data, n_ev.value, ctypes.byref(n_ev),
                                  ctypes.byref(adv)), "trace")
    spine = np.zeros(n_slots, dtype=np.int64)
    lev = ctypes.c_int64()
    N.check(lib.pic_revolve_spine(n_steps, n_slots, spine.ctypes.data, n_slots, ctypes.byref(lev)), "spine")
    return ev[: n_ev.value], int(adv.value), spine[: lev.value]


def test_binomial_schedule_reverses_every_step_at_the_optimal_cost():
    """The library's schedule, run against its bookkeeping of the slots (no
    GPU): every adjoint step runs once, from the state it needs, in the order
    n-1 .. 0; forward steps stored along the spine plus the recomputed ones
    equal the optimum of an exhaustive search for every run of up to 40
    steps with 1 to 6 slots."""
    A = _adj()
    for n_steps in range(1, 41):
        for n_slots in range(1, 7):
            ev, adv, spine = _trace(n_steps, n_slots)
            adj = ev[ev[:, 0] == 2, 1]
            assert list(adj) == list(range(n_steps - 1, -1, -1)), (n_steps, n_slots)
            assert adv + int(spine[-1]) == _binomial_cost(n_steps, n_slots), (n_steps, n_slots)
            assert spine[0] == 0 and np.all(np.diff(spine) > 0) and len(spine) <= n_slots
            assert A.revolve_plan(n_steps, n_slots) == (adv, len(spine))


def test_binomial_plan_of_the_full_electrode():
    """985 801 steps (the 5 um full electrode, 10 pulses) in 43 float32 state
    slots (160 GB of 3.7 GB states): under 4 recomputed steps per step, and the
    cost falls as slots are added."""
    A = _adj()
    rec43, lev43 = A.revolve_plan(985801, 43)
    rec20, _ = A.revolve_plan(985801, 20)
    assert lev43 == 43
    assert rec43 < 4 * 985801
    assert rec20 > rec43
    # a slot per step: nothing to recompute
    assert A.revolve_plan(50, 50) == (0, 50)


@pytest.mark.gpu
@pytest.mark.parametrize("wall", ["absorbing", "reflecting"])
def test_binomial_schedule_gives_the_segment_gradient(wall):
    """Float64: the binomial schedule (1, 2, 3 and 6 slots, tracks deposited
    again on every recomputed step) gives the gradient and k_s of the segment
    schedule (kept densities) to 1e-10."""
    A = _adj()
    cfg = make_config("fast_dense", lateral_boundary=wall)
    ks0, g0, _ = A.ks_and_gradient(cfg, None, checkpoint_every=5, dtype="float64", schedule="segments")
    for slots in (1, 2, 3, 6):
        ks, g, tm = A.ks_and_gradient(cfg, None, dtype="float64", schedule="binomial", slots=slots)
        assert tm["plan"]["schedule"] == "binomial" and tm["plan"]["slots"] == slots
        assert ks == pytest.approx(ks0, rel=1e-12)
        np.testing.assert_allclose(g, g0, rtol=1e-10, atol=1e-12 * np.abs(g0).max())


@pytest.mark.gpu
def test_binomial_schedule_float32_column():
    """Float32, the 10 um r = 0.02 cm column (1622 steps): 8 binomial slots
    against the segment schedule, to 1e-6 relative per parameter."""
    A = _adj()
    cfg = make_config("column_10um_r02")
    ks0, g0, _ = A.ks_and_gradient(cfg, None, checkpoint_every=64, dtype="float32", schedule="segments")
    ks, g, tm = A.ks_and_gradient(cfg, None, dtype="float32", schedule="binomial", slots=8)
    assert tm["plan"]["recompute_steps"] == A.revolve_plan(1622, 8)[0]
    # two float32 runs differ in the order of the deposition's atomic adds
    assert ks == pytest.approx(ks0, rel=1e-9)
    np.testing.assert_allclose(g, g0, rtol=1e-6)


@pytest.mark.gpu
def test_truncated_run_gradient_equals_its_central_differences():
    """max_steps: the gradient of the k_s of the first 12 steps (float64,
    binomial, 3 slots) equals central differences of that truncated k_s."""
    A = _adj()
    cfg = make_config("fast_dense")
    theta = A.base_parameters(cfg)
    ks, grad, tm = A.ks_and_gradient(cfg, theta, dtype="float64", max_steps=12, schedule="binomial", slots=3)
    assert tm["plan"]["steps"] == 12

    def fwd(th):
        run = A.AdjointRun(cfg, th, dtype="float64", max_steps=12, schedule="binomial", slots=1)
        try:
            return run.forward()
        finally:
            run.release()

    assert ks == pytest.approx(fwd(theta), rel=1e-13)
    fd = _central(fwd, theta)
    np.testing.assert_allclose(grad, fd, rtol=1e-5, atol=1e-7 * np.abs(fd).max())


@pytest.mark.gpu
def test_full_electrode_gradient_in_180_gb():
    """The 5 um full electrode (1068 x 1068 x 406, 463 M voxels): float32
    forward + adjoint of its first 100 steps (a track-depositing stretch of
    the first pulse) under a 180 GB device-memory limit -- the binomial
    schedule, with as many 3.7 GB state slots as fit -- against central
    differences of float64 forward runs of the same 100 steps, for all six
    parameters; peak device memory within the limit."""
    import torch

    A = _adj()
    P = pkg()
    cfg = P.SimulationConfig(E_MeV_u=56.2, voltage_V=300.0, electrode_gap_cm=0.2, pulse_duration_s=540e-6,
                             repetition_rate_hz=50.0, dose_rate_Gy_s=8.91, grid_size_um=5.0, sampled_radius_cm=0.265,
                             n_pulses=10, seed=1, max_voxels=2e9)
    assert (cfg.no_xy, cfg.no_z_with_buffer) == (1068, 406)
    limit = 180e9
    torch.cuda.empty_cache()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    theta = A.base_parameters(cfg)
    ks, grad, tm = A.ks_and_gradient(cfg, theta, dtype="float32", max_steps=100, memory_limit=limit)
    peak = torch.cuda.max_memory_allocated() - base
    plan = tm["plan"]
    assert plan["schedule"] == "binomial" and plan["slots"] >= 30, plan
    assert peak <= limit, (peak, plan)
    torch.cuda.empty_cache()

    def fwd(th):
        run = A.AdjointRun(cfg, th, dtype="float64", max_steps=100, schedule="binomial", slots=1)
        try:
            return run.forward()
        finally:
            run.release()
            torch.cuda.empty_cache()

    k64 = fwd(theta)
    assert abs(ks - k64) <= 1e-6, (ks, k64)
    for q in range(6):
        tp, tmn = theta.copy(), theta.copy()
        tp[q] *= 1 + REL_STEP
        tmn[q] *= 1 - REL_STEP
        fd = (fwd(tp) - fwd(tmn)) / (tp[q] - tmn[q])
        assert abs(grad[q] - fd) <= 1e-4 * abs(fd), (A.PARAMS[q], grad[q], fd)


def _adjoint_step(g, pos, neg, dens, lp, ln):
    """One pic_adjoint_step (per-step derivative sums) on copies of lambda
    (a reflecting wall folds its input in place)."""
    import ctypes

    import torch

    N = importlib.import_module(pkg().__name__ + "._native")
    lib = N.load()
    awb = ctypes.c_int64()
    N.check(lib.pic_adjoint_workspace_bytes(ctypes.byref(g), ctypes.byref(awb)), "pic_adjoint_workspace_bytes")
    ws = torch.zeros(int(awb.value), dtype=torch.uint8, device="cuda")
    lp_in, ln_in = lp.clone(), ln.clone()
    lp_out, ln_out = torch.full_like(lp, float("nan")), torch.full_like(ln, float("nan"))
    grad = torch.zeros(5, dtype=torch.float64, device="cuda")
    N.check(lib.pic_adjoint_step(ctypes.byref(g), pos.data_ptr(), neg.data_ptr(),
                                 None if dens is None else dens.data_ptr(), lp_in.data_ptr(), ln_in.data_ptr(),
                                 lp_out.data_ptr(), ln_out.data_ptr(), grad.data_ptr(), ws.data_ptr(), ws.numel(),
                                 torch.cuda.current_stream().cuda_stream), "pic_adjoint_step")
    torch.cuda.synchronize()
    status = ws[64:68].view(torch.int32).item()
    return lp_out.cpu().numpy(), ln_out.cpu().numpy(), grad.cpu().numpy(), status


# Grids of the streaming adjoint's kernel-level check: (config overrides,
# tile rows, planes per work item).
STREAM_ADJOINT_CASES = {
    # the 10 um chamber at r = 0.035 cm: 14-row tiles, 32-plane items
    "short_items": (dict(sampled_radius_cm=0.035), 14, 32),
    # a thin chamber (no_z 8, kpitch 16) 1608 columns wide: 16-row tiles and
    # 2 626 work items of 64 planes (at least 6 per SM on 152 SMs)
    "long_items": (dict(sampled_radius_cm=0.8, electrode_gap_cm=0.008), 16, 64),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(STREAM_ADJOINT_CASES))
@pytest.mark.parametrize("wall", ["absorbing", "reflecting"])
@pytest.mark.parametrize("deposit", [False, True])
def test_stream_adjoint_step_equals_the_flat_one(case, wall, deposit):
    """pic_adjoint_step with the streaming kernel (adjoint_variant STREAM)
    against the flat kernel (adjoint_variant FLAT) on the same random state, lambda and
    deposition pairs, on grids whose tiles and work items are ragged, with
    32- and 64-plane work items: lambda_s of every column, the ring's
    included, to 1e-6 of its scale; the step's five derivative sums to 1e-5
    relative."""
    import torch

    eng_mod = importlib.import_module(pkg().__name__ + ".engine")
    N = importlib.import_module(pkg().__name__ + "._native")
    overrides, tile_rows, planes = STREAM_ADJOINT_CASES[case]
    cfg = make_config("column_10um_r02", lateral_boundary=wall, **overrides)
    n, nzb = int(cfg.no_xy), int(cfg.no_z_with_buffer)
    kp = (nzb + 7) // 8 * 8
    assert (n - 2) % tile_rows and (n - 2) % planes, n  # ragged last tile and last item
    if planes == 64:
        items = -(-(n - 2) // tile_rows) * -(-(n - 2) // 64)
        assert kp == 16 and items >= 6 * torch.cuda.get_device_properties(0).multi_processor_count, items
    rng = np.random.default_rng(7)
    state = rng.uniform(0.0, 1e6, size=(2, n, n, kp)).astype(np.float32)
    state[..., 0] = 0.0
    state[..., nzb - 1:] = 0.0
    lam = rng.normal(size=(2, n, n, kp)).astype(np.float32)
    # lambda is zero on the end planes and the padding, as every adjoint step leaves it
    lam[..., 0] = 0.0
    lam[..., nzb - 1:] = 0.0
    dp = (n + 3) // 4 * 4
    pairs = np.zeros((n, dp, 2), dtype=np.float32)
    if deposit:
        pairs[:, :n] = rng.uniform(0.0, 2e5, size=(n, n, 2))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    pos, neg, lp, ln = dev(state[0]), dev(state[1]), dev(lam[0]), dev(lam[1])
    dens = dev(pairs) if deposit else None
    out = {}
    for variant in (N.PIC_VARIANT_FLAT, N.PIC_VARIANT_STREAM):
        g = eng_mod.make_grid(cfg, "float32")
        g.adjoint_variant = variant
        out[variant] = _adjoint_step(g, pos, neg, dens, lp, ln)
    f, s = out[N.PIC_VARIANT_FLAT], out[N.PIC_VARIANT_STREAM]
    assert s[3] == 0 and np.all(np.isfinite(s[0])) and np.all(np.isfinite(s[1]))
    for q in (0, 1):
        scale = np.abs(f[q]).max()
        np.testing.assert_allclose(s[q], f[q], rtol=0, atol=1e-6 * scale)
    np.testing.assert_allclose(s[2], f[2], rtol=1e-5, atol=1e-9 * np.abs(f[2]).max())


@pytest.mark.gpu
@pytest.mark.parametrize("wall", ["absorbing", "reflecting"])
def test_stream_variant_gradient(wall):
    """The whole gradient with the streaming step and adjoint kernels forced on
    a 10 um chamber (r = 0.035 cm, 1622 steps): equal to the flat kernels'
    to 1e-5 relative per parameter."""
    A = _adj()
    cfg = make_config("column_10um_r02", sampled_radius_cm=0.035, lateral_boundary=wall)
    ks0, g0, _ = A.ks_and_gradient(cfg, None, dtype="float32", shape={"variant": "flat", "adjoint_variant": "flat"})
    ks1, g1, _ = A.ks_and_gradient(cfg, None, dtype="float32",
                                   shape={"variant": "stream", "adjoint_variant": "stream"})
    assert abs(ks1 - ks0) <= 1e-6
    np.testing.assert_allclose(g1, g0, rtol=1e-5)


def test_fit_parameters_validates_its_names():
    A = _adj()
    cfg = make_config("column_10um_r02")
    with pytest.raises(ValueError):
        A.fit_parameters([cfg], [1.0], names=("voltage_V",))
    with pytest.raises(ValueError):
        A.fit_parameters([cfg, cfg], [1.0], names=("alpha",))


@pytest.mark.gpu
def test_fit_two_parameters_to_a_saturation_curve(oracle):
    """Fit alpha and mu- together to a synthetic k_s(V) curve: the 10 um,
    r = 0.02 cm column at 8 voltages over 50-400 V, targets from the float64
    oracle at alpha x 1.3 and mu- x 0.85; Levenberg-Marquardt steps from the
    float32 adjoint's Jacobian recover both from the reference values."""
    A = _adj()
    alpha0 = pkg().RECOMBINATION_ALPHA_CM3_S
    volts = np.linspace(50.0, 400.0, 8)
    cfgs = [make_config("column_10um_r02", voltage_V=float(v)) for v in volts]
    true = {"alpha": 1.3 * alpha0, "mu_negative": 0.85 * cfgs[0].mu_negative}
    target = []
    for c in cfgs:
        th = A.base_parameters(c, true["alpha"])
        th[2] = true["mu_negative"]
        target.append(oracle.run(A.config_at(c, th), mode="batched", alpha_cm3_s=th[0], threads=16,
                                 keep_fields=False)["ks"])
    values, history = A.fit_parameters(cfgs, target, names=("alpha", "mu_negative"), iterations=8)
    assert values["alpha"] == pytest.approx(true["alpha"], rel=1e-3)
    assert values["mu_negative"] == pytest.approx(true["mu_negative"], rel=1e-3)
    assert history[-1][1] < 1e-6 * history[0][1]


def test_binomial_schedule_on_long_runs_matches_the_closed_form():
    """Longer runs (up to 5 000 steps, 2 to 12 slots): every adjoint step
    once, in order, from its own state, and forward steps (spine + recomputed)
    equal Griewank's closed form t l - beta(s+1, t-1) = t l - C(s+t, s+1), t
    the fewest repetitions with C(s+t, s) >= l (s = 1: l (l-1) / 2)."""
    from math import comb

    def closed_form(l, s):
        if l <= 1:
            return 0
        if s == 1:
            return l * (l - 1) // 2
        t = 0
        while comb(s + t, s) < l:
            t += 1
        return t * l - comb(s + t, s + 1)

    for n_steps, n_slots in [(97, 2), (500, 3), (1000, 5), (2500, 7), (5000, 12), (5000, 2)]:
        ev, adv, spine = _trace(n_steps, n_slots)
        adj = ev[ev[:, 0] == 2, 1]
        assert np.array_equal(adj, np.arange(n_steps - 1, -1, -1)), (n_steps, n_slots)
        assert adv + int(spine[-1]) == closed_form(n_steps, n_slots), (n_steps, n_slots)
        # no advance starts past the run or runs off its end
        adv_ev = ev[ev[:, 0] == 1]
        assert np.all(adv_ev[:, 1] + adv_ev[:, 2] <= n_steps)
