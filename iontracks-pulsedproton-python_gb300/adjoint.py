"""Gradients of k_s: the hand-written adjoint of the fused step behind
``torch.autograd.Function``.

``k_s = I / (I - R)`` (the reference forms it from its running totals,
pulsed_ion_chamber/solver_numba.py:311-350): ``I``, the injected charge, is
fixed by the tracks; ``R``, the recombined charge, depends on the recombination
coefficient ``alpha``, the mobilities ``mu+``/``mu-``, the diffusion
coefficients ``D+``/``D-`` and the voltage ``V`` through the Lax-Wendroff
weights of every step (pulsed_ion_chamber/config.py:477-480):

    s = D dt / h^2,  c = mu E dt / h,  E = V / gap,
    lat = s, zm = s + c(c+1)/2, zp = s + c(c-1)/2, cen = 1 - c^2 - 6s,
    a = alpha dt.

The derivative is taken at fixed ``dt``, step count and track schedule. In the
reference those come from discrete rules (``dt`` from a 1 % geometric ladder,
step counts by ``int``), so they are piecewise constant in the parameters and
this is the derivative almost everywhere -- what central differences of the
reference give away from a rung.

Method (reverse mode with checkpoints):

1. forward (``pic_adjoint_forward``): the float32 (or float64) run of
   :func:`run_simulation_b200`, storing the state every ``checkpoint_every``
   steps and keeping each depositing step's 2D density;
2. backward (``pic_adjoint_backward``), one segment of ``checkpoint_every``
   steps at a time from the last: recompute the segment's states from its
   checkpoint with the kept densities, then run the adjoint steps backwards
   over them, carrying ``lambda = dR/du`` across segments and summing
   ``dR/ds+, dR/dc+, dR/ds-, dR/dc-, dR/da`` over the steps (per block on
   the device, one final reduction);
3. the chain rule to the six parameters, in float64 on the host.

``dk_s/dtheta = k_s^2 / I * dR/dtheta``.
"""

from __future__ import annotations

import copy
import ctypes
from time import perf_counter
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from .config import lax_wendroff_weights
from .constants import RECOMBINATION_ALPHA_CM3_S
from .engine import ChamberEngine
from .pulses import TrackSampler, build_track_schedule
from .state import collection_efficiency

PARAMS = ("alpha", "mu_positive", "mu_negative", "D_positive", "D_negative", "voltage_V")


def base_parameters(config, alpha_cm3_s: Optional[float] = None) -> np.ndarray:
    """``theta = (alpha, mu+, mu-, D+, D-, V)`` of a configuration."""
    alpha = RECOMBINATION_ALPHA_CM3_S if alpha_cm3_s is None else float(alpha_cm3_s)
    return np.array([alpha, config.mu_positive, config.mu_negative, config.D_positive, config.D_negative,
                     config.voltage_V], dtype=np.float64)


def config_at(config, theta: Sequence[float]):
    """A copy of ``config`` with the transport parameters and field of
    ``theta`` and everything else -- dt, step counts, schedule, grid --
    unchanged (alpha is passed separately to the solvers)."""
    c = copy.copy(config)
    _, c.mu_positive, c.mu_negative, c.D_positive, c.D_negative, c.voltage_V = (float(x) for x in theta)
    c.Efield_V_cm = c.voltage_V / c.electrode_gap_cm
    return c


def _weights(config, theta):
    """The step's weights at theta and the configuration's dt (the same
    arithmetic as the configuration's own scheme coefficients, so the base
    theta gives the plain solver's weights bit for bit)."""
    alpha, mu_p, mu_n, d_p, d_n, volts = (float(x) for x in theta)
    e_field = volts / config.electrode_gap_cm
    dt, h = config.dt, config.unit_length_cm
    pos = lax_wendroff_weights(d_p, mu_p, e_field, dt, h)
    neg = lax_wendroff_weights(d_n, mu_n, e_field, dt, h)
    return pos, neg, alpha * dt, e_field


class AdjointRun:
    """One configuration's k_s and, on request, its gradient.

    ``theta`` = (alpha, mu+, mu-, D+, D-, V) (default: the configuration's
    own, with the reference's alpha). ``checkpoint_every`` = steps between
    stored states (memory: one state per checkpoint, a segment buffer of
    ``checkpoint_every`` states, and the 2D density of every step with
    tracks).
    """

    def __init__(self, config, theta=None, checkpoint_every: int = 64, dtype: str = "float32", rng=None,
                 use_graphs: bool = False):
        import torch

        if dtype not in ("float32", "float64"):
            raise ValueError(f"dtype must be 'float32' or 'float64', got {dtype!r}")
        if int(checkpoint_every) < 1:
            raise ValueError("checkpoint_every must be >= 1")
        self.torch = torch
        self.config = config
        self.theta = base_parameters(config) if theta is None else np.asarray(theta, dtype=np.float64).copy()
        if self.theta.shape != (6,):
            raise ValueError("theta must hold (alpha, mu+, mu-, D+, D-, V)")
        self.K = int(checkpoint_every)
        self.dtype = dtype
        self.use_graphs = bool(use_graphs)
        self.rng = rng if rng is not None else np.random.default_rng(config.seed)
        self.lib = N.load()
        self._eng = None
        self.ks = None
        self.timings = {}

    def _issue(self, launch) -> None:
        """Run ``launch(stream)`` -- one whole-pass library call -- on the
        device: captured into a CUDA graph on a private stream and replayed
        once (one submission for thousands of small launches), or launched
        directly on the current stream."""
        torch = self.torch
        dev = self._eng.device
        cur = torch.cuda.current_stream(dev)
        if not self.use_graphs:
            launch(cur.cuda_stream)
            return
        lib = self.lib
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(cur)
        N.check(lib.pic_capture_begin(side.cuda_stream), "pic_capture_begin")
        h = ctypes.c_void_p()
        try:
            launch(side.cuda_stream)
        except Exception:
            lib.pic_capture_end(side.cuda_stream, ctypes.byref(h))
            if h.value:
                lib.pic_graph_destroy(h)
            raise
        N.check(lib.pic_capture_end(side.cuda_stream, ctypes.byref(h)), "pic_capture_end")
        try:
            N.check(lib.pic_graph_launch(h, side.cuda_stream), "pic_graph_launch")
            side.synchronize()
        finally:
            lib.pic_graph_destroy(h)
        cur.wait_stream(side)

    # ---- forward ---------------------------------------------------------
    def forward(self) -> float:
        """Run the checkpointed forward solve; returns k_s."""
        torch = self.torch
        cfg = self.config
        t0 = perf_counter()
        total = int(cfg.total_time_steps)
        schedule = build_track_schedule(cfg, self.rng)
        n_tracks = int(schedule.sum())
        xs, ys = TrackSampler(self.rng, cfg.mid_xy, cfg.sampling_radius, cfg.no_xy).sample(n_tracks)
        self.offsets = np.zeros(total + 1, dtype=np.int64)
        np.cumsum(schedule, out=self.offsets[1:])
        eng = ChamberEngine(cfg, dtype=self.dtype, max_tracks=max(1, n_tracks))
        (pl, pzm, pzp, pc), (nl, nzm, nzp, nc), adt, _ = _weights(cfg, self.theta)
        g = eng.grid
        g.p_lat, g.p_zm, g.p_zp, g.p_cen = pl, pzm, pzp, pc
        g.n_lat, g.n_zm, g.n_zp, g.n_cen = nl, nzm, nzp, nc
        g.alpha_dt = adt
        eng.upload_tracks(xs, ys)
        self._eng = eng
        self.n_seg = -(-total // self.K)
        field = int(g.no_xy) ** 2 * int(g.kpitch)
        self.field = field
        dev, tdt = eng.device, eng.pos[0].dtype
        n = int(g.no_xy)
        self.dslot = 2 * n * ((n + 3) // 4 * 4)  # one step's deposition pairs
        n_dep = int(np.count_nonzero(schedule))
        es = 4 if self.dtype == "float32" else 8
        need = (self.n_seg + self.K) * 2 * field * es + n_dep * self.dslot * es + 4 * field * es
        free, _ = torch.cuda.mem_get_info(dev)
        if need > 0.9 * free:
            raise MemoryError(f"the gradient needs {need / 2**30:.2f} GiB of device memory for checkpoints, "
                              f"the segment buffer and the kept densities; {free / 2**30:.2f} GiB is free "
                              f"(raise checkpoint_every to trade memory for recomputation)")
        self.ckpt = torch.empty((2, max(self.n_seg, 1), field), dtype=tdt, device=dev)
        self.dens_keep = torch.empty((max(n_dep, 1), self.dslot), dtype=tdt, device=dev)
        off = np.ascontiguousarray(self.offsets)
        self._issue(lambda st: N.check(self.lib.pic_adjoint_forward(
            ctypes.byref(g), eng.pos[0].data_ptr(), eng.neg[0].data_ptr(), eng.pos[1].data_ptr(),
            eng.neg[1].data_ptr(), total, eng.xs.data_ptr(), eng.ys.data_ptr(), off.ctypes.data_as(ctypes.c_void_p),
            self.dens_keep.data_ptr(), eng.counts.data_ptr(), eng.tally.data_ptr(), self.ckpt[0].data_ptr(),
            self.ckpt[1].data_ptr(), self.K, field, eng.workspace.data_ptr(), eng.workspace.numel(), st),
            "pic_adjoint_forward"))
        tallies = eng.tallies(total)
        eng.check_status()
        # running float64 totals, as the solver and the reference form them
        self.injected = float(np.cumsum(tallies[:, 0])[-1])
        self.recombined = float(np.cumsum(tallies[:, 1])[-1])
        self.ks = 1.0 / collection_efficiency(tallies[:, 0], tallies[:, 1], total)[-1]
        self.timings["forward_s"] = perf_counter() - t0
        return self.ks

    # ---- backward --------------------------------------------------------
    def gradient_of_recombined(self) -> np.ndarray:
        """dR/d(s+, c+, s-, c-, a), summed over the run in float64."""
        if self._eng is None:
            raise RuntimeError("call forward() first")
        torch = self.torch
        eng = self._eng
        g = eng.grid
        lib = self.lib
        t0 = perf_counter()
        total = int(self.config.total_time_steps)
        K, field = self.K, self.field
        dev, tdt = eng.device, eng.pos[0].dtype
        states = torch.empty((2, K, field), dtype=tdt, device=dev)
        lam = torch.zeros((2, 2, field), dtype=tdt, device=dev)  # [buffer][species]
        grad = torch.zeros(5, dtype=torch.float64, device=dev)
        awb = ctypes.c_int64()
        N.check(lib.pic_adjoint_workspace_bytes(ctypes.byref(g), ctypes.byref(awb)), "pic_adjoint_workspace_bytes")
        adj_ws = torch.zeros(int(awb.value), dtype=torch.uint8, device=dev)
        off = np.ascontiguousarray(self.offsets)
        self._issue(lambda st: N.check(lib.pic_adjoint_backward(
            ctypes.byref(g), self.ckpt[0].data_ptr(), self.ckpt[1].data_ptr(), field, total, K,
            off.ctypes.data_as(ctypes.c_void_p), self.dens_keep.data_ptr(), states[0].data_ptr(),
            states[1].data_ptr(), lam[0, 0].data_ptr(), lam[0, 1].data_ptr(), lam[1, 0].data_ptr(),
            lam[1, 1].data_ptr(), grad.data_ptr(), eng.workspace.data_ptr(),
            eng.workspace.numel(), adj_ws.data_ptr(), adj_ws.numel(), st), "pic_adjoint_backward"))
        out = grad.cpu().numpy()
        eng.check_status()
        self.timings["backward_s"] = perf_counter() - t0
        return out

    def backward(self) -> np.ndarray:
        """dk_s/dtheta for theta = (alpha, mu+, mu-, D+, D-, V), float64."""
        gs = self.gradient_of_recombined()
        return self.chain(gs)

    def chain(self, gs: np.ndarray) -> np.ndarray:
        """dk_s/dtheta from dR/d(s+, c+, s-, c-, a)."""
        cfg = self.config
        alpha, mu_p, mu_n, d_p, d_n, volts = self.theta
        dt, h, gap = cfg.dt, cfg.unit_length_cm, cfg.electrode_gap_cm
        e_field = volts / gap
        g_sp, g_cp, g_sn, g_cn, g_a = (float(x) for x in gs)
        dR = np.array([
            g_a * dt,                                  # alpha
            g_cp * e_field * dt / h,                   # mu+
            g_cn * e_field * dt / h,                   # mu-
            g_sp * dt / h**2,                          # D+
            g_sn * dt / h**2,                          # D-
            (g_cp * mu_p + g_cn * mu_n) * dt / (h * gap),  # V
        ])
        return self.ks**2 / self.injected * dR

    def release(self) -> None:
        if self._eng is not None:
            self._eng.close()
            self._eng = None
        self.ckpt = None
        self.dens_keep = None


def ks_and_gradient(config, theta=None, checkpoint_every: int = 64, dtype: str = "float32", rng=None,
                    use_graphs: bool = False):
    """``(k_s, dk_s/dtheta, timings)`` for theta = (alpha, mu+, mu-, D+, D-, V)."""
    run = AdjointRun(config, theta, checkpoint_every, dtype, rng, use_graphs)
    try:
        ks = run.forward()
        grad = run.backward()
        return ks, grad, dict(run.timings)
    finally:
        run.release()


def _autograd_function():
    import torch

    class KsFunction(torch.autograd.Function):
        """k_s(theta) with the adjoint as its backward. theta: float64 tensor
        (alpha, mu+, mu-, D+, D-, V)."""

        @staticmethod
        def forward(ctx, theta, config, checkpoint_every, dtype):
            run = AdjointRun(config, theta.detach().cpu().numpy(), checkpoint_every, dtype)
            ks = run.forward()
            ctx.run = run
            return torch.tensor(ks, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            run = ctx.run
            try:
                g = run.backward()
            finally:
                run.release()
            return torch.from_numpy(g) * grad_out.to(torch.float64).cpu(), None, None, None

    return KsFunction


_KS_FN = None


def ks_b200(theta, config, checkpoint_every: int = 64, dtype: str = "float32"):
    """Differentiable k_s: ``ks_b200(theta, config)`` with ``theta`` a float64
    tensor (alpha, mu+, mu-, D+, D-, V) that may require grad; backward runs the
    adjoint sweep. The forward is the GB300 solve of ``config`` at ``theta``
    (fixed dt, step count and tracks)."""
    global _KS_FN
    if _KS_FN is None:
        _KS_FN = _autograd_function()
    return _KS_FN.apply(theta, config, int(checkpoint_every), dtype)


def fit_alpha(configs, ks_target, alpha0: float, iterations: int = 8, checkpoint_every: int = 64,
              dtype: str = "float32", tol: float = 1e-7):
    """Fit the recombination coefficient to a k_s curve.

    ``configs`` (e.g. one chamber at several voltages) and ``ks_target`` (their
    measured or reference k_s) define the loss ``L = sum (k_s(alpha) - target)^2``;
    each iteration runs every configuration forward and backward (the adjoint
    gives dk_s/dalpha) and takes the gradient step ``-dL/dalpha`` scaled by the
    Gauss-Newton curvature ``2 sum (dk_s/dalpha)^2`` -- for this one-parameter
    least-squares problem, the step that lands on the minimum of the
    linearised loss. Returns ``(alpha, history)``, history = [(alpha, loss)].
    """
    alpha = float(alpha0)
    target = np.asarray(ks_target, dtype=np.float64)
    history = []
    for _ in range(int(iterations)):
        ks = np.zeros(len(configs))
        dks = np.zeros(len(configs))
        for q, cfg in enumerate(configs):
            theta = base_parameters(cfg, alpha)
            k, grad, _ = ks_and_gradient(cfg, theta, checkpoint_every, dtype)
            ks[q], dks[q] = k, grad[0]
        r = ks - target
        loss = float(np.sum(r * r))
        history.append((alpha, loss))
        grad_l = 2.0 * float(np.sum(r * dks))
        curv = 2.0 * float(np.sum(dks * dks))
        if curv <= 0.0:
            break
        step = grad_l / curv
        alpha -= step
        if abs(step) <= tol * abs(alpha):
            break
    return alpha, history
