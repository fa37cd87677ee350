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

Method (reverse mode with checkpoints), one of two schedules:

* "segments" (short runs):
  1. forward (``pic_adjoint_forward``): the float32 (or float64) run of
     :func:`run_simulation_b200`, storing the state every ``checkpoint_every``
     steps and keeping each depositing step's 2D density;
  2. backward (``pic_adjoint_backward``), one segment of ``checkpoint_every``
     steps at a time from the last: recompute the segment's states from its
     checkpoint with the kept densities, then run the adjoint steps backwards
     over them, carrying ``lambda = dR/du`` across segments and summing
     ``dR/ds+, dR/dc+, dR/ds-, dR/dc-, dR/da`` over the steps (per block on
     the device, one final reduction).
* "binomial" (runs whose segments and kept densities do not fit, e.g. the
  5 um full electrode: 3.7 GB per state, 985 801 steps): a fixed number of
  state slots sized to the memory limit and Griewank's binomial schedule
  (``pic_revolve_forward`` / ``pic_revolve_backward``), which reverses the
  run with the fewest recomputed steps those slots allow; recomputed steps
  deposit their tracks again.

Then the chain rule to the six parameters, in float64 on the host.

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
from .constants import recombination_alpha
from .engine import ChamberEngine
from .pulses import TrackSampler, build_track_schedule
from .state import collection_efficiency

PARAMS = ("alpha", "mu_positive", "mu_negative", "D_positive", "D_negative", "voltage_V")


def base_parameters(config, alpha_cm3_s: Optional[float] = None) -> np.ndarray:
    """``theta = (alpha, mu+, mu-, D+, D-, V)`` of a configuration."""
    alpha = recombination_alpha(config) if alpha_cm3_s is None else float(alpha_cm3_s)
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


SCHEDULES = ("auto", "segments", "binomial")


def revolve_plan(n_steps: int, n_slots: int):
    """``(recomputed steps, stored states)`` of the binomial schedule that
    reverses ``n_steps`` steps with ``n_slots`` state slots (no device work)."""
    lib = N.load()
    rec, lev = ctypes.c_int64(), ctypes.c_int64()
    N.check(lib.pic_revolve_plan(int(n_steps), int(n_slots), ctypes.byref(rec), ctypes.byref(lev)),
            "pic_revolve_plan")
    return int(rec.value), int(lev.value)


class AdjointRun:
    """One configuration's k_s and, on request, its gradient.

    ``theta`` = (alpha, mu+, mu-, D+, D-, V) (default: the configuration's
    own, with the reference's alpha). ``checkpoint_every`` = steps between
    stored states of the "segments" schedule (memory: one state per
    checkpoint, a segment buffer of ``checkpoint_every`` states, and the 2D
    density of every step with tracks). ``schedule``: "segments", "binomial"
    (as many state slots as ``memory_limit`` leaves room for), or "auto" --
    segments when they fit, else binomial. ``memory_limit``: device bytes the
    gradient may hold in all (fields, tracks, tallies, checkpoints, adjoint
    buffers); default 90 % of the free memory. ``max_steps``: differentiate
    the first ``max_steps`` steps only (k_s of a run stopped there, from the
    tallies so far, as ``1 / f_t`` at its last step). ``slots``: the binomial
    schedule's state slots (default: as many as the memory limit allows, at
    most one per step). ``shape``: launch shape of the step kernels
    (``{"variant": "flat" | "stream", ..., "adjoint_variant": ...}``);
    default: the autotuned step shape (as :func:`run_simulation_b200`) and the
    library's choice of adjoint kernel for the grid.
    """

    def __init__(self, config, theta=None, checkpoint_every: int = 64, dtype: str = "float32", rng=None,
                 use_graphs: bool = False, max_steps: Optional[int] = None, memory_limit: Optional[float] = None,
                 schedule: str = "auto", slots: Optional[int] = None, shape: Optional[dict] = None):
        import torch

        if dtype not in ("float32", "float64"):
            raise ValueError(f"dtype must be 'float32' or 'float64', got {dtype!r}")
        if int(checkpoint_every) < 1:
            raise ValueError("checkpoint_every must be >= 1")
        if schedule not in SCHEDULES:
            raise ValueError(f"schedule must be one of {SCHEDULES}, got {schedule!r}")
        if max_steps is not None and int(max_steps) < 1:
            raise ValueError("max_steps must be >= 1")
        if slots is not None and int(slots) < 1:
            raise ValueError("slots must be >= 1")
        self.torch = torch
        self.config = config
        self.theta = base_parameters(config) if theta is None else np.asarray(theta, dtype=np.float64).copy()
        if self.theta.shape != (6,):
            raise ValueError("theta must hold (alpha, mu+, mu-, D+, D-, V)")
        self.K = int(checkpoint_every)
        self.dtype = dtype
        self.use_graphs = bool(use_graphs)
        self.rng = rng if rng is not None else np.random.default_rng(config.seed)
        self.max_steps = None if max_steps is None else int(max_steps)
        self.memory_limit = None if memory_limit is None else float(memory_limit)
        self.schedule = schedule
        self.slots_wanted = None if slots is None else int(slots)
        self.shape = None if shape is None else dict(shape)
        self.lib = N.load()
        self._eng = None
        self.ks = None
        self.plan = {}
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
        cfg = self.config
        t0 = perf_counter()
        total = int(cfg.total_time_steps)
        if self.max_steps is not None:
            total = min(total, self.max_steps)
        self.n_steps = total
        schedule = build_track_schedule(cfg, self.rng)[:total]
        n_tracks = int(schedule.sum())
        xs, ys = TrackSampler(self.rng, cfg.mid_xy, cfg.sampling_radius, cfg.no_xy).sample(n_tracks)
        self.offsets = np.zeros(total + 1, dtype=np.int64)
        np.cumsum(schedule, out=self.offsets[1:])
        eng = ChamberEngine(cfg, dtype=self.dtype, max_tracks=max(1, n_tracks), tally_steps=max(total, 1),
                            shape=self.shape)
        if self.shape is None:
            from .autotune import tune

            tune(eng, quick=True)  # on the fresh (zero) fields: leaves them zero
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
        n = int(g.no_xy)
        self.dslot = 2 * n * ((n + 3) // 4 * 4)  # one step's deposition pairs
        n_dep = int(np.count_nonzero(schedule))
        es = 4 if self.dtype == "float32" else 8
        state = 2 * field * es
        # beyond the engine: lambda (two states) now or later, and the schedule's own
        seg_need = (self.n_seg + self.K) * state + n_dep * self.dslot * es
        avail = self._available(2 * state)
        kind = self.schedule
        if kind == "auto":
            kind = "segments" if seg_need <= avail else "binomial"
        if kind == "segments" and seg_need > avail:
            raise MemoryError(f"the segment schedule needs {seg_need / 2**30:.2f} GiB of device memory for "
                              f"checkpoints, the segment buffer and the kept densities; {avail / 2**30:.2f} GiB "
                              f"is available (raise checkpoint_every, or use schedule='binomial')")
        self.kind = kind
        self.torch.cuda.synchronize(eng.device)
        t1 = perf_counter()
        if kind == "binomial":
            self._forward_binomial(total, state, avail)
        else:
            self._forward_segments(total, n_dep)
        self.torch.cuda.synchronize(eng.device)
        self.timings["forward_device_s"] = perf_counter() - t1
        tallies = eng.tallies(total)
        eng.check_status()
        # running float64 totals, as the solver and the reference form them
        self.injected = float(np.cumsum(tallies[:, 0])[-1])
        self.recombined = float(np.cumsum(tallies[:, 1])[-1])
        self.ks = 1.0 / collection_efficiency(tallies[:, 0], tallies[:, 1], total)[-1]
        self.timings["forward_s"] = perf_counter() - t0
        return self.ks

    def _available(self, extra: int) -> float:
        """Device bytes left for checkpoints once ``extra`` more are held."""
        torch = self.torch
        eng = self._eng
        free, _ = torch.cuda.mem_get_info(eng.device)
        avail = 0.9 * free - extra
        if self.memory_limit is not None:
            held = sum(t.numel() * t.element_size() for t in (*eng.pos, *eng.neg, *eng.dens, eng.counts, eng.tally,
                                                              eng.workspace, eng.xs, eng.ys))
            avail = min(avail, self.memory_limit - held - extra)
        return avail

    def _forward_binomial(self, total: int, state: int, avail: float) -> None:
        torch = self.torch
        eng = self._eng
        g = eng.grid
        n_slots = min(max(total, 1), int(avail // state))
        if self.slots_wanted is not None:
            if self.slots_wanted > n_slots and self.slots_wanted <= max(total, 1):
                raise MemoryError(f"{self.slots_wanted} state slots of {state / 2**30:.2f} GiB do not fit; "
                                  f"{max(avail, 0) / 2**30:.2f} GiB is available")
            n_slots = min(self.slots_wanted, max(total, 1))
        if n_slots < 1:
            raise MemoryError(f"the binomial schedule needs at least one {state / 2**30:.2f} GiB state slot; "
                              f"{max(avail, 0) / 2**30:.2f} GiB is available")
        recompute, levels = revolve_plan(total, n_slots)
        self.plan = {"schedule": "binomial", "slots": n_slots, "slot_bytes": state, "recompute_steps": recompute,
                     "stored_states": levels, "steps": total}
        self.n_slots = n_slots
        self.slots = torch.empty((2, n_slots, self.field), dtype=eng.pos[0].dtype, device=eng.device)
        off = np.ascontiguousarray(self.offsets)
        self._issue(lambda st: N.check(self.lib.pic_revolve_forward(
            ctypes.byref(g), eng.pos[0].data_ptr(), eng.neg[0].data_ptr(), eng.pos[1].data_ptr(),
            eng.neg[1].data_ptr(), total, eng.xs.data_ptr(), eng.ys.data_ptr(), off.ctypes.data_as(ctypes.c_void_p),
            eng.dens[0].data_ptr(), eng.counts.data_ptr(), eng.tally.data_ptr(), self.slots[0].data_ptr(),
            self.slots[1].data_ptr(), self.field, n_slots, eng.workspace.data_ptr(), eng.workspace.numel(), st),
            "pic_revolve_forward"))

    def _forward_segments(self, total: int, n_dep: int) -> None:
        torch = self.torch
        eng = self._eng
        g = eng.grid
        field = self.field
        dev, tdt = eng.device, eng.pos[0].dtype
        self.plan = {"schedule": "segments", "checkpoint_every": self.K, "checkpoints": self.n_seg,
                     "recompute_steps": total - self.n_seg, "steps": total}
        self.ckpt = torch.empty((2, max(self.n_seg, 1), field), dtype=tdt, device=dev)
        self.dens_keep = torch.empty((max(n_dep, 1), self.dslot), dtype=tdt, device=dev)
        off = np.ascontiguousarray(self.offsets)
        self._issue(lambda st: N.check(self.lib.pic_adjoint_forward(
            ctypes.byref(g), eng.pos[0].data_ptr(), eng.neg[0].data_ptr(), eng.pos[1].data_ptr(),
            eng.neg[1].data_ptr(), total, eng.xs.data_ptr(), eng.ys.data_ptr(), off.ctypes.data_as(ctypes.c_void_p),
            self.dens_keep.data_ptr(), eng.counts.data_ptr(), eng.tally.data_ptr(), self.ckpt[0].data_ptr(),
            self.ckpt[1].data_ptr(), self.K, field, eng.workspace.data_ptr(), eng.workspace.numel(), st),
            "pic_adjoint_forward"))

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
        total = self.n_steps
        K, field = self.K, self.field
        dev, tdt = eng.device, eng.pos[0].dtype
        lam = torch.zeros((2, 2, field), dtype=tdt, device=dev)  # [buffer][species]
        grad = torch.zeros(5, dtype=torch.float64, device=dev)
        awb = ctypes.c_int64()
        N.check(lib.pic_adjoint_workspace_bytes(ctypes.byref(g), ctypes.byref(awb)), "pic_adjoint_workspace_bytes")
        adj_ws = torch.zeros(int(awb.value), dtype=torch.uint8, device=dev)
        off = np.ascontiguousarray(self.offsets)
        torch.cuda.synchronize(dev)
        t1 = perf_counter()
        if self.kind == "binomial":
            # the forward's field pairs are free now: they are the working states
            self._issue(lambda st: N.check(lib.pic_revolve_backward(
                ctypes.byref(g), self.slots[0].data_ptr(), self.slots[1].data_ptr(), field, self.n_slots, total,
                eng.xs.data_ptr(), eng.ys.data_ptr(), off.ctypes.data_as(ctypes.c_void_p), eng.dens[0].data_ptr(),
                eng.pos[0].data_ptr(), eng.neg[0].data_ptr(), eng.pos[1].data_ptr(), eng.neg[1].data_ptr(),
                lam[0, 0].data_ptr(), lam[0, 1].data_ptr(), lam[1, 0].data_ptr(), lam[1, 1].data_ptr(),
                grad.data_ptr(), eng.workspace.data_ptr(), eng.workspace.numel(), adj_ws.data_ptr(), adj_ws.numel(),
                st), "pic_revolve_backward"))
            torch.cuda.synchronize(dev)
            self.timings["backward_device_s"] = perf_counter() - t1
            out = grad.cpu().numpy()
            eng.check_status()
            self._check_finite(out)
            self.timings["backward_s"] = perf_counter() - t0
            return out
        states = torch.empty((2, K, field), dtype=tdt, device=dev)
        self._issue(lambda st: N.check(lib.pic_adjoint_backward(
            ctypes.byref(g), self.ckpt[0].data_ptr(), self.ckpt[1].data_ptr(), field, total, K,
            off.ctypes.data_as(ctypes.c_void_p), self.dens_keep.data_ptr(), states[0].data_ptr(),
            states[1].data_ptr(), lam[0, 0].data_ptr(), lam[0, 1].data_ptr(), lam[1, 0].data_ptr(),
            lam[1, 1].data_ptr(), grad.data_ptr(), eng.workspace.data_ptr(),
            eng.workspace.numel(), adj_ws.data_ptr(), adj_ws.numel(), st), "pic_adjoint_backward"))
        torch.cuda.synchronize(dev)
        self.timings["backward_device_s"] = perf_counter() - t1
        out = grad.cpu().numpy()
        eng.check_status()
        self._check_finite(out)
        self.timings["backward_s"] = perf_counter() - t0
        return out

    @staticmethod
    def _check_finite(out) -> None:
        # a streaming adjoint step whose bounded wait expired poisons its
        # block's slot with NaN
        if not np.all(np.isfinite(out)):
            raise RuntimeError("the adjoint sweep gave a non-finite gradient (a kernel gave up on a bounded wait, "
                               "or the run overflowed); results are invalid")

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
        self.slots = None


def ks_and_gradient(config, theta=None, checkpoint_every: int = 64, dtype: str = "float32", rng=None,
                    use_graphs: bool = False, **schedule_kw):
    """``(k_s, dk_s/dtheta, timings)`` for theta = (alpha, mu+, mu-, D+, D-, V).
    ``schedule_kw``: ``max_steps``, ``memory_limit``, ``schedule``, ``slots``,
    ``shape`` of :class:`AdjointRun`; the timings include the schedule's
    ``plan``."""
    run = AdjointRun(config, theta, checkpoint_every, dtype, rng, use_graphs, **schedule_kw)
    try:
        ks = run.forward()
        grad = run.backward()
        return ks, grad, dict(run.timings, plan=dict(run.plan))
    finally:
        run.release()


def _autograd_function():
    import torch

    class KsFunction(torch.autograd.Function):
        """k_s(theta) with the adjoint as its backward. theta: float64 tensor
        (alpha, mu+, mu-, D+, D-, V)."""

        @staticmethod
        def forward(ctx, theta, config, checkpoint_every, dtype, schedule_kw):
            run = AdjointRun(config, theta.detach().cpu().numpy(), checkpoint_every, dtype, **schedule_kw)
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
            return torch.from_numpy(g) * grad_out.to(torch.float64).cpu(), None, None, None, None

    return KsFunction


_KS_FN = None


def ks_b200(theta, config, checkpoint_every: int = 64, dtype: str = "float32", **schedule_kw):
    """Differentiable k_s: ``ks_b200(theta, config)`` with ``theta`` a float64
    tensor (alpha, mu+, mu-, D+, D-, V) that may require grad; backward runs the
    adjoint sweep. The forward is the GB300 solve of ``config`` at ``theta``
    (fixed dt, step count and tracks). ``schedule_kw``: ``max_steps``,
    ``memory_limit``, ``schedule`` of :class:`AdjointRun`."""
    global _KS_FN
    if _KS_FN is None:
        _KS_FN = _autograd_function()
    return _KS_FN.apply(theta, config, int(checkpoint_every), dtype, dict(schedule_kw))


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


FITTABLE = PARAMS[:5]  # shared by a chamber's configurations; V is each configuration's own


def fit_parameters(configs, ks_target, names=("alpha",), start=None, iterations: int = 10,
                   checkpoint_every: int = 64, dtype: str = "float32", tol: float = 1e-7, damping: float = 1e-3):
    """Fit any of (alpha, mu+, mu-, D+, D-) to a k_s curve.

    ``configs`` (e.g. one chamber at several voltages) and ``ks_target``
    define ``L = sum_q (k_s(config_q; theta) - target_q)^2`` over parameters
    ``names`` shared by all configurations (the rest of each configuration's
    theta stays its own, alpha defaulting to the reference's). Each
    iteration runs every configuration forward and backward -- the adjoint
    gives the Jacobian ``J[q, p] = dk_s(config_q) / dtheta_p`` -- and takes a
    Levenberg-Marquardt step in relative coordinates (theta_p (1 + x_p), so
    that alpha ~ 1e-6 and mu ~ 1 are on one scale):
    ``(J'^T J' + damping diag(J'^T J')) x = -J'^T r``, J' = J theta. A step that
    raises the loss is retaken with ten times the damping.
    ``start``: {name: value} (default: the first configuration's own values).
    Returns ``(values, history)``: {name: fitted value}, [(values, loss)].
    """
    names = tuple(names)
    for nm in names:
        if nm not in FITTABLE:
            raise ValueError(f"cannot fit {nm!r}: choose from {FITTABLE}")
    idx = [PARAMS.index(nm) for nm in names]
    target = np.asarray(ks_target, dtype=np.float64)
    if len(target) != len(configs):
        raise ValueError("one target k_s per configuration")
    base = [base_parameters(c) for c in configs]
    values = np.array([base[0][i] for i in idx], dtype=np.float64)
    if start:
        for k, nm in enumerate(names):
            if nm in start:
                values[k] = float(start[nm])

    def evaluate(vals, with_grad):
        ks = np.zeros(len(configs))
        jac = np.zeros((len(configs), len(names)))
        for q, cfg in enumerate(configs):
            theta = base[q].copy()
            theta[idx] = vals
            if with_grad:
                k, grad, _ = ks_and_gradient(cfg, theta, checkpoint_every, dtype)
                jac[q] = grad[idx]
            else:
                run = AdjointRun(cfg, theta, checkpoint_every, dtype)
                try:
                    k = run.forward()
                finally:
                    run.release()
            ks[q] = k
        r = ks - target
        return float(np.sum(r * r)), r, jac

    loss, r, jac = evaluate(values, True)
    history = [(dict(zip(names, values.tolist())), loss)]
    lam = float(damping)
    for _ in range(int(iterations)):
        js = jac * values  # relative coordinates
        a = js.T @ js
        g = js.T @ r
        accepted = False
        for _retry in range(6):
            x = np.linalg.solve(a + lam * np.diag(np.diag(a)), -g)
            trial = values * (1.0 + x)
            if np.any(trial <= 0.0):
                lam *= 10.0
                continue
            t_loss, _, _ = evaluate(trial, False)
            if t_loss <= loss:
                accepted = True
                break
            lam *= 10.0
        if not accepted:
            break
        step = np.max(np.abs(x))
        values = trial
        lam = max(lam / 10.0, 1e-12)
        loss, r, jac = evaluate(values, True)
        history.append((dict(zip(names, values.tolist())), loss))
        if step <= tol:
            break
    return dict(zip(names, values.tolist())), history
