"""Benchmark of the GB300 hot path: fused Lax-Wendroff step + track deposition.

Workload (default): the 5 um full-electrode chamber -- 56.2 MeV/u protons,
300 V over 0.2 cm, 540 us pulses at 50 Hz, 8.91 Gy/s, sampled radius 0.265 cm,
seed 1: a 1068 x 1068 x 406 grid (463 M voxels, 7.4 GB of float32 fields
double-buffered), 25 057 919 tracks per pulse over 2 948 pulse steps. A timed
step is one time step inside the first pulse: the step's ~8 500 tracks
deposited and the whole grid swept.

Metric: interior voxel-steps per second (interior = (no_xy-2)^2 (nzb-2), the
reference's unit, profiling/bench_gh200.py:191). The fields (7.4 GB) are far
larger than the 129 MB L2, so every step streams from HBM; no L2 flush is
needed between steps.

Lines printed (rank 0, one JSON object each):
  --impl gb300 (default): value (device-resident inputs), e2e through
    run_simulation_b200 (host sampling, H2D of tracks, D2H of tallies), the
    step kernel's roofline against the measured HBM copy bandwidth, the FP64
    CPU oracle timed on a bounded sample as cpu_baseline, SM clocks sampled
    during the timed region.
  --impl reference: the FP64 CPU oracle (the reference's algorithm restated
    in C with OpenMP) on the same workload, on all host cores.

Multi-GPU (torchrun, one rank per GPU): independent replicas of the workload,
no collective on the data path; value = all ranks' voxel-steps / max time.
"""

from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
PACKAGE = "iontracks-pulsedproton-python_gb300"
BYTES_PER_VOXEL_STEP = 16  # float32: read n+ and n-, write both next fields

BEAM = dict(E_MeV_u=56.2, voltage_V=300.0, electrode_gap_cm=0.2, pulse_duration_s=540e-6,
            repetition_rate_hz=50.0, dose_rate_Gy_s=8.91)
WORKLOADS = {
    # name: (description, SimulationConfig kwargs)
    "full_electrode_5um": ("5 um full electrode, r=0.265 cm, 1068x1068x406, 10 pulses, seed 1",
                           dict(BEAM, grid_size_um=5.0, sampled_radius_cm=0.265, n_pulses=10, seed=1,
                                max_voxels=2e9)),
    "column_5um_r15": ("5 um column, r=0.15 cm, 608x608x406, 8.91 Gy/s, seed 1 (profiling size: 2.4 GB of fields)",
                       dict(BEAM, grid_size_um=5.0, sampled_radius_cm=0.15, seed=1, max_voxels=2e9)),
    "column_5um_r05": ("5 um column, r=0.05 cm, 208x208x406, 8.91 Gy/s, seed 1",
                       dict(BEAM, grid_size_um=5.0, sampled_radius_cm=0.05, seed=1, max_voxels=2e9)),
    "column_10um_r008": ("10 um column, r=0.008 cm, 24x24x206, seed 1",
                         dict(BEAM, grid_size_um=10.0, sampled_radius_cm=0.008, seed=1)),
}


def _pkg():
    return importlib.import_module(PACKAGE)


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return world, rank


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_bytes(workload):
    """dram bytes per step-kernel launch from the committed ncu summary."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    return d.get(workload, {}).get("dram_bytes_per_launch")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.gpu = gpu_index
        # raw samples (the JSON line carries their summary); PIC_CLOCKS_DIR keeps them
        self.path = Path(os.environ.get("PIC_CLOCKS_DIR", tempfile.gettempdir())) / f"pic_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def _shape(args):
    shape = {"variant": args.variant}
    for key in ("tile_rows", "planes_per_item", "stages", "consumer_warps", "ctas_per_sm"):
        v = getattr(args, key)
        if v:
            shape[key] = v
    return shape


def _config(workload):
    desc, kw = WORKLOADS[workload]
    return desc, _pkg().SimulationConfig(**kw)


def _interior(cfg):
    return (cfg.no_xy - 2) ** 2 * (cfg.no_z_with_buffer - 2)


def _workload_config(cfg, desc, timed_tracks, world):
    """The line's ``config``: the same dict on both arms' lines."""
    read_mb = 2 * int(cfg.no_xy) ** 2 * ((int(cfg.no_z_with_buffer) + 7) // 8 * 8) * 4 / 1e6
    l2_note = (f"each step reads {read_mb:.0f} MB of float32 fields, more than the 129 MB L2: inputs larger than "
               "L2, no flush needed" if read_mb > 129 else
               f"each step reads {read_mb:.0f} MB of float32 fields, less than the 129 MB L2: L2-resident between "
               "steps (no flush; an upper bound, not an HBM measurement)")
    return {"workload": desc, "grid": [int(cfg.no_xy), int(cfg.no_xy), int(cfg.no_z_with_buffer)],
            "interior_voxels": int(_interior(cfg)), "tracks_in_timed_steps": int(timed_tracks), "l2": l2_note,
            "parallelism": f"replicas x{world}"}


def cpu_sample(cfg, steps=3, warmup=2, threads=None):
    """FP64 oracle (the reference algorithm in C/OpenMP, batched deposition)
    on pulse steps of the workload, on all host cores. The first ``warmup``
    steps (page first-touch of the 15 GB of float64 fields) are run but not
    timed; returns (voxel-steps/s, cores, timed seconds)."""
    from oracle import oracle

    cores = threads or oracle.cores_used()
    oracle.set_threads(cores)
    res = oracle.run(cfg, mode="batched", max_steps=warmup + steps, keep_fields=False)
    timed = float(res["step_wall_s"][warmup:].sum())
    return _interior(cfg) * steps / timed, cores, timed


def run_reference(args):
    world, rank = _dist()
    if rank != 0:
        return 0
    desc, cfg = _config(args.workload)
    # K timed steps after W untimed ones, bounded (about 0.2 s per full-electrode
    # step on 16 cores) so that the run ends within a few minutes
    steps = max(1, min(args.steps, args.ref_max_steps))
    warmup = max(1, min(args.warmup, 5))
    v, cores, wall = cpu_sample(cfg, steps=steps, warmup=warmup)
    sched = _pkg().build_track_schedule(cfg, np.random.default_rng(cfg.seed))
    line = {
        "impl": "reference", "metric": "interior voxel-steps/s", "value": v, "unit": "voxel-steps/s",
        "n_gpus": world, "steps": steps, "warmup": warmup, "ms_per_step": wall / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": _workload_config(cfg, desc, sched[warmup:warmup + steps].sum(), world),
        "cpu_baseline": {"value": v, "unit": "voxel-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{steps} pulse steps of the workload (deposition + sweep) after {warmup} untimed, "
                                   f"FP64 oracle (C/OpenMP restatement of the reference kernels), {wall:.1f} s timed"},
        "e2e": {"value": v, "unit": "voxel-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _oracle_sweep_fixture():
    """Per-configuration float64 oracle results of the 64-grid sweep
    (tests/golden/oracle_sweep64.json, made by tests/golden/make_oracle_fixtures.py),
    or None when the file is absent."""
    p = ROOT / "tests" / "golden" / "oracle_sweep64.json"
    return json.loads(p.read_text())["configs"] if p.exists() else None


def _max_abs_diff(a, b):
    """max |a - b| over pairs, where two non-finite values (a configuration the
    reference's scheme does not survive: its k_s is NaN) count as agreeing and
    one non-finite value against a finite one counts as infinite."""
    worst = 0.0
    for x, y in zip(a, b):
        fx, fy = np.isfinite(x), np.isfinite(y)
        if not fx and not fy:
            continue
        worst = max(worst, abs(x - y) if fx and fy else float("inf"))
    return worst


def sweep_measure(n_configs=64, batched_only=False, rank=0, world=1, variant="auto", warmup=3):
    """The 64-configuration saturation sweep: one batched run against the same
    configurations solved one after another with the plain solver on the
    same GPU, both end to end (host track sampling, uploads, all steps,
    read-back). Returns this rank's numbers (its share of the sweep)."""
    import torch

    pkg = _pkg()
    every = pkg.saturation_sweep_configs()[: max(1, n_configs)]
    idx = list(range(len(every)))[rank::world]  # the sweep's configurations shared out over the GPUs
    cfgs = [every[i] for i in idx]
    vox = sum(_interior(c) * int(c.total_time_steps) for c in cfgs)
    # warm-up (``warmup`` rounds): load the kernels, pay first-use costs
    # outside the timing
    for _ in range(max(1, warmup)):
        pkg.run_batched_b200(cfgs[:2], variant=variant)
        pkg.run_simulation_b200(cfgs[0], progress=False, return_fields=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch = pkg.run_batched_b200(cfgs, variant=variant)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    plain, t_plain, dks = None, None, None
    if not batched_only:
        t0 = time.perf_counter()
        plain = [pkg.run_simulation_b200(c, progress=False, return_fields=False) for c in cfgs]
        torch.cuda.synchronize()
        t_plain = time.perf_counter() - t0
        dks = _max_abs_diff([b.ks for b in batch], [p.ks for p in plain])
    fx = _oracle_sweep_fixture()
    dks_oracle = None
    if fx is not None and len(fx) == 64:
        dks_oracle = _max_abs_diff([b.ks for b in batch], [fx[i]["ks"] for i in idx])
    return {"configs": len(cfgs), "interior_voxel_steps": vox, "batched_s": t_batch, "sequential_plain_s": t_plain,
            "speedup_vs_sequential": None if t_plain is None else t_plain / t_batch,
            "max_abs_dks_batched_vs_plain": dks, "max_abs_dks_batched_vs_fp64_oracle": dks_oracle,
            "n_total": len(every)}


def run_sweep(args):
    """--workload saturation_sweep: the sweep alone, shared out over ranks."""
    import torch
    import torch.distributed as dist

    world, rank = _dist()
    if world > 1:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    replicas = importlib.import_module(PACKAGE + ".replicas")
    m = sweep_measure(args.sweep_configs, args.batched_only, rank, world, args.sweep_variant, args.warmup)
    value = replicas.whole_job_rate(m["interior_voxel_steps"], m["batched_s"])
    t_batch = replicas.max_over_ranks(m["batched_s"])
    vox = replicas.sum_over_ranks(m["interior_voxel_steps"])
    t_plain, dks = m["sequential_plain_s"], m["max_abs_dks_batched_vs_plain"]
    if t_plain is not None:
        t_plain = replicas.max_over_ranks(t_plain)
        dks = replicas.max_over_ranks(dks)
    dko = m["max_abs_dks_batched_vs_fp64_oracle"]
    if dko is not None:
        dko = replicas.max_over_ranks(dko)
    if world > 1:
        dist.destroy_process_group()
    if rank == 0:
        line = {
            "metric": "interior voxel-steps/s, 64-config saturation sweep", "value": value,
            "unit": "voxel-steps/s", "n_gpus": world, "steps": int(max(c.total_time_steps for c in
                                                                        _pkg().saturation_sweep_configs())),
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": SWEEP_DESC.format(n=m["n_total"]), "interior_voxel_steps": vox,
                       "warmup_unit": "a two-configuration batched run and one plain solve"},
            "batched_s": t_batch, "sequential_plain_s": t_plain,
            "speedup_vs_sequential": None if t_plain is None else t_plain / t_batch,
            "max_abs_dks_batched_vs_plain": dks, "max_abs_dks_batched_vs_fp64_oracle": dko,
        }
        print(json.dumps(line), flush=True)
    return 0


SWEEP_DESC = ("saturation sweep: {n} of 64 configs, 25-400 V log-spaced, gaps 0.1/0.2/0.3 cm, 1-100 Gy/s, "
              "100-1000 us pulses, 5/10 um voxels, r 0.008-0.03 cm, seeds 1-64")


ADJOINT_CFG = dict(BEAM, grid_size_um=10.0, sampled_radius_cm=0.02, seed=1)


def adjoint_measure(warmup=3, reps=3):
    """A full gradient dk_s/d(alpha, mu+, mu-, D+, D-, V) (checkpointed
    forward + reverse sweep, checkpoints every 64 steps, float32) against one
    plain forward solve of the same chamber, both end to end through the
    package API, on the 10 um, r = 0.02 cm column at 300 V (medians)."""
    import torch

    pkg = _pkg()
    adj = importlib.import_module(PACKAGE + ".adjoint")
    cfg = pkg.SimulationConfig(**ADJOINT_CFG)
    for _ in range(max(1, warmup)):
        pkg.run_simulation_b200(cfg, progress=False, return_fields=False)
        adj.ks_and_gradient(cfg, checkpoint_every=64)
    plain, full, parts = [], [], []
    for _ in range(max(1, reps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = pkg.run_simulation_b200(cfg, progress=False, return_fields=False)
        torch.cuda.synchronize()
        plain.append(time.perf_counter() - t)
        t = time.perf_counter()
        ks, grad, tm = adj.ks_and_gradient(cfg, checkpoint_every=64)
        torch.cuda.synchronize()
        full.append(time.perf_counter() - t)
        parts.append(tm)
    p, f = statistics.median(plain), statistics.median(full)
    return {"ratio": f / p, "plain_forward_s": p, "adjoint_total_s": f,
            "adjoint_forward_s": statistics.median(t["forward_s"] for t in parts),
            "adjoint_backward_s": statistics.median(t["backward_s"] for t in parts),
            "ks": ks, "ks_plain": res.ks, "dks_dtheta": list(grad), "parameters": list(adj.PARAMS),
            "workload": f"10 um column, r 0.02 cm, {cfg.no_xy}x{cfg.no_xy}x{cfg.no_z_with_buffer}, "
                        f"{cfg.total_time_steps} steps, 300 V / 0.2 cm, 8.91 Gy/s, seed 1; checkpoints every 64 "
                        "steps"}


def run_adjoint(args):
    """--workload adjoint: the gradient-over-forward ratio alone."""
    world, rank = _dist()
    m = adjoint_measure(args.warmup, args.steps)
    if rank == 0:
        line = {
            "metric": "full adjoint gradient wall time / one plain forward solve", "value": m["ratio"], "unit": "x",
            "n_gpus": world, "steps": max(1, args.steps), "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": m.pop("workload"), "parameters": m.pop("parameters")},
        }
        line.update({k: v for k, v in m.items() if k != "ratio"})
        print(json.dumps(line), flush=True)
    return 0


def run_adjoint_full(args):
    """Forward + adjoint of the 5 um full electrode (1068 x 1068 x 406) under
    a device-memory limit (default 180 GB): the binomial schedule with as many
    float32 state slots as fit, over the first --adjoint-steps steps (the
    whole 985 801-step run takes hours: its cost is projected from the
    measured per-step times and the schedule's exact recomputation count).
    One plain forward solve of the same steps is timed beside it."""
    import torch

    world, rank = _dist()
    pkg = _pkg()
    adj = importlib.import_module(PACKAGE + ".adjoint")
    desc, cfg = _config(args.adjoint_workload)
    n = int(args.adjoint_steps)
    limit = float(args.memory_limit_gb) * 1e9
    shape = None if args.variant == "auto" else {"variant": args.variant}
    for _ in range(max(1, args.warmup)):
        adj.ks_and_gradient(cfg, max_steps=min(n, 8), memory_limit=limit, shape=shape)
        torch.cuda.empty_cache()
    runs, plain = [], []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = pkg.run_simulation_b200(cfg, progress=False, return_fields=False, max_steps=n, shape=shape)
        torch.cuda.synchronize()
        plain.append(time.perf_counter() - t)
        del res
        torch.cuda.empty_cache()
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        t = time.perf_counter()
        ks, grad, tm = adj.ks_and_gradient(cfg, max_steps=n, memory_limit=limit, shape=shape)
        torch.cuda.synchronize()
        tm["total_s"] = time.perf_counter() - t
        tm["peak_bytes"] = torch.cuda.max_memory_allocated() - base
        runs.append((ks, grad, tm))
        torch.cuda.empty_cache()
    med = lambda key: statistics.median(r[2][key] for r in runs)  # noqa: E731
    plan = runs[-1][2]["plan"]
    t_step = med("forward_device_s") / n
    t_adj = (med("backward_device_s") - plan["recompute_steps"] * t_step) / n
    full = int(cfg.total_time_steps)
    rec_full, _ = adj.revolve_plan(full, plan["slots"])
    proj = full * t_step + rec_full * t_step + full * t_adj
    if rank == 0:
        ks, grad, _ = runs[-1]
        print(json.dumps({
            "metric": "forward + adjoint wall time / one plain forward solve (same steps)",
            "value": statistics.median(r[2]["total_s"] for r in runs) / statistics.median(plain), "unit": "x",
            "n_gpus": world, "steps": len(runs), "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc + f"; first {n} steps; device memory limit {limit / 1e9:.0f} GB",
                       "parameters": list(adj.PARAMS)},
            "plan": plan, "peak_device_bytes": max(r[2]["peak_bytes"] for r in runs),
            "plain_forward_s": statistics.median(plain), "adjoint_total_s": med("total_s"),
            "forward_device_s": med("forward_device_s"), "backward_device_s": med("backward_device_s"),
            "step_ms": 1e3 * t_step, "adjoint_step_ms": 1e3 * t_adj,
            "full_run": {"steps": full, "slots": plan["slots"], "recompute_steps": rec_full,
                         "projected_s": proj, "projected_vs_forward": proj / (full * t_step)},
            "ks": ks, "dks_dtheta": list(grad),
        }), flush=True)
    return 0


def run_full_electrode_run(args):
    """The whole 10-pulse run of the 5 um full electrode (seed 1, 985 801
    steps, 97 % of them without tracks) through run_simulation_b200, once,
    end to end: its k_s and tallies, the wall time and the mean time per
    step over the run, with the pulse and idle step counts beside them."""
    import torch

    world, rank = _dist()
    pkg = _pkg()
    desc, cfg = _config("full_electrode_5um")
    total = int(cfg.total_time_steps)
    pulse = int(cfg.pulse_time_steps) * int(cfg.n_pulses)
    steps = total if args.run_steps <= 0 else min(total, int(args.run_steps))
    # warm-up: load the library, resolve the launch shape (8 steps)
    pkg.run_simulation_b200(cfg, progress=False, return_fields=False, max_steps=8)
    torch.cuda.synchronize()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t0 = time.perf_counter()
        res = pkg.run_simulation_b200(cfg, progress=False, return_fields=False,
                                      max_steps=None if steps == total else steps)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    vox = _interior(cfg)
    if rank == 0:
        print(json.dumps({
            "metric": "interior voxel-steps/s, whole 10-pulse run", "value": vox * steps / wall,
            "unit": "voxel-steps/s", "n_gpus": world, "steps": steps, "warmup": 8,
            "ms_per_step": 1e3 * wall / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": _workload_config(cfg, desc + "; the whole run", 0, world),
            "ks": res.ks, "wall_s": wall, "total_steps": total, "pulse_steps": pulse, "idle_steps": total - pulse,
            "injected": float(res.injected_positive.sum()), "recombined": float(res.recombination.sum()),
            "tracks": int(res.track_density_xy.sum()), "clocks": clk.summary(),
        }), flush=True)
    return 0


def run_gb300(args):
    import torch
    import torch.distributed as dist

    world, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    pkg = _pkg()
    eng_mod = importlib.import_module(PACKAGE + ".engine")
    native = importlib.import_module(PACKAGE + "._native")
    desc, cfg = _config(args.workload)
    replicas = importlib.import_module(PACKAGE + ".replicas")
    rng = np.random.default_rng(replicas.replica_seed(cfg.seed, rank))
    sched = pkg.build_track_schedule(cfg, rng)
    n_steps = args.warmup + args.steps
    if n_steps > cfg.pulse_time_steps:
        raise SystemExit("warmup + steps must fit in the first pulse")
    counts = sched[:n_steps]
    xs, ys = pkg.TrackSampler(rng, cfg.mid_xy, cfg.sampling_radius, cfg.no_xy).sample(int(counts.sum()))
    shape = _shape(args)
    eng = eng_mod.ChamberEngine(cfg, dtype=args.dtype, max_tracks=len(xs), tally_steps=n_steps, shape=shape)
    tuned = None
    if args.variant == "auto" and not args.no_tune:
        at = importlib.import_module(PACKAGE + ".autotune")
        tuned = at.tune(eng, quick=True, reps=5)
        shape = dict(tuned["shape"])
    resolved = eng_mod.resolve_shape(eng.grid)
    eng.upload_tracks(xs, ys, non_blocking=False)
    off = np.zeros(n_steps + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    stream = torch.cuda.current_stream()

    # warm-up steps, then K timed steps
    eng.run_segment(off[: args.warmup + 1])
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    lib = native.load()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        launches0 = lib.pic_kernel_launches()
        t_start.record(stream)
        eng.run_segment(off[args.warmup:] - off[args.warmup], track_base=int(off[args.warmup]))
        t_end.record(stream)
        torch.cuda.synchronize()
        launches = lib.pic_kernel_launches() - launches0  # the library's own count of its kernel launches
    ms = t_start.elapsed_time(t_end)
    vox = _interior(cfg)
    # all ranks' voxel-steps over the slowest rank's time
    value = replicas.whole_job_rate(vox * args.steps, ms / 1e3)
    ms = replicas.max_over_ranks(ms)
    if world > 1:
        dist.barrier()

    # dominant kernel: the fused step, one launch per step, event-timed on
    # its own stream, with this step's deposition density applied
    import ctypes

    g = eng.grid
    reps = max(5, min(50, args.steps))
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    cur = eng.parity
    for r in range(reps):
        evs[r][0].record(stream)
        rc = lib.pic_step(ctypes.byref(g), eng.pos[cur].data_ptr(), eng.neg[cur].data_ptr(),
                          eng.pos[cur ^ 1].data_ptr(), eng.neg[cur ^ 1].data_ptr(), eng.dens[0].data_ptr(), None,
                          eng.tally[0].data_ptr(), eng.workspace.data_ptr(), eng.workspace.numel(),
                          stream.cuda_stream)
        native.check(rc, "pic_step")
        evs[r][1].record(stream)
        cur ^= 1
    torch.cuda.synchronize()
    step_ms = statistics.median(a.elapsed_time(b) for a, b in evs)
    at = importlib.import_module(PACKAGE + ".autotune")
    idle_ms = at.time_shape(eng, resolved, reps=reps, with_deposition=False)
    peak, peak_kind = _peaks()
    achieved = BYTES_PER_VOXEL_STEP * vox / (step_ms / 1e3) / 1e9
    idle_achieved = BYTES_PER_VOXEL_STEP * vox / (idle_ms / 1e3) / 1e9
    traffic = _traffic_bytes(args.workload)
    eng.close()
    del eng
    torch.cuda.empty_cache()

    # end to end through the public solver call (the pulse's schedule and
    # track sampling on the host, H2D of tracks, D2H of tallies): by default
    # the whole first pulse (every step depositing), over which the pulse's
    # one-time host work is spread as it is in a run
    e2e = None
    e2e_steps = int(args.e2e_steps) if args.e2e_steps > 0 else int(cfg.pulse_time_steps)
    if rank == 0 or world > 1:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = pkg.run_simulation_b200(cfg, rng=np.random.default_rng(replicas.replica_seed(cfg.seed, rank)),
                                      progress=False, max_steps=e2e_steps, return_fields=False, shape=shape)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        tracks = float(sched[:e2e_steps].sum())  # the whole run's schedule
        e2e_rate = replicas.whole_job_rate(vox * res.steps_completed, e2e_s)
        e2e_s = replicas.max_over_ranks(e2e_s)
        e2e = {"value": e2e_rate, "unit": "voxel-steps/s",
               "h2d_bytes_per_step": 16.0 * tracks / e2e_steps, "d2h_bytes_per_step": 32,
               "steps": int(res.steps_completed), "wall_s": e2e_s,
               "includes": "schedule + track sampling on the host, H2D of tracks, all steps, D2H of tallies"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, cores, wall = cpu_sample(cfg, steps=args.cpu_steps)
        cpu = {"value": v, "unit": "voxel-steps/s", "cores": cores, "kind": "port",
               "sample": f"{args.cpu_steps} pulse steps of the same workload after 2 untimed (page first-touch), "
                         f"FP64 oracle, {wall:.1f} s timed"}

    # the benchmark's other two ratios, on the same line: the 64-grid sweep
    # (batched vs the same solves one after another) and the 10 um column's
    # gradient (full adjoint vs one forward solve), each end to end through
    # the package's API on this GPU
    sweep = adjoint = None
    if not args.no_extras:
        if world == 1:
            torch.cuda.empty_cache()
            sweep = sweep_measure()
            sweep["workload"] = SWEEP_DESC.format(n=sweep.pop("n_total"))
            adjoint = adjoint_measure(warmup=3, reps=5)
        else:
            sweep = adjoint = {"skipped": "measured by the single-GPU run only"}

    if rank == 0:
        line = {
            "metric": "interior voxel-steps/s", "value": value, "unit": "voxel-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.dtype == "float32" else "f64",
            "data": "synthetic",
            "config": _workload_config(cfg, desc, counts[args.warmup:].sum(), world),
            "launch_shape": resolved,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "kernel": "stream_step_kernel" if resolved["variant"] == "stream" else "step_kernel",
                         "kernel_ms": step_ms,
                         "algorithmic_bytes_per_launch": BYTES_PER_VOXEL_STEP * vox,
                         "idle_step": {"kernel_ms": idle_ms, "achieved": idle_achieved, "frac": idle_achieved / peak,
                                       "note": "the same kernel on a step without deposition (97 % of the "
                                               "steps of the 10-pulse run)"}},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "sweep": sweep,
            "adjoint": adjoint,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["saturation_sweep", "adjoint", "adjoint_full_electrode",
                                                               "full_electrode_run"], default="full_electrode_5um")
    ap.add_argument("--run-steps", dest="run_steps", type=int, default=0,
                    help="full_electrode_run: stop after this many steps (0: the whole run)")
    ap.add_argument("--dtype", choices=["float32", "float64"], default="float32")
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="steps of the end-to-end run (0: the whole first pulse)")
    ap.add_argument("--cpu-steps", dest="cpu_steps", type=int, default=50,
                    help="pulse steps of the float64 oracle timed for the cpu_baseline (~0.2 s each at full size)")
    ap.add_argument("--ref-max-steps", dest="ref_max_steps", type=int, default=300,
                    help="--impl reference: at most this many timed steps")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", dest="no_extras", action="store_true",
                    help="skip the sweep and gradient measurements embedded in the default line")
    ap.add_argument("--batched-only", dest="batched_only", action="store_true",
                    help="saturation_sweep: time the batched run only (profiling)")
    ap.add_argument("--sweep-variant", dest="sweep_variant", choices=["auto", "flat", "stream", "mixed"], default="auto",
                    help="saturation_sweep: the batched step kernel (run_batched_b200's variant)")
    ap.add_argument("--sweep-configs", dest="sweep_configs", type=int, default=64,
                    help="saturation_sweep: run the first N of the 64 configurations (profiling-size cases)")
    ap.add_argument("--adjoint-steps", dest="adjoint_steps", type=int, default=1000,
                    help="adjoint_full_electrode: steps of the run differentiated")
    ap.add_argument("--adjoint-workload", dest="adjoint_workload", choices=sorted(WORKLOADS),
                    default="full_electrode_5um", help="adjoint_full_electrode: the chamber (profiling-size cases)")
    ap.add_argument("--memory-limit-gb", dest="memory_limit_gb", type=float, default=180.0,
                    help="adjoint_full_electrode: device memory the gradient may hold")
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-shape autotuner")
    ap.add_argument("--variant", choices=["auto", "flat", "stream"], default="auto")
    ap.add_argument("--tile-rows", dest="tile_rows", type=int, default=0)
    ap.add_argument("--planes-per-item", dest="planes_per_item", type=int, default=0)
    ap.add_argument("--stages", type=int, default=0)
    ap.add_argument("--consumer-warps", dest="consumer_warps", type=int, default=0)
    ap.add_argument("--ctas-per-sm", dest="ctas_per_sm", type=int, default=0)
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "saturation_sweep":
        return run_sweep(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "full_electrode_run":
        return run_full_electrode_run(args)
    if args.workload == "adjoint_full_electrode":
        return run_adjoint_full(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
