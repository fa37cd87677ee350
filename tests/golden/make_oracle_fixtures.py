"""Whole-run fixtures from the float64 oracle for the configurations too big to
run through the reference itself here: every configuration of the 64-grid
saturation sweep and the eight plain-method runs at scale (5 um voxels,
r = 0.05 cm, 208 x 208 x 406, 8.91 and 89.1 Gy/s, seeds 1-4).

The oracle (oracle/pic_oracle.c + oracle/oracle.py) is the float64 restatement
of the reference's batched driver (pulsed_ion_chamber/solver_numba_parallel.py:
526-723), pinned bit-for-bit at kernel level and to 1e-9 on whole runs against
fixtures the reference produced (tests/test_oracle.py). The configurations
come from this package's SimulationConfig mirror, pinned to the reference's
derived scalars (tests/test_config_mirror.py).

Per run it records k_s, the run's total injected and recombined charge, the
number of tracks and a SHA-256 of the track histogram (uint32, C order), so
the GPU tests compare a float32 run with float64 numbers without re-running
the oracle (about 10 minutes of 8 CPU cores for all 72 runs).

Usage::

    python tests/golden/make_oracle_fixtures.py            # both files
    python tests/golden/make_oracle_fixtures.py --only sweep
"""

from __future__ import annotations

import argparse
import hashlib
import json
import multiprocessing as mp
import os
import sys
import time
import warnings
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
PACKAGE = "iontracks-pulsedproton-python_gb300"
SWEEP_FILE = HERE / "oracle_sweep64.json"
SCALE_FILE = HERE / "oracle_column_5um_r05.json"


def _setup():
    for p in (str(ROOT), str(ROOT / "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)


def histogram_sha256(track_density_xy) -> str:
    import numpy as np

    return hashlib.sha256(np.ascontiguousarray(np.asarray(track_density_xy).astype(np.uint32)).tobytes()).hexdigest()


def _sweep_config(i):
    _setup()
    import importlib

    return importlib.import_module(PACKAGE).saturation_sweep_configs()[i]


def _scale_config(name, seed):
    _setup()
    from goldens import make_config

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return make_config(name, seed=seed)


def _job(args):
    kind, key = args
    _setup()
    from oracle import oracle

    oracle.set_threads(1)
    cfg = _sweep_config(key) if kind == "sweep" else _scale_config(*key)
    t0 = time.perf_counter()
    res = oracle.run(cfg, mode="batched", keep_fields=False)
    td = res["track_density_xy"]
    return kind, key, {
        "no_xy": int(cfg.no_xy), "nzb": int(cfg.no_z_with_buffer), "total_time_steps": int(cfg.total_time_steps),
        "seed": int(cfg.seed), "voltage_V": float(cfg.voltage_V), "dose_rate_Gy_s": float(cfg.dose_rate_Gy_s),
        "n_tracks": int(td.sum()), "track_sha256": histogram_sha256(td),
        "ks": float(res["ks"]), "injected_sum": float(res["injected"].sum()),
        "recombined_sum": float(res["recombined"].sum()), "oracle_wall_s": round(time.perf_counter() - t0, 2),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["sweep", "scale"])
    ap.add_argument("--workers", type=int, default=os.cpu_count())
    a = ap.parse_args()
    _setup()
    jobs = []
    if a.only in (None, "scale"):
        jobs += [("scale", (name, seed)) for name in ("column_5um_r05_d8p91", "column_5um_r05_d89p1")
                 for seed in (1, 2, 3, 4)]
    if a.only in (None, "sweep"):
        import importlib

        cfgs = importlib.import_module(PACKAGE).saturation_sweep_configs()
        # largest first, so that the pool's tail is short
        order = sorted(range(len(cfgs)), key=lambda i: -cfgs[i].no_xy ** 2 * cfgs[i].no_z_with_buffer
                       * cfgs[i].total_time_steps)
        jobs += [("sweep", i) for i in order]
    t0 = time.perf_counter()
    sweep, scale = {}, {}
    with mp.get_context("spawn").Pool(a.workers) as pool:
        for kind, key, rec in pool.imap_unordered(_job, jobs):
            if kind == "sweep":
                sweep[key] = rec
            else:
                scale[f"{key[0]}_seed{key[1]}"] = rec
            print(f"{kind} {key}: k_s {rec['ks']:.12f} ({rec['oracle_wall_s']} s)", flush=True)
    note = ("float64 oracle (C restatement of the reference's batched driver), one run per configuration; "
            "track_sha256 = SHA-256 of the uint32 track histogram in C order")
    if sweep:
        SWEEP_FILE.write_text(json.dumps({"note": note, "configs": [sweep[i] for i in sorted(sweep)]}, indent=1))
    if scale:
        SCALE_FILE.write_text(json.dumps({"note": note, "runs": scale}, indent=1))
    print(f"done in {time.perf_counter() - t0:.0f} s")


if __name__ == "__main__":
    main()
