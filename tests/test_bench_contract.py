"""The benchmark's output contract, on the paths that need no GPU: the
reference arm (the FP64 CPU oracle) prints one JSON line with the keys the
line of the GB300 arm carries, ranks other than 0 print nothing and exit 0,
and fewer than 3 warm-up steps are refused."""

from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
KEYS = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def _bench(*argv, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *argv], cwd=ROOT, env=e, capture_output=True,
                          text=True, timeout=600)


def test_reference_arm_line():
    p = _bench("--impl", "reference", "--workload", "column_10um_r008", "--steps", "3", "--warmup", "3")
    assert p.returncode == 0, p.stderr
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["metric"] == "interior voxel-steps/s" and d["unit"] == "voxel-steps/s"
    assert d["value"] > 0 and d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["higher_is_better"] is True and d["vs_baseline"] is None
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"] and "24x24x206" in d["config"]["workload"]
    # the same config dict as the GB300 arm's line: the workload, its grid and
    # the tracks of the timed steps (the GB300 arm builds it with the same helper)
    c = d["config"]
    assert c["grid"] == [24, 24, 206] and c["interior_voxels"] == 22 * 22 * 204
    assert {"tracks_in_timed_steps", "l2", "parallelism"} <= set(c)
    sys.path.insert(0, str(ROOT))
    import bench

    assert set(c) == set(bench._workload_config(bench._config("column_10um_r008")[1], "x", 0, 1))


def test_reference_arm_other_ranks_silent():
    p = _bench("--impl", "reference", "--workload", "column_10um_r008", "--steps", "3", "--warmup", "3",
               env={"RANK": "1", "WORLD_SIZE": "2"})
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


def test_warmup_floor():
    p = _bench("--impl", "reference", "--workload", "column_10um_r008", "--steps", "3", "--warmup", "2")
    assert p.returncode != 0 and "--warmup must be >= 3" in p.stderr
