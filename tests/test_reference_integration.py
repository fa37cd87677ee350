"""The reference's own command line and benchmark driving the b200 backend,
and its own run-record writers consuming a b200 Result (CPU, in a container
that has the reference checkout; skipped elsewhere).

* The shipped patch (iontracks-pulsedproton-python_gb300/integration/
  reference_b200_backend.patch) applies cleanly to a copy of the reference and
  adds ``--backend b200`` to examples/ifj_aic144/run_markus_2mm.py, a ``b200``
  backend to profiling/bench_gpu.py and ``run_simulation_b200`` to the
  package's exports. Run without a GPU, the patched CLI reaches this
  package's solver, which refuses loudly (no CPU fallback).
* ``tests/golden/b200_result_aic144_dev.npz`` holds the Result of
  ``run_simulation_b200`` on the CLI's dev tier, recorded on a GB300 by
  tests/golden/make_b200_record.py. The reference's writers
  (pulsed_ion_chamber/output.py:63-92, :124-195) write it and read it back;
  its CSV matches the one they write from the reference's own run of the
  same configuration (tests/golden/run_aic144_dev.npz) to 1e-5 relative.
"""

from __future__ import annotations

import importlib.util
import os
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
STUBS = GOLDEN / "_stubs"
PATCH = ROOT / "iontracks-pulsedproton-python_gb300" / "integration" / "reference_b200_backend.patch"


def _reference_root() -> Path:
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return Path(mod.REFERENCE_ROOT)


REF = _reference_root()
needs_reference = pytest.mark.skipif(not (REF / "pulsed_ion_chamber").is_dir(),
                                     reason="the reference checkout is not present here")


@pytest.fixture
def patched_reference(tmp_path):
    dst = tmp_path / "ref"
    shutil.copytree(REF, dst, ignore=shutil.ignore_patterns(".git", "__pycache__", "*.pyc"))
    p = subprocess.run(["patch", "-p1", "--forward", "-i", str(PATCH)], cwd=dst, capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    return dst


@needs_reference
def test_backend_patch_applies_and_adds_the_backend(patched_reference):
    cli = (patched_reference / "examples" / "ifj_aic144" / "run_markus_2mm.py").read_text()
    assert '"b200"' in cli and "run_simulation_b200(config, progress=True)" in cli
    bench = (patched_reference / "profiling" / "bench_gpu.py").read_text()
    assert 'backend == "b200"' in bench
    init = (patched_reference / "pulsed_ion_chamber" / "__init__.py").read_text()
    assert '"run_simulation_b200"' in init


@needs_reference
def test_patched_cli_dispatches_to_the_b200_solver(patched_reference):
    """`run_markus_2mm.py dev --backend b200` runs the reference's CLI (numba
    and pandas replaced by the test stand-ins) up to this package's solver:
    the header names solver_b200 and, without a GPU, the solver's own
    refusal ends the run."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("checks the dispatch on a machine without a GPU")
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([str(STUBS), str(patched_reference), str(ROOT)])
    p = subprocess.run([sys.executable, "examples/ifj_aic144/run_markus_2mm.py", "dev", "--backend", "b200"],
                       cwd=patched_reference, env=env, capture_output=True, text=True, timeout=300)
    assert "Backend               : solver_b200, GPU" in p.stdout, p.stdout + p.stderr
    assert p.returncode != 0 and "run_simulation_b200 needs a CUDA device" in p.stderr


def _reference_output_module():
    for p in (str(STUBS), str(REF)):
        if p not in sys.path:
            sys.path.insert(0, p)
    import pulsed_ion_chamber.output as output

    return output


def _namespace(config, **arrays):
    from types import SimpleNamespace

    return SimpleNamespace(config=config, **arrays)


@needs_reference
def test_reference_writers_consume_a_b200_result(tmp_path):
    fx = GOLDEN / "b200_result_aic144_dev.npz"
    if not fx.exists():
        pytest.skip("no recorded b200 Result (tests/golden/make_b200_record.py on a GB300)")
    from goldens import make_config

    output = _reference_output_module()
    cfg = make_config("aic144_dev")
    z = np.load(fx)
    b200 = _namespace(cfg, time_s=z["time_s"], f_t=z["f_t"], ks=float(z["ks"]), n_positive=z["n_positive"],
                      n_negative=z["n_negative"], injected_positive=z["injected_positive"],
                      injected_negative=z["injected_negative"], recombination=z["recombination"],
                      track_density_xy=z["track_density_xy"])
    r = np.load(GOLDEN / "run_aic144_dev.npz")  # the reference's own run (run_simulation_numba)
    numba = _namespace(cfg, time_s=r["time_s"], f_t=r["f_t"], ks=float(r["ks"]), n_positive=r["n_positive"],
                       n_negative=r["n_negative"], injected_positive=r["injected"], injected_negative=r["injected"],
                       recombination=r["recombination"], track_density_xy=r["track_density_xy"])
    for name, res in (("b200", b200), ("numba", numba)):
        paths = output.save_run_record(res, tmp_path / name)
        assert set(paths) == {"csv", "track_density", "meta"}
    got = output.load_run_record(tmp_path / "b200")
    want = output.load_run_record(tmp_path / "numba")
    # the record round-trips the b200 Result (%.12e in the CSV)
    table = output.collected_charge_table(b200)
    for col in output.COLLECTED_CHARGE_COLUMNS:
        np.testing.assert_allclose(got.table[col], table[col], rtol=1e-11, atol=0)
    # and matches the reference's record of the same configuration
    np.testing.assert_array_equal(got.track_density_xy, want.track_density_xy)
    np.testing.assert_array_equal(got.table["time"], want.table["time"])
    for col in output.COLLECTED_CHARGE_COLUMNS[1:]:
        w = want.table[col]
        np.testing.assert_allclose(got.table[col], w, rtol=0, atol=1e-5 * np.abs(w).max())
    assert abs(got.meta["ks"] - want.meta["ks"]) <= 1e-5 and abs(got.meta["ks"] - 1.0580) <= 1e-4
    assert got.meta["injected_ion_pairs"] == pytest.approx(want.meta["injected_ion_pairs"], rel=1e-5)
    assert got.meta["recombined_ion_pairs"] == pytest.approx(want.meta["recombined_ion_pairs"], rel=1e-5)
    assert {k: got.meta[k] for k in got.meta if k not in ("f", "ks", "injected_ion_pairs", "recombined_ion_pairs")} \
        == {k: want.meta[k] for k in want.meta if k not in ("f", "ks", "injected_ion_pairs", "recombined_ion_pairs")}
