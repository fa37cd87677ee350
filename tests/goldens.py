"""Loading the golden fixtures that tests/golden/make_golden.py produced by
running the reference solver (pulsed_ion_chamber) itself."""

import importlib
import json
import warnings
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
PACKAGE = "iontracks-pulsedproton-python_gb300"


def pkg():
    return importlib.import_module(PACKAGE)


def config_json(name):
    return json.loads((GOLDEN / f"config_{name}.json").read_text())


def make_config(name, **overrides):
    """The package's SimulationConfig built from a fixture's keyword set, with
    the LET and track radius the reference computed for it."""
    d = config_json(name)
    kw = dict(d["kwargs"])
    kw.update(overrides)
    kw.setdefault("LET_keV_um", d["LET_keV_um"])
    kw.setdefault("track_radius_cm", d["track_radius_cm"])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return pkg().SimulationConfig(**kw)


def run_fixture(name):
    z = np.load(GOLDEN / f"{name}.npz")
    out = {k: z[k] for k in z.files}
    out["meta"] = json.loads(str(out.pop("meta_json")))
    return out


def run_config(name):
    """Config of a run_* / step_* fixture."""
    fx = run_fixture(name)
    return make_config(fx["meta"]["config"], **fx["meta"]["overrides"]), fx


def available(name):
    return (GOLDEN / f"{name}.npz").exists()


def oracle_fixture(name):
    """Whole-run float64 oracle results written by
    tests/golden/make_oracle_fixtures.py (``oracle_sweep64`` or
    ``oracle_column_5um_r05``)."""
    return json.loads((GOLDEN / f"{name}.json").read_text())


def histogram_sha256(track_density_xy) -> str:
    """SHA-256 of a track histogram as uint32 in C order (the fixtures' form)."""
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(np.asarray(track_density_xy).astype(np.uint32)).tobytes()).hexdigest()
