"""Test-only stand-in for pandas.read_csv, enough for the reference's
stopping-power table lookup (golden-fixture generation only)."""

import numpy as np


class _Frame(dict):
    @property
    def columns(self):
        return list(self.keys())


def read_csv(path, skiprows=0):
    with open(path) as fh:
        lines = fh.read().splitlines()[skiprows:]
    header = lines[0].split(",")
    rows = [ln.split(",") for ln in lines[1:] if ln.strip()]
    data = np.array(rows, dtype=np.float64)
    return _Frame({name: data[:, c] for c, name in enumerate(header)})
