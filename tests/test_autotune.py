"""The autotuner's choice logic without a GPU: the timing calls are replaced
by a deterministic cost of the launch shape, so the test sees which shape is
applied, when a multi-step launch is kept, and that a cached choice is reused
without timing anything."""

import importlib
import types

import pytest

from goldens import make_config, pkg


@pytest.fixture()
def tuner(monkeypatch, tmp_path):
    at = importlib.import_module(pkg().__name__ + ".autotune")
    monkeypatch.setattr(at, "CACHE", tmp_path / "tuning.json")
    monkeypatch.setattr(at, "_key", lambda grid, with_dep: f"test|{grid.no_xy}|{grid.nzb}|{int(with_dep)}")
    calls = {"shape": 0, "segment": []}

    def cost(shape):
        # cheapest: flat, 7 planes per item; the rest by a fixed ordering
        c = 1.0 + 0.01 * abs(shape.get("planes_per_item", 0) - 7) + 0.001 * shape.get("tile_rows", 0)
        return c if shape.get("variant") == "flat" else c + 0.5

    def time_shape(engine, shape, reps=10, with_deposition=True):
        calls["shape"] += 1
        return cost(shape)

    def time_segment(engine, k, n_steps=128, reps=3):
        calls["segment"].append(k)
        return {0: 0.010, 32: 0.008, 256: 0.009}[k]

    monkeypatch.setattr(at, "time_shape", time_shape)
    monkeypatch.setattr(at, "time_segment", time_segment)
    return at, calls, cost


def _engine(name, **kw):
    eng_mod = importlib.import_module(pkg().__name__ + ".engine")
    return types.SimpleNamespace(grid=eng_mod.make_grid(make_config(name, **kw)))


def test_fastest_shape_and_steps_per_launch_are_applied_and_cached(tuner):
    at, calls, cost = tuner
    e = _engine("column_10um_r008")  # 24 x 24 x 206: flat, small enough for multi-step launches
    best = at.tune(e, quick=True)
    tried = best["tried"]
    assert tried and calls["shape"] == len(tried)
    shape, ms = min(tried, key=lambda t: t[1])
    assert best["ms"] == ms and ms == min(cost(s) for s, _ in tried)
    assert best["shape"] == dict(shape, steps_per_launch=32)  # 8 us/step against 10 with graphs
    assert calls["segment"] == [0, 32, 256]
    for k, v in best["shape"].items():
        if k != "variant":
            assert getattr(e.grid, k) == v, k

    # a second grid object of the same chamber: the cached choice, nothing timed
    e2 = _engine("column_10um_r008")
    again = at.tune(e2, quick=True)
    assert again["shape"] == best["shape"] and calls["shape"] == len(tried) and len(calls["segment"]) == 3
    assert e2.grid.steps_per_launch == 32 and e2.grid.planes_per_item == e.grid.planes_per_item


def test_large_grids_keep_one_launch_a_step(tuner):
    at, calls, _ = tuner
    e = _engine("column_5um_r05_d8p91")  # 208 x 208 x 406: above the multi-step cell limit
    assert int(e.grid.no_xy) ** 2 * int(e.grid.kpitch) > at.MULTI_MAX_CELLS
    best = at.tune(e, quick=True, use_cache=False)
    assert "steps_per_launch" not in best["shape"] and calls["segment"] == []
    assert e.grid.steps_per_launch == 0
    assert not (at.CACHE).exists()  # use_cache=False writes nothing
