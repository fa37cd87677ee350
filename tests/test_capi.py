"""The C-ABI library builds for sm_103a, loads without a GPU, and exports
every entry point include/pic_gb300.h declares (no compute call here)."""

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from goldens import pkg

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "pic_gb300.h"


def _declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pic_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import importlib

    native = importlib.import_module(pkg().__name__ + "._native")
    return native.load()


def test_header_declares_the_entry_points():
    names = _declared()
    for must in ("pic_step", "pic_deposit", "pic_run_segment", "pic_last_error", "pic_graph_create"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_exported_symbols_are_c_linkage():
    import importlib

    native = importlib.import_module(pkg().__name__ + "._native")
    out = subprocess.run(["nm", "-D", "--defined-only", str(native.library_path())], capture_output=True, text=True)
    syms = {line.split()[-1] for line in out.stdout.splitlines() if line.strip()}
    for name in _declared():
        assert name in syms, name


def test_binding_covers_the_header(lib):
    import importlib

    native = importlib.import_module(pkg().__name__ + "._native")
    assert set(_declared()) == set(native.EXPORTS)


def test_host_only_calls_without_a_gpu(lib):
    assert lib.pic_abi_version() == 8
    native = __import__("importlib").import_module(pkg().__name__ + "._native")
    assert native.ABI_VERSION == 8
    assert lib.pic_kernel_launches() == 0  # nothing launched without a GPU
    assert ctypes.sizeof(native.PicGrid) == 200  # 5 int64, 14 double, 11 int32, padded to 8
    assert lib.pic_kpitch(406) == 408
    assert lib.pic_kpitch(408) == 408
    assert lib.pic_kpitch(3) == 8
    assert lib.pic_dens_pitch(1068) == 1068 and lib.pic_dens_pitch(25) == 28


def test_step_workspace_holds_the_track_lists_of_the_binned_deposition(lib):
    """The fixed part (tally partials of 152 x 32 blocks, counter, status)
    plus, for no_xy <= 4096 and truncation boxes of at most 64 cells, for
    each of 8 steps a count per 62 x 62-cell tile (padded to 256 bytes) and
    4096 track indices per tile, the boxes (4 int16) and factors (2 x 64 of
    the field type) of 65536 tracks, and 8 steps' deposition pairs."""
    import importlib

    P = pkg()
    E = importlib.import_module(P.__name__ + ".engine")
    beam = dict(E_MeV_u=56.2, voltage_V=300.0, electrode_gap_cm=0.2, pulse_duration_s=540e-6,
                repetition_rate_hz=50.0, dose_rate_Gy_s=8.91)
    fixed = 152 * 32 * 4 * 8 + 256
    for um, r, n in ((10.0, 0.008, 24), (5.0, 0.265, 1068)):
        cfg = P.SimulationConfig(**dict(beam, grid_size_um=um, sampled_radius_cm=r, seed=1, max_voxels=2e9))
        assert int(cfg.no_xy) == n
        g = E.make_grid(cfg)
        b = ctypes.c_int64()
        assert lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(b)) == 0
        tiles = ((n + 61) // 62) ** 2
        pairs = (n * ((n + 3) // 4 * 4) * 2 * 4 + 255) // 256 * 256
        assert b.value == (fixed + (8 * 4 * tiles + 255) // 256 * 256 + 8 * tiles * 4096 * 4 + 65536 * 8
                           + 65536 * 128 * 4 + 8 * pairs)
    assert E.apply_shape(g, {"deposit_variant": "binned"}).deposit_variant == 2
    with pytest.raises(ValueError):
        E.apply_shape(g, {"deposit_variant": "tiles"})


def test_invalid_grid_is_refused_before_any_device_work(lib):
    import importlib

    native = importlib.import_module(pkg().__name__ + "._native")
    g = native.PicGrid()
    g.no_xy, g.nzb, g.kpitch, g.no_z, g.nze = 2, 10, 16, 4, 3
    g.cutoff_voxels = 1.0
    b = ctypes.c_int64()
    rc = lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(b))
    assert rc == native.PIC_E_INVALID
    assert b"no_xy" in lib.pic_last_error()
    g.no_xy, g.kpitch = 8, 12
    assert lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(b)) == native.PIC_E_INVALID
    assert b"kpitch" in lib.pic_last_error()
    g.kpitch, g.nze = 16, 0
    assert lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(b)) == native.PIC_E_INVALID
    g.nze = 3
    g.mid_xy, g.scoring_radius_sq = 4.3, 9.0
    assert lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(b)) == native.PIC_E_INVALID
    assert b"mid_xy" in lib.pic_last_error()
    g.mid_xy, g.scoring_radius_sq = 4.0, 0.0
    assert lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(b)) == native.PIC_E_INVALID
    g.scoring_radius_sq = 9.0
    g.steps_per_launch = 257
    assert lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(b)) == native.PIC_E_INVALID
    assert b"steps_per_launch" in lib.pic_last_error()
    g.steps_per_launch = 256
    g.deposit_variant = 3
    assert lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(b)) == native.PIC_E_INVALID
    assert b"deposit_variant" in lib.pic_last_error()
    g.deposit_variant = native.PIC_DEPOSIT_BINNED
    assert lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(b)) == native.PIC_OK
    assert b.value > 0
    rc = lib.pic_step(ctypes.byref(g), None, None, None, None, None, None, None, None, 0, None)
    assert rc == native.PIC_E_INVALID


def test_noalloc_status_refuses_a_null_status_before_device_work(lib):
    import importlib

    native = importlib.import_module(pkg().__name__ + "._native")
    assert lib.pic_step_noalloc_status(0, None, None) == native.PIC_E_INVALID
    assert b"status is null" in lib.pic_last_error()


def test_grid_descriptor_from_config():
    import importlib

    from goldens import make_config

    eng = importlib.import_module(pkg().__name__ + ".engine")
    cfg = make_config("column_10um_r008")
    g = eng.make_grid(cfg)
    assert (g.no_xy, g.nzb, g.kpitch, g.no_z, g.nze) == (24, 206, 208, 200, 3)
    (pl, pzm, pzp, pc), _ = cfg.scheme_coefficients()
    assert (g.p_lat, g.p_zm, g.p_zp, g.p_cen) == (pl, pzm, pzp, pc)
    assert g.alpha_dt == 1.6e-6 * cfg.dt
    with pytest.raises(ValueError):
        eng.make_grid(cfg, dtype="float16")


def test_public_calls_fail_loudly_without_a_gpu():
    """No CPU fallback: every public entry point refuses to run without a
    CUDA device (and refuses bad arguments before looking for one)."""
    import torch

    from goldens import make_config

    P = pkg()
    cfg = make_config("fast")
    with pytest.raises(ValueError, match="chunk_steps"):
        P.run_simulation_b200(cfg, progress=False, chunk_steps=0)
    if torch.cuda.is_available():
        pytest.skip("checks the behaviour without a GPU")
    calls = [
        lambda: P.run_simulation_b200(cfg, progress=False),
        lambda: P.run_batched_b200([cfg]),
        lambda: P.ks_and_gradient(cfg),
        lambda: P.fit_parameters([cfg, cfg], [1.01, 1.02], names=("alpha",)),
    ]
    for call in calls:
        with pytest.raises(RuntimeError, match="needs a CUDA device"):
            call()


def test_launch_shape_resolution_without_a_gpu():
    import importlib

    from goldens import make_config

    eng = importlib.import_module(pkg().__name__ + ".engine")
    big = eng.make_grid(make_config("full_electrode_5um_10p"))
    s = eng.resolve_shape(big)
    assert s["variant"] == "stream"
    # 13 consumer warps, about three k-vectors a thread: 12 rows of 104
    assert s["tile_rows"] == 12 and s["consumer_warps"] == 13 and s["stages"] >= 4
    # 1066 planes x 89 tiles: about 12 work items per SM
    assert 32 <= s["planes_per_item"] <= 64
    small = eng.make_grid(make_config("column_10um_r008"))
    assert eng.resolve_shape(small)["variant"] == "flat"
    # 208 x 208 x 408 = 17.7 M cells: flat by default (faster below ~1e8
    # cells); streaming when asked, with few planes per item so that 30
    # j-tiles still give every SM work
    mid = eng.make_grid(make_config("column_5um_r05_d8p91"))
    assert eng.resolve_shape(mid)["variant"] == "flat"
    s = eng.resolve_shape(eng.make_grid(make_config("column_5um_r05_d8p91"), shape={"variant": "stream"}))
    assert s["variant"] == "stream" and 4 <= s["planes_per_item"] <= 8
    f64 = eng.make_grid(make_config("full_electrode_5um_10p"), dtype="float64")
    assert eng.resolve_shape(f64)["variant"] == "flat"
    forced = eng.make_grid(make_config("fast"), shape={"variant": "stream", "tile_rows": 3, "stages": 4})
    s = eng.resolve_shape(forced)
    assert (s["variant"], s["tile_rows"], s["stages"]) == ("stream", 3, 4)
    bad = eng.make_grid(make_config("fast"), dtype="float64", shape={"variant": "stream"})
    with pytest.raises(RuntimeError, match="float32"):
        eng.resolve_shape(bad)
    with pytest.raises(ValueError, match="launch-shape"):
        eng.make_grid(make_config("fast"), shape={"warps": 3})
    wide = eng.make_grid(make_config("sweep_hi"), shape={"variant": "stream"})
    s = eng.resolve_shape(wide)
    assert s["stages"] >= 4


def test_autotuner_candidates_are_shapes_the_library_accepts():
    """Every streaming shape the quick autotuner would time on the full
    electrode (and on a 10 um column) passes the library's own checks, wide
    12-16-warp forms included (no GPU: shape resolution is host code)."""
    import importlib

    from goldens import make_config

    eng = importlib.import_module(pkg().__name__ + ".engine")
    at = importlib.import_module(pkg().__name__ + ".autotune")
    native = importlib.import_module(pkg().__name__ + "._native")
    for name in ("full_electrode_5um_10p", "column_10um_r02"):
        g = eng.make_grid(make_config(name))
        shapes = at.candidate_shapes(g, quick=True)
        assert any(s.get("consumer_warps", 0) >= 12 for s in shapes) or g.no_xy < 64
        for shape in shapes:
            h = native.PicGrid.from_buffer_copy(g)
            for k in eng.SHAPE_FIELDS:
                setattr(h, k, 0)
            eng.apply_shape(h, shape)
            eng.resolve_shape(h)  # raises if the library refuses the shape
