"""pic_step_noalloc: the allocation-free time step, through the C ABI.

For callers that can pass the library device pointers but cannot allocate
device memory themselves (a binding that only holds buffers owned by another
runtime, or code running where cudaMalloc is not allowed), pic_step_noalloc
keeps its scratch -- the 2D track density and the tally workspace -- in a
static device array inside the library. This test checks that two calls in a
row give what the allocating entry points (pic_deposit + pic_step with
caller-allocated scratch) give on the same inputs, within the float32 parity
tolerance of the other tests (1e-5), and that a grid too large for the static
scratch is refused. The cases cover both step kernels (the flat one and the
streaming one, whose copies read the deposition from the static array) and
the status word of the static workspace, read and cleared through
pic_step_noalloc_status.

Kept in a file of its own that is collected last, so that a run that stops at
the first failure has already run every other test; it runs the same alone in
a fresh process.
"""

import ctypes
import importlib

import numpy as np
import pytest

from goldens import make_config, pkg

pytestmark = pytest.mark.gpu

REL = 1e-5


def _mods():
    name = pkg().__name__
    return importlib.import_module(name + "._native"), importlib.import_module(name + ".engine")


def _two_steps_of_tracks(cfg):
    rng = np.random.default_rng(cfg.seed)
    sched = pkg().build_track_schedule(cfg, rng)
    counts = sched[:2]
    xs, ys = pkg().TrackSampler(rng, cfg.mid_xy, cfg.sampling_radius, cfg.no_xy).sample(int(counts.sum()))
    return [(xs[: counts[0]], ys[: counts[0]]), (xs[counts[0]:], ys[counts[0]:])]


# The grid (208 x 208 x 406, 1.8e7 cells) is below the size from which the
# library picks the streaming step by itself, so the flat step runs unless a
# case asks for the streaming one: its bulk copies then read the deposition
# pairs out of the static array.
CASES = [
    ("float32", "absorbing", None),
    ("float32", "reflecting", None),
    ("float64", "absorbing", None),
    ("float32", "absorbing", {"variant": "stream"}),
    ("float32", "reflecting", {"variant": "stream", "tile_rows": 12, "consumer_warps": 15, "stages": 5}),
]


@pytest.mark.parametrize("dtype, wall, shape", CASES, ids=["f32-abs-flat", "f32-refl-flat", "f64-abs-flat",
                                                           "f32-abs-stream", "f32-refl-stream15"])
def test_two_calls_match_the_allocating_entry_points(dtype, wall, shape):
    import torch

    N, eng = _mods()
    lib = N.load()
    cfg = make_config("column_5um_r05_d89p1", lateral_boundary=wall)
    g = eng.make_grid(cfg, dtype=dtype, shape=shape)
    if shape:
        assert eng.resolve_shape(g)["variant"] == "stream"
    tdt = torch.float32 if dtype == "float32" else torch.float64
    shape = (g.no_xy, g.no_xy, g.kpitch)
    dev = torch.device("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    steps = _two_steps_of_tracks(cfg)

    # allocating path: caller-owned density and workspace
    fa = [torch.zeros(shape, dtype=tdt, device=dev) for _ in range(6)]  # pos/neg x 3 time levels
    dens = torch.zeros((g.no_xy, 2 * lib.pic_dens_pitch(g.no_xy)), dtype=tdt, device=dev)  # pairs
    wsb = ctypes.c_int64()
    N.check(lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(wsb)), "pic_step_workspace_bytes")
    ws = torch.zeros(int(wsb.value), dtype=torch.uint8, device=dev)
    counts_a = torch.zeros((g.no_xy, g.no_xy), dtype=torch.int32, device=dev)
    tally_a = torch.zeros((2, 4), dtype=torch.float64, device=dev)
    # allocation-free path
    fb = [torch.zeros(shape, dtype=tdt, device=dev) for _ in range(6)]
    counts_b = torch.zeros((g.no_xy, g.no_xy), dtype=torch.int32, device=dev)
    tally_b = torch.zeros((2, 4), dtype=torch.float64, device=dev)

    for s, (xs, ys) in enumerate(steps):
        dx = torch.from_numpy(np.ascontiguousarray(xs)).to(dev)
        dy = torch.from_numpy(np.ascontiguousarray(ys)).to(dev)
        m = len(xs)
        pin, nin, pout, nout = 2 * s, 2 * s + 1, 2 * s + 2, 2 * s + 3
        dens.zero_()
        N.check(lib.pic_deposit(ctypes.byref(g), dx.data_ptr(), dy.data_ptr(), m, dens.data_ptr(),
                                counts_a.data_ptr(), stream), "pic_deposit")
        N.check(lib.pic_step(ctypes.byref(g), fa[pin].data_ptr(), fa[nin].data_ptr(), fa[pout].data_ptr(),
                             fa[nout].data_ptr(), dens.data_ptr(), None, tally_a[s].data_ptr(), ws.data_ptr(),
                             ws.numel(), stream), "pic_step")
        N.check(lib.pic_step_noalloc(ctypes.byref(g), fb[pin].data_ptr(), fb[nin].data_ptr(), fb[pout].data_ptr(),
                                     fb[nout].data_ptr(), dx.data_ptr(), dy.data_ptr(), m, counts_b.data_ptr(),
                                     tally_b[s].data_ptr(), stream), "pic_step_noalloc")
        torch.cuda.synchronize()
        for t in (pout, nout):
            a = fa[t].double().cpu().numpy()
            b = fb[t].double().cpu().numpy()
            peak = np.abs(a).max()
            assert peak > 0
            np.testing.assert_allclose(b, a, rtol=0, atol=REL * peak)
        np.testing.assert_array_equal(counts_b.cpu().numpy(), counts_a.cpu().numpy())
        np.testing.assert_allclose(tally_b[s].cpu().numpy(), tally_a[s].cpu().numpy(), rtol=REL)
    # no bounded wait ran out: the static workspace's status word reads 0,
    # and reading it with reset leaves it 0
    status = ctypes.c_int32(-1)
    N.check(lib.pic_step_noalloc_status(1, stream, ctypes.byref(status)), "pic_step_noalloc_status")
    assert status.value == 0
    N.check(lib.pic_step_noalloc_status(0, stream, ctypes.byref(status)), "pic_step_noalloc_status")
    assert status.value == 0


def test_grid_beyond_the_static_scratch_is_refused():
    import torch

    N, eng = _mods()
    lib = N.load()
    cfg = make_config("full_electrode_5um_10p", sampled_radius_cm=0.4)  # no_xy = 1608 > 1448
    g = eng.make_grid(cfg)
    assert 2 * g.no_xy * lib.pic_dens_pitch(g.no_xy) * 4 > 16 << 20
    small = [torch.zeros(8, dtype=torch.float32, device="cuda") for _ in range(4)]
    tally = torch.zeros(4, dtype=torch.float64, device="cuda")
    counts = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.pic_step_noalloc(ctypes.byref(g), small[0].data_ptr(), small[1].data_ptr(), small[2].data_ptr(),
                              small[3].data_ptr(), None, None, 0, counts.data_ptr(), tally.data_ptr(),
                              torch.cuda.current_stream().cuda_stream)
    assert rc == N.PIC_E_CAPACITY
    assert b"static scratch" in lib.pic_last_error()
