"""Device state of one chamber run and the calls that advance it.

:class:`ChamberEngine` owns the HBM buffers of one grid -- two float32 (or
float64) buffers per species in the padded ``[no_xy][no_xy][kpitch]`` layout,
two 2D density buffers, the track-centre histogram, the per-step float64
tallies and the step's scratch -- and advances them through the C ABI in
segments of steps. PyTorch only allocates the buffers and supplies the
stream; every kernel is the library's.
"""

from __future__ import annotations

import ctypes
from contextlib import contextmanager

import numpy as np

from . import _native as N
from .constants import recombination_alpha

_DTYPES = {"float32": N.PIC_F32, "float64": N.PIC_F64}
_VARIANTS = {"auto": N.PIC_VARIANT_AUTO, "flat": N.PIC_VARIANT_FLAT, "stream": N.PIC_VARIANT_STREAM}
_DEPOSIT_VARIANTS = {"auto": N.PIC_DEPOSIT_AUTO, "tracks": N.PIC_DEPOSIT_TRACKS, "binned": N.PIC_DEPOSIT_BINNED}
_EXTRA_FIELDS = ("adjoint_variant", "deposit_variant")
SHAPE_FIELDS = ("variant", "tile_rows", "planes_per_item", "stages", "consumer_warps", "ctas_per_sm", "steps_per_launch")


@contextmanager
def nvtx_range(name: str):
    """An NVTX range over the enclosed host work (the library's entry points
    open their own ranges inside it): a launch list taken with ncu --nvtx then
    splits by phase. A no-op unless a profiler is attached."""
    import torch

    torch.cuda.nvtx.range_push(name)
    try:
        yield
    finally:
        torch.cuda.nvtx.range_pop()


def apply_shape(g: N.PicGrid, shape: dict | None) -> N.PicGrid:
    """Sets launch-shape fields of a descriptor from a dict (``variant`` and
    ``adjoint_variant`` may be ``"auto"``, ``"flat"`` or ``"stream"``,
    ``deposit_variant`` ``"auto"``, ``"tracks"`` or ``"binned"``); unknown
    keys raise."""
    for key, val in (shape or {}).items():
        if key not in SHAPE_FIELDS + _EXTRA_FIELDS:
            raise ValueError(f"unknown launch-shape field {key!r}; expected one of {SHAPE_FIELDS + _EXTRA_FIELDS}")
        names = _DEPOSIT_VARIANTS if key == "deposit_variant" else _VARIANTS
        if key in ("variant",) + _EXTRA_FIELDS and isinstance(val, str):
            if val not in names:
                raise ValueError(f"{key} must be one of {sorted(names)}, got {val!r}")
            val = names[val]
        setattr(g, key, int(val))
    return g


def resolve_shape(g: N.PicGrid) -> dict:
    """The launch shape the library will use for this descriptor."""
    out = N.PicGrid()
    N.check(N.load().pic_resolve_shape(ctypes.byref(g), ctypes.byref(out)), "pic_resolve_shape")
    d = {k: int(getattr(out, k)) for k in SHAPE_FIELDS}
    d["variant"] = {v: k for k, v in _VARIANTS.items()}[d["variant"]]
    return d


def make_grid(config, dtype: str = "float32", alpha_cm3_s: float | None = None, shape: dict | None = None) -> N.PicGrid:
    """The ``pic_grid`` descriptor of a configuration (any object with the
    reference SimulationConfig's attributes), with optional launch-shape
    overrides."""
    if dtype not in _DTYPES:
        raise ValueError(f"dtype must be 'float32' or 'float64', got {dtype!r}")
    (p_lat, p_zm, p_zp, p_cen), (n_lat, n_zm, n_zp, n_cen) = config.scheme_coefficients()
    alpha = recombination_alpha(config) if alpha_cm3_s is None else float(alpha_cm3_s)
    g = N.PicGrid()
    g.no_xy = int(config.no_xy)
    g.nzb = int(config.no_z_with_buffer)
    g.kpitch = (g.nzb + 7) // 8 * 8
    g.no_z = int(config.no_z)
    g.nze = int(config.no_z_electrode)
    g.mid_xy = float(config.mid_xy)
    g.scoring_radius_sq = float(config.scoring_radius_sq)
    g.p_lat, g.p_zm, g.p_zp, g.p_cen = map(float, (p_lat, p_zm, p_zp, p_cen))
    g.n_lat, g.n_zm, g.n_zp, g.n_cen = map(float, (n_lat, n_zm, n_zp, n_cen))
    g.alpha_dt = alpha * float(config.dt)
    g.gaussian_factor = float(config.Gaussian_factor)
    g.h2_over_b2 = float(config.unit_length_cm) ** 2 / float(config.track_radius_cm) ** 2
    g.cutoff_voxels = float(config.track_cutoff_voxels)
    g.wall = N.PIC_WALL_REFLECTING if config.lateral_boundary == "reflecting" else N.PIC_WALL_ABSORBING
    g.dtype = _DTYPES[dtype]
    return apply_shape(g, shape)


def device_bytes(config, dtype: str = "float32", max_tracks: int = 0) -> int:
    """HBM the engine allocates for a configuration."""
    n = int(config.no_xy)
    kp = (int(config.no_z_with_buffer) + 7) // 8 * 8
    es = 4 if dtype == "float32" else 8
    dp = (n + 3) // 4 * 4
    return 4 * n * n * kp * es + 4 * n * dp * es + n * n * 4 + int(config.total_time_steps) * 32 + 16 * max_tracks


class ChamberEngine:
    """HBM state of one run plus the entry points that advance it."""

    def __init__(self, config, dtype: str = "float32", alpha_cm3_s: float | None = None, max_tracks: int = 0,
                 device=None, tally_steps: int | None = None, shape: dict | None = None):
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("run_simulation_b200 needs a CUDA device (a GB300); none is visible")
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.lib = N.load()
        N.device_info()  # raises unless the current device is sm_103
        self.config = config
        self.dtype = dtype
        self.grid = make_grid(config, dtype, alpha_cm3_s, shape)
        need = device_bytes(config, dtype, max_tracks)
        free, _total = torch.cuda.mem_get_info(self.device)
        if need > 0.9 * free:
            raise MemoryError(
                f"A {config.no_xy}x{config.no_xy}x{config.no_z_with_buffer} grid needs {need / 2**30:.2f} GiB of "
                f"device memory ({dtype} fields, double-buffered) but only {free / 2**30:.2f} GiB is free."
            )
        g = self.grid
        tdt = torch.float32 if dtype == "float32" else torch.float64
        shape = (g.no_xy, g.no_xy, g.kpitch)
        kw = dict(device=self.device)
        self.pos = [torch.zeros(shape, dtype=tdt, **kw), torch.zeros(shape, dtype=tdt, **kw)]
        self.neg = [torch.zeros(shape, dtype=tdt, **kw), torch.zeros(shape, dtype=tdt, **kw)]
        # deposition pairs (G * density, G * neighbours' sum), rows padded to
        # 4 pairs (pic_dens_pitch)
        self.dens_pitch = (g.no_xy + 3) // 4 * 4
        self.dens = [torch.zeros((g.no_xy, 2 * self.dens_pitch), dtype=tdt, **kw) for _ in range(2)]
        self.counts = torch.zeros((g.no_xy, g.no_xy), dtype=torch.int32, **kw)
        steps = int(config.total_time_steps) if tally_steps is None else int(tally_steps)
        self.tally = torch.zeros((max(steps, 1), 4), dtype=torch.float64, **kw)
        wsb = ctypes.c_int64()
        N.check(self.lib.pic_step_workspace_bytes(ctypes.byref(g), ctypes.byref(wsb)), "pic_step_workspace_bytes")
        self.workspace = torch.zeros(int(wsb.value), dtype=torch.uint8, **kw)
        self.xs = torch.zeros(max(int(max_tracks), 1), dtype=torch.float64, **kw)
        self.ys = torch.zeros(max(int(max_tracks), 1), dtype=torch.float64, **kw)
        self.parity = 0  # fields[parity] holds the current state
        self.step_index = 0  # global step of the next call
        self._graphs = {}

    # ---- tracks --------------------------------------------------------
    def ensure_track_capacity(self, n: int) -> None:
        if n > self.xs.numel():
            torch = self.torch
            self.xs = torch.zeros(int(n), dtype=torch.float64, device=self.device)
            self.ys = torch.zeros(int(n), dtype=torch.float64, device=self.device)
            self._graphs.clear()

    def upload_tracks(self, xs: np.ndarray, ys: np.ndarray, non_blocking: bool = True) -> None:
        """Copy track centres (float64, voxel units) to the device buffer."""
        n = len(xs)
        self.ensure_track_capacity(n)
        if n == 0:
            return
        torch = self.torch
        hx = torch.from_numpy(np.ascontiguousarray(xs, dtype=np.float64))
        hy = torch.from_numpy(np.ascontiguousarray(ys, dtype=np.float64))
        if non_blocking:
            hx, hy = hx.pin_memory(), hy.pin_memory()
        self.xs[:n].copy_(hx, non_blocking=non_blocking)
        self.ys[:n].copy_(hy, non_blocking=non_blocking)

    # ---- stepping ------------------------------------------------------
    def _stream(self, stream):
        return self.torch.cuda.current_stream(self.device).cuda_stream if stream is None else stream

    def run_segment(self, track_offsets: np.ndarray, track_base: int = 0, tally_row: int | None = None,
                    stream=None) -> None:
        """Advance ``len(track_offsets) - 1`` steps. Step ``s`` deposits
        tracks ``track_base + [track_offsets[s], track_offsets[s+1])`` of the
        uploaded track buffer; its tallies land in row ``tally_row + s``
        (default: the global step index)."""
        off = np.ascontiguousarray(track_offsets, dtype=np.int64)
        n_steps = len(off) - 1
        if n_steps <= 0:
            return
        row = self.step_index if tally_row is None else int(tally_row)
        if row + n_steps > self.tally.shape[0]:
            raise ValueError("tally buffer too small for this segment")
        if track_base < 0 or track_base + off[-1] > self.xs.numel():
            raise ValueError("track offsets exceed the uploaded track buffer")
        g = self.grid
        st = self._stream(stream)
        xp = self.xs.data_ptr() + 8 * int(track_base)
        yp = self.ys.data_ptr() + 8 * int(track_base)
        rc = self.lib.pic_run_segment(
            ctypes.byref(g), self.pos[0].data_ptr(), self.neg[0].data_ptr(), self.pos[1].data_ptr(),
            self.neg[1].data_ptr(), self.parity, n_steps, xp, yp,
            off.ctypes.data_as(ctypes.c_void_p), self.dens[0].data_ptr(), self.dens[1].data_ptr(),
            self.step_index & 1, self.counts.data_ptr(), self.tally[row].data_ptr(), self.workspace.data_ptr(),
            self.workspace.numel(), st,
        )
        N.check(rc, "pic_run_segment")
        self.parity = (self.parity + n_steps) & 1
        self.step_index += n_steps

    def run_segment_graphed(self, key, track_offsets: np.ndarray, track_base: int = 0, stream=None) -> None:
        """Same as :meth:`run_segment`, replayed from a CUDA graph.

        The first call with a key captures the segment's launches into a
        graph; later calls with the same key replay it. A graph bakes in the
        buffers, the track offsets and base, and the field and density
        parities, so the key must determine all of them (the caller's job);
        the parities are checked here. Tallies go to a staging block owned by
        the graph and are copied to the run's tally rows after each replay.
        """
        off = np.ascontiguousarray(track_offsets, dtype=np.int64)
        n_steps = len(off) - 1
        if n_steps <= 0:
            return
        row = self.step_index
        if row + n_steps > self.tally.shape[0]:
            raise ValueError("tally buffer too small for this segment")
        if track_base < 0 or track_base + off[-1] > self.xs.numel():
            raise ValueError("track offsets exceed the uploaded track buffer")
        st = self._stream(stream)
        entry = self._graphs.get(key)
        if entry is None:
            torch = self.torch
            stage = torch.zeros((n_steps, 4), dtype=torch.float64, device=self.device)
            g = self.grid
            h = ctypes.c_void_p()
            rc = self.lib.pic_graph_create(
                ctypes.byref(g), self.pos[0].data_ptr(), self.neg[0].data_ptr(), self.pos[1].data_ptr(),
                self.neg[1].data_ptr(), self.parity, n_steps, self.xs.data_ptr() + 8 * int(track_base),
                self.ys.data_ptr() + 8 * int(track_base), off.ctypes.data_as(ctypes.c_void_p),
                self.dens[0].data_ptr(), self.dens[1].data_ptr(), self.step_index & 1, self.counts.data_ptr(),
                stage.data_ptr(), self.workspace.data_ptr(), self.workspace.numel(), st, ctypes.byref(h),
            )
            N.check(rc, "pic_graph_create")
            entry = (h.value, n_steps, stage, self.parity, self.step_index & 1)
            self._graphs[key] = entry
        handle, n, stage, parity, dparity = entry
        if n != n_steps or parity != self.parity or dparity != (self.step_index & 1):
            raise RuntimeError("graph key reused for a segment with a different length or parity")
        N.check(self.lib.pic_graph_launch(handle, st), "pic_graph_launch")
        self.tally[row : row + n_steps].copy_(stage)
        self.parity = (self.parity + n_steps) & 1
        self.step_index += n_steps

    def check_status(self, stream=None) -> None:
        """Raises if a kernel's bounded wait expired since the last check
        (the status word in the step workspace)."""
        st = ctypes.c_int32()
        N.check(self.lib.pic_workspace_status(self.workspace.data_ptr(), 1, self._stream(stream), ctypes.byref(st)),
                "pic_workspace_status")
        if st.value != 0:
            raise RuntimeError(f"a fused-step kernel gave up on a bounded wait (code {st.value}); results are invalid")

    def close(self) -> None:
        for entry in self._graphs.values():
            self.lib.pic_graph_destroy(entry[0])
        self._graphs.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- results -------------------------------------------------------
    def fields(self, as_float64: bool = True):
        """Current (positive, negative) fields as host arrays of shape
        ``(no_xy, no_xy, no_z_with_buffer)``."""
        nzb = self.grid.nzb
        out = []
        for t in (self.pos[self.parity], self.neg[self.parity]):
            a = t[:, :, :nzb].contiguous().cpu().numpy()
            out.append(a.astype(np.float64) if as_float64 else a)
        return out[0], out[1]

    def tallies(self, n_steps: int) -> np.ndarray:
        return self.tally[:n_steps].cpu().numpy()

    def track_density_xy(self) -> np.ndarray:
        return self.counts.cpu().numpy().view(np.uint32).astype(np.float64)
