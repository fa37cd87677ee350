"""ctypes binding of libpic_gb300.so (include/pic_gb300.h).

The library is the product's compute path; there is no fallback. If it is
missing, cannot be built, or the current device is not a GB300 (sm_103),
:func:`lib` raises ``RuntimeError`` with the reason.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

PIC_OK = 0
PIC_E_INVALID = -1
PIC_E_CUDA = -2
PIC_E_DEVICE = -3
PIC_E_CAPACITY = -4
PIC_F32 = 0
PIC_F64 = 1
PIC_WALL_ABSORBING = 0
PIC_WALL_REFLECTING = 1
PIC_VARIANT_AUTO = 0
PIC_VARIANT_FLAT = 1
PIC_VARIANT_STREAM = 2
PIC_DEPOSIT_AUTO = 0
PIC_DEPOSIT_TRACKS = 1
PIC_DEPOSIT_BINNED = 2
# pic_abi_version() of the library these structures mirror
ABI_VERSION = 8

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libpic_gb300.so"
_lock = threading.Lock()
_lib = None


class PicGrid(ctypes.Structure):
    """Mirror of ``struct pic_grid``."""

    _fields_ = [
        ("no_xy", ctypes.c_int64),
        ("nzb", ctypes.c_int64),
        ("kpitch", ctypes.c_int64),
        ("no_z", ctypes.c_int64),
        ("nze", ctypes.c_int64),
        ("mid_xy", ctypes.c_double),
        ("scoring_radius_sq", ctypes.c_double),
        ("p_lat", ctypes.c_double),
        ("p_zm", ctypes.c_double),
        ("p_zp", ctypes.c_double),
        ("p_cen", ctypes.c_double),
        ("n_lat", ctypes.c_double),
        ("n_zm", ctypes.c_double),
        ("n_zp", ctypes.c_double),
        ("n_cen", ctypes.c_double),
        ("alpha_dt", ctypes.c_double),
        ("gaussian_factor", ctypes.c_double),
        ("h2_over_b2", ctypes.c_double),
        ("cutoff_voxels", ctypes.c_double),
        ("wall", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("variant", ctypes.c_int32),
        ("tile_rows", ctypes.c_int32),
        ("planes_per_item", ctypes.c_int32),
        ("stages", ctypes.c_int32),
        ("consumer_warps", ctypes.c_int32),
        ("ctas_per_sm", ctypes.c_int32),
        ("steps_per_launch", ctypes.c_int32),
        ("adjoint_variant", ctypes.c_int32),
        ("deposit_variant", ctypes.c_int32),
    ]


EXPORTS = {
    # name: (restype, argtypes)
    "pic_last_error": (ctypes.c_char_p, []),
    "pic_abi_version": (ctypes.c_int, []),
    "pic_kpitch": (ctypes.c_int64, [ctypes.c_int64]),
    "pic_dens_pitch": (ctypes.c_int64, [ctypes.c_int64]),
    "pic_device_info": (
        ctypes.c_int,
        [ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32),
         ctypes.POINTER(ctypes.c_int32)],
    ),
    "pic_step_workspace_bytes": (ctypes.c_int, [ctypes.POINTER(PicGrid), ctypes.POINTER(ctypes.c_int64)]),
    "pic_workspace_status": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]
    ),
    "pic_resolve_shape": (ctypes.c_int, [ctypes.POINTER(PicGrid), ctypes.POINTER(PicGrid)]),
    "pic_deposit": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p],
    ),
    "pic_step": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "pic_step_noalloc": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    ),
    "pic_step_noalloc_status": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    "pic_sample_disc": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)],
    ),
    "pic_arrival_counts_pcg64": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "pic_sample_disc_pcg64": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int64, ctypes.c_int64,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)],
    ),
    "pic_adjoint_workspace_bytes": (ctypes.c_int, [ctypes.POINTER(PicGrid), ctypes.POINTER(ctypes.c_int64)]),
    "pic_adjoint_step": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
         ctypes.c_void_p],
    ),
    "pic_adjoint_forward": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_void_p],
    ),
    "pic_adjoint_backward": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_void_p],
    ),
    "pic_selftest_waits": (
        ctypes.c_int, [ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p]
    ),
    "pic_revolve_plan": (
        ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    ),
    "pic_revolve_spine": (
        ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    ),
    "pic_revolve_trace": (
        ctypes.c_int,
        [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64),
         ctypes.POINTER(ctypes.c_int64)],
    ),
    "pic_revolve_forward": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_void_p],
    ),
    "pic_revolve_backward": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "pic_batched_persistent": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pic_batched_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    "pic_capture_begin": (ctypes.c_int, [ctypes.c_void_p]),
    "pic_capture_end": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "pic_run_segment": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
         ctypes.c_void_p],
    ),
    "pic_graph_create": (
        ctypes.c_int,
        [ctypes.POINTER(PicGrid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
         ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)],
    ),
    "pic_batched_workspace_bytes": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]),
    "pic_batched_deposit_bytes": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64,
                                                 ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]),
    "pic_batched_segment": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pic_batched_graph_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "pic_batched_stream_workspace_bytes": (
        ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]
    ),
    "pic_batched_stream_prepare": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
         ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p],
    ),
    "pic_batched_stream_segment": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pic_batched_stream_status": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]
    ),
    "pic_graph_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pic_graph_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pic_kernel_launches": (ctypes.c_int64, []),
}


class PicError(RuntimeError):
    def __init__(self, code, what, msg):
        super().__init__(f"{what} failed ({code}): {msg}")
        self.code = code


def library_path() -> Path:
    return _LIB_PATH


def load(path: Path | None = None, build_if_missing: bool = True):
    """Load (building first if needed) and bind the shared library. Needs no GPU."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else _LIB_PATH
        if path is None and build_if_missing:
            from . import build as _build

            try:
                _build.build()
            except Exception as exc:  # no nvcc here: the library must already exist
                if not p.exists():
                    raise RuntimeError(f"libpic_gb300.so is missing and could not be built: {exc}") from exc
        if not p.exists():
            raise RuntimeError(f"libpic_gb300.so not found at {p}; run the package's build.py")
        L = ctypes.CDLL(str(p))
        for name, (res, args) in EXPORTS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        # a library built from other sources would read these structures wrong
        if L.pic_abi_version() != ABI_VERSION:
            raise RuntimeError(f"{p} has ABI {L.pic_abi_version()}, this binding ABI {ABI_VERSION}: rebuild it "
                               "with the package's build.py")
        if path is None:
            _lib = L
        return L


def check(rc: int, what: str) -> None:
    if rc != PIC_OK:
        msg = load().pic_last_error()
        raise PicError(rc, what, msg.decode() if msg else "")


def device_info():
    """(sm_count, total_bytes, cc_major, cc_minor); raises unless sm_103."""
    L = load()
    sms, tot, ma, mi = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
    check(L.pic_device_info(ctypes.byref(sms), ctypes.byref(tot), ctypes.byref(ma), ctypes.byref(mi)),
          "pic_device_info")
    return sms.value, tot.value, ma.value, mi.value


def kpitch(nzb: int) -> int:
    return int(load().pic_kpitch(int(nzb)))
