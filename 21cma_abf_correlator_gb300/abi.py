"""ctypes view of libcorr_cuda.so: structures, status codes, entry points.

The structures mirror include/corr_cuda.h field for field (the same layouts the
reference's Rust mirror pins, corr-rs/src/ffi.rs:63-160); sizes are asserted at
import so a header change cannot go unnoticed.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libcorr_cuda.so"

CORR_ABI_VERSION = 7
CORR_MAX_DEVICES = 8
CORR_SPLIT_BASELINE_RANGE = 0
CORR_SPLIT_PAIR_COVERING = 1
CORR_SPLIT_TIME_SLICE = 2

CORR_X_PLAIN_FP32 = 0
CORR_X_TC_FP16 = 1
CORR_X_TC_FP16_SPLIT = 2

CORRX_ACC_FP32 = 0
CORRX_ACC_FP64 = 1

STATUS_NAMES = {
    0: "CORR_OK",
    1: "CORR_ERR_ARG",
    2: "CORR_ERR_ABI",
    3: "CORR_ERR_CUDA",
    4: "CORR_ERR_CUFFT",
    5: "CORR_ERR_STATE",
    6: "CORR_ERR_BUSY",
    7: "CORR_ERR_NOMEM",
    8: "CORR_ERR_NOT_IMPL",
    9: "CORR_ERR_INTERNAL",
}
globals().update({name: code for code, name in STATUS_NAMES.items()})


class corr_config(C.Structure):
    _fields_ = [
        ("abi_version", C.c_uint32),
        ("struct_size", C.c_uint32),
        ("device_id", C.c_int32),
        ("n_station", C.c_int32),
        ("n_freq", C.c_int32),
        ("frames_per_slot", C.c_int32),
        ("chunk_frames", C.c_int32),
        ("block_slots", C.c_int32),
        ("rows_per_fetch", C.c_int32),
        ("n_devices", C.c_int32),
        ("devices", C.c_int32 * CORR_MAX_DEVICES),
        ("split_mode", C.c_int32),
    ]


class corr_device_plan(C.Structure):
    _fields_ = [
        ("device_id", C.c_int32),
        ("n_station_resident", C.c_int32),
        ("first_baseline", C.c_int32),
        ("n_baseline", C.c_int32),
        ("contiguous", C.c_int32),
    ]


class corr_device_stats(C.Structure):
    _fields_ = [
        ("device_id", C.c_int32),
        ("bytes_h2d", C.c_uint64),
        ("bytes_d2h", C.c_uint64),
        ("transfers", C.c_uint64),
        ("ns_accumulate", C.c_uint64),
        ("ns_slot_free", C.c_uint64),
        ("ns_row_end", C.c_uint64),
        ("ns_rows_wait", C.c_uint64),
        ("ns_fetch", C.c_uint64),
    ]


class corr_staging(C.Structure):
    _fields_ = [
        ("base", C.POINTER(C.c_int8)),
        ("frame_stride", C.c_size_t),
        ("slot_stride", C.c_size_t),
        ("total_bytes", C.c_size_t),
        ("validity_offset", C.c_size_t),
        ("validity_bytes_per_slot", C.c_size_t),
    ]


class corrx_params(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("n_station", C.c_int32),
        ("n_freq", C.c_int32),
        ("max_frames", C.c_int32),
        ("xmode", C.c_int32),
        ("device_id", C.c_int32),
    ]


class corrx_tiles(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("ytile", C.c_int32),
        ("xct", C.c_int32),
        ("xkt", C.c_int32),
        ("fplan", C.c_int32),
        ("ms_fengine", C.c_float),
        ("ms_xengine", C.c_float),
    ]


CORRX_PATTERN_ZERO, CORRX_PATTERN_COUNTER, CORRX_PATTERN_PRNG, CORRX_PATTERN_SINE = 0, 1, 2, 3
CORRX_FRONTEND_MAX_STATIONS = 64


class corrx_frontend(C.Structure):
    """The synthetic front end's settings (corr_gb300.h), one field per option of
    the reference's transmitter (corr-rs/src/bin/replay.rs:41-165)."""
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("pattern", C.c_int32),
        ("seed", C.c_uint64),
        ("tone", C.c_double),
        ("start_counter", C.c_uint64),
        ("n_packets", C.c_uint64),
        ("drop_rate", C.c_double),
        ("gap_at", C.c_uint64),
        ("gap_len", C.c_uint64),
        ("ladder_frames", C.c_uint64),
        ("ladder_steps", C.c_uint64),
        ("sample_delay", C.c_int64 * CORRX_FRONTEND_MAX_STATIONS),
        ("counter_offset", C.c_uint64 * CORRX_FRONTEND_MAX_STATIONS),
    ]


class corrx_tc_geom(C.Structure):
    """The tensor X-engine's geometry for one tile shape (corrx_tc_geometry)."""
    _fields_ = [("struct_size", C.c_uint32)] + [
        (n, C.c_int32) for n in ("ok", "form", "elem", "R", "nb", "regions", "sbo",
                                 "region_stride", "op_stage", "ld_stage", "n_op", "n_ld",
                                 "acc_cols", "n_acc", "tmem_cols", "items", "smem")]


CORRW_SET_AUTO, CORRW_SET_NEW, CORRW_SET_EXPLICIT = 0, 1, 2
CORRW_QUEUE_DROP, CORRW_QUEUE_BLOCK = 0, 1


class corrw_station(C.Structure):
    _fields_ = [
        ("name", C.c_char_p),
        ("group_ip", C.c_char_p),
        ("dest_port", C.c_int32),
        ("board", C.c_char_p),
    ]


class corrw_params(C.Structure):
    """Output file-set writer settings (corr_writer.h; reference corr-rs/src/writer.rs)."""
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("n_station", C.c_int32),
        ("n_freq", C.c_int32),
        ("n_cum", C.c_uint32),
        ("frames_per_slot", C.c_uint32),
        ("rows_per_fetch", C.c_uint32),
        ("sample_rate_hz", C.c_uint64),
        ("data_shift_count", C.c_int32),
        ("daily_files", C.c_int32),
        ("set_policy", C.c_int32),
        ("queue_full", C.c_int32),
        ("queue_rows", C.c_uint32),
        ("fsync_every_rows", C.c_uint32),
        ("dir", C.c_char_p),
        ("file_prefix", C.c_char_p),
        ("file_prefix_format", C.c_char_p),
        ("config_version", C.c_char_p),
        ("config_hash", C.c_char_p),
        ("set_tag", C.c_char_p),
        ("stations", C.POINTER(corrw_station)),
    ]


class corrw_resume(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("has_next_frame_id", C.c_uint32),
        ("rows_written", C.c_uint64),
        ("truncated_rows", C.c_uint64),
        ("next_frame_id", C.c_uint64),
    ]


class corrw_stats(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("sets_opened", C.c_uint32),
        ("rows_written", C.c_uint64),
        ("rows_dropped", C.c_uint64),
        ("max_queued", C.c_uint64),
        ("set_tag", C.c_char * 256),
    ]


# Layouts pinned by the reference's Rust mirror (ffi.rs compile-time asserts).
assert C.sizeof(corr_config) == 76
assert C.sizeof(corr_device_plan) == 20
assert C.sizeof(corr_device_stats) == 72
assert C.sizeof(corr_staging) == 48

NOTIFY_FN = C.CFUNCTYPE(None, C.c_void_p)

# name -> (restype, argtypes); every symbol include/*.h declares.
SIGNATURES = {
    "corr_abi_banner": (C.c_char_p, []),
    "corr_last_error": (C.c_char_p, []),
    "corr_create": (C.c_int, [C.POINTER(corr_config), C.POINTER(C.c_void_p)]),
    "corr_destroy": (C.c_int, [C.c_void_p]),
    "corr_staging_info": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(corr_staging)]),
    "corr_row_accumulate": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32]),
    "corr_row_slot_free": (C.c_int, [C.c_void_p, C.c_int64]),
    "corr_row_slot_free_submit": (C.c_int, [C.c_void_p, C.c_int64, NOTIFY_FN, C.c_void_p]),
    "corr_row_slot_free_finish": (C.c_int, [C.c_void_p, C.c_int64]),
    "corr_row_end": (C.c_int, [C.c_void_p, C.c_uint64]),
    "corr_rows_wait": (C.c_int, [C.c_void_p]),
    "corr_rows_wait_submit": (C.c_int, [C.c_void_p, NOTIFY_FN, C.c_void_p]),
    "corr_rows_ready": (C.c_int, [C.c_void_p]),
    "corr_rows_pending": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "corr_rows_fetch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_int32)]),
    "corr_rows_fetch_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t,
                                         C.POINTER(C.c_int32), NOTIFY_FN, C.c_void_p]),
    "corr_rows_fetch_ready": (C.c_int, [C.c_void_p]),
    "corr_n_baseline": (C.c_int32, [C.c_int32]),
    "corr_baseline_pairs": (C.c_int, [C.c_int32, C.POINTER(C.c_int32), C.c_int32]),
    "corr_n_devices": (C.c_int32, [C.c_void_p]),
    "corr_device_plan_get": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(corr_device_plan)]),
    "corr_device_stations": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.c_int32]),
    "corr_device_baselines": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.c_int32]),
    "corr_device_stats_get": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(corr_device_stats)]),
    "corr_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "corr_host_free": (None, [C.c_void_p]),
    # corr_gb300.h
    "corr_set_xengine": (C.c_int, [C.c_void_p, C.c_int32]),
    "corrx_create": (C.c_int, [C.POINTER(corrx_params), C.POINTER(C.c_void_p)]),
    "corrx_destroy": (C.c_int, [C.c_void_p]),
    "corrx_accumulate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p,
                                   C.c_size_t, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "corrx_scale": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "corrx_set_accumulator": (C.c_int, [C.c_void_p, C.c_int32]),
    "corrx_dump": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    "corrx_set_device_map": (C.c_int, [C.POINTER(C.c_int32), C.c_int32]),
    "corrx_plan_query": (C.c_int, [C.POINTER(corr_config), C.c_int32,
                                   C.POINTER(corr_device_plan), C.POINTER(C.c_int32), C.c_int32,
                                   C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32),
                                   C.c_int32]),
    "corrx_check": (C.c_int, [C.c_void_p]),
    "corrx_get_tiles": (C.c_int, [C.c_void_p, C.POINTER(corrx_tiles)]),
    "corrx_set_tiles": (C.c_int, [C.c_void_p, C.POINTER(corrx_tiles)]),
    "corrx_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(corrx_tiles)]),
    "corr_autotune": (C.c_int, [C.c_void_p, C.POINTER(corrx_tiles)]),
    "corr_get_tiles": (C.c_int, [C.c_void_p, C.POINTER(corrx_tiles)]),
    "corr_set_tiles": (C.c_int, [C.c_void_p, C.POINTER(corrx_tiles)]),
    "corrx_run_fengine": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p,
                                    C.c_size_t, C.c_int32, C.c_int32, C.c_void_p]),
    "corrx_run_xengine": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "corrx_selftest_watchdog": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "corrx_batch_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p,
                                     C.c_size_t, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                     C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "corrx_batch_create_mixed": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32,
                                           C.POINTER(C.c_int32), C.c_void_p, C.c_size_t,
                                           C.c_size_t, C.c_void_p, C.c_size_t,
                                           C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                           C.c_int32, C.c_void_p, C.c_void_p,
                                           C.POINTER(C.c_void_p)]),
    "corrx_batch_create_packets": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32,
                                             C.POINTER(C.c_int32), C.c_void_p, C.c_size_t,
                                             C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p,
                                             C.c_size_t, C.POINTER(C.c_int64),
                                             C.POINTER(C.c_int32), C.c_int32, C.c_void_p,
                                             C.c_void_p, C.POINTER(C.c_void_p)]),
    "corrx_batch_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "corrx_batch_block_ms": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int32]),
    "corrx_batch_destroy": (C.c_int, [C.c_void_p]),
    "corrx_accumulate_noalloc": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                           C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t,
                                           C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "corrx_frontend_fill": (C.c_int, [C.POINTER(corrx_frontend), C.c_int32, C.c_int32,
                                      C.c_int32, C.c_int64, C.c_int32, C.c_void_p, C.c_size_t, C.c_size_t,
                                      C.c_void_p, C.c_size_t, C.c_void_p]),
    "corrx_tc_fft_maps": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p]),
    "corrx_accumulate_packets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t,
                                           C.c_void_p, C.c_size_t, C.c_int32, C.c_void_p,
                                           C.c_size_t, C.c_int32, C.c_int32, C.c_void_p,
                                           C.c_void_p]),
    "corrx_tc_geometry": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    C.POINTER(corrx_tc_geom)]),
    "corrw_open": (C.c_int, [C.POINTER(corrw_params), C.POINTER(C.c_void_p),
                             C.POINTER(corrw_resume)]),
    "corrw_write_row": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int64, C.c_uint64,
                                  C.c_uint64, C.POINTER(C.c_uint64)]),
    "corrw_sync": (C.c_int, [C.c_void_p]),
    "corrw_stats_get": (C.c_int, [C.c_void_p, C.POINTER(corrw_stats)]),
    "corrw_close": (C.c_int, [C.c_void_p]),
}

_lib: C.CDLL | None = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load the in-tree libcorr_cuda.so (built by build.py) and bind every entry point.

    Raises if the library is missing: there is no fallback implementation.
    """
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; "
            "g.build()'); this package has no CPU fallback")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class CorrError(RuntimeError):
    """A failing corr_status together with corr_last_error()."""

    def __init__(self, status: int, what: str, message: str):
        self.status = status
        self.status_name = STATUS_NAMES.get(status, f"status {status}")
        self.message = message
        super().__init__(f"{what} failed: {self.status_name} ({message})")


def check(status: int, what: str) -> None:
    if status != 0:
        msg = load().corr_last_error().decode(errors="replace")
        raise CorrError(status, what, msg)
