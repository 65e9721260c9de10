"""Python host side of the C ABI: the `Correlator` the scheduler drives.

Mirrors the reference's safe Rust wrapper (corr-rs/src/gpu.rs:54-318):
`Correlator.new`, `row_accumulate`, `row_slot_free`, `row_end`, `rows_wait`,
`rows_pending`, `rows_fetch`, plus `staging(station)` returning numpy views of
the pinned staging ring the receive side writes. Every call goes through
libcorr_cuda.so; failures raise `CorrError` carrying the status and
corr_last_error(), as gpu.rs's `check` does.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi


@dataclass(frozen=True)
class StagingView:
    """One station's staging region as numpy arrays over the pinned memory."""

    samples: np.ndarray   # int8 [block_slots, frames_per_slot, 2*n_freq]
    mask: np.ndarray      # uint8 [block_slots, validity_bytes_per_slot]
    info: abi.corr_staging


def make_config(n_station: int, n_freq: int, frames_per_slot: int, chunk_frames: int,
                block_slots: int = 3, rows_per_fetch: int = 1, device_id: int = 0,
                split_mode: int = abi.CORR_SPLIT_BASELINE_RANGE,
                devices: list[int] | None = None) -> abi.corr_config:
    """A corr_config; `devices` (up to CORR_MAX_DEVICES ordinals) spreads the run
    over several devices with `split_mode`, else device_id alone is used."""
    cfg = abi.corr_config()
    cfg.abi_version = abi.CORR_ABI_VERSION
    cfg.struct_size = C.sizeof(abi.corr_config)
    cfg.device_id = device_id
    cfg.n_station = n_station
    cfg.n_freq = n_freq
    cfg.frames_per_slot = frames_per_slot
    cfg.chunk_frames = chunk_frames
    cfg.block_slots = block_slots
    cfg.rows_per_fetch = rows_per_fetch
    cfg.n_devices = 0
    if devices:
        cfg.n_devices = len(devices)
        for i, d in enumerate(devices):
            cfg.devices[i] = d
    cfg.split_mode = split_mode
    return cfg


def plan_query(cfg: abi.corr_config, device_index: int) -> dict:
    """The placement corr_create makes for `cfg` on one device (corrx_plan_query),
    computed on the host without a GPU."""
    lib = abi.load()
    plan = abi.corr_device_plan()
    nb = lib.corr_n_baseline(cfg.n_station)
    st = (C.c_int32 * cfg.n_station)()
    bl = (C.c_int32 * nb)()
    lo = (C.c_int32 * nb)()
    abi.check(lib.corrx_plan_query(C.byref(cfg), device_index, C.byref(plan), st, cfg.n_station,
                                   bl, nb, lo, nb), "corrx_plan_query")
    return {"device_id": plan.device_id, "n_station_resident": plan.n_station_resident,
            "first_baseline": plan.first_baseline, "n_baseline": plan.n_baseline,
            "contiguous": bool(plan.contiguous),
            "stations": list(st[:plan.n_station_resident]),
            "baselines": list(bl[:plan.n_baseline]), "local": list(lo[:plan.n_baseline])}


def set_device_map(physical: list[int] | None) -> None:
    """Run configured device i of later contexts on CUDA device physical[i]
    (corrx_set_device_map); None or [] restores the identity."""
    lib = abi.load()
    phys = physical or []
    arr = (C.c_int32 * max(1, len(phys)))(*phys)
    abi.check(lib.corrx_set_device_map(arr, len(phys)), "corrx_set_device_map")


class Correlator:
    """An owned correlator context (one driving thread, like gpu.rs's Correlator)."""

    def __init__(self, cfg: abi.corr_config):
        self.lib = abi.load()
        self.cfg = cfg
        ctx = C.c_void_p()
        abi.check(self.lib.corr_create(C.byref(cfg), C.byref(ctx)), "corr_create")
        if not ctx.value:
            raise RuntimeError("corr_create reported success but returned a NULL context")
        self.ctx = ctx
        self.n_baseline = self.lib.corr_n_baseline(cfg.n_station)
        self._views: dict[int, StagingView] = {}

    @classmethod
    def new(cls, n_station: int, n_freq: int, frames_per_slot: int, chunk_frames: int,
            block_slots: int = 3, rows_per_fetch: int = 1, device_id: int = 0) -> "Correlator":
        return cls(make_config(n_station, n_freq, frames_per_slot, chunk_frames, block_slots,
                               rows_per_fetch, device_id))

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if self.ctx is not None and self.ctx.value:
            self._views.clear()
            abi.check(self.lib.corr_destroy(self.ctx), "corr_destroy")
        self.ctx = None

    def __enter__(self) -> "Correlator":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    # -- staging ----------------------------------------------------------
    def staging(self, station: int) -> StagingView:
        if station in self._views:
            return self._views[station]
        info = abi.corr_staging()
        abi.check(self.lib.corr_staging_info(self.ctx, station, C.byref(info)),
                  "corr_staging_info")
        base = C.cast(info.base, C.c_void_p).value
        buf = (C.c_int8 * info.total_bytes).from_address(base)
        whole = np.frombuffer(buf, dtype=np.int8)
        nsamp = info.validity_offset
        samples = whole[:nsamp].reshape(self.cfg.block_slots, self.cfg.frames_per_slot,
                                        info.frame_stride)
        mask = whole[nsamp:nsamp + info.validity_bytes_per_slot * self.cfg.block_slots].view(
            np.uint8).reshape(self.cfg.block_slots, info.validity_bytes_per_slot)
        view = StagingView(samples, mask, info)
        self._views[station] = view
        return view

    # -- rows -------------------------------------------------------------
    def row_accumulate(self, slot_seq: int, frames: int) -> None:
        abi.check(self.lib.corr_row_accumulate(self.ctx, slot_seq, frames), "corr_row_accumulate")

    def row_slot_free(self, slot_seq: int) -> None:
        abi.check(self.lib.corr_row_slot_free(self.ctx, slot_seq), "corr_row_slot_free")

    def row_end(self, frames: int) -> None:
        abi.check(self.lib.corr_row_end(self.ctx, frames), "corr_row_end")

    def rows_wait(self) -> None:
        abi.check(self.lib.corr_rows_wait(self.ctx), "corr_rows_wait")

    def rows_pending(self) -> int:
        out = C.c_int32(-1)
        abi.check(self.lib.corr_rows_pending(self.ctx, C.byref(out)), "corr_rows_pending")
        return out.value

    def fetch_bytes(self) -> int:
        return self.n_baseline * self.cfg.n_freq * 8 * self.cfg.rows_per_fetch

    def rows_fetch(self, out: np.ndarray | None = None) -> np.ndarray:
        """Fetch the closed rows as complex64 [rows, n_baseline, n_freq]."""
        if out is None:
            out = np.empty(self.fetch_bytes() // 8, dtype=np.complex64)
        assert out.dtype == np.complex64 and out.flags.c_contiguous
        rows = C.c_int32(-1)
        abi.check(self.lib.corr_rows_fetch(self.ctx, out.ctypes.data_as(C.c_void_p), out.nbytes,
                                           C.byref(rows)), "corr_rows_fetch")
        per_row = self.n_baseline * self.cfg.n_freq
        return out[:rows.value * per_row].reshape(rows.value, self.n_baseline, self.cfg.n_freq)

    def set_xengine(self, mode: int) -> None:
        abi.check(self.lib.corr_set_xengine(self.ctx, mode), "corr_set_xengine")

    def autotune(self) -> dict:
        """Pick the fastest spectra layout and tensor X tile for this context's engine."""
        t = abi.corrx_tiles(struct_size=C.sizeof(abi.corrx_tiles))
        abi.check(self.lib.corr_autotune(self.ctx, C.byref(t)), "corr_autotune")
        return {"ytile": t.ytile, "xct": t.xct, "xkt": t.xkt, "fplan": t.fplan,
                "ms_fengine": t.ms_fengine, "ms_xengine": t.ms_xengine}

    def tiles(self) -> dict:
        t = abi.corrx_tiles(struct_size=C.sizeof(abi.corrx_tiles))
        abi.check(self.lib.corr_get_tiles(self.ctx, C.byref(t)), "corr_get_tiles")
        return {"ytile": t.ytile, "xct": t.xct, "xkt": t.xkt, "fplan": t.fplan}

    def set_tiles(self, ytile: int, xct: int = 0, xkt: int = 0, fplan: int = 0) -> None:
        """Spectra layout, tensor X tile and FFT plan (2: the tensor-core FFT, FP16 form)."""
        t = abi.corrx_tiles(struct_size=C.sizeof(abi.corrx_tiles), ytile=ytile, xct=xct, xkt=xkt,
                            fplan=fplan)
        abi.check(self.lib.corr_set_tiles(self.ctx, C.byref(t)), "corr_set_tiles")

    def stats(self, device_index: int = 0) -> abi.corr_device_stats:
        st = abi.corr_device_stats()
        abi.check(self.lib.corr_device_stats_get(self.ctx, device_index, C.byref(st)),
                  "corr_device_stats_get")
        return st

    def n_devices(self) -> int:
        return self.lib.corr_n_devices(self.ctx)

    def device_plan(self, device_index: int) -> dict:
        """What device `device_index` holds and owns (corr_device_plan_get,
        corr_device_stations, corr_device_baselines)."""
        plan = abi.corr_device_plan()
        abi.check(self.lib.corr_device_plan_get(self.ctx, device_index, C.byref(plan)),
                  "corr_device_plan_get")
        st = (C.c_int32 * max(1, plan.n_station_resident))()
        bl = (C.c_int32 * max(1, plan.n_baseline))()
        abi.check(self.lib.corr_device_stations(self.ctx, device_index, st,
                                                plan.n_station_resident), "corr_device_stations")
        abi.check(self.lib.corr_device_baselines(self.ctx, device_index, bl, plan.n_baseline),
                  "corr_device_baselines")
        return {"device_id": plan.device_id, "n_station_resident": plan.n_station_resident,
                "first_baseline": plan.first_baseline, "n_baseline": plan.n_baseline,
                "contiguous": bool(plan.contiguous),
                "stations": list(st[:plan.n_station_resident]),
                "baselines": list(bl[:plan.n_baseline])}

    @staticmethod
    def baseline_pairs(n_station: int) -> list[tuple[int, int]]:
        lib = abi.load()
        nb = lib.corr_n_baseline(n_station)
        arr = (C.c_int32 * (2 * nb))()
        abi.check(lib.corr_baseline_pairs(n_station, arr, 2 * nb), "corr_baseline_pairs")
        return [(arr[2 * i], arr[2 * i + 1]) for i in range(nb)]
