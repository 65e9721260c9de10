"""ABI behaviour on the GPU: the reference's abi_smoke.c and async_notify.c checks.

Staging layout and zero initialisation, the validity-mask lifecycle, the slot
state machine (BUSY on double submit, STATE on freeing an unsubmitted slot),
the row stack (BUSY when full), zero input -> zero output, reuse after fetch,
and the callback forms (corr-cuda/tests/abi_smoke.c:157-371,
corr-cuda/tests/async_notify.c).
"""

from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OK, ARG, STATE, BUSY = 0, 1, 5, 6


def smoke_config(pkg):
    return pkg.make_config(4, 4096, 16, 8, 3, 2)


def mark_all_valid(c, slot):
    for g in range(c.cfg.n_station):
        c.staging(g).mask[slot, :] = 0xFF


def test_staging_layout_and_mask_lifecycle(pkg, cuda):
    cfg = smoke_config(pkg)
    with pkg.Correlator(cfg) as c:
        lib = c.lib
        fs = 2 * cfg.n_freq
        ss = fs * cfg.frames_per_slot
        samples = ss * cfg.block_slots
        mb = (cfg.frames_per_slot + 7) // 8
        station_stride = samples + mb * cfg.block_slots
        prev = None
        for g in range(cfg.n_station):
            info = c.staging(g).info
            assert info.frame_stride == fs and info.slot_stride == ss
            assert info.validity_bytes_per_slot == mb and info.validity_offset == samples
            assert info.total_bytes == station_stride
            base = C.cast(info.base, C.c_void_p).value
            if prev is not None:
                assert base == prev + station_stride
            prev = base
        st = pkg.abi.corr_staging()
        assert lib.corr_staging_info(c.ctx, cfg.n_station, C.byref(st)) == ARG
        v0 = c.staging(0)
        assert not v0.samples.any() and not v0.mask.any()   # zero initialised
        v0.mask[0, :] = 0xAA
        c.row_accumulate(0, cfg.frames_per_slot)
        c.row_slot_free(0)
        assert not v0.mask.any(), "slot_free must clear the slot's mask"


def test_state_machine_and_row_stack(pkg, cuda):
    cfg = smoke_config(pkg)
    with pkg.Correlator(cfg) as c:
        lib, ctx = c.lib, c.ctx
        row_bytes = c.n_baseline * cfg.n_freq * 8
        out = np.zeros(row_bytes * cfg.rows_per_fetch // 8, dtype=np.complex64)
        rows = C.c_int32(-1)
        assert lib.corr_row_slot_free(ctx, 1) == STATE
        assert lib.corr_row_accumulate(ctx, -1, 1) == ARG
        assert lib.corr_rows_fetch(ctx, out.ctypes.data_as(C.c_void_p), out.nbytes, None) == ARG
        assert lib.corr_rows_fetch(ctx, out.ctypes.data_as(C.c_void_p), 8, C.byref(rows)) == ARG
        assert c.rows_pending() == 0
        assert c.rows_fetch(out).shape[0] == 0
        assert lib.corr_row_accumulate(ctx, 0, 0) == ARG
        assert lib.corr_row_accumulate(ctx, 0, cfg.frames_per_slot + 1) == ARG
        assert lib.corr_row_end(ctx, 0) == ARG
        for seq in range(cfg.block_slots):
            slot = seq % cfg.block_slots
            mark_all_valid(c, slot)
            c.row_accumulate(seq, cfg.frames_per_slot)
            assert lib.corr_row_accumulate(ctx, seq, cfg.frames_per_slot) == BUSY
            c.row_slot_free(seq)
            assert lib.corr_row_slot_free(ctx, seq) == STATE
            if slot % 2 == 1:
                c.row_end(cfg.frames_per_slot)
        assert c.rows_pending() == 1
        c.row_end(cfg.frames_per_slot)
        assert lib.corr_row_end(ctx, cfg.frames_per_slot) == BUSY   # stack of 2 is full
        c.rows_wait()
        got = c.rows_fetch(out)
        assert got.shape[0] == 2
        assert not np.any(got), "all-zero staging must give an all-zero row"
        # fetching clears the rows; the pipeline cycles
        for i in range(cfg.block_slots):
            seq = cfg.block_slots + i
            mark_all_valid(c, seq % cfg.block_slots)
            c.row_accumulate(seq, cfg.frames_per_slot)
            c.row_slot_free(seq)
        c.row_end(cfg.frames_per_slot)
        c.rows_wait()
        assert c.rows_fetch(out).shape[0] == 1
        st = c.stats()
        assert st.transfers > 0 and st.bytes_h2d > 0 and st.bytes_d2h == 3 * row_bytes
    assert pkg.abi.load().corr_destroy(None) == OK


def test_device_introspection(pkg, cuda):
    cfg = smoke_config(pkg)
    with pkg.Correlator(cfg) as c:
        lib = c.lib
        assert lib.corr_n_devices(c.ctx) == 1
        plan = pkg.abi.corr_device_plan()
        assert lib.corr_device_plan_get(c.ctx, 0, C.byref(plan)) == OK
        assert (plan.n_station_resident, plan.first_baseline, plan.n_baseline,
                plan.contiguous) == (4, 0, 10, 1)
        assert lib.corr_device_plan_get(c.ctx, 1, C.byref(plan)) == ARG
        st = (C.c_int32 * 4)()
        assert lib.corr_device_stations(c.ctx, 0, st, 4) == OK and list(st) == [0, 1, 2, 3]
        assert lib.corr_device_stations(c.ctx, 0, st, 3) == ARG
        bl = (C.c_int32 * 10)()
        assert lib.corr_device_baselines(c.ctx, 0, bl, 10) == OK and list(bl) == list(range(10))


def test_multi_device_config_checks(pkg, cuda, lib):
    """Repeated or invisible devices are refused; distinct visible ones are accepted."""
    cfg = smoke_config(pkg)
    n = cuda.cuda.device_count()
    cfg.n_devices = 2
    cfg.devices[0] = 0
    cfg.devices[1] = 0   # repeated entry
    ctx = C.c_void_p()
    assert lib.corr_create(C.byref(cfg), C.byref(ctx)) == ARG
    if n >= 2:
        cfg.devices[1] = 1
        assert lib.corr_create(C.byref(cfg), C.byref(ctx)) == OK
        assert lib.corr_n_devices(ctx) == 2
        assert lib.corr_destroy(ctx) == OK
    cfg.n_devices = 1
    cfg.devices[0] = n   # out of range
    assert lib.corr_create(C.byref(cfg), C.byref(ctx)) == ARG


def test_callbacks(pkg, cuda):
    """Submit forms: callbacks fire once per submit; finish completes the release."""
    cfg = pkg.make_config(2, 8192, 256, 64, 3, 1)
    count = {"n": 0}
    lock = threading.Lock()

    @pkg.abi.NOTIFY_FN
    def on_done(_user):
        with lock:
            count["n"] += 1

    def wait_for(n, seconds=20.0):
        t0 = time.time()
        while time.time() - t0 < seconds:
            with lock:
                if count["n"] >= n:
                    return True
            time.sleep(0.001)
        return False

    rng = np.random.default_rng(3)
    with pkg.Correlator(cfg) as c:
        lib, ctx = c.lib, c.ctx
        for g in range(cfg.n_station):
            c.staging(g).samples[:] = rng.integers(-8, 8, size=c.staging(g).samples.shape)
        assert lib.corr_row_slot_free_submit(ctx, 0, on_done, None) == STATE
        mark_all_valid(c, 0)
        c.row_accumulate(0, cfg.frames_per_slot)
        assert lib.corr_row_slot_free_submit(ctx, 0, on_done, None) == OK
        assert wait_for(1)
        assert lib.corr_row_slot_free_finish(ctx, 0) == OK
        assert not c.staging(0).mask[0].any()
        assert lib.corr_row_slot_free_finish(ctx, 0) == STATE
        # N submits deliver N callbacks
        for seq in range(1, 4):
            mark_all_valid(c, seq % 3)
            c.row_accumulate(seq, cfg.frames_per_slot)
            assert lib.corr_row_slot_free_submit(ctx, seq, on_done, None) == OK
        assert wait_for(4)
        for seq in range(1, 4):
            assert lib.corr_row_slot_free_finish(ctx, seq) == OK
        c.row_end(4 * cfg.frames_per_slot)
        assert lib.corr_rows_wait_submit(ctx, on_done, None) == OK
        assert wait_for(5)
        assert lib.corr_rows_ready(ctx) == OK
        out = np.zeros(c.fetch_bytes() // 8, dtype=np.complex64)
        rows = C.c_int32(-1)
        assert lib.corr_rows_fetch_submit(ctx, out.ctypes.data_as(C.c_void_p), out.nbytes,
                                          C.byref(rows), on_done, None) == OK
        assert rows.value == 1
        assert wait_for(6)
        assert lib.corr_rows_fetch_ready(ctx) == OK
        assert np.abs(out).max() > 0


def test_contexts_leave_no_device_memory_behind(pkg, cuda):
    """Creating and destroying contexts over and over (one device, and four
    configured devices of each split on the one GPU) returns every device byte:
    free memory after twelve cycles is what it was after the first."""
    torch = cuda

    def cycle(devices, split):
        if len(devices) > 1:
            pkg.set_device_map([0] * len(devices))
        try:
            cfg = pkg.make_config(8, 4096, 64, 32, 3, 2, split_mode=split, devices=devices)
            with pkg.Correlator(cfg) as c:
                for g in range(8):
                    c.staging(g).mask[0, :] = 0xFF
                c.row_accumulate(0, 64)
                c.row_end(64)
                c.rows_wait()
                c.rows_fetch()
                c.row_slot_free(0)
        finally:
            pkg.set_device_map(None)
        torch.cuda.synchronize()

    forms = [([0], 0), ([0, 1, 2, 3], 0), ([0, 1, 2, 3], 1), ([0, 1, 2, 3], 2)]
    for d, s in forms:            # first use: kernel modules and per-device set-up
        cycle(d, s)
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        for d, s in forms:
            cycle(d, s)
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 < 8 << 20, f"{(free0 - free1) >> 20} MiB not returned"
