"""The reference host's own integration test, restated against this library (GPU).

corr-rs/tests/abi.rs checks that the shipped configuration, the host's view of
it and the real libcorr_cuda.so agree, and drives a short row end to end
through the staging ring. Its Rust cannot be built here, so its assertions are
restated through the same C ABI, on the geometry that config/correlator.yaml
ships: 4 enabled stations, n_freq 4096, n_cum 97792, one device, the baseline
range split, 256-frame slots and chunks, 8 block slots, 1 row per fetch.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# config/correlator.yaml (fft.n_freq, integration.n_cum, gpu.*, enabled stations)
N_STATION, N_FREQ, N_CUM = 4, 4096, 97792
FPS, CHUNK, BLOCK_SLOTS, ROWS_PER_FETCH = 256, 256, 8, 1
RANGE = 0


def shipped(pkg):
    return pkg.make_config(N_STATION, N_FREQ, FPS, CHUNK, BLOCK_SLOTS, ROWS_PER_FETCH,
                           split_mode=RANGE, devices=[0])


def test_a_context_can_be_created_from_the_shipped_config(pkg, cuda):
    """abi.rs:71-106: the staging layout the library reports."""
    with pkg.Correlator(shipped(pkg)) as c:
        frame_stride = 2 * N_FREQ
        slot_stride = frame_stride * FPS
        mask_bytes = (FPS + 7) // 8
        station_bytes = slot_stride * BLOCK_SLOTS + mask_bytes * BLOCK_SLOTS
        views = [c.staging(g) for g in range(N_STATION)]
        for v in views:
            st = v.info
            assert st.frame_stride == frame_stride
            assert st.slot_stride == slot_stride
            assert st.total_bytes == station_bytes
            assert st.validity_offset == slot_stride * BLOCK_SLOTS
            assert st.validity_bytes_per_slot == mask_bytes
            assert st.base
        addr = [C.cast(v.info.base, C.c_void_p).value for v in views]
        for a, b in zip(addr, addr[1:]):   # stations back to back
            assert b == a + station_bytes


def test_a_full_row_runs_through_the_staging_ring(pkg, cuda):
    """abi.rs:155-224: a short row through the ring; a slot handed over twice, a
    second unfetched row and a too-small fetch buffer are refused; silence in
    the zeroed staging gives exactly zero visibilities."""
    lib = pkg.abi.load()
    with pkg.Correlator(shipped(pkg)) as c:
        short_row = min(N_CUM, 3 * FPS)
        submits, done = 0, 0
        while done < short_row:
            ft = min(short_row - done, FPS)
            if submits >= BLOCK_SLOTS:
                c.row_slot_free(submits - BLOCK_SLOTS)
            c.row_accumulate(submits, ft)
            assert lib.corr_row_accumulate(c.ctx, submits, ft) != 0, \
                "a slot already handed over must not be accepted twice"
            submits += 1
            done += ft
        c.row_end(short_row)
        assert c.rows_pending() == 1
        assert lib.corr_row_end(c.ctx, short_row) != 0, \
            "closing a row with an unfetched row on the stack must be refused"
        c.rows_wait()
        out = np.empty(c.fetch_bytes() // 8, dtype=np.complex64)
        rows = c.rows_fetch(out)
        assert rows.shape[0] == 1
        assert c.rows_pending() == 0
        assert not np.any(out.view(np.uint8)), "zero input produced nonzero output bytes"
        for i in range(submits - 1, max(submits - BLOCK_SLOTS, 0) - 1, -1):
            c.row_slot_free(i)
        tiny = np.zeros(1, dtype=np.complex64)
        n = C.c_int32(-1)
        assert lib.corr_rows_fetch(c.ctx, tiny.ctypes.data_as(C.c_void_p), tiny.nbytes,
                                   C.byref(n)) != 0


def test_bad_slots_and_frame_counts_are_rejected(pkg, cuda):
    """abi.rs:226-254."""
    lib = pkg.abi.load()
    with pkg.Correlator(shipped(pkg)) as c:
        assert lib.corr_row_accumulate(c.ctx, 0, 0) != 0
        assert lib.corr_row_accumulate(c.ctx, 0, FPS + 1) != 0
        assert lib.corr_row_end(c.ctx, 0) != 0
        assert lib.corr_row_slot_free(c.ctx, 0) != 0


def test_destroying_a_context_repeatedly_is_safe(pkg, cuda):
    """abi.rs:256-261."""
    for _ in range(3):
        with pkg.Correlator(shipped(pkg)):
            pass
