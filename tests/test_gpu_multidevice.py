"""Multi-device contexts (time slice, baseline range, pair covering) on the GPU.

The reference's own criterion (corr-cuda/tests/multi_device.c:1-13): splitting
the run over N devices must not change the numbers. A machine with one GPU
runs the N configured devices on it through corrx_set_device_map (each with its
own buffers, streams, engine and share of the slots); the code path is the one
N GPUs take, with peer copies between equal devices. Rows integrate in
complex128, so the partial rows of a time slice add up to the single-device row
bit for bit here, and the range split and pair covering place bit-identical
baselines. Placement and rows are also checked against the float64 oracle.
Same geometry as multi_device.c: 8 stations, n_freq 2048, 3 rows of 96 frames
in 32-frame slots, 16-frame chunks, 3 rows per fetch.
"""

from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np
import pytest

from abi_driver import drive_rows

pytestmark = pytest.mark.gpu

N, NF, N_CUM, FPS, CHUNK, ROWS = 8, 2048, 96, 32, 16, 3
RANGE, COVER, SLICE = 0, 1, 2


@pytest.fixture
def shared_gpu(pkg, cuda):
    """Eight configured devices, all on CUDA device 0."""
    pkg.set_device_map([0] * 8)
    try:
        yield
    finally:
        pkg.set_device_map(None)


@pytest.fixture(scope="module")
def frames():
    rng = np.random.default_rng(20260914)
    return rng.integers(-16, 16, size=(ROWS, N, N_CUM, 2 * NF), dtype=np.int8)


@pytest.fixture(scope="module")
def one_device(pkg, cuda, frames):
    return drive_rows(pkg, frames, N_CUM, FPS, chunk_frames=CHUNK, block_slots=3,
                      rows_per_fetch=ROWS)


def run(pkg, frames, n_dev, split, xmode=0, plans=None):
    return drive_rows(pkg, frames, N_CUM, FPS, chunk_frames=CHUNK, block_slots=3,
                      rows_per_fetch=ROWS, devices=list(range(n_dev)), split_mode=split,
                      xmode=xmode, plans=plans)


def test_one_device_matches_the_oracle(oracle, frames, one_device):
    ref = oracle.correlate_rows(frames, N_CUM)
    assert oracle.rel_rms(one_device, ref) < 1e-6
    assert oracle.normalized_max_err(one_device, ref, N) < 1e-5


@pytest.mark.parametrize("n_dev", [2, 3, 4])
def test_time_slice_equals_one_device(pkg, shared_gpu, frames, one_device, n_dev):
    plans = []
    got = run(pkg, frames, n_dev, SLICE, plans=plans)
    assert len(plans) == n_dev
    for d, p in enumerate(plans):
        assert p["device_id"] == d and p["n_station_resident"] == N
        assert p["stations"] == list(range(N)) and p["baselines"] == list(range(N * (N + 1) // 2))
    assert got.tobytes() == one_device.tobytes(), (
        f"{n_dev}-way time slice differs from one device in "
        f"{np.count_nonzero(got != one_device)} values")


@pytest.mark.parametrize("n_dev", [2, 4, 8])
def test_baseline_range_equals_one_device(pkg, shared_gpu, frames, one_device, n_dev):
    plans = []
    got = run(pkg, frames, n_dev, RANGE, plans=plans)
    nxt = 0
    for p in plans:
        assert p["contiguous"] and p["first_baseline"] == nxt
        nxt += p["n_baseline"]
    assert nxt == N * (N + 1) // 2
    assert got.tobytes() == one_device.tobytes()


@pytest.mark.parametrize("n_dev", [3, 4, 6])
def test_pair_covering_equals_one_device(pkg, shared_gpu, frames, one_device, n_dev):
    plans = []
    got = run(pkg, frames, n_dev, COVER, plans=plans)
    sizes = [p["n_station_resident"] for p in plans]
    assert max(sizes) < N and max(sizes) - min(sizes) <= 1
    owned = sorted(b for p in plans for b in p["baselines"])
    assert owned == list(range(N * (N + 1) // 2))
    assert got.tobytes() == one_device.tobytes(), (
        f"pair covering differs in {np.count_nonzero(got != one_device)} values")


@pytest.mark.parametrize("xmode", [1, 2])
@pytest.mark.parametrize("split,n_dev", [(SLICE, 4), (COVER, 4), (RANGE, 3)])
def test_tensor_forms_split_over_devices(pkg, shared_gpu, oracle, frames, xmode, split, n_dev):
    """The tensor X-engines on every share: the same rows as on one device
    (within float rounding of a different station count per device for pair
    covering), and within their bounds against the oracle."""
    one = drive_rows(pkg, frames, N_CUM, FPS, chunk_frames=CHUNK, block_slots=3,
                     rows_per_fetch=ROWS, xmode=xmode)
    got = run(pkg, frames, n_dev, split, xmode=xmode)
    if split == COVER:
        assert oracle.rel_rms(got, one) < 1e-7
    else:
        assert got.tobytes() == one.tobytes()
    ref = oracle.correlate_rows(frames, N_CUM)
    bar = 1e-5 if xmode == 2 else 1.5e-3 / np.sqrt(N_CUM)
    assert oracle.rel_rms(got, ref) < bar


def test_time_slice_routes_slots_and_counts_bytes(pkg, shared_gpu, frames):
    """Slot sequence s goes to device s % n_devices: each device copies only its
    slots; the others hand their partial rows to device 0, which alone copies
    rows to the host."""
    cfg = pkg.make_config(N, NF, FPS, CHUNK, 3, ROWS, split_mode=SLICE, devices=[0, 1, 2])
    with pkg.Correlator(cfg) as c:
        seq = 0
        for r in range(ROWS):
            for f0 in range(0, N_CUM, FPS):
                if seq >= 3:
                    c.row_slot_free(seq)
                for g in range(N):
                    c.staging(g).samples[seq % 3, :FPS] = frames[r, g, f0:f0 + FPS]
                    c.staging(g).mask[seq % 3, :] = 0xFF
                c.row_accumulate(seq, FPS)
                seq += 1
            c.row_end(N_CUM)
        for s in range(seq - 1, seq - 4, -1):
            c.row_slot_free(s)
        c.rows_wait()
        out = c.rows_fetch()
        assert out.shape[0] == ROWS
        # per slot and station: its frames, and the slot's mask once per chunk
        frame_bytes = 2 * NF * FPS + (FPS // CHUNK) * (FPS // 8)
        row64 = N * (N + 1) // 2 * NF * 16
        for d in range(3):
            st = c.stats(d)
            assert st.device_id == d
            slots = sum(1 for s in range(seq) if s % 3 == d)
            assert st.transfers == slots * (FPS // CHUNK)
            assert st.bytes_h2d == slots * N * frame_bytes
            if d > 0:
                assert st.bytes_d2h == ROWS * row64
        assert c.stats(0).bytes_d2h == out.nbytes


def test_multi_device_callbacks(pkg, shared_gpu, frames):
    """Submit forms over three devices: each callback fires once, after the
    copies of every device that read the slot (all three under pair covering);
    pair covering's scattered baselines refuse the fetch without waiting
    (CORR_ERR_NOT_IMPL, as the reference's async_notify.c expects)."""
    for split in (SLICE, COVER):
        cfg = pkg.make_config(N, NF, FPS, CHUNK, 3, 1, split_mode=split, devices=[0, 1, 2])
        fired = {"slot": 0, "rows": 0, "fetch": 0}
        lock = threading.Lock()

        def bump(key):
            def cb(_user):
                with lock:
                    fired[key] += 1
            return pkg.abi.NOTIFY_FN(cb)

        cbs = {k: bump(k) for k in fired}
        with pkg.Correlator(cfg) as c:
            lib = c.lib
            for g in range(N):
                c.staging(g).samples[0, :FPS] = frames[0, g, :FPS]
                c.staging(g).mask[0, :] = 0xFF
            c.row_accumulate(0, FPS)
            assert lib.corr_row_slot_free_submit(c.ctx, 0, cbs["slot"], None) == 0
            c.row_end(FPS)
            assert lib.corr_rows_wait_submit(c.ctx, cbs["rows"], None) == 0
            out = np.empty(c.fetch_bytes() // 8, dtype=np.complex64)
            rows = C.c_int32(-1)
            st = lib.corr_rows_fetch_submit(c.ctx, out.ctypes.data_as(C.c_void_p), out.nbytes,
                                            C.byref(rows), cbs["fetch"], None)
            if split == COVER:
                # as the reference: scattered baselines have only the blocking fetch
                assert st == 8, "pair covering's fetch without waiting must be NOT_IMPL"
                assert c.rows_fetch().shape[0] == 1
                fired["fetch"] += 1
            else:
                assert st == 0 and rows.value == 1
            t0 = time.time()
            while (fired["slot"], fired["rows"], fired["fetch"]) != (1, 1, 1):
                assert time.time() - t0 < 30, f"callbacks did not all fire: {fired}"
                time.sleep(0.01)
            assert lib.corr_rows_fetch_ready(c.ctx) == 0
            assert lib.corr_row_slot_free_finish(c.ctx, 0) == 0
            assert not c.staging(0).mask[0].any()


def test_device_map_arguments(pkg, lib, cuda):
    bad = (C.c_int32 * 1)(-1)
    assert lib.corrx_set_device_map(bad, 1) == 1
    assert lib.corrx_set_device_map(None, 2) == 1
    assert lib.corrx_set_device_map(None, 0) == 0
    pkg.set_device_map([0, 0])
    try:
        # ordinals beyond the map are not visible devices
        cfg = pkg.make_config(N, NF, FPS, CHUNK, 3, 1, split_mode=SLICE, devices=[0, 2])
        ctx = C.c_void_p()
        assert lib.corr_create(C.byref(cfg), C.byref(ctx)) == 1
        assert b"visible" in lib.corr_last_error()
    finally:
        pkg.set_device_map(None)


@pytest.mark.skipif("not __import__('torch').cuda.is_available() or "
                    "__import__('torch').cuda.device_count() < 2")
def test_two_physical_devices_in_one_process(pkg, cuda, frames, one_device):
    """Kernel attributes are set per device: a context on two real GPUs works
    from the first call on each."""
    got = run(pkg, frames, 2, SLICE)
    assert got.tobytes() == one_device.tobytes()


@pytest.mark.parametrize("split,n_dev", [(RANGE, 2), (COVER, 3)])
def test_more_than_44_stations_split_over_devices(pkg, shared_gpu, oracle, split, n_dev):
    """The reference limits baselines per device (corr-cuda/src/kernels.cu:474-483):
    50 stations (1275 baselines) are accepted once the split leaves every device
    at most 1024, and give the oracle's rows; the time slice, which gives every
    device every baseline, is refused."""
    n, nf, n_cum, fps = 50, 2048, 32, 32
    rng = np.random.default_rng(5000 + split)
    x = rng.integers(-30, 31, size=(1, n, n_cum, 2 * nf), dtype=np.int8)
    plans = []
    got = drive_rows(pkg, x, n_cum, fps, chunk_frames=16, block_slots=3, rows_per_fetch=1,
                     devices=list(range(n_dev)), split_mode=split, plans=plans)
    assert max(p["n_baseline"] for p in plans) <= 1024
    ref = oracle.correlate_rows(x, n_cum)
    assert oracle.rel_rms(got, ref) < 1e-5
    assert oracle.normalized_max_err(got, ref, n) < 1e-5
    cfg = pkg.make_config(n, nf, fps, 16, 3, 1, split_mode=SLICE, devices=[0, 1])
    ctx = C.c_void_p()
    assert pkg.abi.load().corr_create(C.byref(cfg), C.byref(ctx)) == pkg.abi.CORR_ERR_ARG
