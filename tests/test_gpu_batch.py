"""Integration blocks of uneven length in one CUDA-graph launch (corrx_batch_*).

Each block's row is checked against the oracle on exactly its frames (masks
included), the row dumped to pinned host memory must equal the device row, a
second launch of the same graph must reproduce the rows, and every block must
report a positive latency.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("acc64", [False, True], ids=["fp32rows", "fp64rows"])
@pytest.mark.parametrize("xmode", [0, 2])
def test_batch_graph_rows_match_oracle(pkg, cuda, oracle, xmode, acc64):
    """With complex128 accumulators (corrx_set_accumulator) each block integrates
    in one FP64 row of the batch and is dumped, divided, into its complex64 row."""
    torch = cuda
    lib = pkg.abi.load()
    n, nf, pool = 6, 2048, 300
    rng = np.random.default_rng(7)
    x = rng.integers(-40, 41, size=(n, pool, 2 * nf)).astype(np.int8)
    present = rng.random((n, pool)) > 0.02
    mask = np.packbits(present.astype(np.uint8), axis=1, bitorder="little")
    blocks = [(0, 17), (5, 100), (120, 33), (10, 290), (299, 1), (64, 64)]
    first = (C.c_int64 * len(blocks))(*[b[0] for b in blocks])
    frames = (C.c_int32 * len(blocks))(*[b[1] for b in blocks])
    eng = pkg.FxEngine(n, nf, max_frames=48, xmode=xmode)
    if acc64:
        eng.set_accumulator(pkg.abi.CORRX_ACC_FP64)
    xs = torch.from_numpy(x).cuda()
    ms = torch.from_numpy(mask).cuda()
    nb = n * (n + 1) // 2
    rows = torch.zeros((len(blocks), nb, nf), dtype=torch.complex64, device="cuda")
    host = torch.zeros((len(blocks), nb, nf), dtype=torch.complex64).pin_memory()
    h = C.c_void_p()
    st = lib.corrx_batch_create(eng.h, C.c_void_p(xs.data_ptr()), xs.stride(0), xs.stride(1),
                                C.c_void_p(ms.data_ptr()), ms.stride(0), first, frames,
                                len(blocks), C.c_void_p(rows.data_ptr()),
                                C.c_void_p(host.data_ptr()), C.byref(h))
    assert st == 0, lib.corr_last_error()
    stream = torch.cuda.current_stream()
    try:
        outs = []
        for _ in range(2):
            rows.fill_(float("nan"))   # the graph must clear each row itself
            assert lib.corrx_batch_launch(h, C.c_void_p(stream.cuda_stream)) == 0
            torch.cuda.synchronize()
            eng.check()
            outs.append(rows.cpu().numpy().copy())
        lat = (C.c_float * len(blocks))()
        assert lib.corrx_batch_block_ms(h, lat, len(blocks)) == 0
        assert all(v > 0 for v in lat)
        assert np.array_equal(outs[0], outs[1])
        assert np.array_equal(host.numpy(), outs[1])
        tol = 1e-5
        for i, (f0, nfr) in enumerate(blocks):
            ref = oracle.correlate(x[:, f0:f0 + nfr], present[:, f0:f0 + nfr]) / nfr
            assert oracle.rel_rms(outs[1][i], ref) < tol, i
    finally:
        lib.corrx_batch_destroy(h)
        eng.close()


def test_mixed_engine_batch_matches_each_engine_alone(pkg, cuda, oracle):
    """corrx_batch_create_mixed: long blocks on the FP16 form, short ones on the
    split form; every row equals the same block run alone on its engine."""
    torch = cuda
    lib = pkg.abi.load()
    n, nf, pool = 5, 1024, 400
    rng = np.random.default_rng(9)
    x = rng.integers(-40, 41, size=(n, pool, 2 * nf)).astype(np.int8)
    present = rng.random((n, pool)) > 0.02
    mask = np.packbits(present.astype(np.uint8), axis=1, bitorder="little")
    blocks = [(0, 17), (5, 300), (120, 33), (10, 390), (64, 64)]
    which = [1, 0, 1, 0, 1]                       # 0: FP16, 1: split
    first = (C.c_int64 * len(blocks))(*[b[0] for b in blocks])
    frames = (C.c_int32 * len(blocks))(*[b[1] for b in blocks])
    sel = (C.c_int32 * len(blocks))(*which)
    engs = [pkg.FxEngine(n, nf, max_frames=64, xmode=1), pkg.FxEngine(n, nf, max_frames=64, xmode=2)]
    handles = (C.c_void_p * 2)(engs[0].h.value, engs[1].h.value)
    xs = torch.from_numpy(x).cuda()
    ms = torch.from_numpy(mask).cuda()
    nb = n * (n + 1) // 2
    rows = torch.zeros((len(blocks), nb, nf), dtype=torch.complex64, device="cuda")
    h = C.c_void_p()
    st = lib.corrx_batch_create_mixed(handles, 2, sel, C.c_void_p(xs.data_ptr()), xs.stride(0),
                                      xs.stride(1), C.c_void_p(ms.data_ptr()), ms.stride(0),
                                      first, frames, len(blocks), C.c_void_p(rows.data_ptr()),
                                      None, C.byref(h))
    assert st == 0, lib.corr_last_error()
    stream = torch.cuda.current_stream()
    try:
        assert lib.corrx_batch_launch(h, C.c_void_p(stream.cuda_stream)) == 0
        torch.cuda.synchronize()
        for e in engs:
            e.check()
        got = rows.cpu().numpy()
        lat = (C.c_float * len(blocks))()
        assert lib.corrx_batch_block_ms(h, lat, len(blocks)) == 0
        for i, (f0, nfr) in enumerate(blocks):
            acc = engs[which[i]].new_acc()
            engs[which[i]].accumulate(xs, nfr, acc, mask=ms, mask_bit0=f0, frame0=f0)
            engs[which[i]].scale(acc, nfr)
            torch.cuda.synchronize()
            assert np.array_equal(got[i], acc.cpu().numpy()), i
            ref = oracle.correlate(x[:, f0:f0 + nfr], present[:, f0:f0 + nfr]) / nfr
            bar = 1e-5 if which[i] else 1.5e-3 / np.sqrt(nfr)
            assert oracle.rel_rms(got[i], ref) < bar, i
        # engines of different geometry, or a block naming no engine, are refused
        other = pkg.FxEngine(n + 1, nf, max_frames=64, xmode=2)
        try:
            h2 = C.c_void_p()
            bad = (C.c_void_p * 2)(engs[0].h.value, other.h.value)
            assert lib.corrx_batch_create_mixed(
                bad, 2, sel, C.c_void_p(xs.data_ptr()), xs.stride(0), xs.stride(1),
                C.c_void_p(ms.data_ptr()), ms.stride(0), first, frames, len(blocks),
                C.c_void_p(rows.data_ptr()), None, C.byref(h2)) == pkg.abi.CORR_ERR_ARG
            sel_bad = (C.c_int32 * len(blocks))(0, 1, 2, 0, 1)
            assert lib.corrx_batch_create_mixed(
                handles, 2, sel_bad, C.c_void_p(xs.data_ptr()), xs.stride(0), xs.stride(1),
                C.c_void_p(ms.data_ptr()), ms.stride(0), first, frames, len(blocks),
                C.c_void_p(rows.data_ptr()), None, C.byref(h2)) == pkg.abi.CORR_ERR_ARG
        finally:
            other.close()
    finally:
        lib.corrx_batch_destroy(h)
        for e in engs:
            e.close()


@pytest.mark.parametrize("xmode", [0, 2])
def test_packet_batch_matches_oracle(pkg, cuda, oracle, xmode):
    """corrx_batch_create_packets: lost 1024-sample packets zero-filled per block,
    word f of a station belonging to pool frame f; a frame mask combines with it."""
    torch = cuda
    lib = pkg.abi.load()
    n, nf, pool = 5, 4096, 260
    rng = np.random.default_rng(11)
    x = rng.integers(-40, 41, size=(n, pool, 2 * nf)).astype(np.int8)
    P = 2 * nf // 1024
    lost = rng.random((n, pool, P)) < 0.05
    kept = ((~lost).astype(np.uint64) << np.arange(P, dtype=np.uint64)).sum(axis=2).astype(
        np.uint32)
    present = rng.random((n, pool)) > 0.03
    mask = np.packbits(present.astype(np.uint8), axis=1, bitorder="little")
    blocks = [(0, 40), (7, 130), (100, 1), (130, 129), (3, 257)]
    first = (C.c_int64 * len(blocks))(*[b[0] for b in blocks])
    frames = (C.c_int32 * len(blocks))(*[b[1] for b in blocks])
    eng = pkg.FxEngine(n, nf, max_frames=48, xmode=xmode)
    handles = (C.c_void_p * 1)(eng.h.value)
    xs = torch.from_numpy(x).cuda()
    ms = torch.from_numpy(mask).cuda()
    ks = torch.from_numpy(kept.view(np.int32)).cuda()
    nb = n * (n + 1) // 2
    rows = torch.zeros((len(blocks), nb, nf), dtype=torch.complex64, device="cuda")
    h = C.c_void_p()
    st = lib.corrx_batch_create_packets(handles, 1, None, C.c_void_p(xs.data_ptr()),
                                        xs.stride(0), xs.stride(1), C.c_void_p(ms.data_ptr()),
                                        ms.stride(0), C.c_void_p(ks.data_ptr()), ks.stride(0),
                                        first, frames, len(blocks), C.c_void_p(rows.data_ptr()),
                                        None, C.byref(h))
    assert st == 0, lib.corr_last_error()
    try:
        assert lib.corrx_batch_launch(h, C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
        torch.cuda.synchronize()
        eng.check()
        got = rows.cpu().numpy()
        zx = oracle.zero_lost_packets(x, kept)
        for i, (f0, nfr) in enumerate(blocks):
            ref = oracle.correlate(zx[:, f0:f0 + nfr], present[:, f0:f0 + nfr]) / nfr
            assert oracle.rel_rms(got[i], ref) < 1e-5, i
            # the same block through corrx_accumulate_packets gives the same bits
            acc = eng.new_acc()
            eng.accumulate(xs, nfr, acc, mask=ms, mask_bit0=f0, frame0=f0, packets=ks,
                           packets_frame0=f0)
            eng.scale(acc, nfr)
            torch.cuda.synchronize()
            assert np.array_equal(got[i], acc.cpu().numpy()), i
        # a misaligned word array is refused
        h2 = C.c_void_p()
        assert lib.corrx_batch_create_packets(
            handles, 1, None, C.c_void_p(xs.data_ptr()), xs.stride(0), xs.stride(1), None, 0,
            C.c_void_p(ks.data_ptr() + 2), ks.stride(0), first, frames, len(blocks),
            C.c_void_p(rows.data_ptr()), None, C.byref(h2)) == pkg.abi.CORR_ERR_ARG
    finally:
        lib.corrx_batch_destroy(h)
        eng.close()
