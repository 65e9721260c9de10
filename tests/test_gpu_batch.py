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


@pytest.mark.parametrize("xmode", [0, 2])
def test_batch_graph_rows_match_oracle(pkg, cuda, oracle, xmode):
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
