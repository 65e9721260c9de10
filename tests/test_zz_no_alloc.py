"""corrx_accumulate_noalloc: the allocation-free accumulate, checked against corrx_accumulate.

Some callers of this library may not allocate device memory: their host owns
every device byte through its own pool, or they run a real-time loop in which an
allocation (and the device synchronisation it can bring) would break a
deadline, or their device-memory budget is fixed up front. For them the library
keeps the spectra scratch in a fixed 64 MiB device array instead of a buffer
that corrx_create allocates, and the twiddle tables of every transform length in
a second fixed array filled once per device. This file checks, through the C
ABI, that two calls in a row give the same visibilities as the allocating entry
point (same kernels; tolerance 1e-5 relative RMS, the plain-path bar), that the
second call is not disturbed by what the first left in the shared array, that
calls of different transform lengths follow each other correctly, that the FP16
form holds twice the frames (4-byte bins), and that a request larger than the
array is refused with CORR_ERR_ARG. It is collected last on purpose.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_RMS_TOL = 1e-5


def noalloc(pkg, torch, xmode, x, frames, acc, mask=None, mask_bit0=0):
    lib = pkg.abi.load()
    n, _, L = x.shape
    st = lib.corrx_accumulate_noalloc(
        n, L // 2, xmode, C.c_void_p(x.data_ptr()), x.stride(0), x.stride(1),
        C.c_void_p(0 if mask is None else mask.data_ptr()),
        0 if mask is None else mask.stride(0), mask_bit0, frames, C.c_void_p(acc.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st


@pytest.mark.parametrize("xmode", [0, 1, 2])
def test_two_calls_match_allocating_entry_point(pkg, cuda, oracle, xmode):
    torch = cuda
    n, nf, frames = 24, 16384, 20          # 20 <= 21 frames the 64 MiB array holds here
    rng = np.random.default_rng(100 + xmode)
    inputs = [rng.integers(-60, 61, size=(n, frames, 2 * nf)).astype(np.int8) for _ in range(2)]
    present = np.ones((n, frames), dtype=bool)
    present[5, 3] = present[17, 19] = False
    mask = torch.from_numpy(np.packbits(present.astype(np.uint8), axis=1,
                                        bitorder="little")).cuda()
    eng = pkg.FxEngine(n, nf, max_frames=64, xmode=xmode)
    for x_np in inputs:                     # two calls in a row on the shared array
        x = torch.from_numpy(x_np).cuda()
        want = eng.new_acc()
        eng.accumulate(x, frames, want, mask=mask)
        got = torch.zeros_like(want)
        assert noalloc(pkg, torch, xmode, x, frames, got, mask) == 0, \
            pkg.abi.load().corr_last_error()
        torch.cuda.synchronize()
        eng.check()
        g, w = got.cpu().numpy(), want.cpu().numpy()
        # same kernels, same tiles, one pass each: the same bits
        assert np.array_equal(g, w)
        # FP16 spectra: one rounding to 11 bits, errors falling as 1/sqrt(frames)
        tol = REL_RMS_TOL if xmode != 1 else 1.5e-3 / np.sqrt(frames)
        assert oracle.rel_rms(g, oracle.correlate(x_np, present)) < tol
    eng.close()


def test_request_beyond_the_array_is_refused(pkg, cuda):
    torch = cuda
    n, nf = 24, 16384
    x = torch.zeros((n, 22, 2 * nf), dtype=torch.int8, device="cuda")
    acc = torch.zeros((n * (n + 1) // 2, nf), dtype=torch.complex64, device="cuda")
    st = noalloc(pkg, torch, 0, x, 22, acc)
    assert st == pkg.abi.CORR_ERR_ARG
    msg = pkg.abi.load().corr_last_error().decode()
    assert "21 frames" in msg and "split the call" in msg
    torch.cuda.synchronize()
    assert not torch.any(acc)               # nothing was launched


def test_fp16_form_holds_twice_the_frames(pkg, cuda):
    """FP16 spectra take 4 bytes a bin: 42 frames fit at 24 inputs, 43 do not."""
    torch = cuda
    n, nf = 24, 16384
    rng = np.random.default_rng(7)
    x = torch.from_numpy(rng.integers(-60, 61, size=(n, 43, 2 * nf)).astype(np.int8)).cuda()
    acc = torch.zeros((n * (n + 1) // 2, nf), dtype=torch.complex64, device="cuda")
    assert noalloc(pkg, torch, 1, x, 43, acc) == pkg.abi.CORR_ERR_ARG
    assert "42 frames" in pkg.abi.load().corr_last_error().decode()
    assert noalloc(pkg, torch, 1, x, 42, acc) == 0
    eng = pkg.FxEngine(n, nf, max_frames=64, xmode=1)
    want = eng.new_acc()
    eng.accumulate(x, 42, want)
    torch.cuda.synchronize()
    eng.check()
    assert np.array_equal(acc.cpu().numpy(), want.cpu().numpy())
    eng.close()


def test_calls_of_different_lengths_in_a_row(pkg, cuda):
    """Each transform length reads its own twiddle tables: 4096, 16384, 512,
    6144, 14336, 32768 and 22528 channels back to back on one stream, each equal
    to the allocating path."""
    torch = cuda
    rng = np.random.default_rng(11)
    for nf in (4096, 16384, 512, 6144, 14336, 32768, 22528, 4096):
        n, frames = 6, 16
        x = torch.from_numpy(rng.integers(-60, 61, size=(n, frames, 2 * nf)).astype(np.int8)).cuda()
        got = torch.zeros((n * (n + 1) // 2, nf), dtype=torch.complex64, device="cuda")
        assert noalloc(pkg, torch, 0, x, frames, got) == 0
        eng = pkg.FxEngine(n, nf, max_frames=frames)
        want = eng.new_acc()
        eng.accumulate(x, frames, want)
        torch.cuda.synchronize()
        eng.check()
        assert np.array_equal(got.cpu().numpy(), want.cpu().numpy()), f"n_freq {nf}"
        eng.close()
