"""corrx_accumulate_packets: loss at 1024-sample packet granularity.

A clear packet bit zero-fills that packet of the frame before its transform; a
frame with no packet left is skipped like a frame whose validity bit is clear.
Checked against the float64 oracle (zero_lost_packets, then correlate) and, bit
for bit, against the frame-granular path where the two must agree: every
packet kept equals no packet mask, all-or-nothing words equal the frame mask,
and bits past the frame's packet count are ignored.

Tolerance (plain FP32 X-engine, against float64): relative RMS <= 1e-5 and
per-visibility (normalised by sqrt(V_jj V_kk)) <= 1e-5.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def inputs(n, frames, nf, seed, p_lost=0.2):
    rng = np.random.default_rng(seed)
    x = rng.integers(-40, 41, size=(n, frames, 2 * nf)).astype(np.int8)
    P = max(1, 2 * nf // 1024)
    lost = rng.random((n, frames, P)) < p_lost
    kept = ((~lost) * (1 << np.arange(P, dtype=np.uint64))).sum(-1).astype(np.uint32)
    return x, kept


def run(pkg, torch, x, frames, xmode=0, max_frames=16, mask=None, kept=None,
        kept_frame0=0):
    n, _, L = x.shape
    eng = pkg.FxEngine(n, L // 2, max_frames=max_frames, xmode=xmode)
    acc = eng.new_acc()
    xs = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    ms = None if mask is None else torch.from_numpy(np.ascontiguousarray(mask)).cuda()
    ks = None if kept is None else torch.from_numpy(kept.view(np.int32)).cuda()
    eng.accumulate(xs, frames, acc, mask=ms, packets=ks, packets_frame0=kept_frame0)
    torch.cuda.synchronize()
    eng.check()
    out = acc.cpu().numpy()
    eng.close()
    return out


@pytest.mark.parametrize("n,nf,frames", [(6, 4096, 40), (3, 16384, 20), (5, 512, 64),
                                         (24, 2048, 24)])
def test_packets_match_oracle(pkg, cuda, oracle, n, nf, frames):
    x, kept = inputs(n, frames, nf, seed=nf + n)
    ref = oracle.correlate(oracle.zero_lost_packets(x, kept))
    got = run(pkg, cuda, x, frames, kept=kept)
    assert oracle.rel_rms(got, ref) <= TOL
    assert oracle.normalized_max_err(got, ref, n) <= TOL
    # and the loss did something
    assert oracle.rel_rms(oracle.correlate(x), ref) > 1e-3


@pytest.mark.parametrize("xmode", [0, 1, 2])
def test_all_kept_is_no_packet_mask(pkg, cuda, xmode):
    n, nf, frames = 8, 4096, 48
    x, _ = inputs(n, frames, nf, seed=7)
    kept = np.full((n, frames), 0xFFFFFFFF, dtype=np.uint32)   # bits past 8 packets ignored
    a = run(pkg, cuda, x, frames, xmode=xmode)
    b = run(pkg, cuda, x, frames, xmode=xmode, kept=kept)
    assert np.array_equal(a, b)


def test_whole_frame_words_equal_frame_mask(pkg, cuda):
    n, nf, frames = 8, 4096, 48
    x, _ = inputs(n, frames, nf, seed=11)
    rng = np.random.default_rng(12)
    present = rng.random((n, frames)) > 0.25
    mask = np.packbits(present, axis=1, bitorder="little")
    kept = np.where(present, 0xFF, 0).astype(np.uint32)
    a = run(pkg, cuda, x, frames, mask=mask)
    b = run(pkg, cuda, x, frames, kept=kept)
    assert np.array_equal(a, b)


def test_frame_mask_and_packets_combine(pkg, cuda, oracle):
    n, nf, frames = 5, 8192, 36
    x, kept = inputs(n, frames, nf, seed=21, p_lost=0.1)
    rng = np.random.default_rng(22)
    present = rng.random((n, frames)) > 0.2
    mask = np.packbits(present, axis=1, bitorder="little")
    ref = oracle.correlate(oracle.zero_lost_packets(x, kept), present)
    got = run(pkg, cuda, x, frames, mask=mask, kept=kept)
    assert oracle.rel_rms(got, ref) <= TOL


def test_packet_word_offset(pkg, cuda, oracle):
    """Word pmask_frame0 + f belongs to frame f, across max_frames chunks."""
    n, nf, frames, off = 4, 4096, 40, 7
    x, kept = inputs(n, frames, nf, seed=31)
    words = np.zeros((n, frames + off + 3), dtype=np.uint32)
    words[:, off:off + frames] = kept
    ref = oracle.correlate(oracle.zero_lost_packets(x, kept))
    got = run(pkg, cuda, x, frames, kept=words, kept_frame0=off, max_frames=16)
    assert oracle.rel_rms(got, ref) <= TOL


def test_every_packet_lost_is_zero(pkg, cuda):
    n, nf, frames = 4, 2048, 20
    x, _ = inputs(n, frames, nf, seed=41)
    got = run(pkg, cuda, x, frames, kept=np.zeros((n, frames), dtype=np.uint32))
    assert not np.any(got)


def test_bad_arguments(pkg, cuda):
    import ctypes as C
    n, nf, frames = 2, 1024, 4
    eng = pkg.FxEngine(n, nf, max_frames=4)
    acc = eng.new_acc()
    xs = cuda.zeros((n, frames, 2 * nf), dtype=cuda.int8, device="cuda")
    words = cuda.zeros((n, frames + 1), dtype=cuda.int32, device="cuda")
    lib = eng.lib

    def call(pm, f0=0):
        return lib.corrx_accumulate_packets(eng.h, C.c_void_p(xs.data_ptr()), xs.stride(0),
                                            xs.stride(1), None, 0, 0, C.c_void_p(pm), n + 1, f0,
                                            frames, C.c_void_p(acc.data_ptr()), None)
    assert call(words.data_ptr() + 2) == pkg.abi.CORR_ERR_ARG          # misaligned words
    assert call(0) == pkg.abi.CORR_ERR_ARG                             # no words
    assert call(words.data_ptr(), f0=-1) == pkg.abi.CORR_ERR_ARG       # negative word offset
    assert call(words.data_ptr()) == pkg.abi.CORR_OK
    cuda.cuda.synchronize()
    eng.check()
    eng.close()


@pytest.mark.parametrize("xmode,tol", [(0, 1e-5), (2, 1e-5)])
def test_plain_gpu_workload_with_packet_loss(pkg, cuda, oracle, xmode, tol):
    """The 20-input n_freq 8192 workload with its 0.1 % packet loss applied per
    packet (16 packets per frame) rather than per frame."""
    import importlib
    synth = importlib.import_module(pkg.__name__ + ".synth")
    w = synth.WORKLOADS["plain-gpu-20in-nf8192"]
    frames = 48
    x, mask, kept = synth.generate_numpy(w, frames, words=True)
    assert kept is not None and (kept != (1 << 16) - 1).any()
    ref = oracle.correlate(oracle.zero_lost_packets(x, kept))
    got = run(pkg, cuda, x, frames, xmode=xmode, kept=kept)
    assert oracle.rel_rms(got, ref) <= tol
    assert oracle.normalized_max_err(got, ref, w.n_station) <= 2 * tol
