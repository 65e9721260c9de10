"""Full-size integration (24 inputs, n_freq 16384, 4096 frames): size-independent checks.

The whole-row oracle would take minutes on the CPU at this size, so the full
integration is checked through properties that hold exactly:
  * Parseval on every autocorrelation: with X the L-point spectrum of a real
    frame, 2*sum_{k<M} |X_k|^2 - |X_0|^2 = L*sum_t x_t^2 - |X_M|^2, where X_M
    (Nyquist) = sum_t (-1)^t x_t. The right side is integer arithmetic on the
    samples; the left side is what the engine accumulated.
  * A channel subset against an exact float64 DFT of every frame (CPU, numpy):
    all 300 baselines at 16 channels, including the DC bin and the band edge.
  * Accumulating the integration in two calls equals one call.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CHANNELS = np.array([0, 1, 2, 63, 1234, 2047, 3000, 4096, 5555, 8191, 8192, 9000, 12345,
                     16000, 16382, 16383])


@pytest.fixture(scope="module")
def fullsize(pkg, cuda):
    import importlib
    torch = cuda
    synth = importlib.import_module(pkg.__name__ + ".synth")
    w = synth.WORKLOADS["precision-24in-nf16384"]
    x, _ = synth.generate_torch(w, w.frames, seed_offset=77)
    torch.cuda.synchronize()
    return w, x


def run(pkg, torch, w, x, xmode, splits=(0,)):
    eng = pkg.FxEngine(w.n_station, w.n_freq, max_frames=256, xmode=xmode)
    acc = eng.new_acc()
    bounds = list(splits) + [w.frames]
    for a, b in zip(bounds[:-1], bounds[1:]):
        eng.accumulate(x, b - a, acc, frame0=a, mask_bit0=a)
    torch.cuda.synchronize()
    eng.check()
    out = acc.cpu().numpy().astype(np.complex128)
    eng.close()
    return out


@pytest.fixture(scope="module")
def exact_subset(fullsize, oracle):
    """Exact float64 DFT of every frame at CHANNELS -> V for all baselines."""
    w, x = fullsize
    xs = x.cpu().numpy()
    L = w.fft_len
    t = np.arange(L)
    W = np.exp(-2j * np.pi * np.outer(t, CHANNELS) / L)
    Wr, Wi = W.real.copy(), W.imag.copy()
    N, F = w.n_station, w.frames
    Y = np.empty((N, F, CHANNELS.size), dtype=np.complex128)
    step = 256
    for s in range(N):
        for f0 in range(0, F, step):
            blk = xs[s, f0:f0 + step].astype(np.float64)
            Y[s, f0:f0 + step] = blk @ Wr + 1j * (blk @ Wi)
    pairs = oracle.baseline_pairs(N)
    V = np.array([(Y[j] * np.conj(Y[k])).sum(axis=0) for j, k in pairs])
    # Parseval right side per station, in exact integer arithmetic
    parseval = np.zeros(N)
    for s in range(N):
        sumsq = 0
        nyq2 = 0
        for f0 in range(0, F, step):
            blk = xs[s, f0:f0 + step].astype(np.int64)
            sumsq += int((blk ** 2).sum())
            nyq = blk[:, 0::2].sum(axis=1) - blk[:, 1::2].sum(axis=1)
            nyq2 += int((nyq ** 2).sum())
        parseval[s] = float(L * sumsq - nyq2)
    return V, parseval


@pytest.mark.parametrize("xmode,tol", [(0, 1e-5), (2, 1e-5), (1, 1e-4)])
def test_full_integration(pkg, cuda, oracle, fullsize, exact_subset, xmode, tol):
    w, x = fullsize
    V, parseval = exact_subset
    got = run(pkg, cuda, w, x, xmode)
    N = w.n_station
    # Parseval on the autos
    for s in range(N):
        b = oracle.baseline_index(N, s, s)
        lhs = 2.0 * got[b].real.sum() - got[b, 0].real
        assert abs(lhs - parseval[s]) <= tol * parseval[s], (s, lhs, parseval[s])
    # channel subset against the exact DFT
    sub = got[:, CHANNELS]
    rms = oracle.rel_rms(sub, V)
    pv = oracle.normalized_max_err(sub, V, N)
    print(f"full size xmode={xmode}: subset rel RMS {rms:.3e}, per-vis {pv:.3e}")
    assert rms <= tol and pv <= 10 * tol


def test_split_calls_equal_one_call(pkg, cuda, oracle, fullsize):
    w, x = fullsize
    one = run(pkg, cuda, w, x, 0)
    two = run(pkg, cuda, w, x, 0, splits=(0, 1000, 2048, 3333))
    assert oracle.rel_rms(two, one) < 1e-6
