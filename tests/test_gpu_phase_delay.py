"""End-to-end physics check: the fitted delay of every baseline equals the injected delay.

The synthetic inputs share a common Gaussian signal delayed by an integer number
of samples d_i per input (synth.delays_for), generated on the device. A frame
delayed by d samples has X[c] ~ S[c] exp(-2 pi i c d / L), so the cross-spectrum
V_jk[c] = X_j conj(X_k) carries the phase slope of d_j - d_k, and its delay
transform z(tau) = sum_c V_jk[c] exp(2 pi i c tau / L) peaks at tau = d_j - d_k.
The same holds for every X-engine form.
"""

from __future__ import annotations

import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("xmode", [0, 1, 2])
@pytest.mark.parametrize("workload", ["plain-gpu-20in-nf8192", "precision-24in-nf16384"])
def test_fitted_delays_equal_injected(pkg, cuda, xmode, workload):
    torch = cuda
    synth = importlib.import_module(pkg.__name__ + ".synth")
    w = synth.WORKLOADS[workload]
    frames = 64
    x, mask = synth.generate_torch(w, frames)
    eng = pkg.FxEngine(w.n_station, w.n_freq, max_frames=frames, xmode=xmode)
    try:
        acc = eng.new_acc()
        eng.accumulate(x, frames, acc, mask=mask)
        eng.scale(acc, frames)
        torch.cuda.synchronize()
        eng.check()
        v = acc.cpu().numpy().astype(np.complex128)
    finally:
        eng.close()
    L = w.fft_len
    for tone in w.tones:                    # narrowband tones carry no delay
        v[:, tone[0]] = 0
    d = synth.delays_for(w)
    z = np.fft.ifft(v, n=L, axis=1)         # the delay transform, up to a factor L
    lag = np.argmax(np.abs(z), axis=1)
    lag = np.where(lag > L // 2, lag - L, lag)
    wrong = []
    for b, (j, k) in enumerate(pkg.Correlator.baseline_pairs(w.n_station)):
        if j != k and lag[b] != d[j] - d[k]:
            wrong.append((j, k, int(lag[b]), int(d[j] - d[k])))
    assert not wrong, f"{len(wrong)} baselines with the wrong delay, e.g. {wrong[:5]}"
