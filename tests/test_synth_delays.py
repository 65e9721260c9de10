"""The synthetic inputs carry the delays they claim (CPU, float64 oracle).

Pins the sign convention the GPU delay test relies on: the delay transform of
V_jk = X_j conj(X_k) from the oracle peaks at d_j - d_k for every baseline of
the CPU-sized workload.
"""

from __future__ import annotations

import importlib

import numpy as np


def test_oracle_recovers_injected_delays(pkg, oracle):
    synth = importlib.import_module(pkg.__name__ + ".synth")
    w = synth.WORKLOADS["plain-cpu-8in-nf1024"]
    frames = 64
    x, mask = synth.generate_numpy(w, frames)
    present = synth.unpack_mask(mask, frames) if mask is not None else np.ones(
        (w.n_station, frames), dtype=bool)
    v = oracle.correlate(x, present)
    L = w.fft_len
    z = np.fft.ifft(v, n=L, axis=1)
    lag = np.argmax(np.abs(z), axis=1)
    lag = np.where(lag > L // 2, lag - L, lag)
    d = synth.delays_for(w)
    assert len(set(d.tolist())) > 2, "the workload should inject distinct delays"
    for b, (j, k) in enumerate(oracle.baseline_pairs(w.n_station)):
        if j != k:
            assert lag[b] == d[j] - d[k], (j, k)
