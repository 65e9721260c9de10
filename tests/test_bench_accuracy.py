"""bench.py's accuracy report (float64 DFT at a channel subset), on the CPU.

Rows from the float64 oracle must come out exact to single precision; rows
with a planted error must show it; lost frames must be zeroed as the engines do.
"""

from __future__ import annotations

import importlib
from types import SimpleNamespace

import numpy as np
import pytest


def test_accuracy_report_against_the_oracle(oracle):
    torch = pytest.importorskip("torch")
    bench = importlib.import_module("bench")
    rng = np.random.default_rng(4)
    N, nf, F = 3, 256, 20
    x = rng.integers(-20, 21, size=(N, F, 2 * nf)).astype(np.int8)
    present = rng.random((N, F)) > 0.2
    mask = np.packbits(present.astype(np.uint8), axis=1, bitorder="little")
    w = SimpleNamespace(n_station=N, frames=F, fft_len=2 * nf, n_freq=nf)
    ref = oracle.correlate(x, present) / F
    rows = {"plain": torch.from_numpy(ref.astype(np.complex64)),
            "tc": torch.from_numpy((ref * (1 + 1e-3)).astype(np.complex64))}
    rep = bench.accuracy_report(torch, w, torch.from_numpy(x), torch.from_numpy(mask), rows,
                                channels=[0, 1, 17, 200, 255, 300])
    assert rep["channels"] == [0, 1, 17, 200, 255]
    assert rep["vs_fp64"]["plain"]["rel_rms"] < 1e-6
    assert rep["vs_fp64"]["plain"]["max_per_vis"] < 1e-6
    assert abs(rep["vs_fp64"]["tc"]["rel_rms"] - 1e-3) < 1e-5
    assert abs(rep["vs_plain"]["tc"]["rel_rms"] - 1e-3) < 1e-5
