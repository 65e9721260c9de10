"""bench.py's accuracy report (float64 DFT at a channel subset, and the float64
FFT reference over the whole row), on the CPU.

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
    # every visibility of the row against the float64 FFT reference
    assert rep["vs_fp64_full_row"]["plain"]["rel_rms"] < 1e-6
    assert rep["vs_fp64_full_row"]["plain"]["max_per_vis"] < 1e-6
    assert abs(rep["vs_fp64_full_row"]["tc"]["rel_rms"] - 1e-3) < 1e-5


def test_accuracy_report_zeroes_lost_packets(oracle):
    """With packet words the float64 reference zero-fills exactly the lost packets."""
    torch = pytest.importorskip("torch")
    bench = importlib.import_module("bench")
    rng = np.random.default_rng(6)
    N, nf, F = 3, 2048, 12                     # 4 packets of 1024 samples per frame
    x = rng.integers(-20, 21, size=(N, F, 2 * nf)).astype(np.int8)
    kept = rng.integers(0, 16, size=(N, F)).astype(np.uint32) | np.uint32(0xFFFFFFF0)
    w = SimpleNamespace(n_station=N, frames=F, fft_len=2 * nf, n_freq=nf)
    ref = oracle.correlate(oracle.zero_lost_packets(x, kept)) / F
    rows = {"plain": torch.from_numpy(ref.astype(np.complex64))}
    words = torch.from_numpy(kept.view(np.int32))
    rep = bench.accuracy_report(torch, w, torch.from_numpy(x), None, rows,
                                channels=[0, 5, 1000, 2047], words=words)
    assert rep["vs_fp64"]["plain"]["rel_rms"] < 1e-6
    whole = bench.accuracy_report(torch, w, torch.from_numpy(x), None, rows,
                                  channels=[0, 5, 1000, 2047])
    assert whole["vs_fp64"]["plain"]["rel_rms"] > 1e-3      # the packets mattered
