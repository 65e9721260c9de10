"""Pin the CPU oracle to the reference's golden vectors (CPU only).

The fixtures in tests/golden/ were produced by running the reference's own
corr-cuda/tests/gen_golden.py (see make_golden.py). Here the oracle regenerates
the same input, recomputes the rows, and must reproduce the reference's
expect.bin; then a deliberately wrong oracle must NOT reproduce it, which shows
the comparison can see the mistakes the golden test exists for.
"""

from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def load_fixture(name):
    z = np.load(GOLDEN / f"{name}.npz", allow_pickle=False)
    return {k: z[k] for k in z.files}


def regenerate(oracle, fx):
    n, nf, n_cum, rows = (int(fx[k]) for k in ("n_station", "n_freq", "n_cum", "rows"))
    x = oracle.golden_input(n, nf, n_cum, rows, int(fx["seed"]))
    assert hashlib.sha256(x.tobytes()).hexdigest() == str(fx["in_sha256"]), (
        "regenerated golden input differs from the reference's in.bin")
    return x


def test_pair_table_matches_reference(oracle):
    for name in ("golden_partial_slot", "golden_15st"):
        fx = load_fixture(name)
        pairs = np.array(oracle.baseline_pairs(int(fx["n_station"])), dtype=np.int32)
        assert np.array_equal(pairs, fx["pairs"])


def test_oracle_reproduces_golden_partial_slot(oracle):
    fx = load_fixture("golden_partial_slot")
    x = regenerate(oracle, fx)
    got = oracle.correlate_rows(x, int(fx["n_cum"])).astype(np.complex64)
    expect = fx["expect"]
    assert got.shape == expect.shape
    # float64 both sides, rounded once to complex64: agreement to the last few ulps.
    assert oracle.rel_rms(got, expect) < 1e-7
    assert np.allclose(got, expect, rtol=1e-6, atol=1e-6 * np.abs(expect).max())


def test_oracle_reproduces_golden_15st(oracle):
    fx = load_fixture("golden_15st")
    x = regenerate(oracle, fx)
    got = oracle.correlate_rows(x, int(fx["n_cum"]))
    sub = got[:, :, fx["channels"]].astype(np.complex64)
    assert oracle.rel_rms(sub, fx["expect_subset"]) < 1e-7
    np.testing.assert_allclose(got.sum(axis=2), fx["row_baseline_sum"], rtol=1e-6,
                               atol=1e-6 * np.abs(fx["row_baseline_sum"]).max())
    np.testing.assert_allclose((np.abs(got) ** 2).sum(axis=2), fx["row_baseline_sumsq"],
                               rtol=1e-5)


def test_oracle_autocorrelations_are_real(oracle):
    fx = load_fixture("golden_partial_slot")
    x = regenerate(oracle, fx)
    got = oracle.correlate_rows(x, int(fx["n_cum"]))
    n = int(fx["n_station"])
    for i in range(n):
        b = oracle.baseline_index(n, i, i)
        assert np.abs(got[:, b].imag).max() < 1e-9 * np.abs(got[:, b].real).max()


def test_oracle_matches_explicit_dft(oracle):
    """An independent statement of the same sum, by explicit DFT matrix."""
    rng = np.random.default_rng(5)
    n, F, nf = 3, 5, 64
    L = 2 * nf
    x = rng.integers(-128, 128, size=(n, F, L)).astype(np.int8)
    t = np.arange(L)
    W = np.exp(-2j * np.pi * np.outer(t, np.arange(nf)) / L)
    y = x.astype(np.float64) @ W
    ref = np.array([(y[j] * np.conj(y[k])).sum(axis=0) for j, k in oracle.baseline_pairs(n)])
    np.testing.assert_allclose(oracle.correlate(x), ref, rtol=1e-10, atol=1e-8)


def test_missing_frames_equal_zeroed_frames(oracle):
    rng = np.random.default_rng(11)
    n, F, nf = 4, 24, 128
    x = rng.integers(-50, 50, size=(n, F, 2 * nf)).astype(np.int8)
    present = rng.random((n, F)) > 0.2
    zeroed = x * present[:, :, None]
    assert np.array_equal(oracle.correlate(x, present), oracle.correlate(zeroed.astype(np.int8)))


def test_golden_missing_pattern(oracle):
    m = oracle.golden_missing(2, 300)
    # golden.c: every 7th frame with phase 3, shifted by 3 per row.
    assert m[0, 3] and m[0, 10] and not m[0, 4]
    assert m[1, 0] and m[1, 7]
    assert abs(m.mean() - 1 / 7) < 0.01


@pytest.mark.parametrize("mistake", ["keep_nyquist", "swap_conj", "no_scale", "unsigned"])
def test_planted_mistakes_are_caught(oracle, mistake):
    """Plant a mistake in (a copy of) the oracle and check the fixture rejects it."""
    fx = load_fixture("golden_partial_slot")
    x = regenerate(oracle, fx)
    n_cum = int(fx["n_cum"])
    n = int(fx["n_station"])
    pairs = oracle.baseline_pairs(n)
    rows = []
    for r in range(x.shape[0]):
        xf = (x[r].view(np.uint8) if mistake == "unsigned" else x[r]).astype(np.float64)
        L = xf.shape[-1]
        y = np.fft.rfft(xf, axis=-1)
        y = y[..., 1:L // 2 + 1] if mistake == "keep_nyquist" else y[..., :L // 2]
        v = []
        for j, k in pairs:
            a, b = (y[k], y[j]) if mistake == "swap_conj" else (y[j], y[k])
            v.append((a * np.conj(b)).sum(axis=0))
        v = np.array(v)
        rows.append(v if mistake == "no_scale" else v / n_cum)
    wrong = np.stack(rows).astype(np.complex64)
    assert oracle.rel_rms(wrong, fx["expect"]) > 1e-3


def test_packet_zero_fill(oracle):
    """zero_lost_packets clears exactly the 1024-sample packets whose bit is clear;
    all-or-nothing words reproduce the frame-granular mask."""
    rng = np.random.default_rng(5)
    x = rng.integers(-9, 10, size=(3, 5, 4096)).astype(np.int8)
    kept = rng.integers(0, 16, size=(3, 5)).astype(np.uint32) | np.uint32(0xFFFFFFF0)
    z = oracle.zero_lost_packets(x, kept)
    for s in range(3):
        for f in range(5):
            for p in range(4):
                seg, src = z[s, f, p * 1024:(p + 1) * 1024], x[s, f, p * 1024:(p + 1) * 1024]
                assert np.array_equal(seg, src if (kept[s, f] >> p) & 1 else 0 * src)
    present = rng.random((3, 5)) > 0.3
    whole = np.where(present, 0xF, 0).astype(np.uint32)
    a = oracle.correlate(oracle.zero_lost_packets(x, whole))
    b = oracle.correlate(x, present)
    assert np.allclose(a, b, rtol=0, atol=1e-6 * np.abs(b).max())
