"""CPU oracle for the FX correlator path -- TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product: only tests/, the smoke() of
__graft_entry__ and bench.py's CPU-baseline / reference arm may import it. The
library under test (libcorr_cuda.so) never calls it and has no CPU fallback.

It restates, in float64 numpy, the reference's own CPU statement of the path,
corr-cuda/tests/gen_golden.py:
  * baseline numbering (j outer, k inner, j <= k)          gen_golden.py:31-34
  * float64 real FFT of each 2*n_freq frame, Nyquist dropped gen_golden.py:68-69
  * V[j,k] = sum_f y_j * conj(y_k), divided by n_cum         gen_golden.py:72-78
extended with the parts the golden generator leaves to the C driver:
  * a missing frame (validity bit clear, LSB first, bit = frame in slot)
    contributes as all-zero samples                        corr-cuda/tests/golden.c:104-176,
                                                           corr-cuda/src/kernels.cu:159-174
  * rows divide by the caller's frame count, not the valid count
                                                           corr-cuda/include/corr_cuda.h:414-428
and with one extension the reference does not have: a packet-granular loss mask
(one bit per 1024-sample packet, zero_lost_packets). The reference zero-fills a
frame whole when any of its packets is lost (corr-rs/src/assemble.rs:39-45); a
frame whose packets are all kept or all lost gives the same result either way.
Parity is pinned: tests/golden/ holds fixtures produced by running the
reference's gen_golden.py itself (tests/golden/make_golden.py), and
tests/test_oracle_golden.py checks this module against them.
"""

from __future__ import annotations

import numpy as np


def baseline_pairs(n_station: int) -> list[tuple[int, int]]:
    """(j, k) for every baseline, j <= k, row-major (gen_golden.py:31-34)."""
    return [(j, k) for j in range(n_station) for k in range(j, n_station)]


def baseline_index(n_station: int, j: int, k: int) -> int:
    """Row-major index of (j, k), j <= k (reference corr_cuda.cpp:306-309)."""
    return j * n_station - j * (j - 1) // 2 + (k - j)


def spectra(frames_int8: np.ndarray) -> np.ndarray:
    """float64 rfft over the last axis, bins 0..n_freq-1 (Nyquist dropped)."""
    L = frames_int8.shape[-1]
    return np.fft.rfft(frames_int8.astype(np.float64), axis=-1)[..., : L // 2]


def correlate(samples: np.ndarray, present: np.ndarray | None = None,
              frames_chunk: int = 16) -> np.ndarray:
    """Unscaled visibilities sum_f Y_j conj(Y_k): complex128 [n_baseline, n_freq].

    samples: int8 [n_station, frames, 2*n_freq]; present: bool [n_station, frames]
    or None (all present). Missing frames are zeroed before the transform.
    """
    n, F, L = samples.shape
    nf = L // 2
    iu, ju = np.triu_indices(n)
    acc = np.zeros((n, n, nf), dtype=np.complex128)
    for f0 in range(0, F, frames_chunk):
        x = samples[:, f0:f0 + frames_chunk].astype(np.float64)
        if present is not None:
            x = x * present[:, f0:f0 + frames_chunk, None]
        y = np.fft.rfft(x, axis=-1)[..., :nf]             # [n, f, nf]
        acc += np.einsum("jfc,kfc->jkc", y, np.conj(y))
    return acc[iu, ju]                                    # row-major j <= k


PACKET_SAMPLES = 1024


def zero_lost_packets(samples: np.ndarray, kept: np.ndarray) -> np.ndarray:
    """Copy of samples with every lost 1024-sample packet set to zero.

    samples: int8 [n_station, frames, 2*n_freq]; kept: integer [n_station, frames],
    bit p set = packet p (samples p*1024 .. p*1024+1023 of the frame) arrived.
    """
    n, F, L = samples.shape
    P = L // PACKET_SAMPLES
    bits = (kept.astype(np.uint64)[..., None] >> np.arange(P, dtype=np.uint64)) & 1
    x = samples.reshape(n, F, P, PACKET_SAMPLES) * bits.astype(np.int8)[..., None]
    return x.reshape(n, F, L)


def correlate_rows(samples: np.ndarray, n_cum: int, present: np.ndarray | None = None
                   ) -> np.ndarray:
    """Scaled rows exactly as gen_golden.py writes expect.bin, in complex128.

    samples: int8 [rows, n_station, n_cum, 2*n_freq]; returns [rows, n_baseline, n_freq].
    """
    rows = samples.shape[0]
    out = []
    for r in range(rows):
        pr = None if present is None else present[r]
        out.append(correlate(samples[r], pr) / n_cum)
    return np.stack(out)


def golden_input(n_station: int, n_freq: int, n_cum: int, rows: int,
                 seed: int = 20260914) -> np.ndarray:
    """The reference's golden input: gen_golden.py:59-62 (same generator calls)."""
    rng = np.random.default_rng(seed)
    samples = rng.integers(-4, 5, size=(rows, n_station, n_cum, 2 * n_freq)).astype(np.int8)
    samples[0, 0, 0, 0] = -128
    samples[0, 0, 0, 1] = 127
    return samples


def golden_missing(rows: int, n_cum: int) -> np.ndarray:
    """Frames declared missing in the reference's mask-equivalence case:
    (row*3 + frame_in_row) % 7 == 3 (golden.c:101-106). bool [rows, n_cum]."""
    r = np.arange(rows)[:, None]
    f = np.arange(n_cum)[None, :]
    return ((r * 3 + f) % 7) == 3


# -- error metrics -----------------------------------------------------------

def rel_rms(got: np.ndarray, expect: np.ndarray) -> float:
    """Relative RMS over all real and imaginary parts (golden.c:219-228)."""
    g = np.asarray(got).astype(np.complex128)
    e = np.asarray(expect).astype(np.complex128)
    num = np.sum(np.abs(g - e) ** 2)
    den = np.sum(np.abs(e) ** 2)
    return float(np.sqrt(num / den)) if den > 0 else (0.0 if num == 0 else float("inf"))


def normalized_max_err(got: np.ndarray, expect: np.ndarray, n_station: int) -> float:
    """max over (b, c) of |V - V_ref| / sqrt(V_ref[jj] V_ref[kk]).

    The per-visibility error scaled by the autocorrelations of its two inputs,
    which stays meaningful for cross baselines whose expected value is near zero.
    got/expect: [..., n_baseline, n_freq].
    """
    g = np.asarray(got).astype(np.complex128)
    e = np.asarray(expect).astype(np.complex128)
    pairs = baseline_pairs(n_station)
    auto = np.stack([e[..., baseline_index(n_station, i, i), :].real for i in range(n_station)],
                    axis=-2)
    j = np.array([p[0] for p in pairs])
    k = np.array([p[1] for p in pairs])
    norm = np.sqrt(np.maximum(auto[..., j, :] * auto[..., k, :], 1e-300))
    return float(np.max(np.abs(g - e) / norm))


def significant_rel_err(got: np.ndarray, expect: np.ndarray, n_station: int,
                        floor: float = 1e-3) -> tuple[float, float]:
    """(max, rms) elementwise relative error over visibilities with
    |V_ref| > floor*sqrt(V_jj V_kk)."""
    g = np.asarray(got).astype(np.complex128)
    e = np.asarray(expect).astype(np.complex128)
    pairs = baseline_pairs(n_station)
    auto = np.stack([e[..., baseline_index(n_station, i, i), :].real for i in range(n_station)],
                    axis=-2)
    j = np.array([p[0] for p in pairs])
    k = np.array([p[1] for p in pairs])
    norm = np.sqrt(np.maximum(auto[..., j, :] * auto[..., k, :], 1e-300))
    sel = np.abs(e) > floor * norm
    rel = np.abs(g - e)[sel] / np.abs(e)[sel]
    if rel.size == 0:
        return 0.0, 0.0
    return float(rel.max()), float(np.sqrt(np.mean(rel ** 2)))
