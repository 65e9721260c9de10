"""The F-engine's exact-arithmetic identities, checked in float32 (host only).

The first pass of the CUDA F-engine (csrc/fengine_impl.cuh) unpacks an int8
sample b without the conversion unit: the byte b ^ 0x80 placed in the low byte
of the float 2^23 gives x = 2^23 + 128 + b = b + B. It does not subtract B per
sample: its first butterflies form x0 - x2 and x0 + (x2 - 2B), and a first
pass over a split frame forms x[e] + (x[e+M] - 2B) and x[e] - x[e+M]. These are
claimed to be the integer sums and differences exactly, so the spectra are the
ones the unbiased samples give. numpy's float32 operations round to nearest
like the GPU's FADD, so checking every pair of int8 values here checks the
claim.
"""

from __future__ import annotations

import numpy as np

B = np.float32(2.0 ** 23 + 128)


def biased(b: np.ndarray) -> np.ndarray:
    """The float whose bits are 0x4B000000 | ((b ^ 0x80) & 0xff), as the kernel builds it."""
    bits = np.uint32(0x4B000000) | ((b.astype(np.int32) ^ 0x80) & 0xFF).astype(np.uint32)
    return bits.view(np.float32)


def test_unpacked_value_is_sample_plus_offset():
    b = np.arange(-128, 128, dtype=np.int8)
    x = biased(b)
    assert np.array_equal(x - B, b.astype(np.float32))
    assert np.array_equal(x.astype(np.float64), b.astype(np.float64) + float(B))


def test_first_butterflies_remove_the_offset_exactly():
    b = np.arange(-128, 128, dtype=np.int8)
    x0 = biased(b)[:, None]
    x2 = biased(b)[None, :]
    b0 = b.astype(np.float32)[:, None]
    b2 = b.astype(np.float32)[None, :]
    two_b = np.float32(2) * B
    assert two_b == np.float32(2.0 ** 24 + 256)
    diff = x0 - x2                       # Dft<4>::run_biased, kFromInt8Diff
    total = x0 + (x2 - two_b)            # Dft<4>::run_biased, kFromInt8Sum, DftOdd
    assert diff.dtype == np.float32 and total.dtype == np.float32
    assert np.array_equal(diff, b0 - b2)
    assert np.array_equal(total, b0 + b2)


def test_odd_radix_centre_term():
    b = np.arange(-128, 128, dtype=np.int8)
    half = np.float32(0.5) * (np.float32(2) * B)   # DftOdd: x[0] - B from two_b / 2
    assert np.array_equal(biased(b) - half, b.astype(np.float32))


def test_scaling_by_the_split_factor_is_exact():
    """split_store takes h = scale/2 (a power of two) into the twiddle: h*(w*d)
    and (h*w)*d, and h*s, are the same floats for the magnitudes a frame reaches."""
    rng = np.random.default_rng(3)
    for log2_l in (10, 13, 15, 16):
        h = np.float32(2.0 ** -(log2_l - 8) / 2)            # FP16 forms' scale / 2
        for _ in range(4):
            w = rng.standard_normal(4096).astype(np.float32)
            d = (rng.standard_normal(4096) * 4096).astype(np.float32)
            assert np.array_equal((h * w) * d, h * (w * d))
        assert np.float32(0.5) * np.float32(1.0) == np.float32(0.5)   # FP32 rows: h = 1/2
