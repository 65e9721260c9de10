"""FFT plan 2's index arithmetic (fengine_tc.cu), checked on the CPU.

corrx_tc_fft_maps returns the row orders and operand byte offsets that the
tensor-core F-engine uses. These tests check that:
  * every map is a bijection onto its rows, and the offsets are the canonical
    K-major no-swizzle layout its MMA descriptors describe (8-row x 16-byte core
    matrices, 128 bytes between K neighbours, 1024 or 512 between 8-row groups),
    inside the 64 KB operand buffer;
  * the three DFT stages run through exactly these maps (in float64) give
    numpy's FFT, and after stage 3 the rows of Z[k] and Z[M-k] are rows p and
    512 + p (entry i against entry 15 - i), except the self-paired rows 0 and 512;
  * the stage-2 scatter into the stage-3 operand is free of bank conflicts, and
    the stage-1 scatter puts at most two elements in one bank.
A planted mistake in a map must be caught.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

M = 16384


@pytest.fixture(scope="module")
def maps(pkg):
    b = np.zeros(512, np.int32)
    r2 = np.zeros(32 * 16, np.int32)
    r3 = np.zeros(32 * 32, np.int32)
    o12 = np.zeros(512 * 32, np.uint32)
    o3 = np.zeros(1024 * 16, np.uint32)
    ptr = lambda a: C.c_void_p(a.ctypes.data)   # noqa: E731
    assert pkg.abi.load().corrx_tc_fft_maps(ptr(b), ptr(r2), ptr(r3), ptr(o12), ptr(o3)) == 0
    return {"b": b, "r2": r2.reshape(32, 16), "r3": r3.reshape(32, 32),
            "o12": o12.reshape(512, 32), "o3": o3.reshape(1024, 16)}


def test_maps_are_bijections(maps):
    assert sorted(maps["b"]) == list(range(512))
    assert sorted(maps["r2"].ravel()) == list(range(512))
    assert sorted(maps["r3"].ravel()) == list(range(1024))


@pytest.mark.parametrize("key,rows,elems,sbo", [("o12", 512, 32, 1024), ("o3", 1024, 16, 512)])
def test_operand_offsets_are_the_canonical_layout(maps, key, rows, elems, sbo):
    off = maps[key].astype(np.int64)
    r = np.arange(rows)[:, None]
    e = np.arange(elems)[None, :]
    expect = (r >> 3) * sbo + (e >> 2) * 128 + (r & 7) * 16 + (e & 3) * 4
    assert np.array_equal(off, expect)
    assert off.max() + 4 <= 65536 and len(np.unique(off)) == off.size


def three_stage_fft(z, maps):
    """The kernel's stages in float64, through the library's maps."""
    W32 = np.exp(-2j * np.pi * np.outer(np.arange(32), np.arange(32)) / 32)
    W16 = np.exp(-2j * np.pi * np.outer(np.arange(16), np.arange(16)) / 16)
    b = maps["b"]
    A1 = z[512 * np.arange(32)[None, :] + b[:, None]]                     # [row1, a]
    C1 = A1 @ W32.T                                                         # [row1, k1]
    A2 = np.zeros((512, 32), complex)
    for row1 in range(512):
        c, d = b[row1] >> 4, b[row1] & 15
        tw = np.exp(-2j * np.pi * b[row1] * np.arange(32) / M)
        A2[maps["r2"][:, d], c] = C1[row1] * tw
    C2 = A2 @ W32.T                                                         # [row2, k2a]
    A3 = np.zeros((1024, 16), complex)
    for k1 in range(32):
        for d in range(16):
            tw = np.exp(-2j * np.pi * d * np.arange(32) / 512)
            A3[maps["r3"][k1], d] = C2[maps["r2"][k1, d]] * tw
    C3 = A3 @ W16.T                                                         # [row3, k2b]
    Z = np.empty(M, complex)
    for k1 in range(32):
        for k2a in range(32):
            Z[k1 + 32 * k2a + 1024 * np.arange(16)] = C3[maps["r3"][k1, k2a]]
    return Z, C3


def check_stages(maps):
    """The FFT through the maps, and the row decodes the kernel's epilogues assume."""
    rng = np.random.default_rng(8)
    x = rng.integers(-128, 128, size=2 * M).astype(np.float64)
    z = x[0::2] + 1j * x[1::2]
    Z, C3 = three_stage_fft(z, maps)
    ref = np.fft.fft(z)
    assert np.abs(Z - ref).max() <= 1e-9 * np.abs(ref).max()
    # stage-2 epilogue: TMEM row -> (k1, d) = (8 (G >> 2) + (l >> 2), 4 (G & 3) + (l & 3)),
    # G = row >> 5, l = row & 31
    for k1 in range(32):
        for d in range(16):
            row = int(maps["r2"][k1, d])
            g, l = row >> 5, row & 31
            assert (8 * (g >> 2) + (l >> 2), 4 * (g & 3) + (l & 3)) == (k1, d)
    # stage-3 epilogue: thread p < 512 holds Z[p + 1024 i] in row p and Z[M - p - 1024 i]
    # in row 512 + p at entry 15 - i
    for p in range(1, 512):
        k = p + 1024 * np.arange(16)
        assert np.allclose(C3[p], Z[k])
        assert np.allclose(C3[512 + p][::-1], Z[(M - k) % M])
    # rows 0 = (0, 0) and 512 = (0, 16) pair with themselves
    assert np.allclose(C3[0], Z[1024 * np.arange(16)])
    assert np.allclose(C3[512], Z[512 + 1024 * np.arange(16)])


def test_stages_give_the_fft_and_pair_the_rows(maps):
    check_stages(maps)


@pytest.mark.parametrize("which", ["r3", "r2"])
def test_planted_mistake_is_caught(maps, which):
    bad = {k: v.copy() for k, v in maps.items()}
    bad[which][3, 5], bad[which][4, 5] = maps[which][4, 5], maps[which][3, 5]
    with pytest.raises(AssertionError):
        check_stages(bad)


def wavefronts(words):
    banks = {}
    for w in words:
        banks.setdefault(int(w) % 32, set()).add(int(w))
    return max(len(v) for v in banks.values())


def test_scatters_bank_conflicts(maps):
    """Each epilogue warp writes one 4-byte element per lane into the next operand:
    stage 2's scatter hits 32 banks, stage 1's at most two elements per bank."""
    w1 = w2 = 0
    for warp in range(16):
        rows = 128 * (warp >> 2) + 32 * (warp & 3) + np.arange(32)
        b = maps["b"][rows]
        c, d = b >> 4, b & 15
        for k1 in range(32):
            w1 = max(w1, wavefronts(maps["o12"][maps["r2"][k1, d], c] // 4))
        inv = {int(maps["r2"][k1, dd]): (k1, dd) for k1 in range(32) for dd in range(16)}
        kd = np.array([inv[int(r)] for r in rows])
        for k2a in range(32):
            w2 = max(w2, wavefronts(maps["o3"][maps["r3"][kd[:, 0], k2a], kd[:, 1]] // 4))
    assert w2 == 1 and w1 <= 2
