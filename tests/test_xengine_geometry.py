"""The tensor X-engine's index arithmetic, checked on the CPU.

corrx_tc_geometry returns the geometry the kernel uses for a tile shape (it is
the library's own make_geom, no device work). For every feasible shape at 1..44
inputs, these tests restate the kernel's converter item mapping and operand
addressing (xengine_tc.cu) and check that:
  * every (channel, station, 8-frame group) is converted exactly once, by
    at most kMaxItems items per converter thread;
  * every operand store and every MMA operand read stays inside its stage, and a
    region's rows stay clear of the next region;
  * shared memory, TMEM columns and the load ring fit the hardware;
  * a quarter warp's 16-byte operand stores in the paired FP16 form hit eight
    distinct bank slots.
Planted mistakes (overlapping regions or channel halves, a dropped item) must fail.
"""

from __future__ import annotations

import ctypes as C

import pytest

KCONV, KMAX, LBO = 224, 4, 128           # converter threads, items per thread, K core stride
PAIRED, SPLIT_STACKED, SPLIT_WIDE, FP16_WIDE = 2, 0, 1, 3


def skew(r: int) -> int:
    return ((r & 1) | ((r & 2) << 1) | ((r & 4) >> 1)) * 16


def geometry(pkg, n, split, ct, kt):
    g = pkg.abi.corrx_tc_geom(struct_size=C.sizeof(pkg.abi.corrx_tc_geom))
    pkg.abi.check(pkg.abi.load().corrx_tc_geometry(n, int(split), ct, kt, C.byref(g)),
                  "corrx_tc_geometry")
    return {f: getattr(g, f) for f, _ in g._fields_}


def items_of(g, n, ct, kt):
    """(thread, slot) -> (c, s, kq) exactly as the kernel's converters decode q."""
    out = {}
    for wt in range(KCONV):
        for i in range(KMAX):
            q = wt + i * KCONV
            if g["form"] == PAIRED:
                regions = ct // 2
                rest = q // regions
                s_lo = rest % 4
                rest //= 4
                half = rest % 2
                rest //= 2
                groups = (n + 3) // 4
                s = (rest % groups) * 4 + s_lo
                kq = rest // groups
                c = (q % regions) * 2 + half
            else:
                c = q % ct
                rest = q // ct
                s = rest % n
                kq = rest // n
            if q < g["items"] and s < n:
                out[(wt, i)] = (c, s, kq)
    return out


def operand_offsets(g, c, s, kq):
    """Byte offsets in an operand stage of the item's 16-byte stores."""
    region, row = c, 2 * s
    if g["form"] == PAIRED:
        region, row = c >> 1, row + (c & 1) * g["R"]
    rows = [row, row + 1]
    if g["form"] in (SPLIT_STACKED, SPLIT_WIDE):
        rows += [row + g["R"], row + 1 + g["R"]]
    base = region * g["region_stride"] + skew(region)
    return [base + (r >> 3) * g["sbo"] + kq * LBO + (r & 7) * 16 for r in rows]


def shapes():
    for n in range(1, 45):
        for split in (False, True):
            for ct in (2, 4, 8):
                for kt in (16, 32, 64):
                    yield n, split, ct, kt


def check_shape(g, n, split, ct, kt):
    assert g["elem"] == (8 if split else 4)
    assert ct * g["elem"] >= 16                                   # 16-byte TMA rows
    assert g["ld_stage"] == kt * n * ct * g["elem"]
    assert g["smem"] <= 227 * 1024
    assert g["n_op"] in (2, 3) and g["n_ld"] >= 2
    assert g["n_ld"] * g["ld_stage"] + g["n_op"] * g["op_stage"] <= g["smem"]
    assert g["n_acc"] * g["acc_cols"] <= g["tmem_cols"] <= 512
    assert g["tmem_cols"] >= 32 and g["tmem_cols"] & (g["tmem_cols"] - 1) == 0
    assert g["items"] <= KMAX * KCONV
    # every item once
    items = items_of(g, n, ct, kt)
    seen = set(items.values())
    assert len(seen) == len(items), "an item decoded twice"
    assert seen == {(c, s, kq) for c in range(ct) for s in range(n) for kq in range(kt // 8)}
    # stores inside the stage, 16-byte aligned, never two on one address
    writes = set()
    rows_valid = g["R"] + 2 * n if g["form"] != FP16_WIDE else 2 * n
    for (c, s, kq) in seen:
        for off in operand_offsets(g, c, s, kq):
            assert off % 16 == 0 and 0 <= off and off + 16 <= g["op_stage"]
            assert off not in writes
            writes.add(off)
    # a region's valid rows end before the next region starts
    for r in range(g["regions"] - 1):
        end = r * g["region_stride"] + skew(r) + ((rows_valid + 7) // 8) * g["sbo"]
        assert end <= (r + 1) * g["region_stride"] + skew(r + 1)
    # MMA reads: A = 128 rows, B = nb rows, from each region start, per 16-frame K step
    for r in range(g["regions"]):
        start = r * g["region_stride"] + skew(r)
        for ks in range(kt // 16):
            a_end = start + ks * 2 * LBO + 15 * g["sbo"] + 2 * LBO
            b_end = start + ks * 2 * LBO + (g["nb"] // 8 - 1) * g["sbo"] + 2 * LBO
            assert max(a_end, b_end) <= g["op_stage"], (r, ks)
    # paired form: a quarter warp's stores land in eight distinct 16-byte slots
    if g["form"] == PAIRED and ct >= 4:
        for i in range(KMAX):
            for q0 in range(0, KCONV, 8):
                offs = [operand_offsets(g, *items[(wt, i)])[0] for wt in range(q0, q0 + 8)
                        if (wt, i) in items]
                if len(offs) == 8:
                    assert len({(o % 128) // 16 for o in offs}) == 8


def test_every_feasible_shape(pkg):
    feasible = 0
    for n, split, ct, kt in shapes():
        g = geometry(pkg, n, split, ct, kt)
        if not g["ok"]:
            continue
        feasible += 1
        check_shape(g, n, split, ct, kt)
    assert feasible > 100


@pytest.mark.parametrize("n", range(1, 45))
@pytest.mark.parametrize("split", [False, True])
def test_every_input_count_has_a_shape(pkg, n, split):
    assert any(geometry(pkg, n, split, ct, kt)["ok"] for ct in (2, 4, 8) for kt in (16, 32, 64))


def test_planted_mistakes_fail(pkg):
    g = geometry(pkg, 24, False, 4, 64)
    assert g["ok"] and g["form"] == PAIRED
    bad = dict(g, region_stride=g["region_stride"] - g["sbo"])   # regions overlap
    with pytest.raises(AssertionError):
        check_shape(bad, 24, False, 4, 64)
    bad = dict(g, items=g["items"] - 1)                           # an item never converted
    with pytest.raises(AssertionError):
        check_shape(bad, 24, False, 4, 64)
    bad = dict(g, R=40)                                           # halves' rows overlap (2N = 48)
    with pytest.raises(AssertionError):
        check_shape(bad, 24, False, 4, 64)
