"""Chunks in which no station has a valid frame are skipped through the ABI.

Such a chunk contributes exactly zero to the row (all of its frames would be
zero-filled), so the library issues no host-to-device copy and no F/X work
for it. The rows must still equal the float64 oracle on the same masks, and
the device statistics must count only the chunks that were copied.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("xmode", [0, 2])
def test_missing_chunks_are_skipped_and_rows_unchanged(pkg, cuda, oracle, xmode):
    n, nf, fps, chunk, slots = 4, 2048, 64, 16, 3
    cfg = pkg.make_config(n, nf, fps, chunk, slots, 1)
    rng = np.random.default_rng(11 + xmode)
    n_slot_rows = 4
    x = rng.integers(-60, 61, size=(n_slot_rows, n, fps, 2 * nf)).astype(np.int8)
    present = np.ones((n_slot_rows, n, fps), dtype=bool)
    present[1] = False                        # slot 1: every station lost everything
    present[2, :, 16:48] = False              # slot 2: chunks 1 and 2 lost everywhere
    present[2, 1, 20] = True                  # ... except one frame of station 1 (chunk 1)
    present[3, 0, :] = False                  # slot 3: one station lost, others fine
    expect_copies = 4 + 0 + 3 + 4             # chunks with any valid frame
    with pkg.Correlator(cfg) as c:
        if xmode:
            c.set_xengine(xmode)
        for s in range(n_slot_rows):
            slot = s % slots
            if s >= slots:
                c.row_slot_free(s - slots)
            for g in range(n):
                v = c.staging(g)
                v.samples[slot] = x[s, g]
                bits = np.packbits(present[s, g].astype(np.uint8), bitorder="little")
                v.mask[slot, :] = bits
            c.row_accumulate(s, fps)
        c.row_end(n_slot_rows * fps)
        c.rows_wait()
        got = c.rows_fetch()[0]
        st = c.stats()
        assert st.transfers == expect_copies
    xs = np.concatenate([x[s] for s in range(n_slot_rows)], axis=1)          # [n, frames, L]
    ps = np.concatenate([present[s] for s in range(n_slot_rows)], axis=1)
    ref = oracle.correlate(xs, ps) / (n_slot_rows * fps)
    tol = 1e-5 if xmode in (0, 2) else 1e-3
    assert oracle.rel_rms(got, ref) < tol
