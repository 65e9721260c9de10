"""Drive the C ABI the way the reference's scheduler and golden test do.

`drive_rows` is the Python form of corr-cuda/tests/golden.c:123-217: release the
slot before refilling it, fill samples and validity bits through the staging
views, submit every slot of a row, close the row with the caller's frame count,
release the held slots, wait, fetch all rows in one transfer.
"""

from __future__ import annotations

import numpy as np

ALL_VALID, HOST_ZEROED, MASK_MARKED = "all_valid", "host_zeroed", "mask_marked"


def drive_rows(pkg, x: np.ndarray, n_cum: int, frames_per_slot: int, mode: str = ALL_VALID,
               missing: np.ndarray | None = None, present: np.ndarray | None = None,
               xmode: int = 0, block_slots: int = 3, chunk_frames: int | None = None,
               rows_per_fetch: int | None = None, autotune: bool = False,
               fplan: int | None = None, devices: list[int] | None = None,
               split_mode: int = 0, plans: list | None = None):
    """x: int8 [rows, n_station, n_cum, 2*n_freq] -> complex64 [rows, n_baseline, n_freq].

    devices/split_mode: spread the context over several configured devices
    (corr_config.devices); plans: list that receives each device's placement.

    missing: bool [rows, n_cum] frames handled per `mode` (golden.c's three
    preparations); present: bool [rows, n_station, n_cum] per-station validity
    (frames with a clear bit are filled with garbage the device must ignore).
    """
    rows, n, _, L = x.shape
    nf = L // 2
    chunk = chunk_frames or min(frames_per_slot, 128)
    cfg = pkg.make_config(n, nf, frames_per_slot, chunk, block_slots, rows_per_fetch or rows,
                          split_mode=split_mode, devices=devices)
    with pkg.Correlator(cfg) as c:
        if plans is not None:   # what each device holds, as the context reports it
            plans.extend(c.device_plan(d) for d in range(c.n_devices()))
        if xmode:
            c.set_xengine(xmode)
        if autotune:
            c.autotune()
        if fplan is not None:
            t = c.tiles()
            c.set_tiles(t["ytile"], t["xct"], t["xkt"], fplan)
        views = [c.staging(g) for g in range(n)]
        submits = 0
        for r in range(rows):
            for f0 in range(0, n_cum, frames_per_slot):
                ft = min(frames_per_slot, n_cum - f0)
                slot = submits % block_slots
                if submits >= block_slots:
                    c.row_slot_free(submits)
                for g in range(n):
                    v = views[g]
                    assert not v.mask[slot].any(), "slot_free must hand back an empty mask"
                    v.samples[slot, :ft] = x[r, g, f0:f0 + ft]
                    ok = np.ones(ft, dtype=bool)
                    if missing is not None and mode != ALL_VALID:
                        miss = missing[r, f0:f0 + ft]
                        if mode == HOST_ZEROED:
                            v.samples[slot, :ft][miss] = 0
                        else:
                            v.samples[slot, :ft][miss] = 0x5A
                            ok &= ~miss
                    if present is not None:
                        pr = present[r, g, f0:f0 + ft]
                        v.samples[slot, :ft][~pr] = 0x5A
                        ok &= pr
                    bits = np.packbits(ok.astype(np.uint8), bitorder="little")
                    v.mask[slot, :bits.size] |= bits
                c.row_accumulate(submits, ft)
                submits += 1
            c.row_end(n_cum)
        first_held = max(submits - block_slots, 0)
        for s in range(submits - 1, first_held - 1, -1):
            c.row_slot_free(s)
        c.rows_wait()
        assert c.rows_pending() == rows
        out = c.rows_fetch()
        assert out.shape[0] == rows
        return out.copy()
