"""Synthetic run end to end: front end -> C ABI -> output file set -> phase check.

The reference tests its whole chain this way (corr-rs/src/bin/replay.rs sends the
traffic, the correlator writes file sets, tools/phase_check.py fits the delay of
each baseline). Here every step runs in this library on one GPU:

  * the on-device front end fills each staging slot in place with the
    transmitter's packets (pattern, loss, per-station sample delays);
  * corr_row_accumulate / corr_row_end / corr_rows_fetch correlate them;
  * the native writer appends each row to a file set;
  * each baseline's file is read back by the name its metadata gives and its
    phase slope is fitted against the injected delay difference.

    python -m 21cma_abf_correlator_gb300.replay --dir /tmp/run --stations 8 --rows 4

prints one JSON summary (rows, throughput, the worst delay error).
"""

from __future__ import annotations

import argparse
import importlib
import json
import time
from pathlib import Path

import numpy as np

PKG = __package__ or __name__.rsplit(".", 1)[0]


def run(directory: str, n_station: int = 8, n_freq: int = 4096, frames_per_slot: int = 64,
        slots_per_row: int = 4, rows: int = 4, xmode: int = 2, pattern: str = "prng",
        delay_stride: int = 3, drop_rate: float = 0.001, start_counter: int = 0,
        seed: int = 12345) -> dict:
    pkg = importlib.import_module(PKG)
    fe = importlib.import_module(PKG + ".frontend")
    wr = importlib.import_module(PKG + ".writer")
    phase = importlib.import_module(PKG + ".phase")
    spec = fe.ReplaySpec(pattern=pattern, seed=seed, start_counter=start_counter,
                         delay_stride=delay_stride, drop_rate=drop_rate)
    first = spec.first_full_frame(n_freq)
    seq0 = -(-first // frames_per_slot)                 # first slot made of whole frames
    n_cum = frames_per_slot * slots_per_row
    block_slots = 3
    cfg = pkg.make_config(n_station, n_freq, frames_per_slot, frames_per_slot, block_slots, 1)
    names = [f"S{i:02d}" for i in range(n_station)]
    t0 = time.perf_counter()
    with pkg.Correlator(cfg) as c, wr.RowWriter(directory, names, n_freq, n_cum,
                                                f"replay-{n_station}-{n_freq}-{n_cum}",
                                                frames_per_slot=frames_per_slot,
                                                queue_full="block") as w:
        if xmode:
            c.set_xengine(xmode)
        seq = seq0
        for r in range(rows):
            valid = np.zeros(n_station, dtype=np.uint64)
            first_frame = seq * frames_per_slot
            for _ in range(slots_per_row):
                if seq - seq0 >= block_slots:
                    c.row_slot_free(seq - block_slots)
                fe.fill_staging(spec, c, seq)
                for g in range(n_station):
                    bits = np.unpackbits(c.staging(g).mask[seq % block_slots],
                                         bitorder="little")[:frames_per_slot]
                    valid[g] += int(bits.sum())
                c.row_accumulate(seq, frames_per_slot)
                seq += 1
            c.row_end(n_cum)
            c.rows_wait()
            row = c.rows_fetch()[0]
            w.write_row(row, int(time.time() * 1000), r, first_frame, valid)
        w.sync()
        tag = w.stats()["set_tag"]
        for s in range(max(seq - block_slots, seq0), seq):
            c.row_slot_free(s)
    dt = time.perf_counter() - t0

    # read every baseline back through the metadata's file names and fit its delay
    meta = (Path(directory) / f"{tag}-metadata.yaml").read_text().splitlines()
    files = {}
    for line in meta:
        if line.startswith("  - {index:") and "file:" in line:
            fields = dict(kv.split(": ", 1) for kv in line.strip()[3:-1].split(", "))
            files[(int(fields["j"]), int(fields["k"]))] = fields["file"]
    delays = spec.delays(n_station)
    worst = 0.0
    worst_resid = 0.0
    for (j, k), name in files.items():
        if j == k:
            continue
        x = np.fromfile(Path(directory) / name, dtype=np.complex64).reshape(-1, n_freq)
        fit = phase.fit_delay(x, 2 * n_freq, delays[k] - delays[j])
        worst = max(worst, abs(fit["tau_fit"] - (delays[k] - delays[j])))
        worst_resid = max(worst_resid, fit["max_resid"])
    samples = n_station * rows * n_cum * 2 * n_freq
    return {"set": tag, "rows": rows, "baselines": len(files), "n_cum": n_cum,
            "seconds": dt, "gsps": samples / dt / 1e9,
            "worst_delay_error_samples": worst, "worst_phase_residual_rad": worst_resid}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--dir", required=True)
    ap.add_argument("--stations", type=int, default=8)
    ap.add_argument("--n-freq", type=int, default=4096)
    ap.add_argument("--frames-per-slot", type=int, default=64)
    ap.add_argument("--slots-per-row", type=int, default=4)
    ap.add_argument("--rows", type=int, default=4)
    ap.add_argument("--xmode", type=int, default=2, help="0 plain, 1 FP16, 2 FP16 split")
    ap.add_argument("--pattern", default="prng", choices=["prng", "counter", "sine", "zero"])
    ap.add_argument("--delay-stride", type=int, default=3)
    ap.add_argument("--drop-rate", type=float, default=0.001)
    ap.add_argument("--start-counter", type=int, default=0)
    ap.add_argument("--seed", type=int, default=12345)
    a = ap.parse_args()
    print(json.dumps(run(a.dir, a.stations, a.n_freq, a.frames_per_slot, a.slots_per_row, a.rows,
                         a.xmode, a.pattern, a.delay_stride, a.drop_rate, a.start_counter,
                         a.seed)))


if __name__ == "__main__":
    main()
