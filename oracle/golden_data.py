"""Write a golden data directory for the reference's C driver golden.c -- TEST
INFRASTRUCTURE ONLY.

The reference's golden.c (corr-cuda/tests/golden.c:230-320) reads a directory
made by its gen_golden.py: meta.txt ("n_station n_freq n_cum frames_per_slot
rows", then "b j k" per baseline), in.bin (int8 [row][station][frame][2*n_freq])
and expect.bin (complex64 [row][baseline][n_freq]). This script writes the same
three files from the oracle, with the same seeded input (golden_input, the
generator calls of gen_golden.py:59-62) and the oracle's float64 rows, so the
reference's own driver can be run against this library on a machine where the
reference checkout is absent. The input's sha256 is checked against the
fixtures in tests/golden/, which were made by running gen_golden.py itself.

usage: python -m oracle.golden_data CASE OUTDIR
       CASE: golden_partial_slot | golden_15st (corr-cuda/CMakeLists.txt:161,163)
"""

from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

from . import corr_oracle as co

CASES = {
    "golden_partial_slot": (4, 2048, 300, 128, 2),
    "golden_15st": (15, 4096, 200, 64, 2),
}


def write(case: str, outdir: Path) -> None:
    n, nf, n_cum, fps, rows = CASES[case]
    outdir.mkdir(parents=True, exist_ok=True)
    x = co.golden_input(n, nf, n_cum, rows)
    fixture = Path(__file__).resolve().parents[1] / "tests" / "golden" / f"{case}.npz"
    if fixture.exists():
        want = str(np.load(fixture)["in_sha256"])
        got = hashlib.sha256(x.tobytes()).hexdigest()
        if got != want:
            raise SystemExit(f"{case}: input sha256 {got} differs from the reference's {want}")
    x.tofile(outdir / "in.bin")
    co.correlate_rows(x, n_cum).astype(np.complex64).tofile(outdir / "expect.bin")
    with open(outdir / "meta.txt", "w") as f:
        f.write(f"{n} {nf} {n_cum} {fps} {rows}\n")
        for b, (j, k) in enumerate(co.baseline_pairs(n)):
            f.write(f"{b} {j} {k}\n")


if __name__ == "__main__":
    if len(sys.argv) != 3 or sys.argv[1] not in CASES:
        print(__doc__)
        sys.exit(2)
    write(sys.argv[1], Path(sys.argv[2]))
    print(f"{sys.argv[1]}: written to {sys.argv[2]}")
