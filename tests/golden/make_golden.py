"""Generate the golden fixtures by running the reference's own golden generator.

Runs corr-cuda/tests/gen_golden.py from the reference checkout (unmodified, as a
subprocess) for the two cases the reference registers with ctest
(corr-cuda/CMakeLists.txt:161,163):

    golden_partial_slot : 4 stations, n_freq 2048, n_cum 300, 128 frames/slot, 2 rows
    golden_15st         : 15 stations, n_freq 4096, n_cum 200, 64 frames/slot, 2 rows

and stores compact fixtures here:
  * sha256 of its in.bin (the input is regenerated by tests from the same
    seeded numpy calls, and must hash identically) and of expect.bin;
  * expect.bin itself for the small case; for the 15-station case every 16th
    channel of every row and baseline plus float64 per-(row, baseline) sums over
    all channels, which keeps the fixture small.

Usage: python tests/golden/make_golden.py REFERENCE_ROOT
(or set CORR_REFERENCE_DIR). Only needed to regenerate the committed .npz
files; the tests themselves never touch the reference.
"""

from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CASES = {
    "golden_partial_slot": (4, 2048, 300, 128, 2),
    "golden_15st": (15, 4096, 200, 64, 2),
}
SUBSET_STEP = 16


def sha256(path: Path) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for block in iter(lambda: f.read(1 << 20), b""):
            h.update(block)
    return h.hexdigest()


def main() -> int:
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CORR_REFERENCE_DIR")
    if not root:
        print("usage: make_golden.py REFERENCE_ROOT (or set CORR_REFERENCE_DIR)", file=sys.stderr)
        return 2
    ref = Path(root)
    gen = ref / "corr-cuda" / "tests" / "gen_golden.py"
    if not gen.exists():
        print(f"{gen} not found", file=sys.stderr)
        return 2
    for name, (n, nf, n_cum, fps, rows) in CASES.items():
        with tempfile.TemporaryDirectory() as td:
            out = subprocess.run([sys.executable, str(gen), str(n), str(nf), str(n_cum), str(fps),
                                  str(rows), td], capture_output=True, text=True, check=True)
            d = Path(td)
            nb = n * (n + 1) // 2
            expect = np.fromfile(d / "expect.bin", dtype=np.complex64).reshape(rows, nb, nf)
            meta_lines = (d / "meta.txt").read_text().splitlines()
            pairs = np.array([[int(v) for v in line.split()[1:]] for line in meta_lines[1:]],
                             dtype=np.int32)
            fix = dict(
                n_station=n, n_freq=nf, n_cum=n_cum, frames_per_slot=fps, rows=rows,
                seed=20260914, pairs=pairs,
                in_sha256=sha256(d / "in.bin"), expect_sha256=sha256(d / "expect.bin"),
                generator_log=out.stdout,
            )
            if name == "golden_partial_slot":
                fix["expect"] = expect
            else:
                fix["channels"] = np.arange(0, nf, SUBSET_STEP, dtype=np.int32)
                fix["expect_subset"] = expect[:, :, ::SUBSET_STEP].copy()
                e64 = expect.astype(np.complex128)
                fix["row_baseline_sum"] = e64.sum(axis=2)
                fix["row_baseline_sumsq"] = (np.abs(e64) ** 2).sum(axis=2)
            np.savez_compressed(HERE / f"{name}.npz", **fix)
            print(name, "written;", out.stdout.strip().splitlines()[-1])
    return 0


if __name__ == "__main__":
    sys.exit(main())
