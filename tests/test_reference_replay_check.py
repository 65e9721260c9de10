"""The replay chain against the reference's own phase checker (host only).

tools/phase-replay-check.py is how the reference judges a replayed run: every
station carries one deterministic stream shifted by a known number of samples,
and each baseline's phase must follow the exact delay model (error within 5 ps,
closure over baselines, residual at the window-overlap prediction, real
autocorrelations). Here the run is built on the host: the front end's packets
from oracle/frontend_oracle.py (which the GPU front end matches bit for bit,
tests/test_gpu_frontend.py), rows from the float64 correlation oracle, files from
this library's writer; the reference's checker then reads the file set. On the
GPU the same chain (front end, C ABI, writer) is run by
`python -m 21cma_abf_correlator_gb300.replay`, whose files the checker also
passes. Skipped unless CORR_REFERENCE_DIR names a reference checkout.
"""

from __future__ import annotations

import importlib
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

REF = os.environ.get("CORR_REFERENCE_DIR")
CHECKER = Path(REF) / "tools" / "phase-replay-check.py" if REF else None

pytestmark = pytest.mark.skipif(CHECKER is None or not CHECKER.exists(),
                                reason="CORR_REFERENCE_DIR (a reference checkout) not set")


@pytest.mark.parametrize("stride", [0, 5])
def test_reference_checker_passes_the_replay_chain(pkg, oracle, tmp_path, stride):
    fo = importlib.import_module("oracle.frontend_oracle")
    fe = importlib.import_module(pkg.__name__ + ".frontend")
    wr = importlib.import_module(pkg.__name__ + ".writer")
    n, nf, n_cum, rows = 4, 2048, 1024, 2      # the checker assumes 1024-frame rows
    spec = fe.ReplaySpec(pattern="prng", seed=12345, start_counter=0, delay_stride=stride,
                         drop_rate=0.0)
    f0 = spec.first_full_frame(nf)
    x, mask = fo.fill(spec, n, nf, f0, n_cum * rows, spec.delays(n), spec.offsets(n))
    assert np.all(mask == 0xFF)
    x = x.reshape(n, rows, n_cum, 2 * nf).transpose(1, 0, 2, 3)
    vis = oracle.correlate_rows(np.ascontiguousarray(x), n_cum).astype(np.complex64)
    names = [f"S{i:02d}" for i in range(n)]
    with wr.RowWriter(str(tmp_path), names, nf, n_cum, "replay-check",
                      frames_per_slot=256, queue_full="block") as w:
        for r in range(rows):
            w.write_row(vis[r], 1_790_000_000_000 + 1000 * r, r, f0 + r * n_cum, [n_cum] * n)
        w.sync()
    run = subprocess.run([sys.executable, str(CHECKER), str(tmp_path), "--stride", str(stride),
                          "--n-freq", str(nf), "--quiet"],
                         capture_output=True, text=True, timeout=300)
    assert "VERDICT: PASS" in run.stdout, run.stdout + run.stderr
    assert run.returncode == 0
