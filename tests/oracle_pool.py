"""The float64 oracle over a whole integration, spread over the host's cores.

A full row at 24 inputs and n_freq 16384 (4096 frames) is about two minutes of
the oracle on one core; split by frames over a spawn-started process pool (the
partial sums add) it takes seconds on a many-core host. The frames are handed
over through a file the workers map read-only.
"""

from __future__ import annotations

import multiprocessing as mp
import os
import tempfile
from pathlib import Path

import numpy as np


def _partial(args):
    path, present_path, f0, f1 = args
    from oracle import corr_oracle
    x = np.load(path, mmap_mode="r")
    pr = None if present_path is None else np.load(present_path, mmap_mode="r")[:, f0:f1]
    return corr_oracle.correlate(np.ascontiguousarray(x[:, f0:f1]), pr, frames_chunk=16)


class OraclePool:
    """A spawn-context pool of oracle workers (safe beside a CUDA context)."""

    def __init__(self, processes: int | None = None):
        self.n = processes or max(1, os.cpu_count() or 1)
        self.pool = mp.get_context("spawn").Pool(self.n)
        self.dir = tempfile.TemporaryDirectory()

    def close(self):
        self.pool.terminate()
        self.pool.join()
        self.dir.cleanup()

    def correlate(self, x: np.ndarray, present: np.ndarray | None = None) -> np.ndarray:
        """sum_f Y_j conj(Y_k) over all frames: complex128 [n_baseline, n_freq]."""
        d = Path(self.dir.name)
        xp = d / "x.npy"
        np.save(xp, x)
        pp = None
        if present is not None:
            pp = d / "present.npy"
            np.save(pp, present)
        F = x.shape[1]
        cuts = np.linspace(0, F, min(F, 4 * self.n) + 1).astype(int)
        jobs = [(str(xp), None if pp is None else str(pp), int(a), int(b))
                for a, b in zip(cuts[:-1], cuts[1:]) if b > a]
        total = None
        for part in self.pool.imap_unordered(_partial, jobs):
            total = part if total is None else total + part
        return total
