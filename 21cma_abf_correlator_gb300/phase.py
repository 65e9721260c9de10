"""Phase-slope validation of correlated rows (the reference's tools/phase_check.py).

A station whose sample stream is delayed by tau samples relative to another
gives a cross spectrum C(c) = Y_j(c) conj(Y_k(c)) = |Y_j(c)|^2 exp(+2 pi i c tau / L)
with tau = d_k - d_j, so the phase of the row-averaged cross spectrum is a line
in channel with slope 2 pi tau / L. `fit_delay` restates phase_check.py:67-72
(unwrap, least squares) and :97-111 (average the complex rows, not the phases;
tau = slope * L / 2 pi; residual against the theoretical phase, wrapped).
"""

from __future__ import annotations

import numpy as np


def fit_delay(rows: np.ndarray, n_fft: int, tau_theory: float | None = None) -> dict:
    """rows: complex [n_rows, n_freq] (or [n_freq]) of one baseline."""
    x = np.asarray(rows)
    mean = x.mean(axis=0) if x.ndim == 2 else x
    bins = np.arange(mean.shape[-1], dtype=float)
    phase = np.angle(mean)
    unwrapped = np.unwrap(phase)
    A = np.vstack([bins, np.ones_like(bins)]).T
    slope, intercept = np.linalg.lstsq(A, unwrapped, rcond=None)[0]
    out = {"slope": float(slope), "intercept": float(intercept),
           "tau_fit": float(slope * n_fft / (2 * np.pi))}
    if tau_theory is not None:
        theory = np.angle(np.exp(1j * 2 * np.pi * bins * tau_theory / n_fft))
        resid = np.angle(np.exp(1j * (phase - theory)))
        out["max_resid"] = float(np.abs(resid).max())
        out["mean_resid"] = float(np.abs(resid).mean())
    return out
