"""Tensor-core X-engine (tcgen05) against the float64 oracle and the plain path.

Tolerances, stated against the FP64 oracle:
  FP16 split : relative RMS <= 1e-5 and per-visibility (normalised by
               sqrt(V_jj V_kk)) <= 2e-5 -- the same class as the FP32 path;
  FP16       : one rounding to 11 bits per spectrum value; the rounding errors
               are independent across frames, so the row error falls as
               1/sqrt(F): relative RMS <= 1.5e-3/sqrt(F) and per-visibility
               <= 6e-3/sqrt(F) (2.3e-5 and 9.4e-5 at the 4096-frame integration,
               inside the 1e-4 precision target).
"""

from __future__ import annotations

import numpy as np
import pytest

from abi_driver import drive_rows
from test_oracle_golden import load_fixture, regenerate

pytestmark = pytest.mark.gpu

def tol(xmode: int, frames: int) -> dict:
    if xmode == 2:   # CORR_X_TC_FP16_SPLIT
        return dict(rms=1e-5, per_vis=2e-5)
    return dict(rms=1.5e-3 / np.sqrt(frames), per_vis=6e-3 / np.sqrt(frames))   # CORR_X_TC_FP16


@pytest.fixture(scope="module")
def synth(pkg):
    import importlib
    return importlib.import_module(pkg.__name__ + ".synth")


def run_engine(pkg, torch, x, mask, xmode, max_frames=64):
    n, frames, L = x.shape
    eng = pkg.FxEngine(n, L // 2, max_frames=max_frames, xmode=xmode)
    acc = eng.new_acc()
    xs = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    ms = None if mask is None else torch.from_numpy(np.ascontiguousarray(mask)).cuda()
    eng.accumulate(xs, frames, acc, mask=ms)
    torch.cuda.synchronize()
    eng.check()
    out = acc.cpu().numpy()
    eng.close()
    return out


@pytest.mark.parametrize("xmode", [1, 2])
@pytest.mark.parametrize("name,frames", [
    ("precision-24in-nf16384", 64),
    ("plain-gpu-20in-nf8192", 96),
    ("stream-40in-nf16384", 32),
    ("plain-cpu-8in-nf1024", 256),
])
def test_tc_matches_oracle(pkg, cuda, oracle, synth, name, frames, xmode):
    w = synth.WORKLOADS[name]
    x, mask = synth.generate_numpy(w, frames)
    present = None if mask is None else synth.unpack_mask(mask, frames)
    ref = oracle.correlate(x, present)
    got = run_engine(pkg, cuda, x, mask, xmode)
    rms = oracle.rel_rms(got, ref)
    pv = oracle.normalized_max_err(got, ref, w.n_station)
    mx, rrms = oracle.significant_rel_err(got, ref, w.n_station)
    print(f"{name} xmode={xmode}: rel RMS {rms:.3e}, per-vis {pv:.3e}, "
          f"significant max {mx:.3e} rms {rrms:.3e}")
    assert rms <= tol(xmode, frames)["rms"], rms
    assert pv <= tol(xmode, frames)["per_vis"], pv


@pytest.mark.parametrize("n_station", [1, 2, 5, 16, 32, 33, 44])
@pytest.mark.parametrize("xmode", [1, 2])
def test_tc_station_counts(pkg, cuda, oracle, n_station, xmode):
    """Row-block and channel-tile geometry across station counts (1..44)."""
    rng = np.random.default_rng(n_station)
    nf, frames = 1024, 40
    x = rng.integers(-30, 31, size=(n_station, frames, 2 * nf)).astype(np.int8)
    ref = oracle.correlate(x)
    got = run_engine(pkg, cuda, x, None, xmode, max_frames=16)
    assert oracle.rel_rms(got, ref) <= tol(xmode, frames)["rms"]
    assert oracle.normalized_max_err(got, ref, n_station) <= tol(xmode, frames)["per_vis"]


@pytest.mark.parametrize("xmode", [1, 2])
def test_tc_through_abi_golden(pkg, cuda, oracle, xmode):
    fx = load_fixture("golden_15st")
    x = regenerate(oracle, fx)
    got = drive_rows(pkg, x, int(fx["n_cum"]), int(fx["frames_per_slot"]), xmode=xmode)
    rms = oracle.rel_rms(got[:, :, fx["channels"]], fx["expect_subset"])
    print(f"golden_15st xmode={xmode}: rel RMS {rms:.3e}")
    assert rms <= tol(xmode, int(fx["n_cum"]))["rms"]


def test_tc_agrees_with_plain(pkg, cuda, oracle, synth):
    w = synth.WORKLOADS["precision-24in-nf16384"]
    x, _ = synth.generate_numpy(w, 48, seed_offset=9)
    plain = run_engine(pkg, cuda, x, None, 0)
    split = run_engine(pkg, cuda, x, None, 2)
    assert oracle.rel_rms(split, plain) < 1e-5


def test_tc_zero_and_missing_frames(pkg, cuda, oracle):
    """All-missing stations give exact zeros; partial stages are zero-padded."""
    rng = np.random.default_rng(4)
    n, nf, frames = 6, 2048, 37          # 37: a partial last stage
    x = rng.integers(-128, 128, size=(n, frames, 2 * nf)).astype(np.int8)
    present = np.ones((n, frames), dtype=bool)
    present[2] = False                    # station 2 lost everything
    present[4, ::3] = False
    mask = np.packbits(present.astype(np.uint8), axis=1, bitorder="little")
    ref = oracle.correlate(x, present)
    for xmode in (1, 2):
        got = run_engine(pkg, cuda, x, mask, xmode, max_frames=16)
        for k in range(n):
            j0, k0 = min(2, k), max(2, k)
            b = oracle.baseline_index(n, j0, k0)
            assert not np.any(got[b]), "a station with no frames must correlate to exactly 0"
        assert oracle.rel_rms(got, ref) <= tol(xmode, frames)["rms"]
