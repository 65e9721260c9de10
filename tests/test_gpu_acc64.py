"""The FP64 cross-launch integration accumulator.

Every X-engine launch sums its own frames in FP32 and adds that partial sum into
the row once. With a complex64 row (the reference's accumulator,
corr-cuda/src/kernels.cu:252-264) the row's error grows with the number of
launches it integrates; with a complex128 row it stays at one launch's error.
Checked against the float64 oracle on a 65,536-frame integration made of 4096
launches of 16 frames, for the device-resident engine and through the C ABI
(whose rows always integrate in complex128).
"""

from __future__ import annotations

import numpy as np
import pytest

from abi_driver import drive_rows

pytestmark = pytest.mark.gpu

N, NF, PER_LAUNCH = 4, 512, 16
SHORT, LONG = 256, 65536


@pytest.fixture(scope="module")
def frames():
    rng = np.random.default_rng(64)
    common = rng.normal(0.0, 1.0, size=(LONG, 2 * NF))
    x = np.empty((N, LONG, 2 * NF), dtype=np.int8)
    for s in range(N):
        v = 20.0 * (np.sqrt(0.7) * rng.normal(0.0, 1.0, size=(LONG, 2 * NF)) +
                    np.sqrt(0.3) * common)
        x[s] = np.clip(np.round(v), -128, 127).astype(np.int8)
    return x


@pytest.fixture(scope="module")
def reference(oracle, frames):
    return {F: oracle.correlate(frames[:, :F], frames_chunk=512) / F for F in (SHORT, LONG)}


def engine_rows(pkg, cuda, frames, F, precision):
    eng = pkg.FxEngine(N, NF, max_frames=PER_LAUNCH)
    try:
        eng.set_accumulator(precision)
        acc = eng.new_acc()
        xs = cuda.from_numpy(np.ascontiguousarray(frames[:, :F])).cuda()
        eng.accumulate(xs, F, acc)          # F / 16 launches
        out = eng.dump(acc, F)
        cuda.cuda.synchronize()
        eng.check()
        return out.cpu().numpy()
    finally:
        eng.close()


def test_fp64_rows_keep_one_launch_precision(pkg, cuda, oracle, frames, reference):
    err = {}
    for name, prec in (("fp32", pkg.abi.CORRX_ACC_FP32), ("fp64", pkg.abi.CORRX_ACC_FP64)):
        for F in (SHORT, LONG):
            got = engine_rows(pkg, cuda, frames, F, prec)
            err[name, F] = oracle.rel_rms(got, reference[F])
    print("rel RMS vs float64:", {f"{k[0]}@{k[1]}": f"{v:.2e}" for k, v in err.items()})
    # complex128 rows: flat from 16 to 4096 launches, at one launch's error
    assert err["fp64", LONG] < 1.5 * err["fp64", SHORT] + 1e-8
    assert err["fp64", LONG] < 1e-6
    # complex64 rows: the error grows with the launches integrated
    assert err["fp32", LONG] > 3.0 * err["fp64", LONG]


def test_dump_of_fp32_rows_is_the_reference_scaling(pkg, cuda, frames):
    """corrx_dump of a complex64 row equals corrx_scale (acc * (1.0f/frames))."""
    eng = pkg.FxEngine(N, NF, max_frames=PER_LAUNCH)
    try:
        acc = eng.new_acc()
        xs = cuda.from_numpy(np.ascontiguousarray(frames[:, :SHORT])).cuda()
        eng.accumulate(xs, SHORT, acc)
        out = eng.dump(acc, SHORT)
        eng.scale(acc, SHORT)
        cuda.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), acc.cpu().numpy())
    finally:
        eng.close()


def test_abi_long_row_integrates_in_fp64(pkg, cuda, oracle, frames, reference):
    """A 65,536-frame row through the C ABI in 16-frame chunks (4096 chunk
    launches, 64 slots of 1024 frames) stays at one launch's error."""
    x = frames[None]                      # one row
    got = drive_rows(pkg, x, LONG, 1024, chunk_frames=PER_LAUNCH, block_slots=3,
                     rows_per_fetch=1)
    short = drive_rows(pkg, np.ascontiguousarray(frames[None, :, :SHORT]), SHORT, SHORT,
                       chunk_frames=PER_LAUNCH, block_slots=3, rows_per_fetch=1)
    e_long = oracle.rel_rms(got[0], reference[LONG])
    e_short = oracle.rel_rms(short[0], reference[SHORT])
    print(f"ABI rel RMS: {SHORT} frames {e_short:.2e}, {LONG} frames {e_long:.2e}")
    assert e_long < 1.5 * e_short + 1e-8 and e_long < 1e-6
