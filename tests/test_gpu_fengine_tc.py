"""FFT plan 2: the tensor-core F-engine (fengine_tc.cu), n_freq 16384, FP16 spectra.

Checked with the FP16 tensor X-engine against the float64 oracle, next to plan 0
(the CUDA-core FFT) on the same inputs. Plan 2 rounds the data to FP16 once per
DFT stage on top of the FP16 spectra both plans write, and its errors are
independent across frames, so they fall as 1/sqrt(F). Tolerances: relative RMS
<= 2.5e-3/sqrt(F) and per-visibility (normalised by sqrt(V_jj V_kk)) <=
6e-3/sqrt(F). The second is the FP16 form's own bound; the first is 1.7 times its
bound. At 4096 frames they are 3.9e-5 and 9.4e-5. The layouts, missing frames and
lost packets follow the same rules as plan 0.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NF = 16384


def inputs(n, frames, seed, p_missing=0.0, p_lost=0.0):
    rng = np.random.default_rng(seed)
    x = np.clip(np.rint(24 * rng.standard_normal((n, frames, 2 * NF))), -128, 127).astype(np.int8)
    present = rng.random((n, frames)) >= p_missing
    lost = rng.random((n, frames, 32)) < p_lost
    kept = ((~lost).astype(np.uint64) << np.arange(32, dtype=np.uint64)).sum(axis=2).astype(
        np.uint32)
    return x, present, kept


def run(pkg, torch, x, frames, fplan, present=None, kept=None, ytile=None):
    n = x.shape[0]
    eng = pkg.FxEngine(n, NF, max_frames=16, xmode=pkg.abi.CORR_X_TC_FP16)
    t = eng.tiles()
    eng.set_tiles(ytile or NF, t["xct"], t["xkt"], fplan)
    acc = eng.new_acc()
    xs = torch.from_numpy(x).cuda()
    ms = None
    if present is not None:
        ms = torch.from_numpy(np.packbits(present, axis=1, bitorder="little")).cuda()
    ks = None if kept is None else torch.from_numpy(kept.view(np.int32)).cuda()
    eng.accumulate(xs, frames, acc, mask=ms, packets=ks)
    torch.cuda.synchronize()
    eng.check()
    out = acc.cpu().numpy()
    eng.close()
    return out


@pytest.mark.parametrize("n,frames,p_missing", [(3, 16, 0.0), (5, 40, 0.2), (24, 64, 0.0)])
def test_plan2_matches_oracle(pkg, cuda, oracle, n, frames, p_missing):
    x, present, _ = inputs(n, frames, seed=n, p_missing=p_missing)
    pr = present if p_missing else None
    ref = oracle.correlate(x, pr)
    got = run(pkg, cuda, x, frames, 2, present=pr)
    base = run(pkg, cuda, x, frames, 0, present=pr)
    rms, pv = oracle.rel_rms(got, ref), oracle.normalized_max_err(got, ref, n)
    print(f"n={n} F={frames}: plan 2 rel RMS {rms:.3e} per-vis {pv:.3e}; plan 0 "
          f"{oracle.rel_rms(base, ref):.3e} {oracle.normalized_max_err(base, ref, n):.3e}")
    assert rms <= 2.5e-3 / np.sqrt(frames)
    assert pv <= 6e-3 / np.sqrt(frames)
    assert oracle.rel_rms(got, base) <= 2.5e-3 / np.sqrt(frames)


def test_plan2_lost_packets(pkg, cuda, oracle):
    n, frames = 4, 32
    x, _, kept = inputs(n, frames, seed=9, p_lost=0.1)
    ref = oracle.correlate(oracle.zero_lost_packets(x, kept))
    got = run(pkg, cuda, x, frames, 2, kept=kept)
    assert oracle.rel_rms(got, ref) <= 2.5e-3 / np.sqrt(frames)
    assert oracle.normalized_max_err(got, ref, n) <= 6e-3 / np.sqrt(frames)


def test_plan2_layouts_agree(pkg, cuda):
    """Contiguous rows and tiles of the X-engine's width give the same rows."""
    n, frames = 6, 24
    x, _, _ = inputs(n, frames, seed=4)
    eng = pkg.FxEngine(n, NF, max_frames=16, xmode=pkg.abi.CORR_X_TC_FP16)
    xct = eng.tiles()["xct"]
    eng.close()
    a = run(pkg, cuda, x, frames, 2)
    b = run(pkg, cuda, x, frames, 2, ytile=xct)
    assert np.array_equal(a, b)


def test_plan2_only_for_fp16_spectra(pkg, cuda):
    for xmode in (pkg.abi.CORR_X_PLAIN_FP32, pkg.abi.CORR_X_TC_FP16_SPLIT):
        eng = pkg.FxEngine(2, NF, max_frames=16, xmode=xmode)
        t = eng.tiles()
        with pytest.raises(pkg.abi.CorrError):
            eng.set_tiles(NF, t["xct"], t["xkt"], 2)
        eng.close()
    eng = pkg.FxEngine(2, 8192, max_frames=16, xmode=pkg.abi.CORR_X_TC_FP16)
    t = eng.tiles()
    with pytest.raises(pkg.abi.CorrError):   # plan 2 exists at n_freq 16384 only
        eng.set_tiles(8192, t["xct"], t["xkt"], 2)
    eng.close()


@pytest.mark.parametrize("xmode", [1, 2])
def test_autotune_at_16384_keeps_the_cuda_core_plans(pkg, cuda, oracle, xmode):
    """The autotuner picks plan 0 or 1; plan 2 (less precise) is only chosen explicitly."""
    n, frames = 8, 32
    x, _, _ = inputs(n, frames, seed=17)
    eng = pkg.FxEngine(n, NF, max_frames=32, xmode=xmode)
    try:
        t = eng.autotune()
        assert t["fplan"] in (0, 1)
        acc = eng.new_acc()
        eng.accumulate(cuda.from_numpy(x).cuda(), frames, acc)
        cuda.cuda.synchronize()
        eng.check()
        got = acc.cpu().numpy()
    finally:
        eng.close()
    ref = oracle.correlate(x)
    assert oracle.rel_rms(got, ref) <= 2.5e-3 / np.sqrt(frames)


def test_plan2_through_the_abi(pkg, cuda, oracle):
    """corr_set_tiles chooses plan 2 for an ABI context; rows match the oracle."""
    from abi_driver import drive_rows
    rows, n, n_cum = 2, 4, 40
    rng = np.random.default_rng(23)
    x = np.clip(np.rint(24 * rng.standard_normal((rows, n, n_cum, 2 * NF))), -128, 127).astype(
        np.int8)
    got = drive_rows(pkg, x, n_cum, 16, xmode=pkg.abi.CORR_X_TC_FP16, fplan=2)
    ref = oracle.correlate_rows(x, n_cum)
    assert oracle.rel_rms(got, ref) <= 2.5e-3 / np.sqrt(n_cum)


def test_set_xengine_resets_a_plan_the_mode_cannot_use(pkg, cuda):
    cfg = pkg.make_config(2, NF, 16, 16, 3, 1)
    with pkg.Correlator(cfg) as c:
        c.set_xengine(pkg.abi.CORR_X_TC_FP16)
        t = c.tiles()
        c.set_tiles(t["ytile"], t["xct"], t["xkt"], 2)
        assert c.tiles()["fplan"] == 2
        c.set_xengine(pkg.abi.CORR_X_TC_FP16_SPLIT)
        assert c.tiles()["fplan"] == 0
