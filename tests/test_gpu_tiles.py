"""Tile shapes between and inside the engines, and the autotuner that picks them.

The spectra layout (ytile) and the tensor X-engine's tile (channels per CTA x
frames per stage) change only where data sits and which CTA handles which
channel, never the arithmetic of a channel: every shape must give results
bit-identical to every other shape of the same X-engine form, and within the
stated tolerance of the float64 oracle.
"""

from __future__ import annotations

import numpy as np
import pytest

from abi_driver import drive_rows
from test_gpu_tc import tol
from test_oracle_golden import load_fixture, regenerate

pytestmark = pytest.mark.gpu


def _case(n, nf, frames, seed):
    rng = np.random.default_rng(seed)
    x = rng.integers(-50, 51, size=(n, frames, 2 * nf)).astype(np.int8)
    present = rng.random((n, frames)) > 0.05
    mask = np.packbits(present.astype(np.uint8), axis=1, bitorder="little")
    return x, present, mask


def _run(pkg, torch, x, mask, xmode, tiles, max_frames=32):
    n, frames, L = x.shape
    eng = pkg.FxEngine(n, L // 2, max_frames=max_frames, xmode=xmode)
    try:
        if tiles is not None:
            eng.set_tiles(*tiles)
        acc = eng.new_acc()
        xs = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        ms = torch.from_numpy(np.ascontiguousarray(mask)).cuda()
        eng.accumulate(xs, frames, acc, mask=ms)
        torch.cuda.synchronize()
        eng.check()
        return acc.cpu().numpy()
    finally:
        eng.close()


@pytest.mark.parametrize("n_station", [5, 24, 40])
@pytest.mark.parametrize("xmode", [1, 2])
def test_every_tensor_tile_is_bit_identical(pkg, cuda, oracle, n_station, xmode):
    nf, frames = 1024, 45                      # 45: partial 16- and 32-frame stages, 2 passes
    x, present, mask = _case(n_station, nf, frames, 100 + n_station)
    ref = oracle.correlate(x, present)
    probe = pkg.FxEngine(n_station, nf, max_frames=32, xmode=xmode)
    feasible = []
    for ct in (2, 4, 8):
        for kt in (16, 32, 64):
            for ytile in (nf, ct):
                try:
                    probe.set_tiles(ytile, ct, kt)
                except pkg.abi.CorrError:
                    continue
                feasible.append((ytile, ct, kt))
    default = probe.tiles()
    probe.close()
    assert feasible, "no tensor tile accepted"
    # both layouts are accepted: contiguous rows and tiles of the tensor tile's width
    assert any(t[0] == nf for t in feasible) and any(t[0] == t[1] for t in feasible)
    assert (default["ytile"], default["xct"], default["xkt"]) in feasible
    base = _run(pkg, cuda, x, mask, xmode, None)
    assert oracle.rel_rms(base, ref) <= tol(xmode, frames)["rms"]
    assert oracle.normalized_max_err(base, ref, n_station) <= tol(xmode, frames)["per_vis"]
    for t in feasible:
        got = _run(pkg, cuda, x, mask, xmode, t)
        assert np.array_equal(got, base), f"tiles {t} differ from the default tiles"
    print(f"N={n_station} xmode={xmode}: {len(feasible)} shapes bit-identical")


@pytest.mark.parametrize("ytile", [2, 8, 32, 1024])
def test_plain_layouts_are_bit_identical(pkg, cuda, oracle, ytile):
    n, nf, frames = 7, 1024, 40
    x, present, mask = _case(n, nf, frames, 7)
    base = _run(pkg, cuda, x, mask, 0, None)
    got = _run(pkg, cuda, x, mask, 0, (ytile, 0, 0))
    assert np.array_equal(got, base)
    assert oracle.rel_rms(got, oracle.correlate(x, present)) < 1e-5


@pytest.mark.parametrize("nf", [10240, 20480])
@pytest.mark.parametrize("xmode,ytile", [(0, 32), (0, 2048), (1, 8), (2, 4)])
def test_layouts_at_a_length_that_is_not_a_power_of_two(pkg, cuda, oracle, xmode, ytile, nf):
    """n_freq 10240 = 5 x 2048, and 20480, whose frames are transformed as two
    half-length sequences writing every other bin: channel tiles of a power of
    two that divides n_freq give the same bits as contiguous rows (plain form:
    any such width; tensor forms: their own tile width)."""
    n, frames = 6, 24
    x, present, mask = _case(n, nf, frames, 10)
    base = _run(pkg, cuda, x, mask, xmode, None)
    if xmode:
        eng = pkg.FxEngine(n, nf, max_frames=32, xmode=xmode)
        t = eng.tiles()
        eng.close()
        tiles = (ytile, ytile, t["xkt"])
    else:
        tiles = (ytile, 0, 0)
    got = _run(pkg, cuda, x, mask, xmode, tiles)
    assert np.array_equal(got, base)
    bar = tol(xmode, frames)["rms"] if xmode else 1e-5
    assert oracle.rel_rms(got, oracle.correlate(x, present)) < bar


def test_bad_tiles_are_refused(pkg, cuda):
    eng = pkg.FxEngine(24, 1024, max_frames=16, xmode=2)
    try:
        before = eng.tiles()
        for bad in [(3, 8, 16), (1024, 8, 24), (1024, 16, 16), (4, 8, 16), (2048, 8, 16), (0, 8, 16)]:
            with pytest.raises(pkg.abi.CorrError):
                eng.set_tiles(*bad)
        assert eng.tiles() == before
    finally:
        eng.close()


@pytest.mark.parametrize("xmode", [0, 1, 2])
def test_autotune_picks_a_feasible_shape_with_same_results(pkg, cuda, oracle, xmode):
    n, nf, frames = 24, 2048, 40
    x, present, mask = _case(n, nf, frames, 3)
    base = _run(pkg, cuda, x, mask, xmode, None)
    eng = pkg.FxEngine(n, nf, max_frames=32, xmode=xmode)
    try:
        t = eng.autotune()
        assert t["ms_fengine"] > 0 and t["ms_xengine"] > 0
        eng.check()
        tiles = (t["ytile"], t["xct"], t["xkt"], t["fplan"])
        assert eng.tiles() == {k: t[k] for k in ("ytile", "xct", "xkt", "fplan")}
    finally:
        eng.close()
    got = _run(pkg, cuda, x, mask, xmode, tiles)
    # n_freq 2048 has one FFT plan: the same plan, only the tile may differ
    assert np.array_equal(got, base)
    print(f"xmode={xmode}: autotune chose {t}")


def test_autotune_through_abi_golden(pkg, cuda, oracle):
    fx = load_fixture("golden_15st")
    x = regenerate(oracle, fx)
    got = drive_rows(pkg, x, int(fx["n_cum"]), int(fx["frames_per_slot"]), xmode=2, autotune=True)
    rms = oracle.rel_rms(got[:, :, fx["channels"]], fx["expect_subset"])
    assert rms <= tol(2, int(fx["n_cum"]))["rms"]


@pytest.mark.parametrize("xmode", [0, 2])
def test_both_fft_plans_match_the_oracle(pkg, cuda, oracle, xmode):
    """n_freq 16384 has a three-pass and a four-pass FFT plan; both are exact to FP32."""
    n, nf, frames = 6, 16384, 24
    x, present, mask = _case(n, nf, frames, 21)
    ref = oracle.correlate(x, present)
    outs = []
    for fplan in (0, 1):
        eng = pkg.FxEngine(n, nf, max_frames=32, xmode=xmode)
        t = eng.tiles()
        eng.close()
        got = _run(pkg, cuda, x, mask, xmode, (t["ytile"], t["xct"], t["xkt"], fplan))
        assert oracle.rel_rms(got, ref) < 1e-5, f"plan {fplan}"
        assert oracle.normalized_max_err(got, ref, n) < 2e-5, f"plan {fplan}"
        outs.append(got)
    assert oracle.rel_rms(outs[0], outs[1]) < 1e-5


def test_unknown_fft_plan_is_refused(pkg, cuda):
    eng = pkg.FxEngine(4, 1024, max_frames=8, xmode=0)
    try:
        t = eng.tiles()
        with pytest.raises(pkg.abi.CorrError):
            eng.set_tiles(t["ytile"], t["xct"], t["xkt"], 1)   # n_freq 1024 has one plan
        e2 = pkg.FxEngine(4, 12288, max_frames=8, xmode=1)   # one plan too
        try:
            t2 = e2.tiles()
            for bad in (1, 2):
                with pytest.raises(pkg.abi.CorrError):
                    e2.set_tiles(t2["ytile"], t2["xct"], t2["xkt"], bad)
        finally:
            e2.close()
        with pytest.raises(pkg.abi.CorrError):
            eng.set_tiles(t["ytile"], t["xct"], t["xkt"], -1)
    finally:
        eng.close()
