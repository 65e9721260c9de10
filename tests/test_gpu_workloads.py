"""The benchmark workloads' shapes against the float64 oracle (GPU).

Each workload runs at its full station count and channel count, with a frame
count the oracle finishes in seconds; the full-length integrations are covered
by size-independent checks in test_gpu_fullsize.py. Tolerances (plain FP32
path): per-visibility error normalised by sqrt(V_jj V_kk) <= 1e-5, relative RMS
<= 1e-5.
"""

from __future__ import annotations

import numpy as np
import pytest

from abi_driver import drive_rows

pytestmark = pytest.mark.gpu

PER_VIS_TOL = 1e-5
REL_RMS_TOL = 1e-5

CASES = [
    ("plain-cpu-8in-nf1024", 256),      # full integration length
    ("plain-gpu-20in-nf8192", 96),
    ("precision-24in-nf16384", 40),
    ("stream-40in-nf16384", 12),
    ("batching-24in-nf16384", 24),
]


@pytest.fixture(scope="module")
def synth(pkg):
    import importlib
    return importlib.import_module(pkg.__name__ + ".synth")


@pytest.mark.parametrize("name,frames", CASES)
def test_device_resident_plain_matches_oracle(pkg, cuda, oracle, synth, name, frames):
    torch = cuda
    w = synth.WORKLOADS[name]
    x, mask = synth.generate_numpy(w, frames)
    present = None if mask is None else synth.unpack_mask(mask, frames)
    ref = oracle.correlate(x, present)
    eng = pkg.FxEngine(w.n_station, w.n_freq, max_frames=16)
    xs = torch.from_numpy(x).cuda()
    ms = None if mask is None else torch.from_numpy(np.ascontiguousarray(mask)).cuda()
    acc = eng.new_acc()
    eng.accumulate(xs, frames, acc, mask=ms)
    torch.cuda.synchronize()
    eng.check()
    got = acc.cpu().numpy()
    per_vis = oracle.normalized_max_err(got, ref, w.n_station)
    rms = oracle.rel_rms(got, ref)
    assert per_vis < PER_VIS_TOL, f"{name}: per-visibility {per_vis:.3e}"
    assert rms < REL_RMS_TOL, f"{name}: rel RMS {rms:.3e}"
    eng.close()


def test_abi_path_with_packet_loss_matches_oracle(pkg, cuda, oracle, synth):
    """20 inputs, nf=8192, 0.1% packet loss: masks through the staging ring."""
    w = synth.WORKLOADS["plain-gpu-20in-nf8192"]
    frames = 80
    x, mask = synth.generate_numpy(w, frames, seed_offset=3)
    present = synth.unpack_mask(mask, frames)
    # force some loss so the mask path is exercised even at this small size
    present[3, 5] = present[0, 17] = present[19, 79] = False
    ref = oracle.correlate(x, present) / frames
    got = drive_rows(pkg, x[None], frames, frames_per_slot=32, present=present[None],
                     chunk_frames=16)
    assert oracle.normalized_max_err(got[0], ref, w.n_station) < PER_VIS_TOL
    assert oracle.rel_rms(got[0], ref) < REL_RMS_TOL


def test_chunk_and_slot_boundaries_do_not_matter(pkg, cuda, oracle, synth):
    """Same frames, different slot/chunk geometry: same visibilities."""
    w = synth.WORKLOADS["plain-cpu-8in-nf1024"]
    x, _ = synth.generate_numpy(w, 100)
    ref = oracle.correlate(x) / 100
    for fps, chunk in ((100, 100), (64, 7), (13, 13), (33, 1)):
        got = drive_rows(pkg, x[None], 100, frames_per_slot=fps, chunk_frames=chunk,
                         block_slots=4)
        assert oracle.rel_rms(got[0], ref) < REL_RMS_TOL, (fps, chunk)


@pytest.mark.parametrize("xmode", [0, 1, 2])
@pytest.mark.parametrize("n_freq", [512, 1024, 2048, 4096, 6144, 8192, 10240, 12288, 14336,
                                    16384, 18432, 20480, 22528, 24576, 26624, 28672, 30720,
                                    32768])
def test_every_transform_length(pkg, cuda, oracle, n_freq, xmode):
    """Every F-engine size, writing each spectra format (FP32, FP16, FP16 hi/lo):
    the powers of two, the multiples of 2048 that are 3, 5 or 7 x 2^k, and those
    above 16384, whose frames are transformed as two half-length sequences."""
    torch = cuda
    rng = np.random.default_rng(n_freq)
    n, frames = 3, 5
    x = rng.integers(-128, 128, size=(n, frames, 2 * n_freq)).astype(np.int8)
    ref = oracle.correlate(x)
    eng = pkg.FxEngine(n, n_freq, max_frames=4, xmode=xmode)
    acc = eng.new_acc()
    eng.accumulate(torch.from_numpy(x).cuda(), frames, acc)
    torch.cuda.synchronize()
    eng.check()
    got = acc.cpu().numpy()
    # FP16 spectra: one rounding to 11 bits, errors falling as 1/sqrt(frames)
    tol = {0: PER_VIS_TOL, 2: 2e-5, 1: 6e-3 / np.sqrt(frames)}[xmode]
    assert oracle.normalized_max_err(got, ref, n) < tol
    eng.close()


@pytest.mark.parametrize("n_freq", [6144, 10240, 12288, 14336, 18432, 26624, 32768])
def test_abi_at_multiples_of_2048(pkg, cuda, oracle, n_freq):
    """The reference takes any multiple of 2048 (corr-cuda/src/corr_cuda.cpp:501-509):
    rows through the C ABI at the lengths that are not powers of two, with
    missing frames, in the plain form and both tensor forms."""
    rng = np.random.default_rng(n_freq + 1)
    n, n_cum, fps = 5, 48, 16
    x = rng.integers(-40, 41, size=(2, n, n_cum, 2 * n_freq)).astype(np.int8)
    present = np.ones((2, n, n_cum), dtype=bool)
    present[0, 1, 7] = present[1, 4, 40] = present[1, 0, 0] = False
    ref = oracle.correlate_rows(x, n_cum, present)
    for xmode, tol in ((0, REL_RMS_TOL), (2, 2e-5), (1, 1.5e-3 / np.sqrt(n_cum))):
        got = drive_rows(pkg, x, n_cum, fps, present=present, chunk_frames=8, block_slots=3,
                         rows_per_fetch=2, xmode=xmode)
        assert oracle.rel_rms(got, ref) < tol, (n_freq, xmode)
        if xmode == 0:
            assert oracle.normalized_max_err(got, ref, n) < PER_VIS_TOL


@pytest.mark.parametrize("n", [64, 100, 128])
def test_many_stations_on_one_engine(pkg, cuda, oracle, n):
    """The plain X-engine up to 128 stations (two-frame shared-memory stages from
    73 padded stations); the tensor forms stop at 64 with CORR_ERR_NOT_IMPL."""
    torch = cuda
    nf, frames = 1024, 7
    rng = np.random.default_rng(n)
    x = rng.integers(-40, 41, size=(n, frames, 2 * nf)).astype(np.int8)
    eng = pkg.FxEngine(n, nf, max_frames=8)
    try:
        acc = eng.new_acc()
        eng.accumulate(torch.from_numpy(x).cuda(), frames, acc)
        torch.cuda.synchronize()
        eng.check()
        ref = oracle.correlate(x)
        got = acc.cpu().numpy()
        assert oracle.rel_rms(got, ref) < REL_RMS_TOL
        assert oracle.normalized_max_err(got, ref, n) < PER_VIS_TOL
    finally:
        eng.close()
    if n > 64:
        with pytest.raises(pkg.abi.CorrError) as e:
            pkg.FxEngine(n, nf, max_frames=8, xmode=1)
        assert e.value.status == pkg.abi.CORR_ERR_NOT_IMPL


def test_extreme_samples(pkg, cuda, oracle):
    """Full-scale int8 (+127/-128 square waves, impulses): sign handling and range."""
    torch = cuda
    n, nf, frames = 4, 2048, 6
    L = 2 * nf
    x = np.zeros((n, frames, L), dtype=np.int8)
    x[0] = np.where(np.arange(L) % 2 == 0, 127, -128).astype(np.int8)
    x[1, :, 0] = -128
    x[2] = -128
    x[3] = np.random.default_rng(1).integers(-128, 128, size=(frames, L))
    ref = oracle.correlate(x)
    eng = pkg.FxEngine(n, nf, max_frames=8)
    acc = eng.new_acc()
    eng.accumulate(torch.from_numpy(x).cuda(), frames, acc)
    torch.cuda.synchronize()
    got = acc.cpu().numpy()
    assert oracle.rel_rms(got, ref) < REL_RMS_TOL
    eng.close()
