"""The on-device synthetic front end (corrx_frontend_fill) against its oracle.

Bit-exact for every pattern, loss model, ladder, station offset and layout; a
full-size spot check; the staging ring filled in place and driven through the
C ABI; and the physics check of the reference's tools/phase_check.py: the phase
slope of every baseline's cross spectrum gives back the injected delay.
"""

from __future__ import annotations

import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fe(pkg):
    return importlib.import_module(pkg.__name__ + ".frontend")


@pytest.fixture(scope="module")
def fo():
    return importlib.import_module("oracle.frontend_oracle")


def run_fill(torch, fe, spec, n_station, n_freq, frame0, frames):
    x = torch.full((n_station, frames, 2 * n_freq), 99, dtype=torch.int8, device="cuda")
    m = torch.full((n_station, (frames + 7) // 8), 0xAA, dtype=torch.uint8, device="cuda")
    fe.fill(spec, n_freq, frame0, x, m)
    torch.cuda.synchronize()
    return x.cpu().numpy(), m.cpu().numpy()


@pytest.mark.parametrize("pattern", ["zero", "counter", "prng", "sine"])
def test_patterns_loss_and_offsets_bit_exact(pkg, cuda, fe, fo, pattern):
    n_station, n_freq, frames = 3, 4096, 13
    spec = fe.ReplaySpec(pattern=pattern, start_counter=10_000_000_001, n_packets=22,
                         drop_rate=0.03, gap_at=5, gap_len=3, delay_stride=7,
                         sample_delay={2: -5}, offset=(1, 3))
    frame0 = spec.first_full_frame(n_freq) - 1          # includes the partial first frame
    got_x, got_m = run_fill(cuda, fe, spec, n_station, n_freq, frame0, frames)
    ref_x, ref_m = fo.fill(spec, n_station, n_freq, frame0, frames, spec.delays(n_station),
                           spec.offsets(n_station))
    np.testing.assert_array_equal(got_m, ref_m)
    bits = np.unpackbits(ref_m, axis=1, bitorder="little")[:, :frames]
    assert bits.any() and not bits.all()                 # the case has valid and lost frames
    np.testing.assert_array_equal(got_x, ref_x)


def test_ladder_bit_exact(pkg, cuda, fe, fo):
    n_station, n_freq, frames = 4, 2048, 24
    spec = fe.ReplaySpec(pattern="prng", start_counter=5000, delay_stride=3,
                         ladder_frames=4, ladder_steps=3)
    frame0 = 4990
    got_x, got_m = run_fill(cuda, fe, spec, n_station, n_freq, frame0, frames)
    ref_x, ref_m = fo.fill(spec, n_station, n_freq, frame0, frames, spec.delays(n_station),
                           spec.offsets(n_station))
    np.testing.assert_array_equal(got_m, ref_m)
    np.testing.assert_array_equal(got_x, ref_x)


def test_station_range_and_padded_strides(pkg, cuda, fe, fo):
    torch = cuda
    n_freq, frames, L = 4096, 9, 8192
    spec = fe.ReplaySpec(pattern="counter", start_counter=64, drop_rate=0.1, delay_stride=2)
    buf = torch.zeros((3, frames, L + 64), dtype=torch.int8, device="cuda")
    mbuf = torch.zeros((3, 5), dtype=torch.uint8, device="cuda")
    fe.fill_ptr(spec, 4, 3, n_freq, 40, frames, buf.data_ptr(), buf.stride(0), buf.stride(1),
                mbuf.data_ptr(), mbuf.stride(0))
    torch.cuda.synchronize()
    ref_x, ref_m = fo.fill(spec, 7, n_freq, 40, frames, spec.delays(7), spec.offsets(7))
    np.testing.assert_array_equal(buf[:, :, :L].cpu().numpy(), ref_x[4:7])
    assert not buf[:, :, L:].any().item()                # the padding is not written
    np.testing.assert_array_equal(mbuf[:, :2].cpu().numpy(), ref_m[4:7])
    assert not mbuf[:, 2:].any().item()


def test_invalid_arguments_are_refused(pkg, cuda, fe):
    torch = cuda
    x = torch.zeros((1, 2, 2048), dtype=torch.int8, device="cuda")
    with pytest.raises(pkg.CorrError):                    # 1024-sample frames: not whole packets
        fe.fill(fe.ReplaySpec(), 1024, 0, x)
    with pytest.raises(pkg.CorrError):
        fe.fill(fe.ReplaySpec(drop_rate=1.0), 1024 * 2, 0, torch.zeros((1, 2, 4096),
                                                                       dtype=torch.int8,
                                                                       device="cuda"))
    with pytest.raises(pkg.CorrError):                    # stations past 64
        fe.fill_ptr(fe.ReplaySpec(), 60, 8, 2048, 0, 1, x.data_ptr(), 4096, 4096, 0, 0)


def test_full_size_spot_check(pkg, cuda, fe, fo):
    """24 inputs, n_freq 16384, 512 frames: the whole mask, and 48 random packets."""
    torch = cuda
    n_station, n_freq, frames = 24, 16384, 512
    spec = fe.ReplaySpec(pattern="prng", drop_rate=0.001, delay_stride=5, gap_at=1000,
                         gap_len=9)
    frame0 = spec.first_full_frame(n_freq)
    x = torch.empty((n_station, frames, 2 * n_freq), dtype=torch.int8, device="cuda")
    m = torch.empty((n_station, frames // 8), dtype=torch.uint8, device="cuda")
    fe.fill(spec, n_freq, frame0, x, m)
    torch.cuda.synchronize()
    P = spec.packets_per_frame(n_freq)
    delays, offsets = spec.delays(n_station), spec.offsets(n_station)
    ref_m = np.zeros((n_station, frames // 8), dtype=np.uint8)
    for s in range(n_station):
        counters = [(frame0 + f) * P + p for f in range(frames) for p in range(P)]
        ok = fo.packet_arrives(spec, offsets, counters, s).reshape(frames, P).all(axis=1)
        ref_m[s] = np.packbits(ok.astype(np.uint8), bitorder="little")
    np.testing.assert_array_equal(m.cpu().numpy(), ref_m)
    rng = np.random.default_rng(3)
    for _ in range(48):
        s, f, p = int(rng.integers(n_station)), int(rng.integers(frames)), int(rng.integers(P))
        first = ((frame0 + f) * P + p) * 4096 - delays[s]
        ref = fo.prng_sample(np.arange(first, first + 4096, dtype=np.int64), spec.seed)
        got = x[s, f, p * 4096:(p + 1) * 4096].cpu().numpy()
        np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("xmode", [0, 2])
def test_staging_filled_in_place_through_the_abi(pkg, cuda, fe, fo, oracle, xmode):
    """The kernel writes the pinned staging ring; rows equal the oracle's."""
    n, nf, fps, chunk, slots = 4, 4096, 32, 16, 3
    cfg = pkg.make_config(n, nf, fps, chunk, slots, 1)
    spec = fe.ReplaySpec(pattern="prng", start_counter=64 * 2, drop_rate=0.02, delay_stride=11)
    seqs = [2, 3, 4, 5]
    with pkg.Correlator(cfg) as c:
        if xmode:
            c.set_xengine(xmode)
        for seq in seqs:
            if seq - seqs[0] >= slots:
                c.row_slot_free(seq - slots)
            fe.fill_staging(spec, c, seq)
            c.row_accumulate(seq, fps)
        c.row_end(len(seqs) * fps)
        c.rows_wait()
        got = c.rows_fetch()[0]
    frame0 = seqs[0] * fps
    xs, ms = fo.fill(spec, n, nf, frame0, len(seqs) * fps, spec.delays(n), spec.offsets(n))
    present = np.unpackbits(ms, axis=1, bitorder="little")[:, :len(seqs) * fps].astype(bool)
    assert not present.all()
    ref = oracle.correlate(xs, present) / (len(seqs) * fps)
    assert oracle.rel_rms(got, ref) < 1e-5


@pytest.mark.parametrize("xmode", [0, 1, 2])
def test_phase_slope_gives_back_every_injected_delay(pkg, cuda, fe, xmode):
    """tools/phase_check.py's criterion on all 28 baselines of 8 inputs."""
    torch = cuda
    phase = importlib.import_module(pkg.__name__ + ".phase")
    n, nf, frames = 8, 4096, 256
    spec = fe.ReplaySpec(pattern="prng", delay_stride=3, sample_delay={5: -4})
    frame0 = spec.first_full_frame(nf)
    x = torch.empty((n, frames, 2 * nf), dtype=torch.int8, device="cuda")
    fe.fill(spec, nf, frame0, x)
    eng = pkg.FxEngine(n, nf, max_frames=frames, xmode=xmode)
    try:
        acc = eng.new_acc()
        eng.accumulate(x, frames, acc)
        eng.scale(acc, frames)
        eng.check()
        rows = acc.cpu().numpy()
    finally:
        eng.close()
    d = spec.delays(n)
    b = 0
    for j in range(n):
        for k in range(j, n):
            if j != k:
                tau = d[k] - d[j]
                r = phase.fit_delay(rows[b], 2 * nf, tau)
                assert abs(r["tau_fit"] - tau) < 0.02, (j, k, r)
                assert r["max_resid"] < 0.5, (j, k, r)
            b += 1


def test_ladder_rows_step_the_phase_slope(pkg, cuda, fe):
    """One row per ladder step (ladder_frames = frames per row): the fitted delay
    of a baseline is stride * (k - j) * step."""
    torch = cuda
    phase = importlib.import_module(pkg.__name__ + ".phase")
    n, nf, per_row, steps = 4, 4096, 64, 3
    spec = fe.ReplaySpec(pattern="prng", delay_stride=2, ladder_frames=per_row,
                         ladder_steps=steps, start_counter=per_row * 2 * 10)
    origin = spec.first_full_frame(nf)
    assert origin % per_row == 0
    x = torch.empty((n, per_row * steps, 2 * nf), dtype=torch.int8, device="cuda")
    fe.fill(spec, nf, origin, x)
    eng = pkg.FxEngine(n, nf, max_frames=per_row, xmode=0)
    try:
        for step in range(1, steps + 1):
            acc = eng.new_acc()
            eng.accumulate(x, per_row, acc, frame0=(step - 1) * per_row)
            eng.scale(acc, per_row)
            rows = acc.cpu().numpy()
            r = phase.fit_delay(rows[1], 2 * nf, 2 * step)          # baseline (0, 1)
            assert abs(r["tau_fit"] - 2 * step) < 0.02, (step, r)
            r = phase.fit_delay(rows[3], 2 * nf, 6 * step)          # baseline (0, 3)
            assert abs(r["tau_fit"] - 6 * step) < 0.02, (step, r)
    finally:
        eng.close()


def test_front_end_to_files_phase_check(pkg, cuda, fe, tmp_path):
    """The reference's phase test end to end: synthetic front end -> staging ring ->
    C ABI rows -> file set -> read the (0,1) baseline file back by the name its
    metadata gives -> phase slope = injected delay (tools/phase_check.py)."""
    import os
    wr = importlib.import_module(pkg.__name__ + ".writer")
    phase = importlib.import_module(pkg.__name__ + ".phase")
    n, nf, fps, chunk, slots = 4, 4096, 32, 32, 3
    n_cum, n_rows = 64, 3                                  # two slots per row
    tau = 5
    spec = fe.ReplaySpec(pattern="prng", start_counter=2 * 32 * 4, sample_delay={1: tau},
                         drop_rate=0.01)
    cfg = pkg.make_config(n, nf, fps, chunk, slots, 1)
    names = ["S00", "S01", "S02", "S03"]
    seq0 = 4                                               # frame 128 = the first full frame
    with pkg.Correlator(cfg) as c, wr.RowWriter(str(tmp_path), names, nf, n_cum, "h1",
                                                queue_full="block", frames_per_slot=fps) as w:
        seq = seq0
        for r in range(n_rows):
            valid = np.zeros(n, dtype=np.uint64)
            for _ in range(n_cum // fps):
                if seq - seq0 >= slots:
                    c.row_slot_free(seq - slots)
                fe.fill_staging(spec, c, seq)
                for g in range(n):
                    valid[g] += int(np.unpackbits(c.staging(g).mask[seq % slots],
                                                  bitorder="little")[:fps].sum())
                c.row_accumulate(seq, fps)
                seq += 1
            c.row_end(n_cum)
            c.rows_wait()
            row = c.rows_fetch()[0]
            w.write_row(row, 1_790_000_000_000 + 1000 * r, r,
                        (seq0 + r * n_cum // fps) * fps, valid)
        w.sync()
        tag = w.stats()["set_tag"]
    meta = (tmp_path / f"{tag}-metadata.yaml").read_text()
    line = next(l for l in meta.splitlines() if "j: 0, k: 1," in l)
    fname = line.split("file: ")[1].rstrip("}")
    x = np.fromfile(tmp_path / fname, dtype=np.complex64).reshape(-1, nf)
    assert x.shape[0] == n_rows
    r = phase.fit_delay(x, 2 * nf, tau)
    assert abs(r["tau_fit"] - tau) < 0.02 and r["max_resid"] < 0.5, r
    blocks = (tmp_path / f"{tag}-blocks.csv").read_text().splitlines()
    assert len(blocks) == n_rows * n
    assert all(int(b.split(",")[4]) + int(b.split(",")[5]) == n_cum for b in blocks)
    assert os.path.getsize(tmp_path / f"{tag}-time.bin") == 8 * n_rows
