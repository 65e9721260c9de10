"""The synthetic front end's oracle against a literal, per-sample transliteration
of the reference transmitter (corr-rs/src/bin/replay.rs), and the arithmetic the
GPU kernel relies on (digit-sum mod 9, xorshift64 jump matrices), on the CPU.
"""

from __future__ import annotations

import importlib
import math
import random
from types import SimpleNamespace

import numpy as np

fo = importlib.import_module("oracle.frontend_oracle")
M64 = (1 << 64) - 1


# -- replay.rs, one sample at a time, in Python integers ------------------------

def prng_sample_scalar(i: int, seed: int) -> int:          # replay.rs:212-226
    x = ((i & M64) + seed) & M64
    x = (x * 0x9E3779B97F4A7C15) & M64
    x ^= x >> 30
    x = (x * 0xBF58476D1CE4E5B9) & M64
    x ^= x >> 27
    x = (x * 0x94D049BB133111EB) & M64
    x ^= x >> 31
    return ((x >> 8) % 9) - 4


def counter_packet_scalar(counter: int, station: int) -> list[int]:   # replay.rs:235-249
    x = ((counter * 0x9E3779B97F4A7C15) + station * 0x12345678) & M64
    out = []
    for _ in range(4096):
        x ^= (x << 13) & M64
        x ^= x >> 7
        x ^= (x << 17) & M64
        out.append(((x >> 3) % 9) - 4)
    return out


def lost_scalar(counter: int, index: int, drop_rate: float) -> bool:   # replay.rs:421-426
    if drop_rate <= 0.0:
        return False
    x = ((counter * 0x2545F4914F6CDD1D) + index) & M64
    x ^= x >> 33
    return (x % 1_000_000) < int(drop_rate * 1_000_000.0)


def spec(**kw):
    base = dict(pattern="prng", seed=12345, tone=0.05, start_counter=10_000_000_000, n_packets=0,
                drop_rate=0.0, gap_at=0, gap_len=0, ladder_frames=0, ladder_steps=10)
    base.update(kw)
    return SimpleNamespace(**base)


def test_prng_matches_transliteration():
    rng = random.Random(5)
    idx = [rng.randrange(-(1 << 40), 1 << 45) for _ in range(500)] + [-1, 0, 1, -(1 << 63)]
    for seed in (0, 12345, (1 << 64) - 1):
        got = fo.prng_sample(np.array(idx, dtype=np.int64), seed)
        assert [int(v) for v in got] == [prng_sample_scalar(i, seed) for i in idx]


def test_prng_samples_cover_minus4_to_4():
    v = fo.prng_sample(np.arange(100_000, dtype=np.int64), 12345)
    assert set(np.unique(v).tolist()) == set(range(-4, 5))


def test_counter_pattern_matches_transliteration():
    counters = [10_000_000_000, 10_000_000_001, 3, (1 << 62) + 17]
    stations = [0, 5, 23, 63]
    got = fo.counter_packets(counters, stations)
    for r, (c, s) in enumerate(zip(counters, stations)):
        assert got[r].tolist() == counter_packet_scalar(c, s)


def test_sine_pattern_rounding_and_range():
    p = fo.sine_packet(10_000_000_000, 3, 12345, 0.05)
    assert p.min() >= -4 and p.max() <= 4
    phase = (float(10_000_000_000) + 12345.0 * 3.0) * 0.05 * math.tau
    for k in (0, 1, 100, 4095):
        t = phase + float(k) * 0.05 * math.tau / 4096.0
        v = math.sin(t) * 4.0
        assert p[k] == int(math.copysign(math.floor(abs(v) + 0.5), v))


def test_loss_gap_offset_and_end_make_frames_invalid():
    n_freq = 4096                                 # 2 packets per frame
    sp = spec(start_counter=100, n_packets=40, gap_at=10, gap_len=3, drop_rate=0.05)
    offsets = [0, 5]
    frame0, frames = 48, 20                       # counters 96 .. 135
    _, mask = fo.fill(spec(**{**vars(sp), "pattern": "zero"}), 2, n_freq, frame0, frames,
                      [0, 0], offsets)
    for s in range(2):
        first = 100 + offsets[s]
        for f in range(frames):
            ok = True
            for p in range(2):
                c = (frame0 + f) * 2 + p
                n = c - first
                sent = c >= first and n < 40 and not (10 <= n < 13)
                ok &= sent and not lost_scalar(c, s, 0.05)
            assert bool(mask[s, f // 8] >> (f % 8) & 1) == ok, (s, f)
    # bits past `frames` in the last byte stay clear
    assert mask[0, -1] >> (frames % 8) == 0


def test_ladder_steps_the_delay():
    n_freq = 2048                                 # 1 packet per frame
    sp = spec(start_counter=1000, ladder_frames=4, ladder_steps=3)
    origin = fo.ladder_origin(sp, n_freq)
    assert origin == 1000                         # first frame 1000 is already a multiple of 4
    delays = [0, 7]
    ks = [fo.frame_delay(sp, delays, 1, f, n_freq) // 7 for f in range(996, 1020)]
    assert ks == [1] * 8 + [2] * 4 + [3] * 12     # below origin: 1; capped at 3


def test_mod9_digit_sum_identity():
    """The kernel reduces a 64-bit value mod 9 by summing its 24-bit digits."""
    rng = random.Random(9)
    for x in [rng.getrandbits(64) for _ in range(20000)] + [0, M64, 1 << 63, (1 << 48) - 1]:
        r = (x & 0xFFFFFF) + ((x >> 24) & 0xFFFFFF) + (x >> 48)
        assert r % 9 == x % 9


def test_xorshift_jump_matrices():
    """Lane l of the kernel starts at T^(128 l) x0, built by squaring T 7 times."""
    def step(x):
        x ^= (x << 13) & M64
        x ^= x >> 7
        x ^= (x << 17) & M64
        return x

    def apply(cols, x):
        y = 0
        for b in range(64):
            if x >> b & 1:
                y ^= cols[b]
        return y

    P = [step(1 << b) for b in range(64)]
    for _ in range(7):
        P = [apply(P, P[j]) for j in range(64)]
    J = [[1 << b for b in range(64)]]
    for _ in range(1, 32):
        J.append([apply(J[-1], P[j]) for j in range(64)])
    x0 = 0x0123456789ABCDEF
    seq = [x0]
    for _ in range(31 * 128):
        seq.append(step(seq[-1]))
    for lane in (0, 1, 5, 31):
        assert apply(J[lane], x0) == seq[128 * lane]
