"""CPU oracle for the synthetic front end -- TEST INFRASTRUCTURE ONLY.

The checker for corrx_frontend_fill, never the product: only tests/ and the
smoke() of __graft_entry__ may import it. The library has no CPU generator.

It restates, in numpy uint64/float64 arithmetic, the reference's test
transmitter and the receive side's frame assembly:
  * prng_sample (splitmix64-style hash of the sample index)   corr-rs/src/bin/replay.rs:212-226
  * build_packet patterns zero / counter / prng / sine        replay.rs:228-266
  * per-station start counter, sample delay                   replay.rs:361-372
  * gap and uniform loss                                      replay.rs:417-426
  * delay ladder and its origin                               replay.rs:314-320, 431-441
  * frame id = counter / P, packet at (counter % P)*4096      corr-rs/src/frame.rs:74-89
  * a frame is valid only if all P packets arrived            corr-rs/src/assemble.rs:1000-1070
The time-based stall of the transmitter is not modelled.

Parity unpinned: the reference is Rust (no toolchain here) and ships no test
vectors for the transmitter, so this restatement is checked by reading against
the cited lines, by tests/test_frontend_oracle.py (a per-sample pure-Python
transliteration of the same lines) and, end to end, by the phase-slope property
the reference's own tools/phase_check.py tests (fitted delay = injected delay).
"""

from __future__ import annotations

import math

import numpy as np

SAMPLES_PER_PACKET = 4096                 # corr-rs/src/config.rs:26
PATTERNS = ("zero", "counter", "prng", "sine")
_U = np.uint64
_TAU = math.tau                           # f64 nearest to 2*pi, as std::f64::consts::TAU


def _u(x) -> np.ndarray:
    return np.asarray(x, dtype=np.uint64)


def prng_sample(i, seed: int) -> np.ndarray:
    """replay.rs:212-226 for an array of absolute sample indices (int64)."""
    with np.errstate(over="ignore"):
        x = (np.asarray(i, dtype=np.int64).astype(np.uint64) + _U(seed)) * _U(0x9E3779B97F4A7C15)
        x ^= x >> _U(30)
        x *= _U(0xBF58476D1CE4E5B9)
        x ^= x >> _U(27)
        x *= _U(0x94D049BB133111EB)
        x ^= x >> _U(31)
    return (((x >> _U(8)) % _U(9)).astype(np.int16) - 4).astype(np.int8)


def counter_packets(counters, stations) -> np.ndarray:
    """replay.rs:235-249: one 4096-sample packet per (counter, station) pair."""
    counters = _u(counters).ravel()
    stations = _u(stations).ravel()
    with np.errstate(over="ignore"):
        x = counters * _U(0x9E3779B97F4A7C15) + stations * _U(0x12345678)
        out = np.empty((counters.size, SAMPLES_PER_PACKET), dtype=np.int8)
        for k in range(SAMPLES_PER_PACKET):
            x ^= x << _U(13)
            x ^= x >> _U(7)
            x ^= x << _U(17)
            out[:, k] = (((x >> _U(3)) % _U(9)).astype(np.int16) - 4).astype(np.int8)
    return out


def sine_packet(counter: int, station: int, seed: int, tone: float) -> np.ndarray:
    """replay.rs:257-264, each operation rounded on its own, libm sin."""
    phase = (float(counter) + float(seed) * float(station)) * tone * _TAU
    out = np.empty(SAMPLES_PER_PACKET, dtype=np.int8)
    for i in range(SAMPLES_PER_PACKET):
        t = phase + float(i) * tone * _TAU / float(SAMPLES_PER_PACKET)
        v = math.sin(t) * 4.0
        # Rust f64::round: half away from zero (|v| - floor(|v|) is exact)
        r = math.floor(abs(v))
        if abs(v) - r >= 0.5:
            r += 1
        out[i] = r if v >= 0 else -r
    return out


def ladder_origin(spec, n_freq: int) -> int:
    """replay.rs:315-320 (u64 arithmetic)."""
    if spec.ladder_frames <= 0:
        return 0
    first = ((spec.start_counter * SAMPLES_PER_PACKET) % (1 << 64)) // (2 * n_freq)
    return -(-first // spec.ladder_frames) * spec.ladder_frames


def frame_delay(spec, delays, s: int, frame: int, n_freq: int) -> int:
    """replay.rs:431-441: station s's sample delay in `frame`."""
    if spec.ladder_frames <= 0:
        return int(delays[s])
    origin = ladder_origin(spec, n_freq)
    k = 1 + (frame - origin) // spec.ladder_frames if frame >= origin else 1
    if spec.ladder_steps > 0:
        k = min(k, spec.ladder_steps)
    return int(delays[s]) * k


def packet_arrives(spec, offsets, counters: np.ndarray, s: int) -> np.ndarray:
    """replay.rs:361-369 and 411-426: which counters station s put on the wire."""
    counters = np.asarray(counters, dtype=object)
    first = spec.start_counter + int(offsets[s])
    ok = np.array([c >= first for c in counters], dtype=bool)
    n = np.array([c - first for c in counters], dtype=object)
    if spec.n_packets:
        ok &= np.array([v < spec.n_packets for v in n], dtype=bool)
    if spec.gap_len > 0:
        ok &= ~np.array([spec.gap_at <= v < spec.gap_at + spec.gap_len for v in n], dtype=bool)
    if spec.drop_rate > 0.0:
        thr = int(spec.drop_rate * 1_000_000.0)
        c64 = _u([int(c) % (1 << 64) for c in counters])
        with np.errstate(over="ignore"):
            x = c64 * _U(0x2545F4914F6CDD1D) + _U(s)
            x ^= x >> _U(33)
        ok &= ~((x % _U(1_000_000)) < _U(thr))
    return ok


def fill(spec, n_station: int, n_freq: int, frame0: int, frames: int,
         delays, offsets) -> tuple[np.ndarray, np.ndarray]:
    """Frames [frame0, frame0+frames) of every station and their validity mask.

    Returns samples [station][frame][2*n_freq] int8 (the pattern for every
    packet, whether or not it arrived) and mask [station][ceil(frames/8)] uint8,
    bit f (LSB first) set iff all packets of frame frame0+f arrived.
    """
    L = 2 * n_freq
    P = L // SAMPLES_PER_PACKET
    samples = np.zeros((n_station, frames, L), dtype=np.int8)
    mask = np.zeros((n_station, (frames + 7) // 8), dtype=np.uint8)
    for s in range(n_station):
        counters = [(frame0 + f) * P + p for f in range(frames) for p in range(P)]
        arrives = packet_arrives(spec, offsets, counters, s).reshape(frames, P)
        for f in range(frames):
            if arrives[f].all():
                mask[s, f // 8] |= np.uint8(1 << (f % 8))
        if spec.pattern == "counter":
            pk = counter_packets(counters, [s] * len(counters))
            samples[s] = pk.reshape(frames, L)
        elif spec.pattern == "prng":
            for f in range(frames):
                frame = frame0 + f
                first = frame * P * SAMPLES_PER_PACKET - frame_delay(spec, delays, s, frame, n_freq)
                samples[s, f] = prng_sample(np.arange(first, first + L, dtype=np.int64), spec.seed)
        elif spec.pattern == "sine":
            for f in range(frames):
                for p in range(P):
                    c = (frame0 + f) * P + p
                    samples[s, f, p * SAMPLES_PER_PACKET:(p + 1) * SAMPLES_PER_PACKET] = \
                        sine_packet(c, s, spec.seed, spec.tone)
        elif spec.pattern != "zero":
            raise ValueError(f"unknown pattern {spec.pattern!r}")
    return samples, mask
