"""Seeded synthetic int8 voltage streams for the benchmark and test workloads.

Signal model (per input i, sample t):
    x_i[t] = clip(round(sigma*(sqrt(1-rho)*n_i[t] + sqrt(rho)*s[t - d_i]) + tones), -128, 127)
with n_i and s independent N(0,1) streams, d_i an integer delay drawn from the
seed, and optional tones A*cos(2*pi*ch*t/L) (bin `ch` of the L = 2*n_freq FFT).
Packet loss: each 1024-sample packet of each input is lost with probability p;
a frame with any lost packet is declared missing in the validity mask, which is
the reference's frame-granular rule (corr-rs/src/assemble.rs:39-45). With
`words=True` the generators also return the packet-granular form of the same
loss: one 32-bit word per (input, frame), bit p set when packet p arrived
(corrx_accumulate_packets). No public dataset is involved; these stand in for
the front-end streams.

Two back ends with the same model: numpy (CPU; small cases, the oracle's
inputs) and torch on the GPU (large cases; bench inputs are generated in HBM,
outside any timed region).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PACKET_SAMPLES = 1024


@dataclass(frozen=True)
class Workload:
    name: str
    n_station: int
    n_freq: int
    frames: int            # frames per integration
    sigma: float
    rho: float
    max_delay: int         # delays drawn from 0..max_delay
    tones: tuple = ()      # (channel, amplitude, n_inputs or None for all)
    loss: float = 0.0      # packet loss probability
    seed: int = 0
    blocks: int = 1        # integration blocks (batching workload)
    block_frames: tuple = ()  # (lo, hi) frames per block, uniform

    @property
    def fft_len(self) -> int:
        return 2 * self.n_freq

    @property
    def n_baseline(self) -> int:
        return self.n_station * (self.n_station + 1) // 2


# The five workloads of the benchmark specification, named by their shapes.
WORKLOADS = {
    "plain-cpu-8in-nf1024": Workload("plain-cpu-8in-nf1024", 8, 1024, 256, 20.0, 0.3, 7,
                                     seed=1001),
    "plain-gpu-20in-nf8192": Workload("plain-gpu-20in-nf8192", 20, 8192, 2048, 16.0, 0.3, 31,
                                      tones=((1234, 4.0, None),), loss=0.001, seed=1002),
    "precision-24in-nf16384": Workload("precision-24in-nf16384", 24, 16384, 4096, 24.0, 0.2, 63,
                                       seed=1003),
    "batching-24in-nf16384": Workload("batching-24in-nf16384", 24, 16384, 8192, 24.0, 0.2, 63,
                                      loss=0.005, seed=1004, blocks=64,
                                      block_frames=(512, 8192)),
    "stream-40in-nf16384": Workload("stream-40in-nf16384", 40, 16384, 4096, 24.0, 0.2, 127,
                                    tones=((3000, 8.0, 10), (9000, 8.0, 10)), loss=0.002,
                                    seed=1005),
    # Beyond the specification's five: the longest frames accepted (n_freq 32768,
    # 65536-sample frames, transformed as two half-length sequences).
    "wide-24in-nf32768": Workload("wide-24in-nf32768", 24, 32768, 2048, 24.0, 0.2, 63,
                                  seed=1006),
}


def delays_for(w: Workload) -> np.ndarray:
    rng = np.random.default_rng([w.seed, 7])
    return rng.integers(0, w.max_delay + 1, size=w.n_station)


def mask_bytes(frames: int) -> int:
    return (frames + 7) // 8


def _tone_inputs(w: Workload, tone) -> range:
    n = w.n_station if tone[2] is None else min(tone[2], w.n_station)
    return range(n)


def generate_numpy(w: Workload, frames: int, seed_offset: int = 0, words: bool = False):
    """(samples int8 [N, frames, L], mask uint8 [N, ceil(frames/8)] or None)
    [+ packet words uint32 [N, frames] or None with words=True]."""
    L = w.fft_len
    T = frames * L
    rng = np.random.default_rng([w.seed, seed_offset])
    d = delays_for(w)
    s = rng.standard_normal(T + w.max_delay)
    t = np.arange(T, dtype=np.float64)
    out = np.empty((w.n_station, frames, L), dtype=np.int8)
    a, b = math.sqrt(1.0 - w.rho), math.sqrt(w.rho)
    for i in range(w.n_station):
        x = w.sigma * (a * rng.standard_normal(T) +
                       b * s[w.max_delay - d[i]: w.max_delay - d[i] + T])
        for tone in w.tones:
            if i in _tone_inputs(w, tone):
                x += tone[1] * np.cos(2.0 * np.pi * tone[0] * (t % L) / L)
        out[i] = np.clip(np.rint(x), -128, 127).astype(np.int8).reshape(frames, L)
    mask = kept = None
    if w.loss > 0:
        per_frame = w.fft_len // PACKET_SAMPLES
        lost = rng.random((w.n_station, frames, per_frame)) < w.loss
        mask = pack_mask(~lost.any(axis=2))
        kept = ((~lost).astype(np.uint64) << np.arange(per_frame, dtype=np.uint64)).sum(
            axis=2).astype(np.uint32)
    return (out, mask, kept) if words else (out, mask)


def loss_mask_numpy(w: Workload, frames: int, rng) -> np.ndarray:
    per_frame = w.fft_len // PACKET_SAMPLES
    lost = rng.random((w.n_station, frames, per_frame)) < w.loss
    present = ~lost.any(axis=2)
    return pack_mask(present)


def pack_mask(present: np.ndarray) -> np.ndarray:
    """bool [N, frames] -> uint8 [N, ceil(frames/8)], bit f of byte f//8 (LSB first)."""
    return np.packbits(present.astype(np.uint8), axis=1, bitorder="little")


def unpack_mask(mask: np.ndarray, frames: int) -> np.ndarray:
    return np.unpackbits(mask, axis=1, bitorder="little")[:, :frames].astype(bool)


def generate_torch(w: Workload, frames: int, seed_offset: int = 0, device: str = "cuda",
                   words: bool = False):
    """Same model on the GPU with torch's generator: (int8 [N, frames, L], uint8 mask or None)
    [+ packet words int32 [N, frames] (bit patterns of uint32) or None with words=True]."""
    import torch
    L = w.fft_len
    T = frames * L
    g = torch.Generator(device=device)
    g.manual_seed(w.seed * 1000003 + seed_offset)
    d = delays_for(w)
    a, b = math.sqrt(1.0 - w.rho), math.sqrt(w.rho)
    s = torch.randn(T + w.max_delay, generator=g, device=device, dtype=torch.float32)
    out = torch.empty((w.n_station, frames, L), dtype=torch.int8, device=device)
    tone_wave = {}
    for tone in w.tones:
        ph = torch.arange(L, device=device, dtype=torch.float64)
        tone_wave[tone] = (tone[1] * torch.cos(2.0 * math.pi * tone[0] * ph / L)).float()
    for i in range(w.n_station):
        x = torch.randn(T, generator=g, device=device, dtype=torch.float32)
        x.mul_(a).add_(s[w.max_delay - int(d[i]): w.max_delay - int(d[i]) + T], alpha=b)
        x.mul_(w.sigma)
        xv = x.view(frames, L)
        for tone in w.tones:
            if i in _tone_inputs(w, tone):
                xv.add_(tone_wave[tone])
        out[i] = xv.round_().clamp_(-128, 127).to(torch.int8)
        del x, xv
    del s
    mask = kept = None
    if w.loss > 0:
        per_frame = L // PACKET_SAMPLES
        lost = torch.rand((w.n_station, frames, per_frame), generator=g, device=device) < w.loss
        if words:
            bits = torch.arange(per_frame, device=device, dtype=torch.int64)
            k64 = ((~lost).to(torch.int64) << bits).sum(dim=2)
            kept = torch.where(k64 >= 2 ** 31, k64 - 2 ** 32, k64).to(torch.int32)
        present = (~lost.any(dim=2)).to(torch.uint8)
        nb = mask_bytes(frames)
        pad = nb * 8 - frames
        if pad:
            present = torch.cat([present, torch.zeros((w.n_station, pad), dtype=torch.uint8,
                                                      device=device)], dim=1)
        weights = (2 ** torch.arange(8, device=device, dtype=torch.int32)).view(1, 1, 8)
        mask = (present.view(w.n_station, nb, 8).to(torch.int32) * weights).sum(dim=2).to(
            torch.uint8)
    return (out, mask, kept) if words else (out, mask)


def block_plan(w: Workload, seed_offset: int = 0) -> list[tuple[int, int]]:
    """Batching workload: (first frame in the pooled ring, frames) for each block."""
    rng = np.random.default_rng([w.seed, 99, seed_offset])
    lo, hi = w.block_frames
    plan = []
    for _ in range(w.blocks):
        n = int(rng.integers(lo, hi + 1))
        first = int(rng.integers(0, w.frames - n + 1))
        plan.append((first, n))
    return plan
