"""Synthetic front end on the GPU (corrx_frontend_fill), set up like the
reference's test transmitter.

`ReplaySpec` carries the options of corr-rs/src/bin/replay.rs (same names and
defaults, replay.rs:41-165) and resolves them per station the way replay.rs:
361-372 does: a `--sample-delay INDEX:N` entry wins, otherwise the station's
delay is `delay_stride * index`; `--offset INDEX:N` starts one station N packets
late. `fill` writes frames and the validity mask, as the receive side would
assemble them from that traffic, into device memory or the pinned staging ring;
all work runs in libcorr_cuda.so's frontend kernel.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

from . import abi

SAMPLES_PER_PACKET = 4096
PATTERNS = {"zero": abi.CORRX_PATTERN_ZERO, "counter": abi.CORRX_PATTERN_COUNTER,
            "prng": abi.CORRX_PATTERN_PRNG, "sine": abi.CORRX_PATTERN_SINE}


@dataclass
class ReplaySpec:
    pattern: str = "counter"
    seed: int = 12345
    tone: float = 0.05
    start_counter: int = 10_000_000_000
    n_packets: int = 0                     # packets per station (duration * rate); 0 = no end
    drop_rate: float = 0.0
    gap_at: int = 0
    gap_len: int = 0
    sample_delay: dict = field(default_factory=dict)   # station -> samples
    delay_stride: int = 0
    offset: tuple | None = None            # (station, packets)
    ladder_frames: int = 0
    ladder_steps: int = 10

    def delays(self, n_station: int) -> list[int]:
        return [int(self.sample_delay.get(i, self.delay_stride * i)) for i in range(n_station)]

    def offsets(self, n_station: int) -> list[int]:
        out = [0] * n_station
        if self.offset is not None and 0 <= self.offset[0] < n_station:
            out[self.offset[0]] = int(self.offset[1])
        return out

    def packets_per_frame(self, n_freq: int) -> int:
        return 2 * n_freq // SAMPLES_PER_PACKET

    def first_full_frame(self, n_freq: int) -> int:
        """First frame every station sends whole (counters start mid-frame)."""
        P = self.packets_per_frame(n_freq)
        first = self.start_counter + (int(self.offset[1]) if self.offset else 0)
        return -(-first // P)

    def to_c(self, n_station: int) -> abi.corrx_frontend:
        if self.pattern not in PATTERNS:
            raise ValueError(f"pattern must be one of {sorted(PATTERNS)}")
        if n_station > abi.CORRX_FRONTEND_MAX_STATIONS:
            raise ValueError("at most 64 stations")
        fe = abi.corrx_frontend()
        fe.struct_size = C.sizeof(abi.corrx_frontend)
        fe.pattern = PATTERNS[self.pattern]
        fe.seed = self.seed
        fe.tone = self.tone
        fe.start_counter = self.start_counter
        fe.n_packets = self.n_packets
        fe.drop_rate = self.drop_rate
        fe.gap_at = self.gap_at
        fe.gap_len = self.gap_len
        fe.ladder_frames = self.ladder_frames
        fe.ladder_steps = self.ladder_steps
        for i, d in enumerate(self.delays(n_station)):
            fe.sample_delay[i] = d
        for i, o in enumerate(self.offsets(n_station)):
            fe.counter_offset[i] = o
        return fe


def fill_ptr(spec: ReplaySpec, station0: int, n_station: int, n_freq: int, frame0: int,
             frames: int, samples_ptr: int, station_stride: int, frame_stride: int,
             mask_ptr: int, mask_station_stride: int, stream: int = 0) -> None:
    """corrx_frontend_fill on raw device (or pinned host) addresses; 0 skips an output."""
    fe = spec.to_c(abi.CORRX_FRONTEND_MAX_STATIONS)
    abi.check(abi.load().corrx_frontend_fill(
        C.byref(fe), station0, n_station, n_freq, frame0, frames,
        C.c_void_p(samples_ptr or None),
        station_stride, frame_stride, C.c_void_p(mask_ptr or None), mask_station_stride,
        C.c_void_p(stream or None)), "corrx_frontend_fill")


def fill_staging(spec: ReplaySpec, correlator, slot_seq: int, frames: int | None = None,
                 stream=None) -> None:
    """Slot `slot_seq` of an ABI context's pinned staging ring, every station:
    frames [slot_seq*frames_per_slot, ...) as the receive side would leave them.
    The kernel writes the pinned host memory directly; synchronises `stream`."""
    from .engine import _stream_handle
    cfg = correlator.cfg
    fps = cfg.frames_per_slot
    frames = fps if frames is None else frames
    slot = slot_seq % cfg.block_slots
    h = _stream_handle(stream)
    for g in range(cfg.n_station):
        info = correlator.staging(g).info
        base = C.cast(info.base, C.c_void_p).value
        fill_ptr(spec, g, 1, cfg.n_freq, slot_seq * fps, frames,
                 base + slot * info.slot_stride, info.total_bytes, info.frame_stride,
                 base + info.validity_offset + slot * info.validity_bytes_per_slot,
                 info.validity_bytes_per_slot, h)
    import torch
    torch.cuda.synchronize()


def fill(spec: ReplaySpec, n_freq: int, frame0: int, samples, mask=None, stream=None) -> None:
    """Frames [frame0, frame0 + samples.shape[1]) into torch CUDA tensors.

    samples: int8 [n_station, frames, 2*n_freq] (last dim contiguous, strides
    multiples of 16 bytes); mask: optional uint8 [n_station, >= ceil(frames/8)].
    """
    from .engine import _stream_handle
    n_station, frames, L = samples.shape
    assert L == 2 * n_freq and samples.stride(2) == 1 and samples.dtype.itemsize == 1
    fill_ptr(spec, 0, n_station, n_freq, frame0, frames, samples.data_ptr(), samples.stride(0),
             samples.stride(1), 0 if mask is None else mask.data_ptr(),
             0 if mask is None else mask.stride(0), _stream_handle(stream))
