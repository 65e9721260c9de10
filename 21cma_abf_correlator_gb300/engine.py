"""Device-resident FX engine (corr_gb300.h) driven with torch CUDA tensors.

torch supplies device memory and streams only; every byte of F- and X-engine
work runs in libcorr_cuda.so's kernels through `corrx_accumulate`.
"""

from __future__ import annotations

import ctypes as C

from . import abi


def _stream_handle(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class FxEngine:
    """F-engine (FFT) + X-engine over int8 frames already in device memory."""

    def __init__(self, n_station: int, n_freq: int, max_frames: int,
                 xmode: int = abi.CORR_X_PLAIN_FP32, device_id: int = 0):
        self.lib = abi.load()
        p = abi.corrx_params()
        p.struct_size = C.sizeof(abi.corrx_params)
        p.n_station = n_station
        p.n_freq = n_freq
        p.max_frames = max_frames
        p.xmode = xmode
        p.device_id = device_id
        h = C.c_void_p()
        abi.check(self.lib.corrx_create(C.byref(p), C.byref(h)), "corrx_create")
        self.h = h
        self.n_station = n_station
        self.n_freq = n_freq
        self.n_baseline = n_station * (n_station + 1) // 2
        self.max_frames = max_frames
        self.xmode = xmode

    def close(self) -> None:
        if self.h is not None and self.h.value:
            self.lib.corrx_destroy(self.h)
        self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def set_accumulator(self, precision: int) -> None:
        """abi.CORRX_ACC_FP32 (complex64 rows, the default) or abi.CORRX_ACC_FP64
        (complex128 rows: each launch's FP32 sums are added in double)."""
        abi.check(self.lib.corrx_set_accumulator(self.h, precision), "corrx_set_accumulator")
        self.acc64 = precision == abi.CORRX_ACC_FP64

    def new_acc(self):
        """A zeroed row in the engine's accumulator precision."""
        import torch
        dt = torch.complex128 if getattr(self, "acc64", False) else torch.complex64
        return torch.zeros((self.n_baseline, self.n_freq), dtype=dt, device="cuda")

    def dump(self, acc, frames: int, out=None, stream=None):
        """complex64 row = acc / frames (rounded once); returns `out`."""
        import torch
        if out is None:
            out = torch.empty((self.n_baseline, self.n_freq), dtype=torch.complex64,
                              device=acc.device)
        abi.check(self.lib.corrx_dump(self.h, C.c_void_p(acc.data_ptr()), frames,
                                      C.c_void_p(out.data_ptr()),
                                      C.c_void_p(_stream_handle(stream))), "corrx_dump")
        return out

    def accumulate(self, samples, frames: int, acc, mask=None, mask_bit0: int = 0,
                   stream=None, frame0: int = 0, packets=None, packets_frame0: int = 0) -> None:
        """acc += correlation of frames [frame0, frame0+frames) of `samples`.

        samples: int8 CUDA tensor [n_station, n_frames, 2*n_freq] (last dim contiguous,
        strides multiples of 16 bytes); mask: optional uint8 CUDA tensor
        [n_station, mask_bytes] with bit (mask_bit0 + f) LSB-first per frame f;
        packets: optional int32/uint32 CUDA tensor [n_station, n_words], word
        (packets_frame0 + f) of a station holding one bit per 1024-sample packet
        of frame f (bit 0 first); a clear bit zero-fills that packet
        (corrx_accumulate_packets).
        """
        assert samples.dtype.itemsize == 1 and samples.stride(2) == 1
        assert samples.shape[2] == 2 * self.n_freq and samples.shape[0] == self.n_station
        base = samples.data_ptr() + frame0 * samples.stride(1)
        mptr = 0 if mask is None else mask.data_ptr()
        mstride = 0 if mask is None else mask.stride(0)
        if packets is not None:
            assert packets.dtype.itemsize == 4 and packets.stride(1) == 1
            abi.check(self.lib.corrx_accumulate_packets(
                self.h, C.c_void_p(base), samples.stride(0), samples.stride(1),
                C.c_void_p(mptr), mstride, mask_bit0, C.c_void_p(packets.data_ptr()),
                packets.stride(0), packets_frame0, frames, C.c_void_p(acc.data_ptr()),
                C.c_void_p(_stream_handle(stream))), "corrx_accumulate_packets")
            return
        abi.check(self.lib.corrx_accumulate(
            self.h, C.c_void_p(base), samples.stride(0), samples.stride(1), C.c_void_p(mptr),
            mstride, mask_bit0, frames, C.c_void_p(acc.data_ptr()),
            C.c_void_p(_stream_handle(stream))), "corrx_accumulate")

    def scale(self, acc, frames: int, stream=None) -> None:
        abi.check(self.lib.corrx_scale(self.h, C.c_void_p(acc.data_ptr()), frames,
                                       C.c_void_p(_stream_handle(stream))), "corrx_scale")

    def check(self) -> None:
        abi.check(self.lib.corrx_check(self.h), "corrx_check")

    def tiles(self) -> dict:
        """Current (ytile, xct, xkt): spectra tile width and tensor X tile shape."""
        t = abi.corrx_tiles(struct_size=C.sizeof(abi.corrx_tiles))
        abi.check(self.lib.corrx_get_tiles(self.h, C.byref(t)), "corrx_get_tiles")
        return {"ytile": t.ytile, "xct": t.xct, "xkt": t.xkt, "fplan": t.fplan}

    def set_tiles(self, ytile: int, xct: int = 0, xkt: int = 0, fplan: int = 0) -> None:
        t = abi.corrx_tiles(struct_size=C.sizeof(abi.corrx_tiles), ytile=ytile, xct=xct, xkt=xkt,
                            fplan=fplan)
        abi.check(self.lib.corrx_set_tiles(self.h, C.byref(t)), "corrx_set_tiles")

    def autotune(self, stream=None) -> dict:
        """Time every feasible tile shape on this device; keep the fastest F+X pair."""
        t = abi.corrx_tiles(struct_size=C.sizeof(abi.corrx_tiles))
        abi.check(self.lib.corrx_autotune(self.h, C.c_void_p(_stream_handle(stream)), C.byref(t)),
                  "corrx_autotune")
        return {"ytile": t.ytile, "xct": t.xct, "xkt": t.xkt, "fplan": t.fplan,
                "ms_fengine": t.ms_fengine, "ms_xengine": t.ms_xengine}
