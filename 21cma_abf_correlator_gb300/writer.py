"""Output file sets (corr_writer.h) from Python: the reference host's writer
(corr-rs/src/writer.rs) as implemented natively in libcorr_cuda.so.

    with RowWriter(dir, ["S01", "S02"], n_freq, n_cum, config_hash="...") as w:
        w.write_row(rows[0], row_ms, row_index, first_frame_id, valid_frames)

Each row is n_baseline x n_freq complex64 in baseline order (what
Correlator.rows_fetch returns per row). The library's writer thread does the
file work; a full queue drops the row (queue_full="drop") or waits ("block").
"""

from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import abi

_POLICY = {"auto": abi.CORRW_SET_AUTO, "new": abi.CORRW_SET_NEW,
           "explicit": abi.CORRW_SET_EXPLICIT}
_QUEUE = {"drop": abi.CORRW_QUEUE_DROP, "block": abi.CORRW_QUEUE_BLOCK}


class RowWriter:
    def __init__(self, directory: str, station_names: Sequence[str], n_freq: int, n_cum: int,
                 config_hash: str, *, config_version: str = "1", frames_per_slot: int = 0,
                 rows_per_fetch: int = 1, sample_rate_hz: int = 250_000_000,
                 data_shift_count: int = 0, daily_files: bool = True, set_policy: str = "auto",
                 set_tag: str | None = None, queue_rows: int = 4, queue_full: str = "drop",
                 fsync_every_rows: int = 1, file_prefix: str = "",
                 file_prefix_format: str | None = None,
                 station_net: Sequence[tuple[str, int, str]] | None = None):
        self.lib = abi.load()
        n = len(station_names)
        self.n_station, self.n_freq = n, n_freq
        self.n_baseline = n * (n + 1) // 2
        self._keep = []                                   # bytes the C struct points at

        def cs(v):
            if v is None:
                return None
            b = v.encode()
            self._keep.append(b)
            return b

        st = (abi.corrw_station * n)()
        for i, name in enumerate(station_names):
            st[i].name = cs(name)
            if station_net is not None:
                ip, port, board = station_net[i]
                st[i].group_ip, st[i].dest_port, st[i].board = cs(ip), port, cs(board)
        self._stations = st
        p = abi.corrw_params(struct_size=C.sizeof(abi.corrw_params), n_station=n, n_freq=n_freq,
                             n_cum=n_cum, frames_per_slot=frames_per_slot,
                             rows_per_fetch=rows_per_fetch, sample_rate_hz=sample_rate_hz,
                             data_shift_count=data_shift_count, daily_files=int(daily_files),
                             set_policy=_POLICY[set_policy], queue_full=_QUEUE[queue_full],
                             queue_rows=queue_rows, fsync_every_rows=fsync_every_rows,
                             dir=cs(str(directory)), file_prefix=cs(file_prefix),
                             file_prefix_format=cs(file_prefix_format),
                             config_version=cs(config_version), config_hash=cs(config_hash),
                             set_tag=cs(set_tag), stations=st)
        r = abi.corrw_resume(struct_size=C.sizeof(abi.corrw_resume))
        h = C.c_void_p()
        abi.check(self.lib.corrw_open(C.byref(p), C.byref(h), C.byref(r)), "corrw_open")
        self.h = h
        self.resume = {"rows_written": r.rows_written, "truncated_rows": r.truncated_rows,
                       "next_frame_id": r.next_frame_id if r.has_next_frame_id else None}

    def write_row(self, row, row_ms: int, row_index: int, first_frame_id: int,
                  valid_frames: Sequence[int]) -> None:
        a = np.ascontiguousarray(row, dtype=np.complex64)   # the library checks its size
        v = (C.c_uint64 * self.n_station)(*[int(x) for x in valid_frames])
        abi.check(self.lib.corrw_write_row(self.h, C.c_void_p(a.ctypes.data), a.nbytes, row_ms,
                                           row_index, first_frame_id, v), "corrw_write_row")

    def sync(self) -> None:
        abi.check(self.lib.corrw_sync(self.h), "corrw_sync")

    def stats(self) -> dict:
        s = abi.corrw_stats(struct_size=C.sizeof(abi.corrw_stats))
        abi.check(self.lib.corrw_stats_get(self.h, C.byref(s)), "corrw_stats_get")
        return {"sets_opened": s.sets_opened, "rows_written": s.rows_written,
                "rows_dropped": s.rows_dropped, "max_queued": s.max_queued,
                "set_tag": s.set_tag.decode()}

    def close(self) -> None:
        if self.h is not None and self.h.value:
            h, self.h = self.h, None
            abi.check(self.lib.corrw_close(h), "corrw_close")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
