"""Expected output file sets -- TEST INFRASTRUCTURE ONLY.

The checker for the library's file-set writer (corrw_*), never the product: only
tests/ may import it. It restates, in Python, what the reference's host writer
puts on disk for a sequence of rows:
  * file names <P><sj><sk>-<T>.bin and <P><T>-{time.bin,time.txt,blocks.csv,
    metadata.yaml}                                      corr-rs/src/writer.rs:88-148
  * one whole row per baseline file per integration, baseline-major rows;
    time.bin int64 LE ms; time.txt local "%Y-%m-%d %H:%M:%S.mmm";
    blocks.csv row_index,station,first_frame_id,n_cum,valid,zero_filled
                                                        writer.rs:796-866, 1745-1751
  * a new set when a row's local day is later than the set's, named by that
    row's local time                                    writer.rs:575-630, 1652-1659
  * metadata.yaml keys and values                       writer.rs:1867-1973
Parity unpinned: the reference is Rust (no toolchain here) and its tests build
their expectations in code, so this restatement follows those cited lines.
"""

from __future__ import annotations

import os
import time

import numpy as np


def local_stamp(ms: int, fmt: str) -> str:
    return time.strftime(fmt, time.localtime(ms // 1000))


def text_time(ms: int) -> str:
    return f"{local_stamp(ms, '%Y-%m-%d %H:%M:%S')}.{ms % 1000:03d}"


def fmt_f64(v: float) -> str:
    """Rust's Display for f64: shortest round-trip decimal, no exponent."""
    r = repr(float(v))
    if "e" in r or "E" in r:
        from decimal import Decimal
        r = format(Decimal(r), "f")
    if r.endswith(".0"):
        r = r[:-2]
    return r


def pairs(n: int) -> list[tuple[int, int]]:
    return [(j, k) for j in range(n) for k in range(j, n)]


class Names:
    def __init__(self, prefix: str, stamp: str):
        self.prefix, self.stamp = prefix, stamp

    @property
    def tag(self) -> str:
        return self.prefix + self.stamp

    def baseline(self, sj: str, sk: str) -> str:
        return f"{self.prefix}{sj}{sk}-{self.stamp}.bin"


def metadata(g: dict, names: Names, day: str, kind: str, continuation: str | None,
             first_row: tuple[int, int] | None, rows_at_open: int) -> str:
    n, nf, n_cum = len(g["stations"]), g["n_freq"], g["n_cum"]
    frame_rate = g["sample_rate_hz"] / (2 * nf)
    out = [
        "# Written once, when this file set is created. A resumed run checks",
        "# the config_hash rather than rewriting geometry that the existing",
        "# rows were produced with.",
        f"config_version: {g['config_version']}",
        f"config_hash: {g['config_hash']}",
        "format: raw-complex64",
        "byte_order: little_endian",
        "component: {real: float32, imag: float32}",
        "baseline_layout: baseline_major",
        f"n_freq: {nf}",
        f"n_cum: {n_cum}",
        f"n_station: {n}",
        f"n_baseline: {n * (n + 1) // 2}",
        f"sample_rate_hz: {g['sample_rate_hz']}",
        f"bin_width_hz: {fmt_f64(frame_rate)}",
        f"frame_rate_hz: {fmt_f64(frame_rate)}",
        f"row_period_s: {fmt_f64(n_cum / frame_rate)}",
        f"fft: {{type: R2C, length: {2 * nf}, window: rectangular, nyquist: dropped}}",
        "fft_normalisation: none",
        "row_normalisation: divide_by_n_cum",
        "missing_frames: zero_filled",
        "fftshift: false",
        "bin0: DC",
        f"data_shift_count: {g['data_shift_count']}",
        f"frames_per_slot: {g['frames_per_slot']}",
        f"rows_per_fetch: {g['rows_per_fetch']}",
        f"baseline_row_bytes: {nf * 8}",
        "# --- the file set this metadata belongs to ---",
        f"set_prefix: {names.tag}",
        'rows_ms_txt_format: "local YYYY-mm-DD HH:MM:SS.mmm"',
        f"file_prefix: {names.prefix}",
        f"stamp: {names.stamp}",
        f"set_day: {day}",
        f"set_kind: {kind}",
    ]
    if continuation is not None:
        out.append(f"set_continuation_of: {continuation}")
    out += [
        f"first_row_index: {first_row[0] if first_row else 0}",
        f"first_frame_id: {first_row[1] if first_row else 0}",
        f"rows_at_open: {rows_at_open}",
        f"local_timezone: {os.environ.get('TZ', '')}",
        f"local_utc_offset_s: {time.localtime().tm_gmtoff}",
        "stations:",
    ]
    for i, s in enumerate(g["stations"]):
        out.append(f"  - {{index: {i}, name: {s}}}")
    out.append("baselines:")
    for b, (j, k) in enumerate(pairs(n)):
        out.append(f"  - {{index: {b}, j: {j}, k: {k}, "
                   f"file: {names.baseline(g['stations'][j], g['stations'][k])}}}")
    return "\n".join(out) + "\n"


def expected_sets(g: dict, rows: list[dict], first_kind: str = "start") -> dict[str, dict]:
    """{tag: {file name: bytes}} for rows written into fresh daily sets.

    g: stations, n_freq, n_cum, sample_rate_hz, data_shift_count, frames_per_slot,
    rows_per_fetch, config_version, config_hash, file_prefix, file_prefix_format.
    rows: dicts with spectrum [B, n_freq] complex64, ms, row_index,
    first_frame_id, valid (per station).
    """
    stations = g["stations"]
    sets: dict[str, dict] = {}
    cur = None
    day = None
    for r in rows:
        rday = local_stamp(r["ms"], "%Y%m%d")
        if cur is None or rday > day:
            names = Names(g["file_prefix"], local_stamp(r["ms"], g["file_prefix_format"]))
            kind = first_kind if cur is None else "rollover"
            cont = None if cur is None else cur.tag
            files = {names.baseline(stations[j], stations[k]): b"" for j, k in pairs(len(stations))}
            files.update({f"{names.tag}-time.bin": b"", f"{names.tag}-time.txt": b"",
                          f"{names.tag}-blocks.csv": b""})
            files[f"{names.tag}-metadata.yaml"] = metadata(
                g, names, rday, kind, cont, (r["row_index"], r["first_frame_id"]), 0).encode()
            sets[names.tag] = files
            cur, day = names, rday
        files = sets[cur.tag]
        spec = np.ascontiguousarray(r["spectrum"], dtype=np.complex64)
        for b, (j, k) in enumerate(pairs(len(stations))):
            files[cur.baseline(stations[j], stations[k])] += spec[b].tobytes()
        files[f"{cur.tag}-time.bin"] += int(r["ms"]).to_bytes(8, "little", signed=True)
        files[f"{cur.tag}-time.txt"] += (text_time(r["ms"]) + "\n").encode()
        for s, v in enumerate(r["valid"]):
            files[f"{cur.tag}-blocks.csv"] += (
                f"{r['row_index']},{s},{r['first_frame_id']},{g['n_cum']},{v},"
                f"{g['n_cum'] - v}\n").encode()
    return sets

