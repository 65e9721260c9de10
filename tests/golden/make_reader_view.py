"""Read a file set written by this library with the reference's own readers -- TEST
INFRASTRUCTURE ONLY.

The reference's analysis tools read the correlator's output through
tools/corr_common.py (find_sets, pick_set, baseline_files, set_baselines,
metadata_field, rows_ms), tools/compare_blocks.py (load: blocks.csv) and
tools/autospectra.py (station_names, zero_fill_per_station, station_average).
This script writes one deterministic set with corrw_* (the native writer, through
writer.py), runs those readers on it, checks that what they report is what was
written (every spectrum row, row time, validity count, station name and
metadata number), and records their view with the sha256 of every file in
reader_view.json. tests/test_writer_reader_view.py rewrites the same set and
checks its bytes against those hashes, so the files the reference's readers
accepted are the files the writer still produces.

usage: CORR_REFERENCE_DIR=<reference checkout> python tests/golden/make_reader_view.py
"""

from __future__ import annotations

import hashlib
import importlib
import json
import os
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
FIXTURE = HERE / "reader_view.json"

STATIONS = ["S01", "W17", "E03"]
NF, NCUM, ROWS = 16, 8, 4
T0 = 1_790_000_000_123          # ms since the epoch (2026-09-21 UTC)
GEOMETRY = dict(config_version="7", frames_per_slot=4, rows_per_fetch=1,
                sample_rate_hz=250_000_000, file_prefix="corr-",
                file_prefix_format="%Y%m%d-%H%M%S", config_hash="abc123")


def rows():
    """The set's rows: seeded spectra, one-second row times, uneven validity."""
    rng = np.random.default_rng(2026)
    nb = len(STATIONS) * (len(STATIONS) + 1) // 2
    out = []
    for i in range(ROWS):
        spec = (rng.standard_normal((nb, NF)) + 1j * rng.standard_normal((nb, NF)))
        out.append(dict(spectrum=spec.astype(np.complex64), ms=T0 + 1000 * i, row_index=i,
                        first_frame_id=5000 + i * NCUM,
                        valid=[NCUM - (i + s) % 3 for s in range(len(STATIONS))]))
    return out


def write_set(directory: str) -> list[dict]:
    """Write the set into `directory` (TZ must be UTC); return its rows."""
    if str(REPO) not in sys.path:
        sys.path.insert(0, str(REPO))
    wr = importlib.import_module("21cma_abf_correlator_gb300.writer")
    g = GEOMETRY
    rs = rows()
    with wr.RowWriter(directory, STATIONS, NF, NCUM, g["config_hash"],
                      config_version=g["config_version"], frames_per_slot=g["frames_per_slot"],
                      rows_per_fetch=g["rows_per_fetch"], sample_rate_hz=g["sample_rate_hz"],
                      file_prefix=g["file_prefix"], file_prefix_format=g["file_prefix_format"],
                      queue_full="block") as w:
        for r in rs:
            w.write_row(r["spectrum"], r["ms"], r["row_index"], r["first_frame_id"], r["valid"])
        w.sync()
    return rs


def file_hashes(directory: str) -> dict[str, str]:
    return {p.name: hashlib.sha256(p.read_bytes()).hexdigest()
            for p in sorted(Path(directory).iterdir()) if p.is_file()}


def pairs():
    n = len(STATIONS)
    return [(j, k) for j in range(n) for k in range(j, n)]


def reader_view(directory: str, tools_dir: str, rs: list[dict]) -> dict:
    """Run the reference's readers on the set and check them against `rs`."""
    sys.path.insert(0, tools_dir)
    cc = importlib.import_module("corr_common")
    cb = importlib.import_module("compare_blocks")
    au = importlib.import_module("autospectra")

    sets = cc.find_sets(directory, require="metadata.yaml")
    s = cc.pick_set(directory)
    files = cc.baseline_files(s)
    paths = cc.set_baselines(directory)
    fields = {k: cc.metadata_field(s, k)
              for k in ("n_freq", "n_station", "n_cum", "bin_width_hz", "n_baseline")}
    times = cc.rows_ms(s)
    blocks = cb.load(directory)
    names = au.station_names(s, len(STATIONS))
    zero, rows_seen = au.zero_fill_per_station(s, len(STATIONS), ROWS)

    # what they report is what was written
    assert [(j, k) for _, j, k, _ in files] == pairs(), files
    assert [p[0] for p in paths] == list(range(len(pairs())))
    for b, (_, j, k, path) in enumerate(paths):
        got = np.fromfile(path, dtype="<c8").reshape(-1, NF)
        want = np.stack([r["spectrum"][b] for r in rs])
        assert np.array_equal(got, want), path
    assert times == [r["ms"] for r in rs]
    assert int(fields["n_freq"]) == NF and int(fields["n_station"]) == len(STATIONS)
    assert int(fields["n_cum"]) == NCUM
    assert float(fields["bin_width_hz"]) == GEOMETRY["sample_rate_hz"] / (2 * NF)
    assert names == dict(enumerate(STATIONS))
    for r in rs:
        for st, v in enumerate(r["valid"]):
            assert blocks[(r["first_frame_id"], st)] == (r["row_index"], NCUM, v, NCUM - v)
    assert rows_seen == ROWS
    assert zero == [sum(NCUM - r["valid"][st] for r in rs) for st in range(len(STATIONS))]
    autos = {}
    for b, (_, j, k, path) in enumerate(paths):
        if j != k:
            continue
        mean, _, used = au.station_average(path, NF, 0)
        want = np.stack([r["spectrum"][b].real for r in rs]).astype(np.float64).mean(axis=0)
        # station_average sums each block of rows in float32
        assert used == ROWS and np.allclose(mean, want, rtol=1e-6, atol=1e-6), path
        autos[STATIONS[j]] = [float(v) for v in mean]

    return {
        "sets": [[x["tag"], x["layout"]] for x in sets],
        "picked": s["tag"],
        "baseline_files": [[i, j, k, f] for i, j, k, f in files],
        "metadata": fields,
        "rows_ms": times,
        "blocks": sorted([ff, st, *v] for (ff, st), v in blocks.items()),
        "station_names": {str(i): n for i, n in names.items()},
        "zero_fill_per_station": zero,
        "autospectra_mean": autos,
    }


def main() -> None:
    ref = os.environ.get("CORR_REFERENCE_DIR")
    if not ref:
        sys.exit("set CORR_REFERENCE_DIR to the reference checkout")
    os.environ["TZ"] = "UTC"
    time.tzset()
    with tempfile.TemporaryDirectory() as d:
        rs = write_set(d)
        view = reader_view(d, str(Path(ref) / "tools"), rs)
        out = {"files": file_hashes(d), "reader": view,
               "readers": ["tools/corr_common.py", "tools/compare_blocks.py",
                           "tools/autospectra.py"]}
    FIXTURE.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"{FIXTURE.name}: {len(out['files'])} files read by the reference's readers")


if __name__ == "__main__":
    main()
