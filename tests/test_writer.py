"""The native file-set writer (corrw_*) against the restated on-disk format
(oracle/writer_oracle.py, after corr-rs/src/writer.rs). Host-only: no GPU.

Covers what the reference's writer tests cover: every file of a fresh set,
rollover at the local day, resuming with truncation back to the shortest file,
a half-written row, sidecars that ran ahead, a changed configuration refused,
a row of the wrong size refused, and a full queue dropping whole rows.
"""

from __future__ import annotations

import importlib
import os
import time
from pathlib import Path

import numpy as np
import pytest

wo = importlib.import_module("oracle.writer_oracle")

STATIONS = ["S01", "W17", "E03"]
NF, NCUM = 16, 8
DAY = 86_400_000


@pytest.fixture(autouse=True)
def utc():
    old = os.environ.get("TZ")
    os.environ["TZ"] = "UTC"
    time.tzset()
    yield
    if old is None:
        os.environ.pop("TZ", None)
    else:
        os.environ["TZ"] = old
    time.tzset()


def geometry(**kw):
    g = dict(stations=STATIONS, n_freq=NF, n_cum=NCUM, sample_rate_hz=250_000_000,
             data_shift_count=0, frames_per_slot=4, rows_per_fetch=1, config_version="7",
             config_hash="abc123", file_prefix="corr-", file_prefix_format="%Y%m%d-%H%M%S")
    g.update(kw)
    return g


def make_writer(pkg, d, g, **kw):
    wr = importlib.import_module(pkg.__name__ + ".writer")
    args = dict(config_version=g["config_version"], frames_per_slot=g["frames_per_slot"],
                rows_per_fetch=g["rows_per_fetch"], sample_rate_hz=g["sample_rate_hz"],
                file_prefix=g["file_prefix"], file_prefix_format=g["file_prefix_format"],
                queue_full="block")
    args.update(kw)
    return wr.RowWriter(str(d), g["stations"], g["n_freq"], g["n_cum"], g["config_hash"], **args)


def rows_for(ms_list, seed=0, first_index=0):
    rng = np.random.default_rng(seed)
    B = len(STATIONS) * (len(STATIONS) + 1) // 2
    out = []
    for i, ms in enumerate(ms_list):
        spec = (rng.standard_normal((B, NF)) + 1j * rng.standard_normal((B, NF))).astype(np.complex64)
        out.append({"spectrum": spec, "ms": ms, "row_index": first_index + i,
                    "first_frame_id": 1000 + (first_index + i) * NCUM,
                    "valid": [NCUM - (i + s) % 3 for s in range(len(STATIONS))]})
    return out


def write_all(w, rows):
    for r in rows:
        w.write_row(r["spectrum"], r["ms"], r["row_index"], r["first_frame_id"], r["valid"])


def on_disk(d: Path) -> dict[str, bytes]:
    return {p.name: p.read_bytes() for p in d.iterdir() if p.is_file()}


def assert_sets_equal(d: Path, expect: dict[str, dict]):
    got = on_disk(d)
    want = {name: data for files in expect.values() for name, data in files.items()}
    assert sorted(got) == sorted(want)
    for name, data in want.items():
        if name.endswith("-metadata.yaml"):
            assert got[name].decode().splitlines() == data.decode().splitlines(), name
        else:
            assert got[name] == data, name


@pytest.mark.parametrize("queue_rows", [0, 3])
def test_fresh_set_every_file(pkg, tmp_path, queue_rows):
    g = geometry()
    t0 = 1_790_000_000_123
    rows = rows_for([t0 + 1000 * i for i in range(5)])
    with make_writer(pkg, tmp_path, g, queue_rows=queue_rows, queue_full="block") as w:
        assert w.resume["rows_written"] == 0
        write_all(w, rows)
        w.sync()
        st = w.stats()
        assert st["rows_written"] == 5 and st["rows_dropped"] == 0 and st["sets_opened"] == 1
        assert st["set_tag"] == "corr-" + wo.local_stamp(t0, "%Y%m%d-%H%M%S")
    assert_sets_equal(tmp_path, wo.expected_sets(g, rows))


def test_rollover_at_the_local_day(pkg, tmp_path):
    g = geometry()
    midnight = (1_790_000_000_000 // DAY + 1) * DAY
    rows = rows_for([midnight - 1500, midnight - 500, midnight + 250, midnight + 1250,
                     midnight - 100])                                  # last: clock went back
    with make_writer(pkg, tmp_path, g) as w:
        write_all(w, rows)
        w.sync()
        assert w.stats()["sets_opened"] == 2
    expect = wo.expected_sets(g, rows)
    assert len(expect) == 2
    tags = sorted(expect)
    meta = (tmp_path / f"{tags[1]}-metadata.yaml").read_text()
    assert "set_kind: rollover" in meta and f"set_continuation_of: {tags[0]}" in meta
    assert_sets_equal(tmp_path, expect)


def test_resume_truncates_to_the_shortest_file(pkg, tmp_path):
    g = geometry()
    now = int(time.time() * 1000)
    rows = rows_for([now + 10 * i for i in range(4)])
    with make_writer(pkg, tmp_path, g) as w:
        write_all(w, rows)
        w.sync()
        tag = w.stats()["set_tag"]
    names = wo.Names(g["file_prefix"], tag[len(g["file_prefix"]):])
    # a crash: one baseline got half of a 5th row, time.bin a partial record,
    # and blocks.csv a line of a row whose spectra never arrived
    with open(tmp_path / names.baseline("S01", "W17"), "ab") as f:
        f.write(b"\x01" * (NF * 4))
    with open(tmp_path / f"{tag}-time.bin", "ab") as f:
        f.write(b"\x02\x03\x04")
    with open(tmp_path / f"{tag}-blocks.csv", "a") as f:
        f.write("4,0,1032,8,8,0\n")
    more = rows_for([now + 100 + 10 * i for i in range(2)], seed=1, first_index=4)
    with make_writer(pkg, tmp_path, g) as w:                        # AUTO: today's set
        assert w.resume == {"rows_written": 4, "truncated_rows": 0,
                            "next_frame_id": rows[-1]["first_frame_id"] + NCUM}
        assert w.stats()["set_tag"] == tag
        write_all(w, more)
    expect = wo.expected_sets(g, rows + more)
    assert_sets_equal(tmp_path, expect)


def test_spectra_ahead_of_sidecars_are_cut_back(pkg, tmp_path):
    g = geometry()
    now = int(time.time() * 1000)
    rows = rows_for([now + i for i in range(3)])
    with make_writer(pkg, tmp_path, g) as w:
        write_all(w, rows)
        w.sync()
        tag = w.stats()["set_tag"]
    names = wo.Names(g["file_prefix"], tag[len(g["file_prefix"]):])
    for j in range(3):                          # a whole 4th row of spectra, no sidecars
        for k in range(j, 3):
            with open(tmp_path / names.baseline(STATIONS[j], STATIONS[k]), "ab") as f:
                f.write(b"\x00" * (NF * 8))
    with make_writer(pkg, tmp_path, g, set_policy="explicit", set_tag=tag) as w:
        assert w.resume["rows_written"] == 3 and w.resume["truncated_rows"] == 1
    assert_sets_equal(tmp_path, wo.expected_sets(g, rows))


def test_changed_configuration_is_refused(pkg, tmp_path):
    g = geometry()
    now = int(time.time() * 1000)
    with make_writer(pkg, tmp_path, g) as w:
        write_all(w, rows_for([now]))
    with pytest.raises(pkg.CorrError) as e:
        make_writer(pkg, tmp_path, geometry(config_hash="different"))
    assert e.value.status == pkg.abi.CORR_ERR_STATE and "config_hash" in e.value.message
    # a new set for the same day is the way out
    with make_writer(pkg, tmp_path, geometry(config_hash="different"), set_policy="new") as w:
        write_all(w, rows_for([now + 2000]))
        w.sync()
        tag = w.stats()["set_tag"]
    assert "set_kind: second_set" in (tmp_path / f"{tag}-metadata.yaml").read_text()


def test_bad_rows_and_unknown_sets_are_refused(pkg, tmp_path):
    g = geometry()
    with make_writer(pkg, tmp_path, g) as w:
        with pytest.raises(pkg.CorrError) as e:
            w.write_row(np.zeros((6, NF - 1), np.complex64), 0, 0, 0, [NCUM] * 3)
        assert e.value.status == pkg.abi.CORR_ERR_ARG
    with pytest.raises(pkg.CorrError) as e:
        make_writer(pkg, tmp_path, g, set_policy="explicit", set_tag="corr-nope")
    assert e.value.status == pkg.abi.CORR_ERR_STATE


def test_one_set_per_open_without_daily_files(pkg, tmp_path):
    g = geometry()
    midnight = (1_790_000_000_000 // DAY + 1) * DAY
    rows = rows_for([midnight - 10, midnight + 10])
    with make_writer(pkg, tmp_path, g, daily_files=False) as w:
        write_all(w, rows)
        w.sync()
        st = w.stats()
    assert st["sets_opened"] == 1 and st["rows_written"] == 2
    names = [p.name for p in tmp_path.iterdir()]
    assert sum(n.endswith("-blocks.csv") for n in names) == 1


def test_full_queue_drops_whole_rows(pkg, tmp_path):
    g = geometry(n_freq=4096)
    now = int(time.time() * 1000)
    B = 6
    spec = np.ones((B, 4096), np.complex64)
    n_rows = 200
    with make_writer(pkg, tmp_path, g, queue_rows=1, queue_full="drop") as w:
        for i in range(n_rows):
            w.write_row(spec * i, now + i, i, i * NCUM, [NCUM] * 3)
        w.sync()
        st = w.stats()
    assert st["rows_written"] + st["rows_dropped"] == n_rows
    for p in tmp_path.glob("*.bin"):
        if p.name.endswith("-time.bin"):
            assert p.stat().st_size == 8 * st["rows_written"]
        else:
            data = np.fromfile(p, np.complex64)
            assert data.size == 4096 * st["rows_written"]
            rows = data.reshape(-1, 4096)
            assert (rows == rows[:, :1]).all()           # no row mixes two rows
