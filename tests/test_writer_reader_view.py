"""The writer's files, as the reference's own readers see them (host only, no GPU).

tests/golden/reader_view.json was made by tests/golden/make_reader_view.py. That
script wrote a set with this library's writer and read it with the reference's
tools/corr_common.py, compare_blocks.py and autospectra.py. Those readers
reported every spectrum row, row time, validity count, station name and metadata
number as written. Here the same set is written again: its files must hash to
what those readers accepted, and the recorded view must match the rows that
went in. With CORR_REFERENCE_DIR set, the readers are also run live.
"""

from __future__ import annotations

import importlib.util
import json
import os
import time
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _script():
    spec = importlib.util.spec_from_file_location("make_reader_view",
                                                  GOLDEN / "make_reader_view.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture
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


@pytest.fixture(scope="module")
def fixture():
    return json.loads((GOLDEN / "reader_view.json").read_text())


def test_writer_still_writes_the_files_the_readers_accepted(pkg, utc, tmp_path, fixture):
    mk = _script()
    mk.write_set(str(tmp_path))
    assert mk.file_hashes(str(tmp_path)) == fixture["files"]


def test_recorded_reader_view_matches_the_rows(fixture):
    mk = _script()
    rs = mk.rows()
    view = fixture["reader"]
    assert view["rows_ms"] == [r["ms"] for r in rs]
    assert [tuple(b[1:3]) for b in view["baseline_files"]] == mk.pairs()
    assert set(b[3] for b in view["baseline_files"]) <= set(fixture["files"])
    assert view["station_names"] == {str(i): n for i, n in enumerate(mk.STATIONS)}
    assert int(view["metadata"]["n_freq"]) == mk.NF
    assert int(view["metadata"]["n_cum"]) == mk.NCUM
    blocks = {(b[0], b[1]): tuple(b[2:]) for b in view["blocks"]}
    for r in rs:
        for st, v in enumerate(r["valid"]):
            assert blocks[(r["first_frame_id"], st)] == (r["row_index"], mk.NCUM, v, mk.NCUM - v)
    pairs = mk.pairs()
    for name, mean in view["autospectra_mean"].items():
        j = mk.STATIONS.index(name)
        b = pairs.index((j, j))
        want = np.mean([r["spectrum"][b].real.astype(np.float64) for r in rs], axis=0)
        assert np.allclose(mean, want, rtol=1e-6, atol=1e-6)


@pytest.mark.skipif(not os.environ.get("CORR_REFERENCE_DIR"),
                    reason="CORR_REFERENCE_DIR (a reference checkout) not set")
def test_reference_readers_live(pkg, utc, tmp_path, fixture):
    mk = _script()
    rs = mk.write_set(str(tmp_path))
    tools = str(Path(os.environ["CORR_REFERENCE_DIR"]) / "tools")
    view = mk.reader_view(str(tmp_path), tools, rs)
    assert json.loads(json.dumps(view)) == fixture["reader"]
