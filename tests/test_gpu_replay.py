"""The synthetic run end to end (replay.py): front end -> C ABI -> file set ->
phase fit of every baseline file, as the reference's phase test does it."""

from __future__ import annotations

import importlib

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("xmode", [0, 2])
def test_replay_run_recovers_every_delay(pkg, cuda, tmp_path, xmode):
    replay = importlib.import_module(pkg.__name__ + ".replay")
    out = replay.run(str(tmp_path), n_station=6, n_freq=2048, frames_per_slot=32,
                     slots_per_row=2, rows=3, xmode=xmode, delay_stride=4, drop_rate=0.002)
    assert out["rows"] == 3 and out["baselines"] == 21
    assert out["worst_delay_error_samples"] < 0.05, out
    assert out["worst_phase_residual_rad"] < 0.5, out
