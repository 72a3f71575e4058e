"""The toy study's schedule table (host logic, no GPU): size-histogram keys,
the optional schedule file under MOREFIT_GB300_CACHE, and the candidates the
tuner measures."""
import json

import numpy as np


def test_size_histogram_key():
    from morefit_gb300.toystudy import size_histogram_key
    a = size_histogram_key(np.full(512, 2000))
    b = size_histogram_key(np.random.default_rng(1).poisson(2000, 512))
    assert a == b == (11, 11, 9)  # log2 of the median and largest size, and of the toy count
    assert size_histogram_key(np.full(4096, 2000)) != a
    assert size_histogram_key([1]) == (0, 0, 0)


def test_schedule_file_round_trip(tmp_path, monkeypatch):
    from morefit_gb300 import toystudy as T
    monkeypatch.delenv("MOREFIT_GB300_CACHE", raising=False)
    assert T._load_schedules() == {}
    T._store_schedule("k", T.SegmentSchedule(128, 0))  # no file without the variable
    monkeypatch.setenv("MOREFIT_GB300_CACHE", str(tmp_path / "c"))
    assert T._load_schedules() == {}
    T._store_schedule("pwave|float64|dev:152|11,11,9", T.SegmentSchedule(128, 0))
    T._store_schedule("pwave|float64|dev:152|11,11,12", T.SegmentSchedule(64, 512))
    got = T._load_schedules()
    assert got["pwave|float64|dev:152|11,11,9"] == T.SegmentSchedule(128, 0)
    assert got["pwave|float64|dev:152|11,11,12"] == T.SegmentSchedule(64, 512)
    assert json.loads((tmp_path / "c" / "toy_schedules.json").read_text())["pwave|float64|dev:152|11,11,12"] == [64, 512]
    (tmp_path / "c" / "toy_schedules.json").write_text("{not json")
    assert T._load_schedules() == {}  # a damaged file is ignored


def test_candidates_and_names():
    from morefit_gb300 import toystudy as T
    ts = T.ToyStudy.__new__(T.ToyStudy)  # candidates() needs no backend
    c = ts.candidates(np.full(100, 2000))
    assert T.SegmentSchedule(256, 0) in c and T.SegmentSchedule(64, 128) in c
    assert all(s.events_per_block < 2000 for s in c)  # runs as long as the largest segment are left out
    assert T.SegmentSchedule(256, 4096) not in c
    assert str(T.SegmentSchedule(128, 0)) == "b128_seg" and str(T.SegmentSchedule(64, 512)) == "b64_e512"
    assert T.DEFAULT_SCHEDULE == T.SegmentSchedule(256, 0)
