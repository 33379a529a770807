"""Host logic of the trajectory engine's launch-width autotuner
(tngpu.autotune): buckets, the JSON cache and the selection rule, with a
stand-in probe in place of timed launches."""

import json

import pytest

from tngpu import autotune as AT


def test_bucket_rounds_up_to_powers_of_two():
    assert AT.bucket(64, 2, 1024, 32) == "chi64-d2-traj1024-N32"
    assert AT.bucket(48, 2, 1000, 30) == "chi64-d2-traj1024-N32"
    assert AT.bucket(65, 3, 1, 7) == "chi128-d3-traj1-N8"
    assert AT.bucket(0, 2, 0, 1) == "chi1-d2-traj1-N1"


def test_tune_picks_fastest_and_caches(tmp_path):
    path = tmp_path / "w.json"
    cache = AT.WidthCache(str(path))
    times = {1: 3.0, 2: 1.5, 4: 1.0, 8: 1.2}
    calls = []

    def probe(w):
        calls.append(w)
        return times[w]

    w, t = AT.tune("k", probe, cache=cache)
    assert w == 4 and calls == [1, 2, 4, 8] and t == times
    # a second tuner reading the same file hits the cache without probing
    w2, t2 = AT.tune("k", probe, cache=AT.WidthCache(str(path)))
    assert w2 == 4 and t2 == {} and calls == [1, 2, 4, 8]
    data = json.loads(path.read_text())
    assert data["k"]["width"] == 4
    assert data["k"]["seconds_per_traj_step"] == {"1": 3.0, "2": 1.5, "4": 1.0, "8": 1.2}


def test_tune_ties_go_to_the_narrower_width():
    w, _ = AT.tune("k", lambda w: 1.0, widths=(8, 2, 4))
    assert w == 2


def test_tune_rejects_bad_widths_and_failed_probes(tmp_path):
    with pytest.raises(ValueError):
        AT.tune("k", lambda w: 1.0, widths=(3,))
    with pytest.raises(ValueError):
        AT.tune("k", lambda w: 1.0, widths=())
    with pytest.raises(RuntimeError):
        AT.tune("k", lambda w: 0.0, widths=(1, 2))
    # nothing was stored for the failed key
    cache = AT.WidthCache(str(tmp_path / "c.json"))
    with pytest.raises(RuntimeError):
        AT.tune("k", lambda w: float("nan"), cache=cache)
    assert cache.get("k") is None


def test_cache_ignores_corrupt_files_and_foreign_widths(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text("{not json")
    assert AT.WidthCache(str(p)).entries == {}
    p.write_text(json.dumps({"a": {"width": 3}, "b": {"width": 8}, "c": 5}))
    c = AT.WidthCache(str(p))
    assert c.get("a") is None and c.get("b") == 8 and c.get("c") is None


def test_default_cache_path_honours_environment(monkeypatch, tmp_path):
    monkeypatch.setenv("TNGPU_TUNE_CACHE", str(tmp_path / "x.json"))
    assert AT.default_cache_path() == str(tmp_path / "x.json")
    monkeypatch.delenv("TNGPU_TUNE_CACHE")
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    assert AT.default_cache_path() == str(tmp_path / "tngpu" / "engine_widths.json")


def test_unwritable_cache_keeps_the_tuned_width(tmp_path):
    blocker = tmp_path / "file"
    blocker.write_text("")
    cache = AT.WidthCache(str(blocker / "sub" / "w.json"))  # a directory under a file
    with pytest.warns(UserWarning, match="not written"):
        w, t = AT.tune("k", lambda w: {1: 2.0, 2: 1.0, 4: 3.0, 8: 4.0}[w], cache=cache)
    assert w == 2 and len(t) == 4
