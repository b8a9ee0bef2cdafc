"""Launch autotuner: search and cache logic (CPU; the timing itself is a GPU
measurement injected as a function)."""

import pytest

from mkpp_gb300 import autotune as at


def test_candidates_are_valid_and_distinct():
    cands = at.candidates()
    assert len(set(cands)) == len(cands)
    for c in cands:
        assert c.register_variant in (2, 4)
        assert c.blocks_per_sm >= 0 and c.defer_after >= 0
    # Both register budgets, and parking both off and on, are searched.
    assert {c.register_variant for c in cands} == {2, 4}
    assert 0 in {c.defer_after for c in cands} and max(c.defer_after for c in cands) > 0
    # Tail parking: searched, and only where its kernel exists (255 registers).
    assert {c.tail_after for c in cands} == {0, 300}
    assert all(c.register_variant == 2 for c in cands if c.tail_after)


def test_search_picks_the_fastest_and_records_failures():
    cands = at.candidates()
    times = {c: 10.0 + i for i, c in enumerate(cands)}
    fastest = cands[5]
    times[fastest] = 1.0
    failing = cands[3]

    def measure(c):
        if c == failing:
            raise RuntimeError("launch failed")
        return times[c]

    best, table = at.search(measure, cands)
    assert best == fastest
    assert len(table) == len(cands)
    bad = [r for r in table if "error" in r]
    assert len(bad) == 1 and bad[0]["register_variant"] == failing.register_variant
    assert bad[0]["seconds"] == float("inf")


def test_search_takes_the_best_of_repeats():
    cands = at.candidates()[:2]
    calls = {c: iter([5.0, 1.0]) if i == 0 else iter([2.0, 2.0]) for i, c in enumerate(cands)}
    best, table = at.search(lambda c: next(calls[c]), cands, repeats=2)
    assert best == cands[0] and table[0]["seconds"] == 1.0


def test_search_with_no_runnable_candidate_raises():
    def measure(c):
        raise RuntimeError("no GPU")

    with pytest.raises(RuntimeError):
        at.search(measure, at.candidates()[:3])


def test_cache_round_trip(tmp_path):
    path = tmp_path / "tuning.json"
    a, b = at.Candidate(4, 0, 3000), at.Candidate(2, 1, 0)
    gpu = at.gpu_key("NVIDIA GB300", 152)
    at.store("saprc99", gpu, a, [{"seconds": 1.0}], {"cells": 65536}, path)
    at.store("chapman", gpu, b, [], {}, path)
    at.store("saprc99", at.gpu_key("other", 8), b, [], {}, path)
    assert at.lookup("saprc99", gpu, path) == a
    assert at.lookup("chapman", gpu, path) == b
    assert at.lookup("saprc99", at.gpu_key("other", 8), path) == b
    assert at.lookup("small_strato", gpu, path) is None


def test_cache_path_follows_the_environment(tmp_path, monkeypatch):
    monkeypatch.setenv("MKPP_TUNING_CACHE", str(tmp_path / "x.json"))
    assert at.cache_path() == tmp_path / "x.json"
    monkeypatch.delenv("MKPP_TUNING_CACHE")
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    assert at.cache_path() == tmp_path / "mkpp_gb300" / "tuning.json"


def test_cache_entries_without_tail_parking_still_load(tmp_path):
    """A cache written before tail parking was searched has no tail_after:
    it reads back with tail parking off."""
    import json

    path = tmp_path / "tuning.json"
    gpu = at.gpu_key("NVIDIA GB300", 152)
    path.write_text(json.dumps({"saprc99": {gpu: {"choice": {"register_variant": 2, "blocks_per_sm": 0,
                                                            "defer_after": 3000}, "table": []}}}))
    assert at.lookup("saprc99", gpu, path) == at.Candidate(2, 0, 3000, 0)
