"""Host logic of the batch-shape autotuner: keys, choice of the fastest
candidate, persistence of the JSON table and behaviour on a miss.  Timings come
from a fake timer, so no GPU is needed."""
import json

import pytest

from rest_tensors_gb300 import autotune


def batch(*shapes):
    return [dict(nb=nb, naux=naux, nocc=nocc, nvir=nb - nocc, ov=object(), K=object()) for nb, naux, nocc in shapes]


@pytest.fixture(autouse=True)
def table(tmp_path, monkeypatch):
    monkeypatch.setenv("RT_TUNE_TABLE", str(tmp_path / "t.json"))
    autotune.reset_cache()
    yield tmp_path / "t.json"
    autotune.reset_cache()


def test_key_ignores_order_and_separates_form_and_slices():
    a = batch((40, 60, 5), (72, 100, 9))
    b = batch((72, 100, 9), (40, 60, 5))
    assert autotune.shape_key(a, "split", 7) == autotune.shape_key(b, "split", 7)
    assert autotune.shape_key(a, "split", 7) != autotune.shape_key(a, "split", 8)
    assert autotune.shape_key(a, "split", 7) != autotune.shape_key(a, "fp64", 7)
    c = [dict(q, K=None) for q in a]
    assert autotune.shape_key(a, "split", 7) != autotune.shape_key(c, "split", 7)


def test_tune_picks_fastest_and_persists(table):
    cost = {c: 10.0 + i for i, c in enumerate(autotune.CANDIDATES)}
    cost[(1, 4)] = 1.0
    probs = batch((40, 60, 5), (24, 30, 3))
    assert autotune.tune(probs, "split", 7, timer=lambda c: cost[tuple(c)]) == (1, 4)
    data = json.load(open(table))
    assert data["entries"][autotune.shape_key(probs, "split", 7)] == [1, 4]
    autotune.reset_cache()
    seen = []
    t = autotune.lookup(probs, "split", 7, timer=lambda c: seen.append(c) or 0.0)
    assert (t.fuse, t.chunks_per_item) == (1, 4) and seen == []


def test_lookup_miss_tunes_and_float64_needs_no_tuning(table):
    probs = batch((130, 200, 12))
    assert autotune.lookup(probs, "fp64", 7) is None
    assert autotune.lookup(probs, "split", 7, tune_on_miss=False) is None
    calls = []
    t = autotune.lookup(probs, "split", 7, timer=lambda c: calls.append(c) or (0.5 if c == (0, 16) else 2.0))
    assert (t.fuse, t.chunks_per_item) == (0, 16)
    assert len(calls) == len(autotune.CANDIDATES)


def test_corrupt_table_is_ignored(table):
    table.write_text("{not json")
    probs = batch((9, 5, 2))
    assert autotune.lookup(probs, "split", 7, tune_on_miss=False) is None
    autotune.tune(probs, "split", 7, timer=lambda c: 1.0)
    assert json.load(open(table))["version"] == 1
