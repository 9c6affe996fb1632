"""Per-batch-shape launch tuning for ``rt_ri_ov_k_batched`` (split form).

A batch of molecules of uneven sizes leaves the grouped persistent GEMM with two
free choices (``rt_tuning``):

* ``fuse``: form the ri3ao digits inside the GEMM's producer instead of a
  separate slicing pass;
* ``chunks_per_item``: exact contraction chunks per work item (split-K
  granularity; 0 lets the library fill whole waves).

Neither changes more than the last bits of the result (the split-K partials are
summed exactly; only the int64 rescale of one item's sum moves), so the fastest
candidate is taken.  The measured winner of each batch shape is persisted as
JSON, keyed by form, slice count and the sorted list of molecule shapes, in
``$RT_TUNE_TABLE`` or ``~/.cache/rest_tensors_gb300/tune.json``.  A lookup made
while the stream is being captured into a CUDA graph never times anything: a
miss there returns the defaults.
"""
from __future__ import annotations

import json
import os
import tempfile
import threading
from typing import Callable, Dict, Iterable, List, Optional, Sequence, Tuple

CANDIDATES: Tuple[Tuple[int, int], ...] = tuple((f, c) for f in (0, 1) for c in (0, 1, 4, 16))

_lock = threading.Lock()
_table: Optional[Dict[str, List[int]]] = None
_table_path: Optional[str] = None


def table_path() -> str:
    p = os.environ.get("RT_TUNE_TABLE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "rest_tensors_gb300", "tune.json")


def shape_key(problems: Iterable[dict], form: str, nslices: int) -> str:
    """Order-independent key of a batch: form, S and the multiset of shapes.

    Whether ov and K are wanted is part of a shape (they change the products)."""
    shapes = sorted((int(q["nb"]), int(q["naux"]), int(q["nocc"]), int(q["nvir"]),
                     int(q.get("ov") is not None), int(q.get("K") is not None)) for q in problems)
    return "%s/S%d/%s" % (form, nslices, ";".join(",".join(str(v) for v in s) for s in shapes))


def _load() -> Dict[str, List[int]]:
    global _table, _table_path
    path = table_path()
    if _table is None or _table_path != path:
        _table_path = path
        try:
            with open(path) as f:
                data = json.load(f)
            _table = {k: [int(v[0]), int(v[1])] for k, v in data.get("entries", {}).items()}
        except (OSError, ValueError, KeyError, TypeError, IndexError):
            _table = {}
    return _table


def _save(table: Dict[str, List[int]]) -> None:
    path = table_path()
    d = os.path.dirname(path) or "."
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=".tune-", dir=d)
    with os.fdopen(fd, "w") as f:
        json.dump({"version": 1, "candidates": [list(c) for c in CANDIDATES], "entries": table}, f, indent=1,
                  sort_keys=True)
    os.replace(tmp, path)


def reset_cache() -> None:
    """Forget the in-memory copy of the table (the file is re-read on next use)."""
    global _table, _table_path
    with _lock:
        _table = None
        _table_path = None


def tune(problems: Sequence[dict], form: str, nslices: int, timer: Optional[Callable] = None,
         candidates: Sequence[Tuple[int, int]] = CANDIDATES, reps: int = 3, stream=None) -> Tuple[int, int]:
    """Time every candidate on this batch, record and return the fastest.

    ``timer(tuning) -> milliseconds`` may be supplied; by default each candidate
    runs once untimed and then ``reps`` times between CUDA events on ``stream``
    (the outputs of the batch are overwritten)."""
    if timer is None:
        timer = _cuda_timer(problems, form, nslices, reps, stream)
    best, best_ms = None, float("inf")
    for c in candidates:
        ms = float(timer(c))
        if ms < best_ms:
            best, best_ms = c, ms
    key = shape_key(problems, form, nslices)
    with _lock:
        t = _load()
        t[key] = [int(best[0]), int(best[1])]
        _save(t)
    return best


def lookup(problems: Sequence[dict], form: str, nslices: int, stream=None,
           timer: Optional[Callable] = None, tune_on_miss: bool = True):
    """The tuned ``rt_tuning`` of this batch shape, tuning it on a miss.

    Returns None (library defaults) for the float64 form, and on a miss while
    the stream is being captured."""
    from . import Tuning

    if form != "split":
        return None
    key = shape_key(problems, form, nslices)
    with _lock:
        hit = _load().get(key)
    if hit is not None:
        return Tuning(hit[0], hit[1])
    if not tune_on_miss or (timer is None and _capturing()):
        return None
    f, c = tune(problems, form, nslices, timer=timer, stream=stream)
    return Tuning(f, c)


def _capturing() -> bool:
    try:
        import torch

        return bool(torch.cuda.is_available() and torch.cuda.is_current_stream_capturing())
    except Exception:
        return False


def _cuda_timer(problems, form, nslices, reps, stream):
    import torch

    from . import ri_ov_k_batched

    s = stream if stream is not None else torch.cuda.current_stream()

    def run(c):
        ri_ov_k_batched(problems, form=form, nslices=nslices, tuning=c, stream=s)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            ri_ov_k_batched(problems, form=form, nslices=nslices, tuning=c, stream=s)
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    return run
