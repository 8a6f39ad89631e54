"""Launch-shape autotuner for the batched executor.

Times a small set of (threads per CTA, CTAs per SM) choices for the
persistent multi-field launches on the actual batch and keeps the fastest.
Results persist in a JSON cache keyed by the GPU name and the batch's shapes
and level counts ($PRODM_AUTOTUNE_CACHE, default ~/.cache/prodm_gb300/autotune.json).
"""
import hashlib
import json
import os

import torch

CANDIDATES = ((128, 8), (256, 4), (256, 8), (256, 16))


def _cache_path():
    return os.environ.get("PRODM_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "prodm_gb300", "autotune.json"))


def signature(batch):
    key = json.dumps({"gpu": torch.cuda.get_device_name(), "shapes": [list(f.shape) for f in batch.fields],
                      "levels": batch.levels, "B": batch.B}, sort_keys=True)
    return hashlib.sha1(key.encode()).hexdigest()


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(cache):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
    except OSError:
        pass


def tune(batch, reps=3, use_cache=True):
    """Pick and apply the fastest launch shape; returns (threads, ctas_per_sm, timings)."""
    sig = signature(batch)
    cache = _load() if use_cache else {}
    if sig in cache:
        t, c = cache[sig]["threads"], cache[sig]["ctas_per_sm"]
        batch.set_launch(t, c)
        return t, c, cache[sig].get("ms", {})
    timings = {}
    for t, c in CANDIDATES:
        batch.set_launch(t, c)
        batch.refactor()
        batch.reset()
        batch.retrieve()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            batch.refactor()
            batch.reset()
            batch.retrieve()
        e1.record()
        torch.cuda.synchronize()
        timings["%dx%d" % (t, c)] = e0.elapsed_time(e1) / reps
    best = min(timings, key=timings.get)
    t, c = (int(x) for x in best.split("x"))
    batch.set_launch(t, c)
    cache[sig] = {"threads": t, "ctas_per_sm": c, "ms": timings}
    if use_cache:
        _store(cache)
    return t, c, timings
