"""Launch-shape and tile-shape autotuner for the batched executor.

Times launch shapes for the persistent multi-field launches on the actual
batch and keeps the fastest, one stage at a time (coordinate descent): the
row stages (decomposition, recomposition: threads per CTA = warps = fine rows
in flight per CTA, and CTAs per SM, i.e. how many row groups share an SM) and
the encoder (CTAs per SM of its 256-thread chunk workers) and the fused
finest-level decode + recomposition (CTAs per SM of its 8-row units), each timed as the
whole refactor + retrieve step with the other stages at their best shape so
far; then the tile shape of the fused finest levels (values per unit of
consecutive fine rows: 8-row units of long rows, up to 64 rows of short
ones). Results persist in a JSON cache keyed by the GPU name and the batch's
shapes and level counts ($PRODM_AUTOTUNE_CACHE, default
~/.cache/prodm_gb300/autotune.json).
"""
import hashlib
import json
import os

import torch

# (threads per CTA, CTAs per SM) per stage
ROW_CANDIDATES = ((64, 16), (64, 32), (128, 8), (128, 16), (256, 4), (256, 8))
ENCODE_CANDIDATES = ((256, 1), (256, 2), (256, 4), (256, 8))
# the fused finest levels: 256-thread CTAs of 8-row (or longer) units, 2..5 per
# SM (fewer where a unit's tiles do not fit)
FUSED_CANDIDATES = ((256, 2), (256, 3), (256, 4), (256, 5))
STAGE_CANDIDATES = {"decompose": ROW_CANDIDATES, "recompose": ROW_CANDIDATES, "encode": ENCODE_CANDIDATES,
                    "fused": FUSED_CANDIDATES}
DEFAULT = {"decompose": (256, 8), "encode": (256, 8), "recompose": (256, 8), "fused": (256, 5)}
# values per unit of the fused finest levels
UNIT_CANDIDATES = (1056, 2112, 4224)
DEFAULT_UNIT = 2112
# the uniform shapes of the earlier single-shape tuner (still accepted by set_launch)
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


def _time(batch, reps):
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
    return e0.elapsed_time(e1) / reps


def _apply(batch, shapes):
    for stage, v in shapes.items():
        if stage == "fused_unit":
            batch.set_fused_unit(v[0])
        else:
            batch.set_stage_launch(stage, v[0], v[1])


def tune(batch, reps=3, use_cache=True):
    """Pick and apply the fastest launch shape of every stage and the fused
    levels' tile shape; returns (shapes {stage: (threads, ctas_per_sm)} plus
    {"fused_unit": (values,)}, timings {"stage:TxC": ms, "fused_unit:V": ms})."""
    sig = signature(batch)
    cache = _load() if use_cache else {}
    if sig in cache and "stages" in cache[sig]:
        shapes = {k: tuple(v) for k, v in cache[sig]["stages"].items()}
        _apply(batch, shapes)
        return shapes, cache[sig].get("ms", {})
    shapes = dict(DEFAULT)
    _apply(batch, shapes)
    timings = {}
    for stage in ("decompose", "recompose", "encode", "fused"):
        best = None
        for t, c in STAGE_CANDIDATES[stage]:
            batch.set_stage_launch(stage, t, c)
            ms = _time(batch, reps)
            timings["%s:%dx%d" % (stage, t, c)] = ms
            if best is None or ms < best[0]:
                best = (ms, (t, c))
        shapes[stage] = best[1]
        batch.set_stage_launch(stage, *best[1])
    best = None
    for v in UNIT_CANDIDATES:
        batch.set_fused_unit(v)
        ms = _time(batch, reps)
        timings["fused_unit:%d" % v] = ms
        if best is None or ms < best[0]:
            best = (ms, v)
    shapes["fused_unit"] = (best[1],)
    batch.set_fused_unit(best[1])
    cache[sig] = {"stages": {k: list(v) for k, v in shapes.items()}, "ms": timings}
    if use_cache:
        _store(cache)
    return shapes, timings
