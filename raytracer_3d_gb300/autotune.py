"""Autotuner of the step schedule.

The schedule of the step kernel -- kernel variant (TMA-staged planes, plain
planes), CTA size, band length and which of the two slow axes is banded
(the sweep order) -- never changes results, only speed.  The tuner times
each candidate with CUDA events on the handle's own stream using dry steps
(rt_step_dry / rt_batch_dry: the kernel runs from the current state without
advancing it), keeps the fastest, and caches the choice per shape signature
in a JSON file (RT_TUNE_CACHE, default ~/.cache/raytracer_gb300/tune.json).
"""
import json
import os
import time

DEFAULT_CANDIDATES = [
    (variant, band, threads, sweep)
    for variant in ("w2z", "w2q", "w3", "w6", "tma", "group", "plane")
    for threads in (128, 256, 512, 1024)
    for band in (4, 8, 16)
    for sweep in (0, 1)
    if not (variant == "plane" and threads == 1024)
    and not (variant in ("w2z", "w2q", "w3", "w6") and threads == 1024)
    and not (variant == "w6" and threads == 128)
    and not (variant not in ("w2z", "w2q", "w3") and threads == 128)
]


def _cache_path():
    return os.environ.get("RT_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache",
                                                        "raytracer_gb300", "tune.json"))


def _load_cache():
    p = _cache_path()
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(cache):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def _event_timer(stream_ptr):
    import torch
    stream = torch.cuda.ExternalStream(stream_ptr)

    def timed(fn, reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn(reps)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    return timed


def signature(kind, shapes, precision):
    return "%s|%s|%s" % (kind, precision, ";".join("x".join(map(str, s)) for s in shapes))


def tune_model(model, candidates=None, reps=3, use_cache=True):
    """Pick the fastest schedule for one Model; returns (best, table)."""
    key = signature("model", [model.n], model.precision)
    cache = _load_cache() if use_cache else {}
    if use_cache and key in cache:
        best = tuple(cache[key]["best"])
        model.set_tuning(*best)
        return best, cache[key].get("table", [])
    lib = model._lib
    timed = _event_timer(model.stream())
    table = []
    if candidates is None:
        candidates = list(DEFAULT_CANDIDATES)
        if model.precision == "fp64":       # the two-pass binary64 step (every face flux once)
            candidates.append(("split", 8, 256, 0))
    for cand in candidates:
        model.set_tuning(*cand)
        run = lambda k: model._check(lib.rt_step_dry(model.handle, k), "rt_step_dry")  # noqa: E731
        run(1)  # warm-up (shared-memory attribute, caches)
        table.append((cand, timed(run, reps)))
    table.sort(key=lambda x: x[1])
    best = table[0][0]
    model.set_tuning(*best)
    if use_cache:
        cache[key] = {"best": list(best), "table": [[list(c), t] for c, t in table], "when": time.time()}
        _store_cache(cache)
    return best, table


BATCH_CANDIDATES = [
    (band, 512, sweep, persistent, slices, fused)
    for persistent in (256, 512, 0)
    for slices in (256, 512, 0)
    for fused in ((1, 0) if persistent == slices and persistent > 0 else (1,))
    for band in (4, 8)
    for sweep in (0, 1)
]


def tune_batch(batch, candidates=None, reps=2, graph_steps=16, use_cache=True):
    """Pick band / CTA size / sweep order of the plane and group kernels and
    the consumer threads of the two staged classes (0: off) and whether
    they share one launch for a Batch; returns (best, table) with best =
    (band, threads, sweep, persistent, slices, fused)."""
    key = signature("batch4", sorted(m.n for m in batch.models), batch.models[0].precision)
    cache = _load_cache() if use_cache else {}

    def apply(c):
        batch.set_tuning(c[0], c[1], c[2], graph_steps)
        batch.set_persistent(c[3])
        batch.set_slices(c[4])
        batch.set_fused(c[5] if len(c) > 5 else 0)

    if use_cache and key in cache:
        apply(cache[key]["best"])
        return tuple(cache[key]["best"]), cache[key].get("table", [])
    lib = batch._lib
    timed = _event_timer(batch.stream())
    table = []
    for cand in candidates or BATCH_CANDIDATES:
        apply(cand)
        run = lambda k: batch._check(lib.rt_batch_dry(batch._b, k), "rt_batch_dry")  # noqa: E731
        run(1)
        table.append((tuple(cand), timed(run, reps)))
    table.sort(key=lambda x: x[1])
    best = table[0][0]
    apply(best)
    if use_cache:
        cache[key] = {"best": list(best), "table": [[list(c), t] for c, t in table], "when": time.time()}
        _store_cache(cache)
    return best, table
