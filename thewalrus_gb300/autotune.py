"""Autotuner for batched sieve plans.

Chooses the term-chunk size (chunks per resident warp), the warps per CTA, whether uneven
instances share one persistent launch per scalar type and whether the launches run one after
another or overlap on side streams, by timing candidate plans on the GPU.
Results are cached per (GPU, precision, workload signature) in ``_build/autotune.json`` next to
the native library, so a workload shape is tuned once per machine.

Timing: each candidate plan executes once untimed (first execution, graph capture), then
``repeats`` executions are timed with CUDA events on the launching stream when torch is
available, else by host wall clock around execute + read.
"""
import hashlib
import json
import os
import time

from . import _native as nat

__all__ = ["tune", "signature", "DEFAULT_CANDIDATES", "cached_options"]

DEFAULT_CANDIDATES = [
    {"chunk_scale": cs, "max_warps_per_cta": w, "merge_classes": mc, "serial_groups": sg}
    for cs in (0.5, 1.0, 2.0, 4.0)
    for w in (0, 4)
    for mc in (False, True)
    for sg in (False, True)
]
CACHE = os.path.join(nat.BUILD, "autotune.json")


def signature(instances, precision):
    """Workload signature: histogram of (kind, n, dtype, edge multiplicities) plus precision."""
    hist = {}
    for inst in instances:
        s = inst.struct
        key = (s.kind, s.n, s.dtype, tuple(int(r) for r in inst.reps), s.batch_max, s.cutoff)
        hist[key] = hist.get(key, 0) + 1
    text = json.dumps(sorted((list(k), v) for k, v in hist.items())) + precision
    return hashlib.sha1(text.encode()).hexdigest()[:16]


def _device_name():
    try:
        import torch

        return torch.cuda.get_device_name()
    except Exception:  # torch missing or no device: the key still separates precisions
        return "cuda"


def _load_cache():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def cached_options(instances, precision="fp64"):
    """Previously tuned options for this workload on this GPU, or None."""
    key = "%s|%s" % (_device_name(), signature(instances, precision))
    return _load_cache().get(key, {}).get("best")


def _time_plan(plan, repeats):
    try:
        import torch

        stream = torch.cuda.current_stream()
        plan.execute(stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(repeats):
            plan.execute(stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / repeats
    except ImportError:
        plan.execute()
        plan.read()
        t0 = time.perf_counter()
        for _ in range(repeats):
            plan.execute()
        plan.read()
        return (time.perf_counter() - t0) / repeats


def tune(instances, precision="fp64", candidates=None, repeats=2, use_cache=True, use_graph=True):
    """Time every candidate option set on ``instances``; returns (best_options, table).

    ``table`` lists (options, seconds per execution).  The best options are cached.
    """
    instances = list(instances)
    key = "%s|%s" % (_device_name(), signature(instances, precision))
    cache = _load_cache() if use_cache else {}
    if use_cache and key in cache:
        return cache[key]["best"], cache[key]["table"]
    table = []
    for cand in candidates or DEFAULT_CANDIDATES:
        plan = nat.Plan(instances, precision=precision, use_graph=use_graph, **cand)
        try:
            table.append((dict(cand), _time_plan(plan, repeats)))
        finally:
            plan.close()
    best = min(table, key=lambda x: x[1])[0]
    if use_cache:
        cache = _load_cache()
        cache[key] = {"best": best, "table": table}
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        tmp = CACHE + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, CACHE)
    return best, table
