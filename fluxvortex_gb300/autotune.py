"""Launch-shape autotuner: times candidate configurations on the device in use
and remembers the fastest per (device, kernel, problem) key.

``best(key, candidates, run)`` calls ``run(candidate)`` (which must launch the
work on the current stream and leave the device state reusable) once to warm
up and ``reps`` times under CUDA events, per candidate, and returns the
fastest.  Results are cached in memory and in a JSON file next to the built
library (``_lib/autotune.json``, not part of the sources), so later processes
on the same kind of device skip the timing.
"""
from __future__ import annotations

import json
import os
import threading

_lock = threading.Lock()
_cache: dict | None = None


def _path():
    from . import build
    return os.path.join(os.path.dirname(build.LIB), "autotune.json")


def _load():
    global _cache
    if _cache is None:
        try:
            with open(_path()) as f:
                _cache = json.load(f)
        except (OSError, ValueError):
            _cache = {}
    return _cache


def _save():
    try:
        os.makedirs(os.path.dirname(_path()), exist_ok=True)
        tmp = _path() + f".{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(_cache, f, indent=1, sort_keys=True)
        os.replace(tmp, _path())
    except OSError:
        pass


def device_key():
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{p.name}/sm{p.major}{p.minor}/{p.multi_processor_count}"


def best(key, candidates, run, reps=3, use_cache=True):
    """Fastest candidate for ``key`` (a string) on this device; times are kept
    under ``timings`` of the returned record's cache entry."""
    import torch
    full = f"{device_key()}|{key}"
    with _lock:
        c = _load()
        if use_cache and full in c and c[full]["best"] in candidates:
            return c[full]["best"]
    times = {}
    for cand in candidates:
        run(cand)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(reps):
            run(cand)
        e.record()
        torch.cuda.synchronize()
        times[str(cand)] = s.elapsed_time(e) / reps
    pick = min(candidates, key=lambda x: times[str(x)])
    with _lock:
        c = _load()
        c[full] = {"best": pick, "timings_ms": times}
        _save()
    return pick


def lookup(key):
    """Cached record for ``key`` on this device, or None."""
    with _lock:
        return _load().get(f"{device_key()}|{key}")
