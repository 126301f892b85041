"""Launch-shape autotuner with a per-shape JSON cache.

Some kernels of this package take a launch shape that changes only their
speed, never their results (the column-slab width and rows per warp of the
sparse products, the chains per block of the persistent proposal kernel).
`choose` times every candidate shape with CUDA events on the stream the
kernel runs on, keeps the fastest, and remembers it per
(device, kernel, problem shape): in memory for the process and in a JSON file
for later processes, so that a shape is timed once per machine.

Cache file: $HMCLAB_GB300_TUNE_CACHE if set (an empty value keeps the
choices in memory only), else ~/.cache/hmclab_gb300/launch_shapes.json.
Each entry records the choice, the per-candidate times and when it was
measured; a cached choice that is not among the current candidates is timed
again.
"""
import json as _json
import os as _os
import tempfile as _tempfile
import threading as _threading
import time as _time

from hmclab_gb300 import _lib

_lock = _threading.Lock()
_memory = {}


def cache_path():
    env = _os.environ.get("HMCLAB_GB300_TUNE_CACHE")
    if env is not None:
        return env or None
    return _os.path.join(_os.path.expanduser("~"), ".cache", "hmclab_gb300", "launch_shapes.json")


def device_tag(device):
    import torch

    p = torch.cuda.get_device_properties(device)
    return f"{p.name}|sm_{p.major}{p.minor}|{p.multi_processor_count}SM"


def _read(path):
    try:
        with open(path) as f:
            data = _json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def _write(path, key, entry):
    """Merge one entry into the cache file (atomic replace; a cache that
    cannot be written is skipped: the choice stays in memory)."""
    try:
        _os.makedirs(_os.path.dirname(path) or ".", exist_ok=True)
        data = _read(path)
        data[key] = entry
        fd, tmp = _tempfile.mkstemp(dir=_os.path.dirname(path) or ".", prefix=".tune-")
        with _os.fdopen(fd, "w") as f:
            _json.dump(data, f, indent=1, sort_keys=True)
        _os.replace(tmp, path)
    except OSError:
        pass


def _capturing(handle):
    flag = _lib.c_int(0)
    _lib.call("hmc_stream_capturing", handle, _lib._ct.byref(flag))
    return bool(flag.value)


def choose(kind, shape, candidates, run, device, stream_handle, reps=3):
    """The candidate (a tuple of ints) whose `run(candidate)` is fastest.

    `run` enqueues one evaluation with that launch shape on the stream
    `stream_handle`; every candidate must compute the same result.  `shape`
    is any JSON-able description of the problem size.  While the stream is
    being captured into a CUDA graph nothing can be timed: the first
    candidate is returned and nothing is cached."""
    import torch

    candidates = [tuple(int(v) for v in c) for c in candidates]
    key = f"{device_tag(device)}|{kind}|{_json.dumps(shape, sort_keys=True)}"
    with _lock:
        if key in _memory and _memory[key] in candidates:
            return _memory[key]
    path = cache_path()
    if path:
        entry = _read(path).get(key)
        if entry is not None and tuple(entry.get("choice", ())) in candidates:
            with _lock:
                _memory[key] = tuple(entry["choice"])
            return _memory[key]
    if _capturing(stream_handle):
        return candidates[0]
    st = torch.cuda.ExternalStream(stream_handle, device=device)
    times = {}
    for cand in candidates:
        run(cand)  # warm-up: first launch of a kernel variant, attribute set-up
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            run(cand)
        e1.record(st)
        e1.synchronize()
        times[cand] = e0.elapsed_time(e1) / reps
    best = min(candidates, key=lambda c: times[c])
    with _lock:
        _memory[key] = best
    if path:
        _write(path, key, {"choice": list(best), "ms": {",".join(map(str, c)): round(t, 5) for c, t in times.items()},
                           "measured": _time.strftime("%Y-%m-%dT%H:%M:%S")})
    return best


def forget():
    """Drop the in-process choices (the cache file is left alone)."""
    with _lock:
        _memory.clear()
