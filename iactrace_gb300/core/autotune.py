"""Autotuner of the batched render's launch knobs.

Knobs: threads per CTA (block_threads), 32-ray tasks per warp per work tile
(tasks_per_warp: rays each thread traces per tile) and histogram placement
(hist_mode: FP32 shared-memory rows or direct FP64 global atomics). Every
candidate is planned, run once as a warm-up and then REPS more times, each
timed with CUDA events on the batch itself; its time is the median of those
runs (sub-millisecond launches vary by a few percent from run to run). The
fastest is cached in memory and in a JSON file keyed by GPU, library ABI,
the repetition count and the batch's shape signature (per job: facets,
samples, sources, pixels, sensor kind, stage mirrors).

Cache file: $IACTRACE_TUNE_CACHE, else ~/.cache/iactrace_gb300/tune.json.
IACTRACE_TUNE=0 skips tuning (library defaults).
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import threading

import torch

from .. import _native as N

CANDIDATES = [(b, t, h) for b in (256, 128) for t in (16, 32, 64) for h in (1, 2)]
REPS = 5  # timed runs per candidate (median)
_mem: dict = {}
_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("IACTRACE_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache",
                                                                 "iactrace_gb300", "tune.json")


def make_opts(block, tasks, hist) -> N.IactOpts:
    o = N.IactOpts()
    o.block_threads, o.tasks_per_warp, o.hist_mode = int(block), int(tasks), int(hist)
    return o


def _key(batch) -> str:
    props = torch.cuda.get_device_properties(batch.device)
    sig = hashlib.sha1(repr(batch.signature).encode()).hexdigest()[:16]
    return f"{props.name}|sm{props.multi_processor_count}|abi{N.load().iact_abi_version()}|r{REPS}|batch|{sig}"


def _load_file() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, value):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        data = _load_file()
        data[key] = value
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # an unwritable cache only costs re-tuning


def time_candidate(batch, opts, reps: int = REPS) -> float:
    """Median device time (ms) of the batch's launch sequence under `opts`."""
    h, ws = batch._create(opts)
    stream = torch.cuda.current_stream(batch.device)
    try:
        N.check(batch.lib.iact_batch_render(h, stream.cuda_stream))  # warm-up
        times = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            N.check(batch.lib.iact_batch_render(h, stream.cuda_stream))
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        return sorted(times)[len(times) // 2]
    finally:
        torch.cuda.synchronize(batch.device)
        batch.lib.iact_batch_destroy(h)
        del ws


def tune_batch(batch, candidates=CANDIDATES, force: bool = False):
    """Best IactOpts for this batch (cached); None when tuning is off."""
    if os.environ.get("IACTRACE_TUNE", "1") == "0":
        return None
    key = _key(batch)
    with _lock:
        if not force:
            hit = _mem.get(key) or _load_file().get(key)
            if hit is not None:
                _mem[key] = hit
                return make_opts(*hit["knobs"])
        results = []
        for cand in candidates:
            try:
                ms = time_candidate(batch, make_opts(*cand))
            except N.IactError:
                continue  # e.g. histogram rows that do not fit in shared memory
            results.append((ms, cand))
        if not results:
            return None
        results.sort()
        best = {"knobs": list(results[0][1]), "ms": results[0][0],
                "tried": [[list(c), ms] for ms, c in results]}
        _mem[key] = best
        _store(key, best)
        return make_opts(*best["knobs"])


def last_result(batch):
    """The cached tuning record of this batch (knobs, time, candidates), if any."""
    key = _key(batch)
    return _mem.get(key) or _load_file().get(key)


__all__ = ["tune_batch", "time_candidate", "make_opts", "cache_path", "last_result", "CANDIDATES"]
del ctypes
