"""Autotuner for camera-track renders (st_render_frames): picks the schedule
(2-D pixel tiles, or the persistent queue with a chunk of 16..128 steps per
refill check) by timing each candidate on a sample of the track, and caches
the choice per workload signature in a JSON file
($SPACETIME_GB300_AUTOTUNE, default ~/.cache/spacetime_gb300/autotune.json)."""
from __future__ import annotations

import json
import os

from . import _abi

CANDIDATES = [("pixel", 0), ("persistent", 16), ("persistent", 32), ("persistent", 64), ("persistent", 128)]


def cache_path() -> str:
    return os.environ.get("SPACETIME_GB300_AUTOTUNE",
                          os.path.join(os.path.expanduser("~"), ".cache", "spacetime_gb300", "autotune.json"))


def signature(p, bh, ctx) -> str:
    return (f"w{p.width}h{p.height}prec{p.precision}sem{p.semantics}kerr{int(getattr(bh, 'a', 0.0) != 0.0)}"
            f"vol{int(ctx.volume is not None)}disc{int(ctx.disc is not None)}")


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(ctx, cams, bh, p, sample_frames: int = 8, repeats: int = 2, force: bool = False) -> dict:
    """Best (schedule, chunk) for this workload; timings per candidate are
    kept in the cache entry."""
    key = signature(p, bh, ctx)
    cache = _load()
    if key in cache and not force:
        return cache[key]
    step = max(1, len(cams) // sample_frames)
    sample = list(cams[::step])[:sample_frames]
    times = {}
    for sched, chunk in CANDIDATES:
        p.schedule = _abi.ST_SCHED_PIXEL if sched == "pixel" else _abi.ST_SCHED_PERSISTENT
        p.chunk_steps = chunk if chunk else 32
        p.graph = 0
        best = None
        for _ in range(repeats + 1):
            r = ctx.render_frames_raw(sample, bh, p)
            best = r.stats["kernel_ms"] if best is None else min(best, r.stats["kernel_ms"])
        times[f"{sched}:{chunk}"] = best
    choice = min(times, key=times.get)
    sched, chunk = choice.split(":")
    entry = {"schedule": sched, "chunk_steps": int(chunk) or 32, "ms": times, "sample_frames": len(sample)}
    cache[key] = entry
    _store(cache)
    return entry


def apply(p, entry: dict):
    p.schedule = _abi.ST_SCHED_PIXEL if entry["schedule"] == "pixel" else _abi.ST_SCHED_PERSISTENT
    p.chunk_steps = int(entry["chunk_steps"])
    return p
