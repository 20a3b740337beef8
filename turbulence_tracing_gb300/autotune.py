"""Autotuner for the FP32 tracer: picks the thread-block size of the persistent
launch and the brick depth (nodes per brick along the probing axis) of the
node volume by timing them on the GPU.

For a grid shape it builds the volume at each candidate brick depth, traces a
sample of the caller's rays with each candidate block size (CUDA events,
best of `reps` after one warm-up) and keeps the fastest pair.  Results are
cached per (grid shape, probing axis, SM count, device name) in memory and,
when a cache file is given, on disk as JSON, so a shape is timed once.
"""
import json
import os
import threading

import numpy as np
import torch

from . import core

BLOCKS = (64, 128, 256)
BRICK_DEPTHS = (4, 8, 16, 32)

_lock = threading.Lock()
_mem = {}


def _key(shape, probing_axis):
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    return "%dx%dx%d/ax%d/%dsm/%s" % (shape[0], shape[1], shape[2], probing_axis, props.multi_processor_count,
                                      props.name)


def _load(path):
    if path and os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def _time(fn, reps):
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def tune(ne, x, y, z, s0_sample, t_end, extent, probing_axis=2, lwl=1053e-9, ne_max=1.0, phase=True,
         blocks=BLOCKS, brick_depths=BRICK_DEPTHS, reps=2, cache_file=None, force=False):
    """Return {'block': b, 'brick_depth': d, 'ms': {...}} for this grid shape."""
    ne_t = ne if isinstance(ne, torch.Tensor) else torch.as_tensor(np.asarray(ne), device="cuda")
    key = _key(tuple(ne_t.shape), probing_axis)
    with _lock:
        if not force:
            if key in _mem:
                return _mem[key]
            disk = _load(cache_file)
            if key in disk:
                _mem[key] = disk[key]
                return disk[key]
    timings = {}
    best = None
    s0_t = s0_sample if isinstance(s0_sample, torch.Tensor) else torch.as_tensor(np.asarray(s0_sample), device="cuda")
    for bd in brick_depths:
        vol = core.build_volume(ne_t, x, y, z, probing_axis, lwl=lwl, ne_max=ne_max, brick_depth=bd)
        out = core.trace_f32(vol, s0_t, t_end, extent, phase=phase)
        for b in blocks:
            ms = _time(lambda: core.trace_f32(vol, s0_t, t_end, extent, phase=phase, out=out, ws=out["_ws"],
                                              block_size=b), reps)
            timings["%d/%d" % (b, bd)] = ms
            if best is None or ms < best[0]:
                best = (ms, b, bd)
        del vol, out
    res = {"block": best[1], "brick_depth": best[2], "ms": timings, "sample_rays": int(s0_t.shape[-1])}
    with _lock:
        _mem[key] = res
        if cache_file:
            disk = _load(cache_file)
            disk[key] = res
            tmp = cache_file + ".tmp%d" % os.getpid()
            with open(tmp, "w") as f:
                json.dump(disk, f, indent=1, sort_keys=True)
            os.replace(tmp, cache_file)
    return res


def cached(shape, probing_axis=2):
    """The tuned pair for a shape if it has been timed in this process, else None."""
    return _mem.get(_key(shape, probing_axis))
