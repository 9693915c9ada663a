"""Pick the fused kernel's shape per (model, stencil, grid size) by timing.

The fused float32 form has several kernels -- the TMA pipeline (64 x 32
regions, one persistent CTA per SM, with 4 x 1 or 2 x 2 nodes per thread)
and the cp.async kernels (64 x 32 regions with two CTAs per SM, or 64 x 64
regions) -- and a temporal-block depth K (time steps per launch: 2, 3, 4
or 8).  Which is fastest depends on
the model's register and instruction load, the stencil and the grid.  The
first fused run of a configuration times every candidate for a few launches
on scratch copies of the model's arrays (no effect on the model, its
trackers or its stimuli) and caches the winner in a JSON file keyed by the
GPU name, the model, the stencil and the grid's size class (power of two
of the node count).

The cache lives in ``$FWGPU_AUTOTUNE_CACHE`` or
``~/.cache/finitewave_gb300/autotune.json``.
"""
import ctypes
import json
import math
import os
import threading

import torch

from . import _ffi

_lock = threading.Lock()
_memo = {}

# (fused_variant, fused_k) candidates; variants 3 and 4 only where the TMA
# kernels can run (packed weights, nj % 16 == 0).  Variants 5, 6 and 7 are
# not candidates: each was measured slower than variant 3 on the 4096^2
# Aliev-Panfilov workload (weights formed on chip, two-wide float32
# instructions, the row-marching wavefront) and is kept as an explicit
# choice only.
_TMA = [(3, 2), (3, 3), (3, 4), (3, 8), (4, 2), (4, 4), (4, 8)]
_CPASYNC = [(1, 2), (1, 4), (1, 8), (2, 2), (2, 4), (2, 8)]


def cache_path():
    return os.environ.get("FWGPU_AUTOTUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "finitewave_gb300",
        "autotune.json")


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(table):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass   # an unwritable cache only costs a re-tune


def key(model):
    shape = model._shape()
    n = 1
    for s in shape:
        n *= s
    dev = model._device()
    name = torch.cuda.get_device_name(dev)
    return "|".join([name, type(model).__name__, str(model.stencil.kind),
                     "%dD" % len(shape), "2^%d" % int(math.log2(max(n, 1)))])


def _time_candidate(model, args, variant, k, steps, stream, reps=3):
    args.fused_variant = variant
    args.fused_k = k
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    # one warm-up segment, then the fastest of `reps` timed ones
    _ffi.call("fw_step", ctypes.byref(args), 0, steps, stream.cuda_stream)
    best = float("inf")
    for _ in range(reps):
        e0.record(stream)
        _ffi.call("fw_step", ctypes.byref(args), 0, steps, stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def tune(model, steps=96):
    """Time every fused candidate for `model` (initialised, fused form) on
    scratch copies of its arrays; returns {"variant": v, "k": k, "ms": {...}}.
    """
    saved = model.autotune
    model.autotune = False
    try:
        a = model._bare_args()
    finally:
        model.autotune = saved
    keep = []
    for i in range(2):
        c = model._dev["u" if i == 0 else "u_new"].clone()
        keep.append(c)
        a.u[i] = c.data_ptr()
    for i, name in enumerate(model._state_names):
        c = model._dev[name].clone()
        keep.append(c)
        a.state[i] = c.data_ptr()
        c = model._dev[name].clone()
        keep.append(c)
        a.state_b[i] = c.data_ptr()
    a.form = _ffi.FORM_FUSED
    stream = torch.cuda.current_stream()
    tma_ok = a.weights_packed and model._shape()[1] % 16 == 0
    cands = (_TMA if tma_ok else []) + _CPASYNC
    times = {}
    for v, k in cands:
        try:
            times["%d/%d" % (v, k)] = _time_candidate(model, a, v, k, steps,
                                                      stream)
        except _ffi.FwError:
            continue
    del keep
    best = min(times, key=times.get)
    v, k = (int(x) for x in best.split("/"))
    return {"variant": v, "k": k, "ms": times, "steps": steps}


def choose(model):
    """(fused_variant, fused_k) for `model`: from the cache, else tuned now
    and cached."""
    kk = key(model)
    with _lock:
        if kk in _memo:
            r = _memo[kk]
            return r["variant"], r["k"]
        table = _load()
        if kk in table:
            _memo[kk] = table[kk]
            return table[kk]["variant"], table[kk]["k"]
    r = tune(model)
    with _lock:
        _memo[kk] = r
        table = _load()
        table[kk] = r
        _store(table)
    return r["variant"], r["k"]
