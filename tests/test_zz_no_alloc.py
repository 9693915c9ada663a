"""GPU: fw_batch_run_noalloc (tile counters in the library's fixed device
array) against fw_batch_run (caller's scratch), both through the C ABI on
the same plan inputs, two calls in a row (an odd then an even step count,
the second continuing at the first one's offset).  Collected last so that it
also runs after every other test in the same process; it needs nothing from
them."""
import copy
import ctypes

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu

# Both entry points launch the same kernel on the same plan, so the results
# must be identical bit for bit: a tile counter left non-zero by an earlier
# call would shift the tiles and show up here.


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from finitewave_gb300 import _ffi
    _ffi.load()
    import gpu_cases
    return _ffi, gpu_cases


def _cases():
    out = []
    for c in (cases.ap2d_cfg1()[0], cases.models_2d("fk", True)[0],
              cases.models_2d("ms", False)[0]):
        c = copy.copy(c)
        c["trackers"] = [t for t in c["trackers"] if t["kind"] == "at"][:1]
        out.append(c)
    return out


def _build(gc):
    models = []
    for c in _cases():
        m, objs = gc.build(c, npfloat="float32")
        m.initialize()
        models.append((m, objs))
    return models


def _run(_ffi, models, steps, noalloc):
    """Plan the models once for sum(steps) steps, then one batch call per
    entry of `steps`, each at the previous calls' offset."""
    total = sum(steps)
    segs = [m._prepare_segment(total) for m, _ in models]
    assert all(s.n_seg == total for s in segs)
    k = len(segs)
    ptrs = (ctypes.c_void_p * k)(*[ctypes.addressof(s.args) for s in segs])
    n_begin = (ctypes.c_int64 * k)(*[s.n0 for s in segs])
    size = ctypes.c_int64()
    _ffi.call("fw_batch_plan_size", ptrs, k, ctypes.byref(size))
    plan = torch.empty(size.value, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    b = _ffi.Batch()
    _ffi.call("fw_batch_plan", ptrs, k, n_begin, plan.data_ptr(), size.value,
              ctypes.byref(b), stream)
    scratch = None
    if not noalloc:
        nb = ctypes.c_int64()
        _ffi.call("fw_batch_scratch_size", ctypes.byref(nb))
        scratch = torch.zeros(nb.value, dtype=torch.uint8, device="cuda")
    offset = 0
    for n in steps:
        if noalloc:
            _ffi.call("fw_batch_run_noalloc", ctypes.byref(b), offset, n,
                      stream)
        else:
            _ffi.call("fw_batch_run", ctypes.byref(b), scratch.data_ptr(),
                      offset, n, stream)
        offset += n
    torch.cuda.synchronize()
    for (m, _), s in zip(models, segs):
        m._finish_segment(s)
    del plan, scratch


def test_noalloc_matches_scratch_entry(env):
    _ffi, gc = env
    ref = _build(gc)
    got = _build(gc)
    steps = (37, 64)
    _run(_ffi, ref, steps, noalloc=False)
    _run(_ffi, got, steps, noalloc=True)
    # and a second pair of calls on the advanced state
    _run(_ffi, ref, steps, noalloc=False)
    _run(_ffi, got, steps, noalloc=True)
    for (mr, objs_r), (mg, objs_g) in zip(ref, got):
        assert mr.step == mg.step == 2 * sum(steps)
        for name in ["u"] + list(mr._state_names):
            assert np.array_equal(getattr(mg, name), getattr(mr, name)), name
        for tr, tg in zip(objs_r, objs_g):
            assert np.array_equal(tg.output, tr.output)
        assert np.any(getattr(mg, "u") != 0)


def test_noalloc_rejects_bad_arguments(env):
    """A NULL or empty plan and negative offsets or step counts come back
    as FW_ERR_ARG with a message, before any device work.  (The scratch a
    batch needs has a fixed size, which the library checks against the
    fixed array when it is compiled, so no call can ask for more.)"""
    _ffi, _ = env
    lib = _ffi.load()
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.fw_batch_run_noalloc(None, 0, 4, ctypes.c_void_p(stream)) == -1
    assert b"empty plan" in lib.fw_last_error()
    b = _ffi.Batch()
    assert lib.fw_batch_run_noalloc(ctypes.byref(b), 0, 4,
                                    ctypes.c_void_p(stream)) == -1
    ref = _build(env[1])[:1]
    seg = ref[0][0]._prepare_segment(8)
    ptrs = (ctypes.c_void_p * 1)(ctypes.addressof(seg.args))
    n_begin = (ctypes.c_int64 * 1)(seg.n0)
    size = ctypes.c_int64()
    _ffi.call("fw_batch_plan_size", ptrs, 1, ctypes.byref(size))
    plan = torch.empty(size.value, dtype=torch.uint8, device="cuda")
    _ffi.call("fw_batch_plan", ptrs, 1, n_begin, plan.data_ptr(), size.value,
              ctypes.byref(b), stream)
    assert lib.fw_batch_run_noalloc(ctypes.byref(b), -1, 4,
                                    ctypes.c_void_p(stream)) == -1
    assert lib.fw_batch_run_noalloc(ctypes.byref(b), 0, -4,
                                    ctypes.c_void_p(stream)) == -1
    assert b"negative" in lib.fw_last_error()
    torch.cuda.synchronize()
