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

# Both entry points launch the same kernel on the same inputs, so the results
# are expected to be identical; the tolerance only allows for nothing more
# than float32 rounding noise.
ATOL = 1e-6


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
            np.testing.assert_allclose(getattr(mg, name), getattr(mr, name),
                                       rtol=0, atol=ATOL, err_msg=name)
        for tr, tg in zip(objs_r, objs_g):
            np.testing.assert_allclose(tg.output, tr.output, rtol=0,
                                       atol=ATOL)
        assert np.any(getattr(mg, "u") != 0)
