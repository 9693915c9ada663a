"""GPU: the device status word reaches the caller.

A bounded on-chip wait that gives up, or a batch tile that names no tissue,
must end in an exception from ``run()`` rather than in silently wrong fields.
Neither failure is caused by a fault: the TMA kernels are told through
``fw_step_args.debug_flags`` (FW_DEBUG_FORCE_TIMEOUT) to treat their first
pipeline wait as timed out after its copy has arrived, and the batch plan's
tile list is given an out-of-range tissue index, which the batch kernel
checks before it uses it.  After either, the same CUDA context runs a clean
case to the expected result.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gc():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from finitewave_gb300 import _ffi
    _ffi.load()
    import gpu_cases
    return gpu_cases


def _case():
    """Aliev-Panfilov on a 66 x 96 sheet (rows a multiple of 16 nodes, as
    the TMA kernels need), 9-point stencil, a planar voltage stimulus and
    an activation tracker."""
    ni, nj = 66, 96
    rng = np.random.default_rng(5)
    mesh = np.ones((ni, nj), np.int8)
    mesh[rng.random((ni, nj)) < 0.1] = 2
    mesh[0], mesh[-1], mesh[:, 0], mesh[:, -1] = 0, 0, 0, 0
    ang = rng.uniform(-np.pi, np.pi, (ni, nj))
    fib = np.stack([np.cos(ang), np.sin(ang)], -1)
    return dict(model="ap", mesh=mesh, fibers=fib, stencil="aniso9",
                dt=0.01, dr=0.25, t_max=2.0,
                stims=[dict(kind="voltage", t=0, value=1.0,
                            box=[(0, ni), (1, 4)])],
                trackers=[dict(kind="at", threshold=0.5)])


@pytest.mark.parametrize("variant", [3, 4, 6, 7])
def test_forced_timeout_raises(gc, variant):
    from finitewave_gb300 import _ffi
    case = _case()
    m, _ = gc.build(case, npfloat="float32", form="fused", fused_k=4,
                    fused_variant=variant)
    m._debug_flags = _ffi.FW_DEBUG_FORCE_TIMEOUT
    with pytest.raises(RuntimeError, match="bounded on-chip wait"):
        m.run()
    assert int(m._status.item()) & _ffi.FW_DEV_TIMEOUT
    # the context is still usable: the same case without the flag gives
    # bitwise the cp.async kernel's result
    clean, objs = gc.build(case, npfloat="float32", form="fused", fused_k=4,
                           fused_variant=variant)
    clean.run()
    ref, robjs = gc.build(case, npfloat="float32", form="fused", fused_k=4,
                          fused_variant=1)
    ref.run()
    assert np.array_equal(clean.u, ref.u)
    assert np.array_equal(clean.v, ref.v)
    assert np.array_equal(objs[0].output, robjs[0].output)
    assert np.any(clean.u != 0)


def test_batch_tile_out_of_range_raises(gc):
    from finitewave_gb300 import _ffi
    m, _ = gc.build(_case(), npfloat="float32")
    m.initialize()
    seg = m._prepare_segment(8)
    ptrs = (ctypes.c_void_p * 1)(ctypes.addressof(seg.args))
    n_begin = (ctypes.c_int64 * 1)(seg.n0)
    size = ctypes.c_int64()
    _ffi.call("fw_batch_plan_size", ptrs, 1, ctypes.byref(size))
    plan = torch.empty(size.value, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    b = _ffi.Batch()
    _ffi.call("fw_batch_plan", ptrs, 1, n_begin, plan.data_ptr(), size.value,
              ctypes.byref(b), stream)
    # the tile list ends the plan, its entries start with the tissue index
    # (int32): point the first entry at a tissue that does not exist
    entry = 16 if b.kernel == 2 else 8
    first_tile = size.value - entry * b.n_tiles
    plan[first_tile:first_tile + 4] = torch.tensor(
        [b.n_tissues], dtype=torch.int32).view(torch.uint8).to("cuda")
    nb = ctypes.c_int64()
    _ffi.call("fw_batch_scratch_size", ctypes.byref(nb))
    scratch = torch.zeros(nb.value, dtype=torch.uint8, device="cuda")
    _ffi.call("fw_batch_run", ctypes.byref(b), scratch.data_ptr(), 0, 8,
              stream)
    torch.cuda.synchronize()
    m._finish_segment(seg)
    assert int(m._status.item()) & _ffi.FW_DEV_BATCH_FAULT
    with pytest.raises(RuntimeError, match="batch tile"):
        m._check_status()
    # the scratch counters were reset by the launch: a clean plan runs
    assert int(scratch.view(torch.int32)[:2].abs().sum().item()) == 0
