"""GPU: ECG trackers (on-device reduction, fw_ecg_tracker / fw_ecg) against
the reference's golden ECG traces.  Float64: the diffusion is the
reference's (bitwise), the sum over myocytes is a parallel reduction in a
different order, so the traces agree to rounding (1e-12 of the trace's
scale).  Float32: within 1e-3 of the scale."""
import ctypes

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gc():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from finitewave_gb300 import _ffi
    _ffi.load()
    import gpu_cases
    return gpu_cases


@pytest.mark.parametrize("npfloat,rtol", [("float64", 1e-12),
                                          ("float32", 1e-3)])
@pytest.mark.parametrize("dim", [2, 3])
def test_ecg_traces(gc, dim, npfloat, rtol):
    case, g = cases.ecg(dim)
    r = gc.run(case, npfloat=npfloat)
    ecg = np.asarray(r["trackers"][0])
    assert ecg.shape == g["ecg"].shape
    scale = np.abs(g["ecg"]).max()
    assert np.abs(ecg - g["ecg"]).max() <= rtol * scale
    if npfloat == "float64":
        assert np.array_equal(r["u"], g["u"])


def test_fw_ecg_callable(gc):
    """fw_ecg on a state of the 2D case equals the oracle's compute_ecg."""
    from finitewave_gb300 import _ffi
    from oracle import oracle
    case, _ = cases.ecg(2)
    model, _ = gc.build(case)
    model.initialize()
    rng = np.random.default_rng(3)
    u0 = rng.uniform(0, 1, model._shape())
    model.u = u0
    coords = np.array([[25, 2, 0], [10, -3, 1.5], [3, 3, 0]], np.float64)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    ni, nj = model._shape()
    # coords stay in host memory (they are passed to the kernel by value)
    _ffi.call("fw_ecg", _ffi.ISO5, _ffi.F64, model._dev["u"].data_ptr(),
              model.weights.data_ptr(), model._myo_d.data_ptr(), ni, nj, 1,
              coords.ctypes.data, 3, model.dr, out.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    w = oracle.weights("iso5", case["mesh"], 1.0, case["dt"], case["dr"])
    idx = np.flatnonzero(case["mesh"] == 1).astype(np.int64)
    u_tr = np.zeros_like(u0)
    oracle._diffuse("iso5", u_tr, u0, w, idx)
    ref = oracle._ecg(u_tr, u0, coords, case["dr"], idx, u0.shape)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12,
                               atol=1e-15 * np.abs(ref).max())
    cd = torch.as_tensor(coords, device="cuda")
    with pytest.raises(_ffi.FwError, match="host memory"):
        _ffi.call("fw_ecg", _ffi.ISO5, _ffi.F64, model._dev["u"].data_ptr(),
                  model.weights.data_ptr(), model._myo_d.data_ptr(), ni, nj,
                  1, cd.data_ptr(), 3, model.dr, out.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)
