"""GPU: Barkley, Bueno-Orovio and Luo-Rudy 1991 against the reference's
golden vectors.  Float64 plain form: Barkley bitwise (+ - * / only);
Bueno-Orovio (tanh) and LR91 (exp / log / sqrt) within 1e-8 relative.
Float32 (Barkley in the fused form, the others plain with float64 Ca_i):
activation times within one step, fields within the stated tolerances."""
import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu


def _rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = 1e-3 * max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b) / (np.abs(b) + scale)))


@pytest.fixture(scope="module")
def gc():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from finitewave_gb300 import _ffi
    _ffi.load()
    import gpu_cases
    return gpu_cases


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("name", ["bk", "bo", "lr91"])
def test_f64_vs_reference(gc, name, dim):
    case, g = cases.models_extra(name, dim)
    r = gc.run(case)
    at, mv = r["trackers"]
    tol = 0.0 if name == "bk" else 1e-8
    for v in cases.EXTRA_VARS[name]:
        assert _rel_err(r[v], g[v]) <= tol, v
    for v, x in mv.items():
        assert _rel_err(x, g["mv_" + v]) <= tol, v
    if name == "bk":
        assert np.array_equal(at, g["act_t"])
    else:
        assert np.abs(at - g["act_t"]).max() <= 0.01 + 1e-9


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("name", ["bk", "bo", "lr91"])
def test_f32_close(gc, name, dim):
    case, g = cases.models_extra(name, dim)
    r = gc.run(case, npfloat="float32")
    at, _ = r["trackers"]
    both = (at >= 0) & (g["act_t"] >= 0)
    assert ((at >= 0) == (g["act_t"] >= 0)).all()
    assert np.abs(at[both] - g["act_t"][both]).max() <= 0.01 + 1e-6
    atol = {"bk": 5e-3, "bo": 5e-3, "lr91": 0.5}[name]
    assert np.abs(r["u"] - g["u"]).max() <= atol
    if dim == 2 and name == "bk":
        assert r["model"]._fused_choice is not None   # the fused form ran
