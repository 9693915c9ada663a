"""GPU: SymmetricStencil2D weights bitwise equal to the reference's, and an
Aliev-Panfilov run with them bitwise equal to the oracle (float64) and
within tolerance in float32 (fused form)."""
import copy

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    import finitewave_gb300
    finitewave_gb300._ffi.load()
    return finitewave_gb300


class _M:
    def __init__(self, D_model, dt, dr, npfloat="float64"):
        self.D_model, self.dt, self.dr, self.npfloat = D_model, dt, dr, npfloat

    def _device(self):
        return torch.device("cuda")

    def _precision(self):
        return 0 if self.npfloat == "float64" else 1


def test_sym9_weights_bitwise(fg):
    g = cases.load("weights_2d")
    t = fg.CardiacTissue2D(g["mesh"].shape)
    t.mesh = g["mesh"].copy()
    t.fibers = g["fibers"]
    m = _M(float(g["D_model"]), float(g["dt"]), float(g["dr"]))
    t.conductivity = g["cond"]
    w = fg.SymmetricStencil2D().compute_weights(m, t)
    torch.cuda.synchronize()
    assert np.array_equal(np.moveaxis(w.cpu().numpy(), 0, -1), g["w_sym9_carr"])
    st = fg.SymmetricStencil2D()
    st.D_al, st.D_ac = float(g["D_al_b"]), float(g["D_ac_b"])
    t.conductivity = 1.0
    w = st.compute_weights(m, t)
    torch.cuda.synchronize()
    assert np.array_equal(np.moveaxis(w.cpu().numpy(), 0, -1),
                          g["w_sym9_c1_dac0111"])


def test_sym9_run(fg, oracle):
    import gpu_cases
    case, _ = cases.ap2d_aniso_spiral()
    case = copy.copy(case)
    case["stencil"] = "sym9"
    case["t_max"] = 40
    r = gpu_cases.run(case)
    o = oracle.run(case)
    assert np.array_equal(r["u"], o["u"]) and np.array_equal(r["v"], o["v"])
    r32 = gpu_cases.run(case, npfloat="float32")
    assert np.abs(r32["u"] - o["u"]).max() < 5e-3
