"""GPU parity: the sm_103a library against the reference's golden vectors and
the CPU oracle, through the public API (which calls the C ABI).

Tolerances: float64 runs of models built from + - * / only (Aliev-Panfilov,
Mitchell-Schaeffer) and every stencil-weight build are bitwise equal
(``np.array_equal``); Fenton-Karma calls tanh, whose CUDA and C-library
roundings differ in the last ulp, so its fields get |diff| <= 1e-12.
Activation-time outputs are compared exactly.
"""
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
    from finitewave_gb300 import _ffi
    _ffi.load()
    return finitewave_gb300


@pytest.fixture(scope="module")
def gc(fg):
    import gpu_cases
    return gpu_cases


class _M:
    def __init__(self, D_model, dt, dr, npfloat="float64"):
        self.D_model, self.dt, self.dr, self.npfloat = D_model, dt, dr, npfloat
        self.device = None

    def _device(self):
        return torch.device("cuda")

    def _precision(self):
        return 0 if self.npfloat == "float64" else 1


def _weights(fg, stencil, g, cond, fibers=None, D_al=None, D_ac=None):
    shape = g["mesh"].shape
    t = fg.CardiacTissue2D(shape) if len(shape) == 2 \
        else fg.CardiacTissue3D(shape)
    t.mesh = g["mesh"].copy()
    t.conductivity = cond
    t.fibers = fibers
    if D_al is not None:
        stencil.D_al, stencil.D_ac = D_al, D_ac
    m = _M(float(g["D_model"]), float(g["dt"]), float(g["dr"]))
    w = stencil.compute_weights(m, t)
    torch.cuda.synchronize()
    return np.moveaxis(w.cpu().numpy(), 0, -1)


def test_weights_2d_bitwise(fg):
    g = cases.load("weights_2d")
    assert np.array_equal(_weights(fg, fg.IsotropicStencil2D(), g, 1.0),
                          g["w_iso5_c1"])
    assert np.array_equal(_weights(fg, fg.IsotropicStencil2D(), g, g["cond"]),
                          g["w_iso5_carr"])
    assert np.array_equal(
        _weights(fg, fg.AsymmetricStencil2D(), g, g["cond"], g["fibers"]),
        g["w_aniso9_carr"])
    assert np.array_equal(
        _weights(fg, fg.AsymmetricStencil2D(), g, 1.0, g["fibers"],
                 float(g["D_al_b"]), float(g["D_ac_b"])),
        g["w_aniso9_c1_dac0111"])


def test_weights_3d_bitwise(fg):
    g = cases.load("weights_3d")
    assert np.array_equal(_weights(fg, fg.IsotropicStencil3D(), g, 1.0),
                          g["w_iso7_c1"])
    assert np.array_equal(_weights(fg, fg.IsotropicStencil3D(), g, g["cond"]),
                          g["w_iso7_carr"])
    assert np.array_equal(
        _weights(fg, fg.AsymmetricStencil3D(), g, g["cond"], g["fibers"]),
        g["w_aniso19_carr"])
    assert np.array_equal(
        _weights(fg, fg.AsymmetricStencil3D(), g, 1.0, g["fibers"],
                 float(g["D_al_b"]), float(g["D_ac_b"])),
        g["w_aniso19_c1_dac025"])


def test_weights_f32_rounding(fg):
    """FP32 weights are the float64 weights rounded once."""
    g = cases.load("weights_2d")
    t = fg.CardiacTissue2D(g["mesh"].shape)
    t.mesh = g["mesh"].copy()
    t.fibers = g["fibers"]
    m = _M(float(g["D_model"]), float(g["dt"]), float(g["dr"]), "float32")
    w = fg.AsymmetricStencil2D().compute_weights(m, t)
    ref = g["w_aniso9_c1_dac0111"]
    st = fg.AsymmetricStencil2D()
    st.D_al, st.D_ac = float(g["D_al_b"]), float(g["D_ac_b"])
    w = st.compute_weights(m, t)
    assert w.dtype == torch.float32
    assert np.array_equal(np.moveaxis(w.cpu().numpy(), 0, -1),
                          ref.astype(np.float32))


def test_ap2d_cfg1_bitwise(gc):
    """100x100 Aliev-Panfilov planar wave, 5000 FP64 steps: u, v, u_new and
    the activation map equal the reference's bit for bit."""
    case, g = cases.ap2d_cfg1()
    r = gc.run(case)
    assert r["step"] == int(g["step"]) == 5000
    assert r["t"] == float(g["t"])
    assert np.array_equal(r["u"], g["u"])
    assert np.array_equal(r["v"], g["v"])
    assert np.array_equal(r["u_new"], g["u_new"])
    assert np.array_equal(r["trackers"][0], g["act_t"])


def test_ap2d_aniso_spiral_bitwise(gc):
    """42x42 anisotropic, fibrotic, heterogeneous conductivity, S1-S2,
    10^4 FP64 steps, with probes on a stride and a time window."""
    case, g = cases.ap2d_aniso_spiral()
    r = gc.run(case)
    assert r["step"] == 10000
    assert np.array_equal(r["u"], g["u"])
    assert np.array_equal(r["v"], g["v"])
    at, ap, mv = r["trackers"]
    assert np.array_equal(at, g["act_t"])
    assert np.array_equal(ap["u"], g["ap"])
    assert np.array_equal(mv["u"], g["mv_u"])
    assert np.array_equal(mv["v"], g["mv_v"])


@pytest.mark.parametrize("name", ["ms", "fk"])
@pytest.mark.parametrize("aniso", [False, True])
def test_models_2d(gc, oracle, name, aniso):
    case, g = cases.models_2d(name, aniso)
    r = gc.run(case)
    o = oracle.run(case)
    at, mv = r["trackers"]
    assert np.array_equal(at, g["act_t"])
    for v in cases.MODEL_VARS[name]:
        if name == "ms":
            assert np.array_equal(r[v], g[v]), v
            assert np.array_equal(mv[v], g["mv_" + v]), v
        else:
            np.testing.assert_allclose(r[v], o[v], rtol=0, atol=1e-12)
            np.testing.assert_allclose(r[v], g[v], rtol=0, atol=1e-12)
            np.testing.assert_allclose(mv[v], g["mv_" + v], rtol=0,
                                       atol=1e-12)


@pytest.mark.parametrize("aniso", [False, True])
def test_ap3d_bitwise(gc, aniso):
    case, g = cases.ap3d(aniso)
    r = gc.run(case)
    assert np.array_equal(r["u"], g["u"])
    assert np.array_equal(r["v"], g["v"])
    assert np.array_equal(r["trackers"][0], g["act_t"])


def test_trackers_cable(gc):
    """The reference's tracker-test cable: LAT layers, AT with the default
    threshold (every node, non-myocytes included) and a windowed, strided
    AT tracker."""
    case, g = cases.trackers_cable()
    r = gc.run(case)
    lat, at, at_def, at_win = r["trackers"]
    assert lat.shape == g["lat"].shape
    assert np.array_equal(lat, g["lat"])
    assert np.array_equal(at, g["act_t"])
    assert np.array_equal(at_def, g["act_t_default"])
    assert np.array_equal(at_win, g["act_t_windowed"])
    assert np.array_equal(r["u"], g["u"])


def test_stimuli_matrix_area(gc):
    case, g = cases.stimuli_2d()
    r = gc.run(case)
    assert np.array_equal(r["u"], g["u2d"])
    assert np.array_equal(r["v"], g["v2d"])
    assert np.array_equal(r["trackers"][0], g["act_t2d"])


def test_f32_plain_close_to_f64(gc):
    """FP32 plain form against FP64 on the anisotropic spiral: activation
    times within one step on >= 99.9 % of nodes."""
    case, g = cases.ap2d_aniso_spiral()
    r = gc.run(case, npfloat="float32")
    at = r["trackers"][0]
    ref = g["act_t"]
    both = (at >= 0) & (ref >= 0)
    assert ((at >= 0) == (ref >= 0)).mean() >= 0.999
    err_steps = np.abs(at[both] - ref[both]) / case["dt"]
    assert (err_steps <= 1.0 + 1e-6).mean() >= 0.999
    assert np.abs(r["u"] - g["u"]).max() < 5e-3


def test_diffusion_and_ionic_callables(fg, gc, oracle):
    """model.diffusion_kernel(u_new, u, w, indexes) and run_ionic_kernel on
    device tensors reproduce one oracle step bitwise."""
    case, _ = cases.ap2d_aniso_spiral()
    model, _ = gc.build(case)
    model.initialize()
    rng = np.random.default_rng(5)
    u0 = rng.uniform(0, 1, model._shape())
    v0 = rng.uniform(0, 0.5, model._shape())
    model.u = u0
    model.v = v0
    model.run_diffusion_kernel()
    model.run_ionic_kernel()
    torch.cuda.synchronize()
    w = oracle.weights("aniso9", case["mesh"], 1.0, case["dt"], case["dr"],
                       case["conductivity"], case["fibers"])
    idx = np.flatnonzero(case["mesh"] == 1).astype(np.int64)
    un = np.zeros_like(u0)
    v = v0.copy()
    oracle._diffuse("aniso9", un, u0, w, idx)
    oracle._ionic("ap", {"v": v}, un, u0, idx, case["dt"],
                  oracle.MODELS["ap"]["params"])
    assert np.array_equal(model.u_new, un)
    assert np.array_equal(model.v, v)
