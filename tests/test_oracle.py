"""Pin the CPU oracle against the golden vectors produced by the reference.

The oracle (oracle/fw_oracle.c + oracle/oracle.py) is what every GPU parity
test compares against, so it is checked here first: weights, stimuli,
trackers and the Aliev-Panfilov / Mitchell-Schaeffer runs must be bitwise
equal to the reference's float64 results; Fenton-Karma calls tanh, whose
last-ulp rounding differs between numpy and the C library, so its traces get
a 1e-14 absolute tolerance.
"""
import numpy as np
import pytest

import cases


def test_weights_2d(oracle):
    g = cases.load("weights_2d")
    a = (float(g["D_model"]), float(g["dt"]), float(g["dr"]))
    assert np.array_equal(oracle.weights("iso5", g["mesh"], *a),
                          g["w_iso5_c1"])
    assert np.array_equal(oracle.weights("iso5", g["mesh"], *a, g["cond"]),
                          g["w_iso5_carr"])
    assert np.array_equal(
        oracle.weights("aniso9", g["mesh"], *a, g["cond"], g["fibers"]),
        g["w_aniso9_carr"])
    assert np.array_equal(
        oracle.weights("aniso9", g["mesh"], *a, 1.0, g["fibers"],
                       float(g["D_al_b"]), float(g["D_ac_b"])),
        g["w_aniso9_c1_dac0111"])


def test_weights_3d(oracle):
    g = cases.load("weights_3d")
    a = (float(g["D_model"]), float(g["dt"]), float(g["dr"]))
    assert np.array_equal(oracle.weights("iso7", g["mesh"], *a),
                          g["w_iso7_c1"])
    assert np.array_equal(oracle.weights("iso7", g["mesh"], *a, g["cond"]),
                          g["w_iso7_carr"])
    assert np.array_equal(
        oracle.weights("aniso19", g["mesh"], *a, g["cond"], g["fibers"]),
        g["w_aniso19_carr"])
    assert np.array_equal(
        oracle.weights("aniso19", g["mesh"], *a, 1.0, g["fibers"],
                       float(g["D_al_b"]), float(g["D_ac_b"])),
        g["w_aniso19_c1_dac025"])


def test_ap2d_aniso_spiral_bitwise(oracle):
    case, g = cases.ap2d_aniso_spiral()
    r = oracle.run(case)
    assert r["step"] == int(g["step"]) == 10000
    assert r["t"] == float(g["t"])
    for k in ("u", "v"):
        assert np.array_equal(r[k], g[k]), k
    at, ap, mv = r["trackers"]
    assert np.array_equal(at, g["act_t"])
    assert np.array_equal(ap["u"], g["ap"])
    assert np.array_equal(mv["u"], g["mv_u"])
    assert np.array_equal(mv["v"], g["mv_v"])


@pytest.mark.parametrize("name", ["ms", "fk"])
@pytest.mark.parametrize("aniso", [False, True])
def test_models_2d(oracle, name, aniso):
    case, g = cases.models_2d(name, aniso)
    r = oracle.run(case)
    at, mv = r["trackers"]
    assert np.array_equal(at, g["act_t"])
    for v in cases.MODEL_VARS[name]:
        if name == "ms":
            assert np.array_equal(r[v], g[v]), v
            assert np.array_equal(mv[v], g["mv_" + v]), v
        else:
            np.testing.assert_allclose(r[v], g[v], rtol=0, atol=1e-14)
            np.testing.assert_allclose(mv[v], g["mv_" + v], rtol=0,
                                       atol=1e-14)


@pytest.mark.parametrize("aniso", [False, True])
def test_ap3d_bitwise(oracle, aniso):
    case, g = cases.ap3d(aniso)
    r = oracle.run(case)
    for k in ("u", "v"):
        assert np.array_equal(r[k], g[k]), k
    assert np.array_equal(r["trackers"][0], g["act_t"])


def test_trackers_cable(oracle):
    case, g = cases.trackers_cable()
    r = oracle.run(case)
    lat, at, at_def, at_win = r["trackers"]
    assert np.array_equal(lat, g["lat"])
    assert lat.shape[0] == 2
    assert np.array_equal(at, g["act_t"])
    assert np.array_equal(at_def, g["act_t_default"])
    assert np.array_equal(at_win, g["act_t_windowed"])
    assert np.array_equal(r["u"], g["u"])


def test_stimuli(oracle):
    case, g = cases.stimuli_2d()
    r = oracle.run(case)
    assert np.array_equal(r["u"], g["u2d"])
    assert np.array_equal(r["v"], g["v2d"])
    assert np.array_equal(r["trackers"][0], g["act_t2d"])


def test_ap2d_cfg1_bitwise(oracle):
    """The 100x100 Aliev-Panfilov planar-wave case, 5000 steps."""
    case, g = cases.ap2d_cfg1()
    r = oracle.run(case)
    assert r["step"] == int(g["step"]) == 5000
    assert np.array_equal(r["u"], g["u"])
    assert np.array_equal(r["v"], g["v"])
    assert np.array_equal(r["u_new"], g["u_new"])
    assert np.array_equal(r["trackers"][0], g["act_t"])


def _rel_err(a, b):
    """max |a-b| / (|b| + 1e-3 max|b|): relative away from zero, absolute
    (scaled to the field) near it."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = 1e-3 * max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b) / (np.abs(b) + scale)))


# TP06 and Courtemanche call exp/log/sqrt/pow hundreds of times per node-step:
# numpy's and the C library's results differ in the last ulp, and 2000 steps
# of action potential amplify that to ~1e-12 relative.
DETAILED_RTOL = 1e-9


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("name", ["tp06", "crn"])
def test_detailed_models(oracle, name, dim):
    case, g = (cases.tp06 if name == "tp06" else cases.courtemanche)(dim)
    r = oracle.run(case)
    assert r["step"] == 2000
    assert g["u"].max() > 0, "the case must fire an action potential"
    for v in cases.MODEL_VARS[name]:
        assert _rel_err(r[v], g[v]) < DETAILED_RTOL, v
    mv = r["trackers"][0]
    for v, x in mv.items():
        assert _rel_err(x, g["mv_" + v]) < DETAILED_RTOL, v
    if name == "tp06":
        # the reference never updates Ca_i
        assert np.all(r["cai"] == 0.00007)


# The absolute gate on the potential for float64 runs of the detailed
# models: max |dV| <= 1e-9 mV after 10^4 steps through an action potential.
LONG_U_ATOL = 1e-9


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("name", ["tp06", "crn"])
def test_detailed_models_long(oracle, name, dim):
    """10^4 steps through the upstroke: the oracle's potential stays within
    1e-9 mV of the reference's everywhere, and every state variable within
    1e-9 relative."""
    case, g = cases.detailed_long(name, dim)
    r = oracle.run(case)
    assert r["step"] == g["step"] == 10000
    assert g["u"].max() > 0, "the case must fire an action potential"
    du = float(np.max(np.abs(r["u"] - g["u"])))
    assert du <= LONG_U_ATOL, du
    dmv = float(np.max(np.abs(r["trackers"][0]["u"] - g["mv_u"])))
    assert dmv <= LONG_U_ATOL, dmv
    for v in cases.MODEL_VARS[name][1:]:
        assert _rel_err(r[v], g[v]) < DETAILED_RTOL, v


@pytest.mark.parametrize("dim", [2, 3])
def test_ecg_bitwise(oracle, dim):
    """compute_ecg after the diffusion kernel, every tracked step."""
    case, g = cases.ecg(dim)
    r = oracle.run(case)
    assert np.array_equal(r["u"], g["u"])
    assert np.array_equal(r["trackers"][0], g["ecg"])


def _periods_from_layers(layers, cells):
    lats = np.array(layers)
    out = []
    for c in np.atleast_2d(cells):
        row = lats[(slice(None),) + tuple(c)]
        out.append(np.diff(row[row != -1]))
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_spiral_tips_and_periods_bitwise(oracle, dim):
    case, g = cases.tips(dim)
    r = oracle.run(case)
    assert np.array_equal(r["u"], g["u"])
    assert g["tips"].shape[0] > 0
    assert np.array_equal(r["trackers"][0], g["tips"])
    for got, want in zip(_periods_from_layers(r["trackers"][1], g["cells"]),
                         g["periods"]):
        assert np.array_equal(got, want)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("name", ["bk", "bo", "lr91"])
def test_models_extra(oracle, name, dim):
    """Barkley (+ - * / only: bitwise), Bueno-Orovio (tanh) and Luo-Rudy
    1991 (exp / log / sqrt) against the reference."""
    case, g = cases.models_extra(name, dim)
    r = oracle.run(case)
    at, mv = r["trackers"]
    tol = 0.0 if name == "bk" else DETAILED_RTOL
    for v in cases.EXTRA_VARS[name]:
        assert _rel_err(r[v], g[v]) <= tol, v
    for v, x in mv.items():
        assert _rel_err(x, g["mv_" + v]) <= tol, v
    assert np.array_equal(at, g["act_t"])


def test_weights_sym9(oracle):
    """SymmetricStencil2D weights (its own scaling order) bitwise."""
    g = cases.load("weights_2d")
    a = (float(g["D_model"]), float(g["dt"]), float(g["dr"]))
    assert np.array_equal(
        oracle.weights("sym9", g["mesh"], *a, g["cond"], g["fibers"]),
        g["w_sym9_carr"])
    assert np.array_equal(
        oracle.weights("sym9", g["mesh"], *a, 1.0, g["fibers"],
                       float(g["D_al_b"]), float(g["D_ac_b"])),
        g["w_sym9_c1_dac0111"])
