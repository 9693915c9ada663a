"""GPU parity of the detailed ionic models (TP06, Courtemanche) through the
public API: float64 against the reference's golden vectors, float32 (with
compensated float32 ion-concentration accumulators) against float64, and one ionic pass against the
oracle.

The device's exp/log/pow differ from the C library's and numpy's by an ulp or
two, so float64 is compared by relative error (scaled to each field's
magnitude near zero) rather than bitwise.
"""
import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu

# float64 on the GPU vs the reference: a few ulp per transcendental call,
# amplified over 2000 steps through an action potential upstroke.
F64_RTOL = 1e-8
# float32 gates, currents and potential vs float64 (concentrations float64)
F32_U_ATOL = 1.0       # mV, over the whole tissue at t = 20 ms
F32_GATE_ATOL = 2e-2   # gating variables in [0, 1]
F32_CONC_RTOL = 1e-3   # ion concentrations

CONC = {"tp06": {"cai", "casr", "cass", "nai", "Ki"},
        "crn": {"nai", "ki", "cai", "caup", "carel"}}


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


def _case(name, dim):
    return (cases.tp06 if name == "tp06" else cases.courtemanche)(dim)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("name", ["tp06", "crn"])
def test_detailed_f64_vs_reference(gc, name, dim):
    case, g = _case(name, dim)
    r = gc.run(case)
    assert r["step"] == 2000
    errs = {v: _rel_err(r[v], g[v]) for v in cases.MODEL_VARS[name]}
    bad = {v: e for v, e in errs.items() if not e < F64_RTOL}
    assert not bad, bad
    mv = r["trackers"][0]
    for v, x in mv.items():
        assert _rel_err(x, g["mv_" + v]) < F64_RTOL, v
    if name == "tp06":
        assert np.all(r["cai"] == 0.00007)   # frozen in the reference


# The gate for float64 on the potential: max |dV| <= 1e-9 mV after 10^4
# steps through an action potential, absolute, everywhere in the tissue.
LONG_U_ATOL = 1e-9


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("name", ["tp06", "crn"])
def test_detailed_f64_long_absolute(gc, name, dim):
    case, g = cases.detailed_long(name, dim)
    r = gc.run(case)
    assert r["step"] == g["step"] == 10000
    du = float(np.max(np.abs(r["u"] - g["u"])))
    dmv = float(np.max(np.abs(r["trackers"][0]["u"] - g["mv_u"])))
    print(f"{name} {dim}D float64, 10^4 steps: max|dV| {du:.3e} mV "
          f"(field), {dmv:.3e} mV (probes)")
    assert du <= LONG_U_ATOL, du
    assert dmv <= LONG_U_ATOL, dmv
    for v in cases.MODEL_VARS[name][1:]:
        assert _rel_err(r[v], g[v]) < F64_RTOL, v


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("name", ["tp06", "crn"])
def test_detailed_f32_close_to_f64(gc, name, dim):
    case, g = _case(name, dim)
    r = gc.run(case, npfloat="float32")
    m = r["model"]
    for i, v in enumerate(m._state_names):
        # concentrations: compensated float32 pairs, read back as float64
        assert m._dev[v].dtype == torch.float32, v
        assert m._dev[v].dim() == m._dev["u"].dim() + (v in CONC[name]), v
        if v in CONC[name]:
            assert getattr(m, v).dtype == np.float64, v
    du = float(np.max(np.abs(r["u"] - g["u"])))
    assert du < F32_U_ATOL, du
    for v in cases.MODEL_VARS[name][1:]:
        if v in CONC[name]:
            assert _rel_err(r[v], g[v]) < F32_CONC_RTOL, v
        elif v not in ("irel", "oo"):   # currents / derived, not gates
            d = float(np.max(np.abs(r[v] - g[v])))
            assert d < F32_GATE_ATOL, (v, d)


@pytest.mark.parametrize("name", ["tp06", "crn"])
def test_detailed_ionic_callable(gc, oracle, name):
    """run_ionic_kernel on random states in the physiological range equals
    one oracle ionic pass within float64 rounding of the transcendentals."""
    case, _ = _case(name, 2)
    model, _ = gc.build(case)
    model.initialize()
    shape = model._shape()
    rng = np.random.default_rng(11)
    spec = oracle.MODELS[name]
    u0 = rng.uniform(-90, 40, shape)
    un0 = u0 + rng.uniform(-1, 1, shape)
    st = {}
    for v in cases.MODEL_VARS[name][1:]:
        base = spec["init"][v]
        st[v] = base * rng.uniform(0.9, 1.1, shape) if base else \
            rng.uniform(0, 1e-3, shape)
        setattr(model, v, st[v])
    model.u = u0
    model.u_new = un0
    model.run_ionic_kernel()
    torch.cuda.synchronize()
    idx = np.flatnonzero(case["mesh"] == 1).astype(np.int64)
    un = un0.copy()
    ost = {k: x.copy() for k, x in st.items()}
    oracle._ionic(name, ost, un, u0, idx, case["dt"], spec["params"])
    assert _rel_err(model.u_new, un) < 1e-11
    for v in ost:
        assert _rel_err(getattr(model, v), ost[v]) < 1e-11, v
