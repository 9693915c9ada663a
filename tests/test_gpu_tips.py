"""GPU: spiral-wave tips (SpiralWaveCore2D/3DTracker, on-device search and
refinement) and activation periods (Period2D/3DTracker) against the
reference's golden records.  Float64: bitwise (the refinement is the
reference's float64 expression tree, compiled without FMA contraction);
float32 runs of the same case find tips within 0.05 node and periods within
0.05 time units."""
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


def _case(dim):
    case, g = cases.tips(dim)
    case = dict(case)
    case["trackers"] = [dict(kind="tips", threshold=0.5, step=20),
                        dict(kind="period", threshold=0.5,
                             cells=g["cells"].tolist())]
    return case, g


def _rows(out, dim):
    z = np.asarray(out["z"], np.float64) if dim == 3 else \
        -np.ones(len(out["x"]))
    return np.stack([np.asarray(out["x"], np.float64),
                     np.asarray(out["y"], np.float64), z,
                     np.asarray(out["time"], np.float64),
                     np.asarray(out["step"], np.float64)], axis=1)


@pytest.mark.parametrize("dim", [2, 3])
def test_tips_and_periods_f64_bitwise(gc, dim):
    case, g = _case(dim)
    r = gc.run(case)
    assert np.array_equal(r["u"], g["u"])
    tips, periods = r["trackers"]
    assert np.array_equal(_rows(tips, dim), g["tips"])
    for got, want in zip(periods, g["periods"]):
        assert np.array_equal(np.asarray(got), want)


@pytest.mark.parametrize("dim", [2, 3])
def test_tips_and_periods_f32(gc, dim):
    case, g = _case(dim)
    r = gc.run(case, npfloat="float32")
    tips, periods = r["trackers"]
    got = _rows(tips, dim)
    want = g["tips"]
    # every reference tip has a float32 tip at the same step within 0.05
    for row in want:
        same = got[(got[:, 4] == row[4]) & (got[:, 2] == row[2])]
        assert same.size, row
        d = np.hypot(same[:, 0] - row[0], same[:, 1] - row[1]).min()
        assert d < 0.05, (row, d)
    for p, w in zip(periods, g["periods"]):
        assert len(p) == len(w)
        np.testing.assert_allclose(p, w, atol=0.05)
