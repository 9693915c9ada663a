"""GPU: user stimuli and trackers written against the reference's plug-in
interface (``Stim.stimulate``, ``Tracker._track``) run on the host between
device steps, and give the reference's results.

The two classes below restate, on this package's base classes, the ones the
golden fixture was made with (tests/golden/make_golden.py, case
``plugins``): a stimulus that re-excites three rows whenever one node is at
rest, and a tracker that records sums of ``model.u`` and ``model.u_new``
over a patch and a node of ``v`` read through ``model.__dict__``.  Float64
Aliev-Panfilov is bitwise the reference's on the device, so every output is
compared exactly.
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


def _classes(fg):
    class RestimulateWhenQuiet(fg.Stim):
        def __init__(self, time, duration):
            super().__init__(time, duration)
            self.count = 0

        def initialize(self, model):
            self.count = 0

        def stimulate(self, model):
            if model.u[15, 15] < 0.1:
                model.u[1:4, 1:-1] = 1.0
                self.count += 1

    class PatchTracker(fg.Tracker):
        def initialize(self, model):
            self.model = model
            self.output = []

        def _track(self):
            m = self.model
            self.output.append([m.step, m.t, float(m.u[3:6, 3:6].sum()),
                                float(m.u_new[3:6, 3:6].sum()),
                                float(m.__dict__["v"][4, 4])])

    return RestimulateWhenQuiet, PatchTracker


def _model(fg, form=None, npfloat="float64"):
    Restim, Patch = _classes(fg)
    n = 32
    model = fg.AlievPanfilov2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 60
    model.npfloat = npfloat
    model.form = form
    model.prog_bar = False
    model.cardiac_tissue = fg.CardiacTissue2D((n, n))
    ss = fg.StimSequence()
    ss.add_stim(fg.StimVoltageCoord2D(0, 1.0, 0, n, 1, 5))
    rs = Restim(30, 2.0)
    ss.add_stim(rs)
    model.stim_sequence = ss
    pt = Patch()
    pt.start_time = 5
    pt.step = 50
    at = fg.ActivationTime2DTracker()
    at.threshold = 0.5
    seq = fg.TrackerSequence()
    seq.add_tracker(pt)
    seq.add_tracker(at)
    model.tracker_sequence = seq
    return model, rs, pt, at


def test_user_stim_and_tracker_match_reference(fg):
    g = cases.load("plugins")
    model, rs, pt, at = _model(fg)
    model.run()
    assert model.step == int(g["step"])
    assert rs.count == int(g["restim_count"])
    assert np.array_equal(np.asarray(pt.output, np.float64), g["patch"])
    assert np.array_equal(at.output, g["act_t"])
    assert np.array_equal(model.u, g["u"])
    assert np.array_equal(model.v, g["v"])
    # the host copies put into model.__dict__ for the tracker are gone
    assert "v" not in model.__dict__ and "u" not in model.__dict__


def test_user_plugins_with_float32_fused_segments(fg):
    """Between host steps a float32 model keeps its fused kernels: the
    user stimulus fires the same number of times and the patch sums stay
    within float32 accuracy of the reference."""
    g = cases.load("plugins")
    model, rs, pt, at = _model(fg, npfloat="float32")
    model.run()
    assert rs.count == int(g["restim_count"])
    out = np.asarray(pt.output, np.float64)
    assert np.array_equal(out[:, :2], g["patch"][:, :2])
    np.testing.assert_allclose(out[:, 2:], g["patch"][:, 2:], rtol=0,
                               atol=1e-3)
    ok = np.abs(at.output - g["act_t"]) <= 0.01 + 1e-9
    assert ok.mean() >= 0.999
