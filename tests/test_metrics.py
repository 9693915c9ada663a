"""The accuracy measures (finitewave_gb300.metrics) on traces and maps
with known answers."""
import numpy as np
import pytest

from finitewave_gb300 import metrics


def test_apd_threshold_counts_samples_between_crossings():
    u = np.zeros(1000)
    u[100:350] = 1.0
    u[500:760] = 1.0
    assert metrics.apd_threshold(u, 0.1, 0.5, 0) == pytest.approx(25.0)
    assert metrics.apd_threshold(u, 0.1, 0.5, 1) == pytest.approx(26.0)
    assert metrics.apd_threshold(u, 0.1, 0.5, 2) is None


def test_apd90_interpolates_levels():
    dt = 0.5
    t = np.arange(0, 400, dt)
    u = np.full(t.shape, -80.0)
    up = (t >= 10) & (t < 12)
    u[up] = -80 + 120 * (t[up] - 10) / 2          # linear upstroke to 40
    plateau = (t >= 12) & (t < 200)
    u[plateau] = 40.0
    down = (t >= 200) & (t < 300)
    u[down] = 40 - 120 * (t[down] - 200) / 100    # linear repolarisation
    # upstroke at 10 % (t = 10.2), 90 % repolarisation at -68 (t = 290)
    assert metrics.apd90(u, dt) == pytest.approx(290 - 10.2, abs=1e-9)


def test_activation_error_steps():
    a = np.array([[0.0, 0.01, 0.02], [-1.0, 0.05, 0.10]])
    b = np.array([[0.0, 0.02, 0.05], [-1.0, 0.05, -1.0]])
    within, worst, one = metrics.activation_error_steps(a, b, 0.01)
    assert worst == 3 and one == 1
    assert within == pytest.approx(3 / 5)


def test_conduction_velocity_of_a_planar_wave():
    dr, c = 0.25, 0.6
    x = np.arange(40) * dr
    act = np.tile(x / c, (30, 1))
    v = metrics.conduction_velocity(act, dr)
    assert np.nanmedian(v) == pytest.approx(c)
    assert np.isnan(v[:, 0]).all() and np.isnan(v[0, :]).all()
    slow = np.tile(x / (0.9 * c), (30, 1))
    assert metrics.cv_error_percent(slow, act, dr) == pytest.approx(10.0)
