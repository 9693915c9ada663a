"""Accuracy measures of a float32 run against a float64 run of the same
configuration: potential difference, activation-time error in steps, action
potential duration and conduction velocity.

The action potential duration of the reference's model tests
(tests/test_models_2d.py:74-106) is restated in `apd_threshold`; `apd90` is
the duration to 90 % repolarisation.  Conduction velocity comes from the
gradient of an activation-time map (the reference's own velocity tools need
scikit-image; this is the central-difference estimate).
"""
import numpy as np


def apd_threshold(u, dt, threshold, beat_index=0):
    """Duration between the beat's upward crossing of `threshold` and the
    next downward crossing (tests/test_models_2d.py:74-106); None when the
    trace has no such beat."""
    u = np.asarray(u, dtype=np.float64)
    up = np.flatnonzero((u[:-1] < threshold) & (u[1:] >= threshold))
    down = np.flatnonzero((u[:-1] > threshold) & (u[1:] <= threshold))
    if len(up) <= beat_index or len(down) == 0:
        return None
    start = up[beat_index]
    ends = down[down > start]
    if len(ends) == 0:
        return None
    return float((ends[0] - start) * dt)


def apd90(u, dt, beat_index=0):
    """APD90 of one beat: from the upstroke (first sample at or above the
    level 10 % of the way from rest to peak) to the first later sample at or
    below 90 % repolarisation, with linear interpolation between samples.
    Rest is the trace's value before the beat; None without a complete
    beat."""
    u = np.asarray(u, dtype=np.float64)
    if u.size < 3:
        return None
    rest = float(np.min(u))
    peak = float(np.max(u))
    amp = peak - rest
    if amp <= 0:
        return None
    lo = rest + 0.1 * amp
    ups = np.flatnonzero((u[:-1] < lo) & (u[1:] >= lo))
    if len(ups) <= beat_index:
        return None
    i0 = ups[beat_index]
    nxt = ups[beat_index + 1] if len(ups) > beat_index + 1 else u.size - 1
    seg = u[i0:nxt + 1]
    vmax = float(seg.max())
    v90 = vmax - 0.9 * (vmax - rest)
    ipk = i0 + int(np.argmax(seg))
    downs = np.flatnonzero((u[ipk:-1] > v90) & (u[ipk + 1:] <= v90))
    if len(downs) == 0:
        return None
    j = ipk + downs[0]

    def cross(k, level):
        a, b = u[k], u[k + 1]
        return k + (level - a) / (b - a) if b != a else float(k)

    return float((cross(j, v90) - cross(i0, lo)) * dt)


def activation_error_steps(act_a, act_b, dt, mask=None):
    """Activation-time maps (model time, -1 = never) compared in steps:
    (fraction of nodes within one step, largest error in steps, nodes where
    exactly one of the two activated)."""
    a = np.asarray(act_a, dtype=np.float64)
    b = np.asarray(act_b, dtype=np.float64)
    m = np.ones(a.shape, bool) if mask is None else np.asarray(mask, bool)
    both = m & (a >= 0) & (b >= 0)
    one = int((m & ((a >= 0) != (b >= 0))).sum())
    if not both.any():
        return 1.0 if one == 0 else 0.0, 0, one
    d = np.abs(np.rint(a[both] / dt) - np.rint(b[both] / dt))
    within = float((d <= 1).sum() / (both.sum() + one))
    return within, int(d.max()), one


def conduction_velocity(act, dr, mask=None):
    """Local conduction speed 1 / |grad T| (central differences over nodes
    whose neighbours along an axis are activated) at every interior node:
    array of speeds (NaN where undefined)."""
    t = np.asarray(act, dtype=np.float64)
    ok = t >= 0 if mask is None else (t >= 0) & np.asarray(mask, bool)
    g2 = np.zeros(t.shape)
    valid = ok.copy()
    for ax in range(t.ndim):
        fwd = np.roll(t, -1, ax)
        bwd = np.roll(t, 1, ax)
        okf = np.roll(ok, -1, ax)
        okb = np.roll(ok, 1, ax)
        sl = [slice(None)] * t.ndim
        sl[ax] = 0
        okb[tuple(sl)] = False
        sl[ax] = -1
        okf[tuple(sl)] = False
        valid &= okf & okb
        g2 += ((fwd - bwd) / (2 * dr)) ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        v = np.where(valid & (g2 > 0), 1.0 / np.sqrt(g2), np.nan)
    return v


def cv_error_percent(act_a, act_b, dr, mask=None):
    """Difference of the median conduction speeds of two activation maps,
    in percent of the second."""
    va = conduction_velocity(act_a, dr, mask)
    vb = conduction_velocity(act_b, dr, mask)
    both = np.isfinite(va) & np.isfinite(vb)
    if not both.any():
        return None
    ma, mb = float(np.median(va[both])), float(np.median(vb[both]))
    return 100.0 * abs(ma - mb) / mb


def lat_error_steps(count_a, steps_a, count_b, steps_b, mask=None):
    """Local activation times compared crossing by crossing: count_* (N,)
    crossings per node and steps_* (capacity, N) their step indices (the
    device record of LocalActivationTime*Tracker).  Returns (fraction of the
    crossings of b matched by a crossing of a within one step, largest error
    in steps over matched crossings, nodes whose crossing counts differ)."""
    ca = np.asarray(count_a).ravel()
    cb = np.asarray(count_b).ravel()
    sa = np.asarray(steps_a).reshape(-1, ca.size)
    sb = np.asarray(steps_b).reshape(-1, cb.size)
    m = np.ones(ca.size, bool) if mask is None else np.asarray(mask, bool).ravel()
    differ = int((m & (ca != cb)).sum())
    total = int(cb[m].sum())
    k = min(sa.shape[0], sb.shape[0])
    good, worst = 0, 0
    for j in range(k):
        both = m & (ca > j) & (cb > j)
        if not both.any():
            continue
        d = np.abs(sa[j, both].astype(np.int64) - sb[j, both])
        good += int((d <= 1).sum())
        worst = max(worst, int(d.max()))
    return (good / total if total else 1.0), worst, differ
