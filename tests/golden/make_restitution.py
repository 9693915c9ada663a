"""Measure each phenomenological model's restitution range with the float64
oracle and write ``restitution.json`` beside this script.

The batched configuration (256 tissues, Aliev-Panfilov / Mitchell-Schaeffer /
Fenton-Karma) paces every tissue with 8 S1 beats at the model's basic cycle
length (BCL) and then gives an S2 after a coupling interval drawn uniformly
from the model's restitution range.  The reference defines neither
quantity; the BCLs are the intervals its model tests pace at
(``tests/test_models_2d.py:122,168,192``: 60 model time units for
Aliev-Panfilov, 1000 ms for Mitchell-Schaeffer and Fenton-Karma), and the
range is measured here once: [ERP, BCL], ERP the shortest S1-S2 coupling
interval whose S2 still propagates.

Protocol (float64, the reference's explicit scheme through the oracle's C
kernels, dt = 0.01, dr = 0.25, the model's default parameters and
D_model, the isotropic 5-point stencil): a strand of 3 x 116 myocytes inside
the 1-node boundary ring; S1 = voltage stimulus u = 1 on columns 1..5
(``StimVoltageCoord2D``, ``stim_voltage_coord_2d.py:49-67``) at t = b BCL,
b = 0..7; S2 = the same stimulus at t = 7 BCL + CI.  The S2 propagates when
the probe node (row 2, column 100) crosses u >= 0.5 (the local activation
tracker's test, ``local_activation_time_2d_tracker.py:82-83``) a ninth time
-- once per S1 beat and once for the S2 -- within three of the first beat's
travel times to it after the S2.  ERP is bisected
over CI in [0.05, 1] BCL to 1/256 of that interval; the recorded ERP is the
shortest tested interval that propagated.

Test infrastructure: run in the build container (CPU only), a few minutes
per model with one process per model (the oracle's kernels on one thread
each).  ``bench.py`` carries the resulting
ranges as constants; ``tests/test_host.py`` checks that they match
``restitution.json``.
"""
import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

BCL = {"ap": 60.0, "ms": 1000.0, "fk": 1000.0}
DT, DR = 0.01, 0.25
SHAPE = (5, 118)
PROBE = (2, 100)
THRESHOLD = 0.5


def _setup(model):
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    O.set_threads(1)   # a 348-myocyte strand: one thread per process
    spec = O.MODELS[model]
    mesh = np.zeros(SHAPE, dtype=np.int8)
    mesh[1:-1, 1:-1] = 1
    w = O.weights("iso5", mesh, spec["D_model"], DT, DR)
    idx = np.flatnonzero(mesh == 1).astype(np.int64)
    box = np.zeros(SHAPE, dtype=bool)
    box[:, 1:6] = True
    box &= mesh == 1
    return O, spec, w, idx, box


def _pace(model, ci, stop_after=None):
    """Run 8 S1 beats and an S2 at coupling interval ci (None: no S2).
    Returns the probe's crossing times (u >= 0.5 after being below)."""
    O, spec, w, idx, box = _setup(model)
    bcl = BCL[model]
    times = [b * bcl for b in range(8)]
    if ci is not None:
        times.append(7 * bcl + ci)
    init = spec["init"]
    u = init["u"] * np.ones(SHAPE)
    u_new = u.copy() if spec["reset_u_new"] else np.zeros(SHAPE)
    st = {k: init[k] * np.ones(SHAPE) for k in init if k != "u"}
    params = dict(spec["params"])
    t_end = stop_after if stop_after is not None else times[-1] + bcl
    passed = [False] * len(times)
    crossings, above = [], False
    t, n = 0.0, 0
    iters = int(np.ceil(t_end / DT))
    for _ in range(iters):
        for i, ts in enumerate(times):
            if t >= ts and not passed[i]:
                u[box] = 1.0
                passed[i] = True
        O._diffuse("iso5", u_new, u, w, idx)
        O._ionic(model, st, u_new, u, idx, DT, params)
        x = u[PROBE]
        if x >= THRESHOLD and not above:
            crossings.append(t)
        above = x >= THRESHOLD
        t += DT
        n += 1
        u_new, u = u, u_new
    return crossings


def measure(model):
    bcl = BCL[model]
    first = _pace(model, None, stop_after=bcl)
    assert first, f"{model}: the S1 wave does not reach the probe"
    travel = first[0]

    def propagates(ci):
        t_s2 = 7 * bcl + ci
        c = _pace(model, ci, stop_after=t_s2 + 3 * travel)
        return len(c) >= 9

    lo, hi = 0.05 * bcl, bcl
    assert propagates(hi), f"{model}: an S2 one BCL after the last S1 fails"
    if propagates(lo):
        return dict(bcl=bcl, erp=lo, travel_to_probe=travel, note="lower end")
    for _ in range(8):
        mid = 0.5 * (lo + hi)
        if propagates(mid):
            hi = mid
        else:
            lo = mid
    return dict(bcl=bcl, erp=hi, erp_fails_below=lo, travel_to_probe=travel)


def main():
    models = sorted(BCL)
    with mp.get_context("spawn").Pool(len(models)) as pool:
        res = dict(zip(models, pool.map(measure, models)))
    out = {"protocol": "8 S1 at BCL + S2 at CI on columns 1..5 of a 3 x 116 "
                       "strand (dt 0.01, dr 0.25, iso5, float64 oracle); "
                       "propagation: probe (2, 100) crosses u >= 0.5 a "
                       "ninth time; ERP bisected over [0.05, 1] BCL",
           "models": {m: {k: round(v, 6) if isinstance(v, float) else v
                          for k, v in r.items()} for m, r in res.items()}}
    with open(os.path.join(HERE, "restitution.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
