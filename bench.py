"""Benchmark: Aliev-Panfilov 2D, 4096x4096, anisotropic 9-point stencil.

Workload (the 4096^2 spiral-induction configuration): a CardiacTissue2D of
4096x4096 nodes (boundary ring included), diffuse fibrosis (code 2) with
p = 0.2 drawn as the reference's Diffuse2DPattern draws it
(``1 + (np.random.random(shape) <= p)`` under ``np.random.seed``), fibers at
angle 45 deg * g / max|g| with g a seeded standard-normal field smoothed by
a Gaussian of sigma = 64 nodes, AsymmetricStencil2D with D_al = 1,
D_ac = 0.111, dt = 0.01, dr = 0.25, S1 = StimVoltageCoord2D(0, 1, 0, 4096,
1, 6), S2 = StimVoltageCoord2D(31, 1, 2048, 4096, 0, 2048) and an
activation-time tracker at threshold 0.5.  Inputs are synthetic (seeded);
the reference publishes no dataset for this path.

One bench step = ``--chunk`` time steps (default 100 = 1 ms of model time)
of the whole tissue.  ``value`` is myocyte-steps/s of the float32 form with
all state resident in HBM (state ~ 200 MB, larger than the 129 MB L2, so no
flush is needed between steps); ``e2e`` is the same metric through the
public model API with the state uploaded from pinned host memory and the
potential and activation map read back every bench step.  The float64 plain
form is timed beside it (``fp64_plain``).

``batched``: the many-tissue configuration -- 256 independent 2D tissues
of uneven sizes (side log-uniform in [64, 1024]), models drawn from
Aliev-Panfilov / Mitchell-Schaeffer / Fenton-Karma, isotropic or anisotropic,
fibrosis p uniform in [0, 0.3], S1-S2 protocol, a local activation tracker
each -- advanced together by TissueBatch (one persistent float32 launch per
4 steps over a ragged tile list), next to the same tissues in the float64
plain form.

``tp06_slab``: TP06 on a 512 x 512 x 64 slab (10 % fibrosis, fibers
rotating -60..+60 degrees through the depth, AsymmetricStencil3D, S1-S2,
16 probes), plain form, float32 with float64 ion concentrations next to
float64.

``serving``: a trace of 40 simulation requests (Poisson arrivals at 50/s;
TP06 / Courtemanche; 2D tissues of side 256-2048 and 3D left-ventricle
shells on 128^3-256^3 grids; float32 with float64 concentrations; 20-80 ms
of simulated time each, 1/25 of the configuration's 500-2000 ms, which
``--serving-full`` serves) in real time by SimulationServer under an HBM
budget, the requests' chunks on several streams at once: p50 / p99
latency, queueing and service times, myocyte-steps/s and the overlap of
the requests on the device.

``accuracy_f32_vs_f64``: the float32 forms against the float64 plain form
on the headline 4096^2 S1-S2 workload past the S2 into the re-entry
(t = 200 by default, ``--accuracy-tmax``), on the TP06 slab's generator at
128 x 128 x 16 through one beat (450 ms) and on a TP06 192^2 sheet through
one action potential (350 ms): max |dV|, activation and local-activation
time errors in steps, APD90 error at 16 probes, conduction-velocity error in
percent, and whether the thresholds (activation within one step on 99.9 %
of the myocytes, APD90 within 0.5 ms) hold.

The timed window of the headline starts after an untimed lead-in of 3200
steps (``--lead-in``), so it runs after the S2 (step 3100) with both waves
in the tissue.

``--impl reference`` times the reference's algorithm on the host cores: the
C restatement of its numba kernels (oracle/fw_oracle.c, OpenMP over all
cores, float64, precomputed weights) on the same workload, a bounded number
of steps.

Multi-GPU: the path is replicated, not sharded -- each rank advances its own
copy of the tissue (``scaling: weak``); rank 0 prints the line.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = ("Aliev-Panfilov 2D 4096x4096, AsymmetricStencil2D (D_al 1, "
            "D_ac 0.111), 20% diffuse fibrosis, smooth fibers, S1-S2, "
            "activation tracker")
METRIC = ("node-steps/s: batched FP32 vs plain FP64 GPU at LAT err≤1 "
          "step; p50/p99 latency")
UNIT = "myocyte-steps/s"
N = 4096
SEED = 1234
# algorithmic bytes per myocyte-step (u and v read + written, 1 B mesh code,
# two fiber components at the stencil precision)
B_ALG = {"float32": 2 * (4 + 4) + 1 + 2 * 4, "float64": 2 * (8 + 8) + 1 + 2 * 8}


def workload_inputs(n=N, seed=SEED, sigma=64.0):
    import scipy.ndimage as nd
    np.random.seed(seed)
    mesh = (1 + (np.random.random((n, n)) <= 0.2)).astype(np.int8)
    mesh[0, :] = mesh[-1, :] = mesh[:, 0] = mesh[:, -1] = 0
    g = np.random.default_rng(seed).standard_normal((n, n)).astype(np.float32)
    g = nd.gaussian_filter(g, sigma)
    theta = (np.pi / 4) * g / np.abs(g).max()
    fibers = np.stack([np.cos(theta), np.sin(theta)], -1).astype(np.float64)
    return mesh, fibers


# batched workload: 256 independent 2D tissues (see batched_specs)
N_TISSUES = 256
BCL = {"ap": 60.0, "ms": 1000.0, "fk": 1000.0}
# each model's restitution range [ERP, BCL]: ERP is the shortest S1-S2
# coupling interval after 8 S1 beats at the BCL whose S2 still propagates,
# measured once in float64 by tests/golden/make_restitution.py (written to
# tests/golden/restitution.json, which a CPU test keeps equal to these)
RESTITUTION = {"ap": (25.710938, 60.0), "ms": (317.1875, 1000.0),
               "fk": (165.039062, 1000.0)}
B_ALG_BATCH = {("ap", "iso5"): 17, ("ap", "aniso9"): 25,
               ("ms", "iso5"): 17, ("ms", "aniso9"): 25,
               ("fk", "iso5"): 25, ("fk", "aniso9"): 33}


def batched_specs(n_tissues=N_TISSUES, seed=SEED):
    """The batched configuration: side lengths log-uniform in [64, 1024],
    model uniform over Aliev-Panfilov / Mitchell-Schaeffer / Fenton-Karma,
    isotropic or 9-point anisotropic (smooth random fibers, sigma = side/64
    nodes), diffuse fibrosis with p uniform in [0, 0.3]; S1-S2 protocol: 8
    S1 beats from the left edge at the model's basic cycle length, then an
    S2 on the lower-left quadrant after a coupling interval uniform over the
    model's measured restitution range (RESTITUTION).  Seeded; all
    randomness from default_rng(seed)."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_tissues):
        side = int(round(np.exp(rng.uniform(np.log(64), np.log(1024)))))
        model = ("ap", "ms", "fk")[int(rng.integers(3))]
        aniso = bool(rng.integers(2))
        p = float(rng.uniform(0.0, 0.3))
        lo, hi = RESTITUTION[model]
        ci = float(rng.uniform(lo, hi))
        specs.append(dict(side=side, model=model, aniso=aniso, p=p, ci=ci,
                          seed=int(rng.integers(1 << 31))))
    return specs


def batched_tissue(fg, spec, npfloat):
    import scipy.ndimage as nd
    n = spec["side"]
    r = np.random.default_rng(spec["seed"])
    mesh = (1 + (r.random((n, n)) <= spec["p"])).astype(np.int8)
    mesh[0, :] = mesh[-1, :] = mesh[:, 0] = mesh[:, -1] = 0
    tissue = fg.CardiacTissue2D((n, n))
    tissue.mesh = mesh
    cls = {"ap": fg.AlievPanfilov2D, "ms": fg.MitchellSchaeffer2D,
           "fk": fg.FentonKarma2D}[spec["model"]]
    model = cls()
    if spec["aniso"]:
        g = nd.gaussian_filter(r.standard_normal((n, n)), n / 64.0)
        theta = (np.pi / 4) * g / max(np.abs(g).max(), 1e-30)
        tissue.fibers = np.stack([np.cos(theta), np.sin(theta)], -1)
        st = fg.AsymmetricStencil2D()
        st.D_al, st.D_ac = 1.0, 0.111
        model.stencil = st
    model.dt, model.dr = 0.01, 0.25
    bcl = BCL[spec["model"]]
    model.t_max = 7 * bcl + spec["ci"] + bcl
    model.npfloat = npfloat
    model.cardiac_tissue = tissue
    seq = fg.StimSequence()
    for b in range(8):
        seq.add_stim(fg.StimVoltageCoord2D(b * bcl, 1.0, 0, n, 1, 6))
    seq.add_stim(fg.StimVoltageCoord2D(7 * bcl + spec["ci"], 1.0, n // 2, n,
                                       0, n // 2))
    model.stim_sequence = seq
    lat = fg.LocalActivationTime2DTracker()
    lat.threshold = 0.5
    trs = fg.TrackerSequence()
    trs.add_tracker(lat)
    model.tracker_sequence = trs
    return model


def batched_kernel_rate(args, fg, torch, reps, specs):
    """The batched kernel alone on a subset of the batched configuration's
    tissues: CUDA events over one fw_batch_run of `chunk` steps after a
    warm-up through TissueBatch.run; myocyte-steps/s and the fraction of the
    measured copy bandwidth on the subset's myocyte-weighted algorithmic
    bytes."""
    models = [batched_tissue(fg, s, "float32") for s in specs]
    for m in models:
        m.initialize()
    myo = [int(m._myo_d.sum().item()) for m in models]
    b_alg = sum(B_ALG_BATCH[(s["model"], "aniso9" if s["aniso"] else "iso5")]
                * k for s, k in zip(specs, myo)) / sum(myo)
    batch = fg.TissueBatch(models, kernel=args.batch_kernel)
    for _ in range(max(1, args.warmup)):
        for m in models:
            m.t_max = m.t + args.chunk * m.dt
        batch.run(initialize=False)
    stream = torch.cuda.current_stream()
    times = []
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fg._ffi.call("fw_batch_run", ctypes.byref(batch._batch),
                     batch._scratch.data_ptr(), 0, args.chunk,
                     stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    kms = sorted(times)[1]
    value = reps.whole_job(sum(myo) * args.chunk, kms / 1e3)
    peak, _ = peaks()
    achieved = b_alg * value / reps.world / 1e9
    del batch, models
    torch.cuda.empty_cache()
    return {"tissues": len(specs), "myocytes": sum(myo),
            "kernel_value": value, "unit": UNIT,
            "ms_per_time_step": kms / args.chunk,
            "alg_bytes_per_myocyte_step": b_alg,
            "frac": achieved / peak}


def run_batched(args, fg, torch, reps):
    """Batched float32 throughput through TissueBatch.run (one persistent
    launch per 4 steps over all tissues), the same tissues in the float64
    plain form one after another, and the myocyte-weighted algorithmic
    bytes."""
    specs = batched_specs(args.batched_tissues)
    models = [batched_tissue(fg, s, "float32") for s in specs]
    for m in models:
        m.initialize()
    myo = [int(m._myo_d.sum().item()) for m in models]
    b_alg = sum(B_ALG_BATCH[(s["model"], "aniso9" if s["aniso"] else "iso5")]
                * k for s, k in zip(specs, myo)) / sum(myo)
    batch = fg.TissueBatch(models, kernel=args.batch_kernel)
    chunk = args.chunk

    def advance(steps):
        steps0 = [m.step for m in models]
        for m in models:
            m.t_max = m.t + steps * m.dt
        batch.run(initialize=False)
        return sum(k * (m.step - s0) for k, m, s0 in zip(myo, models, steps0))

    for _ in range(args.warmup):
        advance(chunk)
    reps.barrier()
    L = fg._ffi.load()
    # public API: one TissueBatch.run over k_b bench steps (one plan)
    k_b = max(3, args.steps // 4)
    l0 = L.fw_launch_count()
    t0 = time.perf_counter()
    work = advance(k_b * chunk)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    reps.barrier()
    launches = L.fw_launch_count() - l0
    value = reps.whole_job(work, el)
    el = reps.max(el)
    # the kernel alone: fw_batch_run on the last plan, CUDA events (the
    # models' host-side step counters are not advanced; discarded below)
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    kl0 = L.fw_launch_count()
    e0.record(stream)
    fg._ffi.call("fw_batch_run", ctypes.byref(batch._batch),
                 batch._scratch.data_ptr(), 0, chunk, stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    kms = e0.elapsed_time(e1)
    kl = L.fw_launch_count() - kl0
    kernel_value = reps.whole_job(sum(myo) * chunk, kms / 1e3)
    batch_kernel = batch._batch.kernel
    del batch, models
    torch.cuda.empty_cache()
    # the Aliev-Panfilov tissues of the same configuration on their own
    ap_only = batched_kernel_rate(args, fg, torch, reps,
                                  [s for s in specs if s["model"] == "ap"])

    # the same tissues, float64 plain form, one tissue after the other
    s64 = 20
    work64, t64 = 0, 0.0
    for s in specs:
        m = batched_tissue(fg, s, "float64")
        m.form = "plain"
        m.initialize()
        k = int(m._myo_d.sum().item())
        m._run_segment(s64, sync=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m._run_segment(s64, sync=False)
        torch.cuda.synchronize()
        t64 += time.perf_counter() - t0
        work64 += k * s64
        del m
    torch.cuda.empty_cache()
    peak, _ = peaks()
    achieved = b_alg * kernel_value / reps.world / 1e9   # per GPU
    fp64_value = reps.whole_job(work64, t64)
    return {"value": value, "unit": UNIT, "tissues": len(specs),
            "myocytes": sum(myo), "time_steps_per_bench_step": chunk,
            "bench_steps": k_b, "launches": int(launches),
            "ms_per_step": 1e3 * el / k_b,
            "kernel": {"name": {1: "k_batch", 2: "k_batch_tma",
                                3: "k_batch_tma (column pairs, f32x2)"}
                               [batch_kernel],
                       "value": kernel_value,
                       "ms_per_time_step": kms / chunk,
                       "launches_per_bench_step": int(kl)},
            "fp64_plain": {"value": fp64_value, "unit": UNIT,
                           "time_steps": s64},
            "speedup_fp32_batched_over_fp64_plain": value / fp64_value,
            "aliev_panfilov_only": ap_only,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "alg_bytes_per_myocyte_step": b_alg},
            "timing": "value: wall clock over one TissueBatch.run of "
                      "bench_steps x time_steps_per_bench_step steps (host "
                      "planning included), state resident; kernel: CUDA "
                      "events over fw_batch_run; roofline on the kernel"}


# TP06 slab: 512 x 512 x 64, float32 state with float64 concentrations
SLAB = (512, 512, 64)
# algorithmic bytes per myocyte-step: 15 float32 arrays (u, 13 gates, the
# derived oo) + 5 ion concentrations of 8 bytes (compensated float32 pairs),
# read and written; 1 B mesh code; 3 float32 fiber components
B_ALG_TP06 = 2 * (15 * 4 + 5 * 8) + 1 + 3 * 4


def tp06_slab(fg, npfloat, shape=SLAB, seed=SEED):
    """The TP06 slab configuration: 10 % diffuse fibrosis (seeded
    Diffuse3DPattern), fibers (cos phi, sin phi, 0) with phi linear from -60
    to +60 degrees over the interior layers k, AsymmetricStencil3D with
    D_al = 1, D_ac = 0.25 (D_model 0.154: D_long 0.154, D_trans 0.0385
    mm^2/ms), dr = 0.25 mm, dt = 0.01 ms; S1 current on the first interior
    layers at 0 ms, S2 on a corner quarter at 310 ms; u probed at 16 seeded
    myocytes every 10 steps."""
    ni, nj, nk = shape
    np.random.seed(seed)
    mesh = fg.Diffuse3DPattern(None, None, None, None, None, None,
                               0.1).generate(shape)
    tissue = fg.CardiacTissue3D(shape)
    tissue.mesh = mesh
    phi = np.zeros(nk)
    phi[1:-1] = np.deg2rad(np.linspace(-60.0, 60.0, nk - 2))
    fib = np.zeros(shape + (3,))
    fib[..., 0] = np.cos(phi)[None, None, :]
    fib[..., 1] = np.sin(phi)[None, None, :]
    tissue.fibers = fib
    model = fg.TP063D()
    st = fg.AsymmetricStencil3D()
    st.D_al, st.D_ac = 1.0, 0.25
    model.stencil = st
    model.dt, model.dr = 0.01, 0.25
    model.t_max = 1000.0
    model.npfloat = npfloat
    model.cardiac_tissue = tissue
    seq = fg.StimSequence()
    seq.add_stim(fg.StimCurrentCoord3D(0, 100, 1.0, 0, ni, 0, nj, 1, 4))
    seq.add_stim(fg.StimCurrentCoord3D(310, 100, 1.0, ni // 2, ni, nj // 2,
                                       nj, 1, nk - 1))
    model.stim_sequence = seq
    myo = np.argwhere(np.asarray(tissue.mesh) == 1)
    pick = np.random.default_rng(seed).choice(len(myo), 16, replace=False)
    pr = fg.MultiVariable3DTracker()
    pr.cell_ind = myo[pick].tolist()
    pr.var_list = ["u"]
    pr.step = 10
    trs = fg.TrackerSequence()
    trs.add_tracker(pr)
    model.tracker_sequence = trs
    return model


def run_tp06_slab(args, fg, torch, reps):
    """TP06 slab throughput, float32 (float64 concentrations) and float64,
    plain form, state resident (~3 GB, larger than L2)."""
    chunk = args.chunk
    out = {}
    shape = tuple(args.slab)
    for prec, k in (("float32", max(3, args.steps // 10)),
                    ("float64", 2)):
        m = tp06_slab(fg, prec, shape)
        m.initialize()
        myo = int(m._myo_d.sum().item())
        if prec == "float32":
            st_name = {fg._ffi.ANISO19_XY: "ANISO19_XY",
                       fg._ffi.ANISO19: "ANISO19"}.get(m._step_stencil, "?")
            rows = getattr(m, "_wrows", None)
            w_form = (f"{rows.shape[0]} shared weight rows + a 4-byte row "
                      "index per node" if rows is not None
                      else "weight planes")
        for _ in range(2):
            m._run_segment(chunk, sync=False)
        reps.barrier()
        ms, launches = device_steps(m, chunk, k, torch)
        reps.barrier()
        out[prec] = dict(value=reps.whole_job(myo * chunk * k, ms / 1e3),
                         ms_per_step=reps.max(ms) / k, launches=int(launches),
                         myocytes=myo, bench_steps=k)
        del m
        torch.cuda.empty_cache()
    peak, _ = peaks()
    v32 = out["float32"]["value"]
    achieved = B_ALG_TP06 * v32 / reps.world / 1e9
    return {"value": v32, "unit": UNIT, "grid": list(shape),
            "myocytes": out["float32"]["myocytes"],
            "time_steps_per_bench_step": chunk,
            "ms_per_step": out["float32"]["ms_per_step"],
            "bench_steps": out["float32"]["bench_steps"],
            "launches": out["float32"]["launches"],
            "form": "plain",
            "dtype": "f32 (ion concentrations as compensated f32 pairs)",
            "fp64_plain": {"value": out["float64"]["value"], "unit": UNIT},
            "speedup_fp32_over_fp64": v32 / out["float64"]["value"],
            "weights": w_form,
            "roofline": {"bound": "hbm",
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "alg_bytes_per_myocyte_step": B_ALG_TP06,
                         "kernel": f"k_step<ModelTP06, {st_name}, float>"}}


# serving trace: Poisson arrivals of TP06 / Courtemanche requests
SERVE_RATE = 50.0          # requests per second
SERVE_REQUESTS = 40
SERVE_MS = (20.0, 80.0)    # simulated time per request (ms): 1/25 of the
SERVE_MS_FULL = (500.0, 2000.0)  # configuration's 500-2000 ms


def lv_shell(n, wall, rng):
    """A truncated ellipsoidal shell on an n^3 grid (left-ventricle-like):
    outer semi-axes 0.45 n, 0.45 n, 0.7 n around (n/2, n/2, 0.75 n), wall
    `wall` nodes thick, cut at the centre plane; fibers in the wall's
    tangent plane at an angle rotating linearly from +60 deg (endocardium)
    to -60 deg (epicardium) with the normalised wall depth."""
    c = np.array([n / 2, n / 2, 0.75 * n])
    ax = np.array([0.45 * n, 0.45 * n, 0.7 * n])
    g = np.stack(np.meshgrid(*[np.arange(n) + 0.5] * 3, indexing="ij"), -1) - c
    rho = np.sqrt(((g / ax) ** 2).sum(-1))
    rho_i = np.sqrt(((g / (ax - wall)) ** 2).sum(-1))
    shell = (rho <= 1.0) & (rho_i > 1.0) & (g[..., 2] <= 0)
    mesh = shell.astype(np.int8)
    depth = np.clip((rho_i - 1.0) / np.maximum(rho_i - rho, 1e-9), 0.0, 1.0)
    alpha = np.deg2rad(60.0 - 120.0 * depth)
    normal = g / ax ** 2
    normal /= np.maximum(np.linalg.norm(normal, axis=-1, keepdims=True), 1e-12)
    e_c = np.cross(np.array([0.0, 0.0, 1.0]), g)
    nc = np.linalg.norm(e_c, axis=-1, keepdims=True)
    e_c = np.where(nc > 1e-9, e_c / np.maximum(nc, 1e-12),
                   np.array([1.0, 0.0, 0.0]))
    e_l = np.cross(normal, e_c)
    e_l /= np.maximum(np.linalg.norm(e_l, axis=-1, keepdims=True), 1e-12)
    fib = np.cos(alpha)[..., None] * e_c + np.sin(alpha)[..., None] * e_l
    del rng
    return mesh, fib


def serving_trace(fg, n_requests=SERVE_REQUESTS, seed=SEED, ms=SERVE_MS):
    """The serving configuration: Poisson arrivals at 50 requests/s; 70 % 2D
    tissues with side U[256, 2048], 30 % 3D left-ventricle shells on
    128^3..256^3 grids (wall 8-16 nodes, fibers rotating +-60 deg
    transmurally); model TP06 or Courtemanche; simulated time per request
    uniform in `ms` (by default 20-80 ms, 1/25 of the configuration's
    500-2000 ms, so that the trace is served in seconds; ``--serving-full``
    serves the configuration's own durations); float32 state with float64
    concentrations; a current stimulus at t = 0 and an activation-time
    tracker (threshold -20 mV)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / SERVE_RATE)
        tp06 = bool(rng.integers(2))
        dur = float(rng.uniform(*ms))
        if rng.random() < 0.7:
            side = int(rng.integers(256, 2049))
            tissue = fg.CardiacTissue2D((side, side))
            model = fg.TP062D() if tp06 else fg.Courtemanche2D()
            stim = fg.StimCurrentCoord2D(0, 100, 1.0, 0, side, 1, 6)
        else:
            n = int(rng.integers(128, 257))
            wall = int(rng.integers(8, 17))
            mesh, fib = lv_shell(n, wall, rng)
            tissue = fg.CardiacTissue3D((n, n, n))
            tissue.mesh = mesh
            tissue.fibers = fib
            model = fg.TP063D() if tp06 else fg.Courtemanche3D()
            st = fg.AsymmetricStencil3D()
            st.D_al, st.D_ac = 1.0, 0.25
            model.stencil = st
            zs = np.flatnonzero(mesh.any(axis=(0, 1)))
            z0 = int(zs[0]) if zs.size else 1
            stim = fg.StimCurrentCoord3D(0, 100, 1.0, 0, n, 0, n, z0, z0 + 4)
        model.dt, model.dr, model.t_max = 0.01, 0.25, dur
        model.npfloat = "float32"
        model.cardiac_tissue = tissue
        seq = fg.StimSequence()
        seq.add_stim(stim)
        model.stim_sequence = seq
        at = fg.ActivationTime2DTracker()
        at.threshold = -20.0
        trs = fg.TrackerSequence()
        trs.add_tracker(at)
        model.tracker_sequence = trs
        reqs.append(fg.Request(model, arrival=t, name=f"r{i}"))
    return reqs


def run_serving(args, fg, torch, reps):
    """The serving trace through SimulationServer in real time."""
    ms = SERVE_MS_FULL if args.serving_full else SERVE_MS
    reqs = serving_trace(fg, args.serving_requests, ms=ms)
    server = fg.SimulationServer(chunk=args.serving_chunk)
    server.serve(reqs, realtime=True)
    torch.cuda.synchronize()
    st = server.stats()
    n2 = sum(isinstance(r.model.cardiac_tissue, fg.CardiacTissue2D)
             for r in reqs)
    st.update({"unit": UNIT, "requests": len(reqs), "requests_2d": n2,
               "arrival_rate_per_s": SERVE_RATE,
               "simulated_ms_per_request": list(ms),
               "chunk_steps": args.serving_chunk,
               "value_note": "myocyte-steps of the completed requests / "
                             "(last finish - first arrival)"})
    if reps.world > 1:
        st["value"] = reps.whole_job(st["myocyte_steps"], st["makespan_s"])
    return st


def _accuracy_pair(fg, build, probes_at):
    """Run one configuration in float64 (plain) and float32 (default form)
    and compare them with finitewave_gb300.metrics."""
    from finitewave_gb300 import metrics
    import torch
    out = {}
    runs = {}
    for prec in ("float64", "float32"):
        model, at, lat, pr = build(prec)
        t0 = time.perf_counter()
        model.run()
        torch.cuda.synchronize()
        runs[prec] = dict(u=model.u.astype(np.float64), at=at.act_t,
                          lat_count=lat._count.cpu().numpy(),
                          lat_steps=lat._steps.cpu().numpy(),
                          probes=np.asarray(pr.output["u"], np.float64),
                          seconds=time.perf_counter() - t0,
                          dt=model.dt, dr=model.dr,
                          myo=model._myo_d.cpu().numpy().astype(bool),
                          form=("fused" if model._form() == 1 else "plain"))
        del model
        torch.cuda.empty_cache()
    a, b = runs["float32"], runs["float64"]
    myo = b["myo"]
    within, worst, one = metrics.activation_error_steps(a["at"], b["at"],
                                                        b["dt"], myo)
    lw, lworst, ldiff = metrics.lat_error_steps(
        a["lat_count"], a["lat_steps"], b["lat_count"], b["lat_steps"], myo)
    apd_a = [metrics.apd90(a["probes"][:, c], b["dt"])
             for c in range(b["probes"].shape[1])]
    apd_b = [metrics.apd90(b["probes"][:, c], b["dt"])
             for c in range(b["probes"].shape[1])]
    d_apd = [abs(x - y) for x, y in zip(apd_a, apd_b)
             if x is not None and y is not None]
    out.update({
        "max_abs_dV_field": float(np.abs(a["u"] - b["u"])[myo].max()),
        "max_abs_dV_probes": float(np.abs(a["probes"] - b["probes"]).max()),
        "at_within_1_step": within, "at_max_err_steps": worst,
        "at_nodes_activated_in_one_only": one,
        "lat_within_1_step": lw, "lat_max_err_steps": lworst,
        "lat_nodes_count_differs": ldiff,
        "apd90_max_err": max(d_apd) if d_apd else None,
        "apd90_probes": len(d_apd),
        "cv_err_percent": metrics.cv_error_percent(a["at"], b["at"], b["dr"],
                                                   myo),
        "form_f32": a["form"],
        "seconds": {"float64": b["seconds"], "float32": a["seconds"]}})
    return out


def accuracy_ap(fg, n=N, t_max=200.0):
    """Aliev-Panfilov 2D n x n with the headline configuration's generator
    (fibrosis 0.2, fibers smoothed with sigma = n / 64), S1 at t = 0 and S2
    on the lower-left quadrant at t = 31, to t_max (past the S2 into the
    re-entry it induces); activation, local activation (every crossing) and
    u at 16 seeded myocytes every step."""
    mesh, fibers = workload_inputs(n, sigma=n / 64.0)

    def build(prec):
        model, at = build_model(fg, mesh, fibers, prec, None, init=False)
        model.t_max = t_max
        lat = fg.LocalActivationTime2DTracker()
        lat.threshold, lat.capacity = 0.5, int(t_max // 20) + 4
        model.tracker_sequence.add_tracker(lat)
        pr = fg.MultiVariable2DTracker()
        cells = np.argwhere(mesh == 1)
        pr.cell_ind = cells[np.random.default_rng(SEED).choice(
            len(cells), 16, replace=False)].tolist()
        pr.var_list = ["u"]
        model.tracker_sequence.add_tracker(pr)
        return model, at, lat, pr
    return build


def accuracy_tp06(fg, n=192, t_max=350.0):
    """TP06 2D n x n, 10 % fibrosis, smooth fibers, S1 from the left edge,
    to t_max (one full action potential)."""
    import scipy.ndimage as nd
    rng = np.random.default_rng(SEED)
    mesh = (1 + (rng.random((n, n)) <= 0.1)).astype(np.int8)
    g = nd.gaussian_filter(rng.standard_normal((n, n)), n / 32.0)
    theta = (np.pi / 4) * g / np.abs(g).max()
    fibers = np.stack([np.cos(theta), np.sin(theta)], -1)
    interior = np.zeros((n, n), bool)
    interior[1:-1, 1:-1] = True
    cells = np.argwhere((mesh == 1) & interior)
    probe_cells = cells[rng.choice(len(cells), 16, replace=False)].tolist()

    def build(prec):
        tissue = fg.CardiacTissue2D((n, n))
        tissue.mesh = mesh.copy()
        tissue.fibers = fibers
        model = fg.TP062D()
        st = fg.AsymmetricStencil2D()
        st.D_al, st.D_ac = 1.0, 0.25
        model.stencil = st
        model.dt, model.dr, model.t_max = 0.01, 0.25, t_max
        model.npfloat = prec
        model.cardiac_tissue = tissue
        seq = fg.StimSequence()
        seq.add_stim(fg.StimCurrentCoord2D(0, 100, 1.0, 0, n, 1, 6))
        model.stim_sequence = seq
        at = fg.ActivationTime2DTracker()
        at.threshold = -20.0
        lat = fg.LocalActivationTime2DTracker()
        lat.threshold, lat.capacity = -20.0, 4
        pr = fg.MultiVariable2DTracker()
        pr.cell_ind = probe_cells
        pr.var_list = ["u"]
        trs = fg.TrackerSequence()
        for t in (at, lat, pr):
            trs.add_tracker(t)
        model.tracker_sequence = trs
        return model, at, lat, pr
    return build


def accuracy_slab(fg, shape=(128, 128, 16), t_max=450.0):
    """The TP06 slab configuration's generator (10 % fibrosis, fibers
    rotating -60..+60 degrees through the depth, AsymmetricStencil3D) at a
    reduced lateral size, through one beat: the S1 on the first interior
    layers at 0 ms and no S2, to t_max; activation and local activation at
    -20 mV and u at the generator's 16 seeded probe myocytes every step."""

    def build(prec):
        model = tp06_slab(fg, prec, shape)
        model.t_max = t_max
        model.stim_sequence.sequence = model.stim_sequence.sequence[:1]
        pr = model.tracker_sequence.sequence[0]
        pr.step = 1
        at = fg.ActivationTime3DTracker()
        at.threshold = -20.0
        lat = fg.LocalActivationTime3DTracker()
        lat.threshold, lat.capacity = -20.0, 4
        model.tracker_sequence.add_tracker(at)
        model.tracker_sequence.add_tracker(lat)
        return model, at, lat, pr
    return build


# spec accuracy thresholds of the float32 forms against float64
ACC_AT_FRACTION = 0.999     # activation within one step on this fraction
ACC_APD90_MS = 0.5          # APD90 error (ms; model time units for AP)


def _verdict(r):
    """Whether an accuracy record meets the thresholds."""
    ok = r["at_within_1_step"] >= ACC_AT_FRACTION
    if "lat_within_1_step" in r:
        ok &= r["lat_within_1_step"] >= ACC_AT_FRACTION
    if r.get("apd90_max_err") is not None:
        ok &= r["apd90_max_err"] <= ACC_APD90_MS
    return bool(ok)


def accuracy_batched(fg, torch, n_tissues=16, steps=2000):
    """Local activation times of the batched float32 form (TissueBatch, one
    persistent launch over all tissues) against each tissue's float64 plain
    run: the first n_tissues tissues of the batched configuration, `steps`
    time steps of their S1-S2 protocol."""
    from finitewave_gb300 import metrics
    specs = batched_specs()[:n_tissues]
    runs = {}
    for prec in ("float32", "float64"):
        models = [batched_tissue(fg, s, prec) for s in specs]
        for m in models:
            m.t_max = steps * m.dt
        if prec == "float32":
            fg.TissueBatch(models).run()
        else:
            for m in models:
                m.form = "plain"
                m.run()
        torch.cuda.synchronize()
        runs[prec] = [(m.tracker_sequence.sequence[0], m) for m in models]
    good = total = worst = differ = 0
    for (l32, m32), (l64, m64) in zip(runs["float32"], runs["float64"]):
        myo = m64._myo_d.cpu().numpy().astype(bool).ravel()
        c64 = l64._count.cpu().numpy()
        w, wk, d = metrics.lat_error_steps(
            l32._count.cpu().numpy(), l32._steps.cpu().numpy(), c64,
            l64._steps.cpu().numpy(), myo)
        n = int(c64[myo].sum())
        good += w * n
        total += n
        worst = max(worst, wk)
        differ += d
    return {"tissues": len(specs), "time_steps": steps,
            "lat_crossings": total,
            "lat_within_1_step": good / total if total else 1.0,
            "lat_max_err_steps": worst, "lat_nodes_count_differs": differ}


def run_accuracy(args, fg, torch, reps):
    """Float32 against float64 on three configurations: max |dV|, activation
    and local activation time errors in steps, APD90 error at 16 probes,
    conduction-velocity error in percent; and the batched form's local
    activation times against the float64 plain form."""
    out = {"cfg2_4096": dict(
               grid=[args.grid, args.grid], t_max=args.accuracy_tmax,
               units="normalised u; time in model units",
               **_accuracy_pair(fg, accuracy_ap(fg, args.grid,
                                                args.accuracy_tmax), None)),
           "cfg3_slab": dict(
               grid=list(args.accuracy_slab), t_max=450.0, units="mV; ms",
               note="the 512x512x64 slab's generator at %dx%dx%d, S1 only "
                    "(one beat); float64 of the full slab for one beat is "
                    "~45 min of GPU time" % tuple(args.accuracy_slab),
               **_accuracy_pair(fg, accuracy_slab(
                   fg, tuple(args.accuracy_slab)), None)),
           "tp06_2d_192": dict(
               units="mV; ms",
               **_accuracy_pair(fg, accuracy_tp06(fg), None)),
           "batched_16_tissues": accuracy_batched(fg, torch)}
    for k in ("cfg2_4096", "cfg3_slab", "tp06_2d_192"):
        out[k]["meets_thresholds"] = _verdict(out[k])
    out["thresholds"] = {"at_within_1_step_fraction": ACC_AT_FRACTION,
                         "apd90_max_err_ms": ACC_APD90_MS}
    return out


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=10)
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, f[2:]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_model(fg, mesh, fibers, npfloat, form, init=True):
    n = mesh.shape[0]
    tissue = fg.CardiacTissue2D(mesh.shape)
    tissue.mesh = mesh.copy()
    tissue.fibers = fibers
    model = fg.AlievPanfilov2D()
    model.dt, model.dr = 0.01, 0.25
    model.t_max = 1000.0
    model.npfloat = npfloat
    model.form = form
    st = fg.AsymmetricStencil2D()
    st.D_al, st.D_ac = 1.0, 0.111
    model.stencil = st
    model.cardiac_tissue = tissue
    seq = fg.StimSequence()
    seq.add_stim(fg.StimVoltageCoord2D(0, 1.0, 0, n, 1, 6))
    seq.add_stim(fg.StimVoltageCoord2D(31, 1.0, n // 2, n, 0, n // 2))
    model.stim_sequence = seq
    at = fg.ActivationTime2DTracker()
    at.threshold = 0.5
    trs = fg.TrackerSequence()
    trs.add_tracker(at)
    model.tracker_sequence = trs
    if init:
        model.initialize()
    return model, at


def device_steps(model, chunk, iters, torch):
    """Advance iters x chunk steps through fw_step with no host sync;
    returns (elapsed ms by CUDA events, library launches)."""
    from finitewave_gb300 import _ffi
    L = _ffi.load()
    stream = torch.cuda.current_stream()
    l0 = L.fw_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(iters):
        model._run_segment(chunk, sync=False)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), L.fw_launch_count() - l0


class Replicas:
    """The N > 1 path: one process per GPU, each advancing its own replica
    of the workload with no data exchange (the path is not sharded); the
    only collectives are the barriers around timed regions and the maximum
    of the per-rank times.  Whole-job throughput = world x per-rank units /
    max time.  `backend` / `device` are "nccl" / "cuda" on GPUs and "gloo" /
    "cpu" in the host-only tests."""

    def __init__(self, backend="nccl", device="cuda"):
        import torch
        import torch.distributed as dist
        self.torch, self.dist = torch, dist
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.device = device
        self.owned = False
        if self.world > 1 and not dist.is_initialized():
            dist.init_process_group(backend)
            self.owned = True

    def barrier(self):
        if self.device == "cuda":
            self.torch.cuda.synchronize()
        if self.world > 1:
            self.dist.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        t = self.torch.tensor([float(x)], dtype=self.torch.float64,
                              device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def whole_job(self, units_per_rank, seconds_per_rank):
        """Units all ranks processed / the slowest rank's time."""
        return self.world * units_per_rank / self.max(seconds_per_rank)

    def close(self):
        if self.owned:
            self.dist.destroy_process_group()
            self.owned = False


def run_gb300(args):
    import torch

    reps = Replicas("nccl", "cuda")
    world, rank, local = reps.world, reps.rank, reps.local
    torch.cuda.set_device(local)
    import finitewave_gb300 as fg
    from finitewave_gb300 import _ffi
    _ffi.load()

    if args.only in ("tp06", "batched", "serving", "accuracy"):
        # one sub-measurement alone (profiling runs); not the bench line
        fn = {"tp06": run_tp06_slab, "batched": run_batched,
              "serving": run_serving, "accuracy": run_accuracy}[args.only]
        r = fn(args, fg, torch, reps)
        if rank == 0:
            print(json.dumps({"only": args.only, **r}), flush=True)
        reps.close()
        return

    mesh, fibers = workload_inputs(args.grid)
    myo = int((mesh == 1).sum())
    chunk, K, W = args.chunk, args.steps, args.warmup
    form32 = args.form
    barrier, max_over_ranks = reps.barrier, reps.max

    # --- float32 form, state resident -------------------------------------
    model, at = build_model(fg, mesh, fibers, "float32", form32)
    model.fused_k = args.fused_k
    model.fused_variant = args.fused_variant
    # lead-in past the S2 (t = 31), so that the timed steps run the
    # induced re-entry with both waves in the tissue
    lead = args.lead_in
    while lead > 0:
        lead -= model._run_segment(min(lead, 1000), sync=False)
    for _ in range(W):
        model._run_segment(chunk, sync=False)
    barrier()
    with Clocks(local) as clk:
        ms, launches = device_steps(model, chunk, K, torch)
    barrier()
    ms = max_over_ranks(ms)
    ms_per_step = ms / K
    value = world * myo * chunk * K / (ms / 1e3)

    # dominant-kernel timing: launches of one segment averaged
    kms, kl = device_steps(model, chunk, 3, torch)
    choice = getattr(model, "_fused_choice", None)
    kernel_name = ("k_step" if choice is None else
                   "k_fused_tma" if choice[0] == 3 else "k_fused")
    steps_per_launch = (3 * chunk) / max(1, kl)
    per_launch_s = (kms / 1e3) / max(1, kl)
    alg_bytes = B_ALG["float32"] * myo * steps_per_launch
    achieved = alg_bytes / per_launch_s / 1e9
    peak, peak_kind = peaks()
    if args.kernel_only:
        if rank == 0:
            print(json.dumps({"kernel_only": True, "grid": args.grid,
                              "fused_k": args.fused_k,
                              "fused_variant": args.fused_variant,
                              "value": value, "ms_per_step": ms_per_step,
                              "achieved_gbs": achieved,
                              "frac": achieved / peak,
                              "launches": int(launches)}), flush=True)
        return

    # --- e2e through the public API, host buffers ----------------------------
    u_h = torch.empty(mesh.shape, dtype=torch.float32).pin_memory()
    v_h = torch.empty(mesh.shape, dtype=torch.float32).pin_memory()
    u_h.copy_(model._dev["u"].cpu())
    v_h.copy_(model._dev["v"].cpu())
    u_out = torch.empty_like(u_h).pin_memory()
    act_out = torch.empty(mesh.shape, dtype=torch.int32).pin_memory()
    h2d = u_h.numel() * 4 * 2
    d2h = u_out.numel() * 4 + act_out.numel() * 4

    def e2e_step():
        # public API: upload the state, run `chunk` more steps, read back
        model._dev["u"].copy_(u_h, non_blocking=True)
        model._dev["v"].copy_(v_h, non_blocking=True)
        s0 = model.step
        model.t_max = model.t + chunk * model.dt
        model.run(initialize=False)
        u_out.copy_(model._dev["u"], non_blocking=True)
        act_out.copy_(at._act_step, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return model.step - s0

    for _ in range(max(1, W // 2)):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    e2e_steps = 0
    for _ in range(K):
        e2e_steps += e2e_step()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = world * myo * e2e_steps / e2e_s
    del model, at
    torch.cuda.empty_cache()

    # --- float64 plain form, same workload ----------------------------------
    m64, _ = build_model(fg, mesh, fibers, "float64", "plain")
    lead = args.lead_in
    while lead > 0:
        lead -= m64._run_segment(min(lead, 1000), sync=False)
    for _ in range(max(1, W // 2)):
        m64._run_segment(chunk, sync=False)
    barrier()
    k64 = max(3, K // 20)
    ms64, _ = device_steps(m64, chunk, k64, torch)
    ms64 = max_over_ranks(ms64)
    fp64_value = world * myo * chunk * k64 / (ms64 / 1e3)
    del m64
    torch.cuda.empty_cache()

    batched = None
    if not args.no_batched:
        batched = run_batched(args, fg, torch, reps)

    tp06 = None
    if not args.no_tp06:
        tp06 = run_tp06_slab(args, fg, torch, reps)

    accuracy = None
    if not args.no_accuracy:
        accuracy = run_accuracy(args, fg, torch, reps)

    serving = None
    if not args.no_serving:
        serving = run_serving(args, fg, torch, reps)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(mesh, fibers, args.cpu_seconds)
    clocks = clk.summary()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": K, "warmup": W, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded fibrosis and fibers)",
            "config": {
                "workload": WORKLOAD,
                "grid": [N, N], "myocytes": myo,
                "time_steps_per_bench_step": chunk, "form": form32 or "auto",
                "timed_from_step": args.lead_in + W * chunk,
                "l2": "state larger than L2 (no flush needed)",
                "parallelism": f"replicas x{world}"},
            "fp64_plain": {"value": fp64_value, "unit": UNIT,
                           "speedup_fp32_over_fp64": value / fp64_value},
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_kind,
                         "traffic": traffic_from_profiles(
                             myo, steps_per_launch, choice),
                         "kernel": kernel_name,
                         "fused_variant_k": list(choice) if choice else None,
                         "alg_bytes_per_myocyte_step": B_ALG["float32"],
                         "time_steps_per_launch": steps_per_launch},
            "batched": batched,
            "tp06_slab": tp06,
            "serving": serving,
            "accuracy_f32_vs_f64": accuracy,
            "cpu_baseline": cpu,
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    reps.close()


def traffic_from_profiles(myo, steps_per_launch, choice):
    """DRAM bytes per launch of the fused kernel `choice` = (variant, K)
    from the committed ncu summaries, scaled to this workload, or None when
    no capture of that kernel is present."""
    p = os.path.join(ROOT, "profiles", "traffic.json.txt")
    if not os.path.exists(p) or not choice:
        return None
    try:
        with open(p) as f:
            table = json.loads(f.read())
        for d in table.values():
            if (d["variant"], d["k"]) == tuple(choice):
                return d["dram_bytes_per_myocyte_step"] * myo * \
                    steps_per_launch
    except (ValueError, KeyError, TypeError):
        pass
    return None


def cpu_baseline(mesh, fibers, seconds):
    """The oracle's C kernels (OpenMP, all host cores, float64) on the same
    workload for a bounded number of steps."""
    from oracle import oracle
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    w = oracle.weights("aniso9", mesh, 1.0, 0.01, 0.25, 1.0, fibers, 1.0,
                       0.111)
    idx = np.flatnonzero(mesh == 1).astype(np.int64)
    u = np.zeros(mesh.shape)
    u[:, 1:6][mesh[:, 1:6] == 1] = 1.0
    un = np.zeros(mesh.shape)
    v = np.zeros(mesh.shape)
    p = oracle.MODELS["ap"]["params"]

    def step():
        nonlocal u, un
        oracle._diffuse("aniso9", un, u, w, idx)
        oracle._ionic("ap", {"v": v}, un, u, idx, 0.01, p)
        u, un = un, u

    # warm-up: up to 100 steps (or a tenth of the time budget)
    t0 = time.perf_counter()
    for _ in range(100):
        step()
        if time.perf_counter() - t0 >= 0.1 * seconds:
            break
    # timed window: up to 1000 steps within the time budget
    steps = 0
    t0 = time.perf_counter()
    while True:
        step()
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 1000:
            break
    return {"value": idx.size * steps / el, "unit": UNIT, "cores": cores,
            "kind": "port",
            "sample": f"{steps} float64 steps of the 4096^2 workload after a "
                      f"warm-up (diffusion + ionic, OpenMP x{cores}), "
                      f"{el:.1f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh, fibers = workload_inputs()
    per = None
    for _ in range(args.warmup + args.steps):
        per = cpu_baseline(mesh, fibers, args.cpu_seconds / max(1, args.steps))
    cpu = per
    line = {
        "metric": METRIC, "value": cpu["value"], "unit": UNIT,
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
        "warmup": args.warmup,
        # one bench step (args.chunk time steps of the whole grid) at the
        # rate the bounded sample measured
        "ms_per_step": (int((mesh == 1).sum()) * args.chunk / cpu["value"] * 1e3
                        if cpu and cpu.get("value") else None),
        "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded fibrosis and fibers)",
        "config": {"workload": WORKLOAD, "grid": [N, N],
                   "myocytes": int((mesh == 1).sum()),
                   "time_steps_per_bench_step": args.chunk,
                   "form": "float64 CPU restatement (OpenMP)",
                   "parallelism": "rank 0 host cores"},
        "impl": "reference",
        "cpu_baseline": cpu,
        "e2e": {"value": cpu["value"], "unit": UNIT,
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--chunk", type=int, default=100)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default=None, choices=[None, "plain", "fused"])
    ap.add_argument("--fused-k", type=int, default=0)
    ap.add_argument("--fused-variant", type=int, default=0)
    ap.add_argument("--grid", type=int, default=N,
                    help="grid side (profiling runs use a smaller one)")
    ap.add_argument("--kernel-only", action="store_true",
                    help="time only the float32 form (profiling)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched many-tissue measurement")
    ap.add_argument("--batched-tissues", type=int, default=N_TISSUES)
    ap.add_argument("--batch-kernel", default="tma",
                    choices=["tma", "pairs", "cp.async"])
    ap.add_argument("--no-tp06", action="store_true",
                    help="skip the TP06 slab measurement")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the float32 vs float64 accuracy runs")
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the serving trace")
    ap.add_argument("--accuracy-tmax", type=float, default=200.0,
                    help="model time of the 4096^2 float32-vs-float64 run")
    ap.add_argument("--accuracy-slab", type=int, nargs=3,
                    default=(128, 128, 16),
                    help="grid of the TP06 slab float32-vs-float64 run")
    ap.add_argument("--lead-in", type=int, default=3200,
                    help="untimed time steps before the warm-up: the timed "
                         "window starts after the S2 (step 3100)")
    ap.add_argument("--serving-requests", type=int, default=SERVE_REQUESTS)
    ap.add_argument("--serving-chunk", type=int, default=500)
    ap.add_argument("--serving-full", action="store_true",
                    help="serve the configuration's 500-2000 ms per request")
    ap.add_argument("--only", default=None,
                    choices=[None, "tp06", "batched", "serving",
                             "accuracy"],
                    help="run one sub-measurement alone (profiling)")
    ap.add_argument("--slab", type=int, nargs=3, default=list(SLAB),
                    help="TP06 slab shape (profiling runs use a smaller one)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
