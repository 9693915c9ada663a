"""CPU oracle for the monodomain step -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module; the library never does.

It wraps ``fw_oracle.c`` (a C restatement of the reference's numba kernels,
built here with gcc into ``oracle/_build/``) and restates the reference's run
loop ``CardiacModel.run`` (``core/model/cardiac_model.py:130-189``) with the
reference's stimulus and tracker semantics in numpy:

* stimuli: ``StimSequence.stimulate_next`` (``core/stimulation/
  stim_sequence.py:65-77``) with ``Stim.update_status`` (``stim.py:52-56``);
  coordinate boxes use numpy slice semantics (``stim_voltage_coord_2d.py:
  49-67``, ``stim_current_coord_2d.py:60-85``), matrices ``matrix > 0 &
  mesh == 1`` (``stim_voltage_matrix_2d.py``, ``stim_current_matrix_2d.py``),
  areas a coordinate list (``stim_current_area_2d.py:44-94``);
* trackers: ``Tracker.track`` gating (``core/tracker/tracker.py:70-83``),
  activation time (``activation_time_2d_tracker.py:51-63``), local
  activation time (``local_activation_time_2d_tracker.py:58-89``) and
  per-cell probes (``action_potential_2d_tracker.py:46-53``,
  ``multi_variable_2d_tracker.py:58-69``).

Cases are plain dicts so that the oracle shares no code with the library.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfworacle.so")
SRC = os.path.join(HERE, "fw_oracle.c")

CFLAGS = ["-O2", "-fno-fast-math", "-ffp-contract=off", "-fopenmp",
          "-fPIC", "-shared", "-std=c99"]


def build(force=False):
    """Compile fw_oracle.c (gcc, OpenMP) into oracle/_build/libfworacle.so."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [SRC] + [os.path.join(HERE, f) for f in sorted(os.listdir(HERE))
                    if f.startswith("fw_oracle_") and f.endswith(".c")]
    if (not force and os.path.exists(LIB) and
            all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc"] + CFLAGS + srcs + ["-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None
_P = ctypes.c_void_p
_I = ctypes.c_int64
_D = ctypes.c_double


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        sig = {
            "fwo_set_threads": [ctypes.c_int],
            "fwo_weights_2d_iso5": [_P, _P, _I, _I, _D, _D, _D, _P],
            "fwo_weights_3d_iso7": [_P, _P, _I, _I, _I, _D, _D, _D, _P],
            "fwo_weights_2d_aniso9": [_P, _P, _P, _I, _I, _D, _D, _D, _D, _D,
                                      _P],
            "fwo_weights_3d_aniso19": [_P, _P, _P, _I, _I, _I, _D, _D, _D, _D,
                                       _D, _P],
            "fwo_diffuse_2d_iso5": [_P, _P, _P, _P, _I, _I, _I],
            "fwo_diffuse_2d_aniso9": [_P, _P, _P, _P, _I, _I, _I],
            "fwo_diffuse_3d_iso7": [_P, _P, _P, _P, _I, _I, _I, _I],
            "fwo_diffuse_3d_aniso19": [_P, _P, _P, _P, _I, _I, _I, _I],
            "fwo_ionic_ap": [_P, _P, _P, _P, _I] + [_D] * 6,
            "fwo_ionic_ms": [_P, _P, _P, _P, _I] + [_D] * 6,
            "fwo_ionic_fk": [_P, _P, _P, _P, _P, _I] + [_D] * 12,
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int if name == "fwo_set_threads" else None
        for extra in ("fwo_ionic_tp06", "fwo_ionic_crn"):
            if hasattr(L, extra):
                getattr(L, extra).restype = None
        _lib = L
    return _lib


def set_threads(n):
    return lib().fwo_set_threads(int(n))


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


# ------------------------------------------------------------------ weights

def weights(kind, mesh, D_model, dt, dr, conductivity=1.0, fibers=None,
            D_al=1.0, D_ac=1.0 / 9):
    """Stencil weights in the reference layout (*mesh.shape, nw), float64.

    kind: 'iso5' | 'aniso9' | 'iso7' | 'aniso19'.
    """
    mesh = np.ascontiguousarray(mesh, dtype=np.int8)
    cond = np.ascontiguousarray(conductivity * np.ones(mesh.shape))
    L = lib()
    if kind == "iso5":
        w = np.zeros((*mesh.shape, 5))
        L.fwo_weights_2d_iso5(_p(mesh), _p(cond), *mesh.shape, D_model, dt,
                              dr ** 2, _p(w))
    elif kind == "iso7":
        w = np.zeros((*mesh.shape, 7))
        L.fwo_weights_3d_iso7(_p(mesh), _p(cond), *mesh.shape, D_model, dt,
                              dr ** 2, _p(w))
    elif kind == "aniso9":
        f = np.ascontiguousarray(fibers, dtype=np.float64)
        w = np.zeros((*mesh.shape, 9))
        L.fwo_weights_2d_aniso9(_p(mesh), _p(cond), _p(f), *mesh.shape,
                                D_al, D_ac, D_model, dt, dr ** 2, _p(w))
    elif kind == "aniso19":
        f = np.ascontiguousarray(fibers, dtype=np.float64)
        w = np.zeros((*mesh.shape, 19))
        L.fwo_weights_3d_aniso19(_p(mesh), _p(cond), _p(f), *mesh.shape,
                                 D_al, D_ac, D_model, dt, dr ** 2, _p(w))
    else:
        raise ValueError(kind)
    return w


# ------------------------------------------------------------------ models

# Parameter defaults and state initial values of the reference's model
# classes (aliev_panfilov_2d.py:278-299, mitchell_schaeffer_2d.py:47-65,
# fenton_karma_2d.py:80-102).
MODELS = {
    "ap": dict(params=dict(a=0.1, k=8.0, eap=0.01, mu_1=0.2, mu_2=0.3),
               init=dict(u=0.0, v=0.0), D_model=1.0, reset_u_new=False),
    "ms": dict(params=dict(tau_close=150.0, tau_open=120.0, tau_in=0.3,
                           tau_out=6.0, u_gate=0.13),
               init=dict(u=0.0, h=1.0), D_model=1.0, reset_u_new=False),
    "fk": dict(params=dict(tau_d=0.172, tau_o=12.5, tau_r=130.0,
                           tau_si=127.0, tau_v_m=18.2, tau_v_p=10.0,
                           tau_w_m=80.0, tau_w_p=1020.0, k=10.0, u_c=0.13,
                           uc_si=0.85),
               init=dict(u=0.0, v=1.0, w=1.0), D_model=1.0,
               reset_u_new=False),
}


def register_model(name, spec):
    MODELS[name] = spec


def _ionic(model, st, un, u, idx, dt, p):
    L = lib()
    n = idx.size
    if model == "ap":
        L.fwo_ionic_ap(_p(un), _p(u), _p(st["v"]), _p(idx), n, dt, p["a"],
                       p["k"], p["eap"], p["mu_1"], p["mu_2"])
    elif model == "ms":
        L.fwo_ionic_ms(_p(un), _p(u), _p(st["h"]), _p(idx), n, dt,
                       p["tau_close"], p["tau_open"], p["tau_in"],
                       p["tau_out"], p["u_gate"])
    elif model == "fk":
        L.fwo_ionic_fk(_p(un), _p(u), _p(st["v"]), _p(st["w"]), _p(idx), n,
                       dt, p["tau_d"], p["tau_o"], p["tau_r"], p["tau_si"],
                       p["tau_v_m"], p["tau_v_p"], p["tau_w_m"], p["tau_w_p"],
                       p["k"], p["u_c"], p["uc_si"])
    else:
        MODELS[model]["ionic"](L, un, u, st, idx, dt, p)


def _diffuse(kind, un, u, w, idx):
    L = lib()
    if kind in ("iso5", "aniso9"):
        fn = getattr(L, "fwo_diffuse_2d_" + kind)
    else:
        fn = getattr(L, "fwo_diffuse_3d_" + kind)
    fn(_p(un), _p(u), _p(w), _p(idx), idx.size, *u.shape)


# ------------------------------------------------------------------ run

def _box_mask(shape, box):
    m = np.zeros(shape, dtype=bool)
    m[tuple(slice(lo, hi) for lo, hi in box)] = True
    return m


def _stim_mask(stim, mesh):
    if "box" in stim:
        sl = tuple(slice(lo, hi) for lo, hi in stim["box"])
        m = np.zeros(mesh.shape, dtype=bool)
        m[sl] = mesh[sl] == 1
        return m
    if "matrix" in stim:
        return (stim["matrix"] > 0) & (mesh == 1)
    if "coords" in stim:
        c = np.asarray(stim["coords"])
        keep = mesh[tuple(c.T)] == 1
        m = np.zeros(mesh.shape, dtype=bool)
        m[tuple(c[keep].T)] = True
        return m
    raise ValueError(stim)


def run(case):
    """Run one case through the restated reference loop.

    case keys: model, mesh, dt, dr, t_max, stencil ('iso5'...), fibers,
    conductivity, D_al, D_ac, D_model (optional), params (overrides),
    stims (list of dicts: kind 'voltage'|'current', t, value, duration,
    u_max, and one of box / matrix / coords), trackers (list of dicts:
    kind 'at'|'lat'|'probe', threshold, start_time, end_time, step,
    cells, vars), special (optional special_boundaries array),
    init (optional overrides of initial values).
    Returns dict with state arrays, u_new, t, step and tracker outputs.
    """
    spec = MODELS[case["model"]]
    mesh = np.ascontiguousarray(case["mesh"], dtype=np.int8)
    dt, dr, t_max = case["dt"], case["dr"], case["t_max"]
    D_model = case.get("D_model", spec["D_model"])
    kind = case["stencil"]
    w = weights(kind, mesh, D_model, dt, dr, case.get("conductivity", 1.0),
                case.get("fibers"), case.get("D_al", 1.0),
                case.get("D_ac", 1.0 / 9))
    special = case.get("special")
    myo = (mesh == 1) if special is None else (mesh == 1) & (special == 0)
    idx = np.flatnonzero(myo).astype(np.int64)
    params = dict(spec["params"])
    params.update(case.get("params", {}))
    init = dict(spec["init"])
    init.update(case.get("init", {}))
    u = init["u"] * np.ones(mesh.shape)
    u_new = u.copy() if spec["reset_u_new"] else np.zeros(mesh.shape)
    st = {k: init[k] * np.ones(mesh.shape) for k in init if k != "u"}

    stims = [dict(s, passed=False, mask=_stim_mask(s, mesh))
             for s in case.get("stims", [])]
    trackers = []
    for tr in case.get("trackers", []):
        tr = dict(tr)
        tr.setdefault("start_time", 0)
        tr.setdefault("end_time", np.inf)
        tr.setdefault("step", 1)
        if tr["kind"] == "at":
            tr["act_t"] = -np.ones(mesh.shape)
        elif tr["kind"] == "lat":
            tr["act_t"] = [-np.ones(mesh.shape)]
            tr["activated"] = np.zeros(mesh.shape, dtype=bool)
        elif tr["kind"] == "probe":
            tr["samples"] = {v: [] for v in tr["vars"]}
        trackers.append(tr)

    t = 0
    step = 0
    iters = int(np.ceil((t_max - t) / dt))
    for _ in range(iters):
        for s in stims:
            if t >= s["t"] and not s["passed"]:
                if s["kind"] == "voltage":
                    u[s["mask"]] = s["value"]
                else:
                    u[s["mask"]] += dt * s["value"]
                    if s.get("u_max") is not None:
                        u[s["mask"]] = np.where(u[s["mask"]] > s["u_max"],
                                                s["u_max"], u[s["mask"]])
                s["passed"] = t >= (s["t"] + s.get("duration", 0.0))
        _diffuse(kind, u_new, u, w, idx)
        _ionic(case["model"], st, u_new, u, idx, dt, params)
        for tr in trackers:
            if tr["start_time"] > t or t > tr["end_time"]:
                continue
            if step % tr["step"] != 0:
                continue
            if tr["kind"] == "at":
                tr["act_t"] = np.where((tr["act_t"] < 0) &
                                       (u > tr["threshold"]), t, tr["act_t"])
            elif tr["kind"] == "lat":
                cross = (u >= tr["threshold"]) & (~tr["activated"])
                tr["activated"] = np.where(cross, True, tr["activated"])
                back = (u < tr["threshold"]) & tr["activated"]
                tr["activated"] = np.where(back, False, tr["activated"])
                if np.any(tr["act_t"][-1][cross] > -1):
                    tr["act_t"].append(-np.ones(mesh.shape))
                tr["act_t"][-1] = np.where(cross, t, tr["act_t"][-1])
            elif tr["kind"] == "probe":
                ci = tuple(np.atleast_2d(tr["cells"]).T)
                for var in tr["vars"]:
                    arr = u if var == "u" else st[var]
                    tr["samples"][var].append(arr[ci].copy())
        t += dt
        step += 1
        u_new, u = u, u_new
        max_iters = int(np.ceil(t_max / dt))
        if t > t_max or step > max_iters:
            break

    out = {"u": u, "u_new": u_new, "t": t, "step": step}
    out.update(st)
    outs = []
    for tr in trackers:
        if tr["kind"] == "at":
            outs.append(tr["act_t"])
        elif tr["kind"] == "lat":
            outs.append(np.array(tr["act_t"]))
        else:
            outs.append({v: np.squeeze(tr["samples"][v])
                         for v in tr["vars"]})
    out["trackers"] = outs
    return out


def step_count(t_max, dt, t0=0):
    """Number of loop iterations the reference runs (cardiac_model.py:161,
    186-203)."""
    t, step = t0, 0
    iters = int(math.ceil((t_max - t) / dt))
    for _ in range(iters):
        t += dt
        step += 1
        if t > t_max or step > int(math.ceil(t_max / dt)):
            break
    return step
