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
            "fwo_weights_2d_sym9": [_P, _P, _P, _I, _I, _D, _D, _D, _D, _D,
                                    _P],
            "fwo_diffuse_2d_iso5": [_P, _P, _P, _P, _I, _I, _I],
            "fwo_diffuse_2d_aniso9": [_P, _P, _P, _P, _I, _I, _I],
            "fwo_diffuse_3d_iso7": [_P, _P, _P, _P, _I, _I, _I, _I],
            "fwo_diffuse_3d_aniso19": [_P, _P, _P, _P, _I, _I, _I, _I],
            "fwo_ionic_ap": [_P, _P, _P, _P, _I] + [_D] * 6,
            "fwo_ionic_ms": [_P, _P, _P, _P, _I] + [_D] * 6,
            "fwo_ionic_fk": [_P, _P, _P, _P, _P, _I] + [_D] * 12,
            "fwo_ecg": [_P, _P, _P, _I, _D, _P, _I, _I, _I, ctypes.c_int,
                        _P],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int if name == "fwo_set_threads" else None
        for extra in ("fwo_ionic_tp06", "fwo_ionic_crn", "fwo_ionic_bk",
                      "fwo_ionic_bo", "fwo_ionic_lr91"):
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

    kind: 'iso5' | 'aniso9' | 'iso7' | 'aniso19' | 'sym9' (SymmetricStencil2D,
    stepped with the 9-point diffusion).
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
    elif kind == "sym9":
        f = np.ascontiguousarray(fibers, dtype=np.float64)
        w = np.zeros((*mesh.shape, 9))
        L.fwo_weights_2d_sym9(_p(mesh), _p(cond), _p(f), *mesh.shape,
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


def _tips_2d(u, u_new, threshold):
    """_track_tip_line (spiral_wave_core_2d_tracker.py:152-249) restated in
    numpy: cells (i, j), 5 <= i < ni - 5, 5 <= j < nj - 5, crossed by the
    isoline in both u and u_new, refined by _correct_tip_pos; returns
    [x, y] rows in the reference's raster order."""
    ni, nj = u.shape

    def crosses(a):
        c = a[5:ni - 5, 5:nj - 5]
        d1, d2, d3 = (a[6:ni - 4, 5:nj - 5], a[5:ni - 5, 6:nj - 4],
                      a[6:ni - 4, 6:nj - 4])
        up = (c >= threshold) & ((d1 < threshold) | (d2 < threshold) |
                                 (d3 < threshold))
        dn = (c < threshold) & ((d1 >= threshold) | (d2 >= threshold) |
                                (d3 >= threshold))
        return up | dn
    cand = crosses(u) & crosses(u_new)
    ii, jj = np.nonzero(cand)
    ii, jj = ii + 5, jj + 5
    with np.errstate(divide="ignore", invalid="ignore"):
        AC = u[ii, jj] - u[ii, jj + 1] + u[ii + 1, jj + 1] - u[ii + 1, jj]
        GC = u[ii, jj + 1] - u[ii, jj]
        BC = u[ii + 1, jj] - u[ii, jj]
        DC = u[ii, jj] - threshold
        AD = (u_new[ii, jj] - u_new[ii, jj + 1] + u_new[ii + 1, jj + 1] -
              u_new[ii + 1, jj])
        GD = u_new[ii, jj + 1] - u_new[ii, jj]
        BD = u_new[ii + 1, jj] - u_new[ii, jj]
        DD = u_new[ii, jj] - threshold
        Q = BC * AD - BD * AC
        R = GC * AD - GD * AC
        S = DC * AD - DD * AC
        QOnR = Q / R
        SOnR = S / R
        T = AC * QOnR
        U = AC * SOnR - BC + GC * QOnR
        V = GC * SOnR - DC
        disc = U * U - 4. * T * V
        T2 = 2. * T
        sq = np.sqrt(np.where(disc < 0, 0.0, disc))
        xn = (-U - sq) / T2
        xp = (-U + sq) / T2
        yn = -QOnR * xn - SOnR
        yp = -QOnR * xp - SOnR
    ok = (disc >= 0) & (T2 != 0.)
    n_in = (0 <= xn) & (xn <= 1) & (0 <= yn) & (yn <= 1)
    p_in = (0 <= xp) & (xp <= 1) & (0 <= yp) & (yp <= 1)
    cx = np.where(n_in, xn, xp)
    cy = np.where(n_in, yn, yp)
    keep = ok & (n_in | p_in)
    return np.stack([jj[keep] + cy[keep], ii[keep] + cx[keep]], axis=1)


def _ecg(u_tr, u, coords, dr, idx, shape):
    out = np.zeros(len(coords))
    nk = shape[2] if len(shape) == 3 else 1
    lib().fwo_ecg(_p(u_tr), _p(u), _p(coords), len(coords), dr, _p(idx),
                  idx.size, shape[1], nk, len(shape), _p(out))
    return out


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
    kind 'at'|'lat'|'probe'|'ecg'|'tips', threshold, start_time, end_time, step,
    cells, vars), special (optional special_boundaries array),
    init (optional overrides of initial values).
    Returns dict with state arrays, u_new, t, step and tracker outputs.
    """
    spec = MODELS[case["model"]]
    mesh = np.ascontiguousarray(case["mesh"], dtype=np.int8)
    dt, dr, t_max = case["dt"], case["dr"], case["t_max"]
    D_model = case.get("D_model", spec["D_model"])
    wkind = case["stencil"]
    kind = "aniso9" if wkind == "sym9" else wkind
    w = weights(wkind, mesh, D_model, dt, dr, case.get("conductivity", 1.0),
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
        elif tr["kind"] == "ecg":
            tr["coords"] = np.ascontiguousarray(
                np.atleast_2d(tr["coords"]), dtype=np.float64)
            tr["u_tr"] = np.zeros(mesh.shape)
            tr["samples"] = []
        elif tr["kind"] == "tips":
            # SpiralWaveCore*Tracker copies model.u at initialisation, while
            # it is still zero (cardiac_model.py:96-108)
            tr["u_prev"] = np.zeros(mesh.shape)
            tr["rows"] = []
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
            elif tr["kind"] == "tips":
                if u.ndim == 2:
                    layers = [(-1, tr["u_prev"], u)]
                else:
                    layers = [(k, tr["u_prev"][:, :, k], u[:, :, k])
                              for k in range(u.shape[2])]
                for k, up, uc in layers:
                    for x, y in _tips_2d(up, uc, tr["threshold"]):
                        tr["rows"].append((x, y, k, t, step))
                tr["u_prev"] = u.copy()
            elif tr["kind"] == "ecg":
                # ECG2DTracker.calc_ecg (ecg_2d_tracker.py:61-79)
                _diffuse(kind, tr["u_tr"], u, w, idx)
                tr["samples"].append(_ecg(tr["u_tr"], u, tr["coords"], dr,
                                          idx, mesh.shape))
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
        elif tr["kind"] == "ecg":
            outs.append(np.array(tr["samples"]))
        elif tr["kind"] == "tips":
            outs.append(np.array(tr["rows"], dtype=np.float64).reshape(-1, 5))
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


# ------------------------------------------------------------------ detailed
# Parameters in the reference kernels' argument order and initial values
# (tp06_2d.py:81-170 with the signature at :1003-1012; courtemanche_2d.py:
# 122-178 with the signature at :569-577).

TP06_PARAMS = dict(
    ko=5.4, cao=2.0, nao=140.0, Vc=0.016404, Vsr=0.001094, Vss=0.00005468,
    Bufc=0.2, Kbufc=0.001, Bufsr=10.0, Kbufsr=0.3, Bufss=0.4,
    Kbufss=0.00025, Vmaxup=0.006375, Kup=0.00025, Vrel=0.102, k1_=0.15,
    k2_=0.045, k3=0.060, k4=0.005, EC=1.5, maxsr=2.5, minsr=1.0,
    Vleak=0.00036, Vxfer=0.0038, R=8314.472, F=96485.3415, T=310.0,
    RTONF=26.71376, CAPACITANCE=0.185, gkr=0.153, pKNa=0.03, gk1=5.405,
    gna=14.838, gbna=0.00029, KmK=1.0, KmNa=40.0, knak=2.724,
    gcal=0.00003980, gbca=0.000592, knaca=1000, KmNai=87.5, KmCa=1.38,
    ksat=0.1, n_=0.35, gpca=0.1238, KpCa=0.0005, gpk=0.0146, gto=0.294,
    gks=0.392)
TP06_STATE = ["cai", "casr", "cass", "nai", "Ki", "m", "h", "j", "xr1",
              "xr2", "xs", "r", "s", "d", "f", "f2", "fcass", "rr", "oo"]
TP06_INIT = dict(u=-84.5, cai=0.00007, casr=1.3, cass=0.00007, nai=7.67,
                 Ki=138.3, m=0.0, h=0.75, j=0.75, xr1=0.0, xr2=1.0, xs=0.0,
                 r=0.0, s=1.0, d=0.0, f=1.0, f2=1.0, fcass=1.0, rr=1.0,
                 oo=0.0)

_vc = 20100
_vj = _vc * 0.68
CRN_PARAMS = dict(
    gna=7.8, gnab=0.000674, gk1=0.09, gkr=0.0294, gks=0.129, gto=0.1652,
    gcal=0.1238, gcab=0.00113, gkur_coeff=1, F=96485.0, T=310.0, R=8314.0,
    Vc=_vc, Vj=_vj, Vup=_vj * 0.06 * 0.92, Vrel=_vj * 0.06 * 0.08, ibk=0.0,
    cao=1.8, nao=140, ko=5.4, caupmax=15, kup=0.00092, kmnai=10, kmko=1.5,
    kmnancx=87.5, kmcancx=1.38, ksatncx=0.1, kmcmdn=0.00238,
    kmtrpn=0.0005, kmcsqn=0.8, trpnmax=0.07, cmdnmax=0.05, csqnmax=10.0,
    inacamax=1600, inakmax=0.6, ipcamax=0.275, krel=30, iupmax=0.005,
    kq10=3)
CRN_STATE = ["nai", "ki", "cai", "caup", "carel", "m", "h", "j_", "d", "f",
             "oa", "oi", "ua", "ui", "xr", "xs", "fca", "irel", "vrel",
             "urel", "wrel"]
CRN_INIT = dict(u=-84.5, nai=11.2, ki=139, cai=0.000102, caup=1.6,
                carel=1.1, m=0.00291, h=0.965, j_=0.978, d=0.000137,
                f=0.999837, oa=0.000592, oi=0.9992, ua=0.003519, ui=0.9987,
                xs=0.0187, xr=3.29e-05, fca=0.775, irel=0, vrel=1, urel=0,
                wrel=0.9)


def _detailed_ionic(fn_name, names):
    def ionic(L, un, u, st, idx, dt, p):
        ptrs = (ctypes.c_void_p * len(names))(
            *[st[n].ctypes.data for n in names])
        par = (ctypes.c_double * len(p))(*p.values())
        fn = getattr(L, fn_name)
        fn.argtypes = [_P, _P, _P, _P, _I, _D, _P]
        fn(_p(un), _p(u), ptrs, _p(idx), idx.size, dt, par)
    return ionic


register_model("tp06", dict(params=TP06_PARAMS,
                            init={k: TP06_INIT[k] for k in ["u"] + TP06_STATE},
                            D_model=0.154, reset_u_new=True,
                            ionic=_detailed_ionic("fwo_ionic_tp06",
                                                  TP06_STATE)))
register_model("crn", dict(params=CRN_PARAMS,
                           init={k: CRN_INIT[k] for k in ["u"] + CRN_STATE},
                           D_model=0.154, reset_u_new=True,
                           ionic=_detailed_ionic("fwo_ionic_crn", CRN_STATE)))


# Barkley, Bueno-Orovio, Luo-Rudy 1991 (barkley_2d.py:56-75,
# bueno_orovio_2d.py:93-137, luo_rudy91_2d.py:59-103; parameters in the
# order of their ionic_kernel_2d signatures)
BK_PARAMS = dict(a=0.75, b=0.02, eap=0.02)
BO_PARAMS = dict(
    u_o=0.0, u_u=1.55, theta_v=0.3, theta_w=0.13, theta_v_m=0.006,
    theta_o=0.006, tau_v1_m=60, tau_v2_m=1150, tau_v_p=1.4506, tau_w1_m=60,
    tau_w2_m=15, k_w_m=65, u_w_m=0.03, tau_w_p=200, tau_fi=0.11, tau_o1=400,
    tau_o2=6, tau_so1=30.0181, tau_so2=0.9957, k_so=2.0458, u_so=0.65,
    tau_s1=2.7342, tau_s2=16, k_s=2.0994, u_s=0.9087, tau_si=1.8875,
    tau_w_inf=0.07, w_inf_=0.94)
LR91_PARAMS = dict(
    gna=23.0, gsi=0.09, gk=0.282, gk1=0.6047, gkp=0.0183, gb=0.03921,
    ko=5.4, ki=145.0, nai=18.0, nao=140.0, cao=1.8, R=8.314, T=310.0,
    F=96.5, PR_NaK=0.01833)
LR91_STATE = ["m", "h", "j", "d", "f", "x", "cai"]
register_model("bk", dict(params=BK_PARAMS, init=dict(u=0.0, v=0.0),
                          D_model=1.0, reset_u_new=False,
                          ionic=_detailed_ionic("fwo_ionic_bk", ["v"])))
register_model("bo", dict(params=BO_PARAMS,
                          init=dict(u=0.0, v=1.0, w=1.0, s=0.0),
                          D_model=1.0, reset_u_new=False,
                          ionic=_detailed_ionic("fwo_ionic_bo",
                                                ["v", "w", "s"])))
register_model("lr91", dict(params=LR91_PARAMS,
                            init=dict(u=-84.5, m=0.0017, h=0.9832,
                                      j=0.995484, d=0.000003, f=1.0,
                                      x=0.0057, cai=0.0002),
                            D_model=0.1, reset_u_new=True,
                            ionic=_detailed_ionic("fwo_ionic_lr91",
                                                  LR91_STATE)))
