"""Shared case builders: the golden fixtures as oracle case dicts.

Each function loads one fixture written by tests/golden/make_golden.py and
returns (case, golden) where ``case`` is the input description that both the
oracle and the GPU model classes are driven with.
"""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def ap2d_cfg1():
    g = load("ap2d_cfg1")
    n = 102
    case = dict(model="ap", mesh=g["mesh"], dt=0.01, dr=0.25, t_max=50,
                stencil="iso5",
                stims=[dict(kind="voltage", t=0, value=1.0,
                            box=[(0, n), (1, 6)])],
                trackers=[dict(kind="at", threshold=0.5)])
    return case, g


def ap2d_aniso_spiral():
    g = load("ap2d_aniso_spiral")
    n = 42
    case = dict(model="ap", mesh=g["mesh"], dt=0.01, dr=0.25, t_max=100,
                stencil="aniso9", fibers=g["fibers"], conductivity=g["cond"],
                stims=[dict(kind="voltage", t=0, value=1.0,
                            box=[(0, n), (1, 4)]),
                       dict(kind="voltage", t=22, value=1.0,
                            box=[(n // 2, n), (0, n // 2)])],
                trackers=[dict(kind="at", threshold=0.5),
                          dict(kind="probe", cells=[[5, 5], [20, 30],
                                                    [35, 10]],
                               vars=["u"], step=7),
                          dict(kind="probe", cells=[[10, 12], [30, 30]],
                               vars=["u", "v"], step=3, start_time=10,
                               end_time=60)])
    return case, g


MODEL_VARS = {"ap": ["u", "v"], "ms": ["u", "h"], "fk": ["u", "v", "w"]}


def models_2d(name, aniso):
    g = load("models_2d")
    case = dict(model=name, mesh=g["mesh"], dt=0.01, dr=0.25, t_max=40,
                stencil="aniso9" if aniso else "iso5", fibers=g["fibers"],
                stims=[dict(kind="current", t=0, value=5, duration=1.0,
                            box=[(0, 24), (1, 4)], u_max=1.0),
                       dict(kind="current", t=2.5, value=3, duration=0.5,
                            box=[(8, 14), (8, 14)])],
                trackers=[dict(kind="at", threshold=0.5),
                          dict(kind="probe", cells=[[4, 4], [12, 20]],
                               vars=MODEL_VARS[name], step=5)])
    key = f"{name}_{'aniso' if aniso else 'iso'}"
    gold = {v: g[f"{key}_{v}"] for v in MODEL_VARS[name]}
    gold.update({f"mv_{v}": g[f"{key}_mv_{v}"] for v in MODEL_VARS[name]})
    gold["act_t"] = g[f"{key}_act_t"]
    return case, gold


def ap3d(aniso):
    g = load("ap3d")
    case = dict(model="ap", mesh=g["mesh"], dt=0.01, dr=0.25, t_max=20,
                stencil="aniso19" if aniso else "iso7", fibers=g["fibers"],
                stims=[dict(kind="voltage", t=0, value=1.0,
                            box=[(0, 12), (0, 11), (1, 3)]),
                       dict(kind="current", t=8, value=4, duration=0.6,
                            box=[(6, 12), (0, 6), (0, 10)])],
                trackers=[dict(kind="at", threshold=0.5)])
    key = "aniso" if aniso else "iso"
    return case, {"u": g[key + "_u"], "v": g[key + "_v"],
                  "act_t": g[key + "_act_t"]}


def trackers_cable():
    g = load("trackers")
    mesh = np.pad(np.ones((10, 1), np.int8), 1)
    case = dict(model="ap", mesh=mesh, dt=0.01, dr=0.25, t_max=50,
                stencil="iso5",
                stims=[dict(kind="current", t=0, value=5, duration=0.5,
                            box=[(0, 5), (0, 3)]),
                       dict(kind="voltage", t=45, value=1,
                            box=[(0, 5), (0, 10)])],
                trackers=[dict(kind="lat", threshold=0.5),
                          dict(kind="at", threshold=0.5),
                          dict(kind="at", threshold=-40),
                          dict(kind="at", threshold=0.2, step=4,
                               start_time=1.0, end_time=30.0)])
    return case, g


def stimuli_2d():
    g = load("stimuli")
    case = dict(model="ap", mesh=g["mesh2d"], dt=0.01, dr=0.25, t_max=6,
                stencil="iso5",
                stims=[dict(kind="voltage", t=0, value=0.8, matrix=g["m1"]),
                       dict(kind="current", t=1, value=2.5, duration=0.7,
                            matrix=g["m2"], u_max=0.9),
                       dict(kind="current", t=2.0, value=6.0, duration=0.4,
                            coords=g["area_coords"], u_max=1.2)],
                trackers=[dict(kind="at", threshold=0.5)])
    return case, g


TP06_VARS = ["cai", "casr", "cass", "nai", "Ki", "m", "h", "j", "xr1", "xr2",
             "xs", "r", "s", "d", "f", "f2", "fcass", "rr", "oo"]
CRN_VARS = ["nai", "ki", "cai", "caup", "carel", "m", "h", "j_", "d", "f",
            "oa", "oi", "ua", "ui", "xr", "xs", "fca", "irel", "vrel", "urel",
            "wrel"]
MODEL_VARS["tp06"] = ["u"] + TP06_VARS
MODEL_VARS["crn"] = ["u"] + CRN_VARS


def tp06(dim):
    """TP06 2D (anisotropic, fibrotic) or 3D (isotropic), current S1,
    2000 steps, probes of u, m, cai, nai, Ki, casr every 10 steps."""
    g = load("tp06")
    if dim == 2:
        case = dict(model="tp06", mesh=g["mesh2"], fibers=g["fib2"],
                    stencil="aniso9", dt=0.01, dr=0.25, t_max=20,
                    stims=[dict(kind="current", t=0, value=60, duration=1.0,
                                box=[(0, 10), (0, 3)])],
                    trackers=[dict(kind="probe", cells=[[4, 4]],
                                   vars=["u", "m", "cai", "nai", "Ki", "casr"],
                                   step=10)])
    else:
        case = dict(model="tp06", mesh=g["mesh3"], stencil="iso7", dt=0.01,
                    dr=0.25, t_max=20,
                    stims=[dict(kind="current", t=0, value=100, duration=1.0,
                                box=[(0, 6), (0, 3), (0, 5)])],
                    trackers=[dict(kind="probe", cells=[[3, 3, 2]],
                                   vars=["u", "m", "cai", "nai", "Ki", "casr"],
                                   step=10)])
    gold = {v: g[f"d{dim}_{v}"] for v in MODEL_VARS["tp06"]}
    gold.update({f"mv_{v}": g[f"d{dim}_mv_{v}"]
                 for v in ["u", "m", "cai", "nai", "Ki", "casr"]})
    return case, gold


def courtemanche(dim):
    """Courtemanche 2D (isotropic) or 3D (anisotropic), current S1, 2000
    steps, probes of u, cai, nai, xs, xr, irel every 10 steps."""
    g = load("courtemanche")
    probe = dict(kind="probe", cells=[[4, 4]] if dim == 2 else [[3, 3, 2]],
                 vars=["u", "cai", "nai", "xs", "xr", "irel"], step=10)
    if dim == 2:
        case = dict(model="crn", mesh=g["mesh2"], stencil="iso5", dt=0.01,
                    dr=0.25, t_max=20,
                    stims=[dict(kind="current", t=0, value=80, duration=1.0,
                                box=[(0, 10), (0, 4)])],
                    trackers=[probe])
    else:
        case = dict(model="crn", mesh=g["mesh3"], fibers=g["fib3"],
                    stencil="aniso19", dt=0.01, dr=0.25, t_max=20,
                    stims=[dict(kind="current", t=0, value=80, duration=1.0,
                                box=[(0, 6), (0, 3), (0, 5)])],
                    trackers=[probe])
    gold = {v: g[f"d{dim}_{v}"] for v in MODEL_VARS["crn"]}
    gold.update({f"mv_{v}": g[f"d{dim}_mv_{v}"] for v in probe["vars"]})
    return case, gold


def ecg(dim):
    """ECG trackers: the planar 50 x 5 Aliev-Panfilov cable with two leads
    (2D) or the 14 x 10 x 8 anisotropic slab with three leads (3D)."""
    g = load("ecg")
    if dim == 2:
        mesh = np.ones((50, 5), dtype=np.int8)
        mesh[0, :] = mesh[-1, :] = mesh[:, 0] = mesh[:, -1] = 0
        case = dict(model="ap", mesh=mesh, dt=0.0015, dr=0.25, t_max=15,
                    stencil="iso5",
                    stims=[dict(kind="current", t=5, value=5, duration=0.5,
                                box=[(0, 5), (0, 5)])],
                    trackers=[dict(kind="ecg", step=10,
                                   coords=[[25, 2, 0], [10, -3, 1.5]])])
    else:
        case = dict(model="ap", mesh=g["mesh3"], fibers=g["fib3"],
                    stencil="aniso19", dt=0.01, dr=0.25, t_max=10,
                    D_al=1.0, D_ac=1.0 / 9,
                    stims=[dict(kind="voltage", t=0, value=1.0,
                                box=[(0, 14), (0, 3), (0, 8)])],
                    trackers=[dict(kind="ecg", step=5,
                                   coords=[[7, 12, 4], [-2, 5, 3],
                                           [7, 5, 10.5]])])
    return case, {"ecg": g[f"d{dim}_ecg"], "u": g[f"d{dim}_u"]}


def tips(dim):
    """Spiral tips and periods: Aliev-Panfilov S1-S2 cross field on a 64^2
    sheet (2D) or a 48 x 48 x 3 slab (3D), tips every 20 steps, local
    activation (periods) at a few cells."""
    g = load("tips")
    n = 64 if dim == 2 else 48
    shape = (n, n) if dim == 2 else (n, n, 3)
    mesh = np.ones(shape, dtype=np.int8)
    mesh[0], mesh[-1] = 0, 0
    mesh[:, 0], mesh[:, -1] = 0, 0
    if dim == 3:
        mesh[:, :, 0] = mesh[:, :, -1] = 0
    zb = [] if dim == 2 else [(0, 3)]
    case = dict(model="ap", mesh=mesh, dt=0.01, dr=0.25, t_max=60,
                stencil="iso5" if dim == 2 else "iso7",
                stims=[dict(kind="voltage", t=0, value=1.0,
                            box=[(0, n), (1, 4)] + zb),
                       dict(kind="voltage", t=30, value=1.0,
                            box=[(0, n // 2), (0, n)] + zb)],
                trackers=[dict(kind="tips", threshold=0.5, step=20),
                          dict(kind="lat", threshold=0.5)])
    cells = g[f"d{dim}_cells"]
    lens = g[f"d{dim}_period_len"]
    flat = g[f"d{dim}_periods"]
    periods = np.split(flat, np.cumsum(lens)[:-1]) if len(lens) else []
    return case, {"tips": g[f"d{dim}_tips"], "u": g[f"d{dim}_u"],
                  "cells": cells, "periods": periods}


EXTRA_VARS = {"bk": ["u", "v"], "bo": ["u", "v", "w", "s"],
              "lr91": ["u", "m", "h", "j", "d", "f", "x", "cai"]}
MODEL_VARS.update(EXTRA_VARS)


def models_extra(name, dim):
    """Barkley ('bk'), Bueno-Orovio ('bo') or Luo-Rudy 1991 ('lr91') on the
    20^2 anisotropic fibrotic sheet (2D) or the 8 x 8 x 6 block (3D)."""
    g = load("models_extra")
    cv, cd, t_max, thr, var = {"bk": (5, 0.1, 12, 0.5, "v"),
                               "bo": (5, 0.5, 30, 0.5, "v"),
                               "lr91": (100, 1.0, 20, -20.0, "m")}[name]
    if dim == 2:
        case = dict(model=name, mesh=g["mesh2"], fibers=g["fib2"],
                    stencil="aniso9", dt=0.01, dr=0.25, t_max=t_max,
                    stims=[dict(kind="current", t=0, value=cv, duration=cd,
                                box=[(0, 20), (0, 4)])],
                    trackers=[dict(kind="at", threshold=thr),
                              dict(kind="probe", cells=[[10, 11]],
                                   vars=["u", var], step=5)])
    else:
        case = dict(model=name, mesh=g["mesh3"], stencil="iso7", dt=0.01,
                    dr=0.25, t_max=t_max,
                    stims=[dict(kind="current", t=0, value=cv, duration=cd,
                                box=[(0, 8), (0, 3), (0, 6)])],
                    trackers=[dict(kind="at", threshold=thr),
                              dict(kind="probe", cells=[[4, 5, 3]],
                                   vars=["u", var], step=5)])
    gold = {v: g[f"{name}{dim}_{v}"] for v in EXTRA_VARS[name]}
    gold["act_t"] = g[f"{name}{dim}_act_t"]
    gold.update({f"mv_{v}": g[f"{name}{dim}_mv_{v}"] for v in ["u", var]})
    return case, gold


def detailed_long(name, dim):
    """TP06 ('tp06') or Courtemanche ('crn') on the 10 x 10 anisotropic
    fibrotic sheet (2D) or the 6 x 6 x 5 anisotropic block (3D), current S1
    on the first columns, 10^4 steps (t = 100 ms) through the upstroke into
    the plateau; u at two cells every 100 steps."""
    g = load("detailed_long")
    if dim == 2:
        case = dict(model=name, mesh=g["mesh2"], fibers=g["fib2"],
                    stencil="aniso9", dt=0.01, dr=0.25, t_max=100,
                    stims=[dict(kind="current", t=0, value=80, duration=1.0,
                                box=[(0, 10), (0, 3)])],
                    trackers=[dict(kind="probe", cells=[[4, 4], [7, 6]],
                                   vars=["u"], step=100)])
    else:
        case = dict(model=name, mesh=g["mesh3"], fibers=g["fib3"],
                    stencil="aniso19", dt=0.01, dr=0.25, t_max=100,
                    stims=[dict(kind="current", t=0, value=80, duration=1.0,
                                box=[(0, 6), (0, 3), (0, 5)])],
                    trackers=[dict(kind="probe", cells=[[3, 3, 2], [4, 2, 3]],
                                   vars=["u"], step=100)])
    key = f"{name}{dim}"
    gold = {v: g[f"{key}_{v}"] for v in MODEL_VARS[name]}
    gold["mv_u"] = g[f"{key}_mv_u"]
    gold["step"] = int(g[f"{key}_step"])
    return case, gold
