"""Generate the golden fixtures under tests/golden/ from the reference itself.

This script imports the unmodified Finitewave package (pure Python + numba)
from a reference checkout and runs it in the mode its own CI uses
(``NUMBA_DISABLE_JIT=1``, `.github/workflows/test.yml:17-18`): numba's
``njit`` becomes the identity and ``prange`` becomes ``range``, so the
reference's own float64 source runs as plain Python.  numba and the
visualisation-only dependencies (matplotlib, pandas, natsort, ffmpeg,
pyvista, scikit-image) are absent from this container, so tiny stub modules
are written to a temporary directory and put first on ``sys.path``.  None of
the stubbed modules is used by the hot path (stencils, ionic kernels,
stimuli, activation/probe trackers).

Each case stores its inputs (mesh, fibers, conductivity, parameters) and the
reference's outputs in one compressed ``.npz``, so the tests never need the
reference at run time.

Usage::

    python tests/golden/make_golden.py --reference /path/to/Finitewave [case ...]

Nothing in this file is imported by the library, the tests or the benchmark.
"""
import argparse
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_STUBS = {
    "numba/__init__.py": (
        "def njit(*args, **kwargs):\n"
        "    if len(args) == 1 and callable(args[0]) and not kwargs:\n"
        "        return args[0]\n"
        "    return lambda f: f\n"
        "jit = njit\n"
        "prange = range\n"
        "def set_num_threads(n):\n"
        "    pass\n"
        "class config:\n"
        "    NUMBA_NUM_THREADS = 1\n"
        "from . import typed\n"
    ),
    "numba/typed.py": "List = list\n",
    "matplotlib/__init__.py": "",
    "matplotlib/pyplot.py": "",
    "matplotlib/animation.py": "",
    "pandas/__init__.py": "class DataFrame:\n    pass\n",
    "natsort/__init__.py": "natsorted = sorted\n",
    "ffmpeg/__init__.py": "",
    "pyvista/__init__.py": "",
    "skimage/__init__.py": "from . import measure\n",
    "skimage/measure.py": "",
}


def import_reference(ref_path):
    stub_dir = tempfile.mkdtemp(prefix="fw_stubs_")
    for rel, src in _STUBS.items():
        p = os.path.join(stub_dir, rel)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            f.write(src)
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_path)
    sys.path.insert(0, stub_dir)
    import finitewave as fw  # noqa: E402
    return fw


def _seeded_fibers_2d(rng, shape):
    ang = rng.uniform(-np.pi, np.pi, size=shape)
    return np.stack([np.cos(ang), np.sin(ang)], axis=-1)


def _seeded_fibers_3d(rng, shape):
    v = rng.standard_normal(size=(*shape, 3))
    v /= np.linalg.norm(v, axis=-1, keepdims=True)
    return v


def _fibrosis(rng, shape, p):
    """Bernoulli(p) fibrosis (code 2) with the boundary ring already zeroed,
    so the stored mesh equals tissue.mesh after the reference's
    add_boundaries (cardiac_tissue_2d.py:35-45, cardiac_tissue_3d.py:34-46).
    """
    m = np.where(rng.random(shape) < p, 2, 1).astype(np.int8)
    for ax in range(m.ndim):
        idx = [slice(None)] * m.ndim
        idx[ax] = 0
        m[tuple(idx)] = 0
        idx[ax] = -1
        m[tuple(idx)] = 0
    return m


class _Model:
    """Minimal stand-in for the model attributes a stencil reads."""

    def __init__(self, D_model, dt, dr, npfloat="float64"):
        self.D_model = D_model
        self.dt = dt
        self.dr = dr
        self.npfloat = npfloat


# ---------------------------------------------------------------- weights

def case_weights_2d(fw):
    rng = np.random.default_rng(101)
    shape = (14, 12)
    tissue = fw.CardiacTissue2D(shape)
    mesh = _fibrosis(rng, shape, 0.25)
    mesh[3, 4] = 0
    tissue.mesh = mesh
    cond = rng.uniform(0.3, 1.0, size=shape)
    fibers = _seeded_fibers_2d(rng, shape)
    model = _Model(1.3, 0.01, 0.25)
    out = {"mesh": tissue.mesh.copy(), "cond": cond, "fibers": fibers,
           "D_model": model.D_model, "dt": model.dt, "dr": model.dr}
    tissue.conductivity = 1.0
    out["w_iso5_c1"] = fw.IsotropicStencil2D().compute_weights(model, tissue)
    tissue.conductivity = cond
    out["w_iso5_carr"] = fw.IsotropicStencil2D().compute_weights(model, tissue)
    tissue.fibers = fibers
    st = fw.AsymmetricStencil2D()
    out["w_aniso9_carr"] = st.compute_weights(model, tissue)
    tissue.conductivity = 1.0
    st = fw.AsymmetricStencil2D()
    st.D_al, st.D_ac = 1.0, 0.111
    out["w_aniso9_c1_dac0111"] = st.compute_weights(model, tissue)
    out["D_al_b"], out["D_ac_b"] = 1.0, 0.111
    # SymmetricStencil2D (symmetric_stencil_2d.py:31-250)
    st_sym = fw.SymmetricStencil2D()
    st_sym.D_al, st_sym.D_ac = 1.0, 0.111
    out["w_sym9_c1_dac0111"] = st_sym.compute_weights(model, tissue)
    tissue.conductivity = cond
    out["w_sym9_carr"] = fw.SymmetricStencil2D().compute_weights(model, tissue)
    return out


def case_weights_3d(fw):
    rng = np.random.default_rng(202)
    shape = (9, 8, 7)
    tissue = fw.CardiacTissue3D(shape)
    tissue.mesh = _fibrosis(rng, shape, 0.2)
    cond = rng.uniform(0.3, 1.0, size=shape)
    fibers = _seeded_fibers_3d(rng, shape)
    model = _Model(0.154, 0.01, 0.25)
    out = {"mesh": tissue.mesh.copy(), "cond": cond, "fibers": fibers,
           "D_model": model.D_model, "dt": model.dt, "dr": model.dr}
    tissue.conductivity = 1.0
    out["w_iso7_c1"] = fw.IsotropicStencil3D().compute_weights(model, tissue)
    tissue.conductivity = cond
    out["w_iso7_carr"] = fw.IsotropicStencil3D().compute_weights(model, tissue)
    tissue.fibers = fibers
    st = fw.AsymmetricStencil3D()
    out["w_aniso19_carr"] = st.compute_weights(model, tissue)
    tissue.conductivity = 1.0
    st = fw.AsymmetricStencil3D()
    st.D_al, st.D_ac = 1.0, 0.25
    out["w_aniso19_c1_dac025"] = st.compute_weights(model, tissue)
    out["D_al_b"], out["D_ac_b"] = 1.0, 0.25
    return out


# ---------------------------------------------------------------- runs

def _attach(fw, model, trackers):
    seq = fw.TrackerSequence()
    for tr in trackers:
        seq.add_tracker(tr)
    model.tracker_sequence = seq


def case_ap2d_cfg1(fw):
    """AP 2D, 100x100 interior + boundary ring, iso, voltage S1, t=50."""
    n = 102
    tissue = fw.CardiacTissue2D((n, n))
    model = fw.AlievPanfilov2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 50
    model.prog_bar = False
    model.cardiac_tissue = tissue
    ss = fw.StimSequence()
    ss.add_stim(fw.StimVoltageCoord2D(0, 1.0, 0, n, 1, 6))
    model.stim_sequence = ss
    at = fw.ActivationTime2DTracker()
    at.threshold = 0.5
    at.step = 1
    _attach(fw, model, [at])
    model.run()
    return {"mesh": tissue.mesh.copy(), "u": model.u, "v": model.v,
            "u_new": model.u_new, "act_t": at.output, "t": model.t,
            "step": model.step}


def case_ap2d_aniso_spiral(fw):
    """AP 2D, aniso 9-pt + fibrosis + conductivity field, S1-S2, 10^4 steps."""
    rng = np.random.default_rng(303)
    n = 42
    tissue = fw.CardiacTissue2D((n, n))
    tissue.mesh = _fibrosis(rng, (n, n), 0.15)
    tissue.fibers = _seeded_fibers_2d(rng, (n, n))
    tissue.conductivity = rng.uniform(0.6, 1.0, size=(n, n))
    model = fw.AlievPanfilov2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 100
    model.prog_bar = False
    model.cardiac_tissue = tissue
    ss = fw.StimSequence()
    ss.add_stim(fw.StimVoltageCoord2D(0, 1.0, 0, n, 1, 4))
    ss.add_stim(fw.StimVoltageCoord2D(22, 1.0, n // 2, n, 0, n // 2))
    model.stim_sequence = ss
    at = fw.ActivationTime2DTracker()
    at.threshold = 0.5
    ap = fw.ActionPotential2DTracker()
    ap.cell_ind = [[5, 5], [20, 30], [35, 10]]
    ap.step = 7
    mv = fw.MultiVariable2DTracker()
    mv.cell_ind = [[10, 12], [30, 30]]
    mv.var_list = ["u", "v"]
    mv.step = 3
    mv.start_time = 10
    mv.end_time = 60
    _attach(fw, model, [at, ap, mv])
    model.run()
    return {"mesh": tissue.mesh.copy(), "fibers": tissue.fibers,
            "cond": tissue.conductivity, "u": model.u, "v": model.v,
            "act_t": at.output, "ap": ap.output,
            "mv_u": mv.output["u"], "mv_v": mv.output["v"],
            "t": model.t, "step": model.step}


def case_models_2d(fw):
    """MS and FK 2D, iso and aniso, current stimuli (with u_max), probes."""
    out = {}
    rng = np.random.default_rng(404)
    n = 24
    mesh = _fibrosis(rng, (n, n), 0.1)
    fibers = _seeded_fibers_2d(rng, (n, n))
    for name, cls, tmax, stim in [("ms", fw.MitchellSchaeffer2D, 40, 0.5),
                                  ("fk", fw.FentonKarma2D, 40, 0.5)]:
        for aniso in (False, True):
            tissue = fw.CardiacTissue2D((n, n))
            tissue.mesh = mesh.copy()
            if aniso:
                tissue.fibers = fibers
            model = cls()
            model.dt, model.dr, model.t_max = 0.01, 0.25, tmax
            model.prog_bar = False
            model.cardiac_tissue = tissue
            ss = fw.StimSequence()
            ss.add_stim(fw.StimCurrentCoord2D(0, 5, 1.0, 0, n, 1, 4,
                                              u_max=1.0))
            ss.add_stim(fw.StimCurrentCoord2D(2.5, 3, stim, 8, 14, 8, 14))
            model.stim_sequence = ss
            at = fw.ActivationTime2DTracker()
            at.threshold = 0.5
            mv = fw.MultiVariable2DTracker()
            mv.cell_ind = [[4, 4], [12, 20]]
            mv.var_list = list(model.state_vars)
            mv.step = 5
            _attach(fw, model, [at, mv])
            model.run()
            key = f"{name}_{'aniso' if aniso else 'iso'}"
            for var in model.state_vars:
                out[f"{key}_{var}"] = getattr(model, var)
                out[f"{key}_mv_{var}"] = mv.output[var]
            out[f"{key}_act_t"] = at.output
    out["mesh"] = mesh
    out["fibers"] = fibers
    return out


def case_ap3d(fw):
    """AP 3D, iso 7-pt and aniso 19-pt, fibrosis, voltage + current stimuli."""
    out = {}
    rng = np.random.default_rng(505)
    shape = (12, 11, 10)
    mesh = _fibrosis(rng, shape, 0.1)
    fibers = _seeded_fibers_3d(rng, shape)
    for aniso in (False, True):
        tissue = fw.CardiacTissue3D(shape)
        tissue.mesh = mesh.copy()
        if aniso:
            tissue.fibers = fibers
        model = fw.AlievPanfilov3D()
        model.dt, model.dr, model.t_max = 0.01, 0.25, 20
        model.prog_bar = False
        model.cardiac_tissue = tissue
        ss = fw.StimSequence()
        ss.add_stim(fw.StimVoltageCoord3D(0, 1.0, 0, 12, 0, 11, 1, 3))
        ss.add_stim(fw.StimCurrentCoord3D(8, 4, 0.6, 6, 12, 0, 6, 0, 10))
        model.stim_sequence = ss
        at = fw.ActivationTime3DTracker()
        at.threshold = 0.5
        _attach(fw, model, [at])
        model.run()
        key = "aniso" if aniso else "iso"
        out[f"{key}_u"] = model.u
        out[f"{key}_v"] = model.v
        out[f"{key}_act_t"] = at.output
    out["mesh"] = mesh
    out["fibers"] = fibers
    return out


def case_trackers(fw):
    """The reference's own tracker-test cable (12x3 AP) with AT and LAT."""
    out = {}
    ni, nj = 12, 3
    tissue = fw.CardiacTissue2D([ni, nj])
    ss = fw.StimSequence()
    ss.add_stim(fw.StimCurrentCoord2D(0, 5, 0.5, 0, 5, 0, nj))
    ss.add_stim(fw.StimVoltageCoord2D(45, 1, 0, 5, 0, 10))
    model = fw.AlievPanfilov2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 50
    model.prog_bar = False
    model.cardiac_tissue = tissue
    model.stim_sequence = ss
    lat = fw.LocalActivationTime2DTracker()
    lat.threshold = 0.5
    at = fw.ActivationTime2DTracker()
    at.threshold = 0.5
    at2 = fw.ActivationTime2DTracker()   # default threshold -40
    at3 = fw.ActivationTime2DTracker()
    at3.threshold = 0.2
    at3.step = 4
    at3.start_time = 1.0
    at3.end_time = 30.0
    _attach(fw, model, [lat, at, at2, at3])
    model.run()
    out["lat"] = lat.output
    out["act_t"] = at.output
    out["act_t_default"] = at2.output
    out["act_t_windowed"] = at3.output
    out["u"] = model.u
    return out


def case_stimuli(fw):
    """Matrix / area / list stimuli on 2D and 3D AP tissues."""
    out = {}
    rng = np.random.default_rng(606)
    n = 20
    tissue = fw.CardiacTissue2D((n, n))
    tissue.mesh = _fibrosis(rng, (n, n), 0.2)
    m1 = (rng.random((n, n)) < 0.3).astype(np.float64)
    m2 = (rng.random((n, n)) < 0.3).astype(np.int32)
    model = fw.AlievPanfilov2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 6
    model.prog_bar = False
    model.cardiac_tissue = tissue
    ss = fw.StimSequence()
    ss.add_stim(fw.StimVoltageMatrix2D(0, 0.8, m1))
    ss.add_stim(fw.StimCurrentMatrix2D(1, 2.5, 0.7, m2, u_max=0.9))
    area = fw.StimCurrentArea2D(2.0, 6.0, 0.4, u_max=1.2)
    area.add_stim_point(np.array([10, 10]), tissue.mesh, size=4)
    ss.add_stim(area)
    model.stim_sequence = ss
    at = fw.ActivationTime2DTracker()
    at.threshold = 0.5
    _attach(fw, model, [at])
    model.run()
    out.update(mesh2d=tissue.mesh.copy(), m1=m1, m2=m2,
               area_coords=area.coords, u2d=model.u, v2d=model.v,
               act_t2d=at.output)
    return out


def case_tp06(fw):
    """TP06 2D/3D small tissues with a current S1, probes of u and gates."""
    out = {}
    rng = np.random.default_rng(707)
    mesh2 = _fibrosis(rng, (10, 10), 0.1)
    fib2 = _seeded_fibers_2d(rng, (10, 10))
    mesh3 = _fibrosis(rng, (6, 6, 5), 0.1)
    for dim in (2, 3):
        if dim == 2:
            tissue = fw.CardiacTissue2D((10, 10))
            tissue.mesh = mesh2.copy()
            tissue.fibers = fib2
            model = fw.TP062D()
            ss = fw.StimSequence()
            ss.add_stim(fw.StimCurrentCoord2D(0, 60, 1.0, 0, 10, 0, 3))
        else:
            tissue = fw.CardiacTissue3D((6, 6, 5))
            tissue.mesh = mesh3.copy()
            model = fw.TP063D()
            ss = fw.StimSequence()
            ss.add_stim(fw.StimCurrentCoord3D(0, 100, 1.0, 0, 6, 0, 3, 0, 5))
        model.dt, model.dr, model.t_max = 0.01, 0.25, 20
        model.prog_bar = False
        model.cardiac_tissue = tissue
        model.stim_sequence = ss
        tr = (fw.MultiVariable2DTracker() if dim == 2
              else fw.MultiVariable3DTracker())
        tr.cell_ind = [[4, 4]] if dim == 2 else [[3, 3, 2]]
        tr.var_list = ["u", "m", "cai", "nai", "Ki", "casr"]
        tr.step = 10
        # MultiVariable*Tracker.initialize checks model.__dict__ before the
        # model's own initialize() creates the TP06 state arrays
        # (multi_variable_2d_tracker.py:53-56 runs from
        # cardiac_model.py:107-108), so the attributes must exist beforehand.
        for var in tr.var_list:
            if var not in model.__dict__:
                setattr(model, var, None)
        _attach(fw, model, [tr])
        model.run()
        for var in model.state_vars:
            out[f"d{dim}_{var}"] = getattr(model, var)
        for var in tr.var_list:
            out[f"d{dim}_mv_{var}"] = tr.output[var]
    out["mesh2"], out["fib2"], out["mesh3"] = mesh2, fib2, mesh3
    return out


def case_courtemanche(fw):
    """Courtemanche 2D/3D small tissues with a current S1, probes of u,
    Ca_i, Na_i and both potassium gates."""
    out = {}
    rng = np.random.default_rng(808)
    mesh2 = _fibrosis(rng, (10, 10), 0.1)
    mesh3 = _fibrosis(rng, (6, 6, 5), 0.1)
    fib3 = _seeded_fibers_3d(rng, (6, 6, 5))
    for dim in (2, 3):
        ss = fw.StimSequence()
        if dim == 2:
            tissue = fw.CardiacTissue2D((10, 10))
            tissue.mesh = mesh2.copy()
            model = fw.Courtemanche2D()
            ss.add_stim(fw.StimCurrentCoord2D(0, 80, 1.0, 0, 10, 0, 4))
        else:
            tissue = fw.CardiacTissue3D((6, 6, 5))
            tissue.mesh = mesh3.copy()
            tissue.fibers = fib3
            model = fw.Courtemanche3D()
            ss.add_stim(fw.StimCurrentCoord3D(0, 80, 1.0, 0, 6, 0, 3, 0, 5))
        model.dt, model.dr, model.t_max = 0.01, 0.25, 20
        model.prog_bar = False
        model.cardiac_tissue = tissue
        model.stim_sequence = ss
        tr = (fw.MultiVariable2DTracker() if dim == 2
              else fw.MultiVariable3DTracker())
        tr.cell_ind = [[4, 4]] if dim == 2 else [[3, 3, 2]]
        tr.var_list = ["u", "cai", "nai", "xs", "xr", "irel"]
        tr.step = 10
        for var in tr.var_list:  # see case_tp06
            if var not in model.__dict__:
                setattr(model, var, None)
        _attach(fw, model, [tr])
        model.run()
        for var in model.state_vars:
            out[f"d{dim}_{var}"] = getattr(model, var)
        for var in tr.var_list:
            out[f"d{dim}_mv_{var}"] = tr.output[var]
    out["mesh2"], out["mesh3"], out["fib3"] = mesh2, mesh3, fib3
    return out


def case_detailed_long(fw):
    """TP06 and Courtemanche, 2D and 3D, 10^4 steps (t = 0 .. 100 ms at
    dt = 0.01) from a current S1 through the upstroke into the plateau, on
    small fibrotic anisotropic tissues; the whole u field and every state
    variable at the end, and u at two cells every 100 steps."""
    out = {}
    rng = np.random.default_rng(909)
    mesh2 = _fibrosis(rng, (10, 10), 0.1)
    fib2 = _seeded_fibers_2d(rng, (10, 10))
    mesh3 = _fibrosis(rng, (6, 6, 5), 0.1)
    fib3 = _seeded_fibers_3d(rng, (6, 6, 5))
    out["mesh2"], out["fib2"], out["mesh3"], out["fib3"] = (mesh2, fib2,
                                                           mesh3, fib3)
    for name in ("tp06", "crn"):
        for dim in (2, 3):
            cls = {("tp06", 2): fw.TP062D, ("tp06", 3): fw.TP063D,
                   ("crn", 2): fw.Courtemanche2D,
                   ("crn", 3): fw.Courtemanche3D}[(name, dim)]
            model = cls()
            ss = fw.StimSequence()
            if dim == 2:
                tissue = fw.CardiacTissue2D((10, 10))
                tissue.mesh = mesh2.copy()
                tissue.fibers = fib2
                ss.add_stim(fw.StimCurrentCoord2D(0, 80, 1.0, 0, 10, 0, 3))
            else:
                tissue = fw.CardiacTissue3D((6, 6, 5))
                tissue.mesh = mesh3.copy()
                tissue.fibers = fib3
                ss.add_stim(fw.StimCurrentCoord3D(0, 80, 1.0, 0, 6, 0, 3,
                                                  0, 5))
            model.dt, model.dr, model.t_max = 0.01, 0.25, 100
            model.prog_bar = False
            model.cardiac_tissue = tissue
            model.stim_sequence = ss
            tr = (fw.MultiVariable2DTracker() if dim == 2
                  else fw.MultiVariable3DTracker())
            tr.cell_ind = ([[4, 4], [7, 6]] if dim == 2
                           else [[3, 3, 2], [4, 2, 3]])
            tr.var_list = ["u"]
            tr.step = 100
            for var in tr.var_list:  # see case_tp06
                if var not in model.__dict__:
                    setattr(model, var, None)
            _attach(fw, model, [tr])
            model.run()
            key = f"{name}{dim}"
            for var in model.state_vars:
                out[f"{key}_{var}"] = getattr(model, var)
            out[f"{key}_mv_u"] = tr.output["u"]
            out[f"{key}_step"] = model.step
    return out


def plugin_classes(Stim, Tracker):
    """A user stimulus and a user tracker written against the reference's
    plug-in interface (Stim.stimulate, Tracker._track), built on the given
    base classes, so that the test can define the same two classes on the
    GPU package's bases."""

    class RestimulateWhenQuiet(Stim):
        """While active: u = 1 on rows 1..3 whenever node (15, 15) is
        below 0.1; counts its firings."""

        def __init__(self, time, duration):
            super().__init__(time, duration)
            self.count = 0

        def initialize(self, model):
            self.count = 0

        def stimulate(self, model):
            if model.u[15, 15] < 0.1:
                model.u[1:4, 1:-1] = 1.0
                self.count += 1

    class PatchTracker(Tracker):
        """Per active step: step, t, the sums of u and u_new over a 3 x 3
        patch, and v at one node read through the model's __dict__."""

        def initialize(self, model):
            self.model = model
            self.output = []

        def _track(self):
            m = self.model
            self.output.append([m.step, m.t, float(m.u[3:6, 3:6].sum()),
                                float(m.u_new[3:6, 3:6].sum()),
                                float(m.__dict__["v"][4, 4])])

    return RestimulateWhenQuiet, PatchTracker


def case_plugins(fw):
    """Aliev-Panfilov 2D, 32 x 32 isotropic, float64: a planar S1, the user
    stimulus above from t = 30 for 2 time units, the user tracker every 50
    steps from t = 5 and an activation-time tracker; t = 60."""
    Restim, Patch = plugin_classes(fw.Stim, fw.Tracker)
    n = 32
    tissue = fw.CardiacTissue2D((n, n))
    model = fw.AlievPanfilov2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 60
    model.prog_bar = False
    model.cardiac_tissue = tissue
    ss = fw.StimSequence()
    ss.add_stim(fw.StimVoltageCoord2D(0, 1.0, 0, n, 1, 5))
    rs = Restim(30, 2.0)
    ss.add_stim(rs)
    model.stim_sequence = ss
    pt = Patch()
    pt.start_time = 5
    pt.step = 50
    at = fw.ActivationTime2DTracker()
    at.threshold = 0.5
    _attach(fw, model, [pt, at])
    model.run()
    return {"u": model.u, "v": model.v, "act_t": at.output,
            "patch": np.asarray(pt.output, dtype=np.float64),
            "restim_count": rs.count, "step": model.step}


def case_fibrosis(fw):
    """Seeded diffuse fibrosis patterns, 2D and 3D, whole mesh and boxes."""
    out = {}
    np.random.seed(2024)
    out["d2_full"] = fw.Diffuse2DPattern(0.3).generate(shape=(20, 30))
    np.random.seed(2025)
    out["d2_box"] = fw.Diffuse2DPattern(0.5, 3, 15, 4, 22).generate(
        shape=(20, 30))
    np.random.seed(2026)
    mesh = np.ones((20, 30), dtype=np.int8)
    mesh[0, :] = 0
    out["d2_mesh_in"] = mesh.copy()
    out["d2_mesh"] = fw.Diffuse2DPattern(0.2).generate(mesh=mesh)
    np.random.seed(2027)
    out["d3_box"] = fw.Diffuse3DPattern(2, 10, 1, 8, 0, 5, 0.25).generate(
        (12, 9, 6))
    np.random.seed(2028)
    out["d3_full"] = fw.Diffuse3DPattern(None, None, None, None, None, None,
                                         0.1).generate((8, 7, 6))
    return out


def case_ecg(fw):
    """ECG trackers: the reference's planar 50 x 5 Aliev-Panfilov model
    (tests/test_trackers_2d.py:43-58, 261-278) with two leads every 10
    steps, and a 3D anisotropic Aliev-Panfilov slab with three leads."""
    out = {}
    tissue = fw.CardiacTissue2D([50, 5])
    ss = fw.StimSequence()
    ss.add_stim(fw.StimCurrentCoord2D(5, 5, 0.5, 0, 5, 0, 5))
    model = fw.AlievPanfilov2D()
    model.dt, model.dr, model.t_max = 0.0015, 0.25, 15
    model.prog_bar = False
    model.cardiac_tissue = tissue
    model.stim_sequence = ss
    tr = fw.ECG2DTracker()
    tr.start_time = 0
    tr.step = 10
    tr.measure_coords = np.array([[25, 2, 0], [10, -3, 1.5]])
    _attach(fw, model, [tr])
    model.run()
    out["d2_ecg"] = tr.output
    out["d2_u"] = model.u
    rng = np.random.default_rng(909)
    mesh3 = _fibrosis(rng, (14, 10, 8), 0.1)
    fib3 = _seeded_fibers_3d(rng, (14, 10, 8))
    tissue = fw.CardiacTissue3D((14, 10, 8))
    tissue.mesh = mesh3.copy()
    tissue.fibers = fib3
    ss = fw.StimSequence()
    ss.add_stim(fw.StimVoltageCoord3D(0, 1, 0, 14, 0, 3, 0, 8))
    model = fw.AlievPanfilov3D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 10
    model.prog_bar = False
    model.cardiac_tissue = tissue
    model.stim_sequence = ss
    tr = fw.ECG3DTracker()
    tr.step = 5
    tr.measure_coords = np.array([[7, 12, 4], [-2, 5, 3], [7, 5, 10.5]])
    _attach(fw, model, [tr])
    model.run()
    out["d3_ecg"] = tr.output
    out["d3_u"] = model.u
    out["mesh3"], out["fib3"] = mesh3, fib3
    return out


def case_tips(fw):
    """Spiral-wave tips and activation periods: Aliev-Panfilov S1-S2 cross
    field stimulation (S1 columns 1-3 at t = 0, S2 on the first half of
    the rows at t = 30) on a 64^2 sheet and a 48 x 48 x 3 slab (one
    interior layer).  The tips
    are recorded with the reference's own SpiralWaveCore tracker methods
    (its output needs pandas, absent here), the periods from its
    Period2DTracker's layers as its output computes them."""
    out = {}

    def tip_recorder(base):
        class Rec(base):
            def initialize(self, model):
                super().initialize(model)
                self.rec = []

            def _track(self):
                if self.model.u.ndim == 2:
                    layers = [(None, self.u_prev, self.model.u)]
                else:
                    layers = [(k, self.u_prev[:, :, k], self.model.u[:, :, k])
                              for k in range(self.model.u.shape[2])]
                for k, up, uc in layers:
                    for x, y in self.track_tip_line(up, uc, self.threshold):
                        self.rec.append((x, y, -1 if k is None else k,
                                         self.model.t, self.model.step))
                self.u_prev = self.model.u.copy()
        return Rec

    for dim in (2, 3):
        n = 64 if dim == 2 else 48
        shape = (n, n) if dim == 2 else (n, n, 3)
        tissue = (fw.CardiacTissue2D if dim == 2 else fw.CardiacTissue3D)(
            list(shape))
        ss = fw.StimSequence()
        if dim == 2:
            ss.add_stim(fw.StimVoltageCoord2D(0, 1, 0, n, 1, 4))
            ss.add_stim(fw.StimVoltageCoord2D(30, 1, 0, n // 2, 0, n))
            model = fw.AlievPanfilov2D()
            tip = tip_recorder(fw.SpiralWaveCore2DTracker)()
            per = fw.Period2DTracker()
        else:
            ss.add_stim(fw.StimVoltageCoord3D(0, 1, 0, n, 1, 4, 0, 3))
            ss.add_stim(fw.StimVoltageCoord3D(30, 1, 0, n // 2, 0, n, 0, 3))
            model = fw.AlievPanfilov3D()
            tip = tip_recorder(fw.SpiralWaveCore3DTracker)()
            per = fw.Period3DTracker()
        model.dt, model.dr, model.t_max = 0.01, 0.25, 60
        model.prog_bar = False
        model.cardiac_tissue = tissue
        model.stim_sequence = ss
        tip.threshold = 0.5
        tip.step = 20
        cells = [[n // 2, n // 2], [10, 40], [40, 10]] if dim == 2 else \
            [[24, 24, 1], [10, 40, 1]]
        per.cell_ind = cells
        per.threshold = 0.5
        _attach(fw, model, [tip, per])
        model.run()
        rec = np.array(tip.rec, dtype=np.float64).reshape(-1, 5)
        out[f"d{dim}_tips"] = rec
        lats = np.array(per.act_t).T
        periods = [np.diff(row[row != -1]) for row in lats]
        out[f"d{dim}_period_len"] = np.array([len(p) for p in periods])
        out[f"d{dim}_periods"] = np.concatenate(periods) if periods else \
            np.zeros(0)
        out[f"d{dim}_u"] = model.u
        out[f"d{dim}_cells"] = np.array(cells)
    return out


def case_models_extra(fw):
    """Barkley, Bueno-Orovio and Luo-Rudy 1991 on small 2D (anisotropic,
    fibrotic) and 3D (isotropic) tissues, current S1, an activation tracker
    and probes of u and the first state variable."""
    out = {}
    rng = np.random.default_rng(1111)
    mesh2 = _fibrosis(rng, (20, 20), 0.1)
    fib2 = _seeded_fibers_2d(rng, (20, 20))
    mesh3 = _fibrosis(rng, (8, 8, 6), 0.1)
    spec = {"bk": (fw.Barkley2D, fw.Barkley3D, 5, 0.1, 12, 0.5, "v"),
            "bo": (fw.BuenoOrovio2D, fw.BuenoOrovio3D, 5, 0.5, 30, 0.5, "v"),
            "lr91": (fw.LuoRudy912D, fw.LuoRudy913D, 100, 1.0, 20, -20.0,
                     "m")}
    for name, (c2, c3, cv, cd, t_max, thr, var) in spec.items():
        for dim in (2, 3):
            ss = fw.StimSequence()
            if dim == 2:
                tissue = fw.CardiacTissue2D((20, 20))
                tissue.mesh = mesh2.copy()
                tissue.fibers = fib2
                model = c2()
                ss.add_stim(fw.StimCurrentCoord2D(0, cv, cd, 0, 20, 0, 4))
                at, mv = fw.ActivationTime2DTracker(), fw.MultiVariable2DTracker()
                mv.cell_ind = [[10, 11]]
            else:
                tissue = fw.CardiacTissue3D((8, 8, 6))
                tissue.mesh = mesh3.copy()
                model = c3()
                ss.add_stim(fw.StimCurrentCoord3D(0, cv, cd, 0, 8, 0, 3, 0, 6))
                at, mv = fw.ActivationTime3DTracker(), fw.MultiVariable3DTracker()
                mv.cell_ind = [[4, 5, 3]]
            model.dt, model.dr, model.t_max = 0.01, 0.25, t_max
            model.prog_bar = False
            model.cardiac_tissue = tissue
            model.stim_sequence = ss
            at.threshold = thr
            mv.var_list = ["u", var]
            mv.step = 5
            _attach(fw, model, [at, mv])
            model.run()
            for v in model.state_vars:
                out[f"{name}{dim}_{v}"] = getattr(model, v)
            out[f"{name}{dim}_act_t"] = at.output
            for v in mv.var_list:
                out[f"{name}{dim}_mv_{v}"] = mv.output[v]
    out["mesh2"], out["fib2"], out["mesh3"] = mesh2, fib2, mesh3
    return out


CASES = {
    "weights_2d": case_weights_2d,
    "weights_3d": case_weights_3d,
    "ap2d_cfg1": case_ap2d_cfg1,
    "ap2d_aniso_spiral": case_ap2d_aniso_spiral,
    "models_2d": case_models_2d,
    "ap3d": case_ap3d,
    "trackers": case_trackers,
    "stimuli": case_stimuli,
    "tp06": case_tp06,
    "courtemanche": case_courtemanche,
    "detailed_long": case_detailed_long,
    "plugins": case_plugins,
    "fibrosis": case_fibrosis,
    "ecg": case_ecg,
    "tips": case_tips,
    "models_extra": case_models_extra,
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("cases", nargs="*")
    args = ap.parse_args()
    os.environ["NUMBA_DISABLE_JIT"] = "1"
    cwd = tempfile.mkdtemp(prefix="fw_golden_cwd_")
    fw = import_reference(os.path.abspath(args.reference))
    os.chdir(cwd)
    names = args.cases or list(CASES)
    for name in names:
        t0 = time.time()
        np.random.seed(0)
        out = CASES[name](fw)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(f"{name}: {time.time() - t0:.1f} s", flush=True)


if __name__ == "__main__":
    main()
