"""Drive finitewave_gb300's public API with the oracle's case dicts."""
import numpy as np

import finitewave_gb300 as fg

_MODELS = {("ap", 2): fg.AlievPanfilov2D, ("ap", 3): fg.AlievPanfilov3D,
           ("ms", 2): fg.MitchellSchaeffer2D, ("ms", 3): fg.MitchellSchaeffer3D,
           ("fk", 2): fg.FentonKarma2D, ("fk", 3): fg.FentonKarma3D,
           ("tp06", 2): fg.TP062D, ("tp06", 3): fg.TP063D,
           ("crn", 2): fg.Courtemanche2D, ("crn", 3): fg.Courtemanche3D,
           ("bk", 2): fg.Barkley2D, ("bk", 3): fg.Barkley3D,
           ("bo", 2): fg.BuenoOrovio2D, ("bo", 3): fg.BuenoOrovio3D,
           ("lr91", 2): fg.LuoRudy912D, ("lr91", 3): fg.LuoRudy913D}


def register(name, cls2d, cls3d):
    _MODELS[(name, 2)] = cls2d
    _MODELS[(name, 3)] = cls3d


def build(case, npfloat="float64", form=None, fused_k=0, fused_variant=0):
    mesh = np.asarray(case["mesh"])
    dim = mesh.ndim
    tissue = fg.CardiacTissue2D(mesh.shape) if dim == 2 \
        else fg.CardiacTissue3D(mesh.shape)
    tissue.mesh = mesh.astype(np.int8).copy()
    if case["stencil"] in ("aniso9", "aniso19", "sym9"):
        tissue.fibers = case["fibers"]
    tissue.conductivity = case.get("conductivity", 1.0)
    model = _MODELS[(case["model"], dim)]()
    model.dt, model.dr, model.t_max = case["dt"], case["dr"], case["t_max"]
    model.prog_bar = False
    model.npfloat = npfloat
    model.form = form
    model.fused_k = fused_k
    model.fused_variant = fused_variant
    for k, v in case.get("params", {}).items():
        setattr(model, k, v)
    if "D_model" in case:
        model.D_model = case["D_model"]
    if case["stencil"] == "sym9":
        st = fg.SymmetricStencil2D()
    elif case["stencil"] == "aniso9":
        st = fg.AsymmetricStencil2D()
    elif case["stencil"] == "aniso19":
        st = fg.AsymmetricStencil3D()
    else:
        st = None
    if st is not None:
        st.D_al = case.get("D_al", 1.0)
        st.D_ac = case.get("D_ac", 1.0 / 9)
        model.stencil = st
    model.cardiac_tissue = tissue
    seq = fg.StimSequence()
    for s in case.get("stims", []):
        volt = s["kind"] == "voltage"
        if "box" in s:
            flat = [b for pair in s["box"] for b in pair]
            if volt:
                cls = fg.StimVoltageCoord2D if dim == 2 else fg.StimVoltageCoord3D
                seq.add_stim(cls(s["t"], s["value"], *flat))
            else:
                cls = fg.StimCurrentCoord2D if dim == 2 else fg.StimCurrentCoord3D
                seq.add_stim(cls(s["t"], s["value"], s.get("duration", 0.0),
                                 *flat, u_max=s.get("u_max")))
        elif "matrix" in s:
            if volt:
                seq.add_stim(fg.StimVoltageMatrix2D(s["t"], s["value"],
                                                    s["matrix"]))
            else:
                seq.add_stim(fg.StimCurrentMatrix2D(
                    s["t"], s["value"], s.get("duration", 0.0), s["matrix"],
                    u_max=s.get("u_max")))
        else:
            seq.add_stim(fg.StimCurrentArea2D(
                s["t"], s["value"], s.get("duration", 0.0),
                coords=np.asarray(s["coords"]), u_max=s.get("u_max")))
    model.stim_sequence = seq
    trs = fg.TrackerSequence()
    objs = []
    for tr in case.get("trackers", []):
        if tr["kind"] == "at":
            o = fg.ActivationTime2DTracker()
            o.threshold = tr["threshold"]
        elif tr["kind"] == "lat":
            o = fg.LocalActivationTime2DTracker()
            o.threshold = tr["threshold"]
        elif tr["kind"] == "tips":
            o = fg.SpiralWaveCore2DTracker() if dim == 2 \
                else fg.SpiralWaveCore3DTracker()
            o.threshold = tr["threshold"]
        elif tr["kind"] == "period":
            o = fg.Period2DTracker() if dim == 2 else fg.Period3DTracker()
            o.threshold = tr["threshold"]
            o.cell_ind = tr["cells"]
        elif tr["kind"] == "ecg":
            o = fg.ECG2DTracker() if dim == 2 else fg.ECG3DTracker()
            o.measure_coords = np.asarray(tr["coords"], dtype=np.float64)
        else:
            o = fg.MultiVariable2DTracker() if dim == 2 \
                else fg.MultiVariable3DTracker()
            o.cell_ind = tr["cells"]
            o.var_list = list(tr["vars"])
        o.start_time = tr.get("start_time", 0)
        o.end_time = tr.get("end_time", np.inf)
        o.step = tr.get("step", 1)
        trs.add_tracker(o)
        objs.append(o)
    model.tracker_sequence = trs
    return model, objs


def run(case, **kw):
    model, objs = build(case, **kw)
    model.run()
    out = {"u": model.u, "u_new": model.u_new, "t": model.t,
           "step": model.step, "model": model}
    for name in model._state_names:
        out[name] = getattr(model, name)
    out["trackers"] = [o.output for o in objs]
    return out
