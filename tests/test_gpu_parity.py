"""GPU parity: the sm_103a library against the reference's golden vectors and
the CPU oracle, through the public API (which calls the C ABI).

Tolerances: float64 runs of models built from + - * / only (Aliev-Panfilov,
Mitchell-Schaeffer) and every stencil-weight build are bitwise equal
(``np.array_equal``); Fenton-Karma calls tanh, whose CUDA and C-library
roundings differ in the last ulp, so its fields get |diff| <= 1e-12.
Activation-time outputs are compared exactly.
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


@pytest.fixture(scope="module")
def gc(fg):
    import gpu_cases
    return gpu_cases


class _M:
    def __init__(self, D_model, dt, dr, npfloat="float64"):
        self.D_model, self.dt, self.dr, self.npfloat = D_model, dt, dr, npfloat
        self.device = None

    def _device(self):
        return torch.device("cuda")

    def _precision(self):
        return 0 if self.npfloat == "float64" else 1


def _weights(fg, stencil, g, cond, fibers=None, D_al=None, D_ac=None):
    shape = g["mesh"].shape
    t = fg.CardiacTissue2D(shape) if len(shape) == 2 \
        else fg.CardiacTissue3D(shape)
    t.mesh = g["mesh"].copy()
    t.conductivity = cond
    t.fibers = fibers
    if D_al is not None:
        stencil.D_al, stencil.D_ac = D_al, D_ac
    m = _M(float(g["D_model"]), float(g["dt"]), float(g["dr"]))
    w = stencil.compute_weights(m, t)
    torch.cuda.synchronize()
    return np.moveaxis(w.cpu().numpy(), 0, -1)


def test_weights_2d_bitwise(fg):
    g = cases.load("weights_2d")
    assert np.array_equal(_weights(fg, fg.IsotropicStencil2D(), g, 1.0),
                          g["w_iso5_c1"])
    assert np.array_equal(_weights(fg, fg.IsotropicStencil2D(), g, g["cond"]),
                          g["w_iso5_carr"])
    assert np.array_equal(
        _weights(fg, fg.AsymmetricStencil2D(), g, g["cond"], g["fibers"]),
        g["w_aniso9_carr"])
    assert np.array_equal(
        _weights(fg, fg.AsymmetricStencil2D(), g, 1.0, g["fibers"],
                 float(g["D_al_b"]), float(g["D_ac_b"])),
        g["w_aniso9_c1_dac0111"])


def test_weights_3d_bitwise(fg):
    g = cases.load("weights_3d")
    assert np.array_equal(_weights(fg, fg.IsotropicStencil3D(), g, 1.0),
                          g["w_iso7_c1"])
    assert np.array_equal(_weights(fg, fg.IsotropicStencil3D(), g, g["cond"]),
                          g["w_iso7_carr"])
    assert np.array_equal(
        _weights(fg, fg.AsymmetricStencil3D(), g, g["cond"], g["fibers"]),
        g["w_aniso19_carr"])
    assert np.array_equal(
        _weights(fg, fg.AsymmetricStencil3D(), g, 1.0, g["fibers"],
                 float(g["D_al_b"]), float(g["D_ac_b"])),
        g["w_aniso19_c1_dac025"])


def test_weights_f32_rounding(fg):
    """FP32 weights are the float64 weights rounded once."""
    g = cases.load("weights_2d")
    t = fg.CardiacTissue2D(g["mesh"].shape)
    t.mesh = g["mesh"].copy()
    t.fibers = g["fibers"]
    m = _M(float(g["D_model"]), float(g["dt"]), float(g["dr"]), "float32")
    w = fg.AsymmetricStencil2D().compute_weights(m, t)
    ref = g["w_aniso9_c1_dac0111"]
    st = fg.AsymmetricStencil2D()
    st.D_al, st.D_ac = float(g["D_al_b"]), float(g["D_ac_b"])
    w = st.compute_weights(m, t)
    assert w.dtype == torch.float32
    assert np.array_equal(np.moveaxis(w.cpu().numpy(), 0, -1),
                          ref.astype(np.float32))


def test_ap2d_cfg1_bitwise(gc):
    """100x100 Aliev-Panfilov planar wave, 5000 FP64 steps: u, v, u_new and
    the activation map equal the reference's bit for bit."""
    case, g = cases.ap2d_cfg1()
    r = gc.run(case)
    assert r["step"] == int(g["step"]) == 5000
    assert r["t"] == float(g["t"])
    assert np.array_equal(r["u"], g["u"])
    assert np.array_equal(r["v"], g["v"])
    assert np.array_equal(r["u_new"], g["u_new"])
    assert np.array_equal(r["trackers"][0], g["act_t"])


def test_ap2d_aniso_spiral_bitwise(gc):
    """42x42 anisotropic, fibrotic, heterogeneous conductivity, S1-S2,
    10^4 FP64 steps, with probes on a stride and a time window."""
    case, g = cases.ap2d_aniso_spiral()
    r = gc.run(case)
    assert r["step"] == 10000
    assert np.array_equal(r["u"], g["u"])
    assert np.array_equal(r["v"], g["v"])
    at, ap, mv = r["trackers"]
    assert np.array_equal(at, g["act_t"])
    assert np.array_equal(ap["u"], g["ap"])
    assert np.array_equal(mv["u"], g["mv_u"])
    assert np.array_equal(mv["v"], g["mv_v"])


@pytest.mark.parametrize("name", ["ms", "fk"])
@pytest.mark.parametrize("aniso", [False, True])
def test_models_2d(gc, oracle, name, aniso):
    case, g = cases.models_2d(name, aniso)
    r = gc.run(case)
    o = oracle.run(case)
    at, mv = r["trackers"]
    assert np.array_equal(at, g["act_t"])
    for v in cases.MODEL_VARS[name]:
        if name == "ms":
            assert np.array_equal(r[v], g[v]), v
            assert np.array_equal(mv[v], g["mv_" + v]), v
        else:
            np.testing.assert_allclose(r[v], o[v], rtol=0, atol=1e-12)
            np.testing.assert_allclose(r[v], g[v], rtol=0, atol=1e-12)
            np.testing.assert_allclose(mv[v], g["mv_" + v], rtol=0,
                                       atol=1e-12)


@pytest.mark.parametrize("aniso", [False, True])
def test_ap3d_bitwise(gc, aniso):
    case, g = cases.ap3d(aniso)
    r = gc.run(case)
    assert np.array_equal(r["u"], g["u"])
    assert np.array_equal(r["v"], g["v"])
    assert np.array_equal(r["trackers"][0], g["act_t"])


def test_trackers_cable(gc):
    """The reference's tracker-test cable: LAT layers, AT with the default
    threshold (every node, non-myocytes included) and a windowed, strided
    AT tracker."""
    case, g = cases.trackers_cable()
    r = gc.run(case)
    lat, at, at_def, at_win = r["trackers"]
    assert lat.shape == g["lat"].shape
    assert np.array_equal(lat, g["lat"])
    assert np.array_equal(at, g["act_t"])
    assert np.array_equal(at_def, g["act_t_default"])
    assert np.array_equal(at_win, g["act_t_windowed"])
    assert np.array_equal(r["u"], g["u"])


def test_stimuli_matrix_area(gc):
    case, g = cases.stimuli_2d()
    r = gc.run(case)
    assert np.array_equal(r["u"], g["u2d"])
    assert np.array_equal(r["v"], g["v2d"])
    assert np.array_equal(r["trackers"][0], g["act_t2d"])


def _at_agree(at, ref, dt):
    """Fraction of nodes whose activation step agrees within one step
    (never-activated must agree exactly)."""
    same_set = (at >= 0) == (ref >= 0)
    both = (at >= 0) & (ref >= 0)
    ok = same_set.copy()
    ok[both] = np.abs(at[both] - ref[both]) / dt <= 1.0 + 1e-6
    return ok.mean()


@pytest.mark.parametrize("form", ["plain", "fused"])
def test_f32_close_to_f64(gc, form):
    """FP32 forms against the FP64 reference on the anisotropic spiral
    (10^4 steps): activation times within one step on >= 99.9 % of nodes,
    probe traces and the final field within 5e-3."""
    case, g = cases.ap2d_aniso_spiral()
    r = gc.run(case, npfloat="float32", form=form)
    at, ap, mv = r["trackers"]
    assert _at_agree(at, g["act_t"], case["dt"]) >= 0.999
    assert np.abs(r["u"] - g["u"]).max() < 5e-3
    assert np.abs(ap["u"] - g["ap"]).max() < 5e-3
    assert np.abs(mv["v"] - g["mv_v"]).max() < 5e-3


def _fused_case(name, aniso, nj):
    rng = np.random.default_rng(11)
    ni = 150
    mesh = np.where(rng.random((ni, nj)) < 0.15, 2, 1).astype(np.int8)
    ang = rng.uniform(-np.pi, np.pi, (ni, nj))
    fibers = np.stack([np.cos(ang), np.sin(ang)], -1)
    return dict(model=name, mesh=mesh, dt=0.01, dr=0.25, t_max=7.77,
                stencil="aniso9" if aniso else "iso5", fibers=fibers,
                stims=[dict(kind="voltage", t=0, value=1.0,
                            box=[(0, ni), (1, 5)]),
                       dict(kind="current", t=2.0, value=20.0, duration=0.5,
                            box=[(60, 150), (0, 70)], u_max=1.0)],
                trackers=[dict(kind="at", threshold=0.5),
                          dict(kind="probe", cells=[[3, 3], [75, 70],
                                                    [149, 139], [56, 56]],
                               vars=cases.MODEL_VARS[name], step=3),
                          dict(kind="lat", threshold=0.5)])


@pytest.mark.parametrize("name", ["ap", "ms", "fk"])
@pytest.mark.parametrize("aniso", [False, True])
@pytest.mark.parametrize("k", [2, 4, 8])
@pytest.mark.parametrize("variant,nj", [(1, 140), (2, 140), (3, 144), (4, 144),
                                        (6, 144)])
def test_fused_matches_plain_f32(gc, name, aniso, k, variant, nj):
    """Fused temporal blocking vs the plain FP32 form on a grid of several
    tiles (150 x nj), S1 plus a cross-field S2, 777 steps (an odd count, not
    a multiple of k): same activation steps within one step, fields within
    a tolerance that covers FMA-vs-no-FMA rounding.  Variants 1 and 2 stage
    with cp.async; variants 3 and 4 are the persistent TMA pipeline (rows of
    a multiple of 16 nodes) with 4 x 1 and 2 x 2 nodes per thread, variant 6
    the 2 x 2 kernel in two-wide float32 instructions."""
    case = _fused_case(name, aniso, nj)
    ref = gc.run(case, npfloat="float32", form="plain")
    r = gc.run(case, npfloat="float32", form="fused", fused_k=k,
               fused_variant=variant)
    assert int(r["model"]._status.item()) == 0
    assert r["step"] == ref["step"] == 777
    assert _at_agree(r["trackers"][0], ref["trackers"][0], 0.01) >= 0.999
    for v in cases.MODEL_VARS[name]:
        np.testing.assert_allclose(r[v], ref[v], rtol=0, atol=2e-3)
        np.testing.assert_allclose(r["trackers"][1][v], ref["trackers"][1][v],
                                   rtol=0, atol=2e-3)


@pytest.mark.parametrize("name", ["ap", "ms", "fk"])
@pytest.mark.parametrize("aniso", [False, True])
@pytest.mark.parametrize("k", [2, 4, 8])
@pytest.mark.parametrize("variant", [1, 2, 4, 6])
def test_fused_variants_bitwise_equal(gc, name, aniso, k, variant):
    """Every fused kernel (cp.async 64 x 32 and 64 x 64 regions, TMA with
    4 x 1 strips or 2 x 2 blocks, the 2 x 2 kernel in two-wide float32
    instructions) forms each node's diffusion sum as the same FMA chain over
    the stored weights and runs the same ionic update, so fields, state,
    activation times and probe traces agree bitwise with the TMA strip
    kernel (variant 3).  Local activation flags: read from global memory by
    variants 1 and 2, staged with the region by variants 3, 4 and 6."""
    case = _fused_case(name, aniso, 144)
    r3 = gc.run(case, npfloat="float32", form="fused", fused_k=k,
                fused_variant=3)
    rv = gc.run(case, npfloat="float32", form="fused", fused_k=k,
                fused_variant=variant)
    assert int(rv["model"]._status.item()) == 0
    for v in cases.MODEL_VARS[name]:
        assert np.array_equal(rv[v], r3[v]), v
        assert np.array_equal(rv["trackers"][1][v], r3["trackers"][1][v]), v
    assert np.array_equal(rv["trackers"][0], r3["trackers"][0])
    lat3, latv = r3["trackers"][2], rv["trackers"][2]
    assert lat3.shape == latv.shape and lat3.shape[0] >= 1
    assert np.array_equal(latv, lat3, equal_nan=True)


@pytest.mark.parametrize("name", ["ap", "ms", "fk"])
@pytest.mark.parametrize("aniso", [False, True])
@pytest.mark.parametrize("k", [2, 3, 4])
def test_fused_march_bitwise_equal(gc, name, aniso, k):
    """Variant 7 marches 64-column strips down the rows with the K time
    levels in flight (no halo rows, state and tracker flags handed from
    level to level in registers, the levels' rows in shared-memory rings):
    every node's arithmetic is the tile kernels', so fields, state,
    activation times and local activation times are bitwise those of the
    TMA strip kernel (variant 3).  The case without its probe tracker
    (variant 7 takes none)."""
    case = _fused_case(name, aniso, 144)
    case["trackers"] = [t for t in case["trackers"] if t["kind"] != "probe"]
    r3 = gc.run(case, npfloat="float32", form="fused", fused_k=k,
                fused_variant=3)
    r7 = gc.run(case, npfloat="float32", form="fused", fused_k=k,
                fused_variant=7)
    assert int(r7["model"]._status.item()) == 0
    assert r7["step"] == r3["step"] == 777
    for v in cases.MODEL_VARS[name]:
        assert np.array_equal(r7[v], r3[v]), v
    assert np.array_equal(r7["trackers"][0], r3["trackers"][0])
    lat3, lat7 = r3["trackers"][1], r7["trackers"][1]
    assert lat3.shape == lat7.shape and lat3.shape[0] >= 1
    assert np.array_equal(lat7, lat3, equal_nan=True)


def test_fused_march_rejects_probes(gc):
    """Variant 7 takes no probe trackers: asking for it with one raises
    (the automatic choice never picks it then)."""
    import finitewave_gb300 as fg
    case = _fused_case("ap", True, 144)
    m, _ = gc.build(case, npfloat="float32", form="fused", fused_k=4,
                    fused_variant=7)
    with pytest.raises(fg._ffi.FwError, match="probe"):
        m.run()


@pytest.mark.parametrize("name", ["ap", "ms", "fk"])
@pytest.mark.parametrize("k", [2, 3, 4, 8])
def test_fused_weights_on_chip(gc, name, k):
    """Variant 5 forms each region's AsymmetricStencil2D weights on chip in
    float32 from the fibers and myocyte flags (the stored weights are built
    in float64 and rounded): against the plain FP32 form with the fused
    tolerance -- activation steps within one step on >= 99.9 % of the
    nodes, fields and probe traces within 2e-3 -- and against variant 3 (the
    same kernel reading the stored weights) within the same bounds."""
    case = _fused_case(name, True, 144)
    ref = gc.run(case, npfloat="float32", form="plain")
    r3 = gc.run(case, npfloat="float32", form="fused", fused_k=k,
                fused_variant=3)
    r5 = gc.run(case, npfloat="float32", form="fused", fused_k=k,
                fused_variant=5)
    assert int(r5["model"]._status.item()) == 0
    assert r5["step"] == ref["step"] == 777
    for other in (ref, r3):
        assert _at_agree(r5["trackers"][0], other["trackers"][0], 0.01) >= 0.999
        for v in cases.MODEL_VARS[name]:
            np.testing.assert_allclose(r5[v], other[v], rtol=0, atol=2e-3)
            np.testing.assert_allclose(r5["trackers"][1][v],
                                       other["trackers"][1][v],
                                       rtol=0, atol=2e-3)


def test_fused_trackers_cable(gc):
    """LAT layers and the windowed AT tracker in the fused form (which takes
    up to two activation trackers and one LAT tracker; more fall back to the
    plain form)."""
    case, g = cases.trackers_cable()
    lat_c, at_c, at_def_c, at_win_c = case["trackers"]
    case1 = dict(case, trackers=[lat_c, at_c, at_win_c])
    m, _ = gc.build(case1, npfloat="float32", form="fused")
    m.initialize()
    assert m._form() == 1
    r = gc.run(case1, npfloat="float32", form="fused")
    lat, at, at_win = r["trackers"]
    assert lat.shape == g["lat"].shape
    assert np.abs(lat - g["lat"]).max() <= 0.01 + 1e-6
    assert _at_agree(at, g["act_t"], 0.01) == 1.0
    assert _at_agree(at_win, g["act_t_windowed"], 0.04) == 1.0
    r = gc.run(dict(case, trackers=[at_def_c]), npfloat="float32",
               form="fused")
    assert np.array_equal(r["trackers"][0],
                          g["act_t_default"].astype(np.float32))
    # four trackers: the automatic choice is the plain form
    m, _ = gc.build(case, npfloat="float32")
    m.initialize()
    assert m._form() == 0


def test_fused_stimuli_matrix_area(gc):
    case, g = cases.stimuli_2d()
    r = gc.run(case, npfloat="float32", form="fused")
    assert np.abs(r["u"] - g["u2d"]).max() < 1e-3
    assert _at_agree(r["trackers"][0], g["act_t2d"], 0.01) == 1.0


def test_diffusion_and_ionic_callables(fg, gc, oracle):
    """model.diffusion_kernel(u_new, u, w, indexes) and run_ionic_kernel on
    device tensors reproduce one oracle step bitwise."""
    case, _ = cases.ap2d_aniso_spiral()
    model, _ = gc.build(case)
    model.initialize()
    rng = np.random.default_rng(5)
    u0 = rng.uniform(0, 1, model._shape())
    v0 = rng.uniform(0, 0.5, model._shape())
    model.u = u0
    model.v = v0
    model.run_diffusion_kernel()
    model.run_ionic_kernel()
    torch.cuda.synchronize()
    w = oracle.weights("aniso9", case["mesh"], 1.0, case["dt"], case["dr"],
                       case["conductivity"], case["fibers"])
    idx = np.flatnonzero(case["mesh"] == 1).astype(np.int64)
    un = np.zeros_like(u0)
    v = v0.copy()
    oracle._diffuse("aniso9", un, u0, w, idx)
    oracle._ionic("ap", {"v": v}, un, u0, idx, case["dt"],
                  oracle.MODELS["ap"]["params"])
    assert np.array_equal(model.u_new, un)
    assert np.array_equal(model.v, v)


@pytest.mark.parametrize("npfloat", ["float64", "float32"])
@pytest.mark.parametrize("model", ["ap", "tp06"])
def test_in_plane_fibers_skip_zero_planes(gc, model, npfloat):
    """Fibers with no z component leave the eight 19-point weight planes
    that couple k +- 1 with i +- 1 or j +- 1 at zero; the model then steps
    with the 11-plane form (FW_STENCIL_ANISO19_XY), whose sums equal the
    full stencil's bit for bit (the skipped terms are exact zeros) -- read
    from the weight planes or from the table of distinct weight rows with a
    row index per node (weight_rows), which hold the same values."""
    from finitewave_gb300 import _ffi
    case, _ = cases.ap3d(True)
    fib = np.array(case["fibers"], dtype=np.float64)
    phi = np.linspace(-np.pi / 3, np.pi / 3, fib.shape[2])
    fib[..., 0] = np.cos(phi)[None, None, :]
    fib[..., 1] = np.sin(phi)[None, None, :]
    fib[..., 2] = 0.0
    case = dict(case, fibers=fib, model=model)
    if model == "tp06":
        case["t_max"] = 4
        case["stims"] = [dict(kind="current", t=0, value=80, duration=1.0,
                              box=[(0, 12), (0, 11), (1, 3)])]
        case["trackers"] = [dict(kind="at", threshold=-20.0)]
    outs = []
    for form in ("rows", "planes", "full"):
        m, objs = gc.build(case, npfloat=npfloat)
        m.initialize()
        assert m._step_stencil == _ffi.ANISO19_XY
        if form == "rows":
            m._weight_rows(force=True)
            assert m._wrows is not None
            assert m._wrows.shape[0] < m._widx.numel()
            # every node's row holds its eleven weights
            w = m.weights.reshape(m.weights.shape[0], -1)
            planes = w[[0, 1, 2, 3, 4, 5, 6, 7, 8, 11, 12]].t()
            assert torch.equal(m._wrows[m._widx.long(), :11], planes)
        else:
            m._wrows = None
        m._step_stencil = _ffi.ANISO19 if form == "full" else _ffi.ANISO19_XY
        m.run(initialize=False)
        outs.append((m.u, objs[0].output, getattr(m, m._state_names[-1])))
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)
    assert np.any(outs[0][0] != outs[0][0].flat[0])


def _wave_case():
    """Aliev-Panfilov 770 x 1024 (more fused regions than the GPU runs at
    once), 9-point stencil with smooth fibers, 20 % fibrosis, S1 and an S2
    on the lower-left quadrant at t = 3, activation tracker."""
    import scipy.ndimage as nd
    ni, nj = 770, 1024
    rng = np.random.default_rng(77)
    mesh = (1 + (rng.random((ni, nj)) <= 0.2)).astype(np.int8)
    mesh[0, :] = mesh[-1, :] = mesh[:, 0] = mesh[:, -1] = 0
    g = nd.gaussian_filter(rng.standard_normal((ni, nj)), 16)
    th = (np.pi / 4) * g / np.abs(g).max()
    fib = np.stack([np.cos(th), np.sin(th)], -1)
    return dict(model="ap", mesh=mesh, fibers=fib, stencil="aniso9",
                dt=0.01, dr=0.25, t_max=12.0,
                stims=[dict(kind="voltage", t=0, value=1.0,
                            box=[(0, ni), (1, 6)]),
                       dict(kind="voltage", t=3, value=1.0,
                            box=[(ni // 2, ni), (0, nj // 2)])],
                trackers=[dict(kind="at", threshold=0.5)])


def test_fused_bits_do_not_depend_on_tile_order(gc):
    """With many waves of regions per launch, every fused kernel and both
    batched kernels give the same bits, in one segment or in an odd one
    followed by the rest: each launch reads its regions' state from one
    buffer and writes the new state to the other, so no region sees state
    that a neighbouring region of the same launch has already advanced."""
    import finitewave_gb300 as fg
    case = _wave_case()

    def out(m, objs):
        return m.u, m.v, objs[0].output

    runs = {}
    for v in (1, 3, 4, 6, 7):
        m, objs = gc.build(case, npfloat="float32", form="fused", fused_k=4,
                           fused_variant=v)
        m.run()
        runs[f"v{v}"] = out(m, objs)
    m, objs = gc.build(case, npfloat="float32", form="fused", fused_k=4,
                       fused_variant=3)
    m.initialize()
    # the same 1200 steps as two device segments, an odd one first
    assert m._run_segment(555) + m._run_segment(645) == 1200
    runs["v3_split"] = out(m, objs)
    for kernel in ("tma", "pairs", "cp.async"):
        m, objs = gc.build(case, npfloat="float32")
        fg.TissueBatch([m], kernel=kernel, chunk=301).run()
        runs["batch_" + kernel] = out(m, objs)
    ref = runs.pop("v1")
    assert np.any(ref[2] > 3.0)        # the S2 wave activated nodes
    for k, r in runs.items():
        for a, b in zip(r, ref):
            assert np.array_equal(a, b), k
