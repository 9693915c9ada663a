"""GPU: the fused-kernel autotuner times the candidates on scratch copies
(the model, its trackers and stimuli are untouched), caches the winner per
configuration, and the chosen kernel's run agrees with the plain form."""
import json

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu


@pytest.fixture()
def env(tmp_path, monkeypatch):
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    monkeypatch.setenv("FWGPU_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    from finitewave_gb300 import _ffi, autotune
    _ffi.load()
    autotune._memo.clear()
    import gpu_cases
    return gpu_cases, autotune, tmp_path / "tune.json"


def test_autotune_picks_and_caches(env):
    gc, autotune, path = env
    case, _ = cases.ap2d_aniso_spiral()
    model, objs = gc.build(case, npfloat="float32")
    model.initialize()
    u0 = model.u.copy()
    v, k = autotune.choose(model)
    assert (v, k) in autotune._TMA + autotune._CPASYNC
    assert np.array_equal(model.u, u0)          # scratch copies only
    table = json.loads(path.read_text())
    entry = table[autotune.key(model)]
    assert (entry["variant"], entry["k"]) == (v, k) and entry["ms"]
    autotune._memo.clear()
    assert autotune.choose(model) == (v, k)      # from the file


def test_autotuned_run_matches_plain(env):
    gc, autotune, _ = env
    case, _ = cases.models_2d("fk", True)
    fused = gc.run(case, npfloat="float32")      # autotune on by default
    assert fused["model"]._fused_choice is not None
    plain = gc.run(case, npfloat="float32", form="plain")
    for var in cases.MODEL_VARS["fk"]:
        np.testing.assert_allclose(fused[var], plain[var], rtol=0, atol=5e-3)
