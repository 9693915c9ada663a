"""GPU: the reference's basics tests (tests/test_basics.py:8-80) through
the drop-in classes -- state save at t = 3 and reload, and a command that
excites the tissue by assigning into model.u -- plus a bitwise resume check:
saving at t = 3 and continuing from the saved state reproduces the
uninterrupted float64 run."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    import finitewave_gb300
    finitewave_gb300._ffi.load()
    return finitewave_gb300


def test_state_loading(fg, tmp_path):
    n = 5
    tissue = fg.CardiacTissue2D([n, n])
    stim = fg.StimSequence()
    stim.add_stim(fg.StimCurrentCoord2D(0, 10, 0.5, 1, n // 2, n // 2 + 1,
                                        n // 2, n // 2 + 1))
    saver = fg.StateSaverCollection()
    saver.savers.append(fg.StateSaver(str(tmp_path / "state_0"), time=3))
    model = fg.FentonKarma2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 5
    model.cardiac_tissue = tissue
    model.stim_sequence = stim
    model.state_saver = saver
    model.run()
    before = [model.u.copy(), model.v.copy(), model.w.copy()]
    model = fg.FentonKarma2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 5
    model.cardiac_tissue = tissue
    model.state_loader = fg.StateLoader(str(tmp_path / "state_0"))
    model.run()
    after = [model.u.copy(), model.v.copy(), model.w.copy()]
    for b, a in zip(before, after):
        assert np.allclose(b, a, atol=1e-5)


def test_commands(fg):
    n = 5
    tissue = fg.CardiacTissue2D([n, n])
    model = fg.FentonKarma2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 10

    class ExcitationCommand(fg.Command):
        def execute(self, model):
            model.u[1:-1, 1:-1] = 1

    seq = fg.CommandSequence()
    seq.add_command(ExcitationCommand(5))
    model.cardiac_tissue = tissue
    model.stim_sequence = fg.StimSequence()
    model.command_sequence = seq
    model.run()
    assert np.mean(model.u[1:-1, 1:-1]) > 0.5


@pytest.mark.parametrize("cls", ["AlievPanfilov2D", "TP063D"])
def test_resume_is_bitwise(fg, tmp_path, cls):
    """Run to t = 6 straight, or save at t = 3, reload into a fresh model
    (its clock restarted at the saved state) and run the remaining 3: the
    float64 states agree bit for bit."""
    shape = [20, 16] if cls.endswith("2D") else [10, 8, 6]

    def make(t_max):
        tissue = (fg.CardiacTissue2D if len(shape) == 2
                  else fg.CardiacTissue3D)(shape)
        m = getattr(fg, cls)()
        m.dt, m.dr, m.t_max = 0.01, 0.25, t_max
        m.cardiac_tissue = tissue
        seq = fg.StimSequence()
        if len(shape) == 2:
            seq.add_stim(fg.StimVoltageCoord2D(0, 1.0, 0, 20, 0, 3))
        else:
            seq.add_stim(fg.StimCurrentCoord3D(0, 100, 1.0, 0, 10, 0, 3, 0, 6))
        m.stim_sequence = seq
        return m

    ref = make(6)
    ref.run()
    first = make(3)
    # t after 300 steps of dt = 0.01 is 2.9999999999999796 < t_max: a
    # time < 0 saver (save at t >= t_max) would not fire, as in the
    # reference (state_saver.py:80-84); save at t >= 2.995 instead
    first.state_saver = fg.StateSaver(str(tmp_path / "s"), time=2.995)
    first.run()
    second = make(3)
    second.stim_sequence = fg.StimSequence()
    second.state_loader = fg.StateLoader(str(tmp_path / "s"))
    second.run()
    for var in ref.state_vars:
        assert np.array_equal(getattr(second, var), getattr(ref, var)), var


def test_nonfinite_potential_warns(fg):
    """A diverging run (Barkley with a strong stimulus, as in the
    reference, produces NaN) keeps the NaN results and warns."""
    tissue = fg.CardiacTissue2D([12, 12])
    model = fg.Barkley2D()
    model.dt, model.dr, model.t_max = 0.01, 0.25, 12
    model.cardiac_tissue = tissue
    seq = fg.StimSequence()
    seq.add_stim(fg.StimCurrentCoord2D(0, 5, 0.5, 0, 12, 0, 4))
    model.stim_sequence = seq
    with pytest.warns(RuntimeWarning, match="inf or NaN"):
        model.run()
    assert not np.isfinite(model.u).all()
