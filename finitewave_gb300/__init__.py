"""finitewave_gb300 -- Finitewave's explicit monodomain step on a GB300 GPU.

Drop-in GPU versions of the reference's model classes (``AlievPanfilov2D``,
``MitchellSchaeffer2D``, ``FentonKarma2D``, ``TP062D``,
``Courtemanche2D`` and their 3D variants) behind the
reference's own API: ``CardiacTissue2D/3D``, ``model.run()``,
``StimSequence`` with the coordinate / matrix / area stimuli,
``TrackerSequence`` with the activation-time, local-activation-time and
probe trackers, commands and state save / load.  The per-step work runs in
hand-written sm_103a CUDA (``libfwgpu.so``, C ABI in ``include/fwgpu.h``).
"""
from .batch import TissueBatch
from .command import Command, CommandSequence
from .fibrosis import Diffuse2DPattern, Diffuse3DPattern, FibrosisPattern
from .model import (AlievPanfilov2D, AlievPanfilov3D, Barkley2D, Barkley3D,
                    BuenoOrovio2D, BuenoOrovio3D, CardiacModel,
                    Courtemanche2D, Courtemanche3D, FentonKarma2D,
                    FentonKarma3D, LuoRudy912D, LuoRudy913D,
                    MitchellSchaeffer2D, MitchellSchaeffer3D, TP062D, TP063D)
from .serving import Request, SimulationServer, device_footprint
from .state import StateLoader, StateSaver, StateSaverCollection
from .stencil import (AsymmetricStencil2D, AsymmetricStencil3D,
                      IsotropicStencil2D, IsotropicStencil3D, Stencil,
                      SymmetricStencil2D)
from .stimulation import (Stim, StimCurrent, StimCurrentArea2D,
                          StimCurrentArea3D, StimCurrentCoord2D,
                          StimCurrentCoord3D, StimCurrentMatrix2D,
                          StimCurrentMatrix3D, StimSequence, StimVoltage,
                          StimVoltageCoord2D, StimVoltageCoord3D,
                          StimVoltageListMatrix3D, StimVoltageMatrix2D,
                          StimVoltageMatrix3D)
from .tissue import CardiacTissue, CardiacTissue2D, CardiacTissue3D
from .tracker import (ActionPotential2DTracker, ActionPotential3DTracker,
                      ActivationTime2DTracker, ActivationTime3DTracker,
                      ECG2DTracker, ECG3DTracker,
                      LocalActivationTime2DTracker,
                      LocalActivationTime3DTracker, MultiVariable2DTracker,
                      MultiVariable3DTracker, Period2DTracker,
                      Period3DTracker, SpiralWaveCore2DTracker,
                      SpiralWaveCore3DTracker, Tracker, TrackerSequence,
                      Variable2DTracker, Variable3DTracker)

__all__ = [n for n in dir() if not n.startswith("_")]
