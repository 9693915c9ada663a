"""Checkpoint and resume in the reference's on-disk format.

Mirrors ``core/state/state_saver.py`` and ``state_loader.py``: one
``<var>.npy`` per name in ``model.state_vars``, in the model's array shape
and dtype.  Reading a state variable copies it from the device; loading one
uploads it.
"""
from pathlib import Path

import numpy as np


class StateSaver:
    """Save the model state once ``t >= time`` (or at the end when
    ``time < 0``) (core/state/state_saver.py:4-92)."""

    def __init__(self, path=".", time=-1):
        self.path = path
        self.time = time
        self.model = None
        self.passed = False

    def initialize(self, model):
        self.model = model
        self.passed = self.path == ""

    def save(self):
        if self.passed:
            return
        if self.time < 0 and self.model.t < self.model.t_max:
            return
        if self.time >= 0 and self.model.t < self.time:
            return
        if not Path(self.path).exists():
            Path(self.path).mkdir(parents=True, exist_ok=True)
        for var in self.model.state_vars:
            np.save(Path(self.path).joinpath(var + ".npy"),
                    getattr(self.model, var))
        self.passed = True


class StateSaverCollection(StateSaver):
    """Several savers (core/state/state_saver.py:94-122)."""

    def __init__(self):
        super().__init__()
        self.savers = []

    def initialize(self, model):
        self.model = model
        for saver in self.savers:
            saver.initialize(model)

    def save(self):
        for saver in self.savers:
            saver.save()


class StateLoader:
    """Load every state variable from ``path`` before the run loop
    (core/state/state_loader.py)."""

    def __init__(self, path=""):
        self.path = path
        self.model = None
        self.passed = False

    def initialize(self, model):
        self.model = model
        self.passed = self.path == ""
        if not Path(self.path).exists():
            raise FileNotFoundError(f"Unable to load state from {self.path}. "
                                    "Directory does not exist.")

    def load(self):
        if self.passed:
            return
        for var in self.model.state_vars:
            setattr(self.model, var,
                    np.load(Path(self.path).joinpath(var + ".npy")))
        self.passed = True
