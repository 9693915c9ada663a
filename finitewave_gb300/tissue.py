"""Cardiac tissue: the mesh of node codes, fibers and conductivity.

Mirrors ``core/tissue/cardiac_tissue.py`` and ``cpuwave2D/tissue/
cardiac_tissue_2d.py`` / ``cpuwave3D/tissue/cardiac_tissue_3d.py`` of the
reference: mesh codes 0 (no tissue), 1 (myocyte), 2 (fibrosis); the setter
zeroes the outer ring of nodes; ``myo_indexes`` are the flat indices of
``mesh == 1`` (and ``special_boundaries == 0`` when given).  The tissue lives
on the host as numpy arrays, as in the reference; the model uploads it.
"""
import copy

import numpy as np


class CardiacTissue:
    """Base class of a tissue (core/tissue/cardiac_tissue.py:6-100)."""

    def __init__(self):
        self.meta = {}
        self.special_boundaries = None

    @property
    def mesh(self):
        return self._mesh

    @mesh.setter
    def mesh(self, mesh):
        # cardiac_tissue.py:38-52
        if mesh.ndim != self.meta["dim"]:
            raise ValueError("Mesh dimension must match the tissue dimension.")
        self._mesh = mesh
        self.add_boundaries()

    def compute_myo_indexes(self):
        """Flat indices of myocytes (cardiac_tissue.py:54-63)."""
        if self.special_boundaries is not None:
            self.myo_indexes = np.flatnonzero((self.mesh == 1) &
                                              (self.special_boundaries == 0))
            return
        self.myo_indexes = np.flatnonzero(self.mesh == 1)

    def add_boundaries(self):
        raise NotImplementedError

    def add_pattern(self, fibro_pattern):
        fibro_pattern.apply(self)

    def clean(self):
        """Set every fibrosis node (code 2) back to 1 (cardiac_tissue.py:84-89)."""
        self.mesh[self.mesh == 2] = 1

    def clone(self):
        return copy.deepcopy(self)


class CardiacTissue2D(CardiacTissue):
    """2D tissue (cpuwave2D/tissue/cardiac_tissue_2d.py:6-45)."""

    def __init__(self, shape):
        super().__init__()
        self.meta["dim"] = 2
        self.meta["shape"] = shape
        self.mesh = np.ones(shape, dtype=np.int8)
        self.conductivity = 1.0
        self.fibers = None

    def add_boundaries(self):
        self._mesh[0, :] = 0
        self._mesh[:, 0] = 0
        self._mesh[-1, :] = 0
        self._mesh[:, -1] = 0


class CardiacTissue3D(CardiacTissue):
    """3D tissue (cpuwave3D/tissue/cardiac_tissue_3d.py:6-46)."""

    def __init__(self, shape):
        super().__init__()
        self.meta["dim"] = 3
        self.meta["shape"] = shape
        self.mesh = np.ones(shape, dtype=np.int8)
        self.conductivity = 1.0
        self.fibers = None

    def add_boundaries(self):
        self.mesh[0, :, :] = 0
        self.mesh[:, 0, :] = 0
        self.mesh[:, :, 0] = 0
        self.mesh[-1, :, :] = 0
        self.mesh[:, -1, :] = 0
        self.mesh[:, :, -1] = 0
