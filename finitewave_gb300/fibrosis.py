"""Fibrosis patterns: mesh code 2 (fibrosis) drawn per node.

Restates the reference's diffuse patterns (cpuwave2D/fibrosis/
diffuse_2d_pattern.py:24-87, cpuwave3D/fibrosis/diffuse_3d_pattern.py:
27-89) with the same draws from numpy's global generator -- one
``np.random.random(shape)`` over the whole mesh, code ``1 + (r <= density)``
copied into the pattern's box -- so that a given ``np.random.seed`` yields the
reference's mesh node for node.  Input generation on the host: the pattern
is drawn once, before the tissue goes to the device.
"""
from abc import ABC, abstractmethod

import numpy as np


class FibrosisPattern(ABC):
    """core/fibrosis/fibrosis_pattern.py:4-60."""

    @abstractmethod
    def generate(self, shape=None, mesh=None):
        """Return a mesh with the pattern applied."""

    def apply(self, cardiac_tissue):
        cardiac_tissue.mesh = self.generate(mesh=cardiac_tissue.mesh)


def _draw(density, shape):
    return 1 + (np.random.random(shape) <= density).astype(np.int8)


class Diffuse2DPattern(FibrosisPattern):
    """Diffuse fibrosis in the box [x1:x2, y1:y2] (the whole mesh when the
    bounds are None)."""

    def __init__(self, density, x1=None, x2=None, y1=None, y2=None):
        self.x1, self.x2, self.y1, self.y2 = x1, x2, y1, y2
        self.density = density

    def generate(self, shape=None, mesh=None):
        if shape is None and mesh is None:
            raise ValueError("Either shape or mesh must be provided.")
        if shape is not None:
            mesh = np.ones(shape, dtype=np.int8)
        fibr = _draw(self.density, mesh.shape)
        box = (slice(self.x1, self.x2), slice(self.y1, self.y2))
        mesh[box] = fibr[box]
        return mesh


class Diffuse3DPattern(FibrosisPattern):
    """Diffuse fibrosis in the box [x1:x2, y1:y2, z1:z2].  The reference's
    ``apply`` calls ``generate`` without its positional ``shape`` and its
    mesh path indexes z with two scalars (diffuse_3d_pattern.py:81-84);
    here both paths fill the box, drawing the same random numbers."""

    def __init__(self, x1, x2, y1, y2, z1, z2, density):
        self.x1, self.x2, self.y1, self.y2 = x1, x2, y1, y2
        self.z1, self.z2 = z1, z2
        self.density = density

    def generate(self, shape=None, mesh=None):
        if shape is None and mesh is None:
            raise ValueError("Either shape or mesh must be provided.")
        if shape is not None:
            mesh = np.ones(shape, dtype=np.int8)
        fibr = _draw(self.density, mesh.shape)
        box = (slice(self.x1, self.x2), slice(self.y1, self.y2),
               slice(self.z1, self.z2))
        mesh[box] = fibr[box]
        return mesh
