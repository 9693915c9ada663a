"""Stencils: device weight construction and the diffusion-kernel callable.

Mirrors the reference's ``Stencil`` ABC (``core/stencil/stencil.py:14,38``)
and its four implementations.  ``compute_weights(model, tissue)`` builds the
weights on the GPU with ``fw_build_weights`` (float64 arithmetic in the
reference's order, bitwise equal to it) and returns a device tensor of shape
``(nw, *mesh.shape)`` -- weight-major, so that the step kernels read each
weight plane with coalesced loads; the reference returns ``(*mesh.shape,
nw)``.  ``select_diffusion_kernel()`` returns a callable with the reference's
``(u_new, u, w, indexes)`` signature over device tensors.
"""
import numpy as np
import torch

from . import _ffi


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _dev_f64(a, device):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if not a.flags.writeable:
        a = a.copy()
    return torch.as_tensor(a, device=device)


class Stencil:
    """Base class (core/stencil/stencil.py:4-46)."""

    kind = None  # one of _ffi.ISO5 / ANISO9 / ISO7 / ANISO19
    build_kind = None  # weight builder, when it differs from `kind`

    def compute_weights(self, model, cardiac_tissue):
        raise NotImplementedError

    def select_diffusion_kernel(self):
        return DiffusionKernel(self.kind)

    def _build(self, model, cardiac_tissue, fibers=None, D_al=1.0, D_ac=1.0):
        mesh = np.asarray(cardiac_tissue.mesh)
        shape = mesh.shape
        dim = 2 if self.kind in (_ffi.ISO5, _ffi.ANISO9) else 3
        if mesh.ndim != dim:
            raise ValueError(f"{type(self).__name__} needs a {dim}D mesh")
        device = model._device()
        mesh_d = torch.as_tensor(np.ascontiguousarray(mesh, dtype=np.int8),
                                 device=device)
        cond = cardiac_tissue.conductivity
        cond_d = None
        cond_scalar = 0.0
        if np.ndim(cond) == 0:
            cond_scalar = float(cond)
        else:
            cond_d = _dev_f64(np.broadcast_to(cond, shape), device)
        fib_d = None
        if fibers is not None:
            fibers = np.asarray(fibers)
            if fibers.shape != (*shape, dim):
                raise ValueError(f"fibers must have shape {(*shape, dim)}, "
                                 f"got {fibers.shape}")
            fib_d = _dev_f64(fibers, device)
        prec = model._precision()
        nw = _ffi.STENCIL_NW[self.kind]
        dtype = torch.float64 if prec == _ffi.F64 else torch.float32
        w = torch.empty((nw, *shape), dtype=dtype, device=device)
        nk = shape[2] if dim == 3 else 1
        _ffi.call("fw_build_weights", self.build_kind or self.kind, prec,
                  mesh_d.data_ptr(),
                  cond_d.data_ptr() if cond_d is not None else None,
                  cond_scalar, fib_d.data_ptr() if fib_d is not None else None,
                  float(D_al), float(D_ac), float(model.D_model),
                  float(model.dt), float(model.dr ** 2), shape[0], shape[1],
                  nk, w.data_ptr(), _stream())
        return w


class DiffusionKernel:
    """``diffusion_kernel(u_new, u, w, indexes)`` on device tensors.

    Replaces the numba callables diffusion_kernel_2d_iso/_aniso and
    diffusion_kernel_3d_iso/_aniso; u_new is written in place for the flat
    indices in ``indexes`` (numpy or device int64) and returned.
    """

    def __init__(self, kind):
        self.kind = kind

    def __call__(self, u_new, u, w, indexes):
        if not (isinstance(u_new, torch.Tensor) and u_new.is_cuda):
            raise TypeError("u_new must be a CUDA tensor")
        prec = _ffi.F64 if u.dtype == torch.float64 else _ffi.F32
        if u_new.dtype != u.dtype or w.dtype != u.dtype:
            raise TypeError("u_new, u and w must share one dtype")
        idx = torch.as_tensor(np.asarray(indexes, dtype=np.int64)
                              if not isinstance(indexes, torch.Tensor)
                              else indexes, device=u.device).to(torch.int64)
        idx = idx.contiguous()
        shape = u.shape
        nk = shape[2] if len(shape) == 3 else 1
        _ffi.call("fw_diffuse", self.kind, prec, u_new.data_ptr(),
                  u.data_ptr(), w.data_ptr(), idx.data_ptr(), idx.numel(),
                  shape[0], shape[1], nk, _stream())
        return u_new


class IsotropicStencil2D(Stencil):
    """5-point stencil (cpuwave2D/stencil/isotropic_stencil_2d.py:7-94)."""

    kind = _ffi.ISO5

    def compute_weights(self, model, cardiac_tissue):
        return self._build(model, cardiac_tissue)


class AsymmetricStencil2D(Stencil):
    """9-point anisotropic stencil (asymmetric_stencil_2d.py:7-161).

    D_al / D_ac are the longitudinal / cross-fiber diffusion ratios.
    """

    kind = _ffi.ANISO9

    def __init__(self):
        self.D_al = 1
        self.D_ac = 1 / 9

    def compute_weights(self, model, cardiac_tissue):
        if cardiac_tissue.fibers is None:
            raise ValueError("Fibers must be provided for anisotropic "
                             "diffusion.")
        return self._build(model, cardiac_tissue, cardiac_tissue.fibers,
                           self.D_al, self.D_ac)


class SymmetricStencil2D(AsymmetricStencil2D):
    """9-point symmetric anisotropic stencil (cpuwave2D/stencil/
    symmetric_stencil_2d.py:7-250): the diffusion tensor averaged to the
    cell corners and the flux of each corner cell split over its four
    nodes.  Same weight layout and diffusion kernel as AsymmetricStencil2D;
    only the weight construction differs (fw_build_weights with
    FW_STENCIL_SYM9)."""

    build_kind = _ffi.SYM9


class IsotropicStencil3D(Stencil):
    """7-point stencil (cpuwave3D/stencil/isotropic_stencil_3d.py:10-74)."""

    kind = _ffi.ISO7

    def compute_weights(self, model, cardiac_tissue):
        return self._build(model, cardiac_tissue)


class AsymmetricStencil3D(AsymmetricStencil2D):
    """19-point anisotropic stencil (asymmetric_stencil_3d.py:10-105)."""

    kind = _ffi.ANISO19
