"""Module functions of the reference's ``meshoid.kernel_density``
(src/meshoid/kernel_density.py) on the GPU: same names and arguments; inputs
are numpy arrays, scalars or torch tensors, results are torch CUDA tensors.

* ``HsmlIter`` (:15-56): smoothing lengths from given neighbour distances,
  solved by ``mg_hsml_solve`` (the search-free entry of the h solve).
* ``Kernel`` (:82-96), ``kernel2d`` (:59-66), ``kernel3d`` (:69-76): the
  cubic spline, un-normalised and with its 2-D / 3-D normalisation, as
  element-wise device functions (0 beyond q = 1, where the reference's
  kernel2d / kernel3d assign nothing).
"""
from __future__ import annotations

import torch

from ._native import check, load, ptr
from .meshoid import _dev_tensor, _stream

__all__ = ["HsmlIter", "Kernel", "kernel2d", "kernel3d"]

# 40 / (7 pi) and 8 / pi: the 2-D and 3-D normalisations of the spline with
# support radius 1 (kernel_density.py:66,76)
_NORM2D = 40.0 / (7.0 * torch.pi)
_NORM3D = 8.0 / torch.pi


def _device():
    return torch.device("cuda", torch.cuda.current_device())


def _q_tensor(q):
    if isinstance(q, torch.Tensor):
        dev = q.device if q.is_cuda else _device()
        dt = q.dtype if q.dtype in (torch.float32, torch.float64) else torch.float64
        return q.to(device=dev, dtype=dt)
    return torch.as_tensor(q, dtype=torch.float64, device=_device())


def Kernel(q):
    """Un-normalised cubic spline W(q) = 1 - 6 q^2 + 6 q^3 (q <= 1/2),
    2 (1 - q)^3 (q <= 1), 0 beyond (kernel_density.py:82-96); FP32 inputs stay
    FP32, everything else is FP64."""
    q = _q_tensor(q)
    inner = 1 - 6 * q * q + 6 * q * q * q
    a = 1 - q
    outer = 2 * a * a * a
    zero = torch.zeros_like(q)
    return torch.where(q <= 0.5, inner, torch.where(q <= 1.0, outer, zero))


def kernel2d(q):
    """The spline normalised in 2-D, 40 / (7 pi) W(q) (kernel_density.py:59-66)."""
    return Kernel(q) * _NORM2D


def kernel3d(q):
    """The spline normalised in 3-D, 8 / pi W(q) (kernel_density.py:69-76)."""
    return Kernel(q) * _NORM3D


def HsmlIter(neighbor_dists, dim=3, error_norm=1e-6):
    """Smoothing lengths h with norm * sum_j W(d_j / h) = des_ngb, des_ngb the
    row length of neighbor_dists (N, des_ngb) and norm 32/3, 40/7, 8/3 in 3-D,
    2-D, 1-D (kernel_density.py:15-56).  The reference bisects until the
    neighbour number is within error_norm of des_ngb; mg_hsml_solve runs a
    bracketed Newton iteration on the FP32 squared distances to FP32
    round-off, within 1e-6 relative of the reference's h at any error_norm
    it is called with (error_norm is accepted for the signature).  Returns
    (N,) FP64."""
    lib = load()
    d = _dev_tensor(neighbor_dists, torch.float64, _device())
    if d.ndim != 2:
        raise ValueError("HsmlIter: neighbor_dists must be (N, des_ngb)")
    nq, k = d.shape
    if int(dim) not in (1, 2, 3):
        raise ValueError("HsmlIter: dim must be 1, 2 or 3")
    if nq == 0:
        return torch.empty(0, dtype=torch.float64, device=d.device)
    if k < 2:
        raise ValueError("HsmlIter: need at least 2 neighbour distances per row")
    if not bool(torch.isfinite(d).all()):
        raise ValueError("HsmlIter: neighbour distances must be finite")
    d2 = (d * d).float().contiguous()
    h = torch.empty(nq, dtype=torch.float32, device=d.device)
    check(lib.mg_hsml_solve(ptr(d2), nq, k, int(dim), ptr(h), None, _stream()), "mg_hsml_solve")
    return h.double()
