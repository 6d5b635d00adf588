"""Module functions of the reference's ``meshoid.derivatives``
(src/meshoid/derivatives.py) on the GPU: same names and arguments; inputs are
numpy arrays or torch tensors, results are torch CUDA tensors.

* ``gradient_weights`` (:117-138): the (N, nd, k) least-squares derivative
  weights by ``mg_gradient_weights`` (one FP64 normal-matrix solve per
  query).  Its per-particle steps, ``kernel_dx_and_weights`` (:27-52) and
  ``polyfit_leastsq_matrices`` (:55-103), are fused into that kernel and not
  exposed on their own.
* ``nearest_image`` / ``nearest_image_v`` (:8-23): the minimum-image
  coordinate difference, element-wise on the device.
* ``get_num_derivs`` (:106-114): dim at order 1; 2, 5, 9 at order 2.
"""
from __future__ import annotations

import numpy as np
import torch

from ._native import check, load, ptr
from .meshoid import _dev_tensor, _stream

__all__ = ["gradient_weights", "nearest_image", "nearest_image_v", "get_num_derivs"]


def _device(*xs):
    for x in xs:
        if isinstance(x, torch.Tensor) and x.is_cuda:
            return x.device
    return torch.device("cuda", torch.cuda.current_device())


def get_num_derivs(dim, order):
    """Number of derivatives fitted: dim at order 1, else 2 / 5 / 9 in 1-D /
    2-D / 3-D (derivatives.py:106-114)."""
    if order == 1:
        return int(dim)
    return {1: 2, 2: 5, 3: 9}[int(dim)]


def nearest_image(dx_coord, boxsize):
    """dx_coord folded to its nearest periodic image for coordinates in
    [0, boxsize): values with |dx| > boxsize / 2 become
    -copysign(boxsize - |dx|, dx) (derivatives.py:8-14)."""
    dev = _device(dx_coord)
    dx = _dev_tensor(dx_coord, torch.float64, dev)
    box = float(boxsize)
    a = dx.abs()
    return torch.where(a > box / 2, -torch.copysign(box - a, dx), dx)


nearest_image_v = nearest_image


def gradient_weights(pos, ngb, kernel_radius, indices, boxsize=None, weighted=True, order=1):
    """(len(indices), nd, k) FP64 weights W with D(f)[i, d] = sum_j W[i, d, j]
    (f[ngb[i, j]] - f[indices[i]]) (derivatives.py:117-138): row i fits a
    polynomial of the given order to the neighbours ngb[i] of particle
    indices[i], weighted by Kernel(r / kernel_radius[i]) unless weighted is
    False, with minimum-image differences when boxsize is given.  An exactly
    singular moment matrix raises LinAlgError, as np.linalg.inv does there."""
    lib = load()
    dev = _device(pos, ngb, kernel_radius, indices)
    p = _dev_tensor(pos, torch.float64, dev)
    if p.ndim == 1:
        p = p[:, None].contiguous()
    dim = p.shape[1]
    if dim not in (1, 2, 3):
        raise ValueError("gradient_weights: positions must have 1, 2 or 3 coordinates")
    if order not in (1, 2):
        raise ValueError("gradient_weights: order must be 1 or 2")
    nb = _dev_tensor(ngb, torch.int64, dev)
    h = _dev_tensor(kernel_radius, torch.float64, dev)
    idx = _dev_tensor(indices, torch.int64, dev)
    nq = idx.shape[0]
    if nb.ndim != 2 or nb.shape[0] != nq or h.shape[0] != nq:
        raise ValueError("gradient_weights: ngb (N, k), kernel_radius (N,) and indices (N,) must agree")
    k = nb.shape[1]
    nd = get_num_derivs(dim, order)
    out = torch.zeros((nq, nd, k), dtype=torch.float64, device=dev)
    if nq == 0:
        return out
    # the kernel reads pos[ngb] and pos[indices] unchecked: a missing
    # neighbour (cKDTree marks one with the index N) must not reach it
    n = p.shape[0]
    lo = min(int(nb.min()), int(idx.min()))
    hi = max(int(nb.max()), int(idx.max()))
    if k < 1 or lo < 0 or hi >= n:
        raise IndexError("gradient_weights: neighbour and query indices must lie in [0, %d)" % n)
    nsing = torch.zeros(1, dtype=torch.int64, device=dev)
    box = float(boxsize) if boxsize is not None else -1.0
    check(lib.mg_gradient_weights(ptr(p), dim, ptr(nb), k, ptr(h), ptr(idx), nq, box, 1 if weighted else 0,
                                  int(order), ptr(out), ptr(nsing), _stream()), "mg_gradient_weights")
    if int(nsing.item()) > 0:
        raise np.linalg.LinAlgError("Singular matrix")
    return out
