"""Ray tracing of the reference's ``meshoid.radiation`` module
(src/meshoid/radiation/radtransfer.py) on the GPU: same names and
arguments; inputs numpy arrays or torch tensors, results FP64 torch CUDA
tensors (``csrc/mg_radtransfer.cu``).

``radtransfer_singlethread`` walks every pixel's particles from the largest z
to the smallest, as the reference does.  The reference's ``radtransfer``
splits the z-sorted particles into one slab per thread and composes the slabs
with the highest-z slab in front, while inside a slab the lowest z is in
front; with more than one thread its answer therefore depends on the thread
count.  Here ``radtransfer`` returns the single-thread answer (the reference's
on one thread), which both agree on.
"""
from __future__ import annotations

import torch

from ._native import check, load, ptr
from .meshoid import _stream


def _dev(x, device):
    return torch.as_tensor(x, dtype=torch.float64).to(device).contiguous()


def radtransfer_singlethread(j, m, kappa, x, h, gridres, L, center=0, i0=0):
    """(intensity, tau), each (gridres, gridres, bands): emission and
    absorption along z (radtransfer.py:87-200)."""
    lib = load()
    dev = next((t.device for t in (j, m, kappa, x, h) if isinstance(t, torch.Tensor) and t.is_cuda),
               torch.device("cuda", torch.cuda.current_device()))
    m = _dev(m, dev).reshape(-1)
    n = m.shape[0]
    j = _dev(j, dev)
    bands = j.shape[1] if j.ndim == 2 else 1
    j = j.reshape(n, bands)
    kappa = _dev(kappa, dev)
    kappa = (kappa.reshape(n, 1).expand(n, bands) if kappa.numel() == n and (kappa.ndim == 1 or bands == 1)
             else kappa.reshape(n, bands)).contiguous()
    x = _dev(x, dev)
    x = x.reshape(n, x.shape[-1] if x.ndim == 2 else 1)
    if x.shape[1] < 3:
        x = torch.cat([x, torch.zeros((n, 3 - x.shape[1]), dtype=torch.float64, device=dev)], 1).contiguous()
    h = _dev(h, dev).reshape(-1)
    c = torch.as_tensor(center, dtype=torch.float64).reshape(-1).cpu()
    c = (c.expand(3) if c.numel() == 1 else c[:3]).tolist()
    res = int(gridres)
    i0_img = None
    i0_band = None
    i0t = torch.as_tensor(i0, dtype=torch.float64)
    if i0t.numel() == 1 and float(i0t) == 0.0:
        pass
    elif i0t.ndim == 3:
        i0_img = _dev(i0t, dev).reshape(res, res, bands)
    else:
        i0_band = _dev(i0t.reshape(-1).expand(bands) if i0t.numel() == 1 else i0t.reshape(bands), dev)
    npairs_d = torch.zeros(1, dtype=torch.int64, device=dev)
    check(lib.mg_radtransfer_count(ptr(x), ptr(h), ptr(m), n, res, float(L), c[0], c[1], ptr(npairs_d), _stream()),
          "mg_radtransfer_count")
    npairs = int(npairs_d.item())
    wsb = lib.mg_radtransfer_workspace_bytes(n, npairs, res, bands)
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=dev)
    inten = torch.empty((res, res, bands), dtype=torch.float64, device=dev)
    tau = torch.empty_like(inten)
    check(lib.mg_radtransfer(ptr(j), ptr(m), ptr(kappa), ptr(x), ptr(h), n, bands, res, float(L), c[0], c[1], c[2],
                             ptr(i0_band) if i0_band is not None else None, npairs, ptr(inten), ptr(tau), ptr(ws), wsb,
                             _stream()), "mg_radtransfer")
    if i0_img is not None:
        inten = inten + i0_img * torch.exp(-tau)
    return inten, tau


def radtransfer(j, m, kappa, x, h, gridres, L, center=0, i0=0):
    """(gridres, gridres, bands) intensity (radtransfer.py:11-84, on one thread)."""
    return radtransfer_singlethread(j, m, kappa, x, h, gridres, L, center, i0)[0]
