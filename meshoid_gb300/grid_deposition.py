"""Grid deposition functions of the reference's ``meshoid.grid_deposition``
module (src/meshoid/grid_deposition.py) on the GPU: same names, arguments
and grid conventions; inputs are numpy arrays or torch tensors, results are
FP64 torch CUDA tensors.

* ``GridSurfaceDensity`` (:123-295) and ``GridAverage`` (:395-436): the
  tile-binned column deposit of ``mg_surface_density``;
  ``GridSurfaceDensityMultigrid`` (:89-113) deposits each level with it and
  carries the levels up with ``UpsampleGrid`` (:116-120), the bicubic
  interpolating spline applied as two FP64 matrix products on the device.
* ``GridDensity`` (:534-600), ``Grid_PPZ_DataCube`` (:339-392),
  ``Grid_PPZ_DataCube_Multigrid`` (:310-336) and ``WeightedGridInterp3D``
  (:439-531): the 3-D deposits of csrc/mg_deposit.cu.

All of them use the 2-D / 3-D spline kernels with support q <= 1 (the
reference's kernel2d / kernel3d leave q > 1 unassigned while these loops
evaluate them on every node of a particle's bounding square or cube).
"""
from __future__ import annotations

import functools
import threading

import numpy as np
import torch

from ._native import MeshoidError, check, load, ptr
from .meshoid import _stream

__all__ = ["grid_index_to_coordinate", "grid_dx_from_coordinate", "GridSurfaceDensity",
           "GridSurfaceDensityMultigrid", "UpsampleGrid", "UpsampleGrid_PPV", "GridAverage", "GridDensity",
           "Grid_PPZ_DataCube", "Grid_PPZ_DataCube_Multigrid", "WeightedGridInterp3D"]


def _dev(x, device=None):
    t = torch.as_tensor(x, dtype=torch.float64)
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device())
    return t.to(device).contiguous()


def _pos3(x, device):
    x = _dev(x, device)
    if x.ndim == 1:
        x = x[:, None]
    if x.shape[1] < 3:
        p = torch.zeros((x.shape[0], 3), dtype=torch.float64, device=device)
        p[:, :x.shape[1]] = x
        x = p
    return x[:, :3].contiguous()


def _device_of(*xs):
    for x in xs:
        if isinstance(x, torch.Tensor) and x.is_cuda:
            return x.device
    return torch.device("cuda", torch.cuda.current_device())


def _center3(center):
    c = [float(v) for v in (center.tolist() if isinstance(center, torch.Tensor) else list(center))]
    return (c + [0.0, 0.0, 0.0])[:3]


def grid_index_to_coordinate(index, grid_length, grid_center, N_grid, box_size=None):
    """Cell-centre coordinate of grid index i along one axis,
    grid_center - grid_length / 2 + grid_length / N_grid (i + 1/2), wrapped
    into [0, box_size) when box_size is given (grid_deposition.py:16-45);
    element-wise on the device."""
    i = torch.as_tensor(index, device=_device_of(index)).to(torch.float64)
    x = grid_center - 0.5 * grid_length + grid_length / N_grid * (0.5 + i)
    if box_size is not None:
        return torch.remainder(x, box_size)
    return x


def grid_dx_from_coordinate(x, index, grid_length, grid_center, N_grid, box_size=None):
    """Nearest-image difference from x to the centre of cell index
    (grid_deposition.py:48-85); element-wise on the device."""
    from .derivatives import nearest_image
    xg = grid_index_to_coordinate(index, grid_length, grid_center, N_grid, box_size)
    dx = xg - torch.as_tensor(x, dtype=torch.float64, device=xg.device)
    if box_size is not None:
        return nearest_image(dx, box_size)
    return dx


def GridSurfaceDensity(f, x, h, center, size, res=100, box_size=-1, parallel=True, conservative=False):
    """Column density on a (res, res) grid of pixel nodes (grid_deposition.py:123-295)."""
    lib = load()
    dev = _device_of(f, x, h)
    x3, ff, hh = _pos3(x, dev), _dev(f, dev), _dev(h, dev)
    c = _center3(center)
    n = x3.shape[0]
    grid = torch.empty((res, res), dtype=torch.float64, device=dev)
    wsb = lib.mg_surface_density_workspace_bytes(n, int(res))
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=dev)
    check(lib.mg_surface_density(ptr(x3), ptr(hh), ptr(ff), n, c[0], c[1], float(size), int(res),
                                 1 if conservative else 0, ptr(grid), ptr(ws), wsb, _stream()), "mg_surface_density")
    return grid


def _cubic_bspline_basis(t, x):
    """(len(x), len(t) - 4) values of the cubic B-splines on the knot vector t
    at the points x (Cox-de Boor recursion); a point equal to the last knot
    belongs to the last non-empty interval."""
    x = np.asarray(x, dtype=np.float64)
    span = np.clip(np.searchsorted(t, x, side="right") - 1, 3, len(t) - 5)
    b = np.zeros((len(x), len(t) - 1))
    b[np.arange(len(x)), span] = 1.0
    for d in range(1, 4):
        nb = np.zeros((len(x), len(t) - 1 - d))
        for j in range(len(t) - 1 - d):
            left, right = t[j + d] - t[j], t[j + d + 1] - t[j + 1]
            v = np.zeros(len(x))
            if left > 0:
                v += (x - t[j]) / left * b[:, j]
            if right > 0:
                v += (t[j + d + 1] - x) / right * b[:, j + 1]
            nb[:, j] = v
        b = nb
    return b[:, :len(t) - 4]


@functools.lru_cache(maxsize=32)
def _upsample_matrix(n):
    """(2n, n) FP64 matrix U with U @ g @ U.T == UpsampleGrid(g) for an (n, n)
    grid g (grid_deposition.py:116-120).  RectBivariateSpline(x1, x1, g) with
    s = 0 is the tensor product of 1-D cubic interpolating splines whose
    interior knots are x1[2:-2] (FITPACK's interpolation knots: the
    "not-a-knot" spline) on the cell centres x1 = (i + 1/2) / n; evaluating it
    at the finer centres x2 = (i + 1/4 ... ) / (2n) clamps points outside
    [x1[0], x1[-1]] to that interval, so the first and last rows copy the edge
    value.  U = E C^-1 with C the basis at x1 and E the basis at clamped x2."""
    if n < 4:
        raise ValueError("UpsampleGrid needs a grid of at least 4 x 4 cells")
    x1 = np.linspace(0.5 / n, 1 - 0.5 / n, n)
    x2 = np.linspace(0.25 / n, 1 - 0.25 / n, 2 * n)
    t = np.r_[[x1[0]] * 4, x1[2:n - 2], [x1[-1]] * 4]
    c = _cubic_bspline_basis(t, x1)
    e = _cubic_bspline_basis(t, np.clip(x2, x1[0], x1[-1]))
    u = np.linalg.solve(c.T, e.T).T
    u.setflags(write=False)
    return u


_upsample_dev = {}
_upsample_lock = threading.Lock()


def UpsampleGrid(grid):
    """Doubles an (N, N) map's resolution with the bicubic interpolating
    spline through its cell centres (grid_deposition.py:116-120), as
    U @ grid @ U.T in FP64 on the grid's device (N >= 4)."""
    dev = _device_of(grid)
    g = _dev(grid, dev)
    n = g.shape[0]
    if g.ndim != 2 or g.shape[1] != n:
        raise ValueError("UpsampleGrid needs a square 2-D grid")
    key = (n, str(dev))
    with _upsample_lock:
        u = _upsample_dev.get(key)
        if u is None:
            u = torch.from_numpy(np.array(_upsample_matrix(n))).to(dev)
            _upsample_dev[key] = u
    return u @ g @ u.T


def UpsampleGrid_PPV(grid):
    """Doubles the plane resolution of an (N, N, M) cube by 2x2 replication
    (grid_deposition.py:298-307)."""
    g = _dev(grid, _device_of(grid))
    return g.repeat_interleave(2, 0).repeat_interleave(2, 1)


def GridSurfaceDensityMultigrid(f, x, h, center, size, res=128, box_size=-1, N_grid_kernel=8, parallel=True):
    """Surface density built over maps of 8, 16, ..., res pixel nodes
    (grid_deposition.py:89-113): level i (2^(i+1) nodes) takes the particles
    with size / 2^(i+1) <= h / N_grid_kernel < size / 2^i, the finest level
    everything below; particles with h / N_grid_kernel >= size / 4 are not
    deposited.  Each level is a GridSurfaceDensity deposit added to the
    coarser levels carried up by UpsampleGrid.  res must be a power of 2 of
    at least 8 (the reference raises a string there, which is a TypeError)."""
    res = int(res)
    if not (res != 0 and res & (res - 1) == 0):
        raise ValueError("Multigrid resolution must be a power of 2")
    dev = _device_of(f, x, h)
    ff, x3, hh = _dev(f, dev), _pos3(x, dev), _dev(h, dev)
    bins = float(size) / 2.0 ** np.arange(0, round(np.log2(res) + 1))
    bins[0] = np.inf
    bins[-1] = 0.0
    grid = torch.zeros((4, 4), dtype=torch.float64, device=dev)
    hk = hh / N_grid_kernel
    for i in range(2, len(bins) - 1):
        grid = UpsampleGrid(grid)
        sel = (hk < bins[i]) & (hk >= bins[i + 1])
        if bool(sel.any()):
            grid += GridSurfaceDensity(ff[sel], x3[sel], hh[sel], center, size, res=grid.shape[0])
    return grid


def GridAverage(f, x, h, center, size, res=100, box_size=-1):
    """Column-weighted average of f along sightlines (grid_deposition.py:395-436)."""
    dev = _device_of(f, x, h)
    ff = _dev(f, dev)
    num = GridSurfaceDensity(ff, x, h, center, size, res)
    den = GridSurfaceDensity(torch.ones_like(ff), x, h, center, size, res)
    return num / den


def GridDensity(f, x, h, center, size, res=100, box_size=-1.0):
    """Density of a conserved quantity on a (res, res, res) grid
    (grid_deposition.py:534-600); box_size >= 0 wraps the deposit periodically."""
    lib = load()
    dev = _device_of(f, x, h)
    x3, ff, hh = _pos3(x, dev), _dev(f, dev), _dev(h, dev)
    c = _center3(center)
    periodic = box_size is not None and box_size >= 0
    n = x3.shape[0]
    grid = torch.empty((res, res, res), dtype=torch.float64, device=dev)
    skipped = torch.zeros(1, dtype=torch.int64, device=dev)
    npairs = torch.zeros(1, dtype=torch.int64, device=dev)
    check(lib.mg_grid_density_count(ptr(x3), ptr(hh), n, c[0], c[1], c[2], float(size), int(res),
                                    1 if periodic else 0, ptr(npairs), _stream()), "mg_grid_density_count")
    npairs = int(npairs.item())
    wsb = lib.mg_grid_density_workspace_bytes(n, npairs, int(res))
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=dev)
    check(lib.mg_grid_density(ptr(x3), ptr(hh), ptr(ff), n, c[0], c[1], c[2], float(size), int(res),
                              1 if periodic else 0, ptr(grid), ptr(skipped), npairs, ptr(ws), wsb, _stream()),
          "mg_grid_density")
    if periodic and int(skipped.item()) > 0:
        raise MeshoidError("GridDensity: %d particles span more than 4 res + 8 periodic grid nodes per axis"
                           % int(skipped.item()))
    return grid


def Grid_PPZ_DataCube(f, x, h, center, size, z, h_z, res, box_size=-1):
    """(res[0], res[0], res[1]) position-position-Z cube of f
    (grid_deposition.py:339-392): size = (plane side, Z extent), z and h_z the
    particles' data coordinate and its width, center[2] the Z centre."""
    lib = load()
    dev = _device_of(f, x, h, z, h_z)
    x3, ff, hh, zz, hz = _pos3(x, dev), _dev(f, dev), _dev(h, dev), _dev(z, dev), _dev(h_z, dev)
    c = _center3(center)
    size = [float(v) for v in (size.tolist() if isinstance(size, torch.Tensor) else list(size))]
    res = [int(v) for v in (res.tolist() if isinstance(res, torch.Tensor) else list(res))]
    grid = torch.empty((res[0], res[0], res[1]), dtype=torch.float64, device=dev)
    check(lib.mg_ppz_cube(ptr(x3), ptr(hh), ptr(ff), ptr(zz), ptr(hz), x3.shape[0], c[0], c[1], c[2], size[0],
                          size[1], res[0], res[1], ptr(grid), _stream()), "mg_ppz_cube")
    return grid


def Grid_PPZ_DataCube_Multigrid(f, x, h, center, size, z, h_z, res, box_size=-1, N_grid_kernel=8):
    """Multigrid PPZ cube (grid_deposition.py:310-336): plane resolutions
    2, 4, ..., res[0]; a particle is deposited (Grid_PPZ_DataCube) at the level
    whose node spacing brackets h / N_grid_kernel, and each level is carried to
    the next by 2x2 replication (UpsampleGrid_PPV :298-307).  res[0] must be a
    power of 2 (the reference raises a string there, which is a TypeError)."""
    res = [int(v) for v in (res.tolist() if isinstance(res, torch.Tensor) else list(res))]
    if not (res[0] != 0 and res[0] & (res[0] - 1) == 0):
        raise ValueError("Multigrid resolution must be a power of 2")
    dev = _device_of(f, x, h, z, h_z)
    ff, x3, hh, zz, hz = _dev(f, dev), _pos3(x, dev), _dev(h, dev), _dev(z, dev), _dev(h_z, dev)
    levels = int(round(np.log2(res[0])))
    bins = float(size[0]) / 2.0 ** np.arange(0, levels + 1)
    bins[0] = np.inf
    bins[-1] = 0.0
    grid = torch.zeros((1, 1, res[1]), dtype=torch.float64, device=dev)
    hk = hh / N_grid_kernel
    for i in range(levels):
        grid = grid.repeat_interleave(2, 0).repeat_interleave(2, 1)
        sel = (hk < bins[i]) & (hk >= bins[i + 1])
        if bool(sel.any()):
            grid += Grid_PPZ_DataCube(ff[sel], x3[sel], hh[sel], center, size, zz[sel], hz[sel],
                                      [grid.shape[0], res[1]])
    return grid


def WeightedGridInterp3D(f, wt, x, h, center, size, res=100, box_size=-1):
    """Weighted kernel interpolation of f to the (res, res, res) cell centres
    (grid_deposition.py:439-531); a cell that no particle's kernel reaches
    takes the f of the nearest particle (ties by index)."""
    lib = load()
    dev = _device_of(f, wt, x, h)
    x3, ff, ww, hh = _pos3(x, dev), _dev(f, dev), _dev(wt, dev), _dev(h, dev)
    c = _center3(center)
    result = torch.empty((res, res, res), dtype=torch.float64, device=dev)
    weight = torch.empty_like(result)
    n_empty = torch.zeros(1, dtype=torch.int64, device=dev)
    check(lib.mg_weighted_interp3d(ptr(x3), ptr(hh), ptr(ff), ptr(ww), x3.shape[0], c[0], c[1], c[2], float(size),
                                   int(res), ptr(result), ptr(weight), ptr(n_empty), _stream()),
          "mg_weighted_interp3d")
    if int(n_empty.item()) > 0:
        from .meshoid import Meshoid
        dx = float(size) / (res - 1)
        coord = torch.linspace(dx / 2 - float(size) / 2, float(size) / 2 - dx / 2, res, dtype=torch.float64,
                               device=dev)
        empty = torch.nonzero(weight == 0)
        targets = torch.stack([coord[empty[:, 0]], coord[empty[:, 1]], coord[empty[:, 2]]], 1)
        targets = targets + torch.tensor(c, dtype=torch.float64, device=dev)
        index = Meshoid(x3, kernel_radius=hh, des_ngb=max(1, min(32, x3.shape[0])))
        nn = index._nn(targets)
        result[empty[:, 0], empty[:, 1], empty[:, 2]] = ff[nn]
    return result
