"""CPU oracle for the meshoid particle-neighbourhood path (TEST INFRASTRUCTURE).

This module is the checker used by ``tests/``, ``__graft_entry__.smoke()`` and
by ``bench.py``'s CPU-baseline arm.  The product package (``meshoid_gb300``)
never imports it.

* Neighbour search: ``scipy.spatial.cKDTree.query`` -- the same third-party
  call the reference makes (src/meshoid/Meshoid.py:145,157,410) -- followed by
  the exact-set rule ``orc_knn_decide`` (k smallest by FP64 (d2, index)).
* Everything else: ``meshoid_oracle.c``, a plain-C FP64 restatement of
  HsmlIter (src/meshoid/kernel_density.py:15-56), gradient_weights
  (src/meshoid/derivatives.py:27-138), KernelAverage (src/meshoid/Meshoid.py:
  172-177,368-381), GridSurfaceDensity(_conservative)_core
  (src/meshoid/grid_deposition.py:187-295; its multigrid schedule :89-120
  carries levels up with scipy's RectBivariateSpline, as the reference does),
  Grid_PPZ_DataCube (:339-392),
  WeightedGridInterp3D (:439-531), GridDensity (:534-600) and
  radtransfer_singlethread (src/meshoid/radiation/radtransfer.py:87-200).
* ``OracleMeshoid`` mirrors the reference's ``Meshoid`` class
  (src/meshoid/Meshoid.py:12-750) on top of those functions.

The oracle is pinned against golden vectors produced by the reference itself
(tests/golden/make_golden.py), see tests/test_oracle.py.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

__all__ = [
    "build_oracle",
    "load_oracle",
    "knn",
    "hsml_iter",
    "gradient_weights",
    "apply_weights",
    "kernel_average",
    "surface_density",
    "surface_density_multigrid",
    "upsample_grid",
    "grid_density",
    "ppz_cube",
    "weighted_interp3d",
    "ppz_cube_multigrid",
    "radtransfer",
    "moment_condition",
    "OracleMeshoid",
    "set_threads",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmeshoid_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)


def build_oracle(force: bool = False) -> str:
    """Compile meshoid_oracle.c with gcc (-O3 -fopenmp, no FP contraction)."""
    src = os.path.join(_HERE, "meshoid_oracle.c")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)):
        return _LIB_PATH
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c11",
           "-shared", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def load_oracle():
    global _lib
    if _lib is not None:
        return _lib
    build_oracle()
    lib = ctypes.CDLL(_LIB_PATH)
    lib.orc_num_threads.restype = ctypes.c_int
    lib.orc_set_num_threads.argtypes = [ctypes.c_int]
    lib.orc_hsml_iter.restype = ctypes.c_int64
    lib.orc_hsml_iter.argtypes = [_dp, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_double, ctypes.c_int, _dp]
    lib.orc_gradient_weights.restype = ctypes.c_int64
    lib.orc_gradient_weights.argtypes = [_dp, ctypes.c_int, _i64p, ctypes.c_int, _dp, _i64p,
                                         ctypes.c_int64, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_int, _dp]
    lib.orc_apply_weights.restype = None
    lib.orc_apply_weights.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i64p,
                                      ctypes.c_int, _i64p, ctypes.c_int64, _dp, ctypes.c_int, _dp]
    lib.orc_kernel_average.restype = None
    lib.orc_kernel_average.argtypes = [_dp, _i64p, ctypes.c_int, _dp, ctypes.c_int64, _dp, _dp]
    lib.orc_surface_density.restype = None
    lib.orc_surface_density.argtypes = [_dp, _dp, _dp, ctypes.c_int64, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_int, _dp]
    lib.orc_grid_density.restype = None
    lib.orc_grid_density.argtypes = [_dp, _dp, _dp, ctypes.c_int64, _dp, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_double, _dp]
    lib.orc_ppz_cube.restype = None
    lib.orc_ppz_cube.argtypes = [_dp, _dp, _dp, _dp, _dp, ctypes.c_int64, _dp, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_int, ctypes.c_int, _dp]
    lib.orc_weighted_interp3d.restype = None
    lib.orc_weighted_interp3d.argtypes = [_dp, _dp, _dp, _dp, ctypes.c_int64, _dp, ctypes.c_double, ctypes.c_int,
                                          _dp]
    lib.orc_radtransfer.restype = None
    lib.orc_radtransfer.argtypes = [_dp, _dp, _dp, _dp, _dp, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, _dp, _dp, _dp, _dp]
    lib.orc_knn_decide.restype = None
    lib.orc_knn_decide.argtypes = [_dp, ctypes.c_int, _i64p, ctypes.c_int64, _i64p, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_double, _i64p, _dp]
    _lib = lib
    return lib


def set_threads(n: int) -> int:
    lib = load_oracle()
    if n and n > 0:
        lib.orc_set_num_threads(int(n))
    return lib.orc_num_threads()


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int64)
    return a, a.ctypes.data_as(_i64p)


def knn(pos, k, boxsize=None, queries=None, extra=8, workers=-1, tree=None):
    """k nearest neighbours (self included) of pos[queries] among pos.

    cKDTree proposes k+extra candidates; the exact set is then decided as the
    k smallest by (FP64 d2, index).  Returns (dist (Nq,k) f64, ngb (Nq,k) i64),
    ascending like cKDTree.query.
    """
    from scipy.spatial import cKDTree

    pos = np.ascontiguousarray(pos, dtype=np.float64)
    n, dim = pos.shape
    if queries is None:
        queries = np.arange(n)
    queries = np.asarray(queries, dtype=np.int64)
    kc = min(n, k + extra)
    if tree is None:
        tree = cKDTree(pos, boxsize=boxsize)
    cd, cand = tree.query(pos[queries], kc, workers=workers)
    cand = np.asarray(cand, dtype=np.int64).reshape(len(queries), kc)
    cd = np.asarray(cd).reshape(len(queries), kc)
    # Exact ties can straddle the k-th place; cKDTree orders tied points
    # arbitrarily, so rows whose last candidate is (nearly) as close as the k-th
    # are re-queried with more candidates until every tie is included.
    while kc < n:
        need = cd[:, -1] <= cd[:, k - 1] * (1 + 1e-9) + 1e-300
        if not need.any():
            break
        kc2 = min(n, 2 * kc)
        d2, c2 = tree.query(pos[queries[need]], kc2, workers=workers)
        grow_c = np.full((len(queries), kc2), n, dtype=np.int64)
        grow_d = np.full((len(queries), kc2), np.inf)
        grow_c[:, :kc] = cand
        grow_d[:, :kc] = cd
        grow_c[need] = np.asarray(c2).reshape(-1, kc2)
        grow_d[need] = np.asarray(d2).reshape(-1, kc2)
        cand, cd, kc = grow_c, grow_d, kc2
    cand = np.where(cand >= n, -1, cand)
    lib = load_oracle()
    ngb = np.empty((len(queries), k), dtype=np.int64)
    dist = np.empty((len(queries), k), dtype=np.float64)
    posc, pp = _d(pos)
    qc, qp = _i(queries)
    cc, cp = _i(cand)
    lib.orc_knn_decide(pp, dim, qp, len(queries), cp, kc, k,
                       float(boxsize) if boxsize else -1.0,
                       ngb.ctypes.data_as(_i64p), dist.ctypes.data_as(_dp))
    return dist, ngb


def hsml_iter(ngbdist, dim=3, error_norm=1e-13, max_iter=500):
    """kernel_density.py:15-56 (HsmlIter), FP64; returns (h, n_capped)."""
    lib = load_oracle()
    d, dp = _d(ngbdist)
    n, k = d.shape
    out = np.empty(n)
    capped = lib.orc_hsml_iter(dp, n, k, dim, error_norm, max_iter, out.ctypes.data_as(_dp))
    return out, int(capped)


def num_derivs(dim, order):
    return dim if order == 1 else {1: 2, 2: 5, 3: 9}[dim]


def gradient_weights(pos, ngb, h, indices, boxsize=None, weighted=True, order=1):
    """derivatives.py:118-138 (gradient_weights): (Nq, nd, k) FP64 weights."""
    lib = load_oracle()
    pos, pp = _d(pos)
    if pos.ndim == 1:
        pos = pos[:, None]
    dim = pos.shape[1]
    ngb, np_ = _i(ngb)
    hh, hp = _d(h)
    idx, ip = _i(indices)
    nq, k = ngb.shape
    nd = num_derivs(dim, order)
    out = np.zeros((nq, nd, k))
    sing = lib.orc_gradient_weights(pp, dim, np_, k, hp, ip, nq,
                                    float(boxsize) if boxsize else -1.0,
                                    1 if weighted else 0, order, out.ctypes.data_as(_dp))
    return out, int(sing)


def moment_condition(pos, ngb, h, indices, boxsize=None, order=1, weighted=True):
    """2-norm condition number of each particle's least-squares moment matrix
    (derivatives.py:56-103 with coordinates scaled by h).  Rows whose matrix is
    near-singular have no reproducible FP64 answer (LAPACK and any other
    elimination order disagree), so tests compare only well-conditioned rows."""
    pos = np.asarray(pos, dtype=np.float64)
    if pos.ndim == 1:
        pos = pos[:, None]
    dim = pos.shape[1]
    ngb = np.asarray(ngb)
    idx = np.asarray(indices)
    dx = pos[ngb] - pos[idx][:, None, :]
    if boxsize:
        dx = _nearest_image_v(dx, boxsize)
    hh = np.asarray(h, dtype=np.float64)[:, None]
    w = _kernel(np.linalg.norm(dx, axis=2) / hh) if weighted else np.ones(ngb.shape)
    a = dx / hh[:, :, None]
    if order == 2:
        cols = [a[..., d] for d in range(dim)] + [0.5 * a[..., d] ** 2 for d in range(dim)]
        if dim > 1:
            cols += [a[..., d % dim] * a[..., (d + 1) % dim] for d in range(num_derivs(dim, 2) - 2 * dim)]
        a = np.stack(cols, axis=-1)
    M = np.einsum("ij,ijk,ijl->ikl", w, a, a)
    return np.linalg.cond(M)


def apply_weights(W, ngb, indices, f, row0=0, nrows=None):
    """Meshoid.py:258,268: einsum('ikj,ij...->i...k', W, f[ngb] - f[mask])."""
    lib = load_oracle()
    W, wp = _d(W)
    nq, nd_total, k = W.shape
    if nrows is None:
        nrows = nd_total - row0
    f = np.asarray(f, dtype=np.float64)
    fshape = f.shape[1:]
    f2 = np.ascontiguousarray(f.reshape(f.shape[0], -1))
    nc = f2.shape[1]
    ngb, np_ = _i(ngb)
    idx, ip = _i(indices)
    top = max(int(ngb.max(initial=0)), int(idx.max(initial=0)))
    if top >= f2.shape[0]:  # numpy's np.take / fancy indexing raise here (Meshoid.py:258)
        raise IndexError(f"index {top} is out of bounds for axis 0 with size {f2.shape[0]}")
    out = np.empty((nq, nc, nrows))
    lib.orc_apply_weights(wp, nd_total, row0, nrows, np_, k, ip, nq,
                          f2.ctypes.data_as(_dp), nc, out.ctypes.data_as(_dp))
    return out.reshape((nq,) + fshape + (nrows,))


def kernel_average(ngbdist, ngb, h, f):
    lib = load_oracle()
    d, dp = _d(ngbdist)
    ngb, np_ = _i(ngb)
    hh, hp = _d(h)
    ff, fp = _d(f)
    nq, k = d.shape
    out = np.empty(nq)
    lib.orc_kernel_average(dp, np_, k, hp, nq, fp, out.ctypes.data_as(_dp))
    return out


def surface_density(f, x, h, center, size, res, conservative=False):
    """grid_deposition.py:123-295 (GridSurfaceDensity): (res, res) FP64 map."""
    lib = load_oracle()
    ff, fp = _d(f)
    x = np.asarray(x, dtype=np.float64)
    if x.shape[1] < 3:
        x = np.c_[x, np.zeros((x.shape[0], 3 - x.shape[1]))]
    xx, xp = _d(x)
    hh, hp = _d(h)
    out = np.empty((res, res))
    lib.orc_surface_density(fp, xp, hp, len(ff), float(center[0]), float(center[1]),
                            float(size), int(res), 1 if conservative else 0,
                            out.ctypes.data_as(_dp))
    return out


def upsample_grid(grid):
    """UpsampleGrid (grid_deposition.py:116-120): scipy's RectBivariateSpline
    through the N^2 cell centres, evaluated at the (2N)^2 finer centres --
    the same third-party call the reference makes."""
    from scipy.interpolate import RectBivariateSpline
    n = grid.shape[0]
    x1 = np.linspace(0.5 / n, 1 - 0.5 / n, n)
    x2 = np.linspace(0.25 / n, 1 - 0.25 / n, 2 * n)
    return RectBivariateSpline(x1, x1, grid)(x2, x2)


def surface_density_multigrid(f, x, h, center, size, res=128, N_grid_kernel=8):
    """GridSurfaceDensityMultigrid (grid_deposition.py:89-113): maps of 8, 16,
    ..., res nodes; a particle goes to the level whose size / 2^(i+1) <=
    h / 8 < size / 2^i (the finest takes everything below), each level is
    carried to the next by upsample_grid."""
    if not (res != 0 and res & (res - 1) == 0):
        raise ValueError("Multigrid resolution must be a power of 2")
    h = np.asarray(h, dtype=np.float64)
    bins = float(size) / 2.0 ** np.arange(0, round(np.log2(res) + 1))
    bins[0] = np.inf
    bins[-1] = 0
    grid = np.zeros((4, 4))
    for i in range(2, len(bins) - 1):
        grid = upsample_grid(grid)
        idx = (h / N_grid_kernel < bins[i]) & (h / N_grid_kernel >= bins[i + 1])
        if np.any(idx):
            grid += surface_density(np.asarray(f)[idx], np.asarray(x)[idx], h[idx], center, size, grid.shape[0])
    return grid


def _pos3(x):
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x[:, None]
    if x.shape[1] < 3:
        x = np.c_[x, np.zeros((x.shape[0], 3 - x.shape[1]))]
    return np.ascontiguousarray(x)


def grid_density(f, x, h, center, size, res=100, box_size=-1.0):
    """GridDensity (grid_deposition.py:534-600): (res, res, res) FP64 density grid."""
    lib = load_oracle()
    ff, fp = _d(f)
    xx, xp = _d(_pos3(x))
    hh, hp = _d(h)
    cc, cp = _d(np.asarray(center, dtype=np.float64)[:3])
    out = np.empty((res, res, res))
    lib.orc_grid_density(fp, xp, hp, len(ff), cp, float(size), int(res),
                         -1.0 if box_size is None else float(box_size), out.ctypes.data_as(_dp))
    return out


def ppz_cube(f, x, h, center, size, z, h_z, res):
    """Grid_PPZ_DataCube (grid_deposition.py:339-392): (res[0], res[0], res[1])."""
    lib = load_oracle()
    ff, fp = _d(f)
    xx, xp = _d(_pos3(x))
    hh, hp = _d(h)
    zz, zp = _d(z)
    hz, hzp = _d(h_z)
    cc, cp = _d(np.asarray(center, dtype=np.float64)[:3])
    out = np.empty((int(res[0]), int(res[0]), int(res[1])))
    lib.orc_ppz_cube(fp, xp, hp, zp, hzp, len(ff), cp, float(size[0]), float(size[1]), int(res[0]), int(res[1]),
                     out.ctypes.data_as(_dp))
    return out


def ppz_cube_multigrid(f, x, h, center, size, z, h_z, res, N_grid_kernel=8):
    """Grid_PPZ_DataCube_Multigrid (grid_deposition.py:310-336): levels of
    2^l plane nodes, each particle deposited at the level its h / 8 falls in,
    coarser levels upsampled by 2x2 replication (UpsampleGrid_PPV :298-307)."""
    res0 = int(res[0])
    if not (res0 != 0 and res0 & (res0 - 1) == 0):
        raise ValueError("Multigrid resolution must be a power of 2")
    h = np.asarray(h, dtype=np.float64)
    bins = float(size[0]) / 2.0 ** np.arange(0, round(np.log2(res0) + 1))
    bins[0] = np.inf
    bins[-1] = 0
    grid = np.zeros((1, 1, int(res[1])))
    for i in range(len(bins) - 1):
        grid = grid.repeat(2, 0).repeat(2, 1)
        ni = grid.shape[0]
        idx = (h / N_grid_kernel < bins[i]) & (h / N_grid_kernel >= bins[i + 1])
        if np.any(idx):
            grid += ppz_cube(np.asarray(f)[idx], np.asarray(x)[idx], h[idx], center, size, np.asarray(z)[idx],
                             np.asarray(h_z)[idx], [ni, int(res[1])])
    return grid


def weighted_interp3d(f, wt, x, h, center, size, res=100):
    """WeightedGridInterp3D (grid_deposition.py:439-531): (res, res, res)."""
    lib = load_oracle()
    ff, fp = _d(f)
    ww, wp = _d(wt)
    xx, xp = _d(_pos3(x))
    hh, hp = _d(h)
    cc, cp = _d(np.asarray(center, dtype=np.float64)[:3])
    out = np.empty((res, res, res))
    lib.orc_weighted_interp3d(fp, wp, xp, hp, len(ff), cp, float(size), int(res), out.ctypes.data_as(_dp))
    return out


def radtransfer(j, m, kappa, x, h, gridres, L, center=0, i0=0):
    """radtransfer_singlethread (radtransfer.py:87-200): (I, tau), each
    (gridres, gridres, bands)."""
    lib = load_oracle()
    jj = np.ascontiguousarray(np.asarray(j, dtype=np.float64).reshape(len(m), -1))
    bands = jj.shape[1]
    kk = np.ascontiguousarray(np.asarray(kappa, dtype=np.float64).reshape(len(m), bands))
    mm, mp = _d(m)
    xx, xp = _d(_pos3(x))
    hh, hp = _d(h)
    cc, cp = _d(np.broadcast_to(np.asarray(center, dtype=np.float64), (3,)).copy())
    ii = None if np.isscalar(i0) and i0 == 0 else np.ascontiguousarray(np.broadcast_to(
        np.asarray(i0, dtype=np.float64), (bands,)))
    inten = np.empty((gridres, gridres, bands))
    tau = np.empty_like(inten)
    lib.orc_radtransfer(jj.ctypes.data_as(_dp), mp, kk.ctypes.data_as(_dp), xp, hp, len(mm), bands, int(gridres),
                        float(L), cp, None if ii is None else ii.ctypes.data_as(_dp), inten.ctypes.data_as(_dp),
                        tau.ctypes.data_as(_dp))
    return inten, tau


def _kernel(q):
    q = np.asarray(q, dtype=np.float64)
    return np.where(q <= 0.5, 1 - 6 * q ** 2 + 6 * q ** 3, np.where(q <= 1.0, 2 * (1 - q) ** 3, 0.0))


def _nearest_image_v(dx, boxsize):
    return np.where(np.abs(dx) > boxsize / 2, -np.copysign(boxsize - np.abs(dx), dx), dx)


class OracleMeshoid:
    """Mirror of the reference ``Meshoid`` (src/meshoid/Meshoid.py:12-750) on the oracle."""

    def __init__(self, pos, m=None, kernel_radius=None, des_ngb=None, boxsize=None,
                 verbose=False, particle_mask=None, n_jobs=-1):
        self.tree = None
        pos = np.asarray(pos, dtype=np.float64)
        if pos.ndim == 1:
            pos = pos[:, None]
        self.verbose = verbose
        self.N, self.dim = pos.shape
        if particle_mask is None:
            self.particle_mask = np.arange(self.N)
        else:
            pm = np.asarray(particle_mask)
            self.particle_mask = np.arange(len(pm))[pm] if pm.dtype == bool else pm
        self.Nmask = len(self.particle_mask)
        if des_ngb is None:
            des_ngb = {1: 4, 2: 20, 3: 32}[self.dim]
        self.des_ngb = des_ngb
        self.n_jobs = n_jobs
        self.volnorm = {1: 2.0, 2: np.pi, 3: 4 * np.pi / 3}[self.dim]
        self.boxsize = boxsize
        self.pos = pos
        if boxsize is None:
            self.center = np.median(self.pos, axis=0)
            self.L = 2 * np.percentile(np.sum((self.pos - self.center) ** 2, axis=1), 90) ** 0.5
        else:
            self.center = np.ones(3) * boxsize / 2
            self.L = boxsize
        if m is None:
            m = np.repeat(1.0, self.N)
        self.m = np.asarray(m)[self.particle_mask]
        self.ngb = None
        self.ngbdist = None
        self.kernel_radius = kernel_radius
        self.dweights = self.d2weights = self.dweights_3rdorder = None
        self.density = None
        self.vol = None
        if self.kernel_radius is None:
            self.TreeUpdate()
        else:
            self.vol = self.volnorm * self.kernel_radius ** self.dim / self.des_ngb
            self.density = self.m / self.vol

    def reset_dweights(self):
        self.dweights = self.d2weights = self.dweights_3rdorder = None

    def BuildTree(self):
        from scipy.spatial import cKDTree
        self.tree = cKDTree(self.pos, boxsize=self.boxsize)

    def TreeUpdate(self):
        if self.tree is None:
            self.BuildTree()
        self.ngbdist, self.ngb = knn(self.pos, self.des_ngb, self.boxsize, self.particle_mask,
                                     workers=self.n_jobs, tree=self.tree)
        self.kernel_radius, _ = hsml_iter(self.ngbdist, dim=self.dim, error_norm=1e-13)
        self.density = self.des_ngb * self.m[self.particle_mask] / (self.volnorm * self.kernel_radius ** self.dim)
        self.vol = self.m[self.particle_mask] / self.density

    def ComputeDWeights(self, order=1, weighted=True):
        w, _ = gradient_weights(self.pos, self.ngb, self.kernel_radius, self.particle_mask,
                                self.boxsize, weighted, order)
        if order == 1:
            self.dweights = w
        else:
            self.d2weights, self.dweights_3rdorder = w[:, self.dim:, :], w[:, :self.dim, :]

    def get_kernel_weights(self):
        if self.ngbdist is None or self.kernel_radius is None:
            self.TreeUpdate()
        K = _kernel(self.ngbdist / self.kernel_radius[:, None])
        return K / np.sum(K, axis=1)[:, None]

    def KDE(self, grid, bandwidth=None):
        """Meshoid.py:722-750: 1-D kernel density estimate on the grid points;
        each particle adds Kernel(|g - x| / bw) / bw * 4/3 to the grid points
        within bw of it (the ball query of the reference)."""
        if self.dim != 1:
            raise Exception("KDE only implemented in 1D")
        if bandwidth is None:
            bandwidth = self.SmoothingLength()
        grid = np.asarray(grid, dtype=np.float64)
        bw = np.broadcast_to(np.asarray(bandwidth, dtype=np.float64), (len(self.pos),))
        order = np.argsort(grid, kind="stable")
        gs = grid[order]
        f = np.zeros_like(grid)
        x = np.asarray(self.pos, dtype=np.float64).reshape(len(self.pos), -1)[:, 0]
        for d, b in zip(x, bw):
            a, e = np.searchsorted(gs, d - b, "left"), np.searchsorted(gs, d + b, "right")
            idx = order[a:e]
            dist = np.abs(grid[idx] - d)
            keep = dist <= b
            f[idx[keep]] += _kernel(dist[keep] / b) / b * 4.0 / 3
        return f

    def SmoothingLength(self):
        if self.kernel_radius is None:
            self.TreeUpdate()
        return self.kernel_radius

    def Density(self):
        if self.density is None:
            self.TreeUpdate()
        return self.density

    def Volume(self):
        return self.vol

    def NearestNeighbors(self):
        if self.ngb is None:
            self.TreeUpdate()
        return self.ngb

    def NeighborDistance(self):
        if self.ngbdist is None:
            self.TreeUpdate()
        return self.ngbdist

    def D(self, f, order=1, weighted=True):
        if self.ngb is None:
            self.TreeUpdate()
        if order == 1:
            if self.dweights is None:
                self.ComputeDWeights(1, weighted)
            return apply_weights(self.dweights, self.ngb, self.particle_mask, f)
        if self.dweights_3rdorder is None:
            self.ComputeDWeights(2, weighted)
        return apply_weights(self.dweights_3rdorder, self.ngb, self.particle_mask, f)

    def D2(self, f, weighted=True):
        if self.ngb is None:
            self.TreeUpdate()
        if self.d2weights is None:
            self.ComputeDWeights(2, weighted)
        return apply_weights(self.d2weights, self.ngb, self.particle_mask, f)

    def Curl(self, v):
        dv = self.D(v[self.particle_mask])
        return np.c_[dv[:, 1, 2] - dv[:, 2, 1], dv[:, 0, 2] - dv[:, 2, 0], dv[:, 0, 1] - dv[:, 1, 0]]

    def Div(self, v):
        dv = self.D(v[self.particle_mask])
        return dv[:, 0, 0] + dv[:, 1, 1] + dv[:, 2, 2]

    def KernelAverage(self, f):
        if self.ngb is None:
            self.TreeUpdate()
        return kernel_average(self.ngbdist, self.ngb, self.kernel_radius, np.asarray(f, dtype=np.float64))

    def KernelVariance(self, f):
        if self.ngb is None:
            self.TreeUpdate()
        return np.std(np.asarray(f)[self.ngb], axis=1)

    def Integrate(self, f):
        if self.kernel_radius is None:
            self.TreeUpdate()
        elif self.vol is None:
            self.vol = self.volnorm * self.kernel_radius ** self.dim
        return np.einsum("i,i...->...", self.vol, np.asarray(f)[self.particle_mask])

    def SurfaceDensity(self, f=None, size=None, center=None, res=128, smooth_fac=1.0, conservative=False):
        if f is None:
            f = self.m
        if center is None:
            center = self.center
        if size is None:
            size = self.L
        h = np.clip(smooth_fac * self.kernel_radius, 2 * size / res, 1e100)
        return surface_density(f, self.pos, h, center, size, res, conservative)

    def Reconstruct(self, f, target_points, order=1):
        if self.tree is None:
            self.BuildTree()
        target_points = np.asarray(target_points, dtype=np.float64)
        target_neighbors = self.tree.query(target_points, workers=self.n_jobs)[1]
        unique_neighbors, neighbor_idx = np.unique(target_neighbors, return_inverse=True)
        f_target = np.take(f, target_neighbors, axis=0).astype(np.float64)
        if order == 0:
            return f_target
        dx = target_points - self.pos.take(target_neighbors, axis=0)
        if self.boxsize is not None:
            dx = _nearest_image_v(dx, self.boxsize)
        if not np.array_equal(self.particle_mask, unique_neighbors):
            self.particle_mask = unique_neighbors
            self.TreeUpdate()
            self.reset_dweights()
        gradf = self.D(f, order=order).take(neighbor_idx, axis=0)
        f_target += np.einsum("ij,i...j->i...", dx, gradf)
        if order == 1:
            return f_target
        d2f = self.D2(f).take(neighbor_idx, axis=0)
        f_target += 0.5 * np.einsum("ij,ij...->i...", dx * dx, d2f[..., :3])
        for d in range(self.dim):
            f_target += np.einsum("i,i...->i...", dx[:, d] * dx[:, (d + 1) % self.dim], d2f[..., self.dim + d])
        return f_target

    def InterpToGrid(self, f, size=None, center=None, res=128, order=1, return_grid=False):
        """Meshoid.py:504-555: Reconstruct at the cell centres of a res^3 grid;
        return_grid adds the centre offsets X, Y, Z (relative to center)."""
        if center is None:
            center = self.center
        if size is None:
            size = self.L
        x = np.linspace(-size / 2, size / 2, res + 1)
        x = (x[1:] + x[:-1]) / 2
        X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
        pts = np.c_[X.flatten(), Y.flatten(), Z.flatten()] + center
        out = self.Reconstruct(f, pts, order).reshape((res, res, res) + np.shape(f)[1:])
        if return_grid:
            return X, Y, Z, out
        return out

    def ProjectedAverage(self, f, size=None, center=None, res=128, smooth_fac=1.0):
        """Meshoid.py:645-680 -> GridAverage (grid_deposition.py:395-436): the
        column deposit of f over the column deposit of 1 (same pixel nodes and
        footprints as SurfaceDensity; kernel2d is zero beyond q = 1)."""
        if center is None:
            center = self.center
        if size is None:
            size = self.L
        h = np.clip(smooth_fac * self.kernel_radius, 2 * size / res, 1e100)
        num = surface_density(np.asarray(f, dtype=np.float64), self.pos, h, center, size, res, False)
        den = surface_density(np.ones(len(self.pos)), self.pos, h, center, size, res, False)
        with np.errstate(invalid="ignore", divide="ignore"):
            return num / den

    def DepositToGrid(self, f, weights=None, size=None, center=None, res=128):
        """Meshoid.py:557-593: GridDensity of f with h clipped below at one
        grid spacing (weights is accepted and unused, as in the reference)."""
        if center is None:
            center = self.center
        if size is None:
            size = self.L
        h = np.clip(self.kernel_radius, size / (res - 1), 1e100)
        return grid_density(f, self.pos, h, center, size, res, -1.0 if self.boxsize is None else self.boxsize)

    def Projection(self, f, size=None, center=None, res=128, smooth_fac=1.0):
        """Meshoid.py:682-720: GridAverage of f * vol."""
        return self.ProjectedAverage(np.asarray(f) * self.vol, size, center, res, smooth_fac)

    def Slice(self, f, size=None, plane="z", center=None, res=128, order=1, return_grid=False):
        if center is None:
            center = self.center
        if size is None:
            size = self.L
        if self.tree is None:
            self.TreeUpdate()
        x, y = np.linspace(-size / 2, size / 2, res), np.linspace(-size / 2, size / 2, res)
        x, y = np.meshgrid(x, y, indexing="ij")
        grid = np.c_[x.flatten(), y.flatten(), np.zeros(res * res)] + center
        if plane == "x":
            grid = np.c_[np.zeros(res * res), x.flatten(), y.flatten()] + center
        elif plane == "y":
            grid = np.c_[x.flatten(), np.zeros(res * res), y.flatten()] + center
        fg = self.Reconstruct(f, grid, order)
        shape = (res, res) + tuple(np.shape(f)[1:])
        if return_grid:
            return x, y, fg.reshape(shape)
        return fg.reshape(shape)
