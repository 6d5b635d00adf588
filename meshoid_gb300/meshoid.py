"""GB300 drop-in for the reference ``meshoid.Meshoid`` class (src/meshoid/Meshoid.py:12-750).

Same constructor and method names, argument meanings and output shapes; the
arrays live on the GPU as torch tensors.  Every numerical step runs in the
sm_103a kernels of ``libmeshoid_gb300.so`` through its C ABI; the host code
only allocates, orders and reshapes.  There is no CPU fallback: without a CUDA
device or the built library, construction raises.

Internal layout: particles are held in "slot" order (Morton order of their
cells).  Queries (the particle mask) are processed in slot order for locality
and every per-query result is written straight to its mask position.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _native as N
from ._native import check, ptr
from .profiling import stage

__all__ = ["Meshoid", "set_order2_refinement", "set_order2_method"]

_NORM = {1: 8.0 / 3.0, 2: 40.0 / 7.0, 3: 32.0 / 3.0}
_VOLNORM = {1: 2.0, 2: math.pi, 3: 4.0 * math.pi / 3.0}


def _stream():
    return ctypes_stream(torch.cuda.current_stream())


def ctypes_stream(s):
    import ctypes
    return ctypes.c_void_p(s.cuda_stream)


def set_order2_refinement(enabled):
    """Switch the order-2 refinement step of the derivative sweep on or off
    for the whole process (mg_grad_set_refine; off by default; not in the
    reference; it acts on the "fp32" order-2 method of set_order2_method).
    On, a row whose FP32 second derivatives may miss the
    tolerance is refined once in FP32 with a float-float residual
    (MG_Q_REFINED) instead of being re-solved in FP64; singular rows and rows
    above the condition threshold are still re-solved.  Returns the previous
    setting."""
    return bool(N.load().mg_grad_set_refine(1 if enabled else 0))


_ORDER2_METHODS = ("float-float", "fp32")
_order2_method = ["float-float"]


def set_order2_method(method):
    """Select how D(f, order=2) and D2(f) are computed, process-wide; returns
    the previous method (not in the reference).

    "float-float" (default): separations, kernel weights, basis, moment
    matrices and right-hand sides in float-float, solved with a float-float
    Cholesky factor cached per neighbour set, at a float-float smoothing
    length (mg_grad2_moments, mg_grad2_solve); rows that are singular or
    above the condition threshold are re-solved in FP64 from the FP64
    positions and fields.  Meets 1e-5 of the reference's FP64 answer
    wherever that answer is reproducible.
    "fp32": the FP32 sweep of mg_grad_sweep with its FP64 re-solve of flagged
    rows (and the optional refinement step of set_order2_refinement); faster
    on smooth fields, ~1e-7 cond accurate."""
    if method not in _ORDER2_METHODS:
        raise ValueError(f"order-2 method must be one of {_ORDER2_METHODS}")
    prev = _order2_method[0]
    _order2_method[0] = method
    return prev


def _dev_tensor(x, dtype, device):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=device).contiguous()


def _np_median(x: torch.Tensor) -> torch.Tensor:
    """np.median(x, axis=0) semantics (mean of the two middle values for even N)."""
    s, _ = torch.sort(x, dim=0)
    n = x.shape[0]
    if n % 2:
        return s[n // 2]
    return 0.5 * (s[n // 2 - 1] + s[n // 2])


def _np_percentile(v: torch.Tensor, q: float) -> torch.Tensor:
    """np.percentile(v, q) with linear interpolation."""
    s, _ = torch.sort(v)
    pos = (v.shape[0] - 1) * q / 100.0
    lo = int(math.floor(pos))
    hi = min(lo + 1, v.shape[0] - 1)
    frac = pos - lo
    return s[lo] + (s[hi] - s[lo]) * frac


_plain_rf_cache = {}


def _plain_radius_factor(k):
    """Radius factor of the plain seed: calibrated next to the packaged seed
    network (same quantile of r_k / h_seed), else 1.4."""
    if k not in _plain_rf_cache:
        rf = 1.4
        try:
            import os
            from .seed_model import default_model_path
            path = default_model_path(k)
            if os.path.exists(path):
                with np.load(path) as z:
                    if "meta_plain_radius_factor" in z.files:
                        rf = float(z["meta_plain_radius_factor"])
        except Exception:
            pass
        _plain_rf_cache[k] = rf
    return _plain_rf_cache[k]


class Meshoid:
    """Particle-neighbourhood operations on one GPU.

    Parameters mirror the reference constructor (src/meshoid/Meshoid.py:15-25).
    Extra keyword arguments:

    seed : "plain" | "learned" | SeedModel | tensor
        How the first search radius of each query is guessed: from the
        particle count of its adaptive cell ("plain"), by the trained seed
        network ("learned" uses the packaged default model), or given as an
        (Nmask,) tensor of first guesses of h in row order (radius_factor
        then defaults to 1).  The converged neighbour sets and smoothing
        lengths do not depend on the seed.
    radius_factor : float
        First search radius = radius_factor * seed h.
    device : torch device (default: current CUDA device).
    """

    def __init__(self, pos, m=None, kernel_radius=None, des_ngb=None, boxsize=None, verbose=False,
                 particle_mask=None, n_jobs=-1, seed="plain", radius_factor=None, device=None,
                 max_passes=16, grid_level=None, level_bias=1, cond_threshold=(30.0, 1e6),
                 brick_threshold=64):
        if not torch.cuda.is_available():
            raise RuntimeError("meshoid_gb300 needs a CUDA device (GB300); no CPU path exists")
        self._lib = N.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.tree = None
        pos = _dev_tensor(pos, torch.float64, self.device)
        if pos.ndim == 1:
            pos = pos[:, None]
        self.verbose = verbose
        self.N, self.dim = pos.shape
        if not bool(torch.isfinite(pos).all()):
            raise ValueError("positions contain NaN or infinity")
        if self.dim < 1 or self.dim > 3:
            raise ValueError("positions must be 1-, 2- or 3-dimensional")
        if self.N < 1:
            raise ValueError("empty particle set")
        self._full_mask = particle_mask is None
        if particle_mask is None:
            self.particle_mask = torch.arange(self.N, device=self.device)
        else:
            pm = torch.as_tensor(np.asarray(particle_mask) if not isinstance(particle_mask, torch.Tensor)
                                 else particle_mask, device=self.device)
            self.particle_mask = torch.nonzero(pm).flatten() if pm.dtype == torch.bool else pm.long()
        self.Nmask = int(self.particle_mask.numel())
        if des_ngb is None:
            des_ngb = {1: 4, 2: 20, 3: 32}[self.dim]
        self.des_ngb = int(des_ngb)
        if self.des_ngb < 2 or self.des_ngb > N.MG_MAX_K:
            raise ValueError(f"des_ngb must be in [2, {N.MG_MAX_K}]")
        if self.des_ngb > self.N:
            raise ValueError("des_ngb exceeds the number of particles")
        self.n_jobs = n_jobs
        self.volnorm = _VOLNORM[self.dim]
        self.boxsize = boxsize
        self.pos = pos
        self._center = None
        self._L = None
        if boxsize is not None:
            if boxsize <= 0:
                raise ValueError("boxsize must be positive")
            if bool(((pos < 0) | (pos >= boxsize)).any()):
                raise ValueError("coordinates must lie in [0, boxsize) for a periodic box")
            self._center = torch.ones(3, dtype=torch.float64, device=self.device) * boxsize / 2
            self._L = boxsize
        if m is None:
            m = torch.ones(self.N, dtype=torch.float64, device=self.device)
        self._m_full = _dev_tensor(m, torch.float64, self.device)
        self.m = self._m_full if self._full_mask else self._m_full[self.particle_mask].contiguous()
        self.seed = seed
        self.radius_factor = radius_factor
        self.max_passes = int(max_passes)
        self.level_bias = int(level_bias)
        # cells with more particles than this get refinement tables (0: binary search only)
        self.brick_threshold = int(brick_threshold)
        # rows whose moment-matrix condition estimate exceeds this (order 1, order 2)
        # are re-solved in FP64; 0 disables the re-solve
        self.cond_threshold = tuple(float(t) for t in cond_threshold)
        self._grid_level = grid_level
        self.stats = None
        self._ngb_slots = None
        self._hsml_q = None
        self._hsml_lo_q = None
        self._hsml_pair = None  # float-float h of the queries (hi, lo)
        self._g2 = None         # (weighted, moments buffer, bytes): cached order-2 moment matrices
        self._ngb_user = None
        self._ngbdist_user = None
        self.dweights = self.d2weights = self.dweights_3rdorder = None
        self.sliceweights = None
        self.kernel_radius = None
        self.density = None
        self.vol = None
        self._build_cells()
        self._set_queries()
        if kernel_radius is None:
            self.TreeUpdate()
        else:
            self.kernel_radius = _dev_tensor(kernel_radius, torch.float64, self.device)
            self.vol = self.volnorm * self.kernel_radius ** self.dim / self.des_ngb
            self.density = self.m / self.vol

    # ------------------------------------------------------------------ defaults for maps
    # src/meshoid/Meshoid.py:81-87: median position and twice the 90th-percentile
    # radius about it (box centre / box size when periodic).  Computed on first
    # use; they only serve as map defaults.
    @property
    def center(self):
        if self._center is None:
            self._center = _np_median(self.pos)
        return self._center

    @center.setter
    def center(self, value):
        self._center = _dev_tensor(value, torch.float64, self.device)

    @property
    def L(self):
        if self._L is None:
            r2 = torch.sum((self.pos - self.center) ** 2, dim=1)
            self._L = float(2.0 * float(_np_percentile(r2, 90.0)) ** 0.5)
        return self._L

    @L.setter
    def L(self, value):
        self._L = float(value)

    # ------------------------------------------------------------------ index
    def _build_cells(self):
        lib = self._lib
        n = self.N
        L = self._grid_level or lib.mg_default_grid_level(n)
        dev = self.device
        self._frame = torch.empty(8, dtype=torch.float64, device=dev)
        self._keys = torch.empty(n, dtype=torch.int64, device=dev)
        self._order = torch.empty(n, dtype=torch.int32, device=dev)
        self._rank = torch.empty(n, dtype=torch.int32, device=dev)
        self._pos_hi = torch.empty((n, 4), dtype=torch.float32, device=dev)
        self._pos_lo = torch.empty((n, 4), dtype=torch.float32, device=dev)
        self._pos64 = torch.empty((n, 3), dtype=torch.float64, device=dev)
        self._cell_start = torch.empty((1 << (3 * L)) + 1, dtype=torch.int32, device=dev)
        if self.brick_threshold > 0:
            cap = min(lib.mg_brick_capacity(n, L, self.brick_threshold), lib.mg_brick_capacity(n, L, 64))
            self._brick_of = torch.empty(1 << (3 * L), dtype=torch.int32, device=dev)
            self._bricks = torch.empty((cap, N.MG_BRICK_WORDS), dtype=torch.int32, device=dev)
        else:
            cap = 0
            self._brick_of = self._bricks = None
        c = N.MgCells()
        c.n = n
        c.dim = self.dim
        c.grid_level = L
        c.boxsize = float(self.boxsize) if self.boxsize is not None else -1.0
        c.frame = self._frame.data_ptr()
        c.keys = self._keys.data_ptr()
        c.order = self._order.data_ptr()
        c.rank = self._rank.data_ptr()
        c.pos_hi = self._pos_hi.data_ptr()
        c.pos_lo = self._pos_lo.data_ptr()
        c.pos64 = self._pos64.data_ptr()
        c.cell_start = self._cell_start.data_ptr()
        c.brick_of = self._brick_of.data_ptr() if cap else None
        c.bricks = self._bricks.data_ptr() if cap else None
        c.brick_capacity = cap
        c.brick_threshold = self.brick_threshold
        self._cells = c
        wsb = lib.mg_build_cells_workspace_bytes(n, L)
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        with stage("build_cells"):
            check(lib.mg_build_cells(ptr(self.pos), self._cells, ptr(ws), wsb, _stream()), "mg_build_cells")
        self.tree = True  # the spatial index stands in for the reference's cKDTree

    def BuildTree(self):
        self._build_cells()

    def _set_queries(self):
        """Slot-ordered query list for the current particle mask, and the output row of each."""
        mask = self.particle_mask
        if self._full_mask or (self.Nmask == self.N and
                               bool(torch.equal(mask, torch.arange(self.N, device=self.device)))):
            self._queries = None
            self._out_rows = self._order  # slot s -> particle order[s] == mask position
        else:
            slots = self._rank[mask].long()
            sorted_slots, perm = torch.sort(slots)
            self._queries = sorted_slots.to(torch.int32).contiguous()
            self._out_rows = perm.to(torch.int32).contiguous()
        self.Nmask = int(mask.numel())

    # ------------------------------------------------------------------ seeds
    def _seed_h(self):
        lib = self._lib
        nq = self.Nmask
        seed = torch.empty(nq, dtype=torch.float32, device=self.device)
        if isinstance(self.seed, torch.Tensor):
            g = self.seed.to(device=self.device, dtype=torch.float32).reshape(-1)
            if g.numel() != nq:
                raise ValueError(f"seed tensor has {g.numel()} entries, expected {nq}")
            return g[self._out_rows.long()].contiguous(), self.radius_factor or 1.0  # row order -> query order
        if isinstance(self.seed, str) and self.seed == "plain":
            with stage("seed"):
                check(lib.mg_seed_plain(self._cells, ptr(self._queries), nq, self.des_ngb, ptr(seed), _stream()),
                      "mg_seed_plain")
            factor = self.radius_factor or _plain_radius_factor(self.des_ngb)
        else:
            from .seed_model import resolve_model
            model = resolve_model(self.seed, self.device, self.des_ngb)
            with stage("seed"):
                seed = model.predict(self._cells, self._queries, nq, self.des_ngb)
            factor = self.radius_factor or model.radius_factor
        return seed, factor

    # ------------------------------------------------------------------ tree update
    def TreeUpdate(self):
        """Neighbours and smoothing lengths of the masked particles
        (src/meshoid/Meshoid.py:147-170)."""
        lib = self._lib
        nq = self.Nmask
        k = self.des_ngb
        seed, factor = self._seed_h()
        ngb = torch.empty((nq, k), dtype=torch.int32, device=self.device)
        hsml = torch.empty(nq, dtype=torch.float32, device=self.device)
        hsml_lo = torch.empty(nq, dtype=torch.float32, device=self.device)
        qstatus = torch.empty(nq, dtype=torch.int32, device=self.device)
        stats = torch.zeros(16, dtype=torch.int64, device=self.device)
        wsb = lib.mg_knn_hsml_workspace_bytes(nq, k)
        ws = torch.empty(wsb, dtype=torch.uint8, device=self.device)
        with stage("knn_hsml"):
            st = lib.mg_knn_hsml(self._cells, ptr(self._queries), nq, k, ptr(seed), float(factor),
                                 self.level_bias, self.max_passes, ptr(ngb), ptr(hsml), ptr(hsml_lo), ptr(qstatus),
                                 ptr(stats),
                                 ptr(ws), wsb, _stream())
        check(st, "mg_knn_hsml")
        self.stats = stats
        self._qstatus = qstatus
        unresolved = int(stats[4])  # the search counts the queries it left unresolved
        if unresolved:
            bad = (qstatus & N.MG_Q_UNRESOLVED).ne(0)
            idx = torch.nonzero(bad).flatten()[:4]
            code = (-hsml[idx]).long().tolist()
            radius = ws[:4 * nq].view(torch.float32)[idx].tolist()
            raise N.MeshoidError(f"neighbour search did not resolve {unresolved} queries within "
                                 f"{self.max_passes} passes (reason*1e6+count {code}, last radius {radius})")
        self._ngb_slots = ngb
        self._hsml_q = hsml
        self._hsml_lo_q = hsml_lo
        # the order-2 sweep's float-float h: the search's own for k <= 32 (its
        # row solve works in float-float); for k > 32 polished on first use
        self._hsml_pair = (hsml, hsml_lo) if k <= 32 else None
        self._g2 = None
        self._ngb_user = None
        self._ngbdist_user = None
        h = torch.empty(nq, dtype=torch.float64, device=self.device)
        self.density = torch.empty(nq, dtype=torch.float64, device=self.device)
        self.vol = torch.empty(nq, dtype=torch.float64, device=self.device)
        mq = self._m_full if self._full_mask else self._m_full[self.particle_mask].contiguous()
        check(lib.mg_density(ptr(self._out_rows), ptr(hsml), ptr(hsml_lo), nq, ptr(mq), k, self.dim, ptr(h),
                             ptr(self.density),
                             ptr(self.vol), _stream()), "mg_density")
        self.kernel_radius = h

    def reset_dweights(self):
        self.dweights = self.d2weights = self.dweights_3rdorder = None
        self._g2 = None

    # ------------------------------------------------------------------ accessors
    @property
    def ngb(self):
        if self._ngb_slots is None:
            return None
        if self._ngb_user is None:
            self._neighbor_lists()
        return self._ngb_user

    @property
    def ngbdist(self):
        if self._ngb_slots is None:
            return None
        if self._ngbdist_user is None:
            self._neighbor_lists()
        return self._ngbdist_user

    def _neighbor_lists(self):
        nq, k = self._ngb_slots.shape
        idx = torch.empty((nq, k), dtype=torch.int64, device=self.device)
        dist = torch.empty((nq, k), dtype=torch.float64, device=self.device)
        check(self._lib.mg_neighbor_dist(self._cells, ptr(self._queries), nq, ptr(self._ngb_slots), k,
                                         ptr(idx), ptr(dist), _stream()), "mg_neighbor_dist")
        rows = self._out_rows.long()
        ui = torch.empty_like(idx)
        ud = torch.empty_like(dist)
        ui[rows] = idx
        ud[rows] = dist
        self._ngb_user, self._ngbdist_user = ui, ud

    def _kth_distance(self):
        """Distance to the k-th (farthest) neighbour of each query, internal query order (FP64)."""
        nq, k = self._ngb_slots.shape
        idx = torch.empty((nq, k), dtype=torch.int64, device=self.device)
        dist = torch.empty((nq, k), dtype=torch.float64, device=self.device)
        check(self._lib.mg_neighbor_dist(self._cells, ptr(self._queries), nq, ptr(self._ngb_slots), k,
                                         ptr(idx), ptr(dist), _stream()), "mg_neighbor_dist")
        return dist[:, -1]

    def Volume(self):
        return self.vol

    def NearestNeighbors(self):
        if self._ngb_slots is None:
            self.TreeUpdate()
        return self.ngb

    def NeighborDistance(self):
        if self._ngb_slots is None:
            self.TreeUpdate()
        return self.ngbdist

    def ComputeDWeights(self, order=1, weighted=True):
        """Materialise the least-squares derivative weights (src/meshoid/
        Meshoid.py:110-140 -> derivatives.py:118-138) in FP64: order 1 sets
        dweights (Nmask, dim, k); order 2 sets d2weights (second-derivative
        rows) and dweights_3rdorder (first-derivative rows).  Neighbours in the
        order of self.ngb.  D and D2 do not need them (they contract on the
        fly).  An exactly singular moment matrix raises LinAlgError, as the
        reference's np.linalg.inv does."""
        ngb = self.ngb
        if ngb is None:
            self.TreeUpdate()
            ngb = self.ngb
        nq, k = ngb.shape
        nd = self.dim if order == 1 else {1: 2, 2: 5, 3: 9}[self.dim]
        out = torch.empty((nq, nd, k), dtype=torch.float64, device=self.device)
        nsing = torch.zeros(1, dtype=torch.int64, device=self.device)
        idx = self.particle_mask.long().contiguous()
        pos = self.pos.reshape(self.N, self.dim).contiguous()
        box = float(self.boxsize) if self.boxsize is not None else -1.0
        check(self._lib.mg_gradient_weights(ptr(pos), self.dim, ptr(ngb.contiguous()), k,
                                            ptr(self.kernel_radius.contiguous()), ptr(idx), nq, box,
                                            1 if weighted else 0, int(order), ptr(out), ptr(nsing), _stream()),
              "mg_gradient_weights")
        if int(nsing.item()) > 0:
            raise np.linalg.LinAlgError("Singular matrix")
        if order == 1:
            self.dweights = out
        else:
            self.d2weights, self.dweights_3rdorder = out[:, self.dim:, :], out[:, :self.dim, :]

    def get_kernel_weights(self):
        """K(d / h) / sum K over each row of ngbdist (src/meshoid/Meshoid.py:172-177)."""
        if self.ngbdist is None or self.kernel_radius is None:
            self.TreeUpdate()
        d = self.ngbdist.contiguous()
        nq, k = d.shape
        w = torch.empty_like(d)
        check(self._lib.mg_kernel_weights(ptr(d), ptr(self.kernel_radius.contiguous()), nq, k, ptr(w), _stream()),
              "mg_kernel_weights")
        return w

    def KDE(self, grid, bandwidth=None):
        """Kernel density estimate of the points on a 1-D grid (src/meshoid/
        Meshoid.py:722-750): each particle adds Kernel(|g - x| / bw) / bw * 4/3
        to the grid points within bw; bandwidth defaults to the smoothing
        lengths (an array, or here also a scalar)."""
        if self.dim != 1:
            raise Exception("KDE only implemented in 1D")
        if bandwidth is None:
            bandwidth = self.SmoothingLength()
        g = _dev_tensor(grid, torch.float64, self.device).reshape(-1).contiguous()
        bw = _dev_tensor(bandwidth, torch.float64, self.device).reshape(-1)
        x = self.pos.reshape(-1)
        if bw.numel() == 1:
            bw = bw.expand(x.numel())
        n = min(x.numel(), bw.numel())  # zip(self.pos, bandwidth)
        x, bw = x[:n].contiguous(), bw[:n].contiguous()
        f = torch.zeros_like(g)
        wsb = self._lib.mg_kde_1d_workspace_bytes(g.numel())
        ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=self.device)
        check(self._lib.mg_kde_1d(ptr(x), ptr(bw), n, ptr(g), g.numel(), ptr(f), ptr(ws), wsb, _stream()),
              "mg_kde_1d")
        return f

    def SmoothingLength(self):
        if self.kernel_radius is None:
            self.TreeUpdate()
        return self.kernel_radius

    def Density(self):
        if self.density is None:
            self.TreeUpdate()
        return self.density

    # ------------------------------------------------------------------ fields
    def _fields(self, f):
        """(N, ...) field -> slot-order FP32 hi/lo planes (N, nfp) and the trailing shape."""
        f = _dev_tensor(f, torch.float64, self.device)
        if f.shape[0] != self.N:
            raise ValueError(f"field has {f.shape[0]} rows, expected N = {self.N}")
        shape = tuple(f.shape[1:])
        f2 = f.reshape(self.N, -1).contiguous()
        nf = f2.shape[1]
        nfp = (nf + 3) & ~3
        hi = torch.empty((self.N, nfp), dtype=torch.float32, device=self.device)
        lo = torch.empty((self.N, nfp), dtype=torch.float32, device=self.device)
        with stage("load_fields"):
            check(self._lib.mg_load_fields(self._cells, ptr(f2), nf, ptr(hi), ptr(lo), _stream()), "mg_load_fields")
        return hi, lo, nf, shape

    def _fields3(self, f):
        """(N, ...) field -> slot-order three-plane split hi + mid + lo (N, nfp)."""
        f = _dev_tensor(f, torch.float64, self.device)
        if f.shape[0] != self.N:
            raise ValueError(f"field has {f.shape[0]} rows, expected N = {self.N}")
        shape = tuple(f.shape[1:])
        f2 = f.reshape(self.N, -1).contiguous()
        nf = f2.shape[1]
        nfp = (nf + 3) & ~3
        planes = torch.empty((3, self.N, nfp), dtype=torch.float32, device=self.device)
        with stage("load_fields"):
            check(self._lib.mg_load_fields3(self._cells, ptr(f2), nf, ptr(planes[0]), ptr(planes[1]), ptr(planes[2]),
                                            _stream()), "mg_load_fields3")
        return planes, nf, shape

    def _hsml_ff(self):
        """Float-float smoothing lengths (hi, lo) of the queries: the root of
        HsmlIter's equation polished from the FP32 solve (computed once per
        neighbour set)."""
        if self._hsml_pair is None:
            nq = self.Nmask
            hi = torch.empty(nq, dtype=torch.float32, device=self.device)
            lo = torch.empty(nq, dtype=torch.float32, device=self.device)
            with stage("hsml_polish"):
                check(self._lib.mg_hsml_polish(self._cells, ptr(self._queries), nq, ptr(self._ngb_slots),
                                               self.des_ngb, ptr(self._hsml_q), ptr(hi), ptr(lo), _stream()),
                      "mg_hsml_polish")
            self._hsml_pair = (hi, lo)
        return self._hsml_pair

    def _order2_moments(self, weighted):
        """Cached float-float moment matrices of the order-2 fit (the analogue
        of the reference's dweights_3rdorder / d2weights cache, Meshoid.py:
        110-140; dropped by TreeUpdate and reset_dweights)."""
        key = bool(weighted)
        if self._g2 is None or self._g2[0] != key:
            hi, lo = self._hsml_ff()
            nq = self.Nmask
            mb = self._lib.mg_grad2_moments_bytes(nq, self.dim)
            mom = torch.empty(mb, dtype=torch.uint8, device=self.device)
            with stage("grad2_moments"):
                check(self._lib.mg_grad2_moments(self._cells, ptr(self._queries), nq, ptr(self._ngb_slots),
                                                 self.des_ngb, ptr(hi), ptr(lo), 1 if weighted else 0,
                                                 float(self.cond_threshold[1]), ptr(mom), mb, _stream()),
                      "mg_grad2_moments")
            self._g2 = (key, mom, mb)
        return self._g2

    def _sweep2(self, f, weighted, want2):
        """Order-2 derivatives by the float-float path (mg_grad2_solve)."""
        _, mom, mb = self._order2_moments(weighted)
        hi, lo = self._hsml_ff()
        planes, nf, shape = self._fields3(f)
        nq = self.Nmask
        nd2 = {1: 1, 2: 3, 3: 6}[self.dim]
        d1 = torch.empty((nq, nf, self.dim), dtype=torch.float32, device=self.device)
        d2 = torch.empty((nq, nf, nd2), dtype=torch.float32, device=self.device)
        self._gstatus = torch.zeros(nq, dtype=torch.int32, device=self.device)
        wsb = self._lib.mg_grad2_solve_workspace_bytes(nq)
        ws = torch.empty(wsb, dtype=torch.uint8, device=self.device)
        with stage("grad2_solve"):
            check(self._lib.mg_grad2_solve(self._cells, ptr(self._queries), nq, ptr(self._ngb_slots), self.des_ngb,
                                           ptr(hi), ptr(lo), 1 if weighted else 0, ptr(mom), mb, ptr(planes[0]),
                                           ptr(planes[1]), ptr(planes[2]), nf, ptr(self._out_rows), ptr(d1), ptr(d2),
                                           ptr(self._gstatus), ptr(ws), wsb, _stream()), "mg_grad2_solve")
        if want2:
            return d2.reshape((nq,) + shape + (nd2,))
        return d1.reshape((nq,) + shape + (self.dim,))

    def _sweep(self, f, order, weighted, want2):
        if self._ngb_slots is None:
            self.TreeUpdate()
        if order == 2 and _order2_method[0] == "float-float":
            return self._sweep2(f, weighted, want2)
        hi, lo, nf, shape = self._fields(f)
        nq = self.Nmask
        nd2 = {1: 1, 2: 3, 3: 6}[self.dim]
        d1 = torch.empty((nq, nf, self.dim), dtype=torch.float32, device=self.device)
        d2 = torch.empty((nq, nf, nd2), dtype=torch.float32, device=self.device) if order == 2 else None
        self._gstatus = torch.zeros(nq, dtype=torch.int32, device=self.device)
        thr = self.cond_threshold[order - 1]
        wsb = self._lib.mg_grad_sweep_workspace_bytes(nq)
        ws = torch.empty(wsb, dtype=torch.uint8, device=self.device) if thr > 0 else None
        with stage("grad_sweep"):
            st = self._lib.mg_grad_sweep(self._cells, ptr(self._queries), nq, ptr(self._ngb_slots), self.des_ngb,
                                         ptr(self._hsml_q), ptr(self._hsml_lo_q), order, 1 if weighted else 0, ptr(hi), ptr(lo), nf,
                                         ptr(self._out_rows), ptr(d1), ptr(d2), ptr(self._gstatus), float(thr),
                                         ptr(ws), wsb if ws is not None else 0, _stream())
        check(st, "mg_grad_sweep")
        if want2:
            return d2.reshape((nq,) + shape + (nd2,))
        return d1.reshape((nq,) + shape + (self.dim,))

    def D(self, f, order=1, weighted=True):
        """Least-squares gradient (src/meshoid/Meshoid.py:237-268): (Nmask, ..., dim)."""
        if order not in (1, 2):
            raise ValueError("order must be 1 or 2")
        return self._sweep(f, order, weighted, want2=False)

    def D2(self, f, weighted=True):
        """Second derivatives [xx,yy,zz,xy,yz,zx] (src/meshoid/Meshoid.py:270-295)."""
        return self._sweep(f, 2, weighted, want2=True)

    def _masked_field(self, v):
        """v[particle_mask] as Curl and Div take it (src/meshoid/Meshoid.py:310,
        :330), laid out as the N-row field that D indexes.  D then indexes that
        field with global neighbour indices and with the mask itself
        (np.take(f, ngb), f[particle_mask], Meshoid.py:258); for a partial mask
        this works only when every such index is below Nmask, and otherwise
        raises IndexError, as numpy does in the reference."""
        v = _dev_tensor(v, torch.float64, self.device)
        vm = v[self.particle_mask]
        if vm.shape[0] == self.N:
            return vm
        top = max(int(self.particle_mask.max()), int(self.ngb.max()))
        if top >= vm.shape[0]:
            raise IndexError(f"index {top} is out of bounds for axis 0 with size {vm.shape[0]} "
                             "(the field is indexed by particle_mask before D, as in the reference)")
        full = torch.zeros((self.N,) + tuple(vm.shape[1:]), dtype=torch.float64, device=self.device)
        full[:vm.shape[0]] = vm
        return full

    def Curl(self, v):
        """Curl of an (N, 3) vector field (src/meshoid/Meshoid.py:297-315):
        with dv = D(v[particle_mask]), dv[:, c, d] = d v_c / d x_d, the
        reference's combination [dv[:,1,2] - dv[:,2,1], dv[:,0,2] - dv[:,2,0],
        dv[:,0,1] - dv[:,1,0]] (kept as written there, signs included)."""
        dv = self.D(self._masked_field(v))
        return torch.stack([dv[:, 1, 2] - dv[:, 2, 1], dv[:, 0, 2] - dv[:, 2, 0], dv[:, 0, 1] - dv[:, 1, 0]], dim=1)

    def Div(self, v):
        """Divergence of an (N, 3) vector field (src/meshoid/Meshoid.py:317-331),
        from D of v[particle_mask]."""
        dv = self.D(self._masked_field(v))
        return dv[:, 0, 0] + dv[:, 1, 1] + dv[:, 2, 2]

    def KernelAverage(self, f):
        """Kernel-weighted neighbour average (src/meshoid/Meshoid.py:368-381)."""
        if self._ngb_slots is None:
            self.TreeUpdate()
        hi, lo, nf, shape = self._fields(f)
        out = torch.empty((self.Nmask, nf), dtype=torch.float64, device=self.device)
        check(self._lib.mg_kernel_average(self._cells, ptr(self._queries), self.Nmask, ptr(self._ngb_slots),
                                          self.des_ngb, ptr(self._hsml_q), ptr(hi), ptr(lo), nf,
                                          ptr(self._out_rows), ptr(out), _stream()), "mg_kernel_average")
        return out.reshape((self.Nmask,) + shape)

    def KernelVariance(self, f):
        """Standard deviation of f over each particle's neighbours, self included
        (src/meshoid/Meshoid.py:351-366): (Nmask, ...) FP64."""
        if self._ngb_slots is None:
            self.TreeUpdate()
        hi, lo, nf, shape = self._fields(f)
        out = torch.empty((self.Nmask, nf), dtype=torch.float64, device=self.device)
        check(self._lib.mg_kernel_variance(self._cells, ptr(self._queries), self.Nmask, ptr(self._ngb_slots),
                                           self.des_ngb, ptr(hi), ptr(lo), nf, ptr(self._out_rows), ptr(out),
                                           _stream()), "mg_kernel_variance")
        return out.reshape((self.Nmask,) + shape)

    def Integrate(self, f):
        """Volume integral sum_i vol_i f_i over the masked particles
        (src/meshoid/Meshoid.py:333-349)."""
        if self.kernel_radius is None:
            self.TreeUpdate()
        elif self.vol is None:
            self.vol = self.volnorm * self.kernel_radius ** self.dim
        f = _dev_tensor(f, torch.float64, self.device)[self.particle_mask]
        return torch.einsum("i,i...->...", self.vol, f)

    # ------------------------------------------------------------------ maps
    def _sightline_average(self, f, size, center, res, smooth_fac):
        """GridAverage (src/meshoid/grid_deposition.py:395-436): the column
        deposit of f divided by the column deposit of 1, on the pixel nodes and
        footprints of SurfaceDensity (0/0 gives NaN, as in the reference)."""
        ones = torch.ones(self.N, dtype=torch.float64, device=self.device)
        num = self.SurfaceDensity(f, size=size, center=center, res=res, smooth_fac=smooth_fac)
        den = self.SurfaceDensity(ones, size=size, center=center, res=res, smooth_fac=smooth_fac)
        return num / den

    def ProjectedAverage(self, f, size=None, center=None, res=128, smooth_fac=1.0):
        """Kernel-weighted average of f along sightlines (src/meshoid/Meshoid.py:645-680): (res, res)."""
        return self._sightline_average(f, size, center, res, smooth_fac)

    def Projection(self, f, size=None, center=None, res=128, smooth_fac=1.0):
        """The reference's Projection (src/meshoid/Meshoid.py:682-720): the
        sightline average of f * vol, (res, res)."""
        f = _dev_tensor(f, torch.float64, self.device)
        return self._sightline_average(f * self.vol, size, center, res, smooth_fac)

    def SurfaceDensity(self, f=None, size=None, center=None, res=128, smooth_fac=1.0, conservative=False):
        """Column density map (src/meshoid/Meshoid.py:595-643): (res, res) FP64."""
        if f is None:
            f = self.m
        if center is None:
            center = self.center
        if size is None:
            size = self.L
        center = [float(c) for c in (center.tolist() if isinstance(center, torch.Tensor) else center)]
        f = _dev_tensor(f, torch.float64, self.device)
        h = torch.clamp(smooth_fac * self.kernel_radius, min=2 * size / res, max=1e100).contiguous()
        pos3 = self._pos3()
        n = pos3.shape[0]
        if f.shape[0] != n or h.shape[0] != n:
            raise ValueError("SurfaceDensity needs f and the smoothing lengths for all N particles")
        grid = torch.empty((res, res), dtype=torch.float64, device=self.device)
        wsb = self._lib.mg_surface_density_workspace_bytes(n, res)
        ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=self.device)
        check(self._lib.mg_surface_density(ptr(pos3), ptr(h), ptr(f), n, center[0], center[1], float(size), int(res),
                                           1 if conservative else 0, ptr(grid), ptr(ws), wsb, _stream()),
              "mg_surface_density")
        return grid

    def DepositToGrid(self, f, weights=None, size=None, center=None, res=128):
        """Density of a conserved quantity on a (res, res, res) grid
        (src/meshoid/Meshoid.py:557-593 -> GridDensity): smoothing lengths
        clipped below at one grid spacing; with a box the deposit wraps
        periodically.  weights is accepted and unused, as in the reference.
        The reference only runs with a box (GridDensity compares box_size < 0,
        which fails for None); here no box means open boundaries."""
        from . import grid_deposition as gd
        if center is None:
            center = self.center
        if size is None:
            size = self.L
        h = torch.clamp(self.kernel_radius, min=size / (res - 1), max=1e100)
        return gd.GridDensity(f, self._pos3(), h, center, size, res=res,
                              box_size=-1.0 if self.boxsize is None else self.boxsize)

    def _pos3(self):
        if self.dim == 3:
            return self.pos
        p = torch.zeros((self.N, 3), dtype=torch.float64, device=self.device)
        p[:, :self.dim] = self.pos
        return p

    def _nn(self, targets):
        targets = _dev_tensor(targets, torch.float64, self.device)
        nt = targets.shape[0]
        t3 = torch.zeros((nt, 3), dtype=torch.float64, device=self.device)
        t3[:, :targets.shape[1]] = targets[:, :3]
        nn = torch.empty(nt, dtype=torch.int64, device=self.device)
        wsb = self._lib.mg_nn_query_workspace_bytes(nt)
        ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=self.device)
        check(self._lib.mg_nn_query(self._cells, ptr(t3), nt, ptr(nn), ptr(ws), wsb, _stream()), "mg_nn_query")
        return nn

    def Reconstruct(self, f, target_points, order=1):
        """Value of f at arbitrary points from the nearest particle's Taylor
        expansion (src/meshoid/Meshoid.py:383-440).  Like the reference, order
        >= 1 sets particle_mask to the unique nearest particles and recomputes
        their neighbours and smoothing lengths."""
        target_points = _dev_tensor(target_points, torch.float64, self.device)
        nn = self._nn(target_points)
        unique, inv = torch.unique(nn, sorted=True, return_inverse=True)
        f = _dev_tensor(f, torch.float64, self.device)
        f_t = f[nn].clone()
        if order == 0:
            return f_t
        dx = target_points - self.pos[nn]
        if self.boxsize is not None:
            b = float(self.boxsize)
            dx = torch.where(dx.abs() > b / 2, -torch.copysign(b - dx.abs(), dx), dx)
        if not (unique.numel() == self.particle_mask.numel() and bool(torch.equal(unique, self.particle_mask))):
            self.particle_mask = unique
            self._full_mask = False
            self._set_queries()
            self.TreeUpdate()
            self.reset_dweights()
        grad = self.D(f, order=order)[inv].double()
        f_t += torch.einsum("ij,i...j->i...", dx, grad)
        if order == 1:
            return f_t
        d2f = self.D2(f)[inv].double()
        f_t += 0.5 * torch.einsum("ij,ij...->i...", dx * dx, d2f[..., :3])
        for d in range(self.dim):
            f_t += torch.einsum("i,i...->i...", dx[:, d] * dx[:, (d + 1) % self.dim], d2f[..., self.dim + d])
        return f_t

    def InterpToGrid(self, f, size=None, center=None, res=128, order=1, return_grid=False):
        """Reconstruction of f at the cell centres of a res^3 grid
        (src/meshoid/Meshoid.py:504-555)."""
        if center is None:
            center = self.center
        if size is None:
            size = self.L
        center = _dev_tensor(center, torch.float64, self.device)
        edges = torch.linspace(-size / 2, size / 2, res + 1, dtype=torch.float64, device=self.device)
        x = 0.5 * (edges[1:] + edges[:-1])
        X, Y, Z = torch.meshgrid(x, x, x, indexing="ij")
        pts = torch.stack([X.flatten(), Y.flatten(), Z.flatten()], 1) + center
        f_grid = self.Reconstruct(f, pts, order)
        shape = (res, res, res) + tuple(f_grid.shape[1:])
        if return_grid:
            return X, Y, Z, f_grid.reshape(shape)
        return f_grid.reshape(shape)

    def Slice(self, f, size=None, plane="z", center=None, res=128, order=1, return_grid=False):
        """Values of f on a res x res plane (src/meshoid/Meshoid.py:442-502)."""
        if center is None:
            center = self.center
        if size is None:
            size = self.L
        center = _dev_tensor(center, torch.float64, self.device)
        lin = torch.linspace(-size / 2, size / 2, res, dtype=torch.float64, device=self.device)
        x, y = torch.meshgrid(lin, lin, indexing="ij")
        z = torch.zeros(res * res, dtype=torch.float64, device=self.device)
        if plane == "x":
            grid = torch.stack([z, x.flatten(), y.flatten()], 1) + center
        elif plane == "y":
            grid = torch.stack([x.flatten(), z, y.flatten()], 1) + center
        else:
            grid = torch.stack([x.flatten(), y.flatten(), z], 1) + center
        fg = self.Reconstruct(f, grid[:, :self.dim], order)
        shape = (res, res) + tuple(np.shape(f)[1:])
        if return_grid:
            return x, y, fg.reshape(shape)
        return fg.reshape(shape)
