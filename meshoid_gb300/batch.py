"""Many snapshots through one C call (``mg_batched_run``), captured once in a
CUDA graph and replayed.

The reference processes snapshots one ``Meshoid`` at a time
(src/meshoid/Meshoid.py:15-105), then ``D`` (:237-268) and ``SurfaceDensity``
(:595-643) on each.  ``SnapshotBatch`` does the same work for a list of
snapshots with one host launch: per snapshot the cell index, plain seed,
neighbours and smoothing lengths, first derivatives of its fields and a column
density map of its masses, all stream-ordered without host synchronisation.
Results are identical to the per-snapshot ``Meshoid`` path with the same cell
parameters.

    batch = SnapshotBatch([(pos0, m0, f0), (pos1, m1, f1), ...], des_ngb=32, map_res=1024)
    batch.run()                       # graph replay; raises if a search did not finish
    batch.hsml[i], batch.grad[i], batch.maps[i]
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np
import torch

from . import _native as N
from ._native import check, ptr
from .meshoid import _dev_tensor, _np_median, _np_percentile, _plain_radius_factor, _stream

__all__ = ["SnapshotBatch", "tune_cell_parameters"]


def _map_frame(pos):
    """Map centre and size of Meshoid.SurfaceDensity's defaults: the median
    position and twice the 90th-percentile distance from it
    (src/meshoid/Meshoid.py:81-87)."""
    c = _np_median(pos)
    r2 = torch.sum((pos - c) ** 2, dim=1)
    return float(c[0]), float(c[1]), float(2.0 * float(_np_percentile(r2, 90.0)) ** 0.5)


class SnapshotBatch:
    """Snapshots: sequence of (pos (n,3), m (n,) or None, fields (n, nf) or
    (n,) or None).  Arrays may be numpy or torch; they are copied to the GPU
    once.  cell_params: per-snapshot (grid_level, level_bias, brick_threshold)
    or None for the defaults (see ``tune_cell_parameters``).

    lanes: the snapshots are split into this many groups (largest first, each
    to the group with the fewest particles so far) that run concurrently on
    their own streams, each with its own workspace, forked from and joined
    back to the launching stream (inside the captured graph as well), so that
    small snapshots, which cannot fill the GPU alone, overlap.  The 64
    snapshots of the benchmark batch: 318 ms in one lane, 209 ms in 4, 199 ms
    in 6 or 8 (GB300)."""

    def __init__(self, snapshots, des_ngb=32, map_res=1024, graph=True, cell_params=None, radius_factor=None,
                 device=None, lanes=8):
        if not torch.cuda.is_available():
            raise RuntimeError("meshoid_gb300 needs a CUDA device (GB300); no CPU path exists")
        self._lib = N.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.k = int(des_ngb)
        self.map_res = int(map_res) if map_res else 0
        self.radius_factor = float(radius_factor or _plain_radius_factor(self.k))
        self.pos, self.m, self.fields, self.hsml, self.grad, self.maps = [], [], [], [], [], []
        descs = (N.MgSnapshot * len(snapshots))()
        for i, snap in enumerate(snapshots):
            pos, m, f = (tuple(snap) + (None, None))[:3]
            pos = _dev_tensor(pos, torch.float64, self.device)
            if pos.ndim != 2 or pos.shape[1] != 3:
                raise ValueError("snapshot positions must be (n, 3)")
            n = pos.shape[0]
            if n < self.k:
                raise ValueError(f"snapshot {i} has fewer than des_ngb particles")
            if not bool(torch.isfinite(pos).all()):
                raise ValueError(f"snapshot {i}: positions contain NaN or infinity")
            m = torch.ones(n, dtype=torch.float64, device=self.device) if m is None else \
                _dev_tensor(m, torch.float64, self.device)
            if f is not None:
                f = _dev_tensor(f, torch.float64, self.device)
                f = f.reshape(n, -1).contiguous()
            nf = 0 if f is None else f.shape[1]
            h = torch.empty(n, dtype=torch.float64, device=self.device)
            g = torch.empty((n, nf, 3), dtype=torch.float32, device=self.device) if nf else None
            mp = torch.empty((self.map_res, self.map_res), dtype=torch.float64, device=self.device) \
                if self.map_res else None
            self.pos.append(pos)
            self.m.append(m)
            self.fields.append(f)
            self.hsml.append(h)
            self.grad.append(g)
            self.maps.append(mp)
            d = descs[i]
            d.n = n
            d.pos = pos.data_ptr()
            d.mass = m.data_ptr()
            d.fields = f.data_ptr() if nf else None
            d.nf = nf
            gl, lb, bt = (cell_params[i] if cell_params is not None and cell_params[i] is not None else (0, 1, 64))
            d.grid_level, d.level_bias, d.brick_threshold = int(gl), int(lb), int(bt)
            d.hsml = h.data_ptr()
            d.grad = g.data_ptr() if nf else None
            if mp is not None:
                cx, cy, size = _map_frame(pos)
                d.map = mp.data_ptr()
                d.map_cx, d.map_cy, d.map_size, d.map_res = cx, cy, size, self.map_res
            else:
                d.map = None
        self._descs = descs
        self.n_total = int(sum(p.shape[0] for p in self.pos))
        # lanes: longest-processing-time split by particle count
        ns = len(snapshots)
        lanes = max(1, min(int(lanes), ns))
        load = [0] * lanes
        members = [[] for _ in range(lanes)]
        for i in sorted(range(ns), key=lambda i: -self.pos[i].shape[0]):
            j = min(range(lanes), key=lambda j: load[j])
            members[j].append(i)
            load[j] += self.pos[i].shape[0]
        self._lanes = []
        order = []  # lane-major snapshot order of the counters
        ustore = torch.zeros(ns, dtype=torch.int32, device=self.device)
        sstore = torch.zeros((ns, 16), dtype=torch.int64, device=self.device)
        off = 0
        for mem in members:
            if not mem:
                continue
            d = (N.MgSnapshot * len(mem))()
            for t, i in enumerate(mem):
                ctypes.memmove(ctypes.byref(d[t]), ctypes.byref(descs[i]), ctypes.sizeof(N.MgSnapshot))
            wsb = self._lib.mg_batched_workspace_bytes(d, len(mem), self.k)
            if wsb == 0:
                raise ValueError("invalid snapshot batch")
            ws = torch.empty(wsb, dtype=torch.uint8, device=self.device)
            self._lanes.append((d, len(mem), ws, wsb, ustore[off:off + len(mem)], sstore[off:off + len(mem)],
                                torch.cuda.Stream(device=self.device)))
            order.extend(mem)
            off += len(mem)
        inv = [0] * ns
        for k_, i in enumerate(order):
            inv[i] = k_
        self._inv = torch.as_tensor(inv, device=self.device)
        self._ustore, self._sstore = ustore, sstore
        self._graph = None
        if graph:
            # one eager run on a side stream (the library's first launches load
            # its kernels), then capture
            s = torch.cuda.Stream(device=self.device)
            s.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(s):
                self._launch()
            torch.cuda.current_stream(self.device).wait_stream(s)
            torch.cuda.synchronize(self.device)
            self._graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self._graph):
                self._launch()

    @property
    def unresolved(self):
        """Per snapshot (input order): queries whose search did not finish."""
        return self._ustore[self._inv]

    @property
    def stats(self):
        """Per snapshot (input order): the 16 counters of mg_knn_hsml."""
        return self._sstore[self._inv]

    def _launch(self):
        from .meshoid import ctypes_stream
        main = torch.cuda.current_stream(self.device)
        for d, n, ws, wsb, ust, sst, s in self._lanes:
            s.wait_stream(main)
            with torch.cuda.stream(s):
                check(self._lib.mg_batched_run(d, n, self.k, self.radius_factor, ptr(ust), ptr(sst), ptr(ws), wsb,
                                               ctypes_stream(s)), "mg_batched_run")
        for lane in self._lanes:
            main.wait_stream(lane[6])

    def launch(self):
        """Queue the whole batch on the current stream (graph replay when
        captured); no host synchronisation."""
        if self._graph is not None:
            self._graph.replay()
        else:
            self._launch()

    def run(self):
        """launch(), then check that every search finished (one host sync)."""
        self.launch()
        bad = self.unresolved.cpu()
        if int(bad.sum()):
            raise N.MeshoidError(f"neighbour search did not resolve {bad.tolist()} queries per snapshot")
        return self


# ---- autotuner for the cell parameters -------------------------------------------
_tune_cache = {}
_tune_lock = threading.Lock()


def _size_class(n):
    return int(round(np.log2(max(n, 1))))


def tune_cell_parameters(pos, des_ngb=32, candidates=None, repeats=2, key=None):
    """Pick (grid_level, level_bias, brick_threshold) for a snapshot by timing
    the cell index + neighbour search of each candidate on it (CUDA events).
    Results are cached per key (default: size class round(log2 n) and des_ngb)
    under a lock; later snapshots of the same class reuse the choice."""
    from .meshoid import Meshoid
    from . import profiling
    pos = _dev_tensor(pos, torch.float64, torch.device("cuda", torch.cuda.current_device()))
    n = pos.shape[0]
    key = key if key is not None else (_size_class(n), int(des_ngb))
    with _tune_lock:
        if key in _tune_cache:
            return _tune_cache[key]
        lib = N.load()
        Ld = lib.mg_default_grid_level(n)
        if candidates is None:
            candidates = [(Ld, 0, 64), (Ld, 1, 64), (min(Ld + 1, 9), 0, 0), (Ld, 0, 0)]
        best, best_t = None, float("inf")
        rec = profiling.StageRecorder()
        for gl, lb, bt in candidates:
            Meshoid(pos, des_ngb=des_ngb, grid_level=gl, level_bias=lb, brick_threshold=bt)  # warm
            torch.cuda.synchronize()
            rec.reset()
            profiling.set_recorder(rec)
            try:
                for _ in range(repeats):
                    Meshoid(pos, des_ngb=des_ngb, grid_level=gl, level_bias=lb, brick_threshold=bt)
                torch.cuda.synchronize()
            finally:
                profiling.set_recorder(None)
            t = sum(v for s, v in rec.totals().items() if s in ("build_cells", "seed", "knn_hsml"))
            if t < best_t:
                best, best_t = (gl, lb, bt), t
        _tune_cache[key] = best
        return best
