"""Shared helpers for the GPU parity tests (tolerances live in the tests)."""
import numpy as np


def as_np(t):
    try:
        import torch
        if isinstance(t, torch.Tensor):
            return t.detach().double().cpu().numpy() if t.is_floating_point() else t.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(t)


def sets_equal_rows(a, b):
    """Row-wise set equality of neighbour index arrays; returns the mismatching row count."""
    a = np.sort(np.asarray(a), axis=1)
    b = np.sort(np.asarray(b), axis=1)
    return int(np.sum(np.any(a != b, axis=1)))


def row_rel_err(got, ref, floor_frac=1e-3):
    """Per-row ||got - ref|| / max(||ref||, floor_frac * median ||ref||)."""
    got = np.asarray(got, dtype=np.float64).reshape(len(got), -1)
    ref = np.asarray(ref, dtype=np.float64).reshape(len(ref), -1)
    scale = np.linalg.norm(ref, axis=1)
    floor = floor_frac * max(np.median(scale), 1e-300)
    return np.linalg.norm(got - ref, axis=1) / np.maximum(scale, floor)


def summary(err):
    err = np.asarray(err)
    return f"max {err.max():.3g} rms {np.sqrt(np.mean(err ** 2)):.3g}"


def order2_errors(got1, got2, ref):
    """Per-row error of an order-2 result: got1 (rows, F, dim) first
    derivatives, got2 (rows, F, nd2) second derivatives, ref (rows, F, dim +
    nd2) the oracle's.  Each part of each field is measured by row_rel_err on
    its own; the row's error is the largest of them."""
    got1 = np.asarray(got1, dtype=np.float64)
    got2 = np.asarray(got2, dtype=np.float64)
    n = len(ref)
    ref = np.asarray(ref, dtype=np.float64).reshape(n, -1, ref.shape[-1])
    got1 = got1.reshape(n, ref.shape[1], -1)
    got2 = got2.reshape(n, ref.shape[1], -1)
    dim = got1.shape[2]
    e = np.zeros(n)
    for j in range(ref.shape[1]):
        e = np.maximum(e, row_rel_err(got1[:, j], ref[:, j, :dim]))
        e = np.maximum(e, row_rel_err(got2[:, j], ref[:, j, dim:]))
    return e


def order2_reference(pos, ngb, h, rows, f, boxsize=None, weighted=True, nudge=1e-12, tol=1e-5):
    """The oracle's order-2 answer (D and D2 of f, (rows, F, dim + nd2)) at
    smoothing lengths h, and the rows whose FP64 answer is not reproducible
    to tol: those that move by more than tol / 4 when h is scaled by
    1 + nudge.  A row that sensitive (near-singular moment matrix, condition
    ~1e10 and above) carries FP64 rounding noise of that order in the
    reference itself, so a second FP64 implementation -- another elimination
    order, another summation order -- differs from it by about twice that."""
    from oracle import oracle as O
    f = np.asarray(f, dtype=np.float64)
    f2 = f.reshape(len(f), -1)
    W, _ = O.gradient_weights(pos, ngb, h, rows, boxsize, weighted, 2)
    ref = O.apply_weights(W, ngb, rows, f2)
    W, _ = O.gradient_weights(pos, ngb, np.asarray(h) * (1.0 + nudge), rows, boxsize, weighted, 2)
    alt = O.apply_weights(W, ngb, rows, f2)
    dim = np.asarray(pos).reshape(len(pos), -1).shape[1]
    exempt = order2_errors(alt[..., :dim], alt[..., dim:], ref) > 0.25 * tol
    return ref, exempt


def far_clump(n_bg=20000, n_clump=8000, sigma=5e-8, seed=71):
    """A uniform box [0, 1000]^3 with a tight Gaussian clump (sigma) at
    (900, 900, 900): the clump's neighbour separations are ~1e-10 of the
    coordinates' distance from the frame centre.  The background keeps out
    of a ball of radius 250 around the clump, so that no background
    particle has clump members among its 32 nearest (seen from outside, the
    whole clump lies at one distance to ~1e-9)."""
    rng = np.random.default_rng(seed)
    c = np.array([900.0, 900.0, 900.0])
    bg = rng.uniform(0.0, 1000.0, (2 * n_bg, 3))
    bg = bg[np.sum((bg - c) ** 2, axis=1) > 250.0 ** 2][:n_bg]
    cl = c + sigma * rng.standard_normal((n_clump, 3))
    return np.vstack([bg, cl])


def hilo_d2(pos, q, rows):
    """The search's FP32 squared distances from query q to the particles rows:
    positions relative to the frame centre (the cube of side max extent,
    padded, over the bounding box), split into FP32 hi + lo, separations
    (hb - ha) + (lb - la) in FP32, squares summed in FP32."""
    lo, hi = pos.min(0), pos.max(0)
    mag = np.abs(np.r_[lo, hi]).max()
    side = (hi - lo).max() * (1.0 + 1.0 / 1048576.0) + mag * 1e-12
    r = pos - (lo + 0.5 * side)
    h = r.astype(np.float32)
    lw = (r - h.astype(np.float64)).astype(np.float32)
    s = (h[rows] - h[q]) + (lw[rows] - lw[q])
    return (s * s).sum(axis=1, dtype=np.float32), float(np.abs(h[q]).max())
