"""CPU emulation of the order-2 derivative sweep's FP32 arithmetic (k_grad in
meshoid_gb300/csrc/mg_grad.cu) and of its refinement step (k_grad<DIM, 2, NF,
true>, switched by mg_grad_set_refine), against FP64 least squares at the same
h (src/meshoid/derivatives.py:56-138 with coordinates scaled by h).

Workload: seeded rows of the clump mixture (64 Gaussian clumps + 20% uniform
background) with the 16 Fourier scalar fields (|k| <= 32) and the 3-vector
field (|k| <= 8) of the 2^24 benchmark target, at N = 2^22.  The test pins the
numerical argument for the step: the FP32 answer misses the order-2 tolerance
(2e-6 cond + 1e-5 per field and row) on a fraction of the rows, all of which
the sweep's flags catch (mostly the matrix rounding test); one step with the
residual carried in
float-float brings every row whose factor succeeds and whose condition
estimate is <= 1e7 far inside it.  This emulates the arithmetic, not the
kernel: the GPU tests check the kernel.
"""
import numpy as np
import pytest

from gpu_util import row_rel_err

f32 = np.float32
N, NS, K = 1 << 22, 3000, 32
ND = 9


def fma(a, b, c):
    """FP32 fused multiply-add: the FP32 product is exact in FP64, one rounding."""
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(f32)


def two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    return s, ((a - (s - bb).astype(f32)).astype(f32) + (b - bb).astype(f32)).astype(f32)


def hilo(v):
    hi = v.astype(f32)
    return hi, (v - hi.astype(np.float64)).astype(f32)


def basis(x):
    return np.stack([x[..., 0], x[..., 1], x[..., 2], 0.5 * x[..., 0] ** 2, 0.5 * x[..., 1] ** 2,
                     0.5 * x[..., 2] ** 2, x[..., 0] * x[..., 1], x[..., 1] * x[..., 2], x[..., 2] * x[..., 0]], -1)


def basis32(x):
    h = f32(0.5)
    return np.stack([x[..., 0], x[..., 1], x[..., 2], (h * x[..., 0] * x[..., 0]).astype(f32),
                     (h * x[..., 1] * x[..., 1]).astype(f32), (h * x[..., 2] * x[..., 2]).astype(f32),
                     (x[..., 0] * x[..., 1]).astype(f32), (x[..., 1] * x[..., 2]).astype(f32),
                     (x[..., 2] * x[..., 0]).astype(f32)], -1).astype(f32)


def spline32(q):
    inner = fma((q * q).astype(f32), fma(f32(6), q, f32(-6)), f32(1))
    a = np.maximum(f32(1) - q, f32(0)).astype(f32)
    outer = (f32(2) * a * a * a).astype(f32)
    return np.where(q <= f32(0.5), inner, outer).astype(f32)


def chol_solve(L, b):
    """FP32 forward and back substitution with the packed lower factor, as chol_solve<N>."""
    x = b.copy()
    for i in range(ND):
        t = x[..., i].copy()
        for p in range(i):
            t = (t - L[:, None, i * (i + 1) // 2 + p] * x[..., p]).astype(f32)
        x[..., i] = (t / L[:, None, i * (i + 1) // 2 + i]).astype(f32)
    for i in range(ND - 1, -1, -1):
        t = x[..., i].copy()
        for p in range(i + 1, ND):
            t = (t - L[:, None, p * (p + 1) // 2 + i] * x[..., p]).astype(f32)
        x[..., i] = (t / L[:, None, i * (i + 1) // 2 + i]).astype(f32)
    return x


@pytest.fixture(scope="module")
def sample():
    from scipy.spatial import cKDTree

    from meshoid_gb300 import synthetic as S
    from oracle import oracle as O
    pos = S.clump_mixture(N, seed=7)
    q = np.sort(np.random.default_rng(3).choice(N, NS, replace=False))
    dist, ngb = O.knn(pos, K, queries=q, tree=cKDTree(pos))
    h, _ = O.hsml_iter(dist, 3, 1e-13)
    idx = np.unique(np.concatenate([ngb.ravel(), q]))
    f = np.c_[S.fourier_fields(pos[idx], 16, seed=8), S.fourier_fields(pos[idx], 3, seed=9, kmax=8)]
    return pos[q], pos[ngb], h.astype(f32), f[np.searchsorted(idx, ngb)], f[np.searchsorted(idx, q)]


def test_refinement_step_meets_the_order2_tolerance(sample):
    pq, pn, h32, fj, fi = sample
    F = fj.shape[2]
    hinv = (f32(1) / h32).astype(f32)
    hd = h32.astype(np.float64)
    # FP64 truth at the FP32 h
    x64 = (pn - pq[:, None]) / hd[:, None, None]
    r64 = np.sqrt((x64 ** 2).sum(-1))
    w64 = np.where(r64 <= 0.5, 1 - 6 * r64 ** 2 + 6 * r64 ** 3, np.where(r64 <= 1, 2 * (1 - r64) ** 3, 0.0))
    a64 = basis(x64)
    A64 = np.einsum("nk,nki,nkj->nij", w64, a64, a64)
    sol64 = np.einsum("nij,nfj->nfi", np.linalg.pinv(A64, rcond=1e-15),
                      np.einsum("nk,nki,nkf->nfi", w64, a64, fj - fi[:, None]))
    cond = np.linalg.cond(A64)
    # FP32 pass: separations and field differences from the hi/lo splits
    qh, ql = hilo(pq)
    nh, nl = hilo(pn)
    s_, e_ = two_sum(nh, np.broadcast_to(-qh[:, None], nh.shape).astype(f32))
    d32, e2 = two_sum(s_, (nl - ql[:, None]).astype(f32))
    dlo = (e2 + e_).astype(f32)
    x32 = (d32 * hinv[:, None, None]).astype(f32)
    r2 = np.zeros(x32.shape[:2], f32)
    for c in range(3):
        r2 = fma(x32[..., c], x32[..., c], r2)
    w32 = spline32(np.sqrt(r2).astype(f32))
    a32 = basis32(x32)
    wa = (w32[..., None] * a32).astype(f32)
    fh_j, fl_j = hilo(fj)
    fh_i, fl_i = hilo(fi)
    df = ((fh_j - fh_i[:, None]).astype(f32) + (fl_j - fl_i[:, None]).astype(f32)).astype(f32)
    M = np.zeros((NS, ND * (ND + 1) // 2), f32)
    rhs = np.zeros((NS, F, ND), f32)
    cmp = np.zeros((NS, F, ND), f32)
    cabs = np.zeros((NS, F), f32)
    for j in range(K):
        for i in range(ND):
            for jj in range(i + 1):
                M[:, i * (i + 1) // 2 + jj] = fma(wa[:, j, i], a32[:, j, jj], M[:, i * (i + 1) // 2 + jj])
        cabs = fma(w32[:, j, None], np.abs(df[:, j]), cabs)
        for m in range(ND):  # Kahan-compensated right-hand sides
            y = fma(wa[:, j, m, None], df[:, j], -cmp[:, :, m])
            t = (rhs[:, :, m] + y).astype(f32)
            cmp[:, :, m] = ((t - rhs[:, :, m]).astype(f32) - y).astype(f32)
            rhs[:, :, m] = t
    L = M.copy()
    ok = np.ones(NS, bool)
    for j in range(ND):
        s = L[:, j * (j + 1) // 2 + j].copy()
        for p in range(j):
            s = (s - L[:, j * (j + 1) // 2 + p] ** 2).astype(f32)
        ok &= s > 0
        d = np.sqrt(np.where(s > 0, s, f32(1))).astype(f32)
        L[:, j * (j + 1) // 2 + j] = d
        for i in range(j + 1, ND):
            t = L[:, i * (i + 1) // 2 + j].copy()
            for p in range(j):
                t = (t - L[:, i * (i + 1) // 2 + p] * L[:, j * (j + 1) // 2 + p]).astype(f32)
            L[:, i * (i + 1) // 2 + j] = (t * (f32(1) / d)).astype(f32)
    # condition estimate trace(M) trace(M^-1), as cond_estimate<9>
    tri = np.zeros(NS, f32)
    for c in range(ND):
        xv = np.zeros((NS, ND), f32)
        for i in range(c, ND):
            t = np.full(NS, f32(1) if i == c else f32(0))
            for p in range(c, i):
                t = (t - L[:, i * (i + 1) // 2 + p] * xv[:, p]).astype(f32)
            xv[:, i] = (t / L[:, i * (i + 1) // 2 + i]).astype(f32)
            tri = (tri + xv[:, i] ** 2).astype(f32)
    cest = (sum(M[:, i * (i + 1) // 2 + i] for i in range(ND)) * tri).astype(np.float64)
    X = chol_solve(L, rhs)
    # the sweep's flags
    em = 6e-8 * cest
    tol = 1e-5 + 2e-6 * cest
    n1 = (X[..., :3].astype(np.float64) ** 2).sum(-1)
    n2 = (X[..., 3:].astype(np.float64) ** 2).sum(-1)
    flag_matrix = ((em[:, None] ** 2) * (n1 + n2) > tol[:, None] ** 2 * n2).any(1)
    flag_rhs = ((em[:, None] * cabs) ** 2 > tol[:, None] ** 2 * (rhs.astype(np.float64) ** 2).sum(-1)).any(1)

    # one refinement step, as the kernel computes it
    xl = (fma(d32, np.broadcast_to(hinv[:, None, None], d32.shape), -x32) +
          (dlo * hinv[:, None, None]).astype(f32)).astype(f32)
    res = np.zeros_like(rhs)
    for j in range(K):
        sh = np.zeros((NS, F), f32)
        sl = np.zeros((NS, F), f32)
        for c in range(3):
            p = (x32[:, j, c, None] * X[..., c]).astype(f32)
            pe = fma(np.broadcast_to(x32[:, j, c, None], p.shape), X[..., c], -p)
            sh, te = two_sum(sh, p)
            sl = (sl + ((te + pe).astype(f32) + (xl[:, j, c, None] * X[..., c]).astype(f32))).astype(f32)
        quad = np.zeros((NS, F), f32)
        for m in range(3, ND):
            quad = fma(np.broadcast_to(a32[:, j, m, None], quad.shape), X[..., m], quad)
        dh, de = two_sum(fh_j[:, j], -fh_i)
        dlf = ((fl_j[:, j] - fl_i).astype(f32) + de).astype(f32)
        e = (((dh - sh).astype(f32) + (dlf - sl).astype(f32)).astype(f32) - quad).astype(f32)
        for m in range(ND):
            res[:, :, m] = fma(wa[:, j, m, None], e, res[:, :, m])
    Xr = (X + chol_solve(L, res)).astype(f32)

    def ratio(Y):
        hh = hd[:, None, None]
        e1 = np.stack([row_rel_err(Y[:, c, :3] / hh[:, 0], sol64[:, c, :3] / hh[:, 0]) for c in range(F)], 1)
        e2 = np.stack([row_rel_err(Y[:, c, 3:] / hh[:, 0] ** 2, sol64[:, c, 3:] / hh[:, 0] ** 2)
                       for c in range(F)], 1)
        return (np.maximum(e1, e2) / (2e-6 * cond[:, None] + 1e-5)).max(1)

    good = cond < 1e8
    before, after = ratio(X), ratio(Xr)
    kept = ok & good & (cest <= 1e7)
    print(f"\nflags: matrix {flag_matrix.mean():.3f} rhs {flag_rhs.mean():.3f} factor failed {(~ok).mean():.3f} "
          f"estimate>1e5 {(cest > 1e5).mean():.3f}; FP32 misses the bound on {(before[good] > 1).mean():.3f} "
          f"(worst {before[good].max():.2f}x); refined worst {after[kept].max():.4f}x on {kept.mean():.3f}")
    assert (before[good] > 1).mean() > 0.01          # the FP32 answer alone is not enough
    flagged = flag_matrix | flag_rhs | (cest > 1e5) | ~ok
    assert np.all(flagged[good & (before > 1)])      # and the sweep flags every such row
    assert flag_rhs.mean() < 0.01
    assert kept.mean() > 0.95
    assert after[kept].max() < 0.1                  # one step: far inside the bound
