"""Mixed precision and many right-hand sides at full size: N = 2^24 clump
mixture (64 Gaussian clumps, widths log-uniform in [1e-3, 1e-1], Dirichlet(1)
weights, 20% uniform background), 16 scalar Fourier fields (8 modes each,
|k| in [1, 32]) plus a 3-vector field, i.e. F = 19 components in one sweep,
first- and second-order derivatives, against the FP64 oracle on a seeded
sample of 10,000 queries, end to end (the oracle at its own h); the max and
rms error of every field are reported.  The neighbour sets, their FP64
distances and h of all 16,777,216 rows are checked as well, in chunks of
2^20 queries on all host cores.

Order 1 runs the FP32 sweep (FP64 re-solve of flagged rows); order 2 the
float-float sweep at the float-float h.  Both are held to 1e-5; at order 2
rows whose FP64 answer is not reproducible (it moves by more than 2.5e-6 when
h is scaled by 1 + 1e-12) are exempt, and their fraction is asserted small."""
import os

import numpy as np
import pytest

from gpu_util import order2_reference, row_rel_err, sets_equal_rows

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N = 1 << 24
NS = 10000
CHUNK = 1 << 20
D1_TOL = 1e-5
D2_TOL = 1e-5


@pytest.fixture(scope="module")
def clumps():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scipy.spatial import cKDTree

    from meshoid_gb300 import Meshoid
    from meshoid_gb300 import synthetic as S
    from oracle import oracle as O
    pos = S.clump_mixture(N, seed=7)
    pos_t = torch.as_tensor(pos, device="cuda")
    f = torch.cat([S.fourier_fields_torch(pos_t, 16, seed=8), S.fourier_fields_torch(pos_t, 3, seed=9, kmax=8)], 1)
    M = Meshoid(pos_t, des_ngb=32)
    q = np.sort(np.random.default_rng(1).choice(N, NS, replace=False))
    tree = cKDTree(pos)
    dist, ngb = O.knn(pos, 32, queries=q, tree=tree)
    return pos, f, M, q, dist, ngb, tree


def _per_field(got, ref):
    """(NS, F, c) arrays -> per-field row-relative errors (NS, F)."""
    return np.stack([row_rel_err(got[:, j], ref[:, j]) for j in range(got.shape[1])], 1)


def _report(name, e):
    lines = [f"{name} field {j:2d}: max {e[:, j].max():.2e} rms {np.sqrt(np.mean(e[:, j] ** 2)):.2e}"
             for j in range(e.shape[1])]
    print("\n" + "\n".join(lines))


def test_clumps_2e24_tree_and_order1(clumps):
    from oracle import oracle as O
    pos, f, M, q, dist, ngb, _ = clumps
    qt = torch.as_tensor(q, device="cuda")
    assert sets_equal_rows(M.ngb[qt].cpu().numpy(), ngb) == 0
    h_ref, _ = O.hsml_iter(dist, 3, 1e-13)
    h = M.kernel_radius[qt].cpu().numpy()
    assert np.max(np.abs(h / h_ref - 1)) <= 1e-6
    W, _ = O.gradient_weights(pos, ngb, h_ref, q, None, True, 1)
    ref = O.apply_weights(W, ngb, q, f.cpu().numpy())
    got = M.D(f)[qt].double().cpu().numpy()
    e = _per_field(got, ref)
    _report("D order 1 (end to end)", e)
    assert e.max() <= D1_TOL
    W, _ = O.gradient_weights(pos, ngb, h, q, None, True, 1)
    e = _per_field(got, O.apply_weights(W, ngb, q, f.cpu().numpy()))
    _report("D order 1 (oracle at the GPU's h)", e)
    assert e.max() <= D1_TOL


def test_clumps_2e24_all_rows_sets_and_h(clumps):
    from oracle import oracle as O
    pos, f, M, q, dist, ngb, tree = clumps
    O.set_threads(os.cpu_count() or 1)
    ngb_gpu, dist_gpu, h_gpu = M.ngb, M.ngbdist, M.kernel_radius
    bad_sets, dist_bad, eh = 0, 0.0, []
    for c0 in range(0, N, CHUNK):
        qc = np.arange(c0, min(N, c0 + CHUNK))
        dc, nc = O.knn(pos, 32, queries=qc, tree=tree)
        bad_sets += sets_equal_rows(ngb_gpu[c0:c0 + len(qc)].cpu().numpy(), nc)
        dd = dist_gpu[c0:c0 + len(qc)].double().cpu().numpy()
        dist_bad = max(dist_bad, float(np.max(np.abs(dd - dc) / np.maximum(dc, 1e-300))))
        h_ref, _ = O.hsml_iter(dc, 3, 1e-13)
        eh.append(np.abs(h_gpu[c0:c0 + len(qc)].double().cpu().numpy() / h_ref - 1))
    eh = np.concatenate(eh)
    print(f"\nall {N} rows: neighbour sets differing {bad_sets}, distance rel err max {dist_bad:.2e}, "
          f"h rel err max {eh.max():.2e} rms {np.sqrt(np.mean(eh ** 2)):.2e}")
    assert bad_sets == 0
    assert dist_bad <= 1e-14
    assert eh.max() <= 1e-6


def test_clumps_2e24_order2(clumps):
    from oracle import oracle as O
    pos, f, M, q, dist, ngb, _ = clumps
    qt = torch.as_tensor(q, device="cuda")
    h_ref, _ = O.hsml_iter(dist, 3, 1e-13)
    fn = f.cpu().numpy()
    ref, exempt = order2_reference(pos, ngb, h_ref, q, fn)  # (NS, F, 9): 3 first + 6 second derivatives
    g1 = M.D(f, order=2)[qt].double().cpu().numpy()
    g2 = M.D2(f)[qt].double().cpu().numpy()
    e1 = _per_field(g1, ref[..., :3])
    e2 = _per_field(g2, ref[..., 3:])
    ok = ~exempt
    print(f"\norder 2: exempt rows {exempt.mean():.4f}")
    _report("D order 2 (end to end, reproducible rows)", e1[ok])
    _report("D2 (end to end, reproducible rows)", e2[ok])
    assert exempt.mean() < 0.03
    assert e1[ok].max() <= D2_TOL
    assert e2[ok].max() <= D2_TOL
