"""Full-size checks on the GPU (Plummer sphere, N = 2^22, des_ngb = 32 -- the
benchmark workload).  The oracle cannot run the whole set in seconds, so
parity is checked on a seeded sample of 20,000 queries (neighbour sets,
FP64 distances, h, first derivatives of the benchmark's five field components)
plus size-independent properties over all particles."""
import numpy as np
import pytest

from gpu_util import as_np, row_rel_err, sets_equal_rows, summary

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N_FULL = 1 << 22


@pytest.fixture(scope="module")
def full():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshoid_gb300 import Meshoid
    from meshoid_gb300 import synthetic as S
    pos = S.plummer(N_FULL, seed=2)
    m = np.full(N_FULL, 1.0 / N_FULL)
    v = S.rotation_velocity(pos, seed=3)
    M = Meshoid(pos, m, des_ngb=32)
    f = np.c_[np.log(as_np(M.density)), pos[:, 0] * pos[:, 1] * pos[:, 2], v]
    return pos, m, f, M


def test_full_sampled_parity(full):
    from scipy.spatial import cKDTree

    from oracle import oracle as O
    pos, m, f, M = full
    rng = np.random.default_rng(0)
    q = np.sort(rng.choice(N_FULL, 20000, replace=False))
    tree = cKDTree(pos)
    dist, ngb = O.knn(pos, 32, queries=q, tree=tree)
    got_ngb = as_np(M.ngb)[q]
    assert sets_equal_rows(got_ngb, ngb) == 0
    np.testing.assert_allclose(as_np(M.ngbdist)[q], dist, rtol=1e-14, atol=0)
    h_ref, _ = O.hsml_iter(dist, 3, 1e-13)
    h = as_np(M.kernel_radius)[q]
    assert np.max(np.abs(h / h_ref - 1)) <= 1e-6, summary(np.abs(h / h_ref - 1))
    W, _ = O.gradient_weights(pos, ngb, h_ref, q, None, True, 1)
    ref = O.apply_weights(W, ngb, q, f)
    got = as_np(M.D(f))[q]
    e = row_rel_err(got, ref)
    assert e.max() <= 1e-5, summary(e)


def test_full_properties(full):
    pos, m, f, M = full
    k = 32
    ngb = M.ngb
    # self is a neighbour (distance 0) of every particle; rows are sorted ascending
    assert bool((ngb[:, 0] == torch.arange(N_FULL, device=ngb.device)).all())
    d = M.ngbdist
    assert bool((d[:, 1:] >= d[:, :-1]).all())
    # h solves norm * sum_j W(d_j / h) = k (FP64 check over all particles)
    h = M.kernel_radius
    qq = d / h[:, None]
    w = torch.where(qq <= 0.5, 1 - 6 * qq ** 2 + 6 * qq ** 3, torch.where(qq <= 1.0, 2 * (1 - qq) ** 3,
                                                                            torch.zeros_like(qq)))
    n = (32.0 / 3.0) * w.sum(1)
    assert float((n - k).abs().max()) <= 2e-4 * k
    # D of a linear field is exact; kernel average of a constant is the constant
    lin = 2.0 * pos[:, 0] - 3.0 * pos[:, 1] + 0.5 * pos[:, 2]
    dl = as_np(M.D(lin))
    assert np.max(np.abs(dl - np.array([2.0, -3.0, 0.5]))) <= 3e-5
    ka = as_np(M.KernelAverage(np.full(N_FULL, 3.0)))
    assert np.max(np.abs(ka - 3.0)) <= 3e-6
