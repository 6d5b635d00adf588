"""The order-2 refinement step of the FP32 derivative sweep (k_grad<DIM, 2, 4,
true>, switched by mg_grad_set_refine; the "fp32" order-2 method of
set_order2_method) on the GPU, against the FP64 oracle.

Rows whose FP32 order-2 answer fails the matrix-rounding test are refined once
in FP32 with a float-float residual instead of being re-solved in FP64.  The
test runs order 2 with the step off and on, on a Plummer sphere and on a clump
mixture with fields that vary inside the kernel, and checks that
  * the refined answers meet the same per-row bound against the oracle as the
    FP64 path (the oracle evaluated at the GPU's h: the sweep's arithmetic);
  * some rows carry MG_Q_REFINED, no row carries both MG_Q_REFINED and
    MG_Q_FP64_SOLVE, and fewer rows reach the FP64 re-solve than with the
    step off.
Reference arithmetic: src/meshoid/derivatives.py:56-138, Meshoid.py:270-295.
"""
import numpy as np
import pytest

from gpu_util import row_rel_err, summary

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

D2_A, D2_B = 2e-6, 1e-5


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _run(M, f, on):
    import meshoid_gb300
    prev_m = meshoid_gb300.set_order2_method("fp32")
    prev = meshoid_gb300.set_order2_refinement(on)
    try:
        d2 = M.D2(f).double().cpu().numpy()
        d1 = M.D(f, order=2).double().cpu().numpy()
        st = M._gstatus.cpu().numpy()
    finally:
        meshoid_gb300.set_order2_refinement(prev)
        meshoid_gb300.set_order2_method(prev_m)
    return d1, d2, st


@pytest.mark.parametrize("kind", ["plummer", "clumps"])
def test_order2_refinement_vs_oracle(kind):
    from meshoid_gb300 import Meshoid
    from meshoid_gb300 import _native as NAT
    from meshoid_gb300 import synthetic as S
    from oracle import oracle as O
    n = 1 << 15
    if kind == "plummer":
        pos = S.plummer(n, seed=41)
        f = np.c_[np.log1p(np.sum(pos ** 2, 1)), pos[:, 0] * pos[:, 1] * pos[:, 2],
                  S.rotation_velocity(pos, seed=42)]
    else:
        pos = S.clump_mixture(n, seed=43)
        f = S.fourier_fields(pos, 8, seed=44)
    M = Meshoid(pos, des_ngb=32, cond_threshold=(30.0, 1e5))
    h = M.kernel_radius.cpu().numpy()
    ngb = M.ngb.cpu().numpy().astype(np.int64)
    q = np.arange(n)
    W, _ = O.gradient_weights(pos, ngb, h, q, None, True, 2)
    ref = O.apply_weights(W, ngb, q, f)  # (n, F, 9)
    cond = O.moment_condition(pos, ngb, h, q, order=2)
    ok = np.isfinite(cond) & (cond < 1e8)
    res = {}
    for on in (False, True):
        d1, d2, st = _run(M, f, on)
        res[on] = st
        for got, sl in ((d1, slice(0, 3)), (d2, slice(3, 9))):
            e = np.stack([row_rel_err(got[:, j], ref[:, j, sl]) for j in range(f.shape[1])], 1).max(1)
            bound = D2_A * cond + D2_B
            assert np.all(e[ok] <= bound[ok]), (on, f"worst excess {np.max(e[ok] / bound[ok]):.3g}", summary(e[ok]))
    refined = (res[True] & NAT.MG_Q_REFINED) != 0
    fp64_on = (res[True] & NAT.MG_Q_FP64_SOLVE) != 0
    fp64_off = (res[False] & NAT.MG_Q_FP64_SOLVE) != 0
    print(f"\n{kind}: FP64 rows off {fp64_off.mean():.4f}, on {fp64_on.mean():.4f}, refined {refined.mean():.4f}")
    assert not np.any(refined & fp64_on)
    assert not np.any((res[False] & NAT.MG_Q_REFINED) != 0)
    assert fp64_on.sum() < fp64_off.sum()
    if fp64_off.mean() > 0.01:
        assert refined.sum() > 0
