"""Order-2 derivatives -- D(f, order=2) and D2(f) -- on the GPU against the
reference's own outputs and the FP64 oracle, end to end (each side at its own
smoothing lengths).

Tolerance: every row within 1e-5, row-relative, of the reference's FP64
answer, the first- and second-derivative parts of every field measured
separately (tests/gpu_util.order2_errors).  Rows whose FP64 answer is not
reproducible are exempt: those whose oracle answer moves by more than 2.5e-6
when h is scaled by 1 + 1e-12 (a near-singular moment matrix; the reference
raises LinAlgError on an exactly singular one, src/meshoid/derivatives.py:132).
The exempt fraction is asserted small, and the max / rms errors are printed.

Reference: src/meshoid/derivatives.py:27-138, src/meshoid/Meshoid.py:237-295,
src/meshoid/kernel_density.py:15-56 (the h the fit is evaluated at).
"""
import numpy as np
import pytest

from gpu_util import as_np, order2_errors, order2_reference, row_rel_err, sets_equal_rows, summary

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _mesh(*a, **k):
    from meshoid_gb300 import Meshoid
    return Meshoid(*a, **k)


def _d2_errors(got2, ref, dim):
    """Second-derivative part only (the goldens store D2 alone)."""
    got2 = np.asarray(got2, dtype=np.float64)
    n = len(ref)
    ref = ref.reshape(n, -1, ref.shape[-1])
    got2 = got2.reshape(n, ref.shape[1], -1)
    e = np.zeros(n)
    for j in range(ref.shape[1]):
        e = np.maximum(e, row_rel_err(got2[:, j], ref[:, j, dim:]))
    return e


def _report(name, e, exempt):
    ok = ~exempt
    print(f"\n{name}: rows {len(e)}, exempt {exempt.mean():.4f}, {summary(e[ok])}")
    assert exempt.mean() < 0.05, name
    assert e[ok].max() <= TOL, (name, summary(e[ok]), np.argsort(-np.where(ok, e, 0))[:5])


# ---- the reference's own outputs -----------------------------------------------------

@pytest.mark.parametrize("name,kw,dim", [
    ("uniform_1024", {"des_ngb": 32}, 3),
    ("periodic_768", {"des_ngb": 32, "boxsize": 1.0}, 3),
    ("uniform2d_900", {}, 2),
    ("uniform_ngb64_1200", {"des_ngb": 64}, 3),
])
def test_order2_goldens(golden, name, kw, dim):
    g = golden(name)
    if "D2" not in g:
        pytest.skip("the reference raised LinAlgError on this set")
    M = _mesh(g["pos"], g.get("m"), **kw)
    ngb = g["ngb"].astype(np.int64)
    rows = np.arange(len(g["pos"]))
    ref, exempt = order2_reference(g["pos"], ngb, g["hsml"], rows, g["f"], boxsize=kw.get("boxsize"))
    e = _d2_errors(as_np(M.D2(g["f"])), ref, dim)
    # the oracle restates the reference: on the reproducible rows its D2 is the golden output
    gd2 = g["D2"].reshape(ref[..., dim:].shape)
    e_or = np.max([row_rel_err(ref[:, j, dim:], gd2[:, j]) for j in range(ref.shape[1])], axis=0)
    assert e_or[~exempt].max() <= 1e-7, summary(e_or[~exempt])
    if "D1_order2" in g:
        e = np.maximum(e, row_rel_err(as_np(M.D(g["f"], order=2)), g["D1_order2"]))
    _report(name, e, exempt)


def test_order2_golden_lowdim(golden):
    """1-D (default des_ngb 4; and des_ngb 8 on a periodic line) and a periodic
    2-D box: their order-2 fits have 2 and 5 unknowns."""
    g = golden("lowdim")
    for key, x, f, kw, dim in (("1", g["x1"], g["f1"], {}, 1), ("p", g["xp"], g["fp"], {"des_ngb": 8, "boxsize": 1.0}, 1),
                               ("2", g["x2"], g["f2"], {"boxsize": 1.0}, 2)):
        if f"D2_{key}" not in g:
            continue
        M = _mesh(x, **kw)
        ngb = g[f"ngb{key}"].astype(np.int64)
        rows = np.arange(len(x))
        ref, exempt = order2_reference(x, ngb, g[f"hsml{key}"], rows, f, boxsize=kw.get("boxsize"))
        e = _d2_errors(as_np(M.D2(f)), ref, dim)
        _report(f"lowdim {key}", e, exempt)


def test_order2_golden_notebook(golden):
    """The reference's test notebook (test/test_gradients.ipynb) at N = 2000:
    periodic box, des_ngb = 100, D2 of every product x_i x_j."""
    g = golden("notebook_2000")
    x = g["x"]
    M = _mesh(x, des_ngb=100, boxsize=1.0)
    ngb = g["ngb"].astype(np.int64)
    rows = np.arange(len(x))
    for i in range(3):
        for j in range(i, 3):
            f = x[:, i] * x[:, j]
            ref, exempt = order2_reference(x, ngb, g["hsml"], rows, f, boxsize=1.0)
            _report(f"notebook D2 x{i}x{j}", _d2_errors(as_np(M.D2(f)), ref, 3), exempt)


# ---- the oracle at larger sizes ------------------------------------------------------

def _sets():
    from meshoid_gb300 import synthetic as S
    n = 1 << 16
    u = S.uniform(n, seed=51)
    p = S.plummer(n, seed=52)
    c = S.clump_mixture(n, seed=53)
    return [
        ("uniform", u, S.fourier_fields(u, 3, seed=54, kmax=8), {"des_ngb": 32}),
        ("plummer", p, np.c_[np.log1p(np.sum(p ** 2, 1)), p[:, 0] * p[:, 1] * p[:, 2], S.rotation_velocity(p, seed=55)],
         {"des_ngb": 32}),
        ("clumps", c, S.fourier_fields(c, 8, seed=56), {"des_ngb": 32}),
        ("periodic", S.uniform(1 << 15, seed=57), None, {"des_ngb": 32, "boxsize": 1.0}),
        ("2-D", S.uniform(1 << 15, seed=58, dim=2), None, {}),
    ]


@pytest.mark.parametrize("case", range(5))
def test_order2_vs_oracle(case):
    from oracle import oracle as O
    name, pos, f, kw = _sets()[case]
    if f is None:
        f = np.sin(2 * np.pi * pos @ np.arange(1, pos.shape[1] + 1)) + pos[:, 0] ** 2
    M = _mesh(pos, **kw)
    R = O.OracleMeshoid(pos, **kw)
    assert sets_equal_rows(as_np(M.ngb), R.ngb) == 0
    rows = np.arange(len(pos))
    ref, exempt = order2_reference(pos, R.ngb, R.kernel_radius, rows, f, boxsize=kw.get("boxsize"))
    d1 = as_np(M.D(f, order=2))
    d2 = as_np(M.D2(f))
    e = order2_errors(d1, d2, ref)
    _report(f"{name} N={len(pos)}", e, exempt)


def test_hsml_polish_float_float():
    """The float-float root of HsmlIter's equation that the order-2 fit uses:
    within 1e-9 of the oracle's FP64 bisection (the FP32 solve is within
    1e-6)."""
    from meshoid_gb300 import synthetic as S
    from oracle import oracle as O
    for pos in (S.clump_mixture(1 << 16, seed=61), S.plummer(1 << 16, seed=62)):
        M = _mesh(pos, des_ngb=32)
        R = O.OracleMeshoid(pos, des_ngb=32)
        hi, lo = M._hsml_ff()  # query (slot) order; out_rows maps to particle rows
        h = np.empty(len(pos))
        h[as_np(M._out_rows).astype(np.int64)] = as_np(hi) + as_np(lo)
        err = np.abs(h / R.kernel_radius - 1)
        print(f"\npolished h: {summary(err)}")
        assert err.max() <= 1e-9, summary(err)
