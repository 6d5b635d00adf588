"""Batched snapshots (mg_batched_run, one CUDA graph): every snapshot's
smoothing lengths and first derivatives equal the per-snapshot Meshoid path
with the same cell parameters bit for bit, and its column density map agrees
to FP32 accumulation order; graph replay and an
eager launch agree; the first snapshots are also checked against the oracle."""
import numpy as np
import pytest

from gpu_util import as_np, row_rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _snapshots():
    from meshoid_gb300 import synthetic as S
    out = []
    for i, n in enumerate([3000, 9000, 20000, 5000, 40000, 1500]):
        pos = S.plummer(n, seed=40 + i) if i % 2 == 0 else S.clump_mixture(n, seed=40 + i)
        m = np.random.default_rng(i).uniform(0.5, 1.5, n)
        f = np.c_[np.sin(3 * pos[:, 0]), pos[:, 1] * pos[:, 2], S.fourier_fields(pos, 2, seed=i, kmax=4)]
        out.append((pos, m, f))
    return out


@pytest.fixture(scope="module")
def batch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshoid_gb300.batch import SnapshotBatch
    snaps = _snapshots()
    B = SnapshotBatch(snaps, des_ngb=32, map_res=256, graph=True).run()
    return snaps, B


def test_batch_matches_meshoid(batch):
    from meshoid_gb300 import Meshoid
    snaps, B = batch
    for i, (pos, m, f) in enumerate(snaps):
        M = Meshoid(pos, m, des_ngb=32)
        np.testing.assert_array_equal(as_np(B.hsml[i]), as_np(M.kernel_radius))
        np.testing.assert_array_equal(as_np(B.grad[i]), as_np(M.D(f)))
        sd = as_np(M.SurfaceDensity(M.m, res=256))
        # tiles accumulate in FP32 shared-memory atomics: order-dependent at ~1e-7
        assert np.max(np.abs(as_np(B.maps[i]) - sd)) <= 1e-6 * np.abs(sd).max()


def test_replay_and_eager_agree(batch):
    from meshoid_gb300.batch import SnapshotBatch
    snaps, B = batch
    h0 = [as_np(h) for h in B.hsml]
    g0 = [as_np(g) for g in B.grad]
    B.run()  # second replay
    E = SnapshotBatch(snaps[:3], des_ngb=32, map_res=256, graph=False).run()
    for i in range(3):
        np.testing.assert_array_equal(as_np(B.hsml[i]), h0[i])
        np.testing.assert_array_equal(as_np(B.grad[i]), g0[i])
        np.testing.assert_array_equal(as_np(E.hsml[i]), h0[i])
        np.testing.assert_array_equal(as_np(E.grad[i]), g0[i])
    assert int(B.unresolved.sum()) == 0


def test_batch_vs_oracle(batch):
    from oracle import oracle as O
    snaps, B = batch
    for i in (0, 1):
        pos, m, f = snaps[i]
        R = O.OracleMeshoid(pos, m, des_ngb=32)
        h = as_np(B.hsml[i])
        assert np.max(np.abs(h / R.kernel_radius - 1)) <= 1e-6
        assert row_rel_err(as_np(B.grad[i]), R.D(f)).max() <= 1e-5
        sr = R.SurfaceDensity(R.m, res=256)
        assert np.max(np.abs(as_np(B.maps[i]) - sr)) <= 1e-5 * np.max(np.abs(sr))


def test_autotuner_caches_a_valid_choice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshoid_gb300 import synthetic as S
    from meshoid_gb300.batch import tune_cell_parameters
    pos = S.plummer(30000, seed=5)
    c1 = tune_cell_parameters(pos, key=("test", 30000))
    c2 = tune_cell_parameters(S.plummer(30000, seed=6), key=("test", 30000))
    assert c1 == c2 and len(c1) == 3 and c1[1] in (0, 1)


def test_batch_2e21_snapshot_vs_oracle():
    """A batch with a 2^21 Plummer snapshot (the size at the top of the
    64-snapshot benchmark batch) and two small ones, 1024^2 maps (large
    footprints go through the per-tile pairs path): the large snapshot's h,
    D and map against the oracle."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshoid_gb300 import synthetic as S
    from meshoid_gb300.batch import SnapshotBatch
    from oracle import oracle as O
    n = 1 << 21
    pos = S.plummer(n, seed=46)
    m = np.random.default_rng(46).uniform(0.5, 1.5, n)
    f = np.c_[np.sin(3 * pos[:, 0]), pos[:, 1] * pos[:, 2]]
    small = [(S.clump_mixture(30000, seed=47), None, None), (S.plummer(5000, seed=48), None, None)]
    B = SnapshotBatch([(pos, m, f)] + small, des_ngb=32, map_res=1024, graph=True).run()
    assert int(B.unresolved.sum()) == 0
    R = O.OracleMeshoid(pos, m, des_ngb=32)
    h = as_np(B.hsml[0])
    assert np.max(np.abs(h / R.kernel_radius - 1)) <= 1e-6
    e = row_rel_err(as_np(B.grad[0]), R.D(f))
    assert e.max() <= 1e-5, e.max()
    sr = R.SurfaceDensity(R.m, res=1024)
    err = np.max(np.abs(as_np(B.maps[0]) - sr)) / np.max(np.abs(sr))
    print(f"\n2^21 snapshot: h max {np.max(np.abs(h / R.kernel_radius - 1)):.2e}, D max {e.max():.2e}, map {err:.2e}")
    assert err <= 1e-5
