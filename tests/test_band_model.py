"""The FP64 re-decision band of the neighbour search's warp path, modelled on
the CPU: candidates whose FP32 squared distance (from the hi/lo positions)
lies within the band around the k-th one, T, are re-ranked with exact FP64
distances (meshoid_gb300/csrc/mg_knn.cu, resolve_band_fp64 / band_abs).

A band of 1e-5 of T alone misses the positions' hi/lo representation error,
~2^-46 |x| per axis of a separation, which decides for pairs closer than
~1e-9 of their coordinates: on a tight clump far from the frame centre some
rows' FP64 k nearest then have a member whose FP32 distance lies above the
band (or a non-member below it), and no re-ranking can repair the row.  The
band widened by 2 sqrt(T) dd + dd^2, dd = 3e-14 |x|, leaves none, and stays
within the 32 entries the re-ranking holds (tests/gpu_util.far_clump: 8,000
particles with sigma 5e-8 at (900, 900, 900) in a [0, 1000]^3 box of
20,000).  The GPU test of the same
fixture is tests/test_gpu_parity.py::test_far_tight_clump.

Reference: the neighbour sets of cKDTree.query (src/meshoid/Meshoid.py:157),
FP64 distances.
"""
import numpy as np
import pytest

from gpu_util import far_clump, hilo_d2

scipy_spatial = pytest.importorskip("scipy.spatial")


def _count(pos, k=32, extra=16):
    tree = scipy_spatial.cKDTree(pos)
    q = np.arange(20000, len(pos))  # the clump
    _, nb = tree.query(pos[q], k + extra)
    bad_rel = bad_wide = over = 0
    for qi, row in zip(q, nb):
        d2f, xm = hilo_d2(pos, qi, row)
        T = np.sort(d2f)[k - 1]
        dd = 3e-14 * xm
        for wabs, tag in ((0.0, "rel"), (2.0 * np.sqrt(T) * dd + dd * dd, "wide")):
            lo_b, hi_b = T * (1 - 1e-5) - wabs, T * (1 + 1e-5) + wabs
            miss = bool((d2f[:k] > hi_b).any() or (d2f[k:] < lo_b).any())
            if tag == "rel":
                bad_rel += miss
            else:
                bad_wide += miss
                over += int(((d2f >= lo_b) & (d2f <= hi_b)).sum() > 32)
    return bad_rel, bad_wide, over


def test_far_clump_needs_the_widened_band():
    bad_rel, bad_wide, over = _count(far_clump())
    print(f"\nrows misranked beyond the band: relative only {bad_rel}, widened {bad_wide}; bands over 32: {over}")
    assert bad_rel >= 1  # the fixture exercises the hole
    assert bad_wide == 0 and over == 0
