"""Host-side logic of the grid module, checked on CPU: the spline matrix that
carries GridSurfaceDensityMultigrid's levels up (src/meshoid/grid_deposition.py:
116-120) and the level schedule (:89-113), with the per-level deposit taken
from the oracle so that no GPU is needed."""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")


def test_upsample_matrix_matches_reference_upsample(golden):
    from meshoid_gb300 import grid_deposition as GD
    g = golden("surface_multigrid_1500")
    for src, ref in (("g8", "up8"), ("g32", "up32")):
        u = GD._upsample_matrix(g[src].shape[0])
        np.testing.assert_allclose(u @ g[src] @ u.T, g[ref], rtol=0, atol=1e-13 * np.abs(g[ref]).max())
    u = GD._upsample_matrix(4)
    np.testing.assert_allclose(u.sum(1), 1.0, rtol=0, atol=1e-14)  # constants are reproduced
    with pytest.raises(ValueError):
        GD._upsample_matrix(2)


def test_multigrid_schedule_on_host(golden, monkeypatch):
    from meshoid_gb300 import grid_deposition as GD

    def deposit(f, x, h, center, size, res=100, **kw):
        return torch.from_numpy(O.surface_density(f.numpy(), x.numpy(), h.numpy(), center, size, res))

    monkeypatch.setattr(GD, "_device_of", lambda *xs: torch.device("cpu"))
    monkeypatch.setattr(GD, "GridSurfaceDensity", deposit)
    g = golden("surface_multigrid_1500")
    got = GD.GridSurfaceDensityMultigrid(g["m"], g["pos"], g["hsml"], g["center"], float(g["size"]),
                                         res=int(g["res"])).numpy()
    np.testing.assert_allclose(got, g["mg"], rtol=0, atol=1e-12 * np.abs(g["mg"]).max())


def test_multigrid_needs_power_of_two():
    from meshoid_gb300 import grid_deposition as GD
    x = np.zeros((4, 3))
    with pytest.raises(ValueError):
        GD.GridSurfaceDensityMultigrid(np.ones(4), x, np.ones(4), [0, 0], 1.0, res=48)
    with pytest.raises(ValueError):
        GD.Grid_PPZ_DataCube_Multigrid(np.ones(4), x, np.ones(4), [0, 0, 0], [1.0, 1.0], np.zeros(4), np.ones(4),
                                       [24, 8])
