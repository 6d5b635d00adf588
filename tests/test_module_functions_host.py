"""The package's module-level surface, checked on CPU: every public name that
the reference's ``meshoid/__init__.py`` star-imports (src/meshoid/Meshoid.py,
grid_deposition.py, kernel_density.py, derivatives.py) exists, and the
element-wise helpers follow the reference's formulas (evaluated here on CPU
tensors by pointing their device choice at the CPU)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

# public functions of src/meshoid/{Meshoid,grid_deposition,kernel_density,derivatives}.py
REFERENCE_EXPORTS = [
    "Meshoid",
    "grid_index_to_coordinate", "grid_dx_from_coordinate", "GridSurfaceDensityMultigrid", "UpsampleGrid",
    "GridSurfaceDensity", "UpsampleGrid_PPV", "Grid_PPZ_DataCube_Multigrid", "Grid_PPZ_DataCube",
    "GridAverage", "WeightedGridInterp3D", "GridDensity",
    "HsmlIter", "kernel2d", "kernel3d", "Kernel",
    "nearest_image", "nearest_image_v", "gradient_weights", "get_num_derivs",
]


def test_package_exports_reference_names():
    import meshoid_gb300
    missing = [n for n in REFERENCE_EXPORTS if not callable(getattr(meshoid_gb300, n, None))]
    assert not missing, missing


def test_kernels_follow_the_spline(monkeypatch):
    from meshoid_gb300 import kernel_density as KD
    monkeypatch.setattr(KD, "_device", lambda: torch.device("cpu"))
    q = np.linspace(0, 1.4, 141)
    w = np.where(q <= 0.5, 1 - 6 * q ** 2 + 6 * q ** 3, np.where(q <= 1.0, 2 * (1 - q) ** 3, 0.0))
    np.testing.assert_allclose(KD.Kernel(q).numpy(), w, rtol=1e-15, atol=1e-16)
    np.testing.assert_allclose(KD.kernel2d(q).numpy(), w * 1.8189136353359467, rtol=1e-15, atol=1e-16)
    np.testing.assert_allclose(KD.kernel3d(q).numpy(), w * 2.546479089470325, rtol=1e-15, atol=1e-16)
    assert KD.Kernel(torch.tensor(q, dtype=torch.float32)).dtype == torch.float32
    assert float(KD.Kernel(0.25)) == pytest.approx(1 - 6 * 0.0625 + 6 * 0.015625)


def test_nearest_image_and_grid_coordinates(monkeypatch):
    from meshoid_gb300 import derivatives as DV
    from meshoid_gb300 import grid_deposition as GD
    monkeypatch.setattr(DV, "_device", lambda *xs: torch.device("cpu"))
    monkeypatch.setattr(GD, "_device_of", lambda *xs: torch.device("cpu"))
    dx = np.array([-0.9, -0.6, -0.5, -0.2, 0.0, 0.3, 0.5, 0.51, 0.99])
    ref = np.where(np.abs(dx) > 0.5, -np.copysign(1.0 - np.abs(dx), dx), dx)
    np.testing.assert_array_equal(DV.nearest_image(dx, 1.0).numpy(), ref)
    assert DV.nearest_image_v is DV.nearest_image
    i = np.arange(8)
    x = 0.9 - 0.5 * 2.0 + 2.0 / 8 * (0.5 + i)
    np.testing.assert_allclose(GD.grid_index_to_coordinate(i, 2.0, 0.9, 8).numpy(), x, rtol=1e-15)
    np.testing.assert_allclose(GD.grid_index_to_coordinate(i, 2.0, 0.9, 8, box_size=1.0).numpy(), x % 1.0,
                               rtol=1e-15, atol=1e-15)
    xg = x % 1.0
    d = xg - 0.95
    ref = np.where(np.abs(d) > 0.5, -np.copysign(1.0 - np.abs(d), d), d)
    np.testing.assert_allclose(GD.grid_dx_from_coordinate(0.95, i, 2.0, 0.9, 8, box_size=1.0).numpy(), ref,
                               rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(GD.grid_dx_from_coordinate(0.95, i, 2.0, 0.9, 8).numpy(), x - 0.95, rtol=1e-14)


def test_num_derivs():
    from meshoid_gb300 import get_num_derivs
    assert [get_num_derivs(d, 1) for d in (1, 2, 3)] == [1, 2, 3]
    assert [get_num_derivs(d, 2) for d in (1, 2, 3)] == [2, 5, 9]
