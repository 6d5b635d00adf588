"""Pin the CPU oracle against golden vectors produced by the reference itself.

tests/golden/*.npz were generated by tests/golden/make_golden.py, which runs
the reference meshoid's own source.  These checks run on CPU only.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _sets_equal(a, b):
    return all(set(x) == set(y) for x, y in zip(np.asarray(a), np.asarray(b)))


@pytest.mark.parametrize("name,kw", [
    ("uniform_1024", {}),
    ("periodic_768", {"boxsize": 1.0}),
    ("plummer_1536", {}),
    ("uniform2d_900", {}),
    ("uniform_ngb64_1200", {"des_ngb": 64}),
])
def test_oracle_neighbours_and_hsml(golden, name, kw):
    g = golden(name)
    M = O.OracleMeshoid(g["pos"], g.get("m"), **kw)
    assert _sets_equal(M.ngb, g["ngb"])
    np.testing.assert_allclose(M.ngbdist, g["ngbdist"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(M.kernel_radius, g["hsml"], rtol=1e-12)
    np.testing.assert_allclose(M.density, g["density"], rtol=1e-11)


def test_oracle_uniform_derivatives_and_maps(golden):
    g = golden("uniform_1024")
    M = O.OracleMeshoid(g["pos"], g["m"], des_ngb=32)
    np.testing.assert_allclose(M.D(g["f"]), g["D1"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(M.D(g["pos"]), g["Dpos"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(M.KernelAverage(g["f"]), g["KA"], rtol=1e-12, atol=1e-14)
    c = np.array([0.5, 0.5, 0.5])
    np.testing.assert_allclose(M.SurfaceDensity(M.m, center=c, size=1.0, res=48), g["SD"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(M.SurfaceDensity(M.m, center=c, size=1.0, res=48, conservative=True), g["SDc"],
                               rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(M.center, g["center"])
    np.testing.assert_allclose(M.L, g["L"])


def test_oracle_periodic(golden):
    g = golden("periodic_768")
    M = O.OracleMeshoid(g["pos"], des_ngb=32, boxsize=1.0)
    np.testing.assert_allclose(M.D(g["f"]), g["D1"], rtol=1e-9, atol=1e-9)


def test_oracle_plummer(golden):
    g = golden("plummer_1536")
    M = O.OracleMeshoid(g["pos"], des_ngb=32)
    lr = np.log(M.density)
    np.testing.assert_allclose(M.D(lr), g["D_logrho"], rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(M.D(g["v"]), g["D_v"], rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(M.KernelAverage(lr), g["KA"], rtol=1e-12)
    np.testing.assert_allclose(M.SurfaceDensity(M.m, center=np.zeros(3), size=4.0, res=40), g["SD"], rtol=1e-11)


def test_oracle_2d(golden):
    g = golden("uniform2d_900")
    M = O.OracleMeshoid(g["pos"])
    np.testing.assert_allclose(M.D(g["f"]), g["D1"], rtol=1e-9, atol=1e-9)
    if "D2" in g:
        ok = O.moment_condition(M.pos, M.ngb, M.kernel_radius, M.particle_mask, order=2) < 1e6
        assert ok.mean() > 0.95
        np.testing.assert_allclose(M.D2(g["f"])[ok], g["D2"][ok], rtol=1e-7, atol=1e-7)


def test_oracle_ngb64_order2(golden):
    g = golden("uniform_ngb64_1200")
    M = O.OracleMeshoid(g["pos"], des_ngb=64)
    np.testing.assert_allclose(M.D(g["f"]), g["D1"], rtol=1e-9, atol=1e-9)
    ok = O.moment_condition(M.pos, M.ngb, M.kernel_radius, M.particle_mask, order=2) < 1e6
    assert ok.mean() > 0.95
    np.testing.assert_allclose(M.D2(g["f"])[ok], g["D2"][ok], rtol=1e-7, atol=1e-7)
    np.testing.assert_allclose(M.KernelAverage(g["f"]), g["KA"], rtol=1e-12)


def test_oracle_mask(golden):
    g = golden("mask_1000")
    M = O.OracleMeshoid(g["pos"], des_ngb=32)
    M.particle_mask = g["mask"].astype(np.int64)
    M.TreeUpdate()
    M.reset_dweights()
    assert _sets_equal(M.ngb, g["ngb"])
    np.testing.assert_allclose(M.kernel_radius, g["hsml"], rtol=1e-12)
    np.testing.assert_allclose(M.D(g["f"]), g["D1"], rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("order", [0, 1, 2])
def test_oracle_slice(golden, order):
    g = golden("slice_1024")
    if f"slice{order}" not in g:
        pytest.skip("reference raised for this order")
    M = O.OracleMeshoid(g["pos"], des_ngb=32)
    s = M.Slice(g["f"], center=np.array([0.5, 0.5, 0.5]), size=0.8, order=order, res=12)
    np.testing.assert_allclose(s, g[f"slice{order}"], rtol=1e-8, atol=1e-8)
    np.testing.assert_array_equal(np.asarray(M.particle_mask), g[f"mask{order}"])


def test_oracle_conservative_deposit_keeps_mass():
    """The conservative surface density (src/meshoid/grid_deposition.py:232-295)
    deposits each particle's whole f over its footprint: with every footprint
    inside the map, sum(grid) dx^2 = sum(f)."""
    rng = np.random.default_rng(5)
    p = 0.25 + 0.5 * rng.random((3000, 3))
    m = rng.uniform(0.5, 1.5, 3000)
    M = O.OracleMeshoid(p, m, des_ngb=32)
    assert M.kernel_radius.max() < 0.25
    res = 64
    sd = M.SurfaceDensity(m, center=np.array([0.5, 0.5, 0.5]), size=1.0, res=res, conservative=True)
    assert abs(sd.sum() / (res - 1) ** 2 / m.sum() - 1) < 1e-13


def test_oracle_known_answers():
    """D of a linear field is exact (README.md:190-220 of the reference)."""
    rng = np.random.default_rng(0)
    pos = rng.random((3000, 3))
    M = O.OracleMeshoid(pos, des_ngb=32)
    f = 2.0 * pos[:, 0] - 3.0 * pos[:, 1] + 0.5 * pos[:, 2]
    np.testing.assert_allclose(M.D(f), np.tile([2.0, -3.0, 0.5], (3000, 1)), atol=1e-10)
    np.testing.assert_allclose(M.KernelAverage(np.full(3000, 7.0)), 7.0, rtol=1e-14)


def test_oracle_extras(golden):
    """KernelVariance, Integrate, ProjectedAverage, Projection, InterpToGrid."""
    g = golden("extras_800")
    M = O.OracleMeshoid(g["pos"], g["m"], des_ngb=32)
    np.testing.assert_allclose(M.kernel_radius, g["hsml"], rtol=1e-12)
    np.testing.assert_allclose(M.KernelVariance(g["f"]), g["kvar"], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(M.KernelVariance(g["fv"]), g["kvar_v"], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(M.Integrate(g["f"]), g["integral"], rtol=1e-11)
    np.testing.assert_allclose(M.Integrate(g["fv"]), g["integral_v"], rtol=1e-11)
    c = np.array([0.1, -0.2, 0.05])
    np.testing.assert_allclose(M.ProjectedAverage(g["f"], center=c, size=3.0, res=40), g["pavg"], rtol=1e-10)
    np.testing.assert_allclose(M.Projection(g["f"], center=c, size=3.0, res=40), g["proj"], rtol=1e-10)
    if "interp" in g:
        np.testing.assert_allclose(M.InterpToGrid(g["f"], center=c, size=1.5, res=5, order=1), g["interp"],
                                   rtol=1e-8, atol=1e-8)


def test_oracle_deposit3d(golden):
    """DepositToGrid on a periodic box, GridDensity without a box, the PPZ data
    cube and WeightedGridInterp3D (src/meshoid/grid_deposition.py:339-600)."""
    g = golden("deposit3d_600")
    M = O.OracleMeshoid(g["pos_b"], g["m_b"], des_ngb=32, boxsize=1.0)
    np.testing.assert_allclose(M.kernel_radius, g["hsml_b"], rtol=1e-12)
    mx = np.abs(g["dep_box"]).max()
    np.testing.assert_allclose(M.DepositToGrid(g["m_b"], res=12), g["dep_box"], rtol=0, atol=1e-12 * mx)
    size, res = float(g["size"]), int(g["res"])
    h = np.clip(g["hsml"], size / (res - 1), 1e100)
    np.testing.assert_allclose(O.grid_density(g["m"], g["pos"], h, g["center"], size, res, -1.0), g["dep_open"],
                               rtol=0, atol=1e-12 * np.abs(g["dep_open"]).max())
    np.testing.assert_allclose(O.ppz_cube(g["m"], g["pos"], g["hsml"], g["center_ppz"], [size, 1.6], g["z"], g["h_z"],
                                          [12, 10]), g["ppz"], rtol=0, atol=1e-12 * np.abs(g["ppz"]).max())
    np.testing.assert_allclose(O.weighted_interp3d(g["f"], g["wt"], g["pos"], g["hsml"], g["center"], 3.0, 10),
                               g["winterp"], rtol=1e-12)
    np.testing.assert_allclose(O.ppz_cube_multigrid(g["m"], g["pos"], g["hsml"], g["center_ppz"], [size, 1.6],
                                                    g["z"], g["h_z"], [16, 10]), g["ppz_mg"], rtol=0,
                               atol=1e-12 * np.abs(g["ppz_mg"]).max())


def test_oracle_surface_multigrid(golden):
    """GridSurfaceDensityMultigrid and its UpsampleGrid
    (src/meshoid/grid_deposition.py:89-120)."""
    g = golden("surface_multigrid_1500")
    got = O.surface_density_multigrid(g["m"], g["pos"], g["hsml"], g["center"], float(g["size"]), int(g["res"]))
    np.testing.assert_allclose(got, g["mg"], rtol=0, atol=1e-12 * np.abs(g["mg"]).max())
    np.testing.assert_allclose(O.upsample_grid(g["g8"]), g["up8"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(O.upsample_grid(g["g32"]), g["up32"], rtol=0, atol=1e-14)


def test_oracle_notebook(golden):
    """The reference's test notebook (test/test_gradients.ipynb) at N = 2000:
    periodic box, des_ngb = 100, D, D2 of the products x_i x_j, Reconstruct
    orders 0-2, Slice and InterpToGrid at order 2, in the notebook's order."""
    g = golden("notebook_2000")
    x = g["x"]
    M = O.OracleMeshoid(x, des_ngb=100, boxsize=1)
    assert _sets_equal(M.ngb, g["ngb"])
    np.testing.assert_allclose(M.kernel_radius, g["hsml"], rtol=1e-12)

    def close(got, ref):
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * max(1.0, np.abs(ref).max()))

    close(M.D(x), g["Dx"])
    for i in range(3):
        for j in range(3):
            d2 = M.D2(x[:, i] * x[:, j])
            if i <= j:
                close(d2, g[f"D2_{i}{j}"])
    for order in (0, 1, 2):
        close(M.Reconstruct(x, g["x2"], order=order), g[f"rec{order}"])
    for i, j in ((0, 0), (0, 1), (1, 2)):
        close(M.Reconstruct(x[:, i] * x[:, j], g["x2"], order=2), g[f"rec2_{i}{j}"])
    c = np.array([0.5, 0.5, 0.5])
    close(M.Slice(np.sin(x[:, 0] * np.pi * 2), center=c, size=1.0, order=2, res=24), g["slice2"])
    X, Y, Z, f = M.InterpToGrid(np.sin(x[:, 1] * np.pi * 2), center=c, size=1.0, order=2, res=6, return_grid=True)
    close(f, g["gf"])
    for a, key in ((X, "gX"), (Y, "gY"), (Z, "gZ")):
        close(a, g[key])


def test_oracle_lowdim(golden):
    """1-D points (default des_ngb 4; des_ngb 8 on a periodic line) and a
    periodic 2-D box: neighbours, h, D, D2, KernelAverage."""
    g = golden("lowdim")

    def close(got, ref, tol=1e-12):
        np.testing.assert_allclose(got, ref, rtol=0, atol=tol * np.abs(ref).max())

    M = O.OracleMeshoid(g["x1"])
    assert _sets_equal(M.ngb, g["ngb1"])
    np.testing.assert_allclose(M.kernel_radius, g["hsml1"], rtol=1e-12)
    close(M.D(g["f1"]), g["D1_1"])
    close(M.KernelAverage(g["f1"]), g["KA1"])
    M = O.OracleMeshoid(g["xp"], des_ngb=8, boxsize=1.0)
    assert _sets_equal(M.ngb, g["ngbp"])
    np.testing.assert_allclose(M.kernel_radius, g["hsmlp"], rtol=1e-12)
    close(M.D(g["fp"]), g["D1_p"])
    close(M.D2(g["fp"]), g["D2_p"], 1e-10)
    M = O.OracleMeshoid(g["x2"], boxsize=1.0)
    assert _sets_equal(M.ngb, g["ngb2"])
    np.testing.assert_allclose(M.kernel_radius, g["hsml2"], rtol=1e-12)
    close(M.D(g["f2"]), g["D1_2"])
    close(M.D2(g["f2"]), g["D2_2"], 1e-10)
    close(M.KernelAverage(g["f2"]), g["KA2"])


def test_oracle_radtransfer(golden):
    """radtransfer_singlethread (src/meshoid/radiation/radtransfer.py:87-200)
    with and without a background; radtransfer on one thread equals it."""
    g = golden("radtransfer_500")
    I, t = O.radtransfer(g["j"], g["m"], g["kappa"], g["pos"], g["hsml"], 24, 4.0, g["center"], 0)
    np.testing.assert_allclose(I, g["I0"], rtol=0, atol=1e-13 * np.abs(g["I0"]).max())
    np.testing.assert_allclose(t, g["tau0"], rtol=1e-13)
    np.testing.assert_array_equal(g["Ipar"], g["I0"])
    I, t = O.radtransfer(g["j"], g["m"], g["kappa"], g["pos"], g["hsml"], 24, 4.0, g["center"], g["i0"])
    np.testing.assert_allclose(I, g["I1"], rtol=1e-13)
    np.testing.assert_allclose(t, g["tau1"], rtol=1e-13)


def test_oracle_weights_and_kde(golden):
    """get_kernel_weights, ComputeDWeights (order 1) and KDE
    (src/meshoid/Meshoid.py:110-177, :722-750) against the reference."""
    g = golden("weights_kde_1024")
    M = O.OracleMeshoid(g["pos"], des_ngb=32)
    np.testing.assert_allclose(M.kernel_radius, g["hsml"], rtol=1e-12)
    np.testing.assert_allclose(M.get_kernel_weights()[:256], g["kweights"], rtol=1e-10, atol=1e-14)
    M.ComputeDWeights(order=1)
    np.testing.assert_allclose(M.dweights[:256], g["dweights"], rtol=1e-8, atol=1e-8)
    M1 = O.OracleMeshoid(g["x1"], des_ngb=12)
    np.testing.assert_allclose(M1.kernel_radius, g["hsml1"], rtol=1e-12)
    np.testing.assert_allclose(M1.KDE(g["grid"]), g["kde"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(M1.KDE(g["grid"], bandwidth=np.full(len(g["x1"]), 0.05)), g["kde_bw"], rtol=1e-10,
                               atol=1e-12)


def test_oracle_curl_div(golden):
    """Curl / Div (src/meshoid/Meshoid.py:297-331) with the full mask, with a
    mask whose neighbour indices all lie below Nmask (the reference's indexing
    of v[particle_mask] then works), and after a Slice rewrote the mask (the
    reference raises IndexError)."""
    g = golden("curl_div_800")
    M = O.OracleMeshoid(g["pos"], des_ngb=32)
    np.testing.assert_allclose(M.Curl(g["v"]), g["curl"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(M.Div(g["v"]), g["div"], rtol=1e-9, atol=1e-9)
    Mm = O.OracleMeshoid(g["pos"], des_ngb=32, particle_mask=np.arange(400))
    assert _sets_equal(Mm.ngb, g["ngb_mask"])
    np.testing.assert_allclose(Mm.Curl(g["v"]), g["curl_mask"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(Mm.Div(g["v"]), g["div_mask"], rtol=1e-9, atol=1e-9)
    assert int(g["curl_after_slice_indexerror"]) == 1
    Ms = O.OracleMeshoid(g["pos"], des_ngb=32)
    Ms.Slice(g["pos"][:, 0], center=np.array([0.5, 0.5, 0.5]), size=1.0, res=8, order=1)
    with pytest.raises(IndexError):
        Ms.Curl(g["v"])
