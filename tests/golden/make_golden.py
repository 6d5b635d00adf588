"""Generate golden input/output vectors by running the reference meshoid itself.

Run where the reference source is available, giving the path of its ``src``
directory as the first argument or in MESHOID_REF_SRC:

    python tests/golden/make_golden.py /path/to/meshoid/src
    MESHOID_REF_SRC=/path/to/meshoid/src GOLDEN_ONLY=case_curl_div python tests/golden/make_golden.py

The reference needs numba, which is not installed; ``_numba_stub`` stands in
for it (decorators become no-ops), so the reference's own Python source runs
unmodified as plain Python.  Sizes are kept small because that is slow
(~1 ms per particle).  Each case stores its inputs next to the reference
outputs, so the tests never need the reference at run time.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MESHOID_REF_SRC", "")
if not REF_SRC or not os.path.isdir(os.path.join(REF_SRC, "meshoid")):
    sys.exit("usage: make_golden.py <meshoid src directory> (or set MESHOID_REF_SRC)")
sys.path.insert(0, os.path.join(HERE, "_numba_stub"))
sys.path.insert(0, REF_SRC)
sys.dont_write_bytecode = True

from meshoid import Meshoid  # noqa: E402  (the reference)

sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from meshoid_gb300 import synthetic  # noqa: E402


def try_call(fn, *a, **k):
    """The reference raises LinAlgError when a moment matrix is singular
    (src/meshoid/derivatives.py:132); such outputs are recorded as absent."""
    try:
        return fn(*a, **k)
    except np.linalg.LinAlgError:
        return None


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    out = {}
    for k, v in arrays.items():
        if v is None:
            print(f"  {name}: {k} raised LinAlgError in the reference; not stored")
            continue
        v = np.asarray(v)
        if v.dtype == np.int64:
            v = v.astype(np.int32)
        out[k] = v
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


def case_uniform():
    """Small uniform cube, des_ngb=32: hsml, density, D order 1/2, D2, KernelAverage, maps."""
    pos = synthetic.uniform(1024, seed=7)
    m = np.full(len(pos), 1.0 / len(pos))
    f = synthetic.config1_field(pos)
    M = Meshoid(pos, m, des_ngb=32)
    d1 = M.D(f)
    dv = M.D(pos)  # vector field: D of the coordinates (linear, exact)
    d1o2 = try_call(M.D, f, order=2)
    d2 = try_call(M.D2, f)
    ka = M.KernelAverage(f)
    sd = M.SurfaceDensity(M.m, center=np.array([0.5, 0.5, 0.5]), size=1.0, res=48)
    sdc = M.SurfaceDensity(M.m, center=np.array([0.5, 0.5, 0.5]), size=1.0, res=48, conservative=True)
    save("uniform_1024", pos=pos, m=m, f=f, ngb=M.ngb, ngbdist=M.ngbdist, hsml=M.kernel_radius,
         density=M.density, vol=M.vol, D1=d1, Dpos=dv, D1_order2=d1o2, D2=d2, KA=ka, SD=sd, SDc=sdc,
         center=M.center, L=M.L)


def case_periodic():
    """Periodic unit box: neighbours and derivatives use the nearest image."""
    pos = synthetic.uniform(768, seed=11)
    f = np.sin(2 * np.pi * pos[:, 0]) + np.cos(2 * np.pi * pos[:, 2])
    M = Meshoid(pos, des_ngb=32, boxsize=1.0)
    save("periodic_768", pos=pos, f=f, ngb=M.ngb, ngbdist=M.ngbdist, hsml=M.kernel_radius,
         density=M.density, D1=M.D(f), D2=try_call(M.D2, f))


def case_plummer():
    """Plummer sphere (large density range), des_ngb=32, unit masses."""
    pos = synthetic.plummer(1536, seed=3)
    M = Meshoid(pos, des_ngb=32)
    lr = np.log(M.density)
    v = synthetic.rotation_velocity(pos, seed=4)
    save("plummer_1536", pos=pos, v=v, ngb=M.ngb, ngbdist=M.ngbdist, hsml=M.kernel_radius,
         density=M.density, D_logrho=M.D(lr), D_v=M.D(v), KA=M.KernelAverage(lr),
         SD=M.SurfaceDensity(M.m, center=np.zeros(3), size=4.0, res=40), center=M.center, L=M.L)


def case_2d():
    """2-D points, default des_ngb (20)."""
    rng = np.random.default_rng(5)
    pos = rng.random((900, 2))
    f = np.sin(3 * pos[:, 0]) * pos[:, 1]
    M = Meshoid(pos)
    save("uniform2d_900", pos=pos, f=f, ngb=M.ngb, ngbdist=M.ngbdist, hsml=M.kernel_radius,
         density=M.density, D1=M.D(f), D2=try_call(M.D2, f))


def case_ngb64():
    """des_ngb=64 (more than one warp of neighbours)."""
    pos = synthetic.uniform(1200, seed=13)
    f = pos[:, 0] ** 2 - pos[:, 1] * pos[:, 2]
    M = Meshoid(pos, des_ngb=64)
    save("uniform_ngb64_1200", pos=pos, f=f, ngb=M.ngb, ngbdist=M.ngbdist, hsml=M.kernel_radius,
         density=M.density, D1=M.D(f), D2=try_call(M.D2, f), KA=M.KernelAverage(f))


def case_slice():
    """Slice (Reconstruct on a plane grid) order 0/1/2; it rewrites particle_mask."""
    pos = synthetic.uniform(1024, seed=21)
    f = np.sin(2 * np.pi * pos[:, 0])
    out = {}
    for order in (0, 1, 2):
        M = Meshoid(pos, des_ngb=32)
        out[f"slice{order}"] = try_call(M.Slice, f, center=np.array([0.5, 0.5, 0.5]), size=0.8, order=order,
                                        res=12)
        out[f"mask{order}"] = M.particle_mask
    save("slice_1024", pos=pos, f=f, **out)


def case_mask():
    """Query subset: neighbours come from all particles.  The constructor's own
    particle_mask path indexes the already-masked masses a second time
    (src/meshoid/Meshoid.py:92,169) and fails for general masks, so the subset
    is set the way Reconstruct does it (:422-425): assign, then TreeUpdate."""
    pos = synthetic.uniform(1000, seed=17)
    f = pos[:, 0] * pos[:, 1] + pos[:, 2]
    mask = np.sort(np.random.default_rng(1).choice(1000, 300, replace=False))
    M = Meshoid(pos, des_ngb=32)
    M.particle_mask = mask
    M.TreeUpdate()
    M.reset_dweights()
    save("mask_1000", pos=pos, f=f, mask=mask, ngb=M.ngb, ngbdist=M.ngbdist, hsml=M.kernel_radius,
         D1=M.D(f))


def case_extras():
    """KernelVariance, Integrate, ProjectedAverage, Projection and InterpToGrid
    on a small Plummer sphere (scalar and 2-component fields).

    GridAverage (src/meshoid/grid_deposition.py:395-436) evaluates kernel2d on
    every pixel of a particle's bounding square, also where q > 1, and kernel2d
    (src/meshoid/kernel_density.py:59-66) assigns nothing for q > 1: compiled,
    the reference reads an unassigned local there; run as Python it raises.
    The kernel's support is q <= 1, so here kernel2d is extended by 0 beyond
    it for this case."""
    import meshoid.grid_deposition as gd
    k2 = gd.kernel2d
    gd.kernel2d = lambda q: k2(q) if q <= 1.0 else 0.0
    pos = synthetic.plummer(800, seed=23)
    m = np.random.default_rng(3).uniform(0.5, 1.5, len(pos))
    f = np.log1p(np.sum(pos ** 2, 1)) + 0.3 * pos[:, 0]
    fv = np.c_[np.sin(pos[:, 0]), pos[:, 1] * pos[:, 2]]
    M = Meshoid(pos, m, des_ngb=32)
    c = np.array([0.1, -0.2, 0.05])
    save("extras_800", pos=pos, m=m, f=f, fv=fv, hsml=M.kernel_radius, kvar=M.KernelVariance(f),
         kvar_v=M.KernelVariance(fv), integral=M.Integrate(f), integral_v=M.Integrate(fv),
         pavg=M.ProjectedAverage(f, center=c, size=3.0, res=40), proj=M.Projection(f, center=c, size=3.0, res=40),
         interp=try_call(M.InterpToGrid, f, center=c, size=1.5, res=5, order=1))


def case_deposit3d():
    """3-D deposition (src/meshoid/grid_deposition.py): DepositToGrid on a
    periodic box (Meshoid.py:557-593 -> GridDensity :534-600), GridDensity
    called directly without a box (box_size=-1; DepositToGrid itself only runs
    with a box: GridDensity compares box_size < 0, which fails for None), the
    PPZ data cube (Grid_PPZ_DataCube :339-392) and WeightedGridInterp3D
    (:439-531).  All evaluate kernel3d (src/meshoid/kernel_density.py:71-78) on
    every node of a particle's bounding cube, also where q > 1, where it
    assigns nothing; as for case_extras it is extended by 0 beyond q = 1."""
    import meshoid.grid_deposition as gd
    k3 = gd.kernel3d
    gd.kernel3d = lambda q: k3(q) if q <= 1.0 else 0.0
    rng = np.random.default_rng(41)
    # periodic box: DepositToGrid as the class calls it
    pos_b = rng.random((600, 3))
    m_b = rng.uniform(0.5, 1.5, len(pos_b))
    Mb = Meshoid(pos_b, m_b, des_ngb=32, boxsize=1.0)
    dep_box = Mb.DepositToGrid(m_b, res=12)
    # open boundaries: GridDensity on a Plummer sphere, h clipped as DepositToGrid does
    pos = synthetic.plummer(600, seed=43)
    m = rng.uniform(0.5, 1.5, len(pos))
    M = Meshoid(pos, m, des_ngb=32)
    c = np.array([0.05, -0.1, 0.02])
    size, res = 2.5, 14
    h_open = np.clip(M.kernel_radius, size / (res - 1), 1e100)
    dep_open = gd.GridDensity(m, pos, h_open, c, size, res=res, box_size=-1.0)
    # PPZ cube: velocity-like third coordinate
    z = 0.3 * rng.normal(size=len(pos))
    h_z = rng.uniform(0.05, 0.2, len(pos))
    cz = np.array([c[0], c[1], 0.02])
    ppz = gd.Grid_PPZ_DataCube(m, pos, M.kernel_radius, cz, np.array([size, 1.6]), z, h_z,
                               np.array([12, 10], dtype=np.int32), box_size=-1)
    # multigrid PPZ cube: particles deposited at the level their h / 8 falls in
    # (its progress print goes to stdout)
    ppz_mg = gd.Grid_PPZ_DataCube_Multigrid(m, pos, M.kernel_radius, cz, np.array([size, 1.6]), z, h_z,
                                            np.array([16, 10], dtype=np.int32), box_size=-1)
    # weighted interpolation to cell centres (empty cells take the nearest particle)
    f = np.log1p(np.sum(pos ** 2, 1)) + 0.2 * pos[:, 2]
    wt = rng.uniform(0.2, 1.0, len(pos))
    winterp = gd.WeightedGridInterp3D(f, wt, pos, M.kernel_radius, c, 3.0, res=10, box_size=-1)
    save("deposit3d_600", pos_b=pos_b, m_b=m_b, hsml_b=Mb.kernel_radius, dep_box=dep_box,
         pos=pos, m=m, hsml=M.kernel_radius, center=c, size=size, res=res, dep_open=dep_open,
         z=z, h_z=h_z, center_ppz=cz, ppz=ppz, ppz_mg=ppz_mg, f=f, wt=wt, winterp=winterp)


def case_radtransfer():
    """Emission/absorption ray tracing (src/meshoid/radiation/radtransfer.py:
    87-200, radtransfer_singlethread; radtransfer :11-84 equals it on one
    thread).  The module imports astropy (absent) for functions not used here,
    and its package __init__ imports other modules: both are stood in for
    (test scaffolding) and radtransfer.py itself is loaded from its file."""
    import importlib.util
    import types
    units = types.ModuleType("astropy.units")
    units.quantity = types.SimpleNamespace(Quantity=object)
    astropy = types.ModuleType("astropy")
    astropy.units = units
    astropy.constants = types.ModuleType("astropy.constants")
    sys.modules.update({"astropy": astropy, "astropy.units": units, "astropy.constants": astropy.constants})
    rad = types.ModuleType("meshoid.radiation")
    rad.__path__ = [os.path.join(REF_SRC, "meshoid", "radiation")]
    sys.modules["meshoid.radiation"] = rad
    spec = importlib.util.spec_from_file_location("meshoid.radiation.radtransfer",
                                                  os.path.join(REF_SRC, "meshoid", "radiation", "radtransfer.py"))
    rt = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(rt)
    rng = np.random.default_rng(61)
    pos = synthetic.plummer(500, seed=62)
    m = rng.uniform(0.5, 1.5, len(pos))
    M = Meshoid(pos, m, des_ngb=32)
    h = M.kernel_radius
    kappa = rng.uniform(0.02, 0.3, (len(pos), 3))
    j = rng.uniform(0.1, 2.0, (len(pos), 3))
    c = np.array([0.1, -0.05, 0.02])
    I0, tau0 = rt.radtransfer_singlethread(j, m, kappa, pos.copy(), h, 24, 4.0, c, 0)
    i0 = np.array([0.5, 1.0, 2.0])
    I1, tau1 = rt.radtransfer_singlethread(j, m, kappa, pos.copy(), h, 24, 4.0, c, i0)
    Ipar = rt.radtransfer(j, m, kappa, pos.copy(), h, 24, 4.0, c, 0)
    save("radtransfer_500", pos=pos, m=m, hsml=h, kappa=kappa, j=j, center=c, I0=I0, tau0=tau0, i0=i0, I1=I1,
         tau1=tau1, Ipar=Ipar)


def case_surface_multigrid():
    """GridSurfaceDensityMultigrid (src/meshoid/grid_deposition.py:89-120): a
    Plummer sphere whose h / 8 spans all levels of a 64^2 map, plus its
    bicubic UpsampleGrid (:116-120) on a random 8^2 and 32^2 grid."""
    import meshoid.grid_deposition as gd
    pos = synthetic.plummer(1500, seed=57)
    rng = np.random.default_rng(58)
    m = rng.uniform(0.5, 1.5, len(pos))
    M = Meshoid(pos, m, des_ngb=32)
    c = np.array([0.03, -0.02, 0.0])
    size, res = 3.0, 64
    mg = gd.GridSurfaceDensityMultigrid(m, pos, M.kernel_radius, c, size, res=res)
    g8 = rng.normal(size=(8, 8))
    g32 = rng.normal(size=(32, 32))
    save("surface_multigrid_1500", pos=pos, m=m, hsml=M.kernel_radius, center=c, size=size, res=res, mg=mg,
         g8=g8, up8=gd.UpsampleGrid(g8), g32=g32, up32=gd.UpsampleGrid(g32))


def case_notebook():
    """The reference's own test notebook (test/test_gradients.ipynb) at a
    small size: a periodic unit box with des_ngb = 100; D of the coordinates,
    D2 of every product x_i x_j, Reconstruct of the coordinates at random
    targets (orders 0, 1, 2) and of the products (order 2), a Slice of
    sin(2 pi x) at order 2 and InterpToGrid of sin(2 pi y) at order 2 with
    return_grid -- called in that sequence on one object, as the notebook
    does (Reconstruct rewrites particle_mask and the neighbour lists)."""
    from itertools import product
    rng = np.random.default_rng(42)
    x = rng.random((2000, 3))
    M = Meshoid(x, des_ngb=100, boxsize=1)
    out = dict(x=x, ngb=M.ngb, hsml=M.kernel_radius, Dx=M.D(x))
    for i, j in product(range(3), range(3)):
        d2 = try_call(M.D2, x[:, i] * x[:, j])
        if i <= j:  # x_i x_j and x_j x_i are the same field
            out[f"D2_{i}{j}"] = d2
    x2 = rng.random((200, 3))
    out["x2"] = x2
    for order in (0, 1, 2):
        out[f"rec{order}"] = try_call(M.Reconstruct, x, x2, order=order)
    for i, j in ((0, 0), (0, 1), (1, 2)):
        out[f"rec2_{i}{j}"] = try_call(M.Reconstruct, x[:, i] * x[:, j], x2, order=2)
    out["slice2"] = try_call(M.Slice, np.sin(x[:, 0] * np.pi * 2), center=np.array([0.5, 0.5, 0.5]), size=1.0,
                             order=2, res=24)
    grid = try_call(M.InterpToGrid, np.sin(x[:, 1] * np.pi * 2), center=np.array([0.5, 0.5, 0.5]), size=1.0,
                    order=2, res=6, return_grid=True)
    if grid is not None:
        out.update(gX=grid[0], gY=grid[1], gZ=grid[2], gf=grid[3])
    save("notebook_2000", **out)


def case_lowdim():
    """1-D points (default des_ngb 4, and des_ngb 8 on a periodic line) and a
    periodic 2-D box (default des_ngb 20): neighbours, h, D and D2 (1-D
    order 2 fits 2 derivatives, 2-D 5), KernelAverage."""
    rng = np.random.default_rng(77)
    x1 = rng.random((400, 1))
    f1 = np.sin(5 * x1[:, 0]) + x1[:, 0] ** 2
    M1 = Meshoid(x1)
    xp = rng.random((300, 1))
    fp = np.sin(2 * np.pi * xp[:, 0])
    Mp = Meshoid(xp, des_ngb=8, boxsize=1.0)
    x2 = rng.random((600, 2))
    f2 = np.sin(2 * np.pi * x2[:, 0]) * np.cos(2 * np.pi * x2[:, 1])
    M2 = Meshoid(x2, boxsize=1.0)
    save("lowdim", x1=x1, f1=f1, ngb1=M1.ngb, ngbdist1=M1.ngbdist, hsml1=M1.kernel_radius, D1_1=M1.D(f1),
         D2_1=try_call(M1.D2, f1), KA1=M1.KernelAverage(f1),
         xp=xp, fp=fp, ngbp=Mp.ngb, hsmlp=Mp.kernel_radius, D1_p=Mp.D(fp), D2_p=try_call(Mp.D2, fp),
         x2=x2, f2=f2, ngb2=M2.ngb, hsml2=M2.kernel_radius, D1_2=M2.D(f2), D2_2=try_call(M2.D2, f2),
         KA2=M2.KernelAverage(f2))


def case_weights_kde():
    """get_kernel_weights (src/meshoid/Meshoid.py:172-177), ComputeDWeights
    order 1 and 2 (:110-140 -> derivatives.py:118-138) on a small 3-D set,
    and KDE (:722-750) on a 1-D set with its default bandwidth (the smoothing
    lengths) and with a given one."""
    pos = synthetic.uniform(1024, seed=7)
    M = Meshoid(pos, des_ngb=32)
    kw = M.get_kernel_weights()
    M.ComputeDWeights(order=1)
    dw1 = M.dweights
    try_call(M.ComputeDWeights, order=2)
    ok2 = M.d2weights is not None
    rng = np.random.default_rng(92)
    x1 = np.sort(rng.random(300))[:, None]
    M1 = Meshoid(x1, des_ngb=12)
    grid = np.linspace(-0.2, 1.2, 200)
    kde = M1.KDE(grid)
    bw = np.full(len(x1), 0.05)
    kde_bw = M1.KDE(grid, bandwidth=bw)
    # the first 256 rows of the (N, k) and (N, 3, k) weights keep the file small
    save("weights_kde_1024", pos=pos, ngb=M.ngb, hsml=M.kernel_radius, kweights=kw[:256], dweights=dw1[:256],
         d2weights=M.d2weights[:256] if ok2 else None, dweights3=M.dweights_3rdorder[:256] if ok2 else None,
         x1=x1, hsml1=M1.kernel_radius, grid=grid, kde=kde, kde_bw=kde_bw)


def case_curl_div():
    """Curl and Div (src/meshoid/Meshoid.py:297-331), which index the field by
    particle_mask before taking D.  Two well separated clusters of 400 points:
    with the full mask; with the mask = the first cluster's indices (every
    neighbour index is then below Nmask, so the reference's indexing of the
    masked field with global neighbour indices works); and after a Slice has
    rewritten the mask, where the reference raises IndexError (recorded)."""
    rng = np.random.default_rng(2024)
    pos = np.r_[rng.random((400, 3)), 10.0 + rng.random((400, 3))]
    x, y, z = pos.T
    v = np.c_[-y + 0.3 * np.sin(2 * z), x + z * y, 0.5 * x * x - np.cos(y)]
    M = Meshoid(pos, des_ngb=32)
    out = dict(pos=pos, v=v, curl=M.Curl(v), div=M.Div(v))
    Mm = Meshoid(pos, des_ngb=32, particle_mask=np.arange(400))
    out.update(curl_mask=Mm.Curl(v), div_mask=Mm.Div(v), ngb_mask=Mm.ngb)
    Ms = Meshoid(pos, des_ngb=32)
    Ms.Slice(x, center=np.array([0.5, 0.5, 0.5]), size=1.0, res=8, order=1)
    raised = 0
    try:
        Ms.Curl(v)
    except IndexError:
        raised = 1
    out["curl_after_slice_indexerror"] = np.array(raised)
    save("curl_div_800", **out)


if __name__ == "__main__":
    only = os.environ.get("GOLDEN_ONLY", "").split(",")
    for fn in (case_uniform, case_periodic, case_plummer, case_2d, case_ngb64, case_slice, case_mask, case_extras,
               case_deposit3d, case_radtransfer, case_weights_kde, case_surface_multigrid, case_notebook, case_lowdim, case_curl_div):
        if only != [""] and fn.__name__ not in only:
            continue
        t = time.time()
        fn()
        print(f"{fn.__name__}: {time.time() - t:.1f} s")
