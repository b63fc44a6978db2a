"""GPU ray-driven (Amanatides-Woo / Joseph, sys_mat/rd.py) and pixel-driven
(sys_mat/pd.py) projectors against the reference's golden vectors and the
FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def _call(mod, name, g, bp, joseph=None):
    kw = {k: float(g[k]) for k in ("du", "su", "d_pix", "dv", "sv") if k in g}
    if joseph is not None:
        kw["joseph"] = joseph
    geo = [float(g["DSO"]), float(g["DSD"])] if "DSO" in g else []
    x = g["vol"] if "vol" in g else g["img"]
    if bp:
        return getattr(mod, name)(g["y"], g["angs"], x.shape, *geo, **kw)
    det = [int(g["nu"])] + ([int(g["nv"])] if "nv" in g else [])
    return getattr(mod, name)(x, g["angs"], *det, *geo, **kw)


@pytest.mark.parametrize("tag,joseph", [("aw", False), ("joseph", True)])
def test_rd_golden(vg, golden, tag, joseph):
    from vir_gb300.sys_mat import rd
    for case, geo in ((f"rd_par_{tag}_10", "par_2d"), (f"rd_fan_{tag}", "fan_2d"),
                      (f"rd_cone_{tag}", "cone_3d")):
        g = golden[case]
        fp = _call(rd, "aw_fp_" + geo, g, False, joseph)
        assert fp.dtype == np.float32 and fp.shape == g["sino"].shape
        assert rel(fp, g["sino"]) < 2e-5, case
        assert rel(_call(rd, "aw_bp_" + geo, g, True, joseph), g["bp"]) < 2e-5, case


@pytest.mark.parametrize("tag,joseph", [("aw", False), ("joseph", True)])
def test_rd_axis_aligned_fix(vg, golden, orc, tag, joseph):
    from vir_gb300.sys_mat import rd
    g = golden[f"rd_par_{tag}_14"]
    fp = _call(rd, "aw_fp_par_2d", g, False, joseph)
    assert rel(fp[1:], g["sino"][1:]) < 2e-5            # the reference, off axis
    assert rel(fp, _call(orc, "aw_fp_par_2d", g, False, joseph)) < 2e-5


@pytest.mark.parametrize("case", ["pd_par", "pd_fan", "pd_cone"])
def test_pd_golden(vg, golden, case):
    from vir_gb300.sys_mat import pd
    g = golden[case]
    geo = case.split("_")[1] + ("_3d" if case == "pd_cone" else "_2d")
    fp = _call(pd, "pd_fp_" + geo, g, False)
    assert fp.dtype == np.float32 and fp.shape == g["sino"].shape
    assert rel(fp, g["sino"]) < 2e-5
    assert rel(_call(pd, "pd_bp_" + geo, g, True), g["bp"]) < 2e-5


@pytest.mark.parametrize("joseph", [False, True])
def test_rd_2d_vs_oracle(vg, orc, joseph):
    from vir_gb300 import phantoms as ph
    from vir_gb300.sys_mat import rd
    img, _ = ph.ellipse_phantom(96, 8, seed=6, d_pix=0.8, vmax=1.0)
    angs = np.linspace(0, np.pi, 60, endpoint=False)
    angf = np.linspace(0, 2 * np.pi, 60, endpoint=False)
    y = np.random.default_rng(8).random((60, 150)).astype(np.float32)
    # float32 ray parameters: the fan's t runs from the source (|t| ~ DSO = 150),
    # so its segment lengths carry ~1e-5 absolute rounding, as the reference's do
    for name, args, tol in (("par_2d", (angs, 150), 2e-5),
                            ("fan_2d", (angf, 150, 150.0, 300.0), 1e-4)):
        kw = dict(du=0.9, su=0.3, d_pix=0.8, joseph=joseph)
        fp = getattr(rd, "aw_fp_" + name)(img, *args, **kw)
        assert rel(fp, getattr(orc, "aw_fp_" + name)(img, *args, **kw)) < tol, name
        bargs = (args[0], img.shape) + args[2:]
        bp = getattr(rd, "aw_bp_" + name)(y, *bargs, **kw)
        bo = getattr(orc, "aw_bp_" + name)(y, *bargs, **kw)
        if joseph:
            # a ray whose length is within rounding of a multiple of the 0.5 step
            # gains or loses its last sample, which lies on the image edge: the
            # border pixels differ by up to one splat, the interior does not
            assert rel(bp[1:-1, 1:-1], bo[1:-1, 1:-1]) < tol, name
            assert rel(bp, bo) < 1e-2, name
        else:
            assert rel(bp, bo) < tol, name


@pytest.mark.parametrize("geo", ["par", "fan", "fan_near", "fan_wide"])
def test_joseph_bp_2d_vs_oracle(vg, orc, geo):
    """The 2D Joseph back projection (per-cell sums in registers before the
    atomics) on a non-square 200 x 130 image with rays 0.2 mm apart against
    0.7 mm pixels (several rays per pixel), zero rays, a source 12 mm from the
    image corner and a wide fan (edge rays at 41 degrees)."""
    from vir_gb300.sys_mat import rd
    rng = np.random.default_rng(21)
    na, nu = 90, 700
    angs = np.linspace(0, np.pi if geo == "par" else 2 * np.pi, na, endpoint=False)
    y = rng.random((na, nu)).astype(np.float32)
    y[:, ::7] = 0.0  # zero rays are skipped
    kw = dict(du=0.2, su=0.4, d_pix=0.7, joseph=True)
    fan = {"fan": (220.0, 400.0), "fan_near": (95.0, 300.0), "fan_wide": (220.0, 80.0)}
    args = (angs, (200, 130)) + fan.get(geo, ())
    name = "par" if geo == "par" else "fan"
    bp = getattr(rd, "aw_bp_%s_2d" % name)(y, *args, **kw)
    bo = getattr(orc, "aw_bp_%s_2d" % name)(y, *args, **kw)
    # interior exact to float32 rounding; the border as in test_rd_2d_vs_oracle
    assert rel(bp[1:-1, 1:-1], bo[1:-1, 1:-1]) < 2e-5
    assert rel(bp, bo) < 1e-2


@pytest.mark.parametrize("joseph", [False, True])
def test_rd_cone_vs_oracle(vg, orc, joseph):
    """nu != nv: the rows come from nv (rd.py:688 uses nu)."""
    from vir_gb300.sys_mat import rd
    rng = np.random.default_rng(9)
    vol = rng.random((20, 18, 14)).astype(np.float32)
    angs = np.linspace(0, 2 * np.pi, 16, endpoint=False)
    kw = dict(du=1.2, dv=1.1, su=0.2, sv=-0.3, d_pix=1.0, joseph=joseph)
    fp = rd.aw_fp_cone_3d(vol, angs, 36, 28, 50.0, 90.0, **kw)
    assert rel(fp, orc.aw_fp_cone_3d(vol, angs, 36, 28, 50.0, 90.0, **kw)) < 1e-4
    y = rng.random(fp.shape).astype(np.float32)
    bp = rd.aw_bp_cone_3d(y, angs, vol.shape, 50.0, 90.0, **kw)
    assert rel(bp, orc.aw_bp_cone_3d(y, angs, vol.shape, 50.0, 90.0, **kw)) < 1e-4


def test_rd_aw_adjoint(vg):
    """The AW pair is a scaled transpose: BP = A^T y du / (na d_pix^2)."""
    import torch
    from vir_gb300.sys_mat import rd
    g = torch.Generator(device="cuda").manual_seed(2)
    x = torch.rand((80, 70), device="cuda", generator=g)
    y = torch.rand((45, 120), device="cuda", generator=g)
    angs = np.linspace(0, 2 * np.pi, 45, endpoint=False)
    A = rd.aw_fp_fan_2d(x, angs, 120, 120.0, 250.0, du=1.1, d_pix=1.0)
    B = rd.aw_bp_fan_2d(y, angs, (80, 70), 120.0, 250.0, du=1.1, d_pix=1.0)
    f = float(np.float32(1.1))
    lhs = (A.double() * y.double()).sum().item()
    rhs = (x.double() * B.double()).sum().item() * 45 / f
    assert abs(lhs - rhs) / lhs < 1e-5


def test_pd_vs_oracle(vg, orc):
    from vir_gb300 import phantoms as ph
    from vir_gb300.sys_mat import pd
    img, _ = ph.ellipse_phantom(64, 6, seed=7, d_pix=1.0, vmax=1.0)
    angs = np.linspace(0, np.pi, 40, endpoint=False)
    angf = np.linspace(0, 2 * np.pi, 40, endpoint=False)
    y = np.random.default_rng(10).random((40, 100)).astype(np.float32)
    for name, args in (("par_2d", (angs, 100)), ("fan_2d", (angf, 100, 100.0, 200.0))):
        kw = dict(du=1.1, su=0.2, d_pix=1.0)
        fp = getattr(pd, "pd_fp_" + name)(img, *args, **kw)
        assert rel(fp, getattr(orc, "pd_fp_" + name)(img, *args, **kw)) < 2e-5, name
        bargs = (args[0], img.shape) + args[2:]
        bp = getattr(pd, "pd_bp_" + name)(y, *bargs, **kw)
        assert rel(bp, getattr(orc, "pd_bp_" + name)(y, *bargs, **kw)) < 2e-5, name
    vol = np.random.default_rng(11).random((16, 16, 12)).astype(np.float32)
    a3 = np.linspace(0, 2 * np.pi, 12, endpoint=False)
    kw = dict(du=1.2, dv=1.3, su=0.1, sv=0.2, d_pix=1.0)
    fp = pd.pd_fp_cone_3d(vol, a3, 30, 24, 40.0, 80.0, **kw)
    assert rel(fp, orc.pd_fp_cone_3d(vol, a3, 30, 24, 40.0, 80.0, **kw)) < 2e-5
    ys = np.random.default_rng(12).random(fp.shape).astype(np.float32)
    bp = pd.pd_bp_cone_3d(ys, a3, vol.shape, 40.0, 80.0, **kw)
    assert rel(bp, orc.pd_bp_cone_3d(ys, a3, vol.shape, 40.0, 80.0, **kw)) < 2e-5


def test_pd_cone_columns_vs_oracle(vg, orc):
    """Cone pixel-driven FP and BP, one warp per column: x, y not multiples of
    the 2 x 4 column patch, 300 slices (three z chunks of 128, the last
    ragged), zero voxels, a detector taller than the volume's shadow, and a
    coarse detector (pitch 0.3 mm under 0.8 mm voxels: footprints over more
    than 4 cells take the general walk)."""
    from vir_gb300.sys_mat import pd
    rng = np.random.default_rng(23)
    shape = (13, 10, 300)
    vol = rng.random(shape).astype(np.float32)
    vol[:, :, ::5] = 0.0
    a3 = np.linspace(0, 2 * np.pi, 9, endpoint=False)
    # the float32 footprint ends (~13 mm off axis) carry ~1.5e-5 mm of rounding:
    # up to 5e-5 of a 0.3 mm cell's overlap, the same in the per-pixel kernels
    for du, nu, nv, tol in ((1.1, 28, 420, 2e-5), (0.3, 90, 1300, 1e-4)):
        kw = dict(du=du, dv=0.9 * du / 1.1, su=0.3, sv=-0.4, d_pix=0.8)
        fp = pd.pd_fp_cone_3d(vol, a3, nu, nv, 200.0, 320.0, **kw)
        assert rel(fp, orc.pd_fp_cone_3d(vol, a3, nu, nv, 200.0, 320.0, **kw)) < tol, du
        ys = rng.random((9, nu, nv)).astype(np.float32)
        bp = pd.pd_bp_cone_3d(ys, a3, shape, 200.0, 320.0, **kw)
        assert rel(bp, orc.pd_bp_cone_3d(ys, a3, shape, 200.0, 320.0, **kw)) < 2e-5, du


@pytest.mark.parametrize("geo", ["par", "fan"])
def test_pd_fp_2d_runs_vs_oracle(vg, orc, geo):
    """2D pixel-driven FP, one thread per run of 32 pixels along y: 45 x 70
    image (runs cut short at the column end), zero pixels inside runs, views
    all round (footprints moving both ways along u; at 90 and 270 degrees the
    fan's direction changes across the image)."""
    from vir_gb300.sys_mat import pd
    rng = np.random.default_rng(31)
    img = rng.random((45, 70)).astype(np.float32)
    img[:, 3::9] = 0.0
    img[7] = 0.0
    angs = np.linspace(0, 2 * np.pi, 36, endpoint=False)
    kw = dict(du=0.7, su=0.25, d_pix=0.9)
    args = (angs, 160) + (() if geo == "par" else (90.0, 170.0))
    fp = getattr(pd, "pd_fp_%s_2d" % geo)(img, *args, **kw)
    assert rel(fp, getattr(orc, "pd_fp_%s_2d" % geo)(img, *args, **kw)) < 2e-5


def test_joseph_cone_bp_z_faces_vs_oracle(vg, orc):
    """Cone Joseph BP with detector rows beyond both z faces, so samples
    splat onto the first and last slices (half of their corners outside the
    volume)."""
    from vir_gb300.sys_mat import rd
    rng = np.random.default_rng(33)
    shape = (10, 9, 16)
    angs = np.linspace(0, 2 * np.pi, 14, endpoint=False)
    kw = dict(du=1.1, dv=0.7, su=0.2, sv=-0.1, d_pix=1.0, joseph=True)
    y = rng.random((14, 30, 48)).astype(np.float32)
    bp = rd.aw_bp_cone_3d(y, angs, shape, 50.0, 90.0, **kw)
    assert rel(bp, orc.aw_bp_cone_3d(y, angs, shape, 50.0, 90.0, **kw)) < 1e-4


@pytest.mark.parametrize("geo", ["par", "fan"])
def test_aw_bp_gather_boundary_rays(vg, orc, geo):
    """The 2D AW back projection's gather form where rays run exactly along
    pixel boundaries (integer u on a 1 mm grid, views at 0, 45, 90 ... deg):
    such a ray belongs to the row or column the walk enters, as in the oracle's
    walk, and 45-degree rays through pixel corners split nothing twice."""
    from vir_gb300.sys_mat import rd
    rng = np.random.default_rng(17)
    angs = np.linspace(0, 2 * np.pi if geo == "fan" else np.pi, 8, endpoint=False)
    y = rng.random((8, 97)).astype(np.float32)
    if geo == "par":
        kw = dict(du=1.0, d_pix=1.0)
        bp = rd.aw_bp_par_2d(y, angs, (64, 64), **kw)
        bo = orc.aw_bp_par_2d(y, angs, (64, 64), **kw)
        tol = 2e-5
    else:
        kw = dict(du=2.0, d_pix=1.0)
        bp = rd.aw_bp_fan_2d(y, angs, (64, 64), 100.0, 200.0, **kw)
        bo = orc.aw_bp_fan_2d(y, angs, (64, 64), 100.0, 200.0, **kw)
        tol = 1e-4
    assert rel(bp, bo) < tol


def test_aw_bp_gather_fan_benchmark_geometry(vg, orc):
    """The gather at the fan SIRT geometry (512^2, 720 views, 768 bins of
    1.2 mm, DSO 500, DSD 1000, 0.9 mm pixels): against the FP64 walk within
    4e-4 of the peak (float32 ray positions some 300 mm from the centre carry
    ~3e-5 mm, which near-axis chord splits magnify; the float32 walk itself
    is at 6e-4), and the transpose of the walk's forward projection within
    1e-5 in the dot test."""
    import torch
    from vir_gb300.sys_mat import rd
    rng = np.random.default_rng(23)
    angs = np.linspace(0, 2 * np.pi, 720, endpoint=False)
    y = rng.random((720, 768)).astype(np.float32)
    kw = dict(du=1.2, d_pix=0.9)
    bp = rd.aw_bp_fan_2d(y, angs, (512, 512), 500.0, 1000.0, **kw)
    bo = orc.aw_bp_fan_2d(y, angs, (512, 512), 500.0, 1000.0, **kw)
    assert rel(bp, bo) < 4e-4
    x = torch.rand((512, 512), device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    A = rd.aw_fp_fan_2d(x, angs, 768, 500.0, 1000.0, **kw)
    B = rd.aw_bp_fan_2d(torch.from_numpy(y).cuda(), angs, (512, 512), 500.0, 1000.0, **kw)
    lhs = float((A.double() * torch.from_numpy(y).cuda().double()).sum())
    rhs = float((x.double() * B.double()).sum()) * 720 * 0.9 ** 2 / float(np.float32(1.2))
    assert abs(lhs - rhs) / lhs < 1e-5


@pytest.mark.parametrize("geo", ["par", "fan"])
def test_aw_bp_gather_odd_image(vg, orc, geo):
    """Odd, non-square images (the last 2 x 2 patch of a row or column half
    outside) and a detector shifted off centre, against the FP64 walk."""
    from vir_gb300.sys_mat import rd
    rng = np.random.default_rng(41)
    na, nu = 30, 90
    angs = np.linspace(0.2, 0.2 + (2 * np.pi if geo == "fan" else np.pi), na, endpoint=False)
    y = rng.random((na, nu)).astype(np.float32)
    kw = dict(du=0.9, su=1.7, d_pix=0.8)
    if geo == "par":
        bp = rd.aw_bp_par_2d(y, angs, (37, 53), **kw)
        bo = orc.aw_bp_par_2d(y, angs, (37, 53), **kw)
        tol = 2e-5
    else:
        bp = rd.aw_bp_fan_2d(y, angs, (37, 53), 90.0, 160.0, **kw)
        bo = orc.aw_bp_fan_2d(y, angs, (37, 53), 90.0, 160.0, **kw)
        tol = 1e-4
    assert bp.shape == (37, 53)
    assert rel(bp, bo) < tol


def test_aw_bp_gather_deterministic(vg):
    """The gather form sums each pixel's rays in a fixed order: repeated
    back projections are bit-identical (the atomic scatter's were not)."""
    from vir_gb300.sys_mat import rd
    rng = np.random.default_rng(43)
    angs = np.linspace(0, 2 * np.pi, 120, endpoint=False)
    y = rng.random((120, 200)).astype(np.float32)
    runs = [rd.aw_bp_fan_2d(y, angs, (150, 150), 200.0, 380.0, du=1.1, d_pix=1.0) for _ in range(3)]
    assert all(np.array_equal(runs[0], r) for r in runs[1:])
