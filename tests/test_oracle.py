"""Pins the FP64 oracle against golden vectors produced by the reference
itself (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


@pytest.mark.parametrize("case", ["siddon2d_a", "siddon2d_b"])
def test_siddon2d_fp_bit_exact(golden, orc, case):
    g = golden[case]
    out = orc.siddons_fp_2d(g["img"], g["angs"], int(g["n_dets"]), float(g["d_det"]),
                            float(g["d_pix"]), mode="ref")
    # float32-rounded accumulation reproduces fp_2d_par.siddons_fp_2d bit for bit
    assert np.array_equal(out.astype(np.float32), g["sino"])
    fp64 = orc.siddons_fp_2d(g["img"], g["angs"], int(g["n_dets"]), float(g["d_det"]),
                             float(g["d_pix"]))
    assert rel(fp64, g["sino"]) < 1e-6


@pytest.mark.parametrize("case", ["siddon2d_a", "siddon2d_b"])
def test_siddon2d_adjoint(golden, orc, case):
    g = golden[case]
    img = g["img"]
    y = np.random.default_rng(1).random(g["sino"].shape).astype(np.float32)
    A = orc.siddons_fp_2d(img, g["angs"], int(g["n_dets"]), float(g["d_det"]), float(g["d_pix"]))
    At = orc.siddons_bp_2d(y, g["angs"], img.shape, float(g["d_det"]), float(g["d_pix"]))
    lhs = (A * y).sum()
    rhs = (img.astype(np.float64) * At).sum()
    assert abs(lhs - rhs) / abs(lhs) < 1e-12


@pytest.mark.parametrize("case", ["dd_par_a", "dd_par_b"])
def test_dd_par(golden, orc, case):
    g = golden[case]
    fp = orc.dd_fp_par_2d(g["img"], g["angs"], int(g["nu"]), float(g["du"]), float(g["su"]),
                          float(g["d_pix"]))
    assert rel(fp, g["sino"]) < 2e-5
    bp = orc.dd_bp_par_2d(g["y"], g["angs"], g["img"].shape, float(g["du"]), float(g["su"]),
                          float(g["d_pix"]))
    assert rel(bp, g["bp"]) < 2e-5


@pytest.mark.parametrize("case", ["dd_fan_a", "dd_fan_b"])
def test_dd_fan(golden, orc, case):
    g = golden[case]
    args = (float(g["DSO"]), float(g["DSD"]), float(g["du"]), float(g["su"]), float(g["d_pix"]))
    fp = orc.dd_fp_fan_2d(g["img"], g["angs"], int(g["nu"]), *args)
    assert rel(fp, g["sino"]) < 2e-5
    bp = orc.dd_bp_fan_2d(g["y"], g["angs"], g["img"].shape, *args)
    assert rel(bp, g["bp"]) < 2e-5


def test_dd_mass_conservation(orc):
    """Each parallel DD view sums to sum(img) * d_pix^2 / du (every pixel's
    projected footprint lies on the detector)."""
    img = np.random.default_rng(3).random((40, 40)).astype(np.float32)
    ang = np.linspace(0, np.pi, 16, endpoint=False)
    s = orc.dd_fp_par_2d(img, ang, 90, du=0.9, d_pix=1.1)
    want = img.astype(np.float64).sum() * 1.1 ** 2 / 0.9
    assert np.allclose(s.sum(axis=1), want, rtol=1e-6)


@pytest.mark.parametrize("fan", [0, 1])
def test_dd_scaled_adjoint(orc, fan):
    """<FP x, y> = na * d_pix^2 / du * <x, BP y> (the reference BP is A^T/(na d_pix)
    and FP is A d_pix/du)."""
    rng = np.random.default_rng(4)
    x = rng.random((28, 28)).astype(np.float32)
    ang = np.linspace(0, 2 * np.pi, 20, endpoint=False)
    y = rng.random((20, 50)).astype(np.float32)
    if fan:
        A = orc.dd_fp_fan_2d(x, ang, 50, 60.0, 110.0, du=1.1, d_pix=0.8)
        B = orc.dd_bp_fan_2d(y, ang, x.shape, 60.0, 110.0, du=1.1, d_pix=0.8)
    else:
        A = orc.dd_fp_par_2d(x, ang, 50, du=1.1, d_pix=0.8)
        B = orc.dd_bp_par_2d(y, ang, x.shape, du=1.1, d_pix=0.8)
    lhs = (A * y).sum()
    # the DD functions cast du and d_pix to float32 first (dd.py:653)
    d, u = float(np.float32(0.8)), float(np.float32(1.1))
    rhs = (x * B).sum() * 20 * d * d / u
    assert abs(lhs - rhs) / lhs < 1e-12


def test_dd_cone(golden, orc):
    g = golden["dd_cone"]
    kw = dict(du=float(g["du"]), dv=float(g["dv"]), su=float(g["su"]), sv=float(g["sv"]),
              d_pix=float(g["d_pix"]))
    fp = orc.dd_fp_cone_3d(g["vol"], g["angs"], int(g["nu"]), int(g["nv"]), float(g["DSO"]),
                           float(g["DSD"]), **kw)
    # the oracle states the intended sweep: it matches the reference with tmp_u
    # cleared per line, and not the reference as shipped (stale tmp_u)
    assert rel(fp, g["sino_fixed"]) < 2e-5
    assert rel(fp, g["sino_ref"]) > 1e-2
    bp = orc.dd_bp_cone_3d(g["y"], g["angs"], g["vol"].shape, float(g["DSO"]), float(g["DSD"]),
                           **kw)
    assert rel(bp, g["bp"]) < 2e-5
    # scaled adjoint: <FP x, y> = na d_pix^3 / (du dv) <x, BP y>
    na = g["angs"].size
    lhs = (fp * g["y"]).sum()
    f = {k: float(np.float32(v)) for k, v in kw.items()}
    rhs = (g["vol"] * bp).sum() * na * f["d_pix"] ** 3 / (f["du"] * f["dv"])
    assert abs(lhs - rhs) / lhs < 1e-12


def test_sf_fan(golden, orc):
    g = golden["sf_fan"]
    fp = orc.sf_fp_fan_2d(g["img"], g["angs"], int(g["nu"]), float(g["DSO"]), float(g["DSD"]),
                          float(g["du"]), float(g["d_pix"]))
    assert rel(fp, g["sino"]) < 1e-6
    y = np.random.default_rng(5).random(fp.shape).astype(np.float32)
    bp = orc.sf_bp_fan_2d(y, g["angs"], g["img"].shape, float(g["DSO"]), float(g["DSD"]),
                          float(g["du"]), float(g["d_pix"]))
    assert abs((fp * y).sum() - (g["img"] * bp).sum()) / (fp * y).sum() < 1e-12


def test_sf_par_rect(golden, orc):
    g = golden["sf_par_rect"]
    fp = orc.separable_footprint_fp_2d(g["img"], g["angs"], int(g["n_dets"]), float(g["d_det"]),
                                       float(g["d_pix"]))
    assert rel(fp, g["sino"]) < 1e-6
    y = np.random.default_rng(6).random(fp.shape).astype(np.float32)
    bp = orc.separable_footprint_bp_2d(y, g["angs"], g["img"].shape, float(g["d_det"]),
                                       float(g["d_pix"]))
    assert abs((fp * y).sum() - (g["img"] * bp).sum()) / (fp * y).sum() < 1e-12


def test_filter_sino(golden, orc):
    n = 0
    for case in golden.cases:
        if not case.startswith("filter_"):
            continue
        g = golden[case]
        out = orc.filter_sino(g["sino"], du=float(g["du"]), filter_type=str(g["filter_type"]),
                              cutoff=float(g["cutoff"]), real_space=bool(g["real_space"]))
        assert np.allclose(out, g["filtered"], rtol=0, atol=1e-12), case
        n += 1
    assert n == 28


def test_list_c(golden, orc):
    """The reference's own C list projector (projection_c.c) against the
    oracle's CSR gather/scatter over the same Siddon list."""
    d = golden["siddons_cone"]
    g = golden["list_c"]
    fp = orc.list_fp(g["phantom"], d["ind"], d["len"], d["off"])
    assert rel(fp, g["sino"]) < 1e-6
    bp = orc.list_bp(g["y"], d["ind"], d["len"], d["off"], g["phantom"].size)
    assert rel(bp, g["bp"].ravel()) < 1e-6


def test_sirt_rule(golden, orc):
    g = golden["sirt_par"]
    nu = int(g["nu"])
    fp = lambda x: orc.dd_fp_par_2d(x, g["angs"], nu)
    bp = lambda s: orc.dd_bp_par_2d(s, g["angs"], g["img"].shape)
    x = orc.sirt(g["sino"], fp, bp, g["img"].shape, gamma=float(g["gamma"]), iters=int(g["iters"]))
    assert rel(x, g["x"]) < 1e-4


SQ_GEO = ("du", "dv", "dsrc_p", "dsrc_z", "su", "sv", "ssrc_p", "ssrc_z", "d_pix")


def square_kw(g):
    return {k: float(g[k]) for k in SQ_GEO}


@pytest.mark.parametrize("case", ["square_a", "square_b"])
def test_dd_square(golden, orc, case):
    g = golden[case]
    kw = square_kw(g)
    fp = orc.dd_fp_square(g["vol"], int(g["nu"]), int(g["nv"]), int(g["nsrc_p"]),
                          int(g["nsrc_z"]), float(g["DSO"]), float(g["DSD"]), **kw)
    assert rel(fp, g["sino"]) < 2e-6
    bp = orc.dd_bp_square(g["y"], g["vol"].shape, float(g["DSO"]), float(g["DSD"]), **kw)
    assert rel(bp, g["bp"]) < 2e-6
    # FP = A d_pix^2 / (du dv) and BP = A^T exactly (dd.py:930, 1135)
    f = lambda v: float(np.float32(v))
    lhs = (fp * g["y"]).sum()
    rhs = (g["vol"].astype(np.float64) * bp).sum() * f(kw["d_pix"]) ** 2 / (f(kw["du"]) * f(kw["dv"]))
    assert abs(lhs - rhs) / abs(lhs) < 1e-12


def test_dd_square_rejects_rectangular(orc):
    with pytest.raises(ValueError, match="nx must equal ny"):
        orc.dd_fp_square(np.zeros((4, 5, 3), np.float32), 8, 8, 2, 2, 20.0, 36.0)


def test_sirt_square_rule(golden, orc):
    """sirt_dd.sirt (executed from the reference source around its own square
    projectors) against the FP64 oracle's rule on the oracle's projectors."""
    g = golden["sirt_square"]
    DSO, DSD = (float(v) for v in g["gem_prms"])
    nx, ny, nz, d_pix = g["img_prms"]
    nsrc_p, nsrc_z, dsrc_p, dsrc_z, ssrc_p, ssrc_z = g["src_prms"]
    nu, nv, du, dv, su, sv = g["det_prms"]
    gamma, iters = g["srt_prms"]
    kw = dict(du=du, dv=dv, dsrc_p=dsrc_p, dsrc_z=dsrc_z, su=su, sv=sv, ssrc_p=ssrc_p,
              ssrc_z=ssrc_z, d_pix=d_pix)
    shape = (int(nx), int(ny), int(nz))
    fp = lambda x: orc.dd_fp_square(x, int(nu), int(nv), int(nsrc_p), int(nsrc_z), DSO, DSD, **kw)
    bp = lambda s: orc.dd_bp_square(s, shape, DSO, DSD, **kw)
    assert rel(fp(np.ones(shape, np.float32)), g["W_sino"]) < 2e-6
    x = orc.sirt(g["sino"], fp, bp, shape, gamma=float(gamma), iters=int(iters))
    assert rel(x, g["x"]) < 1e-4


# --- ray-driven (rd.py) and pixel-driven (pd.py) --------------------------------

def _rd_call(orc, name, g, bp, joseph=None):
    kw = {k: float(g[k]) for k in ("du", "su", "d_pix", "dv", "sv") if k in g}
    if joseph is not None:
        kw["joseph"] = joseph
    geo = [float(g["DSO"]), float(g["DSD"])] if "DSO" in g else []
    x = g["vol"] if "vol" in g else g["img"]
    if bp:
        return getattr(orc, name)(g["y"], g["angs"], x.shape, *geo, **kw)
    det = [int(g["nu"])] + ([int(g["nv"])] if "nv" in g else [])
    return getattr(orc, name)(x, g["angs"], *det, *geo, **kw)


@pytest.mark.parametrize("tag,joseph", [("aw", False), ("joseph", True)])
def test_rd(golden, orc, tag, joseph):
    for case, geo in ((f"rd_par_{tag}_10", "par_2d"), (f"rd_fan_{tag}", "fan_2d"),
                      (f"rd_cone_{tag}", "cone_3d")):
        g = golden[case]
        assert rel(_rd_call(orc, "aw_fp_" + geo, g, False, joseph), g["sino"]) < 1e-5, case
        assert rel(_rd_call(orc, "aw_bp_" + geo, g, True, joseph), g["bp"]) < 1e-5, case


@pytest.mark.parametrize("tag,joseph", [("aw", False), ("joseph", True)])
def test_rd_axis_aligned_fix(golden, orc, tag, joseph):
    """Detector wider than the image: the reference's 0-degree rays beside the
    image walk its edge row (rd.py:52-64); every other view agrees."""
    g = golden[f"rd_par_{tag}_14"]
    fp = _rd_call(orc, "aw_fp_par_2d", g, False, joseph)
    assert rel(fp[1:], g["sino"][1:]) < 1e-5
    assert g["sino"][0].sum() > fp[0].sum() + 1.0    # the over-count, not reproduced
    # rays beside the image see nothing
    u = 1.0 * (np.arange(14) - 6.5 + 0.2)
    assert np.all(fp[0][np.abs(u) > 6.0] == 0.0)


@pytest.mark.parametrize("case", ["pd_par", "pd_fan", "pd_cone"])
def test_pd(golden, orc, case):
    g = golden[case]
    geo = case.split("_")[1] + ("_3d" if case == "pd_cone" else "_2d")
    assert rel(_rd_call(orc, "pd_fp_" + geo, g, False), g["sino"]) < 1e-5
    assert rel(_rd_call(orc, "pd_bp_" + geo, g, True), g["bp"]) < 1e-5


def test_tv_ops(golden, orc):
    """grad / div / grad_abs / div_abs / pyT of tv.py:98-224 (reference source)."""
    g = golden["tv_ops"]
    assert np.allclose(orc.tv_grad(g["x"]), g["grad"], rtol=0, atol=1e-12)
    assert np.allclose(orc.tv_div(g["z"]), g["div"], rtol=0, atol=1e-12)
    assert np.allclose(orc.tv_grad_abs(g["x"]), g["grad_abs"], rtol=0, atol=1e-12)
    assert np.allclose(orc.tv_div_abs(g["z"]), g["div_abs"], rtol=0, atol=1e-12)
    assert np.allclose(orc.tv_project(g["AA"]), g["pyT"], rtol=0, atol=1e-12)
    # div is the negative adjoint of grad
    rng = np.random.default_rng(0)
    x, z = rng.normal(size=(9, 7)), rng.normal(size=(2, 9, 7))
    assert abs((orc.tv_grad(x) * z).sum() + (x * orc.tv_div(z)).sum()) < 1e-10


def _water(e):
    """The synthetic water attenuation curve of the beam-hardening fixtures."""
    return 0.17 + 2500.0 * np.asarray(e, np.float64) ** -3.0


def test_beamhard_oracle(golden, orc):
    p = golden["bh_poly"]
    li, coefs, mu = p["line_ints"], p["coefs"], float(p["mu"])
    assert np.array_equal(orc.bh_poly(li, coefs, mu), p["cor_f64coefs"])
    assert np.array_equal(orc.bh_poly(li, [float(c) for c in coefs], mu), p["cor_pycoefs"])
    assert np.array_equal(orc.bh_poly(li, coefs, np.float64(mu)), p["cor_f64mu"])
    t = golden["bh_table"]
    assert np.array_equal(orc.bh_table(t["line_ints"], t["energies"], t["counts"],
                                       float(t["atten_eff"]), t["attens"]), t["cor"])
    lut = golden["bh_lut"]
    assert np.array_equal(orc.bh_lut(lut["line_ints"], lut["coefs"], float(lut["mu"])), lut["cor"])
    c = golden["bh_coefs2_fan"]
    n = 512
    gam = np.linspace(-n + 1, n - 1, n) * (float(c["fan_angle"]) / n) / 2.0
    co = orc.bh_sphere_fan_coefs(c["energies"], c["counts"], gam, float(c["src_iso"]),
                                 float(c["atten_eff"]), _water(c["energies"]))
    assert np.allclose(co, c["coefs"], rtol=1e-12, atol=0)


def test_beamhard_host_logic(golden):
    """The host side of vir_gb300.beamhard (no device): numpy's step types for
    the polynomial, the interp1d table, the sphere fits and the water tub."""
    from types import SimpleNamespace
    from vir_gb300 import beamhard as bh
    assert bh._poly_types(np.float32, np.array([0.1, 0.2, 0.3]), 0.2) == (1, np.float64)
    assert bh._poly_types(np.float32, [0.1, 0.2, 0.3], 0.2) == (31, np.float32)
    assert bh._poly_types(np.float32, np.array([0.1, 0.2, 0.3]), np.float64(0.2))[0] == 0
    assert bh._poly_types(np.float64, [0.1, 0.2, 0.3], 0.2) == (0, np.float64)
    c = golden["bh_coefs2_fan"]
    n = 512
    g = SimpleNamespace(geom="Fan beam", src_iso=float(c["src_iso"]),
                        gammas=lambda k: np.linspace(-k + 1, k - 1, k) * (float(c["fan_angle"]) / k) / 2.0)
    co = bh.beamhard_coefs2(c["energies"], c["counts"], g, float(c["atten_eff"]),
                            mixatten=lambda m, e: _water(e))
    assert np.allclose(co, c["coefs"], rtol=1e-12, atol=0)
    with pytest.raises(ValueError):
        bh.beamhard_coefs2(c["energies"], c["counts"], g, float(c["atten_eff"]))
    t = golden["bh_table"]
    x, y = bh.spectrum_table(t["energies"], t["counts"], float(t["atten_eff"]), t["attens"])
    assert np.all(np.diff(x) > 0) and x[0] == 0.0 and y[-1] == 80 * float(t["atten_eff"])
    tub = bh.water_tub_phantom(64, 1.0, 20)
    ii, jj = np.indices((64, 64))
    assert np.array_equal(tub, (ii - 32) ** 2 + (jj - 32) ** 2 < 400)


def test_beamhard_float32_search_keys():
    """The lookup kernel searches float32 keys (x rounded toward -inf for
    searchsorted 'left', toward +inf for 'right'); for float32 samples that
    finds numpy's float64 index exactly, on and beside every key."""
    import torch
    from vir_gb300 import beamhard as bh
    rng = np.random.default_rng(0)
    x = np.sort(rng.random(2000) * 10)
    x[:5] = [0, 0.5, 1.0, 2.0, 3.0]
    y = rng.random(2000)
    xf = x.astype(np.float32)
    v = np.concatenate([(rng.random(100000) * 10).astype(np.float32), xf,
                        np.nextafter(xf, np.float32(np.inf)), np.nextafter(xf, np.float32(-np.inf))])
    for up, side in ((False, "left"), (True, "right")):
        seg, keys = bh._interp_table(x, y, torch.device("cpu"), True, up)
        k = keys.numpy()
        assert k.dtype == np.float32
        assert np.array_equal(np.searchsorted(k, v, side), np.searchsorted(x, v.astype(np.float64), side))
        s = seg.numpy()
        assert np.array_equal(s[:-1, 2], (y[1:] - y[:-1]) / (x[1:] - x[:-1])) and s[-1, 2] == 0


def _traj_geoms(h):
    from vir_gb300 import trajectory as tr
    G = tr.Geom(nViews=int(h["nViews"]), coverage=float(h["coverage"]), zTran=float(h["zTran"]))
    GI = tr.Geom(nViews=int(h["int_nViews"]), coverage=float(h["int_coverage"]),
                 angle0=float(h["int_angle0"]), zTran=float(h["int_zTran"]))
    return G, GI


def test_trajectory_host_logic(golden):
    """vir_gb300.trajectory's host side against the reference: Geom's views,
    z positions and interpZ, sino_hel_subset, the per-view affine matrices
    and the axial indices of sino_axl2hel."""
    from vir_gb300 import trajectory as tr
    h = golden["traj_hel2axl"]
    G, _ = _traj_geoms(h)
    assert np.array_equal(G.Z, h["gH_Z"]) and np.array_equal(G.Views, h["gH_Views"])
    iz = golden["traj_interpZ"]
    r = G.interpZ(iz["zA"], float(iz["angle"]), int(iz["nRows"]))
    assert all(np.array_equal(np.asarray(a), iz[f"r{k}"]) for k, a in enumerate(r))
    s = golden["traj_subset"]
    GS, _ = _traj_geoms(h)
    sub = tr.sino_hel_subset(h["sinoH"], GS, int(s["nRows"]), s["z"])
    assert np.array_equal(sub, s["sub"]) and np.array_equal(GS.Views, s["Views"])
    assert np.array_equal(GS.Z, s["Z"])
    f = golden["traj_fp_phantom"]
    M = tr.view_matrices(f["phantom"].shape, f["views"], f["Z"])
    assert np.allclose(M, f["mats"], rtol=1e-6, atol=1e-6)


def test_trajectory_oracle(golden, orc):
    from vir_gb300 import trajectory as tr
    for case in ("traj_axl2hel", "traj_axl2hel_z"):
        a = golden[case]
        nA, nR, _ = a["sinoA"].shape
        idx, zz, wrap, n = tr.axl2hel_index(nA, nR, int(a["nRowsH"]), a["viewsH"], int(a["nAngsH"]),
                                            float(a["pitch"]), a.get("Z"))
        assert n == a["viewsH"].size and wrap.sum() == 3
        assert np.array_equal(orc.axl2hel(a["sinoA"], idx, zz, wrap, int(a["nRowsH"])), a["sinoH"])
    h = golden["traj_hel2axl"]
    G, GI = _traj_geoms(h)
    src, A, Z = h["sinoH"], h["angsA"], h["zA"]
    sh = (A.size, Z.size, src.shape[2])
    pp, wp, pn, wn = tr._tables(G, [Z] * A.size, A, src.shape[1])
    assert np.array_equal(orc.rebin_rows(src, pp, wp, sh), h["a1"], equal_nan=True)
    assert np.array_equal(orc.rebin_rows(src, pn, wn, sh), h["a2"], equal_nan=True)
    bp, bwp, bn, bwn = tr._tables(G, [Z] * A.size, A + np.pi, src.shape[1])
    assert np.array_equal(orc.rebin_rows(src, bp, bwp, sh, True), h["b1"], equal_nan=True)
    assert np.array_equal(orc.rebin_rows(src, bn, bwn, sh, True), h["b2"], equal_nan=True)
    Zs = [tr.censpace(4, c=z) for z in GI.Z]
    pp, wp, pn, wn = tr._tables(G, Zs, list(GI.Views), src.shape[1])
    shi = (GI.nViews, 4, src.shape[2])
    assert np.array_equal(orc.rebin_rows(src, pp, wp, shi), h["i1"], equal_nan=True)
    assert np.array_equal(orc.rebin_rows(src, pn, wn, shi), h["i2"], equal_nan=True)
    f = golden["traj_fp_phantom"]
    assert rel(orc.rotsum_fp(f["phantom"], f["mats"]), f["sino"]) < 1e-6


def test_trajectory_interpZ_batch():
    """The all-angles evaluation of Geom.interpZ that builds the rebinning
    tables equals one interpZ call per angle, exactly (views on, between
    and past the sampled angles; integer and fractional rotation counts)."""
    from vir_gb300 import trajectory as tr
    rng = np.random.default_rng(3)
    for nV, cov, zt, a0, nR, nz in [(96, 4 * np.pi, 8.0, 0.0, 6, 7), (250, 2.7 * np.pi, 5.0, 0.3, 9, 11),
                                    (64, 2 * np.pi, 0.0, 0.0, 4, 5), (200, 6 * np.pi, 20., 0.1, 12, 30)]:
        G = tr.Geom(nViews=nV, coverage=cov, zTran=zt, angle0=a0)
        Z = np.linspace(-zt / 2 if zt else -2, zt / 2 if zt else 2, nz)
        angs = np.concatenate([np.linspace(0, 2 * np.pi, 30, endpoint=False), G.Views[:5],
                               G.Views[:5] + np.pi, rng.random(10) * 7])
        bat = tr._interpZ_batch(G, Z, angs, nR)
        for i, a in enumerate(angs):
            ref = G.interpZ(Z, a, nR)
            for k in range(8):
                assert np.array_equal(np.asarray(ref[k]), bat[k][i], equal_nan=True), (nV, i, k)


def test_fbp_weights_vs_reference(golden, orc):
    """The pre-weight of vir's fan FBP (processing/reconstruction.py:99-107),
    both detector forms, against the reference's own function."""
    g = golden["fbp_weights"]
    e = orc.cosine_weighting(g["sino"], g["cols_pos"], float(g["src_iso"]), float(g["det_off"]),
                             equispaced=True)
    a = orc.cosine_weighting(g["sino"], g["cols_ang"], float(g["src_iso"]), float(g["det_off"]),
                             equispaced=False)
    assert rel(e, g["equispaced"]) < 1e-15
    assert rel(a, g["equiangular"]) < 1e-15
    # the flat-detector pre-weight of the GPU fan FBP is the equispaced form
    # at the bin centres scaled to the isocentre
    from vir_gb300.reconstruction import fan_preweight
    w = orc.fan_preweight(96, 1.2, 0.3, 500.0, 1000.0)
    assert rel(fan_preweight(96, 1.2, 0.3, 500.0, 1000.0), w) < 1e-15


def test_hsieh_backprojection_vs_reference(golden, orc):
    """The 1/L^2-weighted linear-interpolation pixel backprojection of
    processing/proj2.py:580-616 (clipped indices) against the reference's
    own function; fbp2d_bp and fdk share its interpolation step."""
    g = golden["fbp_hsieh"]
    img = orc.fan_backproject_hsieh(g["sino"], g["views"], g["cols"], float(g["src_iso"]),
                                    tuple(g["dPixels"]), tuple(int(v) for v in g["nPixels"]),
                                    float(g["detOff"]), tuple(g["pixOff"]))
    assert img.shape == g["img"].shape
    assert rel(img, g["img"]) < 1e-13


def test_fbp2d_bp_flat_fan_reduces_to_parallel(orc):
    """The flat-detector fan backprojection tends to the parallel one as the
    source recedes (DSD = DSO -> infinity): U -> 1, s -> p."""
    rng = np.random.default_rng(5)
    q = rng.random((24, 64))
    angs = np.linspace(0, np.pi, 24, endpoint=False)
    par = orc.fbp2d_bp(q, angs, (20, 22), du=1.0, d_pix=1.3)
    fan = orc.fbp2d_bp(q, angs, (20, 22), fan=True, DSO=1e7, DSD=1e7, du=1.0, d_pix=1.3)
    assert rel(fan, par) < 1e-5


def test_fdk_box_equals_full_volume(orc):
    """The oracle FDK over a sub-box (only the rows the box reaches filtered)
    equals the same voxels of the full volume."""
    rng = np.random.default_rng(6)
    sino = rng.random((10, 40, 30)).astype(np.float32)
    angs = np.linspace(0, 2 * np.pi, 10, endpoint=False)
    kw = dict(du=1.1, dv=0.9, su=0.2, sv=-0.3, d_pix=0.8)
    full = orc.fdk(sino, angs, (14, 12, 16), 60.0, 110.0, **kw)
    box = ((3, 9), (2, 7), (5, 13))
    part = orc.fdk(sino, angs, (14, 12, 16), 60.0, 110.0, box=box, **kw)
    assert rel(part, full[3:9, 2:7, 5:13]) < 1e-13


def test_sf_cone_vs_analytic_sphere(golden, orc, sphere_vol):
    """The separable-footprint cone projector (SF-TR, A2 amplitude) of a
    voxelised sphere against vir's detector-area-averaged analytic cone-beam
    projection of the sphere (analytic_sino.py:563, golden fixture): equal
    within the voxelisation error (0.5 mm voxels, radius 7 mm)."""
    g = golden["sphere_cone_vol"]
    vol = sphere_vol(48, 0.5, g["sphere"])
    sf = orc.sf_fp_cone_3d(vol, g["angs"], int(g["nu"]), int(g["nv"]), float(g["DSO"]),
                           float(g["DSD"]), du=float(g["du"]), dv=float(g["dv"]), d_pix=0.5)
    ref = g["proj"]
    assert np.linalg.norm(sf - ref) / np.linalg.norm(ref) < 0.025
    assert abs(sf.sum() / ref.sum() - 1) < 0.005


def test_sf_cone_adjoint(orc):
    rng = np.random.default_rng(8)
    x = rng.random((12, 10, 8))
    y = rng.random((5, 30, 20))
    a = np.linspace(0.3, 6.0, 5)
    kw = dict(du=1.1, dv=0.9, su=0.2, sv=-0.1, d_pix=1.0)
    A = orc.sf_fp_cone_3d(x, a, 30, 20, 40.0, 80.0, **kw)
    B = orc.sf_bp_cone_3d(y, a, x.shape, 40.0, 80.0, **kw)
    assert abs((A * y).sum() - (x * B).sum()) / abs((A * y).sum()) < 1e-12


def _aw_bp_by_chords(orc, sino, angs, shape, fan, DSO, DSD, du, su, d_pix):
    """The gather form of the 2D Amanatides-Woo back projection, restated in
    FP64: every ray adds s times its chord through each pixel, the overlap of
    its parameter intervals between the pixel's x planes and its y planes
    (t_k = (lo + k d - o) / h), clipped to the ray's [t_entry, t_exit]; a ray
    within 1e-6 of an axis stays in the row or column it enters (rd.py's
    walk set-up, rd.py:52-109, with the axis-parallel ray clipped to its slab)."""
    f = lambda v: float(np.float32(v))
    du, su, d_pix, DSO, DSD = f(du), f(su), f(d_pix), f(DSO), f(DSD)
    c, s = orc.trig(angs, np.float32)
    nx, ny = shape
    na, nu = sino.shape
    n = (nx, ny)
    lo = [-d_pix * k / 2.0 for k in n]
    hi = [d_pix * k / 2.0 for k in n]
    out = np.zeros(shape)
    for ia in range(na):
        for iu in range(nu):
            u = du * (iu - (nu / 2.0 - 0.5) + su)
            if fan:
                o = np.array([DSO * c[ia], DSO * s[ia]])
                v = np.array([-(DSD - DSO) * c[ia] - u * s[ia] - o[0],
                              -(DSD - DSO) * s[ia] + u * c[ia] - o[1]])
                h = v / np.sqrt(v @ v)
            else:
                o = np.array([-u * s[ia], u * c[ia]])
                h = np.array([c[ia], s[ia]])
            te, tx = -np.inf, np.inf
            for a in range(2):
                if abs(h[a]) > 1e-6:
                    t0, t1 = sorted(((lo[a] - o[a]) / h[a], (hi[a] - o[a]) / h[a]))
                elif lo[a] <= o[a] < hi[a]:
                    t0, t1 = -np.inf, np.inf
                else:
                    t0, t1 = np.inf, -np.inf
                te, tx = max(te, t0), min(tx, t1)
            if not tx > te:
                continue
            iv = []
            for a in range(2):
                if abs(h[a]) > 1e-6:
                    tp = (lo[a] + np.arange(n[a] + 1) * d_pix - o[a]) / h[a]
                    iv.append((np.minimum(tp[:-1], tp[1:]), np.maximum(tp[:-1], tp[1:])))
                else:
                    r = min(max(o[a] + te * h[a], lo[a] + 1e-6), hi[a] - 1e-6)
                    ir = min(max(int(np.floor((r - lo[a]) / d_pix)), 0), n[a] - 1)
                    on = np.arange(n[a]) == ir
                    iv.append((np.where(on, -np.inf, np.inf), np.where(on, np.inf, -np.inf)))
            (ax, bx), (ay, by) = iv
            ch = (np.minimum(np.minimum(bx[:, None], by[None, :]), tx)
                  - np.maximum(np.maximum(ax[:, None], ay[None, :]), te))
            out += float(sino[ia, iu]) * np.maximum(ch, 0.0)
    return out / na / d_pix / d_pix * du


@pytest.mark.parametrize("fan", [False, True])
def test_aw_bp_chords_equal_the_walk(orc, fan):
    """The chord formulation of the GPU's gather-form AW back projection
    equals the FP64 walk's segment sums (to the walk's own rounding), also
    for rays along pixel boundaries at 0, 45 and 90 degrees and with a
    shifted detector."""
    rng = np.random.default_rng(61)
    for shape, na, nu, du, su in (((24, 18), 8, 41, 1.0, 0.0), ((17, 23), 6, 37, 0.7, 1.3)):
        angs = np.linspace(0, 2 * np.pi if fan else np.pi, na, endpoint=False)
        y = rng.random((na, nu)).astype(np.float32)
        geo = (40.0, 90.0) if fan else (0.0, 0.0)
        walk = (orc.aw_bp_fan_2d(y, angs, shape, *geo, du=du, su=su, d_pix=1.0) if fan
                else orc.aw_bp_par_2d(y, angs, shape, du=du, su=su, d_pix=1.0))
        ch = _aw_bp_by_chords(orc, y, angs, shape, fan, *geo, du, su, 1.0)
        assert rel(ch, walk) < 1e-12
