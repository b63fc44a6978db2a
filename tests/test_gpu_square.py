"""GPU distance-driven pair of the translational square geometry
(dd_fp_square / dd_bp_square) and its SIRT (sirt_dd.sirt) against the
reference's golden vectors and the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SQ_GEO = ("du", "dv", "dsrc_p", "dsrc_z", "su", "sv", "ssrc_p", "ssrc_z", "d_pix")

# the geometry of the reference's own SIRT script (sirt_dd.py:81-138)
SCRIPT = dict(n=64, nz=64, nu=129, nv=64, nsrc_p=96, nsrc_z=10, DSO=40.0, DSD=72.0,
              kw=dict(du=1.0, dv=1.0, dsrc_p=0.5, dsrc_z=0.5, su=0.0, sv=32.0, ssrc_p=0.0,
                      ssrc_z=-27.0, d_pix=1.0))


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def fscale(kw):
    f = lambda v: float(np.float32(v))
    return f(kw["d_pix"]) ** 2 / (f(kw["du"]) * f(kw["dv"]))


@pytest.mark.parametrize("case", ["square_a", "square_b"])
def test_square_golden(vg, golden, case):
    from vir_gb300.sys_mat import dd
    g = golden[case]
    kw = {k: float(g[k]) for k in SQ_GEO}
    fp = dd.dd_fp_square(g["vol"], int(g["nu"]), int(g["nv"]), int(g["nsrc_p"]),
                         int(g["nsrc_z"]), float(g["DSO"]), float(g["DSD"]), **kw)
    assert fp.shape == g["sino"].shape and fp.dtype == np.float32
    assert rel(fp, g["sino"]) < 2e-5
    bp = dd.dd_bp_square(g["y"], g["vol"].shape, float(g["DSO"]), float(g["DSD"]), **kw)
    assert bp.shape == g["bp"].shape
    assert rel(bp, g["bp"]) < 2e-5


@pytest.mark.parametrize("shape,det,src", [((40, 40, 28), (72, 50), (7, 4)),
                                           ((33, 33, 17), (45, 31), (5, 3))])
def test_square_vs_oracle_and_adjoint(vg, orc, shape, det, src):
    from vir_gb300.sys_mat import dd
    rng = np.random.default_rng(7)
    vol = rng.random(shape).astype(np.float32)
    kw = dict(du=0.9, dv=1.1, dsrc_p=1.3, dsrc_z=0.8, su=0.4, sv=9.0, ssrc_p=-0.6, ssrc_z=-6.0,
              d_pix=0.75)
    args = (*det, *src, 45.0, 80.0)
    fp = dd.dd_fp_square(vol, *args, **kw)
    fo = orc.dd_fp_square(vol, *args, **kw)
    assert rel(fp, fo) < 2e-5
    y = rng.random(fp.shape).astype(np.float32)
    bp = dd.dd_bp_square(y, shape, 45.0, 80.0, **kw)
    bo = orc.dd_bp_square(y, shape, 45.0, 80.0, **kw)
    assert rel(bp, bo) < 2e-5
    lhs = (fp.astype(np.float64) * y).sum()
    rhs = (vol.astype(np.float64) * bp).sum() * fscale(kw)
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_square_rejects_rectangular(vg):
    from vir_gb300.sys_mat import dd
    with pytest.raises(ValueError, match="nx must equal ny"):
        dd.dd_fp_square(np.zeros((8, 9, 4), np.float32), 10, 10, 2, 2, 20.0, 36.0)
    with pytest.raises(ValueError, match="nx must equal ny"):
        dd.dd_bp_square(np.zeros((2, 2, 10, 10, 4), np.float32), (8, 9, 4), 20.0, 36.0)


def test_sirt_square_golden(vg, golden):
    """vir_gb300.sys_mat.sirt_dd.sirt against the reference's own sirt
    (sirt_dd.py:37-76) run on its own projectors."""
    from vir_gb300.sys_mat import sirt_dd
    g = golden["sirt_square"]
    gem = tuple(float(v) for v in g["gem_prms"])
    nx, ny, nz, d_pix = g["img_prms"]
    img = (int(nx), int(ny), int(nz), float(d_pix))
    sp = g["src_prms"]
    src = (int(sp[0]), int(sp[1]), *(float(v) for v in sp[2:]))
    dp = g["det_prms"]
    det = (int(dp[0]), int(dp[1]), *(float(v) for v in dp[2:]))
    srt = (float(g["srt_prms"][0]), int(g["srt_prms"][1]))
    x = sirt_dd.sirt(g["sino"], g["W_sino"], g["W_img"], gem, img, src, det, srt)
    assert x.dtype == np.float32 and x.shape == g["x"].shape
    assert rel(x, g["x"]) < 1e-4


def test_sirt_square_vs_oracle(vg, orc):
    """Four SIRT updates on a 24^3 problem against the FP64 oracle's rule."""
    import torch
    from vir_gb300.sys_mat import dd, sirt_dd
    n, nz, nu, nv, nsp, nsz = 24, 24, 49, 30, 12, 4
    kw = dict(du=1.0, dv=1.0, dsrc_p=0.5, dsrc_z=0.5, su=0.0, sv=12.0, ssrc_p=0.0,
              ssrc_z=-10.0, d_pix=1.0)
    DSO, DSD = 16.0, 28.0
    vol = np.zeros((n, n, nz), np.float32)
    vol[8:16, 9:15, 6:18] = 1.0
    sino = orc.dd_fp_square(vol, nu, nv, nsp, nsz, DSO, DSD, **kw).astype(np.float32)
    W_sino = dd.dd_fp_square(np.ones(vol.shape, np.float32), nu, nv, nsp, nsz, DSO, DSD, **kw)
    W_img = dd.dd_bp_square(np.ones(sino.shape, np.float32), vol.shape, DSO, DSD, **kw)
    prms = ((DSO, DSD), (n, n, nz, kw["d_pix"]),
            (nsp, nsz, kw["dsrc_p"], kw["dsrc_z"], kw["ssrc_p"], kw["ssrc_z"]),
            (nu, nv, kw["du"], kw["dv"], kw["su"], kw["sv"]), (1.0, 5))
    x = sirt_dd.sirt(sino, W_sino, W_img, *prms)
    fp = lambda z: orc.dd_fp_square(z, nu, nv, nsp, nsz, DSO, DSD, **kw)
    bp = lambda s: orc.dd_bp_square(s, vol.shape, DSO, DSD, **kw)
    xo = orc.sirt(sino, fp, bp, vol.shape, gamma=1.0, iters=5)
    assert rel(x, xo) < 1e-4
    # CUDA tensors in -> CUDA tensor out, same values
    xt = sirt_dd.sirt(torch.from_numpy(sino).cuda(), torch.from_numpy(W_sino).cuda(),
                      torch.from_numpy(W_img).cuda(), *prms)
    assert xt.is_cuda and np.array_equal(xt.cpu().numpy(), x)


def test_square_script_size_properties(vg):
    """The reference script's geometry (64^3, 96 x 10 sources, 129 x 64
    cells): the pair is an adjoint to FP32 accuracy, and SIRT on the script's
    cube phantom lowers the data residual at every update."""
    import torch
    from vir_gb300.sys_mat import dd, sirt_dd
    S = SCRIPT
    kw = S["kw"]
    args = (S["nu"], S["nv"], S["nsrc_p"], S["nsrc_z"], S["DSO"], S["DSD"])
    shape = (S["n"], S["n"], S["nz"])
    gen = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand(shape, device="cuda", generator=gen)
    y = torch.rand((S["nsrc_p"], S["nsrc_z"], S["nv"], S["nu"], 4), device="cuda", generator=gen)
    A = dd.dd_fp_square(x, *args, **kw)
    B = dd.dd_bp_square(y, shape, S["DSO"], S["DSD"], **kw)
    lhs = (A.double() * y.double()).sum().item()
    rhs = (x.double() * B.double()).sum().item() * fscale(kw)
    assert abs(lhs - rhs) / lhs < 1e-5
    vol = torch.zeros(shape, device="cuda")
    vol[24:40, 24:40, 24:40] = 1.0  # sirt_dd.py:85-86
    sino = dd.dd_fp_square(vol, *args, **kw)
    W_sino = dd.dd_fp_square(torch.ones(shape, device="cuda"), *args, **kw)
    W_img = dd.dd_bp_square(torch.ones_like(sino), shape, S["DSO"], S["DSD"], **kw)
    prms = ((S["DSO"], S["DSD"]), (S["n"], S["n"], S["nz"], kw["d_pix"]),
            (S["nsrc_p"], S["nsrc_z"], kw["dsrc_p"], kw["dsrc_z"], kw["ssrc_p"], kw["ssrc_z"]),
            (S["nu"], S["nv"], kw["du"], kw["dv"], kw["su"], kw["sv"]))
    res = []
    for it in (2, 4, 8):
        xk = sirt_dd.sirt(sino, W_sino, W_img, *prms, (1.0, it))
        res.append(float((dd.dd_fp_square(xk, *args, **kw) - sino).norm()))
    assert res[0] > res[1] > res[2], res
