"""GPU parity: the CUDA kernels (through the C ABI) against the FP64 oracle
and the reference's golden vectors.  Tolerances are stated per test."""
import numpy as np
import pytest

from vir_gb300 import phantoms as ph

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


# --- Siddon 2D ---------------------------------------------------------------

@pytest.mark.parametrize("case", ["siddon2d_a", "siddon2d_b"])
def test_siddon_fp_golden(vg, golden, case):
    from vir_gb300.sys_mat import fp_2d_par
    g = golden[case]
    out = fp_2d_par.siddons_fp_2d(g["img"], g["angs"], int(g["n_dets"]), float(g["d_det"]),
                                  float(g["d_pix"]))
    assert out.dtype == np.float32 and out.shape == g["sino"].shape
    # FP32 Kahan sum vs the reference's float32-rounded sum: ~1 ulp per term
    assert rel(out, g["sino"]) < 2e-6


def test_siddon_c1_voxel_sequences(vg, orc):
    """Config C1 geometry (256^2, 180 views over pi, 367 bins at 1 mm): every
    ray visits the same voxels, in the same order, with the same FP64
    lengths as the FP64 restatement of fp_2d_par.py."""
    import torch
    from vir_gb300 import _core
    from vir_gb300._lib import call
    angs = np.linspace(0, np.pi, 180, endpoint=False)
    cnt_o, h_o, len_o = orc.siddons_trace_2d((256, 256), angs, 367, 1.0, 1.0)
    dev = torch.device("cuda")
    trig = _core.trig_cache.get(angs, None, dev)
    cnt = torch.empty((180, 367), dtype=torch.int32, device=dev)
    h = torch.empty((180, 367), dtype=torch.int64, device=dev)
    ln = torch.empty((180, 367), dtype=torch.float64, device=dev)
    call("vg_siddon2d_trace", 256, 256, _core.ptr(trig), 180, 367, 1.0, 1.0, _core.ptr(cnt),
         _core.ptr(h), _core.ptr(ln), _core.stream(dev))
    torch.cuda.synchronize()
    assert np.array_equal(cnt.cpu().numpy(), cnt_o)
    assert np.array_equal(h.cpu().numpy().view(np.uint64), h_o)
    # lengths are the same FP64 numbers summed in the same order
    assert np.array_equal(ln.cpu().numpy(), len_o)
    assert int(cnt_o.sum()) == orc.siddons_count_2d((256, 256), angs, 367)


def test_siddon_division_correctly_rounded(vg):
    """The Siddon kernels' FP64 quotients (reciprocal plus one FMA correction)
    equal the correctly rounded quotients bit for bit: on the plane-crossing
    operands of the C1 geometry (every view and ray, every 4th plane of each
    axis, as the kernels form them) and on 2 M random operands spanning 1e-10
    to 1e10 over 1e-17 to 1e3."""
    import torch
    from vir_gb300 import _core
    from vir_gb300._lib import call
    dev = torch.device("cuda")
    angs = np.linspace(0, np.pi, 180, endpoint=False)
    trig = _core.trig_cache.get(angs, None, dev).cpu().numpy().reshape(-1, 2)
    n, n_dets, d_det, d_pix = 256, 367, 1.0, 1.0
    k = np.arange(n_dets, dtype=np.float64)
    det = d_det * ((k - n_dets * 0.5) + 0.5)
    edges = d_pix * (np.arange(0, n + 1, 4, dtype=np.float64) - n * 0.5)
    A, B = [], []
    for dx, dy in trig:
        x0, y0 = det * -dy, det * dx
        if dx != 0.0:
            A.append((edges[None, :] - x0[:, None]).ravel()); B.append(np.full(A[-1].size, dx))
        if dy != 0.0:
            A.append((edges[None, :] - y0[:, None]).ravel()); B.append(np.full(A[-1].size, dy))
    rng = np.random.default_rng(41)
    m = 2_000_000
    A.append(rng.choice([-1.0, 1.0], m) * 10.0 ** rng.uniform(-10, 10, m))
    B.append(rng.choice([-1.0, 1.0], m) * 10.0 ** rng.uniform(-17, 3, m))
    a, b = np.concatenate(A), np.concatenate(B)
    ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    q = torch.empty_like(ta)
    call("vg_div_rn_check", _core.ptr(ta), _core.ptr(tb), a.size, _core.ptr(q), _core.stream(dev))
    torch.cuda.synchronize()
    ref = a / b
    bad = np.flatnonzero(q.cpu().numpy().view(np.uint64) != ref.view(np.uint64))
    assert bad.size == 0, (bad.size, a[bad[:3]], b[bad[:3]])


@pytest.mark.parametrize("shape,n_dets,d_det,d_pix,na,span", [
    ((256, 256), 367, 1.0, 1.0, 180, np.pi),     # config C1
    ((40, 33), 61, 0.7, 1.3, 37, 2 * np.pi),     # ragged, non power-of-two pitch
    ((1, 17), 5, 1.0, 1.0, 8, np.pi),             # degenerate image
])
def test_siddon_fp_bp_vs_oracle(vg, orc, shape, n_dets, d_det, d_pix, na, span):
    from vir_gb300.sys_mat import fp_2d_par
    rng = np.random.default_rng(7)
    img = rng.random(shape).astype(np.float32)
    angs = np.linspace(0, span, na, endpoint=False)
    fp = fp_2d_par.siddons_fp_2d(img, angs, n_dets, d_det, d_pix)
    fo = orc.siddons_fp_2d(img, angs, n_dets, d_det, d_pix)
    assert rel(fp, fo) < 2e-6
    y = rng.random(fp.shape).astype(np.float32)
    bo = orc.siddons_bp_2d(y, angs, shape, d_det, d_pix)
    for method in ("scatter", "gather"):
        bp = fp_2d_par.siddons_bp_2d(y, angs, shape, d_det, d_pix, method=method)
        assert rel(bp, bo) < 2e-6, method
        # adjoint (dot-product) test of the GPU pair
        lhs = (fp.astype(np.float64) * y).sum()
        rhs = (img.astype(np.float64) * bp).sum()
        assert abs(lhs - rhs) / abs(lhs) < 1e-6, method


# --- distance-driven 2D ---------------------------------------------------------

@pytest.mark.parametrize("case", ["dd_par_a", "dd_par_b"])
def test_dd_par_golden(vg, golden, case):
    from vir_gb300.sys_mat import dd
    g = golden[case]
    fp = dd.dd_fp_par_2d(g["img"], g["angs"], int(g["nu"]), float(g["du"]), float(g["su"]),
                         float(g["d_pix"]))
    assert rel(fp, g["sino"]) < 5e-5
    bp = dd.dd_bp_par_2d(g["y"], g["angs"], g["img"].shape, float(g["du"]), float(g["su"]),
                         float(g["d_pix"]))
    assert rel(bp, g["bp"]) < 5e-5


@pytest.mark.parametrize("case", ["dd_fan_a", "dd_fan_b"])
def test_dd_fan_golden(vg, golden, case):
    from vir_gb300.sys_mat import dd
    g = golden[case]
    a = (float(g["DSO"]), float(g["DSD"]), float(g["du"]), float(g["su"]), float(g["d_pix"]))
    fp = dd.dd_fp_fan_2d(g["img"], g["angs"], int(g["nu"]), *a)
    assert rel(fp, g["sino"]) < 5e-5
    bp = dd.dd_bp_fan_2d(g["y"], g["angs"], g["img"].shape, *a)
    assert rel(bp, g["bp"]) < 5e-5


@pytest.mark.parametrize("fan", [0, 1])
def test_dd_c2_vs_oracle(vg, orc, fan):
    """Config C2 sizes (512^2, 720 views, 768 bins of 1.2 mm, DSO 500, DSD
    1000, d_pix 0.9): FP and BP against the FP64 oracle."""
    from vir_gb300.sys_mat import dd
    img, _ = ph.ellipse_phantom(512, 10, seed=2, d_pix=0.9)
    angs = np.linspace(0, 2 * np.pi, 720, endpoint=False)
    y = np.random.default_rng(8).random((720, 768)).astype(np.float32)
    if fan:
        fp = dd.dd_fp_fan_2d(img, angs, 768, 500.0, 1000.0, du=1.2, d_pix=0.9)
        fo = orc.dd_fp_fan_2d(img, angs, 768, 500.0, 1000.0, du=1.2, d_pix=0.9)
        bp = dd.dd_bp_fan_2d(y, angs, img.shape, 500.0, 1000.0, du=1.2, d_pix=0.9)
        bo = orc.dd_bp_fan_2d(y, angs, img.shape, 500.0, 1000.0, du=1.2, d_pix=0.9)
    else:
        fp = dd.dd_fp_par_2d(img, angs, 768, du=1.2, d_pix=0.9)
        fo = orc.dd_fp_par_2d(img, angs, 768, du=1.2, d_pix=0.9)
        bp = dd.dd_bp_par_2d(y, angs, img.shape, du=1.2, d_pix=0.9)
        bo = orc.dd_bp_par_2d(y, angs, img.shape, du=1.2, d_pix=0.9)
    # FP32 geometry (as the reference) against FP64: max error relative to the peak
    assert rel(fp, fo) < 1e-4
    assert rel(bp, bo) < 1e-4
    assert np.sqrt(np.mean((fp - fo) ** 2)) / np.abs(fo).max() < 1e-5


def test_dd_adjoint_gpu(vg):
    from vir_gb300.sys_mat import dd
    rng = np.random.default_rng(9)
    x = rng.random((96, 80)).astype(np.float32)
    angs = np.linspace(0, 2 * np.pi, 90, endpoint=False)
    y = rng.random((90, 150)).astype(np.float32)
    A = dd.dd_fp_fan_2d(x, angs, 150, 120.0, 240.0, du=0.9, d_pix=1.1)
    B = dd.dd_bp_fan_2d(y, angs, x.shape, 120.0, 240.0, du=0.9, d_pix=1.1)
    d, u = float(np.float32(1.1)), float(np.float32(0.9))
    lhs = (A.astype(np.float64) * y).sum()
    rhs = (x.astype(np.float64) * B).sum() * 90 * d * d / u
    assert abs(lhs - rhs) / lhs < 1e-5


def test_dd_torch_in_torch_out(vg):
    import torch
    from vir_gb300.sys_mat import dd
    x = torch.rand(64, 64, device="cuda")
    angs = np.linspace(0, np.pi, 30, endpoint=False)
    s = dd.dd_fp_par_2d(x, angs, 96)
    assert isinstance(s, torch.Tensor) and s.is_cuda and s.shape == (30, 96)
    s2 = dd.dd_fp_par_2d(x.cpu().numpy(), angs, 96)
    assert np.array_equal(s.cpu().numpy(), s2)


def test_errors_are_loud(vg):
    from vir_gb300 import VirGpuError
    from vir_gb300.sys_mat import dd
    with pytest.raises(VirGpuError):
        dd.dd_fp_fan_2d(np.ones((64, 64), np.float32), np.zeros(3), 10, 10.0, 20.0)  # image wider than DSO
    with pytest.raises(ValueError):
        dd.dd_bp_par_2d(np.ones((3, 10), np.float32), np.zeros(4), (8, 8))


def test_deterministic(vg):
    from vir_gb300.sys_mat import dd
    img, _ = ph.ellipse_phantom(128, 6, seed=3)
    angs = np.linspace(0, np.pi, 60, endpoint=False)
    a = dd.dd_bp_par_2d(dd.dd_fp_par_2d(img, angs, 200), angs, img.shape)
    b = dd.dd_bp_par_2d(dd.dd_fp_par_2d(img, angs, 200), angs, img.shape)
    assert np.array_equal(a, b)


# --- filter / FBP / SIRT -------------------------------------------------------

def test_filter_golden(vg, golden):
    from vir_gb300 import filtration
    for case in golden.cases:
        if not case.startswith("filter_"):
            continue
        g = golden[case]
        out = filtration.filter_sino(g["sino"], du=float(g["du"]),
                                     filter_type=str(g["filter_type"]),
                                     cutoff=float(g["cutoff"]), real_space=bool(g["real_space"]))
        ref = g["filtered"]
        assert np.abs(out - ref).max() < 2e-6 * np.abs(ref).max() + 1e-6, case


def test_filter_fft_route(vg, golden, orc):
    """The FFT route (shared-memory rFFT per row, used from 256 bins on)
    against the reference's outputs, the FP64 oracle at the C4 detector width
    (1024 bins, z = 2048) and at 300 bins (z = 1024), and the direct
    convolution with a row weight."""
    import torch
    from vir_gb300 import filtration
    for case in golden.cases:
        if not case.startswith("filter_"):
            continue
        g = golden[case]
        x = torch.from_numpy(g["sino"].astype(np.float32)).cuda()
        out = filtration.filter_rows_device(x, float(g["du"]), str(g["filter_type"]),
                                            float(g["cutoff"]), bool(g["real_space"]),
                                            method="fft").cpu().numpy()
        ref = g["filtered"]
        assert np.abs(out - ref).max() < 2e-6 * np.abs(ref).max() + 1e-6, case
    rng = np.random.default_rng(30)
    for nu, ftype in ((1024, "ramp"), (300, "hann")):
        sino = rng.random((64, nu)).astype(np.float32)
        got = filtration.filter_sino(sino, du=0.8, filter_type=ftype, cutoff=0.5)
        ref = orc.filter_sino(sino, du=0.8, filter_type=ftype, cutoff=0.5)
        assert np.abs(got - ref).max() < 2e-6 * np.abs(ref).max(), (nu, ftype)
        w = torch.from_numpy(rng.random(nu).astype(np.float32)).cuda()
        xs = torch.from_numpy(sino).cuda()
        a = filtration.filter_rows_device(xs, 0.8, ftype, 0.5, row_weight=w, method="fft")
        b = filtration.filter_rows_device(xs, 0.8, ftype, 0.5, row_weight=w, method="direct")
        assert (a - b).abs().max().item() < 2e-6 * b.abs().max().item(), (nu, ftype)


@pytest.mark.parametrize("geom", ["par", "fan"])
def test_fbp_disc(vg, geom):
    """FBP of exact line integrals of one uniform disc reconstructs its value
    (1.0) inside and 0 outside."""
    from vir_gb300 import reconstruction as rc
    e = ph.Ellipses(*(np.array([v]) for v in (10.0, -20.0, 60.0, 60.0, 0.0, 1.0)))
    n, d_pix = 256, 1.0
    if geom == "par":
        angs = np.linspace(0, np.pi, 360, endpoint=False)
        y = ph.sino_par(e, angs, 400, du=1.0)
        rec = rc.fbp_2d(y.astype(np.float32), angs, (n, n), du=1.0, d_pix=d_pix)
    else:
        angs = np.linspace(0, 2 * np.pi, 720, endpoint=False)
        y = ph.sino_fan(e, angs, 600, 300.0, 600.0, du=1.2)
        rec = rc.fbp_2d(y.astype(np.float32), angs, (n, n), geom="fan", DSO=300.0, DSD=600.0,
                        du=1.2, d_pix=d_pix)
    c = (np.arange(n) + 0.5 - n / 2) * d_pix
    X, Y = np.meshgrid(c, c, indexing="ij")
    r = np.hypot(X - 10.0, Y + 20.0)
    inside = rec[r < 50].mean()
    outside = np.abs(rec[(r > 70) & (np.hypot(X, Y) < 110)]).mean()
    assert abs(inside - 1.0) < 0.01, inside
    assert outside < 0.01, outside


def test_sirt_golden(vg, golden):
    from vir_gb300 import reconstruction as rc
    g = golden["sirt_par"]
    x = rc.sirt_2d(g["sino"], g["angs"], g["img"].shape, geom="par", iters=int(g["iters"]),
                   gamma=float(g["gamma"]))
    assert rel(x, g["x"]) < 1e-4


@pytest.mark.parametrize("geom", ["par", "fan"])
def test_sirt_vs_oracle(vg, orc, geom):
    from vir_gb300 import reconstruction as rc
    img, _ = ph.ellipse_phantom(96, 8, seed=4, d_pix=1.0)
    angs = np.linspace(0, 2 * np.pi, 120, endpoint=False)
    kw = dict(DSO=150.0, DSD=300.0, du=1.5) if geom == "fan" else dict(du=1.0)
    if geom == "fan":
        fp = lambda x: orc.dd_fp_fan_2d(x, angs, 160, 150.0, 300.0, du=1.5)
        bp = lambda s: orc.dd_bp_fan_2d(s, angs, img.shape, 150.0, 300.0, du=1.5)
    else:
        fp = lambda x: orc.dd_fp_par_2d(x, angs, 160, du=1.0)
        bp = lambda s: orc.dd_bp_par_2d(s, angs, img.shape, du=1.0)
    y = fp(img).astype(np.float32)
    xo = orc.sirt(y, fp, bp, img.shape, iters=11)
    for graph in (False, True):
        x = rc.sirt_2d(y, angs, img.shape, geom=geom, iters=11, graph=graph, **kw)
        assert rel(x, xo) < 2e-4
        # equal final RMSE against the phantom within 1e-4 relative
        r_gpu = np.sqrt(np.mean((x - img) ** 2))
        r_orc = np.sqrt(np.mean((xo - img) ** 2))
        assert abs(r_gpu - r_orc) / r_orc < 1e-4


@pytest.mark.parametrize("fan", [False, True])
@pytest.mark.parametrize("shape,nu,na,su", [
    ((37, 53), 71, 1, 0.3),      # ragged image, a single view
    ((1, 29), 40, 9, -0.5),      # one-pixel-wide image
    ((64, 64), 24, 12, 2.0),     # detector narrower than the image, shifted
    ((48, 40), 700, 7, 0.0),     # detector much wider than the image
])
def test_dd_edge_cases_vs_oracle(vg, orc, fan, shape, nu, na, su):
    from vir_gb300.sys_mat import dd
    rng = np.random.default_rng(11)
    img = rng.random(shape).astype(np.float32)
    angs = np.linspace(0.1, 0.1 + 2 * np.pi, na, endpoint=False)
    y = rng.random((na, nu)).astype(np.float32)
    kw = dict(du=0.9, su=su, d_pix=1.1)
    if fan:
        geo = (120.0, 240.0)
        fp, fo = dd.dd_fp_fan_2d(img, angs, nu, *geo, **kw), orc.dd_fp_fan_2d(img, angs, nu, *geo, **kw)
        bp = dd.dd_bp_fan_2d(y, angs, shape, *geo, **kw)
        bo = orc.dd_bp_fan_2d(y, angs, shape, *geo, **kw)
    else:
        fp, fo = dd.dd_fp_par_2d(img, angs, nu, **kw), orc.dd_fp_par_2d(img, angs, nu, **kw)
        bp, bo = dd.dd_bp_par_2d(y, angs, shape, **kw), orc.dd_bp_par_2d(y, angs, shape, **kw)
    assert fp.shape == (na, nu) and bp.shape == shape
    assert rel(fp, fo) < 1e-4
    assert rel(bp, bo) < 1e-4


def test_zero_and_empty_inputs(vg):
    """Zero images project to zero; an object outside every ray gives zeros;
    no views is an argument error, not a silent empty result."""
    from vir_gb300 import VirGpuError
    from vir_gb300.sys_mat import dd, fp_2d_par
    angs = np.linspace(0, np.pi, 8, endpoint=False)
    assert not np.any(dd.dd_fp_par_2d(np.zeros((16, 16), np.float32), angs, 20))
    assert not np.any(fp_2d_par.siddons_fp_2d(np.zeros((16, 16), np.float32), angs, 20))
    # detector far off to the side: no overlap anywhere
    assert not np.any(dd.dd_fp_par_2d(np.ones((16, 16), np.float32), angs, 10, su=100.0))
    with pytest.raises((VirGpuError, ValueError)):
        dd.dd_fp_par_2d(np.ones((16, 16), np.float32), np.zeros(0), 20)


@pytest.mark.parametrize("fan", [False, True])
def test_dd_fp_every_tile_variant_vs_oracle(vg, orc, fan):
    """Each forward-projector tile variant (warps x bins per lane, selected
    through vg_dd2d_geom.variant) on an odd 131 x 131 image with 200 bins:
    one block per view for the wide tiles, two for the 192-bin tile, rows
    whose length is not a multiple of the 8-pixel lane segments."""
    import torch
    from vir_gb300 import _lib
    from vir_gb300.reconstruction import SIRT2D
    rng = np.random.default_rng(31)
    img = rng.random((131, 131)).astype(np.float32)
    angs = np.linspace(0.05, 0.05 + 2 * np.pi, 12, endpoint=False)
    kw = dict(du=1.3, su=0.4, d_pix=1.0)
    if fan:
        geo = dict(geom="fan", DSO=200.0, DSD=400.0)
        fo = orc.dd_fp_fan_2d(img, angs, 200, 200.0, 400.0, **kw)
    else:
        geo = dict(geom="par")
        fo = orc.dd_fp_par_2d(img, angs, 200, **kw)
    s = SIRT2D(np.zeros((12, 200), np.float32), angs, img.shape, **geo, **kw)
    x = torch.from_numpy(img).cuda()
    for v in range(1, _lib.load().vg_dd2d_fp_variants() + 1):
        s.g.variant = v
        fp = s.fp(x).cpu().numpy()
        assert rel(fp, fo) < 1e-4, v


def test_sirt_2d_reuses_prepared_state(vg):
    """sirt_2d keeps a geometry's prepared state (weights, buffers, update
    graph): calls with different sinograms (numpy, then a pinned CPU tensor),
    alternating, give bit for bit the iterates of fresh states, and a new
    update count is captured anew."""
    import torch
    from vir_gb300 import reconstruction as rc
    rng = np.random.default_rng(51)
    angs = np.linspace(0, 2 * np.pi, 60, endpoint=False)
    geo = dict(geom="fan", DSO=150.0, DSD=300.0, du=1.5, d_pix=1.0)
    y1 = rng.random((60, 140)).astype(np.float32)
    y2 = rng.random((60, 140)).astype(np.float32)

    def fresh(y, iters):
        s = rc.SIRT2D(y, angs, (96, 96), **geo)
        return s.run(iters - 1).cpu().numpy()

    rc.prepared_sirt.clear()
    a1 = rc.sirt_2d(y1, angs, (96, 96), iters=6, **geo)
    a2 = rc.sirt_2d(torch.from_numpy(y2).pin_memory(), angs, (96, 96), iters=6, **geo)
    a1b = rc.sirt_2d(y1, angs, (96, 96), iters=6, **geo)
    a2c = rc.sirt_2d(y2, angs, (96, 96), iters=9, **geo)
    assert np.array_equal(a1, fresh(y1, 6)) and np.array_equal(a1b, a1)
    assert np.array_equal(np.asarray(a2), fresh(y2, 6))
    assert np.array_equal(a2c, fresh(y2, 9))


def test_sirt_resumes_from_an_iterate(vg):
    """x0 may be an iterate to resume from (the ``initial`` image of
    processing/SIRT/sirt.py:15-29): 2 updates, then 3 more started from their
    iterate, give bit for bit the iterate of 5 updates, on the fan pair and
    on the cone pair."""
    from vir_gb300 import reconstruction as rc
    rng = np.random.default_rng(71)
    angs = np.linspace(0, 2 * np.pi, 60, endpoint=False)
    geo = dict(geom="fan", DSO=150.0, DSD=300.0, du=1.5, d_pix=1.0)
    y = rng.random((60, 140)).astype(np.float32)
    x5 = rc.sirt_2d(y, angs, (96, 96), iters=6, **geo)
    x2 = rc.sirt_2d(y, angs, (96, 96), iters=3, **geo)
    assert np.array_equal(rc.sirt_2d(y, angs, (96, 96), iters=4, x0=x2, **geo), x5)
    a3 = np.linspace(0, 2 * np.pi, 24, endpoint=False)
    y3 = rng.random((24, 24, 20)).astype(np.float32)
    kw = dict(du=1.4, dv=1.4, d_pix=1.0)
    v5 = rc.sirt_3d(y3, a3, (16, 16, 12), 40.0, 80.0, iters=6, **kw)
    v2 = rc.sirt_3d(y3, a3, (16, 16, 12), 40.0, 80.0, iters=3, **kw)
    assert np.array_equal(rc.sirt_3d(y3, a3, (16, 16, 12), 40.0, 80.0, iters=4, x0=v2, **kw), v5)
