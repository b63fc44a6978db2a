"""GPU separable-footprint (2D fan, 2D parallel rectangle) and cone-beam DD
projectors against the reference's golden vectors and the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def dot_rel(A, y, x, B, scale=1.0):
    lhs = (np.asarray(A, np.float64) * y).sum()
    rhs = (np.asarray(x, np.float64) * B).sum() * scale
    return abs(lhs - rhs) / abs(lhs)


# --- separable footprint ------------------------------------------------------

def test_sf_fan_golden(vg, golden):
    from vir_gb300.sys_mat import sp
    g = golden["sf_fan"]
    out = sp.sf_fp_fan_2d(g["img"], g["angs"], int(g["nu"]), float(g["DSO"]), float(g["DSD"]),
                          float(g["du"]), float(g["d_pix"]))
    # FP32 footprint argument vs the reference's FP64 numpy
    assert rel(out, g["sino"]) < 1e-4


def test_sf_fan_vs_oracle_and_adjoint(vg, orc):
    from vir_gb300.sys_mat import sp
    from vir_gb300 import phantoms as ph
    img, _ = ph.ellipse_phantom(128, 6, seed=5, d_pix=1.0, vmax=1.0)
    angs = np.linspace(0, 2 * np.pi, 90, endpoint=False)
    fp = sp.sf_fp_fan_2d(img, angs, 200, 200.0, 400.0, du=1.3, d_pix=1.0)
    fo = orc.sf_fp_fan_2d(img, angs, 200, 200.0, 400.0, du=1.3, d_pix=1.0)
    assert rel(fp, fo) < 1e-4
    y = np.random.default_rng(1).random(fp.shape).astype(np.float32)
    bp = sp.sf_bp_fan_2d(y, angs, img.shape, 200.0, 400.0, du=1.3, d_pix=1.0)
    bo = orc.sf_bp_fan_2d(y, angs, img.shape, 200.0, 400.0, du=1.3, d_pix=1.0)
    assert rel(bp, bo) < 1e-4
    assert dot_rel(fp, y, img, bp) < 1e-4


def test_sf_par_rect_golden_oracle_adjoint(vg, golden, orc):
    from vir_gb300.sys_mat import fp_2d_par
    g = golden["sf_par_rect"]
    out = fp_2d_par.separable_footprint_fp_2d(g["img"], g["angs"], int(g["n_dets"]),
                                              float(g["d_det"]), float(g["d_pix"]))
    assert rel(out, g["sino"]) < 1e-5
    rng = np.random.default_rng(2)
    img = rng.random((70, 50)).astype(np.float32)
    angs = np.linspace(0, np.pi, 45, endpoint=False)
    fp = fp_2d_par.separable_footprint_fp_2d(img, angs, 110, 0.8, 1.1)
    assert rel(fp, orc.separable_footprint_fp_2d(img, angs, 110, 0.8, 1.1)) < 1e-5
    y = rng.random(fp.shape).astype(np.float32)
    bp = fp_2d_par.separable_footprint_bp_2d(y, angs, img.shape, 0.8, 1.1)
    assert rel(bp, orc.separable_footprint_bp_2d(y, angs, img.shape, 0.8, 1.1)) < 1e-5
    assert dot_rel(fp, y, img, bp) < 1e-5


# --- cone-beam DD ------------------------------------------------------------

def test_cone_golden(vg, golden):
    from vir_gb300.sys_mat import dd
    g = golden["dd_cone"]
    kw = dict(du=float(g["du"]), dv=float(g["dv"]), su=float(g["su"]), sv=float(g["sv"]),
              d_pix=float(g["d_pix"]))
    fp = dd.dd_fp_cone_3d(g["vol"], g["angs"], int(g["nu"]), int(g["nv"]), float(g["DSO"]),
                          float(g["DSD"]), **kw)
    assert rel(fp, g["sino_fixed"]) < 5e-5
    bp = dd.dd_bp_cone_3d(g["y"], g["angs"], g["vol"].shape, float(g["DSO"]), float(g["DSD"]),
                          **kw)
    assert rel(bp, g["bp"]) < 5e-5


@pytest.mark.parametrize("shape", [(24, 24, 24), (20, 28, 12)])
def test_cone_vs_oracle(vg, orc, shape):
    from vir_gb300.sys_mat import dd
    rng = np.random.default_rng(3)
    vol = rng.random(shape).astype(np.float32)
    angs = np.linspace(0, 2 * np.pi, 24, endpoint=False)
    kw = dict(du=1.1, dv=0.9, su=0.3, sv=-0.2, d_pix=0.8)
    fp = dd.dd_fp_cone_3d(vol, angs, 56, 40, 60.0, 110.0, **kw)
    fo = orc.dd_fp_cone_3d(vol, angs, 56, 40, 60.0, 110.0, **kw)
    assert rel(fp, fo) < 5e-5
    y = rng.random(fp.shape).astype(np.float32)
    bp = dd.dd_bp_cone_3d(y, angs, shape, 60.0, 110.0, **kw)
    bo = orc.dd_bp_cone_3d(y, angs, shape, 60.0, 110.0, **kw)
    assert rel(bp, bo) < 5e-5
    f = {k: float(np.float32(v)) for k, v in kw.items()}
    assert dot_rel(fp, y, vol, bp, 24 * f["d_pix"] ** 3 / (f["du"] * f["dv"])) < 1e-5


def test_cone_sample_kron(vg, orc):
    from vir_gb300.sys_mat import dd
    vol = np.random.default_rng(4).random((8, 8, 8)).astype(np.float32)
    angs = np.linspace(0, 2 * np.pi, 12, endpoint=False)
    fp = dd.dd_fp_cone_3d(vol, angs, 30, 26, 40.0, 80.0, du=1.0, dv=1.0, d_pix=1.0, sample=2)
    up = np.kron(vol, np.ones((2, 2, 2), np.float32))
    fo = orc.dd_fp_cone_3d(up, angs, 30, 26, 40.0, 80.0, du=1.0, dv=1.0, d_pix=0.5)
    assert rel(fp, fo) < 5e-5


def test_cone_c5_scale_properties(vg):
    """Config C5 sizes (256^3, 360 views, 512x384 detector): the GPU pair is
    an adjoint to FP32 accuracy (dot-product test)."""
    import torch
    from vir_gb300.sys_mat import dd
    n, na, nu, nv = 256, 360, 512, 384
    angs = np.linspace(0, 2 * np.pi, na, endpoint=False)
    kw = dict(du=1.6, dv=1.6, su=0.0, sv=0.0, d_pix=1.0)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((n, n, n), device="cuda", generator=g)
    y = torch.rand((na, nu, nv), device="cuda", generator=g)
    A = dd.dd_fp_cone_3d(x, angs, nu, nv, 600.0, 1100.0, **kw)
    B = dd.dd_bp_cone_3d(y, angs, (n, n, n), 600.0, 1100.0, **kw)
    lhs = (A.double() * y.double()).sum().item()
    d = float(np.float32(1.6))
    rhs = (x.double() * B.double()).sum().item() * na * 1.0 / (d * d)
    assert abs(lhs - rhs) / lhs < 1e-5


def test_cone_wide_detector_vs_oracle(vg, orc):
    """A detector reaching beyond DSD from the centre contains the pole of the
    inverse edge map (rays parallel to the pixel lines) for some views."""
    from vir_gb300.sys_mat import dd
    rng = np.random.default_rng(13)
    vol = rng.random((12, 12, 10)).astype(np.float32)
    angs = np.linspace(0.05, 0.05 + 2 * np.pi, 16, endpoint=False)
    kw = dict(du=1.5, dv=1.2, su=0.0, sv=0.0, d_pix=1.0)
    fp = dd.dd_fp_cone_3d(vol, angs, 110, 24, 30.0, 50.0, **kw)
    fo = orc.dd_fp_cone_3d(vol, angs, 110, 24, 30.0, 50.0, **kw)
    assert rel(fp, fo) < 5e-5
    y = rng.random(fp.shape).astype(np.float32)
    bp = dd.dd_bp_cone_3d(y, angs, vol.shape, 30.0, 50.0, **kw)
    bo = orc.dd_bp_cone_3d(y, angs, vol.shape, 30.0, 50.0, **kw)
    assert rel(bp, bo) < 5e-5


@pytest.mark.parametrize("pitch", [0.3, 2.0])
def test_cone_bp_pitch_paths(vg, orc, pitch):
    """Back projection on a ragged volume (8 x 8 x 32 tiles cut at its edges)
    at a coarse detector pitch (each voxel meets at most 3 x 3 cells: the
    shared-memory weight tables) and a fine one (a voxel's shadow spans more
    than 3 cells: the per-voxel path) agrees with the oracle."""
    from vir_gb300.sys_mat import dd
    rng = np.random.default_rng(21)
    shape = (18, 21, 37)
    angs = np.linspace(0.1, 0.1 + 2 * np.pi, 20, endpoint=False)
    nu, nv = int(np.ceil(60 / pitch)), int(np.ceil(80 / pitch))
    kw = dict(du=pitch, dv=pitch, su=0.1, sv=0.2, d_pix=0.8)
    y = rng.random((20, nu, nv)).astype(np.float32)
    bp = dd.dd_bp_cone_3d(y, angs, shape, 60.0, 110.0, **kw)
    bo = orc.dd_bp_cone_3d(y, angs, shape, 60.0, 110.0, **kw)
    assert rel(bp, bo) < 5e-5
