"""The 3D cone-beam separable-footprint pair (vg_sf3d_fp / vg_sf3d_bp, the
projector vir's sys_mat/sp.py:93-211 sketches) against the FP64 oracle
(oracle.sf_fp_cone_3d / sf_bp_cone_3d), vir's detector-area-averaged
analytic cone-beam sphere (analytic_sino.py:563, golden fixture) and the
adjoint relation.  Tolerance against the oracle: 5e-5 of the largest value
(float32 footprints and sums on the GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def relmax(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("shape,kw,geo,nuv", [
    ((24, 24, 24), dict(du=1.1, dv=0.9, su=0.3, sv=-0.2, d_pix=0.8), (60.0, 110.0), (56, 40)),
    ((20, 28, 12), dict(du=1.0, dv=1.3, su=-0.4, sv=0.1, d_pix=1.0), (50.0, 90.0), (60, 30)),
    # coarse cells: a u cell meets more than 6 columns of a line (per-cell FP path)
    ((18, 16, 10), dict(du=4.0, dv=3.0, su=0.0, sv=0.0, d_pix=0.5), (40.0, 80.0), (12, 8)),
    # fine cells: a column covers more than 4 u cells (per-voxel BP path)
    ((10, 12, 8), dict(du=0.2, dv=0.25, su=0.1, sv=0.0, d_pix=1.0), (40.0, 80.0), (160, 120)),
])
def test_sf_cone_vs_oracle(vg, orc, shape, kw, geo, nuv):
    from vir_gb300.sys_mat import sp
    rng = np.random.default_rng(3)
    vol = rng.random(shape).astype(np.float32)
    angs = np.linspace(0.05, 0.05 + 2 * np.pi, 18, endpoint=False)
    nu, nv = nuv
    fp = sp.sf_fp_cone_3d(vol, angs, nu, nv, *geo, **kw)
    f = {k: float(np.float32(v)) for k, v in kw.items()}
    fo = orc.sf_fp_cone_3d(vol, angs, nu, nv, float(np.float32(geo[0])), float(np.float32(geo[1])), **f)
    assert fp.shape == (angs.size, nu, nv)
    assert relmax(fp, fo) < 5e-5
    y = rng.random(fp.shape).astype(np.float32)
    bp = sp.sf_bp_cone_3d(y, angs, shape, *geo, **kw)
    bo = orc.sf_bp_cone_3d(y, angs, shape, float(np.float32(geo[0])), float(np.float32(geo[1])), **f)
    assert bp.shape == shape
    assert relmax(bp, bo) < 5e-5
    # exact adjoint pair
    lhs = (fp.astype(np.float64) * y).sum()
    rhs = (vol.astype(np.float64) * bp).sum()
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_sf_cone_wide_detector_vs_oracle(vg, orc):
    """A detector reaching beyond DSD from its centre holds the pole of the
    inverse edge map for some views; those tiles bound no columns through it."""
    from vir_gb300.sys_mat import sp
    rng = np.random.default_rng(13)
    vol = rng.random((12, 12, 10)).astype(np.float32)
    angs = np.linspace(0.05, 0.05 + 2 * np.pi, 16, endpoint=False)
    kw = dict(du=1.5, dv=1.2, su=0.0, sv=0.0, d_pix=1.0)
    fp = sp.sf_fp_cone_3d(vol, angs, 110, 24, 30.0, 50.0, **kw)
    fo = orc.sf_fp_cone_3d(vol, angs, 110, 24, 30.0, 50.0, **kw)
    assert relmax(fp, fo) < 5e-5
    y = rng.random(fp.shape).astype(np.float32)
    bp = sp.sf_bp_cone_3d(y, angs, vol.shape, 30.0, 50.0, **kw)
    bo = orc.sf_bp_cone_3d(y, angs, vol.shape, 30.0, 50.0, **kw)
    assert relmax(bp, bo) < 5e-5


def test_sf_cone_analytic_sphere(vg, golden, sphere_vol):
    """Projection of a voxelised sphere against vir's detector-area-averaged
    analytic cone-beam sphere (0.5 mm voxels, radius 7 mm, 8 views)."""
    from vir_gb300.sys_mat import sp
    g = golden["sphere_cone_vol"]
    vol = sphere_vol(48, 0.5, g["sphere"]).astype(np.float32)
    fp = sp.sf_fp_cone_3d(vol, g["angs"], int(g["nu"]), int(g["nv"]), float(g["DSO"]),
                          float(g["DSD"]), du=float(g["du"]), dv=float(g["dv"]), d_pix=0.5)
    ref = g["proj"]
    assert np.linalg.norm(fp - ref) / np.linalg.norm(ref) < 0.025
    assert abs(fp.sum() / ref.sum() - 1) < 0.005


def test_sf_cone_c5_adjoint(vg):
    """Config C5 sizes (256^3, 360 views, 512 x 384 detector at 1.6 mm, 1 mm
    voxels, DSO 600, DSD 1100): the pair is an adjoint to float32 accuracy."""
    import torch
    from vir_gb300.sys_mat import sp
    n, na, nu, nv = 256, 360, 512, 384
    angs = np.linspace(0, 2 * np.pi, na, endpoint=False)
    kw = dict(du=1.6, dv=1.6, su=0.0, sv=0.0, d_pix=1.0)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((n, n, n), device="cuda", generator=g)
    y = torch.rand((na, nu, nv), device="cuda", generator=g)
    A = sp.sf_fp_cone_3d(x, angs, nu, nv, 600.0, 1100.0, **kw)
    B = sp.sf_bp_cone_3d(y, angs, (n, n, n), 600.0, 1100.0, **kw)
    lhs = (A.double() * y.double()).sum().item()
    rhs = (x.double() * B.double()).sum().item()
    assert abs(lhs - rhs) / lhs < 1e-5


def test_sf_cone_c4_subset_vs_oracle(vg, orc):
    """The C4 detector and distances (1024 x 768 at 0.8 mm, DSO 600, DSD 1100,
    0.5 mm voxels) on a 64^3 central sub-volume and 4 views, against the oracle."""
    from vir_gb300.sys_mat import sp
    rng = np.random.default_rng(5)
    vol = rng.random((64, 64, 64)).astype(np.float32)
    angs = np.linspace(0, 2 * np.pi, 720, endpoint=False)[[0, 90, 180, 257]]
    kw = dict(du=0.8, dv=0.8, su=0.0, sv=0.0, d_pix=0.5)
    fp = sp.sf_fp_cone_3d(vol, angs, 1024, 768, 600.0, 1100.0, **kw)
    fo = orc.sf_fp_cone_3d(vol, angs, 1024, 768, 600.0, 1100.0, **kw)
    assert relmax(fp, fo) < 5e-5
