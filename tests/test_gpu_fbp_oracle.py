"""FBP and FDK against the FP64 oracle (oracle.fbp_2d, fbp_par_dd, fdk), whose
weights and interpolation step are pinned to the reference's own
cosine_weighting (processing/reconstruction.py:99-107) and
fan_backproject_hsieh (processing/proj2.py:580-616) by tests/test_oracle.py.

* fan FBP at the C2 geometry (512^2, 720 views over 2 pi, 768 bins of 1.2 mm,
  DSO 500, DSD 1000, 0.9 mm pixels) on the benchmark's noisy sinogram;
* parallel FBP at the C1 geometry (256^2, 180 views over pi, 367 bins), both
  the pixel-driven route and vir's (pi / 2) dd_bp_par_2d(filter_sino(y));
* FDK at the full C4 geometry (512^3, 720 views, 1024 x 768 at 0.8 mm, DSO
  600, DSD 1100) on sub-volumes at the centre, off centre and near the top
  of the cone.
Tolerance: 1e-5 of the oracle's largest value (FDK: of the volume's peak; the
noisy fan sinogram: 3e-5 of the peak and 1e-5 in L2); float32 filter and sums
on the GPU.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def relmax(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


def f32(v):
    return float(np.float32(v))


@pytest.mark.parametrize("filt", ["ramp", "hann"])
def test_fbp_fan_c2_vs_oracle(vg, orc, filt):
    from vir_gb300 import reconstruction as rc
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import bench
    w = bench.WORKLOAD
    img, angs, y = bench.make_inputs()
    rec = rc.fbp_2d(y, angs, img.shape, geom="fan", DSO=w["DSO"], DSD=w["DSD"], du=w["du"],
                    d_pix=w["d_pix"], filter_type=filt)
    ref = orc.fbp_2d(y, angs, img.shape, fan=True, DSO=f32(w["DSO"]), DSD=f32(w["DSD"]),
                     du=f32(w["du"]), d_pix=f32(w["d_pix"]), filter_type=filt)
    # float32 FFT filtering of a noisy sinogram: the largest error is a few
    # 1e-5 of the image's peak, the error as a whole (L2) below 1e-5
    assert relmax(rec, ref) < 3e-5
    assert np.linalg.norm(rec - ref) / np.linalg.norm(ref) < 1e-5
    # and it reconstructs the phantom: mean error well below the contrast
    assert np.abs(rec - img).mean() < 0.1 * img.max()


def test_fbp_par_c1_vs_oracle(vg, orc):
    from vir_gb300 import phantoms as ph
    from vir_gb300 import reconstruction as rc
    img, e = ph.ellipse_phantom(256, 10, seed=2025, d_pix=1.0)
    angs = np.linspace(0, np.pi, 180, endpoint=False)
    y = ph.sino_par(e, angs, 367, du=1.0).astype(np.float32)
    rec = rc.fbp_2d(y, angs, img.shape, du=1.0, d_pix=1.0)
    ref = orc.fbp_2d(y, angs, img.shape, du=1.0, d_pix=1.0)
    assert relmax(rec, ref) < 1e-5
    # vir's own parallel route on the distance-driven backprojector
    rec_dd = rc.fbp_2d(y, angs, img.shape, du=1.0, d_pix=1.0, method="dd")
    ref_dd = orc.fbp_par_dd(y, angs, img.shape, du=1.0, d_pix=1.0)
    assert relmax(rec_dd, ref_dd) < 1e-5
    # the two routes reconstruct the same object up to their interpolation
    inside = np.hypot(*np.meshgrid(np.arange(256) - 127.5, np.arange(256) - 127.5)) < 100
    assert np.abs(rec_dd - rec)[inside].mean() < 0.05 * img.max()


def test_fdk_c4_subvolumes_vs_oracle(vg, orc):
    import torch
    from vir_gb300 import phantoms as ph
    from vir_gb300 import reconstruction as rc
    from vir_gb300.sys_mat import dd
    n, na, nu, nv, dp, du = 512, 720, 1024, 768, 0.5, 0.8
    DSO, DSD = 600.0, 1100.0
    angs = np.linspace(0, 2 * np.pi, na, endpoint=False)
    e = ph.random_ellipsoids(20, fov_radius=n * dp / 2, seed=2027)
    x = ph.rasterize3d_device(e, n, dp, device="cuda")
    kw = dict(du=du, dv=du, su=0.0, sv=0.0, d_pix=dp)
    y = dd.dd_fp_cone_3d(x, angs, nu, nv, DSO, DSD, **kw)
    del x
    vol = rc.fdk(y, angs, (n, n, n), DSO, DSD, **kw)
    yh = y.cpu().numpy()
    del y
    torch.cuda.empty_cache()
    boxes = [((250, 262), (250, 262), (250, 262)),   # centre
             ((100, 110), (380, 392), (240, 250)),   # off centre in the plane
             ((300, 308), (200, 210), (470, 482))]   # high in z, steep rays
    f = {k: f32(v) for k, v in kw.items()}
    peak = float(vol.abs().max())   # tolerance relative to the volume's peak
    for box in boxes:
        (x0, x1), (y0, y1), (z0, z1) = box
        got = vol[x0:x1, y0:y1, z0:z1].cpu().numpy()
        ref = orc.fdk(yh, angs, (n, n, n), f32(DSO), f32(DSD), box=box, **f)
        assert np.abs(got - ref).max() <= 1e-5 * peak, box
