"""Parity at the benchmark configurations' own sizes, against the FP64 oracle.

The accuracy criterion of the reconstructions: the GPU iterate ends within
1e-4 relative (L2) of the oracle's, and its RMSE against the phantom equals
the oracle's within 1e-4 relative.

* C2: 100 SIRT updates of the 512^2 fan-beam benchmark (720 views, 768 bins of
  1.2 mm, DSO 500, DSD 1000, 0.9 mm pixels, Poisson noise at 1e5 photons/ray),
  through the captured CUDA graph the benchmark replays, vs the oracle's SIRT
  (vir's rule, sys_mat/sirt_dd.py:51-72) on its FP64 DD fan pair.
* C3: the 1024^2 and 512^2 problems of the batched set with the fewest views
  of each geometry, 49 updates (50 iterations) in one batched graph.
* C4 / C5: the cone-beam DD pair at full volume and detector size
  (512^3 and 1024 x 768; 256^3 and 512 x 384) on a subset of the views.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def rmse(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - b) ** 2)))


def _bench():
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import bench
    return bench


def test_c2_sirt_100_updates_vs_oracle(vg, orc):
    import torch
    from vir_gb300 import reconstruction as rc
    b = _bench()
    w = b.WORKLOAD
    img, angs, y = b.make_inputs()
    U = w["updates_per_step"]
    s = rc.SIRT2D(y, angs, img.shape, geom="fan", DSO=w["DSO"], DSD=w["DSD"], du=w["du"],
                  d_pix=w["d_pix"])
    s.capture(U)
    s.run(U)
    x = s.x.cpu().numpy()
    torch.cuda.synchronize()
    fp = lambda z: orc.dd_fp_fan_2d(z, angs, w["nu"], w["DSO"], w["DSD"], du=w["du"],
                                    d_pix=w["d_pix"])
    bp = lambda r: orc.dd_bp_fan_2d(r, angs, img.shape, w["DSO"], w["DSD"], du=w["du"],
                                    d_pix=w["d_pix"])
    xo = orc.sirt(y, fp, bp, img.shape, iters=U + 1)
    assert rel_l2(x, xo) < 1e-4
    r_gpu, r_orc = rmse(x, img), rmse(xo, img)
    assert abs(r_gpu - r_orc) / r_orc < 1e-4
    # a second replay from the reset iterate is the same computation
    s.reset()
    s.run(U)
    assert np.array_equal(s.x.cpu().numpy(), x)


def test_c3_large_problems_vs_oracle(vg, orc):
    from vir_gb300.batched import BatchedSIRT2D
    from vir_gb300.workloads import batched_problems, problem_shapes
    shapes = problem_shapes(64, seed=3)
    pick = []
    for side in (1024, 512):
        for fan in (False, True):
            c = [(na, i) for i, (n, na, f) in enumerate(shapes) if n == side and f == fan]
            pick.append(min(c)[1])
    probs, truth = batched_problems(64, seed=3, only=sorted(pick), with_truth=True)
    assert sorted(p["img_shape"][0] for p in probs) == [512, 512, 1024, 1024]
    b = BatchedSIRT2D(probs, n_streams=4)
    iters = 50
    b.run(iters - 1)
    got = [x.cpu().numpy() for x in b.images()]
    for p, t, g in zip(probs, truth, got):
        a, n, nu = p["ang_arr"], p["img_shape"], p["sino"].shape[1]
        if p["geom"] == "fan":
            fp = lambda x: orc.dd_fp_fan_2d(x, a, nu, p["DSO"], p["DSD"])
            bp = lambda s: orc.dd_bp_fan_2d(s, a, n, p["DSO"], p["DSD"])
        else:
            fp = lambda x: orc.dd_fp_par_2d(x, a, nu)
            bp = lambda s: orc.dd_bp_par_2d(s, a, n)
        xo = orc.sirt(p["sino"], fp, bp, n, iters=iters)
        assert rel_l2(g, xo) < 1e-4, (p["img_shape"], p["geom"])
        r_gpu, r_orc = rmse(g, t), rmse(xo, t)
        assert abs(r_gpu - r_orc) / r_orc < 1e-4, (p["img_shape"], p["geom"])


@pytest.mark.parametrize("cfg", ["c4", "c5"])
def test_cone_full_size_vs_oracle(vg, orc, cfg):
    """FP and BP at the configuration's full volume and detector on a subset
    of its views (the oracle takes seconds per view at 512^3)."""
    import torch
    from vir_gb300 import phantoms as ph
    from vir_gb300.sys_mat import dd
    n, na, nu, nv, dp, du = ((512, 720, 1024, 768, 0.5, 0.8) if cfg == "c4"
                             else (256, 360, 512, 384, 1.0, 1.6))
    DSO, DSD = 600.0, 1100.0
    all_angs = np.linspace(0, 2 * np.pi, na, endpoint=False)
    # views near 0, 45, 90 and 135 degrees plus one off-axis view: both
    # driving axes and the diagonal
    sel = np.array([0, na // 8, na // 4, 3 * na // 8, 5 * na // 13])
    angs = all_angs[sel]
    e = ph.random_ellipsoids(20, fov_radius=n * dp / 2, seed=2027)
    x = ph.rasterize3d_device(e, n, dp, device="cuda")
    xh = x.cpu().numpy()
    kw = dict(du=du, dv=du, su=0.0, sv=0.0, d_pix=dp)
    fp = dd.dd_fp_cone_3d(x, angs, nu, nv, DSO, DSD, **kw).cpu().numpy()
    fo = orc.dd_fp_cone_3d(xh, angs, nu, nv, DSO, DSD, **kw)
    assert rel_l2(fp, fo) < 1e-5
    assert np.abs(fp - fo).max() <= 5e-5 * np.abs(fo).max()
    g = torch.Generator(device="cuda").manual_seed(7)
    y = torch.rand((angs.size, nu, nv), device="cuda", generator=g)
    bp = dd.dd_bp_cone_3d(y, angs, (n, n, n), DSO, DSD, **kw).cpu().numpy()
    del x
    torch.cuda.empty_cache()
    bo = orc.dd_bp_cone_3d(y.cpu().numpy(), angs, (n, n, n), DSO, DSD, **kw)
    assert rel_l2(bp, bo) < 1e-5
    assert np.abs(bp - bo).max() <= 5e-5 * np.abs(bo).max()
