"""The fused, graph-captured cone-beam SIRT update (vg_dd3d_sirt_iter,
reconstruction.SIRT3D): vir's rule (sys_mat/sirt_dd.py:51-72) on the DD cone
pair, against the FP64 oracle's SIRT on its cone pair and against the
unfused path (projector calls and torch elementwise ops)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cone_sirt_vs_oracle_and_unfused(vg, orc):
    import torch
    from vir_gb300 import reconstruction as rc
    from vir_gb300.autograd import ConeGeom, sirt
    rng = np.random.default_rng(9)
    shape = (24, 22, 20)
    vol = rng.random(shape).astype(np.float32)
    angs = np.linspace(0, 2 * np.pi, 30, endpoint=False)
    kw = dict(du=1.2, dv=1.1, su=0.2, sv=-0.1, d_pix=1.0)
    nu, nv, DSO, DSD = 48, 40, 60.0, 110.0
    y = orc.dd_fp_cone_3d(vol, angs, nu, nv, DSO, DSD, **kw).astype(np.float32)
    s = rc.SIRT3D(y, angs, shape, DSO, DSD, **kw)
    for graph in (True, False):
        s.reset()
        x = s.run(10, graph=graph).cpu().numpy()
        fp = lambda z: orc.dd_fp_cone_3d(z, angs, nu, nv, DSO, DSD, **kw)
        bp = lambda r: orc.dd_bp_cone_3d(r, angs, shape, DSO, DSD, **kw)
        xo = orc.sirt(y, fp, bp, shape, iters=11)
        assert np.abs(x - xo).max() <= 2e-4 * np.abs(xo).max()
    geom = ConeGeom(tuple(angs.tolist()), shape, nu, nv, DSO, DSD, **kw)
    xu = sirt(torch.from_numpy(y).cuda(), geom, iters=11).cpu().numpy()
    assert np.abs(x - xu).max() <= 1e-5 * np.abs(xu).max()
