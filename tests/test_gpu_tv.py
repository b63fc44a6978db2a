"""GPU TV primal-dual solver (tv.py) and its helpers against the reference's
own helpers and the FP64 oracle's loop."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tv_ops_golden(vg, golden):
    from vir_gb300 import tv
    g = golden["tv_ops"]
    for name, arg in (("grad", "x"), ("div", "z"), ("grad_abs", "x"), ("div_abs", "z")):
        out = getattr(tv, name)(g[arg].astype(np.float32))
        assert np.abs(out - g[name]).max() < 1e-5 * max(1.0, np.abs(g[name]).max()), name
    AA = g["AA"].astype(np.float32)
    out = tv.pyT(AA)
    assert out is AA                       # in place, as the reference's loop
    assert np.abs(out - g["pyT"]).max() < 1e-6


def test_pdhg_vs_oracle(vg, orc):
    """Ten iterations on a DD parallel-beam problem (the helpers' and the
    fused kernels' FP32 against the oracle's FP64 loop)."""
    import torch
    from vir_gb300 import phantoms as ph
    from vir_gb300 import tv
    from vir_gb300.sys_mat import dd
    img, _ = ph.ellipse_phantom(48, 5, seed=9, d_pix=1.0, vmax=1.0)
    angs = np.linspace(0, np.pi, 40, endpoint=False)
    fp = lambda x: dd.dd_fp_par_2d(x, angs, 72)
    bp = lambda s: dd.dd_bp_par_2d(s, angs, (48, 48))
    y = dd.dd_fp_par_2d(img, angs, 72)
    u = tv.pdhg(y, fp, bp, (48, 48), lam=1.0, theta=1.0, iters=10)
    fo = lambda x: orc.dd_fp_par_2d(x, angs, 72)
    bo = lambda s: orc.dd_bp_par_2d(s, angs, (48, 48))
    uo = orc.tv_pdhg(y, fo, bo, (48, 48), lam=1.0, theta=1.0, iters=10)
    assert np.abs(u - uo).max() <= 1e-4 * np.abs(uo).max()
    # CUDA tensors in, CUDA tensor out
    ut = tv.pdhg(torch.from_numpy(y).cuda(), fp, bp, (48, 48), iters=10)
    assert ut.is_cuda and np.array_equal(ut.cpu().numpy(), u)
