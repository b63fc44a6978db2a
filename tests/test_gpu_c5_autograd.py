"""The differentiable cone projector (autograd.Project) at configuration C5:
256^3 volume of 20 random ellipsoids (1 mm voxels), 360 views over 2 pi,
512 x 384 detector at 1.6 mm, DSO 600 mm, DSD 1100 mm; loss
||A x - y||^2 + 1e-3 TV(x).

* dot-product test of the forward pass against its backward (exact adjoint);
* the loss gradient against central differences along FP64 directions
  (rel err < 1e-3);
* 200 Adam steps against SIRT (vir's rule, sirt_dd.py:51-72) at matched RMSE:
  Adam reaches the RMSE of 50 SIRT updates within its 200 steps and ends
  below it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c5():
    import torch
    from vir_gb300 import phantoms as ph
    from vir_gb300.autograd import ConeGeom
    n, na, nu, nv = 256, 360, 512, 384
    angs = tuple(np.linspace(0, 2 * np.pi, na, endpoint=False).tolist())
    geom = ConeGeom(angs, (n, n, n), nu, nv, 600.0, 1100.0, du=1.6, dv=1.6, d_pix=1.0)
    e = ph.random_ellipsoids(20, fov_radius=n / 2, seed=2027)
    xt = ph.rasterize3d_device(e, n, 1.0, device="cuda")
    y = geom.fp(xt)
    yield geom, xt, y
    del xt, y
    torch.cuda.empty_cache()


def test_c5_project_dot_product(vg, c5):
    import torch
    from vir_gb300.autograd import project
    geom, _, y0 = c5
    g = torch.Generator(device="cuda").manual_seed(1)
    x = torch.rand(geom.img_shape, device="cuda", generator=g).requires_grad_(True)
    w = torch.rand(y0.shape, device="cuda", generator=g)
    Ax = project(x, geom)
    (Ax * w).sum().backward()
    lhs = (Ax.detach().double() * w.double()).sum().item()
    rhs = (x.detach().double() * x.grad.double()).sum().item()
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_c5_loss_gradient_finite_differences(vg, c5):
    import torch
    from vir_gb300.autograd import loss_fn, tv
    geom, xt, y0 = c5
    g = torch.Generator(device="cuda").manual_seed(5)
    y = y0 + 0.01 * torch.randn(y0.shape, device="cuda", generator=g)
    # a point off the phantom, so TV is smooth around it
    x = xt + 0.002 * torch.rand(geom.img_shape, device="cuda", generator=g)
    xg = x.clone().requires_grad_(True)
    loss_fn(xg, y, geom, lam=1e-3).backward()
    grad = xg.grad.double()

    def loss64(z):  # the same loss, accumulated in FP64 on FP32 projections
        r = (geom.fp(z.float()) - y).double()
        return (r * r).sum() + 1e-3 * tv(z.double())

    rng = np.random.default_rng(3)
    for _ in range(3):
        d = torch.from_numpy(rng.standard_normal(geom.img_shape)).cuda()
        d = d / d.norm()
        h = 0.05
        with torch.no_grad():
            fd = ((loss64(x.double() + h * d) - loss64(x.double() - h * d)) / (2 * h)).item()
        an = (grad * d).sum().item()
        assert abs(fd - an) / abs(an) < 1e-3, (fd, an)


def test_c5_adam_vs_sirt_matched_rmse(vg, c5):
    import torch
    from vir_gb300.autograd import reconstruct_adam, sirt
    geom, xt, y = c5
    rmse = lambda x: float(((x - xt) ** 2).mean().sqrt())
    r_sirt = rmse(sirt(y, geom, iters=51))
    trace = []
    xa = reconstruct_adam(y, geom, steps=200, lr=3e-3, lam=1e-3,
                          callback=lambda i, x, L: trace.append(rmse(x)))
    r0 = rmse(torch.zeros_like(xt))
    assert r_sirt < 0.3 * r0
    matched = next((i + 1 for i, r in enumerate(trace) if r <= r_sirt), None)
    assert matched is not None and matched <= 200, (r_sirt, trace[-1])
    assert rmse(xa) < r_sirt
