"""Differentiable projector (dot-product test, finite differences, Adam vs
SIRT) and FDK on the cone geometry; GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cone(n=32, na=48, nu=64, nv=48):
    from vir_gb300.autograd import ConeGeom
    angs = tuple(np.linspace(0, 2 * np.pi, na, endpoint=False).tolist())
    return ConeGeom(angs, (n, n, n), nu, nv, 60.0, 110.0, du=1.3, dv=1.3, d_pix=1.0)


def test_autograd_dot_product(vg):
    import torch
    from vir_gb300.autograd import project
    geom = _cone()
    g = torch.Generator(device="cuda").manual_seed(1)
    x = torch.rand(geom.img_shape, device="cuda", generator=g).requires_grad_(True)
    y = torch.rand((len(geom.angles), geom.nu, geom.nv), device="cuda", generator=g)
    Ax = project(x, geom)
    (Ax * y).sum().backward()
    lhs = (Ax.double() * y.double()).sum().item()
    rhs = (x.detach().double() * x.grad.double()).sum().item()
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_autograd_2d_dot_product(vg):
    import torch
    from vir_gb300.autograd import Geom2D, project
    angs = tuple(np.linspace(0, 2 * np.pi, 60, endpoint=False).tolist())
    geom = Geom2D(angs, (48, 40), 80, du=1.1, d_pix=0.9, DSO=100.0, DSD=180.0, fan=True)
    x = torch.rand(geom.img_shape, device="cuda").requires_grad_(True)
    y = torch.rand((60, 80), device="cuda")
    Ax = project(x, geom)
    (Ax * y).sum().backward()
    lhs = (Ax.double() * y.double()).sum().item()
    rhs = (x.detach().double() * x.grad.double()).sum().item()
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_autograd_finite_differences(vg):
    """Gradient of ||Ax - y||^2 + 1e-3 TV(x) against central differences
    along random directions (rel err < 1e-3)."""
    import torch
    from vir_gb300 import phantoms as ph
    from vir_gb300.autograd import loss_fn
    from vir_gb300.autograd import tv
    geom = _cone(n=24, na=32, nu=48, nv=36)
    vol, _ = ph.ellipsoid_phantom(24, 6, seed=2, vmax=1.0)
    g = torch.Generator(device="cuda").manual_seed(5)
    # a non-flat point, so TV is smooth around it
    x = torch.from_numpy(vol).cuda() + 0.05 * torch.rand(geom.img_shape, device="cuda", generator=g)
    y = geom.fp(torch.from_numpy(vol).cuda())
    y = y + 0.01 * torch.randn(y.shape, device="cuda", generator=g)
    xg = x.clone().requires_grad_(True)
    loss_fn(xg, y, geom).backward()
    grad = xg.grad.double()

    def loss64(z):  # the same loss, accumulated in FP64 on FP32 projections
        r = (geom.fp(z.float()) - y).double()
        return (r * r).sum() + 1e-3 * tv(z.double())

    rng = np.random.default_rng(3)
    for _ in range(3):
        d = torch.from_numpy(rng.standard_normal(geom.img_shape)).cuda()
        d = d / d.norm()
        h = 1e-2
        with torch.no_grad():
            fd = ((loss64(x.double() + h * d) - loss64(x.double() - h * d)) / (2 * h)).item()
        an = (grad * d).sum().item()
        assert abs(fd - an) / abs(an) < 1e-3, (fd, an)


def test_adam_vs_sirt(vg):
    """200 Adam steps on the data + TV loss reach an RMSE comparable to SIRT's."""
    import torch
    from vir_gb300 import phantoms as ph
    from vir_gb300.autograd import reconstruct_adam, sirt
    geom = _cone(n=32, na=64, nu=64, nv=48)
    vol, _ = ph.ellipsoid_phantom(32, 8, seed=4, vmax=0.02)
    xt = torch.from_numpy(vol).cuda()
    y = geom.fp(xt)
    xs = sirt(y, geom, iters=51)
    xa = reconstruct_adam(y, geom, steps=200, lr=2e-4, lam=1e-6)
    rmse = lambda x: float(((x - xt) ** 2).mean().sqrt())
    r0 = float((xt ** 2).mean().sqrt())
    assert rmse(xs) < 0.5 * r0 and rmse(xa) < 0.7 * r0, (rmse(xs), rmse(xa), r0)


def test_fdk_sphere(vg):
    """FDK of exact cone-beam line integrals of a centred sphere recovers its
    value near the mid-plane."""
    import torch
    from vir_gb300 import reconstruction as rc
    n, na, nu, nv = 64, 180, 128, 96
    DSO, DSD, du = 200.0, 400.0, 1.2
    angs = np.linspace(0, 2 * np.pi, na, endpoint=False)
    # analytic line integrals of a unit-value sphere of radius R at the origin
    R = 20.0
    u = du * (np.arange(nu) - nu / 2 + 0.5)
    v = du * (np.arange(nv) - nv / 2 + 0.5)
    U, V = np.meshgrid(u, v, indexing="ij")
    # ray from source (distance DSO) to detector point (u, v) at distance DSD:
    # distance of the ray from the centre = DSO * sqrt(u^2 + v^2) / sqrt(DSD^2 + u^2 + v^2)
    dist = DSO * np.sqrt(U ** 2 + V ** 2) / np.sqrt(DSD ** 2 + U ** 2 + V ** 2)
    chord = 2 * np.sqrt(np.clip(R ** 2 - dist ** 2, 0, None))
    sino = np.broadcast_to(chord, (na, nu, nv)).astype(np.float32).copy()
    rec = rc.fdk(sino, angs, (n, n, n), DSO, DSD, du=du, dv=du, d_pix=1.0)
    c = (np.arange(n) + 0.5 - n / 2)
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    inside = rec[(r < R - 4) & (np.abs(Z) < 6)].mean()
    outside = np.abs(rec[(r > R + 4) & (r < 30) & (np.abs(Z) < 6)]).mean()
    assert abs(inside - 1.0) < 0.02, inside
    assert outside < 0.02, outside
