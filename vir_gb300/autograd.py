"""Differentiable projectors: torch.autograd.Function wrappers whose backward
is the hand-written matched backprojector.

vir's distance-driven pair is scaled, not an exact adjoint (dd.py:721-725,
884-888): the FP returns A x * d_pix/du (2D) or A x * d_pix^2/(du dv)
(cone) and the BP returns A^T y / (na d_pix).  The adjoint of the FP is
therefore the BP times na d_pix^2 / du (2D) or na d_pix^3 / (du dv) (cone);
``backward`` applies exactly that, so gradients are exact (checked by the
dot-product test and finite differences in the tests).

Also here: an isotropic total-variation term, Adam reconstruction of
||A x - y||^2 + lam TV(x), and SIRT on the cone pair for comparison.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from .sys_mat import dd


@dataclass(frozen=True)
class ConeGeom:
    """Arguments of dd_fp_cone_3d / dd_bp_cone_3d (dd.py:815, 829)."""
    angles: tuple
    img_shape: tuple
    nu: int
    nv: int
    DSO: float
    DSD: float
    du: float = 1.0
    dv: float = 1.0
    su: float = 0.0
    sv: float = 0.0
    d_pix: float = 1.0

    @property
    def adjoint_scale(self):
        f = lambda v: float(np.float32(v))
        return len(self.angles) * f(self.d_pix) ** 3 / (f(self.du) * f(self.dv))

    def fp(self, x):
        return dd.dd_fp_cone_3d(x, np.asarray(self.angles), self.nu, self.nv, self.DSO, self.DSD,
                                du=self.du, dv=self.dv, su=self.su, sv=self.sv, d_pix=self.d_pix)

    def bp(self, y):
        return dd.dd_bp_cone_3d(y, np.asarray(self.angles), self.img_shape, self.DSO, self.DSD,
                                du=self.du, dv=self.dv, su=self.su, sv=self.sv, d_pix=self.d_pix)


@dataclass(frozen=True)
class Geom2D:
    """Arguments of dd_fp_{par,fan}_2d / dd_bp_{par,fan}_2d (dd.py:651-745)."""
    angles: tuple
    img_shape: tuple
    nu: int
    du: float = 1.0
    su: float = 0.0
    d_pix: float = 1.0
    DSO: float = 0.0
    DSD: float = 0.0
    fan: bool = False

    @property
    def adjoint_scale(self):
        f = lambda v: float(np.float32(v))
        return len(self.angles) * f(self.d_pix) ** 2 / f(self.du)

    def fp(self, x):
        a = np.asarray(self.angles)
        if self.fan:
            return dd.dd_fp_fan_2d(x, a, self.nu, self.DSO, self.DSD, self.du, self.su, self.d_pix)
        return dd.dd_fp_par_2d(x, a, self.nu, self.du, self.su, self.d_pix)

    def bp(self, y):
        a = np.asarray(self.angles)
        if self.fan:
            return dd.dd_bp_fan_2d(y, a, self.img_shape, self.DSO, self.DSD, self.du, self.su,
                                   self.d_pix)
        return dd.dd_bp_par_2d(y, a, self.img_shape, self.du, self.su, self.d_pix)


class Project(torch.autograd.Function):
    """y = FP(x) with vir's output scaling; backward = exact adjoint."""

    @staticmethod
    def forward(ctx, x, geom):
        ctx.geom = geom
        return geom.fp(x.contiguous())

    @staticmethod
    def backward(ctx, g):
        geom = ctx.geom
        return geom.bp(g.contiguous()) * geom.adjoint_scale, None


def project(x, geom):
    return Project.apply(x, geom)


def tv(x, eps=1e-8):
    """Isotropic total variation sum sqrt(|forward differences|^2 + eps)."""
    d = [torch.diff(x, dim=k, append=x.narrow(k, x.shape[k] - 1, 1)) for k in range(x.ndim)]
    return torch.sqrt(sum(t * t for t in d) + eps).sum()


def loss_fn(x, y, geom, lam=1e-3):
    r = project(x, geom) - y
    return (r * r).sum() + lam * tv(x)


def reconstruct_adam(y, geom, steps=200, lr=1e-3, lam=1e-3, x0=None, callback=None):
    """Adam on ||A x - y||^2 + lam TV(x) through the differentiable projector."""
    y = y.detach()
    x = (torch.zeros(geom.img_shape, device=y.device) if x0 is None else x0.clone()).requires_grad_(True)
    opt = torch.optim.Adam([x], lr=lr)
    for it in range(steps):
        opt.zero_grad(set_to_none=True)
        L = loss_fn(x, y, geom, lam)
        L.backward()
        opt.step()
        if callback is not None:
            callback(it, x.detach(), float(L.detach()))
    return x.detach()


def sirt(y, geom, iters=20, gamma=1.0, x0=1e-5, callback=None, W_sino=None, W_img=None):
    """vir's SIRT rule (sirt_dd.py:23-76; iters - 1 updates) on any pair of
    this module (cone or 2D), on device tensors.  Every step is a separate
    projector call or torch elementwise op (the unfused path)."""
    dev = y.device
    if W_sino is None:
        W_sino = geom.fp(torch.ones(geom.img_shape, device=dev))
    if W_img is None:
        W_img = geom.bp(torch.ones_like(y))
    inv_ws = torch.where(W_sino != 0, 1.0 / W_sino, torch.zeros_like(W_sino))
    inv_wi = torch.where(W_img != 0, 1.0 / W_img, torch.zeros_like(W_img))
    x = torch.full(geom.img_shape, float(np.float32(x0)), device=dev)
    for it in range(1, iters):
        est = geom.fp(x)
        r = torch.where(inv_ws != 0, (y - est) * inv_ws, est)
        upd = geom.bp(r)
        upd = torch.where(inv_wi != 0, upd * inv_wi, upd)
        x = x + gamma * upd
        if callback is not None:
            callback(it, x)
    return x
