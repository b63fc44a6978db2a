"""TV-regularised reconstruction with the preconditioned primal-dual (PDHG,
Chambolle-Pock) iteration of vir's ``tv.py`` (tv.py:200-294), on any
projector pair of this package.

Drop-ins for the reference's helpers (same names and conventions, 2D
images, periodic boundaries through ``np.roll``):

* ``grad(x)`` -> ``(2, nx, ny)`` forward differences ``roll(x, -1, k) - x``
  (tv.py:207-211); ``div(z)`` = ``(z0 - roll(z0, 1, 0)) + (z1 - roll(z1, 1,
  1))`` (tv.py:220-224), so ``div = -grad^T``;
* ``grad_abs`` / ``div_abs`` (tv.py:200-218), the sums used for the
  step-size preconditioners;
* ``pyT(AA)``: for each pixel's pair ``(a1, a2)`` the projection of the
  2 x 1 matrix onto the unit spectral-norm ball, i.e. ``a / max(1, |a|)``
  (tv.py:98-184; the vectorised ``pyT2``, tv.py:24-95, computes the same
  map but cannot run: ``np.min`` with an array as axis, and 0/0 at a = 0).

``pdhg(g, fp, bp, img_shape, lam=1.0, theta=1.0, iters=100)`` runs the
loop of tv.py:262-294: sigma_z = 1 / grad_abs(1) = 1/2, sigma_q = 1 / A 1,
tau = 1 / (A^T 1 + div_abs(1)) = 1 / (A^T 1 + 4), then per iteration
``z = P(z + sigma_z grad u_bar)``, ``q = (q + sigma_q (A u_bar - g)) /
(1 + sigma_q lam)``, ``u += tau (div z - A^T q)``, ``u_bar = u + theta (u -
u_prev)``.  ``fp``/``bp`` are callables on CUDA tensors (any pair here:
distance-driven, Siddon lists, ...); rays with A 1 = 0 get sigma_q = 0 (the
reference divides by zero there).  The elementwise steps are the fused
kernels of csrc/tv.cu.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _core
from ._lib import call


def _t(x):
    return _core.to_device(x)


def grad(x):
    t = _t(x)
    out = torch.stack([torch.roll(t, -1, 0) - t, torch.roll(t, -1, 1) - t])
    return _core.to_host_like(out, x)


def grad_abs(x):
    t = _t(x)
    out = torch.stack([t + torch.roll(t, -1, 0), t + torch.roll(t, -1, 1)])
    return _core.to_host_like(out, x)


def div(x):
    t = _t(x)
    out = (t[0] - torch.roll(t[0], 1, 0)) + (t[1] - torch.roll(t[1], 1, 1))
    return _core.to_host_like(out, x)


def div_abs(x):
    t = _t(x)
    out = (t[0] + torch.roll(t[0], 1, 0)) + (t[1] + torch.roll(t[1], 1, 1))
    return _core.to_host_like(out, x)


def pyT(AA):
    """Projection of every pixel's (a1, a2) onto the unit ball, in place for
    numpy input (the reference's loop writes AA in place) and returned."""
    t = _t(AA)
    m = torch.clamp(torch.sqrt(t[0] * t[0] + t[1] * t[1]), min=1.0)
    out = t / m
    if isinstance(AA, np.ndarray):
        AA[...] = out.cpu().numpy().astype(AA.dtype, copy=False)
        return AA
    if _core.is_torch(AA):
        AA.copy_(out.to(AA.device, AA.dtype))
        return AA
    return out.cpu().numpy()


def pdhg(g, fp, bp, img_shape, lam=1.0, theta=1.0, iters=100, callback=None):
    nx, ny = (int(v) for v in img_shape)
    dev = _core.device_of(g)
    y = _core.to_device(g, dev)
    A1 = fp(torch.ones((nx, ny), device=dev)).contiguous()
    At1 = bp(torch.ones_like(y)).contiguous()
    sigma_q = torch.where(A1 != 0, 1.0 / torch.where(A1 != 0, A1, torch.ones_like(A1)),
                          torch.zeros_like(A1)).contiguous()
    tau = (1.0 / (At1 + 4.0)).contiguous()
    u = torch.zeros((nx, ny), device=dev)
    ub = torch.zeros_like(u)
    z = torch.zeros((2, nx, ny), device=dev)
    q = torch.zeros_like(y)
    st = _core.stream(dev)
    n = y.numel()
    for k in range(int(iters)):
        call("vg_tv_dual", _core.ptr(ub), _core.ptr(z), nx, ny, 0.5, st)
        ax = fp(ub).contiguous()
        call("vg_tv_residual", _core.ptr(q), _core.ptr(ax), _core.ptr(y), _core.ptr(sigma_q),
             _core.f32(lam), n, st)
        atq = bp(q).contiguous()
        call("vg_tv_primal", _core.ptr(u), _core.ptr(ub), _core.ptr(z), _core.ptr(atq),
             _core.ptr(tau), _core.f32(theta), nx, ny, st)
        if callback is not None:
            callback(k, u)
    return _core.to_host_like(u, g)
