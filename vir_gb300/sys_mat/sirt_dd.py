"""SIRT on the translational square geometry, drop-in for vir
``sys_mat/sirt_dd.py`` (``sirt_numba.py`` holds the same functions).

``sirt(sino, W_sino, W_img, gem_prms, img_prms, src_prms, det_prms,
srt_prms)`` (sirt_dd.py:37-76) unpacks

* ``gem_prms = (DSO, DSD)``, ``img_prms = (nx, ny, nz, d_pix)``,
* ``src_prms = (nsrc_p, nsrc_z, dsrc_p, dsrc_z, ssrc_p, ssrc_z)``,
* ``det_prms = (nu, nv, du, dv, su, sv)``, ``srt_prms = (gamma, iters)``,

starts from ``x = 1e-5`` and runs ``iters - 1`` updates
``x += gamma * fast_divide2(BP(fast_divide1(sino, FP(x), W_sino)), W_img)``
with the square-geometry pair of ``dd.py:903, 1104``.  ``fast_divide1``
replaces the estimate by ``(sino - est) / W_sino`` where ``W_sino != 0`` and
leaves it as is elsewhere; ``fast_divide2`` divides by ``W_img`` where it is
non-zero (sirt_dd.py:23-33).

Every update is one call of ``vg_dd_square_sirt_iter``: the forward kernel
writes the weighted residual directly, and the back projection's combine
kernel applies the image weight and the update, so the iterate never leaves
the GPU.  numpy in -> numpy out; CUDA tensors stay on the device.  The
reference prints the iteration number each step; this version does not.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _core
from .._lib import call, dd_square_workspace
from .dd import square_geom


def fast_divide1(sino, sino_est, W_sino):
    """In place: sino_est = (sino - sino_est) / W_sino where W_sino != 0
    (sirt_dd.py:23-27)."""
    dev = _core.device_of(sino, sino_est, W_sino)
    y, e, w = (_core.to_device(a, dev) for a in (sino, sino_est, W_sino))
    r = torch.where(w != 0, (y - e) / torch.where(w != 0, w, torch.ones_like(w)), e)
    _write_back(sino_est, r)


def fast_divide2(image_update, W_img):
    """In place: image_update = image_update / W_img where W_img != 0
    (sirt_dd.py:30-33)."""
    dev = _core.device_of(image_update, W_img)
    u, w = (_core.to_device(a, dev) for a in (image_update, W_img))
    r = torch.where(w != 0, u / torch.where(w != 0, w, torch.ones_like(w)), u)
    _write_back(image_update, r)


def _write_back(dst, t):
    if _core.is_torch(dst):
        dst.copy_(t.to(dst.device, dst.dtype))
    else:
        dst[...] = t.cpu().numpy().astype(dst.dtype, copy=False)


def sirt(sino, W_sino, W_img, gem_prms, img_prms, src_prms, det_prms, srt_prms):
    DSO, DSD = gem_prms
    nx, ny, nz, d_pix = img_prms
    nsrc_p, nsrc_z, dsrc_p, dsrc_z, ssrc_p, ssrc_z = src_prms
    nu, nv, du, dv, su, sv = det_prms
    gamma, iters = srt_prms
    img_shape = (int(nx), int(ny), int(nz))
    g = square_geom(img_shape, nu, nv, nsrc_p, nsrc_z, DSO, DSD, du, dv, dsrc_p, dsrc_z, su, sv,
                    ssrc_p, ssrc_z, d_pix)
    dev = _core.device_of(sino, W_sino, W_img)
    y = _core.to_device(sino, dev)
    ws_sino = _core.to_device(W_sino, dev)
    ws_img = _core.to_device(W_img, dev)
    want = (int(nsrc_p), int(nsrc_z), int(nv), int(nu), 4)
    if tuple(y.shape) != want or tuple(ws_sino.shape) != want:
        raise ValueError(f"sino and W_sino must have shape {want}")
    if tuple(ws_img.shape) != img_shape:
        raise ValueError(f"W_img must have shape {img_shape}")
    x = torch.full(img_shape, float(np.float32(.00001)), dtype=torch.float32, device=dev)
    r = torch.empty_like(y)
    ws = dd_square_workspace(g, dev)
    st = _core.stream(dev)
    for _ in range(1, int(iters)):
        call("vg_dd_square_sirt_iter", ctypes.byref(g), _core.ptr(y), _core.ptr(ws_sino),
             _core.ptr(ws_img), _core.f32(gamma), _core.ptr(x), _core.ptr(r), _core.ptr(ws),
             ws.numel() * 8, st)
    return _core.to_host_like(x, sino)
