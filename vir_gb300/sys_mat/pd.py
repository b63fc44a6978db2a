"""Pixel-driven footprint projectors, drop-in for vir ``sys_mat/pd.py``.

Same names, signatures, return layouts and scales as the reference:
``pd_fp_par_2d(img, ang_arr, nu, du=1.0, su=0.0, d_pix=1.0)`` /
``pd_bp_par_2d(sino, ang_arr, img_shape, ...)`` (pd.py:130, 138),
``pd_fp_fan_2d(img, ang_arr, nu, DSO, DSD, ...)`` / ``pd_bp_fan_2d``
(pd.py:238, 246), ``pd_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0,
dv=1.0, su=0.0, sv=0.0, d_pix=1.0)`` / ``pd_bp_cone_3d`` (pd.py:354, 363).

Each pixel's four corners are projected to the detector and the pixel's
value is spread over the overlapped bins, times 1 / (|sin| + |cos|)
(parallel, cone) or 1 / (|cos(a + g)| + |sin(a + g)|) with g the fan angle
of the pixel centre (fan).  FP returns sino * d_pix, BP img / na / d_pix *
du (* dv for the cone).  The reference's fan FP does not advance the
pixel-centre y after a zero pixel (pd.py:335-339), which perturbs the scale
of the pixels that follow zeros; here every pixel uses its own centre.

The angles are used as given (the reference does not cast them); the GPU
kernels are in csrc/rdpd.cu.
"""
from __future__ import annotations

import ctypes

from .. import _core
from .._lib import call
from .rd import _geom


def _fp(kind, img, ang_arr, nu, nv, DSO, DSD, du, dv, su, sv, d_pix):
    dev = _core.device_of(img)
    x = _core.to_device(img, dev)
    if x.ndim != (3 if kind == 2 else 2):
        raise ValueError("img must be %dD" % (3 if kind == 2 else 2))
    trig = _core.trig_cache.get(ang_arr, None, dev)
    na = trig.numel() // 2
    g = _geom(kind, x.shape, na, nu, nv, du, dv, su, sv, d_pix, DSO, DSD, 0)
    sino = _core.empty((na, int(nu)) + ((int(nv),) if kind == 2 else ()), dev)
    call("vg_pd_fp", ctypes.byref(g), _core.ptr(x), _core.ptr(trig), _core.ptr(sino),
         _core.stream(dev))
    return _core.to_host_like(sino, img)


def _bp(kind, sino, ang_arr, img_shape, DSO, DSD, du, dv, su, sv, d_pix):
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    trig = _core.trig_cache.get(ang_arr, None, dev)
    na = trig.numel() // 2
    if y.ndim != (3 if kind == 2 else 2) or y.shape[0] != na:
        raise ValueError("sino must be (na, nu%s) with na = len(ang_arr)" % (", nv" if kind == 2 else ""))
    nv = y.shape[2] if kind == 2 else 1
    g = _geom(kind, img_shape, na, y.shape[1], nv, du, dv, su, sv, d_pix, DSO, DSD, 0)
    img = _core.empty(tuple(int(v) for v in img_shape), dev)
    call("vg_pd_bp", ctypes.byref(g), _core.ptr(y), _core.ptr(trig), _core.ptr(img),
         _core.stream(dev))
    return _core.to_host_like(img, sino)


def pd_fp_par_2d(img, ang_arr, nu, du=1.0, su=0.0, d_pix=1.0):
    return _fp(0, img, ang_arr, nu, 1, 0.0, 0.0, du, 1.0, su, 0.0, d_pix)


def pd_bp_par_2d(sino, ang_arr, img_shape, du=1.0, su=0.0, d_pix=1.0):
    return _bp(0, sino, ang_arr, img_shape, 0.0, 0.0, du, 1.0, su, 0.0, d_pix)


def pd_fp_fan_2d(img, ang_arr, nu, DSO, DSD, du=1.0, su=0.0, d_pix=1.0):
    return _fp(1, img, ang_arr, nu, 1, DSO, DSD, du, 1.0, su, 0.0, d_pix)


def pd_bp_fan_2d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, su=0.0, d_pix=1.0):
    return _bp(1, sino, ang_arr, img_shape, DSO, DSD, du, 1.0, su, 0.0, d_pix)


def pd_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    return _fp(2, img, ang_arr, nu, nv, DSO, DSD, du, dv, su, sv, d_pix)


def pd_bp_cone_3d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    return _bp(2, sino, ang_arr, img_shape, DSO, DSD, du, dv, su, sv, d_pix)
