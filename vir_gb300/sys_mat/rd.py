"""Ray-driven projectors, drop-in for vir ``sys_mat/rd.py``.

Same names, signatures, return layouts and scales as the reference:

* ``aw_fp_par_2d(img, ang_arr, nu, du=1.0, su=0.0, d_pix=1.0, joseph=False)``
  (rd.py:450) and ``aw_bp_par_2d(sino, ang_arr, img_shape, ...)`` (rd.py:461);
* ``aw_fp_fan_2d(img, ang_arr, nu, DSO, DSD, ...)`` / ``aw_bp_fan_2d``
  (rd.py:544, 556);
* ``aw_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0,
  sv=0.0, d_pix=1.0, joseph=False)`` / ``aw_bp_cone_3d`` (rd.py:652, 665).

``joseph=False`` walks each ray through the pixels (Amanatides-Woo),
``joseph=True`` samples it every 0.5 with (bi/tri)linear interpolation.  The
forward projections return the line integrals (the AW cone ones times
DSD / sqrt(DSD^2 + u^2 + v^2)); the back projections return the scattered
image / na / d_pix^2 * du (2D) or / na * du * dv (cone), as the reference.
Two reference defects are fixed: rays parallel to an axis are clipped to
the slab they lie in (rd.py:52-64 lets rays beside the image walk its edge
row, over-counting axis-aligned views), and cone detector rows use nv
(rd.py:688 uses nu).  ``aw_p_square`` (rd.py:794) is not provided: it calls
``pf.censpace`` with its arguments swapped (rd.py:844-849) and does not run.

Inputs are cast to float32 as ``as_float32`` does, angles included; the GPU
kernels are in csrc/rdpd.cu.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _core
from .._lib import RayGeom, call


def _geom(kind, shape, na, nu, nv, du, dv, su, sv, d_pix, DSO, DSD, joseph):
    f = _core.f32
    nz = int(shape[2]) if len(shape) > 2 else 1
    return RayGeom(int(shape[0]), int(shape[1]), nz, int(na), int(nu), int(nv), f(du), f(dv),
                   f(su), f(sv), f(d_pix), f(DSO), f(DSD), int(kind), int(bool(joseph)))


def _fp(kind, img, ang_arr, nu, nv, DSO, DSD, du, dv, su, sv, d_pix, joseph):
    dev = _core.device_of(img)
    x = _core.to_device(img, dev)
    if x.ndim != (3 if kind == 2 else 2):
        raise ValueError("img must be %dD" % (3 if kind == 2 else 2))
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na = trig.numel() // 2
    g = _geom(kind, x.shape, na, nu, nv, du, dv, su, sv, d_pix, DSO, DSD, joseph)
    sino = _core.empty((na, int(nu)) + ((int(nv),) if kind == 2 else ()), dev)
    call("vg_rd_fp", ctypes.byref(g), _core.ptr(x), _core.ptr(trig), _core.ptr(sino),
         _core.stream(dev))
    return _core.to_host_like(sino, img)


def _bp(kind, sino, ang_arr, img_shape, DSO, DSD, du, dv, su, sv, d_pix, joseph):
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na = trig.numel() // 2
    if y.ndim != (3 if kind == 2 else 2) or y.shape[0] != na:
        raise ValueError("sino must be (na, nu%s) with na = len(ang_arr)" % (", nv" if kind == 2 else ""))
    nv = y.shape[2] if kind == 2 else 1
    g = _geom(kind, img_shape, na, y.shape[1], nv, du, dv, su, sv, d_pix, DSO, DSD, joseph)
    img = _core.empty(tuple(int(v) for v in img_shape), dev)
    call("vg_rd_bp", ctypes.byref(g), _core.ptr(y), _core.ptr(trig), _core.ptr(img),
         _core.stream(dev))
    return _core.to_host_like(img, sino)


def aw_fp_par_2d(img, ang_arr, nu, du=1.0, su=0.0, d_pix=1.0, joseph=False):
    return _fp(0, img, ang_arr, nu, 1, 0.0, 0.0, du, 1.0, su, 0.0, d_pix, joseph)


def aw_bp_par_2d(sino, ang_arr, img_shape, du=1.0, su=0.0, d_pix=1.0, joseph=False):
    return _bp(0, sino, ang_arr, img_shape, 0.0, 0.0, du, 1.0, su, 0.0, d_pix, joseph)


def aw_fp_fan_2d(img, ang_arr, nu, DSO, DSD, du=1.0, su=0.0, d_pix=1.0, joseph=False):
    return _fp(1, img, ang_arr, nu, 1, DSO, DSD, du, 1.0, su, 0.0, d_pix, joseph)


def aw_bp_fan_2d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, su=0.0, d_pix=1.0, joseph=False):
    return _bp(1, sino, ang_arr, img_shape, DSO, DSD, du, 1.0, su, 0.0, d_pix, joseph)


def aw_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0,
                  joseph=False):
    return _fp(2, img, ang_arr, nu, nv, DSO, DSD, du, dv, su, sv, d_pix, joseph)


def aw_bp_cone_3d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0,
                  joseph=False):
    return _bp(2, sino, ang_arr, img_shape, DSO, DSD, du, dv, su, sv, d_pix, joseph)
