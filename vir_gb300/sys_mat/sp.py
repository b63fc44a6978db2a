"""Separable-footprint fan-beam projector, drop-in for vir ``sys_mat/sp.py``.

* ``sf_fp_fan_2d(img, angs, nu, DSO, DSD, du=1.0, d_pix=1.0)`` (sp.py:12-87):
  linear B-spline footprint of half width DSD d_pix / (DSO - yp) centred at
  DSD xp / (DSO - yp), sampled at bin centres, result scaled by d_pix.
* ``sf_bp_fan_2d(sino, angs, img_shape, DSO, DSD, du=1.0, d_pix=1.0)``: its
  exact adjoint (sp.py has no 2D backprojector).

vir's 3D ``CTGeometry`` / ``forward_project`` / ``back_project``
(sp.py:93-211) have no rotation angles and run a 128^3 projection at import;
they are not reproduced.  Runs on the GPU (``vg_sf2d_fp`` / ``vg_sf2d_bp``).
"""
from __future__ import annotations

import ctypes

from .. import _core
from .._lib import SF2DGeom, call


def _geom(nx, ny, na, nu, du, d_pix, DSO, DSD, fan):
    return SF2DGeom(int(nx), int(ny), int(na), int(nu), float(du), float(d_pix), float(DSO),
                    float(DSD), int(fan))


def sf_fp_2d(img, angs, nu, du, d_pix, DSO, DSD, fan):
    dev = _core.device_of(img)
    x = _core.to_device(img, dev)
    trig = _core.trig_cache.get(angs, None, dev)
    na = trig.numel() // 2
    g = _geom(x.shape[0], x.shape[1], na, nu, du, d_pix, DSO, DSD, fan)
    out = _core.empty((na, int(nu)), dev)
    xT = x.t().contiguous()
    call("vg_sf2d_fp", ctypes.byref(g), _core.ptr(x), _core.ptr(xT), _core.ptr(trig),
         _core.ptr(out), _core.stream(dev))
    return _core.to_host_like(out, img)


def sf_bp_2d(sino, angs, img_shape, du, d_pix, DSO, DSD, fan):
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    trig = _core.trig_cache.get(angs, None, dev)
    na = trig.numel() // 2
    if y.shape[0] != na:
        raise ValueError("sino rows must equal the number of angles")
    nx, ny = (int(v) for v in img_shape)
    g = _geom(nx, ny, na, y.shape[1], du, d_pix, DSO, DSD, fan)
    out = _core.empty((nx, ny), dev)
    call("vg_sf2d_bp", ctypes.byref(g), _core.ptr(y), _core.ptr(trig), _core.ptr(out),
         _core.stream(dev))
    return _core.to_host_like(out, sino)


def sf_fp_fan_2d(img, angs, nu, DSO, DSD, du=1.0, d_pix=1.0):
    return sf_fp_2d(img, angs, nu, du, d_pix, DSO, DSD, 1)


def sf_bp_fan_2d(sino, angs, img_shape, DSO, DSD, du=1.0, d_pix=1.0):
    return sf_bp_2d(sino, angs, img_shape, du, d_pix, DSO, DSD, 1)
