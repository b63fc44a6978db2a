"""Separable-footprint fan-beam projector, drop-in for vir ``sys_mat/sp.py``.

* ``sf_fp_fan_2d(img, angs, nu, DSO, DSD, du=1.0, d_pix=1.0)`` (sp.py:12-87):
  linear B-spline footprint of half width DSD d_pix / (DSO - yp) centred at
  DSD xp / (DSO - yp), sampled at bin centres, result scaled by d_pix.
* ``sf_bp_fan_2d(sino, angs, img_shape, DSO, DSD, du=1.0, d_pix=1.0)``: its
  exact adjoint (sp.py has no 2D backprojector).

* ``sf_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0,
  sv=0.0, d_pix=1.0)`` / ``sf_bp_cone_3d(sino, ang_arr, img_shape, ...)``:
  the 3D cone-beam separable-footprint pair that vir's ``CTGeometry`` /
  ``forward_project`` / ``back_project`` (sp.py:93-211, no rotation angles,
  a 128^3 projection at import) stand in for -- trapezoid / rectangle
  footprints with the A2 amplitude of Long, Fessler & Balter (IEEE TMI 2010)
  on the circular cone geometry and layouts of ``dd_fp_cone_3d``; the FP
  returns line integrals, the BP is its exact adjoint.

Runs on the GPU (``vg_sf2d_fp`` / ``vg_sf2d_bp``, ``vg_sf3d_fp`` /
``vg_sf3d_bp``).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _core
from .._lib import DD3DGeom, SF2DGeom, VirGpuError, call, load


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


def _g3(shape, na, nu, nv, du, dv, su, sv, d_pix, DSO, DSD):
    f = _core.f32
    return DD3DGeom(int(shape[0]), int(shape[1]), int(shape[2]), int(na), int(nu), int(nv),
                    f(du), f(dv), f(su), f(sv), f(d_pix), f(DSO), f(DSD))


def sf_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    """Separable-footprint cone-beam forward projection: vol (nx, ny, nz) ->
    sino (na, nu, nv) of line integrals."""
    dev = _core.device_of(img)
    x = _core.to_device(img, dev)
    if x.ndim != 3:
        raise ValueError("img must be 3D (nx, ny, nz)")
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na = trig.numel() // 2
    g = _g3(x.shape, na, nu, nv, du, dv, su, sv, d_pix, DSO, DSD)
    sino = _core.empty((na, int(nu), int(nv)), dev)
    ws = _sf3d_workspace(g, dev)
    call("vg_sf3d_fp", ctypes.byref(g), _core.ptr(x), _core.ptr(trig), _core.ptr(sino),
         _core.ptr(ws), ws.numel() * 8, _core.stream(dev))
    return _core.to_host_like(sino, img)


def _sf3d_workspace(g, dev):
    """Device workspace of vg_sf3d_workspace_bytes(g) bytes (8-byte aligned)."""
    L = load()
    n = int(L.vg_sf3d_workspace_bytes(ctypes.byref(g)))
    if n == 0:
        raise VirGpuError("vg_sf3d_workspace_bytes", 1, L.vg_last_error().decode(errors="replace"))
    return torch.empty((n + 7) // 8, dtype=torch.float64, device=dev)


def sf_bp_cone_3d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    """Exact adjoint of sf_fp_cone_3d: sino (na, nu, nv) -> vol (nx, ny, nz)."""
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    if y.ndim != 3:
        raise ValueError("sino must be 3D (na, nu, nv)")
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na = trig.numel() // 2
    if y.shape[0] != na:
        raise ValueError(f"sino has {y.shape[0]} views, ang_arr {na}")
    g = _g3(img_shape, na, y.shape[1], y.shape[2], du, dv, su, sv, d_pix, DSO, DSD)
    ws = _sf3d_workspace(g, dev)
    vol = _core.empty(tuple(int(v) for v in img_shape), dev)
    call("vg_sf3d_bp", ctypes.byref(g), _core.ptr(y), _core.ptr(trig), _core.ptr(vol),
         _core.ptr(ws), ws.numel() * 8, _core.stream(dev))
    return _core.to_host_like(vol, sino)
