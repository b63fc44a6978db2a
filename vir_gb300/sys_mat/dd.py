"""Distance-driven projectors, drop-in for vir ``sys_mat/dd.py``.

Same names, signatures, return layouts and scales as the reference:

* ``dd_fp_par_2d(img, ang_arr, nu, du=1.0, su=0.0, d_pix=1.0, sample=1)``
  (dd.py:651) -> ``(na, nu)`` sinogram, ``A x * d_pix / du``;
* ``dd_bp_par_2d(sino, ang_arr, img_shape, du=1.0, su=0.0, d_pix=1.0)``
  (dd.py:666) -> ``(nx, ny)`` image, ``A^T y / (na d_pix)``;
* ``dd_fp_fan_2d`` / ``dd_bp_fan_2d`` (dd.py:730, 739), the same with
  ``DSO, DSD`` for a flat detector at ``DSD`` from the source;
* ``dd_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0,
  sv=1.0, d_pix=1.0, sample=1)`` (dd.py:815) -> ``(na, nu, nv)``,
  ``A x * d_pix^2/(du dv)``, and ``dd_bp_cone_3d(sino, ang_arr, img_shape,
  DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0)`` (dd.py:829) ->
  ``A^T y / (na d_pix)``.  The defaults of ``sv`` differ between the two,
  as in the reference; ``sample`` up-samples the volume as ``np.kron`` does
  (dd.py:819-821).  Unlike the reference (dd.py:289, 388), any (nx, ny, nz)
  works, and the FP is the overlap integral the reference's sweep intends
  (its u buffer is not cleared between lines, dd.py:300, 335).

The translational square geometry: ``dd_fp_square(img, nu, nv, nsrc_p,
nsrc_z, DSO, DSD, du=1.0, dv=1.0, dsrc_p=1.0, dsrc_z=1.0, su=0.0, sv=0.0,
ssrc_p=0.0, ssrc_z=0.0, d_pix=1.0)`` (dd.py:903) -> ``(nsrc_p, nsrc_z, nv,
nu, 4)``, ``A x * d_pix^2/(du dv)``, and ``dd_bp_square(sino, img_shape,
DSO, DSD, ...)`` (dd.py:1104) -> ``(nx, ny, nz)``, ``A^T y`` unscaled; both
raise ``ValueError("nx must equal ny")`` as the reference does.

Inputs are cast to float32 as ``as_float32`` does (dd.py:29-36, 653); angles
too, so the per-view driving-axis choice (|sin| >= |cos|, dd.py:478) is made
on the reference's own float32 trig values.  ``sample`` is accepted and, as
in the reference's 2D functions, unused (dd.py:656-658).

Computation runs on the GPU (libvirgpu: gather-form kernels, see
csrc/dd2d.cu).  numpy in -> numpy out; torch CUDA tensors stay on the device.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _core
from .._lib import (DD2DGeom, DD3DGeom, DDSquareGeom, call, dd2d_workspace, dd3d_workspace,
                    dd_square_workspace)


def _geom(nx, ny, na, nu, du, su, d_pix, DSO=0.0, DSD=0.0, fan=0):
    return DD2DGeom(int(nx), int(ny), int(na), int(nu), _core.f32(du), _core.f32(su),
                    _core.f32(d_pix), _core.f32(DSO), _core.f32(DSD), int(fan))


def _fp(img, ang_arr, nu, du, su, d_pix, DSO, DSD, fan):
    dev = _core.device_of(img)
    x = _core.to_device(img, dev)
    if x.ndim != 2:
        raise ValueError("img must be 2D (nx, ny)")
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na = trig.numel() // 2
    g = _geom(x.shape[0], x.shape[1], na, nu, du, su, d_pix, DSO, DSD, fan)
    xT = x.t().contiguous()
    sino = _core.empty((na, nu), dev)
    call("vg_dd2d_fp", ctypes.byref(g), _core.ptr(x), _core.ptr(xT), _core.ptr(trig),
         _core.ptr(sino), _core.stream(dev))
    return _core.to_host_like(sino, img)


def _bp(sino, ang_arr, img_shape, du, su, d_pix, DSO, DSD, fan):
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    if y.ndim != 2:
        raise ValueError("sino must be 2D (na, nu)")
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na = trig.numel() // 2
    if y.shape[0] != na:
        raise ValueError(f"sino has {y.shape[0]} views, ang_arr {na}")
    nx, ny = (int(v) for v in img_shape)
    g = _geom(nx, ny, na, y.shape[1], du, su, d_pix, DSO, DSD, fan)
    img = _core.empty((nx, ny), dev)
    ws = dd2d_workspace(g, dev)
    call("vg_dd2d_bp", ctypes.byref(g), _core.ptr(y), _core.ptr(trig), _core.ptr(img),
         _core.ptr(ws), ws.numel(), _core.stream(dev))
    return _core.to_host_like(img, sino)


def dd_fp_par_2d(img, ang_arr, nu, du=1.0, su=0.0, d_pix=1.0, sample=1):
    return _fp(img, ang_arr, nu, du, su, d_pix, 0.0, 0.0, 0)


def dd_bp_par_2d(sino, ang_arr, img_shape, du=1.0, su=0.0, d_pix=1.0):
    return _bp(sino, ang_arr, img_shape, du, su, d_pix, 0.0, 0.0, 0)


def dd_fp_fan_2d(img, ang_arr, nu, DSO, DSD, du=1.0, su=0.0, d_pix=1.0):
    return _fp(img, ang_arr, nu, du, su, d_pix, DSO, DSD, 1)


def dd_bp_fan_2d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, su=0.0, d_pix=1.0):
    return _bp(sino, ang_arr, img_shape, du, su, d_pix, DSO, DSD, 1)


def _g3(shape, na, nu, nv, du, dv, su, sv, d_pix, DSO, DSD):
    f = _core.f32
    return DD3DGeom(int(shape[0]), int(shape[1]), int(shape[2]), int(na), int(nu), int(nv),
                    f(du), f(dv), f(su), f(sv), f(d_pix), f(DSO), f(DSD))


def dd_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=1.0, d_pix=1.0,
                  sample=1):
    dev = _core.device_of(img)
    x = _core.to_device(img, dev)
    if x.ndim != 3:
        raise ValueError("img must be 3D (nx, ny, nz)")
    d = _core.f32(d_pix)
    if sample != 1:
        for ax in range(3):
            x = x.repeat_interleave(int(sample), dim=ax)
        d = _core.f32(np.float32(d) / np.float32(sample))
        x = x.contiguous()
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na = trig.numel() // 2
    g = _g3(x.shape, na, nu, nv, du, dv, su, sv, d, DSO, DSD)
    ws = dd3d_workspace(g, dev)
    sino = _core.empty((na, int(nu), int(nv)), dev)
    call("vg_dd3d_fp", ctypes.byref(g), _core.ptr(x), _core.ptr(trig), _core.ptr(sino),
         _core.ptr(ws), ws.numel() * 4, _core.stream(dev))
    return _core.to_host_like(sino, img)


def dd_bp_cone_3d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    if y.ndim != 3:
        raise ValueError("sino must be 3D (na, nu, nv)")
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na = trig.numel() // 2
    if y.shape[0] != na:
        raise ValueError(f"sino has {y.shape[0]} views, ang_arr {na}")
    g = _g3(img_shape, na, y.shape[1], y.shape[2], du, dv, su, sv, d_pix, DSO, DSD)
    ws = dd3d_workspace(g, dev)
    vol = _core.empty(tuple(int(v) for v in img_shape), dev)
    call("vg_dd3d_bp", ctypes.byref(g), _core.ptr(y), _core.ptr(trig), _core.ptr(vol),
         _core.ptr(ws), ws.numel() * 4, _core.stream(dev))
    return _core.to_host_like(vol, sino)


def square_geom(img_shape, nu, nv, nsrc_p, nsrc_z, DSO, DSD, du=1.0, dv=1.0, dsrc_p=1.0,
                dsrc_z=1.0, su=0.0, sv=0.0, ssrc_p=0.0, ssrc_z=0.0, d_pix=1.0):
    """vg_dd_square_geom for an (n, n, nz) object (dd.py:907-909, 1110-1112)."""
    nx, ny, nz = (int(v) for v in img_shape)
    if nx != ny:
        raise ValueError("nx must equal ny")
    f = _core.f32
    return DDSquareGeom(nx, nz, int(nu), int(nv), int(nsrc_p), int(nsrc_z), f(DSO), f(DSD),
                        f(du), f(dv), f(dsrc_p), f(dsrc_z), f(su), f(sv), f(ssrc_p), f(ssrc_z),
                        f(d_pix))


def dd_fp_square(img, nu, nv, nsrc_p, nsrc_z, DSO, DSD, du=1.0, dv=1.0, dsrc_p=1.0, dsrc_z=1.0,
                 su=0.0, sv=0.0, ssrc_p=0.0, ssrc_z=0.0, d_pix=1.0):
    shape = tuple(img.shape) if hasattr(img, "shape") else np.shape(img)
    if len(shape) == 3 and shape[0] != shape[1]:
        raise ValueError("nx must equal ny")
    dev = _core.device_of(img)
    x = _core.to_device(img, dev)
    if x.ndim != 3:
        raise ValueError("img must be 3D (nx, ny, nz)")
    g = square_geom(x.shape, nu, nv, nsrc_p, nsrc_z, DSO, DSD, du, dv, dsrc_p, dsrc_z, su, sv,
                    ssrc_p, ssrc_z, d_pix)
    sino = _core.empty((int(nsrc_p), int(nsrc_z), int(nv), int(nu), 4), dev)
    call("vg_dd_square_fp", ctypes.byref(g), _core.ptr(x), _core.ptr(sino), _core.stream(dev))
    return _core.to_host_like(sino, img)


def dd_bp_square(sino, img_shape, DSO, DSD, du=1.0, dv=1.0, dsrc_p=1.0, dsrc_z=1.0, su=0.0,
                 sv=0.0, ssrc_p=0.0, ssrc_z=0.0, d_pix=1.0):
    nx, ny, nz = (int(v) for v in img_shape)
    if nx != ny:
        raise ValueError("nx must equal ny")
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    if y.ndim != 5 or y.shape[4] != 4:
        raise ValueError("sino must be (nsrc_p, nsrc_z, nv, nu, 4)")
    nsrc_p, nsrc_z, nv, nu, _ = y.shape
    g = square_geom(img_shape, nu, nv, nsrc_p, nsrc_z, DSO, DSD, du, dv, dsrc_p, dsrc_z, su, sv,
                    ssrc_p, ssrc_z, d_pix)
    ws = dd_square_workspace(g, dev)
    vol = _core.empty((nx, ny, nz), dev)
    call("vg_dd_square_bp", ctypes.byref(g), _core.ptr(y), _core.ptr(vol), _core.ptr(ws),
         ws.numel() * 8, _core.stream(dev))
    return _core.to_host_like(vol, sino)
