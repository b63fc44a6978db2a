"""2D parallel-beam Siddon projector, drop-in for vir ``sys_mat/fp_2d_par.py``.

* ``siddons_fp_2d(img, Angs, n_dets, d_det=1.0, d_pix=1.0)``
  (fp_2d_par.py:11-64) -> ``(na, n_dets)`` float32 sinogram of exact
  intersection-length line integrals.
* ``separable_footprint_fp_2d(img, Angs, n_dets, d_det=1.0, d_pix=1.0)``
  (fp_2d_par.py:67-125): rectangle footprint (the interval of the four
  projected corners) overlapped with each bin, divided by d_det; and
  ``separable_footprint_bp_2d`` its exact adjoint (GPU: ``vg_sf2d_*``).
* ``siddons_bp_2d(sino, Angs, img_shape, d_det=1.0, d_pix=1.0,
  method="scatter")``: its exact adjoint (no counterpart in fp_2d_par.py; the
  reference's backprojector for Siddon paths is the list scatter of
  projection_c.c:200-208), from the forward segments scattered into
  per-ray slots or (``method="gather"``) recomputed per pixel.

Geometry is FP64 with the reference's operation order, so every ray visits
the same voxels in the same order as the reference; trig uses the angle
array's own dtype exactly as ``np.cos(ang)`` in the reference loop (:23).
"""
from __future__ import annotations

from .. import _core
from .._lib import call


def siddons_fp_2d(img, Angs, n_dets, d_det=1.0, d_pix=1.0):
    dev = _core.device_of(img)
    x = _core.to_device(img, dev)
    if x.ndim != 2:
        raise ValueError("img must be 2D (nX, nY)")
    trig = _core.trig_cache.get(Angs, None, dev)
    na = trig.numel() // 2
    sino = _core.empty((na, int(n_dets)), dev)
    call("vg_siddon2d_fp", _core.ptr(x), x.shape[0], x.shape[1], _core.ptr(trig), na,
         int(n_dets), float(d_det), float(d_pix), _core.ptr(sino), _core.stream(dev))
    return _core.to_host_like(sino, img)


def siddons_bp_2d(sino, Angs, img_shape, d_det=1.0, d_pix=1.0, method="scatter"):
    """method="scatter" (default): the rays retrace their forward segments and
    write into per-(view, pixel) slots, then pixels gather the slots
    (vg_siddon2d_bp_scatter); method="gather": each pixel recomputes the
    crossings of its candidate rays (vg_siddon2d_bp, no workspace)."""
    import torch
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    trig = _core.trig_cache.get(Angs, None, dev)
    na = trig.numel() // 2
    if y.ndim != 2 or y.shape[0] != na:
        raise ValueError("sino must be (len(Angs), n_dets)")
    nx, ny = (int(v) for v in img_shape)
    img = _core.empty((nx, ny), dev)
    if method == "gather":
        call("vg_siddon2d_bp", _core.ptr(y), na, y.shape[1], _core.ptr(trig), nx, ny,
             float(d_det), float(d_pix), _core.ptr(img), _core.stream(dev))
        return _core.to_host_like(img, sino)
    if method != "scatter":
        raise ValueError("method must be 'scatter' or 'gather'")
    L = _core.load()
    nb = int(L.vg_siddon2d_bp_workspace_bytes(nx, ny, na, float(d_det), float(d_pix)))
    ws = torch.empty((nb + 3) // 4, dtype=torch.float32, device=dev)
    call("vg_siddon2d_bp_scatter", _core.ptr(y), na, y.shape[1], _core.ptr(trig), nx, ny,
         float(d_det), float(d_pix), _core.ptr(img), _core.ptr(ws), ws.numel() * 4,
         _core.stream(dev))
    return _core.to_host_like(img, sino)


def separable_footprint_fp_2d(img, Angs, n_dets, d_det=1.0, d_pix=1.0):
    from .sp import sf_fp_2d
    return sf_fp_2d(img, Angs, n_dets, d_det, d_pix, 0.0, 0.0, 0)


def separable_footprint_bp_2d(sino, Angs, img_shape, d_det=1.0, d_pix=1.0):
    from .sp import sf_bp_2d
    return sf_bp_2d(sino, Angs, img_shape, d_det, d_pix, 0.0, 0.0, 0)
