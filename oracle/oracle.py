"""FP64 oracle for the vir projector / reconstruction hot path.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the checker; the ``vir_gb300`` package
never imports it.

The projectors are a C restatement (``vir_oracle.c``, built by ``build()`` into
``oracle/_build/liboracle.so``) of the reference files cited there.  The ramp
filter and the SIRT loop are restated here in numpy (float64):

* ``ramp_filter`` / ``window_filter`` / ``filter_sino`` follow
  ``filtration.py:4-112``, ``:115-235`` and ``:238-309``;
* ``sirt`` follows ``sys_mat/sirt_dd.py:23-76`` (x0 = 1e-5, ``iters - 1``
  updates, divisions guarded where the weight is zero).

Trig tables follow the reference: the angle array is cast as the reference
casts it (float32 for the distance-driven functions, ``dd.py:29-36``; as given
for ``fp_2d_par.siddons_fp_2d``) and numpy's cos/sin of that dtype are passed to
C as float64.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int32)


def build(force: bool = False, ref: str = None) -> str:
    """Compile vir_oracle.c (and, when a vir source tree is given as ``ref``
    or by the VIR_REF environment variable, the reference's C into
    oracle/_ref) with the Makefile beside this file."""
    ref = ref or os.environ.get("VIR_REF", "")
    stale = force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "vir_oracle.c")))
    if stale or ref:
        subprocess.check_call(["make", "-s", "-C", _HERE, "all", f"REF={ref}"])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_siddon_fp_2d.argtypes = [_fp, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int, _dp]
        L.orc_siddon_bp_2d.argtypes = [_fp, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_siddon_trace_2d.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_double, ctypes.c_double, _ip,
                                          ctypes.POINTER(ctypes.c_uint64), _dp]
        L.orc_siddon_count_2d.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_siddon_count_2d.restype = ctypes.c_longlong
        L.orc_dd_fp_2d.argtypes = [ctypes.c_int, _fp, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_dd_bp_2d.argtypes = [ctypes.c_int, _fp, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_dd_fp_cone.argtypes = [_fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int] + \
            [ctypes.c_double] * 7 + [_dp]
        L.orc_dd_bp_cone.argtypes = [_fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int] + \
            [ctypes.c_double] * 7 + [_dp]
        L.orc_sf_fan_2d.argtypes = [ctypes.c_int, _fp, _dp, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                    ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 4
        L.orc_sf_par_rect_2d.argtypes = [ctypes.c_int, _fp, _dp, ctypes.c_int, ctypes.c_int, _dp,
                                         _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double]
        L.orc_dd_fp_square.argtypes = [_fp, _ip, _dp, _dp]
        L.orc_dd_bp_square.argtypes = [_fp, _ip, _dp, _dp]
        i, d = ctypes.c_int, ctypes.c_double
        L.orc_rd_2d.argtypes = [i, i, i, _fp, _dp, i, i, i, i, _dp, _dp, d, d, d, d, d]
        L.orc_rd_cone.argtypes = [i, i, _fp, _dp, i, i, i, i, i, i, _dp, _dp, d, d, d, d, d, d, d]
        L.orc_pd_2d.argtypes = [i, i, _fp, _dp, i, i, i, i, _dp, d, d, d, d, d]
        L.orc_pd_cone.argtypes = [i, _fp, _dp, i, i, i, i, i, i, _dp, d, d, d, d, d, d, d]
        L.orc_list_fp.argtypes = [_fp, _ip, _fp, _ip, ctypes.c_int, _dp]
        L.orc_list_bp.argtypes = [_fp, _ip, _fp, _ip, ctypes.c_int, ctypes.c_int, _dp]
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def num_threads() -> int:
    return lib().orc_num_threads()


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a, t):
    return a.ctypes.data_as(t)


def trig(angles, dtype=None):
    """cos/sin tables as the reference computes them (numpy, in the angle
    array's own dtype, or in ``dtype`` when the reference casts first)."""
    a = np.asarray(angles)
    if dtype is not None:
        a = a.astype(dtype)
    a = np.atleast_1d(a)
    return (np.ascontiguousarray(np.cos(a), dtype=np.float64),
            np.ascontiguousarray(np.sin(a), dtype=np.float64))


# --- Siddon 2D (sys_mat/fp_2d_par.py:11-64) -------------------------------

def siddons_fp_2d(img, Angs, n_dets, d_det=1.0, d_pix=1.0, mode="fp64"):
    """mode "fp64": FP64 accumulation.  mode "ref": float32-rounded
    accumulation, bit-identical to the reference's output."""
    img = _f32(img)
    nx, ny = img.shape
    c, s = trig(Angs)
    out = np.zeros((c.size, n_dets), np.float64)
    lib().orc_siddon_fp_2d(_ptr(img, _fp), nx, ny, _ptr(c, _dp), _ptr(s, _dp), c.size,
                           int(n_dets), float(d_det), float(d_pix), 1 if mode == "ref" else 0,
                           _ptr(out, _dp))
    return out


def siddons_bp_2d(sino, Angs, img_shape, d_det=1.0, d_pix=1.0):
    sino = _f32(sino)
    na, nd = sino.shape
    c, s = trig(Angs)
    out = np.zeros(img_shape, np.float64)
    lib().orc_siddon_bp_2d(_ptr(sino, _fp), na, nd, _ptr(c, _dp), _ptr(s, _dp),
                           int(img_shape[0]), int(img_shape[1]), float(d_det), float(d_pix),
                           _ptr(out, _dp))
    return out


def siddons_trace_2d(img_shape, Angs, n_dets, d_det=1.0, d_pix=1.0):
    """Per ray (count, hash of voxel sequence, FP64 length sum)."""
    c, s = trig(Angs)
    na = c.size
    cnt = np.zeros((na, n_dets), np.int32)
    h = np.zeros((na, n_dets), np.uint64)
    ln = np.zeros((na, n_dets), np.float64)
    lib().orc_siddon_trace_2d(int(img_shape[0]), int(img_shape[1]), _ptr(c, _dp), _ptr(s, _dp),
                              na, int(n_dets), float(d_det), float(d_pix), _ptr(cnt, _ip),
                              h.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), _ptr(ln, _dp))
    return cnt, h, ln


def siddons_count_2d(img_shape, Angs, n_dets, d_det=1.0, d_pix=1.0):
    c, s = trig(Angs)
    return int(lib().orc_siddon_count_2d(int(img_shape[0]), int(img_shape[1]), _ptr(c, _dp),
                                         _ptr(s, _dp), c.size, int(n_dets), float(d_det),
                                         float(d_pix)))


# --- distance-driven (sys_mat/dd.py) ---------------------------------------

def _dd_trig(ang_arr):
    return trig(ang_arr, np.float32)


def dd_fp_par_2d(img, ang_arr, nu, du=1.0, su=0.0, d_pix=1.0):
    img = _f32(img)
    c, s = _dd_trig(ang_arr)
    out = np.zeros((c.size, nu), np.float64)
    lib().orc_dd_fp_2d(0, _ptr(img, _fp), img.shape[0], img.shape[1], _ptr(c, _dp),
                       _ptr(s, _dp), c.size, int(nu), float(np.float32(du)),
                       float(np.float32(su)), float(np.float32(d_pix)), 0.0, 0.0, _ptr(out, _dp))
    return out


def dd_bp_par_2d(sino, ang_arr, img_shape, du=1.0, su=0.0, d_pix=1.0):
    sino = _f32(sino)
    c, s = _dd_trig(ang_arr)
    out = np.zeros(img_shape, np.float64)
    lib().orc_dd_bp_2d(0, _ptr(sino, _fp), sino.shape[0], sino.shape[1], _ptr(c, _dp),
                       _ptr(s, _dp), int(img_shape[0]), int(img_shape[1]), float(np.float32(du)),
                       float(np.float32(su)), float(np.float32(d_pix)), 0.0, 0.0, _ptr(out, _dp))
    return out


def dd_fp_fan_2d(img, ang_arr, nu, DSO, DSD, du=1.0, su=0.0, d_pix=1.0):
    img = _f32(img)
    c, s = _dd_trig(ang_arr)
    out = np.zeros((c.size, nu), np.float64)
    lib().orc_dd_fp_2d(1, _ptr(img, _fp), img.shape[0], img.shape[1], _ptr(c, _dp),
                       _ptr(s, _dp), c.size, int(nu), float(np.float32(du)),
                       float(np.float32(su)), float(np.float32(d_pix)), float(np.float32(DSO)),
                       float(np.float32(DSD)), _ptr(out, _dp))
    return out


def dd_bp_fan_2d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, su=0.0, d_pix=1.0):
    sino = _f32(sino)
    c, s = _dd_trig(ang_arr)
    out = np.zeros(img_shape, np.float64)
    lib().orc_dd_bp_2d(1, _ptr(sino, _fp), sino.shape[0], sino.shape[1], _ptr(c, _dp),
                       _ptr(s, _dp), int(img_shape[0]), int(img_shape[1]), float(np.float32(du)),
                       float(np.float32(su)), float(np.float32(d_pix)), float(np.float32(DSO)),
                       float(np.float32(DSD)), _ptr(out, _dp))
    return out


def dd_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=1.0, d_pix=1.0):
    img = _f32(img)
    c, s = _dd_trig(ang_arr)
    out = np.zeros((c.size, nu, nv), np.float64)
    f = lambda v: float(np.float32(v))
    lib().orc_dd_fp_cone(_ptr(img, _fp), *img.shape, _ptr(c, _dp), _ptr(s, _dp), c.size,
                         int(nu), int(nv), f(du), f(dv), f(su), f(sv), f(d_pix), f(DSO), f(DSD),
                         _ptr(out, _dp))
    return out


def dd_bp_cone_3d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    sino = _f32(sino)
    c, s = _dd_trig(ang_arr)
    out = np.zeros(img_shape, np.float64)
    f = lambda v: float(np.float32(v))
    lib().orc_dd_bp_cone(_ptr(sino, _fp), *sino.shape, _ptr(c, _dp), _ptr(s, _dp),
                         *[int(v) for v in img_shape], f(du), f(dv), f(su), f(sv), f(d_pix),
                         f(DSO), f(DSD), _ptr(out, _dp))
    return out


# --- translational square geometry (sys_mat/dd.py:895-1313) ----------------

def _square_args(n, nz, nu, nv, nsrc_p, nsrc_z, DSO, DSD, du, dv, dsrc_p, dsrc_z, su, sv,
                 ssrc_p, ssrc_z, d_pix):
    # dd.py:916-917 and 1120-1121 cast these to float32; su and sv enter as given
    f = lambda v: float(np.float32(v))
    dims = np.array([n, nz, nu, nv, nsrc_p, nsrc_z], np.int32)
    prm = np.array([f(DSO), f(DSD), f(du), f(dv), f(dsrc_p), f(dsrc_z), float(su), float(sv),
                    f(ssrc_p), f(ssrc_z), f(d_pix)], np.float64)
    return dims, prm


def dd_fp_square(img, nu, nv, nsrc_p, nsrc_z, DSO, DSD, du=1.0, dv=1.0, dsrc_p=1.0, dsrc_z=1.0,
                 su=0.0, sv=0.0, ssrc_p=0.0, ssrc_z=0.0, d_pix=1.0):
    img = _f32(img)
    nx, ny, nz = img.shape
    if nx != ny:
        raise ValueError("nx must equal ny")
    dims, prm = _square_args(nx, nz, nu, nv, nsrc_p, nsrc_z, DSO, DSD, du, dv, dsrc_p, dsrc_z,
                             su, sv, ssrc_p, ssrc_z, d_pix)
    out = np.zeros((nsrc_p, nsrc_z, nv, nu, 4), np.float64)
    lib().orc_dd_fp_square(_ptr(img, _fp), _ptr(dims, _ip), _ptr(prm, _dp), _ptr(out, _dp))
    return out


def dd_bp_square(sino, img_shape, DSO, DSD, du=1.0, dv=1.0, dsrc_p=1.0, dsrc_z=1.0, su=0.0,
                 sv=0.0, ssrc_p=0.0, ssrc_z=0.0, d_pix=1.0):
    sino = _f32(sino)
    nx, ny, nz = (int(v) for v in img_shape)
    if nx != ny:
        raise ValueError("nx must equal ny")
    nsrc_p, nsrc_z, nv, nu, _ = sino.shape
    dims, prm = _square_args(nx, nz, nu, nv, nsrc_p, nsrc_z, DSO, DSD, du, dv, dsrc_p, dsrc_z,
                             su, sv, ssrc_p, ssrc_z, d_pix)
    out = np.zeros((nx, ny, nz), np.float64)
    lib().orc_dd_bp_square(_ptr(sino, _fp), _ptr(dims, _ip), _ptr(prm, _dp), _ptr(out, _dp))
    return out


# --- ray-driven AW / Joseph (sys_mat/rd.py:40-790) --------------------------
# The angles are cast to float32 as as_float32 does (rd.py:453, 464, ...).

def _rd2(fan, joseph, bp, a, shape, angs, nu, du, su, d_pix, DSO, DSD):
    a = _f32(a)
    c, s = trig(angs, np.float32)
    f = lambda v: float(np.float32(v))
    nx, ny = shape
    out = np.zeros((nx, ny) if bp else (c.size, nu), np.float64)
    lib().orc_rd_2d(fan, int(joseph), bp, _ptr(a, _fp), _ptr(out, _dp), nx, ny, c.size, nu,
                    _ptr(c, _dp), _ptr(s, _dp), f(du), f(su), f(d_pix), f(DSO), f(DSD))
    return out


def aw_fp_par_2d(img, ang_arr, nu, du=1.0, su=0.0, d_pix=1.0, joseph=False):
    return _rd2(0, joseph, 0, img, np.shape(img), ang_arr, int(nu), du, su, d_pix, 0.0, 0.0)


def aw_bp_par_2d(sino, ang_arr, img_shape, du=1.0, su=0.0, d_pix=1.0, joseph=False):
    return _rd2(0, joseph, 1, sino, img_shape, ang_arr, np.shape(sino)[1], du, su, d_pix, 0.0, 0.0)


def aw_fp_fan_2d(img, ang_arr, nu, DSO, DSD, du=1.0, su=0.0, d_pix=1.0, joseph=False):
    return _rd2(1, joseph, 0, img, np.shape(img), ang_arr, int(nu), du, su, d_pix, DSO, DSD)


def aw_bp_fan_2d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, su=0.0, d_pix=1.0, joseph=False):
    return _rd2(1, joseph, 1, sino, img_shape, ang_arr, np.shape(sino)[1], du, su, d_pix, DSO, DSD)


def _rd3(joseph, bp, a, shape, angs, nu, nv, DSO, DSD, du, dv, su, sv, d_pix):
    a = _f32(a)
    c, s = trig(angs, np.float32)
    f = lambda v: float(np.float32(v))
    out = np.zeros(tuple(shape) if bp else (c.size, nu, nv), np.float64)
    lib().orc_rd_cone(int(joseph), bp, _ptr(a, _fp), _ptr(out, _dp), *[int(v) for v in shape],
                      c.size, nu, nv, _ptr(c, _dp), _ptr(s, _dp), f(du), f(dv), f(su), f(sv),
                      f(d_pix), f(DSO), f(DSD))
    return out


def aw_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0,
                  joseph=False):
    return _rd3(joseph, 0, img, np.shape(img), ang_arr, int(nu), int(nv), DSO, DSD, du, dv, su,
                sv, d_pix)


def aw_bp_cone_3d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0,
                  joseph=False):
    return _rd3(joseph, 1, sino, img_shape, ang_arr, np.shape(sino)[1], np.shape(sino)[2], DSO, DSD,
                du, dv, su, sv, d_pix)


# --- pixel-driven footprints (sys_mat/pd.py:56-480) --------------------------
# The angles are used as given (pd.py does not cast them).

def _pd2(fan, bp, a, shape, angs, nu, du, su, d_pix, DSO, DSD):
    a = _f32(a)
    ang = np.ascontiguousarray(np.atleast_1d(np.asarray(angs)), np.float64)
    nx, ny = shape
    out = np.zeros((nx, ny) if bp else (ang.size, nu), np.float64)
    lib().orc_pd_2d(fan, bp, _ptr(a, _fp), _ptr(out, _dp), nx, ny, ang.size, nu, _ptr(ang, _dp),
                    float(du), float(su), float(d_pix), float(DSO), float(DSD))
    return out


def pd_fp_par_2d(img, ang_arr, nu, du=1.0, su=0.0, d_pix=1.0):
    return _pd2(0, 0, img, np.shape(img), ang_arr, int(nu), du, su, d_pix, 0.0, 0.0)


def pd_bp_par_2d(sino, ang_arr, img_shape, du=1.0, su=0.0, d_pix=1.0):
    return _pd2(0, 1, sino, img_shape, ang_arr, np.shape(sino)[1], du, su, d_pix, 0.0, 0.0)


def pd_fp_fan_2d(img, ang_arr, nu, DSO, DSD, du=1.0, su=0.0, d_pix=1.0):
    return _pd2(1, 0, img, np.shape(img), ang_arr, int(nu), du, su, d_pix, DSO, DSD)


def pd_bp_fan_2d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, su=0.0, d_pix=1.0):
    return _pd2(1, 1, sino, img_shape, ang_arr, np.shape(sino)[1], du, su, d_pix, DSO, DSD)


def _pd3(bp, a, shape, angs, nu, nv, DSO, DSD, du, dv, su, sv, d_pix):
    a = _f32(a)
    ang = np.ascontiguousarray(np.atleast_1d(np.asarray(angs)), np.float64)
    out = np.zeros(tuple(shape) if bp else (ang.size, nu, nv), np.float64)
    lib().orc_pd_cone(bp, _ptr(a, _fp), _ptr(out, _dp), *[int(v) for v in shape], ang.size, nu, nv,
                      _ptr(ang, _dp), float(du), float(dv), float(su), float(sv), float(d_pix),
                      float(DSO), float(DSD))
    return out


def pd_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    return _pd3(0, img, np.shape(img), ang_arr, int(nu), int(nv), DSO, DSD, du, dv, su, sv, d_pix)


def pd_bp_cone_3d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    return _pd3(1, sino, img_shape, ang_arr, np.shape(sino)[1], np.shape(sino)[2], DSO, DSD, du, dv,
                su, sv, d_pix)


# --- separable footprint (sys_mat/sp.py:12-87, fp_2d_par.py:67-125) -------

def sf_fp_fan_2d(img, angs, nu, DSO, DSD, du=1.0, d_pix=1.0):
    img = _f32(img)
    c, s = trig(angs)
    out = np.zeros((c.size, nu), np.float64)
    lib().orc_sf_fan_2d(0, _ptr(img, _fp), _ptr(out, _dp), img.shape[0], img.shape[1],
                        _ptr(c, _dp), _ptr(s, _dp), c.size, int(nu), float(DSO), float(DSD),
                        float(du), float(d_pix))
    return out


def sf_bp_fan_2d(sino, angs, img_shape, DSO, DSD, du=1.0, d_pix=1.0):
    sino = _f32(sino)
    c, s = trig(angs)
    out = np.zeros(img_shape, np.float64)
    lib().orc_sf_fan_2d(1, _ptr(sino, _fp), _ptr(out, _dp), int(img_shape[0]),
                        int(img_shape[1]), _ptr(c, _dp), _ptr(s, _dp), c.size, sino.shape[1],
                        float(DSO), float(DSD), float(du), float(d_pix))
    return out


def separable_footprint_fp_2d(img, Angs, n_dets, d_det=1.0, d_pix=1.0):
    img = _f32(img)
    c, s = trig(Angs)
    out = np.zeros((c.size, n_dets), np.float64)
    lib().orc_sf_par_rect_2d(0, _ptr(img, _fp), _ptr(out, _dp), img.shape[0], img.shape[1],
                             _ptr(c, _dp), _ptr(s, _dp), c.size, int(n_dets), float(d_det),
                             float(d_pix))
    return out


def separable_footprint_bp_2d(sino, Angs, img_shape, d_det=1.0, d_pix=1.0):
    sino = _f32(sino)
    c, s = trig(Angs)
    out = np.zeros(img_shape, np.float64)
    lib().orc_sf_par_rect_2d(1, _ptr(sino, _fp), _ptr(out, _dp), int(img_shape[0]),
                             int(img_shape[1]), _ptr(c, _dp), _ptr(s, _dp), c.size,
                             sino.shape[1], float(d_det), float(d_pix))
    return out


# --- list projection (projection/projection_c.c:126-219) -------------------

def list_fp(x, ind, length, off):
    x = _f32(x).ravel()
    ind = np.ascontiguousarray(ind, np.int32)
    length = _f32(length)
    off = np.ascontiguousarray(off, np.int32)
    out = np.zeros(off.size - 1, np.float64)
    lib().orc_list_fp(_ptr(x, _fp), _ptr(ind, _ip), _ptr(length, _fp), _ptr(off, _ip),
                      off.size - 1, _ptr(out, _dp))
    return out


def list_bp(sino, ind, length, off, nvox):
    sino = _f32(sino).ravel()
    ind = np.ascontiguousarray(ind, np.int32)
    length = _f32(length)
    off = np.ascontiguousarray(off, np.int32)
    out = np.zeros(int(nvox), np.float64)
    lib().orc_list_bp(_ptr(sino, _fp), _ptr(ind, _ip), _ptr(length, _fp), _ptr(off, _ip),
                      off.size - 1, int(nvox), _ptr(out, _dp))
    return out


# --- ramp filter (filtration.py) -------------------------------------------

def ramp_filter(nu, du=1.0, cutoff=0.5, real_space=True):
    """Half-spectrum ramp filter and its frequencies (filtration.py:4-112)
    with zero padding to the next power of two >= 2*nu."""
    nfu = int(2 ** np.ceil(np.log2(2 * nu)))
    f = np.fft.rfftfreq(nfu, d=du)
    if real_space:
        k = np.fft.fftfreq(nfu, d=1.0 / nfu)
        h = np.zeros(nfu)
        h[0] = 1.0 / (4.0 * du ** 2)
        h[1::2] = -1.0 / (np.pi ** 2 * du ** 2 * k[1::2] ** 2)
        H = du * np.real(np.fft.rfft(h))
    else:
        H = np.abs(f)
    H[np.abs(f) > cutoff * (1.0 / du)] = 0.0
    return H, f


def window_filter(H, f, du=1.0, filter_type="ramp", cutoff=0.5, sigma=0.5):
    """filtration.py:115-235."""
    f_c = cutoff * (1.0 / du)
    fn = f / f_c
    valid = np.abs(f) <= f_c
    W = np.zeros_like(f)
    if filter_type in ("ram-lak", "ramp"):
        return H
    if filter_type == "hann":
        W[valid] = 0.5 + 0.5 * np.cos(np.pi * fn[valid])
    elif filter_type == "hamming":
        W[valid] = 0.54 + 0.46 * np.cos(np.pi * fn[valid])
    elif filter_type == "blackman":
        W[valid] = 0.42 + 0.5 * np.cos(np.pi * fn[valid]) + 0.08 * np.cos(2 * np.pi * fn[valid])
    elif filter_type == "shepp-logan":
        W[0] = 1.0
        m = valid & (f != 0)
        W[m] = np.sin(np.pi * f[m] / (2 * f_c)) / (np.pi * f[m] / (2 * f_c))
    elif filter_type == "cosine":
        W[valid] = np.cos(np.pi * fn[valid] / 2.0)
    elif filter_type == "gaussian":
        W = np.exp(-0.5 * (f / sigma) ** 2)
    else:
        raise ValueError(f"Unknown filter type: {filter_type}")
    return H * W


def filter_sino(sino, du=1.0, filter_type="ramp", cutoff=0.5, real_space=True):
    """filtration.py:238-309: rFFT along the last axis at the padded length,
    multiplied by 2H, inverse, cropped to nu."""
    if filter_type is None:
        return sino
    nu = sino.shape[-1]
    z = int(2 ** np.ceil(np.log2(2 * nu)))
    H, f = ramp_filter(nu, du=du, cutoff=cutoff, real_space=real_space)
    H = window_filter(H, f, du=du, filter_type=filter_type, cutoff=cutoff)
    F = np.fft.rfft(np.asarray(sino, np.float64), axis=-1, n=z)
    F *= 2.0 * H
    return np.fft.irfft(F, n=z, axis=-1)[..., :nu]


# --- FBP / FDK: weights and pixel-driven backprojection ---------------------
#
# vir's fan FBP (processing/reconstruction.py:7-67) cannot run (stale imports
# and keyword arguments), but its parts can: the pre-weight cosine_weighting
# (:99-107) and the 1/L^2-weighted linear-interpolation pixel backprojection
# fan_backproject_hsieh (processing/proj2.py:580-616).  Both are restated
# here as written and pinned against the reference's own functions
# (golden fixtures).  The product reconstructs on vir's flat-detector
# distance-driven geometry instead of Hsieh's equiangular one; fbp2d_bp and
# fdk restate that geometry with the same weights and the same interpolation
# step (_lerp), in float64.

def cosine_weighting(sino, cols, src_iso, det_off=0.0, equispaced=False):
    """processing/reconstruction.py:99-107: each detector column times
    (src_iso - det_off cols / src_iso) / sqrt(src_iso^2 + cols^2)
    (equispaced: cols are positions at the isocentre) or
    src_iso cos(cols) - det_off sin(cols) (equiangular: cols are angles)."""
    cols = np.asarray(cols, np.float64)
    if equispaced:
        w = (src_iso - det_off * cols / src_iso) / np.sqrt(src_iso ** 2 + cols ** 2)
    else:
        w = src_iso * np.cos(cols) - det_off * np.sin(cols)
    return w * np.asarray(sino, np.float64)


def _lerp(row, t, clip):
    """(1 - a) row[j] + a row[j + 1] with j = floor(t), a = t - j
    (proj2.py:607-613).  clip: indices clipped to the row (Hsieh's rule);
    else samples outside the row are zero (the flat-detector kernels)."""
    j = np.floor(t).astype(np.int64)
    a = t - j
    n = row.shape[-1]
    if clip:
        return (1.0 - a) * row[..., np.clip(j, 0, n - 1)] + a * row[..., np.clip(j + 1, 0, n - 1)]
    pad = np.zeros(row.shape[:-1] + (n + 2,), np.float64)
    pad[..., 1:-1] = row
    v0 = pad[..., np.clip(j, -1, n) + 1]
    v1 = pad[..., np.clip(j + 1, -1, n) + 1]
    return v0 + a * (v1 - v0)


def fan_backproject_hsieh(Sino, Views, Cols, src_iso, dPixels=(1.0, 1.0), nPixels=(512, 512),
                          detOff=0.0, pixOff=(0.0, 0.0)):
    """processing/proj2.py:580-616 (pixel grid of calc_image_arrays,
    proj2.py:912-923): filtered rows times cos^2(Cols), then per view the
    equiangular column of every pixel by arctan, linear interpolation with
    clipped indices, weight 1 / (src_iso - X cos + Y sin)^2."""
    Sino = np.asarray(Sino, np.float64)
    nViews, nRows, nCols = Sino.shape
    Cols = np.asarray(Cols, np.float64)
    dCol = Cols[1] - Cols[0]
    Col0 = Cols[0]
    Sino = Sino * (np.cos(Cols) ** 2)
    sv, cv = np.sin(Views), np.cos(Views)
    nX, nY = nPixels
    dX, dY = dPixels
    X = np.linspace(1 - nX, nX - 1, nX) * dX / 2.0
    Y = np.linspace(1 - nY, nY - 1, nY) * dY / 2.0
    X, Y = np.meshgrid(X + pixOff[1], Y + pixOff[0])
    image = np.zeros((nRows, nX, nY))
    for l in range(nViews):
        Yf = src_iso - X * cv[l] + Y * sv[l]
        t = (np.arctan((X * sv[l] + Y * cv[l] - detOff) / Yf) - Col0) / dCol
        for k in range(nRows):
            image[k] += _lerp(Sino[l, k], t, clip=True) / Yf ** 2
    return np.squeeze(image)


def fan_preweight(nu, du=1.0, su=0.0, DSO=1.0, DSD=1.0):
    """The equispaced cosine_weighting of the flat detector: bin centres
    du (j - nu/2 + 0.5 + su) scaled to the isocentre by DSO / DSD."""
    s = du * (np.arange(nu) - nu / 2.0 + 0.5 + su) * DSO / DSD
    return cosine_weighting(np.ones(nu), s, DSO, equispaced=True)


def fbp2d_bp(q, ang_arr, img_shape, fan=False, DSO=0.0, DSD=0.0, du=1.0, su=0.0, d_pix=1.0):
    """Pixel-driven FBP backprojection on vir's distance-driven geometry
    (dd.py:486-494, 527-585; source direction (cos, sin), detector axis
    (-sin, cos)): img = pi / (2 na) sum_views Q(s) / U^2 with o = c x + s y,
    p = -s x + c y; parallel s = p, U = 1; fan s = DSD p / (DSO - o),
    U = (DSO - o) / DSO (the 1/L^2 weight of proj2.py:606-613 normalised at
    the isocentre); Q linear between bin centres du (j - nu/2 + 0.5 + su),
    zero outside the detector.  Geometry values are taken as given (pass the
    float32-rounded values a float32 kernel sees)."""
    q = np.asarray(q, np.float64)
    c, s = _dd_trig(ang_arr)
    na, nu = q.shape
    nx, ny = img_shape
    x = (d_pix * (np.arange(nx) + 0.5 - 0.5 * nx))[:, None]
    y = (d_pix * (np.arange(ny) + 0.5 - 0.5 * ny))[None, :]
    img = np.zeros((nx, ny))
    off = 0.5 * nu - 0.5 - su
    for ia in range(na):
        p = -s[ia] * x + c[ia] * y
        w = 1.0
        if fan:
            d = DSO - (c[ia] * x + s[ia] * y)
            p = DSD * p / d
            w = (DSO / d) ** 2
        img += w * _lerp(q[ia], p / du + off, clip=False)
    return img * (np.pi / (2.0 * na))


def fbp_2d(sino, ang_arr, img_shape, fan=False, DSO=0.0, DSD=0.0, du=1.0, su=0.0, d_pix=1.0,
           filter_type="ramp", cutoff=0.5, real_space=True):
    """Full-scan FBP: (fan) the equispaced pre-weight, filter_sino at the bin
    pitch (fan: at the isocentre, du DSO / DSD), fbp2d_bp."""
    y = np.asarray(sino, np.float64)
    if fan:
        y = y * fan_preweight(y.shape[1], du, su, DSO, DSD)[None, :]
        q = filter_sino(y, du * DSO / DSD, filter_type, cutoff, real_space)
    else:
        q = filter_sino(y, du, filter_type, cutoff, real_space)
    return fbp2d_bp(q, ang_arr, img_shape, fan, DSO, DSD, du, su, d_pix)


def fbp_par_dd(sino, ang_arr, img_shape, du=1.0, su=0.0, d_pix=1.0, filter_type="ramp",
               cutoff=0.5, real_space=True):
    """vir's working parallel FBP over 180 degrees: (pi / 2)
    dd_bp_par_2d(filter_sino(y)) (filtration.py:238-309, dd.py:666-672)."""
    q = filter_sino(np.asarray(sino, np.float64), du, filter_type, cutoff, real_space)
    return (np.pi / 2.0) * dd_bp_par_2d(q.astype(np.float32), ang_arr, img_shape, du, su, d_pix)


def fdk_preweight(nu, nv, du, dv, su, sv, DSD):
    """FDK pre-weight DSD / sqrt(DSD^2 + u^2 + v^2) at the (u, v) bin
    centres: cosine_weighting's equispaced weight on the flat 2D detector."""
    u = du * (np.arange(nu) - 0.5 * nu + 0.5 + su)
    v = dv * (np.arange(nv) - 0.5 * nv + 0.5 + sv)
    return DSD / np.sqrt(DSD ** 2 + u[:, None] ** 2 + v[None, :] ** 2)


def fdk(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0,
        filter_type="ramp", cutoff=0.5, real_space=True, box=None):
    """FDK on the circular cone geometry of dd_fp_cone_3d, sino (na, nu, nv):
    pre-weight (fdk_preweight), filter_sino along u at the isocentre pitch
    du DSO / DSD, then vol = pi / (2 na) sum_views Q(u, v) / U^2 with
    o = c x + s y, p = -s x + c y, U = (DSO - o) / DSO, u = DSD p / (DSO - o),
    v = DSD z / (DSO - o), Q bilinear between bin centres (zero outside).
    ``box`` = ((x0, x1), (y0, y1), (z0, z1)) voxel index ranges returns that
    sub-volume only; per view only the detector rows the box reaches are
    filtered (rows are filtered independently, so this is exact)."""
    sino = np.asarray(sino)
    na, nu, nv = sino.shape
    nx, ny, nz = img_shape
    box = box or ((0, nx), (0, ny), (0, nz))
    (x0, x1), (y0, y1), (z0, z1) = box
    c, s = _dd_trig(ang_arr)
    X = (d_pix * (np.arange(x0, x1) + 0.5 - 0.5 * nx))[:, None, None]
    Y = (d_pix * (np.arange(y0, y1) + 0.5 - 0.5 * ny))[None, :, None]
    Z = (d_pix * (np.arange(z0, z1) + 0.5 - 0.5 * nz))[None, None, :]
    W = fdk_preweight(nu, nv, du, dv, su, sv, DSD)
    pitch = du * DSO / DSD
    iu_off, iv_off = 0.5 * nu - 0.5 - su, 0.5 * nv - 0.5 - sv
    vol = np.zeros((x1 - x0, y1 - y0, z1 - z0))
    for ia in range(na):
        d = DSO - (c[ia] * X + s[ia] * Y)
        tu = DSD * (-s[ia] * X + c[ia] * Y) / d / du + iu_off
        tv = DSD * Z / d / dv + iv_off
        tu, tv = np.broadcast_arrays(tu, tv)
        k0 = max(int(np.floor(tv.min())), 0)
        k1 = min(int(np.floor(tv.max())) + 2, nv)
        if k1 <= k0:
            continue
        rows = (sino[ia, :, k0:k1].astype(np.float64) * W[:, k0:k1]).T   # (rows, nu)
        Q = filter_sino(rows, pitch, filter_type, cutoff, real_space)    # (rows, nu)
        # bilinear: along u in each needed row, then along v
        ju = np.floor(tu).astype(np.int64)
        au = tu - ju
        jv = np.floor(tv).astype(np.int64)
        av = tv - jv
        padQ = np.zeros((nv + 2, nu + 2))
        padQ[k0 + 1:k1 + 1, 1:-1] = Q
        cu0, cu1 = np.clip(ju, -1, nu) + 1, np.clip(ju + 1, -1, nu) + 1
        cv0, cv1 = np.clip(jv, -1, nv) + 1, np.clip(jv + 1, -1, nv) + 1
        q00, q10 = padQ[cv0, cu0], padQ[cv0, cu1]   # (v = jv, u = ju / ju + 1)
        q01, q11 = padQ[cv1, cu0], padQ[cv1, cu1]   # (v = jv + 1)
        a = q00 + av * (q01 - q00)
        b = q10 + av * (q11 - q10)
        vol += (a + au * (b - a)) * (DSO / d) ** 2
    return vol * (np.pi / (2.0 * na))


# --- 3D cone-beam separable footprint (SF-TR) ------------------------------
#
# vir's sys_mat/sp.py:93-211 (CTGeometry, footprint1D, forward_project,
# back_project) is a toy with no rotation angles.  This restates the
# separable-footprint cone projector it stands in for -- trapezoid
# transaxial and rectangle axial footprints with the "A2" amplitude of
# Long, Fessler & Balter, "3D forward and back-projection for X-ray CT using
# separable footprints", IEEE TMI 29(11), 2010 -- on vir's circular cone
# geometry of dd_fp_cone_3d (dd.py:815-888): source at DSO (cos b, sin b),
# o = c x + s y, p = -s x + c y, u = DSD p / (DSO - o), v = DSD z / (DSO - o),
# cells u_j = du (j - nu/2 + su), v_l = dv (l - nv/2 + sv) (edges), volume
# (nx, ny, nz) of cubic voxels d_pix, sinogram (na, nu, nv).  Per voxel and
# view:
#   F1: trapezoid through the sorted projections tau0..tau3 of the column's
#       four corners, height 1, averaged over each u cell;
#   F2: rectangle [M (z - d/2), M (z + d/2)], M = DSD / (DSO - o_centre),
#       averaged over each v cell;
#   amplitude l_phi0 l_theta: l_phi0 = d |r| / max(|r_x|, |r_y|) with r the
#       transaxial ray from the source to the column centre, and
#       l_theta = sqrt(1 + v_c^2 / (u_c^2 + DSD^2)) at the cell centre.
# FP: sino[j, l] = sum_voxels f l_phi0 l_theta(j, l) F1(j) F2(l) (line
# integrals); BP: its exact adjoint.  numpy float64, one view at a time.
# The geometry agrees with vir's detector-area-averaged analytic cone-beam
# sphere (analytic_sino.py:563, a golden fixture): the projection of a
# voxelised sphere is within the voxelisation error of it.

def _sf_trap_cum(u, t0, t1, t2, t3):
    """Integral of the unit-height trapezoid (t0, t1, t2, t3) from -inf to u."""
    r1 = np.maximum(t1 - t0, 1e-300)
    r3 = np.maximum(t3 - t2, 1e-300)
    a = np.where(u <= t0, 0.0, np.where(u <= t1, (u - t0) ** 2 / (2 * r1), 0.0))
    b = np.where((u > t1) & (u <= t2), 0.5 * (t1 - t0) + (u - t1), 0.0)
    c = np.where((u > t2) & (u <= t3), 0.5 * (t1 - t0) + (t2 - t1) + 0.5 * (t3 - t2)
                 - (t3 - u) ** 2 / (2 * r3), 0.0)
    d = np.where(u > t3, 0.5 * (t1 - t0) + (t2 - t1) + 0.5 * (t3 - t2), 0.0)
    return a + b + c + d


def _sf_cone_view(c, s, shape, nu, nv, du, dv, su, sv, d_pix, DSO, DSD):
    """Cells and weights of one view: per voxel and (u cell t, v cell r) the
    cell (j, l) and weight, flattened voxel-major."""
    nx, ny, nz = shape
    d = d_pix
    X = (d * (np.arange(nx) + 0.5 - 0.5 * nx))[:, None]
    Y = (d * (np.arange(ny) + 0.5 - 0.5 * ny))[None, :]
    h = 0.5 * d
    us = []
    for ex in (-h, h):
        for ey in (-h, h):
            o = c * (X + ex) + s * (Y + ey)
            p = -s * (X + ex) + c * (Y + ey)
            us.append(DSD * p / (DSO - o))
    tau = np.sort(np.stack(np.broadcast_arrays(*us), -1), axis=-1)       # (nx, ny, 4)
    oc = c * X + s * Y
    M = np.broadcast_to(DSD / (DSO - oc), (nx, ny))
    rx, ry = np.broadcast_arrays(X - DSO * c, Y - DSO * s)
    lphi = d * np.sqrt(rx ** 2 + ry ** 2) / np.maximum(np.abs(rx), np.abs(ry))
    U0, V0 = du * (-0.5 * nu + su), dv * (-0.5 * nv + sv)
    j0 = np.floor((tau[..., 0] - U0) / du).astype(np.int64)
    j3 = np.floor((tau[..., 3] - U0) / du).astype(np.int64)
    K = int((j3 - j0).max()) + 1
    uj, uw = [], []
    for t in range(K):
        j = j0 + t
        a = U0 + du * j
        tt = np.moveaxis(tau, -1, 0)
        w = (_sf_trap_cum(a + du, *tt) - _sf_trap_cum(a, *tt)) / du
        w = np.where((j >= 0) & (j < nu) & (j <= j3), w * lphi, 0.0)
        uj.append(np.clip(j, 0, nu - 1))
        uw.append(w)
    uj, uw = np.stack(uj, -1), np.stack(uw, -1)                          # (nx, ny, K)
    Z = d * (np.arange(nz) - 0.5 * nz)                                    # slice lower edges
    vs = M[..., None] * Z[None, None, :]
    ve = M[..., None] * (Z + d)[None, None, :]
    q0 = np.floor((vs - V0) / dv).astype(np.int64)
    q1 = np.floor((ve - V0) / dv).astype(np.int64)
    R = int((q1 - q0).max()) + 1
    vq, vw = [], []
    for r in range(R):
        q = q0 + r
        lo, hi = V0 + dv * q, V0 + dv * (q + 1)
        ov = (np.minimum(ve, hi) - np.maximum(vs, lo)) / dv
        ov = np.where((q >= 0) & (q < nv) & (q <= q1) & (ov > 0), ov, 0.0)
        vq.append(np.clip(q, 0, nv - 1))
        vw.append(ov)
    vq, vw = np.stack(vq, -1), np.stack(vw, -1)                          # (nx, ny, nz, R)
    uc = U0 + du * (np.arange(nu) + 0.5)
    vc = V0 + dv * (np.arange(nv) + 0.5)
    lth = np.sqrt(1.0 + vc[None, :] ** 2 / (uc[:, None] ** 2 + DSD ** 2))  # (nu, nv)
    J = np.broadcast_to(uj[:, :, None, :, None], (nx, ny, nz, K, R))
    Q = np.broadcast_to(vq[:, :, :, None, :], (nx, ny, nz, K, R))
    W = uw[:, :, None, :, None] * vw[:, :, :, None, :] * lth[J, Q]
    return J.reshape(nx * ny * nz, -1), Q.reshape(nx * ny * nz, -1), W.reshape(nx * ny * nz, -1)


def sf_fp_cone_3d(img, ang_arr, nu, nv, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    f = np.asarray(img, np.float64)
    c_, s_ = _dd_trig(ang_arr)
    out = np.zeros((c_.size, nu, nv))
    fv = f.reshape(-1, 1)
    for ia in range(c_.size):
        J, Q, W = _sf_cone_view(c_[ia], s_[ia], f.shape, nu, nv, du, dv, su, sv, d_pix, DSO, DSD)
        np.add.at(out[ia], (J.ravel(), Q.ravel()), (W * fv).ravel())
    return out


def sf_bp_cone_3d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0):
    y = np.asarray(sino, np.float64)
    c_, s_ = _dd_trig(ang_arr)
    na, nu, nv = y.shape
    vol = np.zeros(int(np.prod(img_shape)))
    for ia in range(na):
        J, Q, W = _sf_cone_view(c_[ia], s_[ia], tuple(img_shape), nu, nv, du, dv, su, sv, d_pix,
                                DSO, DSD)
        vol += (W * y[ia][J, Q]).sum(-1)
    return vol.reshape(img_shape)


# --- SIRT (sys_mat/sirt_dd.py:23-76) ---------------------------------------

def sirt(sino, fp, bp, img_shape, gamma=1.0, iters=100, x0=1e-5, W_sino=None, W_img=None):
    """x <- x + gamma * (BP((y - FP x) / W_sino)) / W_img with W_sino = FP 1
    and W_img = BP 1, run for ``iters - 1`` updates as ``range(1, iters)``
    does.  ``fp``/``bp`` are FP64 projector callables of this module."""
    sino = np.asarray(sino, np.float64)
    if W_sino is None:
        W_sino = fp(np.ones(img_shape, np.float32))
    if W_img is None:
        W_img = bp(np.ones(sino.shape, np.float32))
    x = np.zeros(img_shape, np.float64) + x0
    for _ in range(1, iters):
        est = fp(x.astype(np.float32))
        r = np.where(W_sino != 0.0, (sino - est) / np.where(W_sino != 0.0, W_sino, 1.0), est)
        upd = bp(r.astype(np.float32))
        upd = np.where(W_img != 0.0, upd / np.where(W_img != 0.0, W_img, 1.0), upd)
        x = x + gamma * upd
    return x


# --- TV primal-dual (tv.py:98-294), numpy float64 -----------------------------

def tv_grad(x):
    """tv.py:207-211"""
    x = np.asarray(x, np.float64)
    return np.stack([np.roll(x, -1, 0) - x, np.roll(x, -1, 1) - x])


def tv_div(z):
    """tv.py:220-224"""
    z = np.asarray(z, np.float64)
    return (z[0] - np.roll(z[0], 1, 0)) + (z[1] - np.roll(z[1], 1, 1))


def tv_grad_abs(x):
    """tv.py:200-204"""
    x = np.asarray(x, np.float64)
    return np.stack([x + np.roll(x, -1, 0), x + np.roll(x, -1, 1)])


def tv_div_abs(z):
    """tv.py:214-218"""
    z = np.asarray(z, np.float64)
    return (z[0] + np.roll(z[0], 1, 0)) + (z[1] + np.roll(z[1], 1, 1))


def tv_project(AA):
    """pyT (tv.py:98-184) for 2 x 1 pairs: the largest singular value is |a|,
    the other 0, so the projection is a / max(1, |a|)."""
    AA = np.asarray(AA, np.float64)
    return AA / np.maximum(1.0, np.sqrt(AA[0] ** 2 + AA[1] ** 2))


def tv_pdhg(g, fp, bp, img_shape, lam=1.0, theta=1.0, iters=100):
    """The solver loop of tv.py:262-294 (sigma_q = 0 where A 1 = 0)."""
    g = np.asarray(g, np.float64)
    A1 = fp(np.ones(img_shape, np.float32))
    sigma_z = 1.0 / tv_grad_abs(np.ones(img_shape))
    sigma_q = np.where(A1 != 0, 1.0 / np.where(A1 != 0, A1, 1.0), 0.0)
    tau = 1.0 / (bp(np.ones(g.shape, np.float32)) + tv_div_abs(np.ones((2,) + tuple(img_shape))))
    u = np.zeros(img_shape)
    ub = np.zeros(img_shape)
    z = np.zeros((2,) + tuple(img_shape))
    q = np.zeros(g.shape)
    for _ in range(iters):
        z = tv_project(z + sigma_z * tv_grad(ub))
        q = (q + sigma_q * (fp(ub.astype(np.float32)) - g)) / (1 + sigma_q * lam)
        u_prev = u
        u = u + tau * (tv_div(z) - bp(q.astype(np.float32)))
        ub = u + theta * (u - u_prev)
    return u


# ---- beam-hardening pre-correction (processing/beamhard.py) ------------------
# The reference's corrections are numpy / scipy expressions; restated here as
# the checker, with numpy's own types (float32 sinograms stay float32 where
# the reference's expression keeps them so).

def bh_poly(line_ints, coefs, mu):
    """beamhard_cor (beamhard.py:39-47): mu (c0 t^2 + c1 t + c2), t = x / mu."""
    t = np.asarray(line_ints) / mu
    return mu * (coefs[0] * t ** 2 + coefs[1] * t + coefs[2])


def bh_spectrum_table(energies, counts, atten_eff, attens):
    """The interp1d table of beamhard_cor_table (beamhard.py:30-34):
    (x, y) = (polyenergetic, monoenergetic) water line integrals of 1000
    thicknesses in [0, 80]."""
    pl = np.linspace(0, 80, 1000)
    pp = -1.0 * np.log(np.sum(counts * np.exp(-1.0 * np.outer(pl, attens)), axis=1)
                       / np.sum(counts)) / atten_eff
    return pp * atten_eff, pl * atten_eff


def bh_table(line_ints, energies, counts, atten_eff, attens):
    """beamhard_cor_table (beamhard.py:16-36): linear interp1d of the table
    at line_ints.clip(0); raises ValueError outside the table as interp1d."""
    from scipy import interpolate
    x, y = bh_spectrum_table(energies, counts, atten_eff, attens)
    return interpolate.interp1d(x, y)(np.asarray(line_ints).clip(0))


def bh_lut(line_ints, coefs, mu):
    """Lookup-table correction of tests/Test_Beamhard/beamhard_test.py:26-27."""
    li = np.asarray(line_ints)
    return li * np.interp(li / mu, np.linspace(0, 40, 4001), coefs)


def bh_sphere_fan_coefs(energies, counts, gammas, src_iso, atten_eff, attens):
    """beamhard_coefs2's fan branch (beamhard.py:50-78): chord lengths of a
    centred sphere of radius 20 (intersection_sino.py:105-121 at view 0) for
    the first 256 of 512 fan angles, polyenergetic path lengths, quadratic fit."""
    r = 20.0
    xi = src_iso * np.sin(gammas)
    f = r ** 2 * (np.cos(gammas) ** 2 + np.sin(gammas) ** 2)
    pl = ((2. * r ** 2 / f) * np.sqrt((f - xi ** 2).clip(0)))[:256]
    pp = -1.0 * np.log(np.sum(counts * np.exp(-1.0 * np.outer(pl, attens)), axis=1)
                       / np.sum(counts)) / atten_eff
    return np.polyfit(pp, pl, 2)


# ---- helical rebinning front-end (trajectory.py) -----------------------------

def rebin_rows(src, pairs, w, shape, reverse=False):
    """The row gathers of sino_hel2axl / sino_hel2axl180 / sino_hel2hel
    (trajectory.py:95-103): float32 rows times float64 weights, summed in
    float64 and stored as float32; pairs (v0, r0, v1, r1) per output row."""
    a = src[pairs[:, 0], pairs[:, 1], :] * w[:, 0:1]
    b = src[pairs[:, 2], pairs[:, 3], :] * w[:, 1:2]
    o = (a + b).astype(np.float32).reshape(shape)
    return o[..., ::-1] if reverse else o


def axl2hel(sinoA, view_index, z_shift, wrap, n_rows_h):
    """sino_axl2hel's sampling (trajectory.py:56-67) with scipy's
    map_coordinates, the reference's own call, for precomputed per-view
    axial indices, z shifts and wrap flags."""
    from scipy.ndimage import map_coordinates
    nA, nR, nC = sinoA.shape
    rows, cols = np.split(np.mgrid[0:n_rows_h, 0:nC], 2, axis=0)
    views = np.zeros([1, n_rows_h, nC])
    out = np.zeros([len(view_index), n_rows_h, nC], np.float32)
    for i, (a, z, wr) in enumerate(zip(view_index, z_shift, wrap)):
        views[:] = a
        if not wr:
            out[i] = map_coordinates(sinoA, (views, rows + z, cols), order=1, mode="constant", cval=0.0)
        else:
            out[i] = map_coordinates(sinoA, (views, (rows + z).clip(0, nR - 1), cols.clip(0, nC - 1)),
                                     order=1, mode="grid-wrap")
    return out


def rotsum_fp(phantom, mats):
    """forward_project_phantom's projection (trajectory.py:27-40) for given
    per-view 3 x 4 affine matrices: the phantom sampled by map_coordinates
    (order 1, cval 0) at each voxel's transformed coordinates (rounded to 6
    decimals) and summed along y."""
    from scipy.ndimage import map_coordinates
    nX, nY, nZ = phantom.shape
    g = np.mgrid[:nX, :nY, :nZ].astype(np.float32)
    out = np.zeros((len(mats), nZ, nX), np.float32)
    for i, m in enumerate(mats):
        c = np.round(np.einsum("rk,kxyz->rxyz", m[:, :3], g) + m[:, 3, None, None, None], 6)
        out[i] = map_coordinates(phantom, c, order=1, mode="constant", cval=0.0).sum(axis=1).T
    return out


# ---- Siddon ray-list set-up (sys_mat/siddon.py:681-751) -----------------------

def siddons_setup(src, trg, nPixels, dPixels=1.0, origin=0.0, epsilon=1e-5):
    """Per-ray set-up of ``siddons`` restated step by step as siddon.py:681-751
    computes it (float32 grid planes and rays, both branches of every
    ``np.where`` evaluated): the alpha range (amin, amax), the first / last
    plane index of each axis with the ``isclose`` rounding, normalised to
    numpy slice bounds as ``g.Xb[i0:iN]`` (:772) reads them, and the validity
    of each ray.  Returns a dict of flat per-ray arrays (float32 / int32)."""
    def three(v, dtype):
        v = np.array(v, dtype=dtype)
        return np.repeat(v, 3) if v.size == 1 else v

    nP, dP, oP = three(nPixels, int), three(dPixels, np.float32), three(origin, np.float32)
    planes = [np.linspace(-nP[a], nP[a], nP[a] + 1, dtype=np.float32) * dP[a] / 2.0 + oP[a]
              for a in range(3)]
    src = np.array(src, dtype=np.float32).reshape(-1, 3)
    trg = np.array(trg, dtype=np.float32).reshape(-1, 3)
    p0 = np.array([b[0] for b in planes], dtype=np.float32)
    pN = np.array([b[-1] for b in planes], dtype=np.float32)
    dST = trg - src
    with np.errstate(divide="ignore", invalid="ignore"):
        alpha0 = np.where(dST != 0.0, (p0 - src) / dST, (p0 - src) / epsilon)
        alphaN = np.where(dST != 0.0, (pN - src) / dST, (pN - src) / epsilon)
    m_min = np.zeros((len(src), 4), dtype=np.float32)
    m_max = np.ones((len(src), 4), dtype=np.float32)
    lt, gt = alpha0 < alphaN, alpha0 > alphaN
    m_min[:, 1:][lt] = alpha0[lt]
    m_max[:, 1:][lt] = alphaN[lt]
    m_min[:, 1:][gt] = alphaN[gt]
    m_max[:, 1:][gt] = alpha0[gt]
    amin, amax = m_min.max(-1), m_max.min(-1)
    first_pos = (nP + 1) - (pN - amin[:, None] * dST - src) / dP
    first_neg = (nP + 1) - (pN - amax[:, None] * dST - src) / dP
    last_pos = (src + amax[:, None] * dST - p0) / dP
    last_neg = (src + amin[:, None] * dST - p0) / dP

    def snap(v, f):
        return np.where(np.isclose(v, np.round(v), atol=epsilon), np.round(v), f(v)).astype(np.int32)

    with np.errstate(invalid="ignore"):
        i0 = np.where(dST > 0.0, snap(first_pos, np.floor), snap(first_neg, np.floor))
        iN = np.where(dST > 0.0, snap(last_pos, np.ceil), snap(last_neg, np.ceil))
    L = (nP + 1).astype(np.int64)
    bound = lambda i: np.clip(np.where(i < 0, i + L, i), 0, L).astype(np.int32)
    valid = (amax > amin) & ~np.isclose(amax, amin, atol=epsilon)
    return dict(amin=amin, amax=amax, i0=bound(i0), iN=bound(iN), valid=valid.astype(np.uint8),
                dist=np.linalg.norm(dST, axis=-1).astype(np.float32), dst=dST)
