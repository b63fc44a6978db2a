"""ctypes list structures of vir ``mpct.py`` (mpct.py:154-260), built from
the Siddon lists this package produces on the GPU.

* ``RaveledRay`` (n, R, L) and ``UnraveledRay`` (n, X, Y, Z, L): the
  structures the C projectors (projection_c.c:126-219) and
  ``proj_ctype.sd_f_proj_c`` / ``sd_b_proj_c`` take (mpct.py:154-165);
* ``list_ctypes_object(sdlist, ravel=False, flat=True)``: the reference's
  conversion of an object-array list (mpct.py:206-260);
* ``csr_ctypes(ind, len, off, ravel=True, nPixels=None)``: the same array
  straight from a CSR list -- e.g. ``siddons(..., flat=True)`` or
  ``siddons_device`` output -- with one host copy of the index and length
  arrays instead of one small array per ray.  The returned ctypes array
  keeps those host arrays alive (attribute ``_keep``).
"""
from __future__ import annotations

import ctypes

import numpy as np

c_int_p = ctypes.POINTER(ctypes.c_int)
c_float_p = ctypes.POINTER(ctypes.c_float)


class UnraveledRay(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("X", c_int_p), ("Y", c_int_p), ("Z", c_int_p),
                ("L", c_float_p)]


class RaveledRay(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("R", c_int_p), ("L", c_float_p)]


def _host(a, dtype):
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(a, dtype=dtype)


def csr_ctypes(ind, ln, off, ravel=True, nPixels=None):
    ind = _host(ind, np.int32)
    ln = _host(ln, np.float32)
    off = _host(off, np.int64)
    nr = off.size - 1
    keep = [ind, ln]
    if ravel:
        arr = (RaveledRay * nr)()
        pi = ind.ctypes.data
        for r in range(nr):
            a, n = int(off[r]), int(off[r + 1] - off[r])
            arr[r].n = n
            if n:
                arr[r].R = ctypes.cast(pi + 4 * a, c_int_p)
                arr[r].L = ctypes.cast(ln.ctypes.data + 4 * a, c_float_p)
    else:
        if nPixels is None:
            raise ValueError("nPixels must be provided if ravel=False")
        xyz = [np.ascontiguousarray(v, np.int32) for v in np.unravel_index(ind, tuple(nPixels))]
        keep += xyz
        arr = (UnraveledRay * nr)()
        for r in range(nr):
            a, n = int(off[r]), int(off[r + 1] - off[r])
            arr[r].n = n
            if n:
                arr[r].X = ctypes.cast(xyz[0].ctypes.data + 4 * a, c_int_p)
                arr[r].Y = ctypes.cast(xyz[1].ctypes.data + 4 * a, c_int_p)
                arr[r].Z = ctypes.cast(xyz[2].ctypes.data + 4 * a, c_int_p)
                arr[r].L = ctypes.cast(ln.ctypes.data + 4 * a, c_float_p)
    arr._keep = keep
    return arr


def list_ctypes_object(sdlist, ravel=False, flat=True):
    """mpct.py:206-260: flat=True -> a ctypes array (by reference) of ray
    structures; flat=False -> an object array of structures by reference."""
    from .sys_mat.siddon import list_count_elem
    count = list_count_elem(sdlist)
    if flat:
        keep = []
        arr = (RaveledRay if ravel else UnraveledRay) * int(np.prod(sdlist.shape))
        out = arr()
        for r, (ray, n) in enumerate(zip(sdlist.flatten(), count.flatten())):
            out[r].n = int(n)
            if ray is None:
                continue
            parts = [np.ascontiguousarray(p, np.float32 if i == len(ray) - 1 else np.int32)
                     for i, p in enumerate(ray)]
            keep += parts
            if ravel:
                out[r].R = parts[0].ctypes.data_as(c_int_p)
                out[r].L = parts[1].ctypes.data_as(c_float_p)
            else:
                out[r].X = parts[0].ctypes.data_as(c_int_p)
                out[r].Y = parts[1].ctypes.data_as(c_int_p)
                out[r].Z = parts[2].ctypes.data_as(c_int_p)
                out[r].L = parts[3].ctypes.data_as(c_float_p)
        out._keep = keep
        return ctypes.byref(out)
    res = np.empty(sdlist.shape, dtype=object)
    for i, ray in np.ndenumerate(sdlist):
        if ray is None:
            continue
        parts = [np.ascontiguousarray(p, np.float32 if k == len(ray) - 1 else np.int32)
                 for k, p in enumerate(ray)]
        s = (RaveledRay(int(count[i]), parts[0].ctypes.data_as(c_int_p),
                        parts[1].ctypes.data_as(c_float_p)) if ravel else
             UnraveledRay(int(count[i]), parts[0].ctypes.data_as(c_int_p),
                          parts[1].ctypes.data_as(c_int_p), parts[2].ctypes.data_as(c_int_p),
                          parts[3].ctypes.data_as(c_float_p)))
        s._keep = parts
        res[i] = ctypes.byref(s)
    return res
