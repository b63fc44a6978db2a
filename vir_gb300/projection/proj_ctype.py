"""ctypes-list projection, drop-in for vir ``projection/proj_ctype.py``.

``sd_f_proj_c(phantom, sino, sdlist_c, ravel=True, C=False, dims=None,
nRays=None)`` and ``sd_b_proj_c(...)`` (proj_ctype.py:27-77) take the ctypes
arrays of ``RaveledRay`` / ``UnraveledRay`` structures that
``mpct.list_ctypes_object`` builds (mpct.py:154-172, 206) and accumulate in
place into ``sino`` (FP) or ``phantom`` (BP), as the C functions
``forward/back_proj_{ravel,unravel}_rays_struct`` do
(projection_c.c:150-219).  The rays are gathered into one CSR list on the
host and projected on the GPU (``vg_list_fp`` / ``vg_list_bp``).  With
``C=True`` the first two arguments are ctypes float pointers and ``dims`` /
``nRays`` give their sizes, as in the reference.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _core
from .proj import list_bp_device, list_fp_device


def _as_array(ptr, n, ctype, dtype):
    if n == 0:
        return np.zeros(0, dtype)
    p = ctypes.cast(ptr, ctypes.POINTER(ctype))
    return np.ctypeslib.as_array(p, shape=(int(n),)).astype(dtype, copy=False)


def _csr_from_structs(sdlist_c, nrays, ravel, dims):
    # mpct.list_ctypes_object(flat=True) hands over ctypes.byref(array)
    sdlist_c = getattr(sdlist_c, "_obj", sdlist_c)
    counts = np.zeros(nrays + 1, np.int64)
    inds, lens = [], []
    nX, nY, nZ = dims
    for r in range(nrays):
        ray = sdlist_c[r]
        n = int(ray.n)
        counts[r + 1] = n
        if n == 0:
            continue
        if ravel:
            R = _as_array(ray.R, n, ctypes.c_int, np.int32)
        else:
            X = _as_array(ray.X, n, ctypes.c_int, np.int64)
            Y = _as_array(ray.Y, n, ctypes.c_int, np.int64)
            Z = _as_array(ray.Z, n, ctypes.c_int, np.int64)
            R = (nY * nZ * X + nZ * Y + Z).astype(np.int32)  # ravel_ray (projection_c.c:88-91)
        inds.append(R)
        lens.append(_as_array(ray.L, n, ctypes.c_float, np.float32))
    off = np.cumsum(counts).astype(np.int32)
    ind = np.concatenate(inds) if inds else np.zeros(0, np.int32)
    ln = np.concatenate(lens) if lens else np.zeros(0, np.float32)
    return ind, ln, off


def _views(phantom, sino, C, dims, nRays):
    if C:
        nX, nY, nZ = dims
        ph = np.ctypeslib.as_array(ctypes.cast(phantom, ctypes.POINTER(ctypes.c_float)),
                                   shape=(nX * nY * nZ,))
        sn = np.ctypeslib.as_array(ctypes.cast(sino, ctypes.POINTER(ctypes.c_float)),
                                   shape=(int(nRays),))
        return ph, sn, (nX, nY, nZ), int(nRays)
    if not (isinstance(sino, np.ndarray) and sino.dtype == np.float32 and
            isinstance(phantom, np.ndarray) and phantom.dtype == np.float32):
        raise TypeError("sd_*_proj_c updates float32 numpy arrays in place")
    return phantom.reshape(-1), sino.reshape(-1), phantom.shape, sino.size


def sd_f_proj_c(phantom, sino, sdlist_c, ravel=True, C=False, dims=None, nRays=None):
    ph, sn, dims, n = _views(phantom, sino, C, dims, nRays)
    ind, ln, off = _csr_from_structs(sdlist_c, n, ravel, dims)
    dev = torch.device("cuda", torch.cuda.current_device())
    x = torch.from_numpy(np.ascontiguousarray(ph)).to(dev)
    out = torch.from_numpy(np.ascontiguousarray(sn)).to(dev)
    list_fp_device(x, torch.from_numpy(ind).to(dev), torch.from_numpy(ln).to(dev),
                   torch.from_numpy(off).to(dev), out=out, accumulate=True)
    sn[:] = out.cpu().numpy()


def sd_b_proj_c(phantom, sino, sdlist_c, ravel=True, C=False, dims=None, nRays=None):
    ph, sn, dims, n = _views(phantom, sino, C, dims, nRays)
    ind, ln, off = _csr_from_structs(sdlist_c, n, ravel, dims)
    dev = torch.device("cuda", torch.cuda.current_device())
    y = torch.from_numpy(np.ascontiguousarray(sn)).to(dev)
    out = torch.from_numpy(np.ascontiguousarray(ph)).to(dev)
    list_bp_device(y, torch.from_numpy(ind).to(dev), torch.from_numpy(ln).to(dev),
                   torch.from_numpy(off).to(dev), ph.size, out=out, accumulate=True)
    ph[:] = out.cpu().numpy()
