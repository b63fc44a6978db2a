"""List projection over Siddon lists, drop-in for vir ``projection/proj.py``.

* ``sd_f_proj(phantom, sdlist, ravel=True, flat=True, sino_shape=None)``
  (proj.py:56-116): sino[r] = sum phantom[ind] * len over each ray's entries.
* ``sd_b_proj(sino, sdlist, nPixels, ravel=True)`` (proj.py:119-150):
  phantom[ind] += sino[r] * len.  The reference's fancy-index ``+=``
  (proj.py:134, 139) drops repeated voxels of a ray; this version
  accumulates them (np.add.at semantics), which is the adjoint of sd_f_proj.

``sdlist`` is the flat CSR tuple ``(ind, len, off)`` or an object array of
per-ray ``[R, L]`` (ravel) / ``[X, Y, Z, L]`` (unraveled) lists, as
``siddons`` returns them.  The projections run on the GPU (``vg_list_fp`` /
``vg_list_bp``); CSR tuples of CUDA tensors stay on the device.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _core
from .._lib import call, load


def _csr_from(sdlist, ravel, shape_vox=None, flat=False):
    """(ind, len, off) as numpy or torch from any of siddons' list forms."""
    if flat or isinstance(sdlist, tuple):
        ind, ln, off = sdlist
        return ind, ln, off, None
    rays = np.asarray(sdlist, dtype=object)
    flat = rays.reshape(-1)
    counts = np.zeros(flat.size + 1, np.int64)
    parts_i, parts_l = [], []
    for r, ray in enumerate(flat):
        if ray is None:
            continue
        if ravel:
            R, L = np.asarray(ray[0]), np.asarray(ray[1])
        else:
            R = np.ravel_multi_index((np.asarray(ray[0]), np.asarray(ray[1]), np.asarray(ray[2])),
                                     shape_vox)
            L = np.asarray(ray[3])
        parts_i.append(R.astype(np.int32))
        parts_l.append(L.astype(np.float32))
        counts[r + 1] = R.size
    off = np.cumsum(counts).astype(np.int32)
    ind = np.concatenate(parts_i) if parts_i else np.zeros(0, np.int32)
    ln = np.concatenate(parts_l) if parts_l else np.zeros(0, np.float32)
    return ind, ln, off, rays.shape


def _dev(a, dtype, dev):
    if isinstance(a, torch.Tensor):
        return a.detach().to(device=dev, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a, dtype={torch.int32: np.int32,
                                                           torch.float32: np.float32}[dtype])).to(dev)


def list_fp_device(x, ind, ln, off, out=None, accumulate=False):
    """CUDA tensors in, CUDA tensor out (nrays,)."""
    nrays = off.numel() - 1
    if out is None:
        out = torch.zeros(max(nrays, 1), dtype=torch.float32, device=x.device)[:nrays]
    call("vg_list_fp", x.data_ptr(), ind.data_ptr(), ln.data_ptr(), off.data_ptr(), nrays,
         out.data_ptr(), int(bool(accumulate)), _core.stream(x.device))
    return out


def list_bp_device(y, ind, ln, off, nvox, out=None, accumulate=False):
    L = load()
    nrays = off.numel() - 1
    dev = y.device
    if out is None:
        out = torch.zeros(nvox, dtype=torch.float32, device=dev)
    ws = torch.empty(int(L.vg_list_bp_workspace_bytes(int(nvox))) // 8, dtype=torch.float64,
                     device=dev)
    call("vg_list_bp", y.data_ptr(), ind.data_ptr(), ln.data_ptr(), off.data_ptr(), nrays,
         int(nvox), out.data_ptr(), int(bool(accumulate)), ws.data_ptr(), ws.numel() * 8,
         _core.stream(dev))
    return out


def sd_f_proj(phantom, sdlist, ravel=True, flat=True, sino_shape=None):
    dev = _core.device_of(phantom)
    x = _core.to_device(phantom, dev).reshape(-1)
    ind, ln, off, rshape = _csr_from(sdlist, ravel, tuple(np.shape(phantom)), flat)
    ind, ln, off = _dev(ind, torch.int32, dev), _dev(ln, torch.float32, dev), _dev(off, torch.int32, dev)
    sino = list_fp_device(x, ind, ln, off)
    shape = sino_shape if sino_shape is not None else (rshape if rshape is not None else sino.shape)
    return _core.to_host_like(sino.reshape(shape), phantom)


def sd_b_proj(sino, sdlist, nPixels, ravel=True):
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev).reshape(-1)
    nP = tuple(int(v) for v in np.atleast_1d(nPixels))
    ind, ln, off, _ = _csr_from(sdlist, ravel, nP)
    ind, ln, off = _dev(ind, torch.int32, dev), _dev(ln, torch.float32, dev), _dev(off, torch.int32, dev)
    x = list_bp_device(y, ind, ln, off, int(np.prod(nP)))
    return _core.to_host_like(x.reshape(nP), sino)
