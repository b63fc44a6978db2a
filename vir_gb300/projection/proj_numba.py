"""CSR list forward projection, drop-in for vir ``projection/proj_numba.py``
and ``projection/proj_cuda.py`` (proj_numba.py:11-56, proj_cuda.py:14-62).

* ``fast_forward_project(phantom_flat, idxs, lengths, offsets, sino_flat)``
  and ``fast_forward_project_p`` (the serial and threaded numba loops): write
  sino_flat[r] = sum phantom_flat[idxs] * lengths over ray r's entries, in
  place (numpy arrays or CUDA tensors);
* ``sd_f_proj_numba(phantom, sdlist, sino_shape)``,
  ``sd_f_proj_numba_p`` and ``sd_f_proj_numba_g`` (the numba-CUDA version):
  the same from a CSR ``sdlist = (idxs, lengths, offsets)``, returning a new
  float32 array of ``sino_shape``.

All of them run the warp-per-ray gather of ``vg_list_fp`` (Kahan-compensated
FP32 sums) on the GPU.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _core
from .proj import _dev, list_fp_device


def _fp_into(phantom_flat, idxs, lengths, offsets, sino_flat):
    dev = _core.device_of(phantom_flat, sino_flat)
    _core.require_cuda()
    x = _dev(phantom_flat, torch.float32, dev).reshape(-1)
    out = list_fp_device(x, _dev(idxs, torch.int32, dev), _dev(lengths, torch.float32, dev),
                         _dev(offsets, torch.int32, dev))
    if isinstance(sino_flat, torch.Tensor):
        sino_flat.copy_(out.reshape(sino_flat.shape).to(sino_flat.device, sino_flat.dtype))
    else:
        sino_flat[...] = out.cpu().numpy().reshape(sino_flat.shape).astype(sino_flat.dtype,
                                                                          copy=False)


def fast_forward_project(phantom_flat, idxs, lengths, offsets, sino_flat):
    _fp_into(phantom_flat, idxs, lengths, offsets, sino_flat)


def fast_forward_project_p(phantom_flat, idxs, lengths, offsets, sino_flat):
    _fp_into(phantom_flat, idxs, lengths, offsets, sino_flat)


def sd_f_proj_numba(phantom, sdlist, sino_shape):
    sino = np.zeros(sino_shape, dtype=np.float32)
    _fp_into(np.asarray(phantom).ravel(), sdlist[0], sdlist[1], sdlist[2], sino.reshape(-1))
    return sino


def sd_f_proj_numba_p(phantom, sdlist, sino_shape):
    return sd_f_proj_numba(phantom, sdlist, sino_shape)


def sd_f_proj_numba_g(phantom, sdlist, sino_shape):
    return sd_f_proj_numba(phantom, sdlist, sino_shape)
