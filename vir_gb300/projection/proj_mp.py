"""Process-pool list projection, drop-in for the plain entry points of vir
``projection/proj_mp.py``.

* ``mp_sd_f_proj(phantom, sdlist, cpus=...)`` / ``mpc_sd_f_proj`` (proj_mp.py:43,
  122): sino[ray] = sum phantom[x, y, z] * len over an unraveled object-array
  list, shaped like the list;
* ``mp_sd_b_proj(sino, sdlist, nPixels, cpus=...)`` / ``mpc_sd_b_proj``
  (proj_mp.py:78, 170): phantom[x, y, z] += sino[ray] * len (float32).

The process pool is replaced by the GPU list kernels (``vg_list_fp`` /
``vg_list_bp``); ``cpus`` is accepted and unused.  The symmetry-folded
variants (``*_t``, ``*_s``, ``*_4sym``) are not provided.
"""
from __future__ import annotations

import numpy as np

from .proj import sd_b_proj, sd_f_proj


def mp_sd_f_proj(phantom, sdlist, cpus=None):
    out = sd_f_proj(np.asarray(phantom, np.float32), sdlist, ravel=False, flat=False)
    return np.asarray(out).reshape(sdlist.shape)


def mp_sd_b_proj(sino, sdlist, nPixels, cpus=None):
    return sd_b_proj(np.asarray(sino, np.float32), sdlist, nPixels, ravel=False)


def mpc_sd_f_proj(phantom, sdlist, cpus=None):
    return mp_sd_f_proj(phantom, sdlist, cpus)


def mpc_sd_b_proj(sino, sdlist, nPixels, cpus=None):
    return mp_sd_b_proj(sino, sdlist, nPixels, cpus)
