"""ctypes binding of libvirgpu.so (the C ABI declared in include/virgpu.h).

The library is loaded from vir_gb300/_build (built in tree by
vir_gb300.build).  There is no CPU fallback: every projector call needs the
library and a CUDA device, and fails loudly with VirGpuError otherwise.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

c_int, c_float, c_double, c_void_p = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p
c_size_t = ctypes.c_size_t


class VirGpuError(RuntimeError):
    """Raised when a libvirgpu entry point returns a non-zero status."""

    def __init__(self, fn, status, msg):
        super().__init__(f"{fn} failed with status {status}: {msg}")
        self.status = status


class DD2DGeom(ctypes.Structure):
    """vg_dd2d_geom (include/virgpu.h)."""
    _fields_ = [("nx", c_int), ("ny", c_int), ("na", c_int), ("nu", c_int),
                ("du", c_float), ("su", c_float), ("d_pix", c_float),
                ("DSO", c_float), ("DSD", c_float), ("fan", c_int), ("variant", c_int)]


class Sirt2DProblem(ctypes.Structure):
    """vg_sirt2d_problem (include/virgpu.h)."""
    _fields_ = [("g", DD2DGeom), ("y", c_void_p), ("inv_w_sino", c_void_p),
                ("inv_w_img", c_void_p), ("trig", c_void_p), ("x", c_void_p), ("xT", c_void_p),
                ("r", c_void_p), ("workspace", c_void_p), ("gamma", c_float), ("pad", c_int)]


class SiddonRays(ctypes.Structure):
    """vg_siddon_rays (include/virgpu.h)."""
    _fields_ = [("n_rays", c_int), ("nx", c_int), ("ny", c_int), ("nz", c_int),
                ("dx", c_float), ("dy", c_float), ("dz", c_float),
                ("xb", c_void_p), ("yb", c_void_p), ("zb", c_void_p),
                ("src", c_void_p), ("dst", c_void_p), ("dist", c_void_p), ("amin", c_void_p),
                ("amax", c_void_p), ("i0", c_void_p), ("iN", c_void_p), ("valid", c_void_p)]


class SiddonsGrid(ctypes.Structure):
    """vg_siddons_grid (include/virgpu.h)."""
    _fields_ = [("nx", c_int), ("ny", c_int), ("nz", c_int),
                ("dx", c_float), ("dy", c_float), ("dz", c_float),
                ("p0", c_float * 3), ("pN", c_float * 3), ("epsilon", c_double),
                ("epsilon_f", c_float), ("pad", c_int)]


class SF2DGeom(ctypes.Structure):
    """vg_sf2d_geom (include/virgpu.h)."""
    _fields_ = [("nx", c_int), ("ny", c_int), ("na", c_int), ("nu", c_int), ("du", c_float),
                ("d_pix", c_float), ("DSO", c_float), ("DSD", c_float), ("fan", c_int)]


class DD3DGeom(ctypes.Structure):
    """vg_dd3d_geom (include/virgpu.h)."""
    _fields_ = [("nx", c_int), ("ny", c_int), ("nz", c_int), ("na", c_int), ("nu", c_int),
                ("nv", c_int), ("du", c_float), ("dv", c_float), ("su", c_float),
                ("sv", c_float), ("d_pix", c_float), ("DSO", c_float), ("DSD", c_float)]


class DDSquareGeom(ctypes.Structure):
    """vg_dd_square_geom (include/virgpu.h)."""
    _fields_ = [("n", c_int), ("nz", c_int), ("nu", c_int), ("nv", c_int), ("nsrc_p", c_int),
                ("nsrc_z", c_int), ("DSO", c_float), ("DSD", c_float), ("du", c_float),
                ("dv", c_float), ("dsrc_p", c_float), ("dsrc_z", c_float), ("su", c_float),
                ("sv", c_float), ("ssrc_p", c_float), ("ssrc_z", c_float), ("d_pix", c_float)]


class RayGeom(ctypes.Structure):
    """vg_ray_geom (include/virgpu.h)."""
    _fields_ = [("nx", c_int), ("ny", c_int), ("nz", c_int), ("na", c_int), ("nu", c_int),
                ("nv", c_int), ("du", c_float), ("dv", c_float), ("su", c_float),
                ("sv", c_float), ("d_pix", c_float), ("DSO", c_float), ("DSD", c_float),
                ("kind", c_int), ("joseph", c_int)]


# name -> argtypes (all return int status)
_PROTOS = {
    "vg_siddon2d_fp": [c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_double, c_double,
                       c_void_p, c_void_p],
    "vg_siddon2d_bp": [c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_double, c_double,
                       c_void_p, c_void_p],
    "vg_siddon2d_trace": [c_int, c_int, c_void_p, c_int, c_int, c_double, c_double, c_void_p,
                          c_void_p, c_void_p, c_void_p],
    "vg_div_rn_check": [c_void_p, c_void_p, c_size_t, c_void_p, c_void_p],
    "vg_siddon2d_bp_scatter": [c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_double,
                               c_double, c_void_p, c_void_p, c_size_t, c_void_p],
    "vg_siddons_setup": [ctypes.POINTER(SiddonsGrid), c_int, c_void_p, c_void_p, c_void_p,
                         c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_siddons_count": [ctypes.POINTER(SiddonRays), c_void_p, c_void_p, c_void_p],
    "vg_siddons_fill": [ctypes.POINTER(SiddonRays), c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_list_fp": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p],
    "vg_list_bp": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_int,
                   c_void_p, c_size_t, c_void_p],
    "vg_dd2d_fp": [ctypes.POINTER(DD2DGeom), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_dd2d_bp": [ctypes.POINTER(DD2DGeom), c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                   c_void_p],
    "vg_dd2d_sirt_iter": [ctypes.POINTER(DD2DGeom), c_void_p, c_void_p, c_void_p, c_float,
                          c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p],
    "vg_dd2d_sirt_residual": [ctypes.POINTER(DD2DGeom), c_void_p, c_void_p, c_void_p, c_void_p,
                              c_void_p, c_void_p, c_void_p, c_size_t, c_void_p],
    "vg_dd2d_sirt_update": [ctypes.POINTER(DD2DGeom), c_void_p, c_float, c_void_p, c_void_p,
                            c_void_p, c_void_p, c_void_p, c_size_t, c_void_p],
    "vg_dd2d_bp_noalloc": [ctypes.POINTER(DD2DGeom), c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_fbp2d_bp": [ctypes.POINTER(DD2DGeom), c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_dd3d_fp": [ctypes.POINTER(DD3DGeom), c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                   c_void_p],
    "vg_dd3d_sirt_iter": [ctypes.POINTER(DD3DGeom), c_void_p, c_void_p, c_void_p, c_float,
                          c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p],
    "vg_sirt2d_batch_items": [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                              c_void_p],
    "vg_sirt2d_batch_run": [c_void_p, c_int, c_int, c_void_p, c_int, c_void_p, c_int, c_void_p,
                            c_int, c_int, c_int, c_void_p, ctypes.c_ulonglong, c_void_p, c_void_p,
                            c_void_p, c_void_p],
    "vg_sf3d_fp": [ctypes.POINTER(DD3DGeom), c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                   c_void_p],
    "vg_sf3d_bp": [ctypes.POINTER(DD3DGeom), c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                   c_void_p],
    "vg_dd3d_bp": [ctypes.POINTER(DD3DGeom), c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                   c_void_p],
    "vg_dd_square_fp": [ctypes.POINTER(DDSquareGeom), c_void_p, c_void_p, c_void_p],
    "vg_dd_square_bp": [ctypes.POINTER(DDSquareGeom), c_void_p, c_void_p, c_void_p, c_size_t,
                        c_void_p],
    "vg_dd_square_sirt_iter": [ctypes.POINTER(DDSquareGeom), c_void_p, c_void_p, c_void_p,
                               c_float, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p],
    "vg_rd_fp": [ctypes.POINTER(RayGeom), c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_rd_bp": [ctypes.POINTER(RayGeom), c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_pd_fp": [ctypes.POINTER(RayGeom), c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_pd_bp": [ctypes.POINTER(RayGeom), c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_tv_dual": [c_void_p, c_void_p, c_int, c_int, c_float, c_void_p],
    "vg_tv_residual": [c_void_p, c_void_p, c_void_p, c_void_p, c_float, c_size_t, c_void_p],
    "vg_tv_primal": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_float, c_int, c_int,
                     c_void_p],
    "vg_fdk_weight_transpose": [ctypes.POINTER(DD3DGeom), c_void_p, c_void_p, c_void_p],
    "vg_fdk_transpose_back": [ctypes.POINTER(DD3DGeom), c_void_p, c_void_p, c_void_p],
    "vg_fdk_bp": [ctypes.POINTER(DD3DGeom), c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_sf2d_fp": [ctypes.POINTER(SF2DGeom), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_sf2d_bp": [ctypes.POINTER(SF2DGeom), c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_transpose": [c_void_p, c_int, c_int, c_void_p, c_void_p],
    "vg_count_nonzero": [c_void_p, ctypes.c_longlong, c_void_p, c_void_p],
    "vg_compact_nonzero": [c_void_p, ctypes.c_longlong, c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_filter_rows": [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p],
    "vg_filter_rows_fft": [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                           c_void_p],
    "vg_bh_poly": [c_void_p, c_int, c_void_p, c_int, c_size_t, c_double, c_double, c_double,
                   c_double, c_int, c_void_p],
    "vg_bh_interp": [c_void_p, c_int, c_void_p, c_int, c_size_t, c_void_p, c_void_p, c_int, c_int,
                     c_int, c_double, c_void_p, c_void_p],
    "vg_rebin_rows": [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_int, c_void_p,
                      c_void_p, c_void_p],
    "vg_axl2hel": [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_int,
                   c_void_p, c_void_p],
    "vg_rotsum_fp": [c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p],
}


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libvirgpu.so (building it first when absent) and bind prototypes."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise VirGpuError("load", -1, f"{path} is missing; run python -m vir_gb300.build")
        L = ctypes.CDLL(path)
        L.vg_last_error.restype = ctypes.c_char_p
        L.vg_status_string.restype = ctypes.c_char_p
        L.vg_version.restype = c_int
        for name, args in _PROTOS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = c_int
        L.vg_dd2d_fp_variants.argtypes = []
        L.vg_dd2d_fp_variants.restype = c_int
        L.vg_dd2d_fp_default_variant.argtypes = [ctypes.POINTER(DD2DGeom)]
        L.vg_dd2d_fp_default_variant.restype = c_int
        L.vg_dd2d_sirt_launches.argtypes = [ctypes.POINTER(DD2DGeom)]
        L.vg_dd2d_sirt_launches.restype = c_int
        L.vg_dd2d_workspace_bytes.argtypes = [ctypes.POINTER(DD2DGeom)]
        L.vg_dd2d_workspace_bytes.restype = c_size_t
        L.vg_dd3d_workspace_bytes.argtypes = [ctypes.POINTER(DD3DGeom)]
        L.vg_dd3d_workspace_bytes.restype = c_size_t
        L.vg_sf3d_workspace_bytes.argtypes = [ctypes.POINTER(DD3DGeom)]
        L.vg_sf3d_workspace_bytes.restype = c_size_t
        L.vg_dd_square_workspace_bytes.argtypes = [ctypes.POINTER(DDSquareGeom)]
        L.vg_dd_square_workspace_bytes.restype = c_size_t
        L.vg_compact_blocks.argtypes = [ctypes.c_longlong]
        L.vg_compact_blocks.restype = c_int
        L.vg_siddon2d_bp_workspace_bytes.argtypes = [c_int, c_int, c_int, c_double, c_double]
        L.vg_siddon2d_bp_workspace_bytes.restype = c_size_t
        L.vg_list_bp_workspace_bytes.argtypes = [c_int]
        L.vg_list_bp_workspace_bytes.restype = c_size_t
        L.vg_dd2d_noalloc_scratch_bytes.argtypes = []
        L.vg_dd2d_noalloc_scratch_bytes.restype = c_size_t
        _lib = L
        return L


def call(name, *args):
    """Invoke an entry point and raise VirGpuError on a non-zero status."""
    L = _lib if _lib is not None else load()
    st = getattr(L, name)(*args)
    if st != 0:
        raise VirGpuError(name, st, L.vg_last_error().decode(errors="replace"))
    return st


def exported_symbols():
    return list(_PROTOS) + ["vg_version", "vg_last_error", "vg_status_string",
                            "vg_dd2d_workspace_bytes", "vg_dd2d_noalloc_scratch_bytes",
                            "vg_dd2d_fp_variants", "vg_dd2d_fp_default_variant", "vg_dd2d_sirt_launches",
                            "vg_list_bp_workspace_bytes", "vg_dd3d_workspace_bytes", "vg_sf3d_workspace_bytes",
                            "vg_dd_square_workspace_bytes", "vg_compact_blocks",
                            "vg_siddon2d_bp_workspace_bytes"]


def dd_square_workspace(g, dev):
    """Device workspace (float64 tensor) for vg_dd_square_bp / _sirt_iter."""
    import torch
    L = _lib if _lib is not None else load()
    n = int(L.vg_dd_square_workspace_bytes(ctypes.byref(g)))
    if n == 0:
        raise VirGpuError("vg_dd_square_workspace_bytes", 1,
                          L.vg_last_error().decode(errors="replace"))
    return torch.empty((n + 7) // 8, dtype=torch.float64, device=dev)


def dd3d_workspace(g, dev):
    """Device workspace (float32 tensor) for vg_dd3d_fp / vg_dd3d_bp."""
    import torch
    L = _lib if _lib is not None else load()
    n = int(L.vg_dd3d_workspace_bytes(ctypes.byref(g)))
    if n == 0:
        raise VirGpuError("vg_dd3d_workspace_bytes", 1, L.vg_last_error().decode(errors="replace"))
    return torch.empty((n + 3) // 4, dtype=torch.float32, device=dev)


def dd2d_workspace(g, dev):
    """Device workspace (a uint8 tensor, 256-byte aligned) for vg_dd2d_bp."""
    import torch
    L = _lib if _lib is not None else load()
    n = int(L.vg_dd2d_workspace_bytes(ctypes.byref(g)))
    if n == 0:
        raise VirGpuError("vg_dd2d_workspace_bytes", 1, L.vg_last_error().decode(errors="replace"))
    t = torch.empty(n + 256, dtype=torch.uint8, device=dev)
    off = (-t.data_ptr()) % 256
    return t[off:off + n]
