"""vir_gb300 -- GB300-native projector / backprojector / reconstruction hot
path of vargasp/vir.

The package mirrors vir's module layout for the functions it replaces
(``vir_gb300.sys_mat.dd``, ``vir_gb300.sys_mat.fp_2d_par``,
``vir_gb300.filtration``, ...) with the same call signatures, return layouts
and scales, and runs them on hand-written sm_103a CUDA kernels in
``libvirgpu.so`` (C ABI: ``include/virgpu.h``), reached through ctypes with
torch CUDA tensors as buffers.  There is no CPU fallback: without the library
or a CUDA device every call raises ``VirGpuError``.
"""
from ._lib import VirGpuError, exported_symbols, library_path  # noqa: F401

__version__ = "0.1.0"


def load():
    """Build (if needed) and load libvirgpu.so; returns the ctypes handle."""
    from ._lib import load as _load
    return _load()


# vir module -> {function name: replacement "module:attr" in this package}
_DROP_INS = {
    "sys_mat.dd": {n: "vir_gb300.sys_mat.dd:" + n for n in
                   ("dd_fp_par_2d", "dd_bp_par_2d", "dd_fp_fan_2d", "dd_bp_fan_2d",
                    "dd_fp_cone_3d", "dd_bp_cone_3d", "dd_fp_square", "dd_bp_square")},
    "sys_mat.sirt_dd": {n: "vir_gb300.sys_mat.sirt_dd:" + n
                        for n in ("sirt", "fast_divide1", "fast_divide2")},
    "sys_mat.sirt_numba": {n: "vir_gb300.sys_mat.sirt_dd:" + n
                           for n in ("sirt", "fast_divide1", "fast_divide2")},
    "sys_mat.sp": {"sf_fp_fan_2d": "vir_gb300.sys_mat.sp:sf_fp_fan_2d"},
    "sys_mat.rd": {n: "vir_gb300.sys_mat.rd:" + n for n in
                   ("aw_fp_par_2d", "aw_bp_par_2d", "aw_fp_fan_2d", "aw_bp_fan_2d",
                    "aw_fp_cone_3d", "aw_bp_cone_3d")},
    "sys_mat.pd": {n: "vir_gb300.sys_mat.pd:" + n for n in
                   ("pd_fp_par_2d", "pd_bp_par_2d", "pd_fp_fan_2d", "pd_bp_fan_2d",
                    "pd_fp_cone_3d", "pd_bp_cone_3d")},
    "sys_mat.fp_2d_par": {n: "vir_gb300.sys_mat.fp_2d_par:" + n
                          for n in ("siddons_fp_2d", "separable_footprint_fp_2d")},
    "filtration": {"filter_sino": "vir_gb300.filtration:filter_sino"},
    "sys_mat.siddon": {n: "vir_gb300.sys_mat.siddon:" + n for n in
                       ("siddons", "list2array", "list2array_iter_ray", "list_count_elem",
                        "list_flatten", "list_ravel", "list_unravel", "ray_ravel", "ray_unravel",
                        "list_index_shift", "ray_index_shift", "list_del_ind", "list_flip",
                        "ray_flip", "ray_boundary", "rays_ave", "list_ave", "rays_weight_ave",
                        "list_weight_ave", "list_convole")},
    "mpct": {"list_ctypes_object": "vir_gb300.mpct:list_ctypes_object"},
    "projection.proj": {n: "vir_gb300.projection.proj:" + n for n in ("sd_f_proj", "sd_b_proj")},
    "projection.proj_ctype": {n: "vir_gb300.projection.proj_ctype:" + n
                              for n in ("sd_f_proj_c", "sd_b_proj_c")},
    "projection.proj_numba": {n: "vir_gb300.projection.proj_numba:" + n
                              for n in ("fast_forward_project", "fast_forward_project_p",
                                        "sd_f_proj_numba", "sd_f_proj_numba_p")},
    "projection.proj_cuda": {"sd_f_proj_numba_g": "vir_gb300.projection.proj_numba:sd_f_proj_numba_g"},
    "trajectory": {n: "vir_gb300.trajectory:" + n
                   for n in ("sino_axl2hel", "sino_hel2axl", "sino_hel2axl180", "sino_hel2hel",
                             "sino_hel_subset", "forward_project_phantom")},
    "processing.beamhard": {n: "vir_gb300.beamhard:" + n
                            for n in ("beamhard_cor", "beamhard_cor_table", "beamhard_coefs",
                                      "beamhard_coefs2", "water_tub_phantom")},
}


def install_into(vir_pkg):
    """Opt-in monkeypatch: replace vir's functions on the hot path with the
    GPU drop-ins of this package (same signatures, layouts and scales).
    ``vir_pkg`` is the imported ``vir`` package; returns the list of
    replaced "module.function" names."""
    import importlib
    done = []
    for mod, fns in _DROP_INS.items():
        try:
            target = importlib.import_module(vir_pkg.__name__ + "." + mod)
        except ImportError:
            continue
        for name, spec in fns.items():
            m, a = spec.split(":")
            setattr(target, name, getattr(importlib.import_module(m), a))
            done.append(f"{mod}.{name}")
    return done
