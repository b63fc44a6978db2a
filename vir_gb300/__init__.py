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
