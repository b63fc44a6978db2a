"""Host-side plumbing shared by the drop-in modules: device buffers (torch
CUDA tensors), numpy <-> device conversion, the current stream, and the
per-view trig tables.

Every public function of the drop-in modules accepts numpy arrays or torch
tensors.  numpy in -> numpy out (the call copies to the GPU and back); a
torch CUDA tensor in -> a torch CUDA tensor out on the same device, with no
host round trip.
"""
from __future__ import annotations

import collections
import ctypes
import threading

import numpy as np
import torch

from ._lib import VirGpuError, call, load  # noqa: F401

_F32 = torch.float32


def require_cuda():
    if not torch.cuda.is_available():
        raise VirGpuError("device", -1, "vir_gb300 needs a CUDA device; none is visible")
    load()


def is_torch(a) -> bool:
    return isinstance(a, torch.Tensor)


def device_of(*arrays):
    for a in arrays:
        if is_torch(a) and a.is_cuda:
            return a.device
    return torch.device("cuda", torch.cuda.current_device())


def to_device(a, dev=None, dtype=_F32) -> torch.Tensor:
    """float32 C-contiguous CUDA tensor holding ``a`` (no copy when it already is one)."""
    require_cuda()
    dev = dev or device_of(a)
    if is_torch(a):
        t = a.detach().to(device=dev, dtype=dtype)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(a), dtype=np.dtype(str(dtype).split(".")[-1])))
        t = t.to(dev, non_blocking=False)
    return t.contiguous()


def to_host_like(t: torch.Tensor, like):
    """Return ``t`` where the caller's input lived: a CUDA tensor for CUDA
    input, a CPU tensor for CPU tensor input, numpy for anything else."""
    if is_torch(like):
        return t if like.is_cuda else t.cpu()
    return t.cpu().numpy()


def ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def stream(dev=None) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def empty(shape, dev, dtype=_F32) -> torch.Tensor:
    return torch.empty(tuple(int(s) for s in shape), dtype=dtype, device=dev)


def host_angles(a) -> np.ndarray:
    if is_torch(a):
        a = a.detach().cpu().numpy()
    return np.atleast_1d(np.asarray(a))


class _TrigCache:
    """Interleaved (cos, sin) float64 device tables, computed on the host with
    numpy exactly as the reference computes them, cached per (angles, dtype,
    device)."""

    def __init__(self, cap=64):
        self._d = collections.OrderedDict()
        self._cap = cap
        self._lock = threading.Lock()

    def get(self, angles, cast=None, dev=None) -> torch.Tensor:
        a = host_angles(angles)
        if cast is not None:
            a = a.astype(cast)
        dev = dev or torch.device("cuda", torch.cuda.current_device())
        key = (a.dtype.str, a.shape, a.tobytes(), str(dev))
        with self._lock:
            t = self._d.get(key)
            if t is not None:
                self._d.move_to_end(key)
                return t
        tab = np.empty((a.size, 2), np.float64)
        tab[:, 0] = np.cos(a).ravel()
        tab[:, 1] = np.sin(a).ravel()
        t = torch.from_numpy(tab.ravel()).to(dev)
        with self._lock:
            self._d[key] = t
            if len(self._d) > self._cap:
                self._d.popitem(last=False)
        return t


trig_cache = _TrigCache()


def f32(v) -> float:
    """Round a scalar to float32 as vir's as_float32 does (dd.py:29-36)."""
    return float(np.float32(v))
