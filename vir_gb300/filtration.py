"""Ramp filtering for FBP, drop-in for vir ``filtration.py``.

``ramp_filter`` and ``window_filter`` design the half-spectrum filter on the
host exactly as the reference does (``filtration.py:4-112``, ``:115-235``;
float64 numpy: they are O(nu) setup).  ``filter_sino`` (``:238-309``)
filters on the GPU by the same route as the reference: zero-padded rFFT,
times 2H, inverse, cropped to nu (``vg_filter_rows_fft``: a shared-memory
FFT per row, float32, O(z log z)).  Below 256 bins the equivalent linear
convolution of the row with the 2*nu - 1 central taps of irfft(2H) is applied
directly (``vg_filter_rows``, compensated sums).  numpy in -> numpy out (float64,
as the reference returns), torch CUDA tensors stay on the device (float32).
"""
from __future__ import annotations

import collections
import threading

import numpy as np
import torch

from . import _core
from ._lib import call


def ramp_filter(nu, du=1.0, cutoff=0.5, zero_pad=True, half_spectrum=True, real_space=True,
                return_freq=False):
    nfu = int(2 ** np.ceil(np.log2(2 * nu))) if zero_pad else nu
    f = np.fft.rfftfreq(nfu, d=du) if half_spectrum else np.fft.fftfreq(nfu, d=du)
    if real_space:
        k = np.fft.fftfreq(nfu, d=1.0 / nfu)
        h = np.zeros(nfu)
        h[0] = 1.0 / (4.0 * du ** 2)
        h[1::2] = -1.0 / (np.pi ** 2 * du ** 2 * k[1::2] ** 2)
        H = du * np.real(np.fft.rfft(h) if half_spectrum else np.fft.fft(h))
    else:
        H = np.abs(f)
    H[np.abs(f) > cutoff * (1.0 / du)] = 0.0
    return (H, f) if return_freq else H


def window_filter(H, f, du=1.0, filter_type="ramp", cutoff=0.5, sigma=0.5):
    f_c = cutoff / du
    fn = f / f_c
    valid = np.abs(f) <= f_c
    W = np.zeros_like(f)
    if filter_type in ("ram-lak", "ramp"):
        return H
    elif filter_type == "hann":
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


_taps_lock = threading.Lock()
_taps = collections.OrderedDict()


def filter_taps(nu, du=1.0, filter_type="ramp", cutoff=0.5, real_space=True):
    """The 2*nu - 1 spatial taps (lags -(nu-1)..nu-1) equivalent to
    filter_sino's padded rFFT multiply, float64."""
    z = int(2 ** np.ceil(np.log2(2 * nu)))
    H, f = ramp_filter(nu, du=du, cutoff=cutoff, zero_pad=True, half_spectrum=True,
                       real_space=real_space, return_freq=True)
    H = window_filter(H, f, du=du, filter_type=filter_type, cutoff=cutoff)
    g = np.fft.irfft(2.0 * H, n=z)
    lags = np.arange(-(nu - 1), nu)
    return g[lags % z]


def _device_taps(nu, du, filter_type, cutoff, real_space, dev):
    key = (int(nu), float(du), str(filter_type), float(cutoff), bool(real_space), str(dev))
    with _taps_lock:
        t = _taps.get(key)
        if t is not None:
            return t
    t = torch.from_numpy(filter_taps(nu, du, filter_type, cutoff, real_space).astype(np.float32))
    t = t.to(dev)
    with _taps_lock:
        _taps[key] = t
        if len(_taps) > 32:
            _taps.popitem(last=False)
    return t


FFT_MIN_NU = 256  # from here on the FFT route is the faster one


def _device_spectrum(nu, du, filter_type, cutoff, real_space, dev):
    """(z, 2H as float32, twiddles W^m, m = 0..z-1, as float32 pairs) on dev."""
    key = ("fft", int(nu), float(du), str(filter_type), float(cutoff), bool(real_space), str(dev))
    with _taps_lock:
        t = _taps.get(key)
        if t is not None:
            return t
    z = int(2 ** np.ceil(np.log2(2 * nu)))
    H, f = ramp_filter(nu, du=du, cutoff=cutoff, zero_pad=True, half_spectrum=True,
                       real_space=real_space, return_freq=True)
    H = window_filter(H, f, du=du, filter_type=filter_type, cutoff=cutoff)
    m = np.arange(z)
    tw = np.stack([np.cos(2 * np.pi * m / z), -np.sin(2 * np.pi * m / z)], -1)
    t = (z, torch.from_numpy((2.0 * H).astype(np.float32)).to(dev),
         torch.from_numpy(tw.astype(np.float32).reshape(-1)).to(dev))
    with _taps_lock:
        _taps[key] = t
        if len(_taps) > 32:
            _taps.popitem(last=False)
    return t


def filter_rows_device(x: torch.Tensor, du=1.0, filter_type="ramp", cutoff=0.5, real_space=True,
                       row_weight=None, method="auto") -> torch.Tensor:
    """Filter a float32 CUDA tensor along its last axis (optionally
    multiplying every row by ``row_weight`` first).  method: "fft",
    "direct", or "auto" (FFT from FFT_MIN_NU bins on)."""
    nu = x.shape[-1]
    rows = x.numel() // nu
    out = torch.empty_like(x)
    wp = _core.ptr(row_weight) if row_weight is not None else None
    if method == "fft" or (method == "auto" and nu >= FFT_MIN_NU):
        z, spec, tw = _device_spectrum(nu, du, filter_type, cutoff, real_space, x.device)
        call("vg_filter_rows_fft", _core.ptr(x), rows, nu, z, _core.ptr(spec), _core.ptr(tw), wp,
             _core.ptr(out), _core.stream(x.device))
        return out
    taps = _device_taps(nu, du, filter_type, cutoff, real_space, x.device)
    call("vg_filter_rows", _core.ptr(x), rows, nu, _core.ptr(taps), wp, _core.ptr(out),
         _core.stream(x.device))
    return out


def filter_sino(sino, du=1.0, filter_type="ramp", cutoff=0.5, real_space=True):
    if filter_type is None:
        return sino
    dev = _core.device_of(sino)
    x = _core.to_device(sino, dev)
    out = filter_rows_device(x, du, filter_type, cutoff, real_space)
    if _core.is_torch(sino):
        return out
    return out.cpu().numpy().astype(np.float64)
