"""Siddon ray lists, drop-in for vir ``sys_mat/siddon.py:siddons``.

``siddons(src, trg, nPixels=128, dPixels=1.0, origin=0.0, ravel=False,
flat=False, epsilon=1e-5)`` returns what the reference returns (siddon.py:636-833):

* ``flat=True``: ``(ind int32, len float32, off int32)``, the CSR form;
* ``ravel=True``: an object array of ``[R int32, L float32]`` per ray;
* otherwise an object array of ``[x_ind, y_ind, z_ind, length]`` per ray;
  rays that miss the grid are ``None``.

The per-ray set-up is vectorised over rays and computed here with the
reference's own numpy arithmetic (grid planes, alpha range, first/last plane
index with ``isclose`` rounding: siddon.py:681-751), so it is bit-identical;
the per-ray loop that sorts the plane crossings and emits (voxel, length)
entries (:754-826, the hot loop) runs on the GPU (``vg_siddons_count`` /
``vg_siddons_fill``) in FP32 with the same operation order.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _core
from .._lib import SiddonRays, VirGpuError, call


def _np3(v, dtype):
    v = np.array(v, dtype=dtype)
    if v.size == 1:
        v = np.repeat(v, 3)
    return v


def _planes(n, d, c):
    # boundspace(n, d, c, dtype=float32) (core_funcs.py:62-81)
    return np.linspace(-n, n, n + 1, dtype=np.float32) * d / 2.0 + c


def prepare(src, trg, nPixels=128, dPixels=1.0, origin=0.0, epsilon=1e-5):
    """Host set-up of siddons: returns (rays shape, grid, per-ray arrays)."""
    nP = _np3(nPixels, int)
    dP = _np3(dPixels, np.float32)
    oP = _np3(origin, np.float32)
    Xb = _planes(nP[0], dP[0], oP[0])
    Yb = _planes(nP[1], dP[1], oP[1])
    Zb = _planes(nP[2], dP[2], oP[2])
    trg = np.array(trg, dtype=np.float32)
    if trg.ndim == 1:
        trg = trg[np.newaxis, :]
    src = np.array(src, dtype=np.float32)
    if src.ndim == 1:
        src = src[np.newaxis, :]
    shape = trg.shape[:-1]
    p0 = np.array([Xb[0], Yb[0], Zb[0]], dtype=np.float32)
    pN = np.array([Xb[-1], Yb[-1], Zb[-1]], dtype=np.float32)
    dST = trg - src
    distance = np.linalg.norm(dST, axis=-1)
    with np.errstate(divide="ignore", invalid="ignore"):
        alpha0 = np.where(dST != 0.0, (p0 - src) / dST, (p0 - src) / epsilon)
        alphaN = np.where(dST != 0.0, (pN - src) / dST, (pN - src) / epsilon)
    m_min = np.zeros(shape + (4,), dtype=np.float32)
    m_max = np.ones(shape + (4,), dtype=np.float32)
    lt, gt = alpha0 < alphaN, alpha0 > alphaN
    m_min[..., 1:][lt] = alpha0[lt]
    m_max[..., 1:][lt] = alphaN[lt]
    m_min[..., 1:][gt] = alphaN[gt]
    m_max[..., 1:][gt] = alpha0[gt]
    amin = np.max(m_min, axis=-1)
    amax = np.min(m_max, axis=-1)
    i0p = (nP + 1) - (pN - amin[..., np.newaxis] * dST - src) / dP
    i0n = (nP + 1) - (pN - amax[..., np.newaxis] * dST - src) / dP
    iNp = (src + amax[..., np.newaxis] * dST - p0) / dP
    iNn = (src + amin[..., np.newaxis] * dST - p0) / dP
    r = lambda v, f: np.where(np.isclose(v, np.round(v), atol=epsilon), np.round(v), f(v)).astype(np.int32)
    with np.errstate(invalid="ignore"):  # axes with dST == 0 carry inf here, unused
        i0 = np.where(dST > 0.0, r(i0p, np.floor), r(i0n, np.floor))
        iN = np.where(dST > 0.0, r(iNp, np.ceil), r(iNn, np.ceil))
    # the reference slices g.Xb[i0:iN] (:772): normalise to numpy slice bounds
    L = (nP + 1).astype(np.int64)
    sl = lambda i: np.clip(np.where(i < 0, i + L, i), 0, L).astype(np.int32)
    i0, iN = sl(i0), sl(iN)
    valid = (amax > amin) & ~np.isclose(amax, amin, atol=epsilon)
    n = int(np.prod(shape))
    flat = lambda a, k: np.ascontiguousarray(np.broadcast_to(a, shape + (k,)).reshape(n, k))
    arrays = dict(src=flat(src, 3).astype(np.float32), dst=flat(dST, 3).astype(np.float32),
                  dist=np.ascontiguousarray(distance.reshape(n), dtype=np.float32),
                  amin=np.ascontiguousarray(amin.reshape(n), dtype=np.float32),
                  amax=np.ascontiguousarray(amax.reshape(n), dtype=np.float32),
                  i0=flat(i0, 3).astype(np.int32), iN=flat(iN, 3).astype(np.int32),
                  valid=np.ascontiguousarray(valid.reshape(n)).astype(np.uint8))
    grid = dict(n=nP, d=dP, Xb=Xb, Yb=Yb, Zb=Zb)
    return shape, grid, arrays


def siddons_device(src, trg, nPixels=128, dPixels=1.0, origin=0.0, epsilon=1e-5, device=None):
    """CSR list (ind, len, off) as CUDA tensors, plus the ray shape."""
    _core.require_cuda()
    dev = device or torch.device("cuda", torch.cuda.current_device())
    shape, grid, A = prepare(src, trg, nPixels, dPixels, origin, epsilon)
    n = int(np.prod(shape))
    T = {k: torch.from_numpy(v).to(dev) for k, v in A.items()}
    G = {k: torch.from_numpy(np.ascontiguousarray(grid[k], np.float32)).to(dev)
         for k in ("Xb", "Yb", "Zb")}
    nP, dP = grid["n"], grid["d"]
    R = SiddonRays(n, int(nP[0]), int(nP[1]), int(nP[2]), float(dP[0]), float(dP[1]),
                   float(dP[2]), G["Xb"].data_ptr(), G["Yb"].data_ptr(), G["Zb"].data_ptr(),
                   T["src"].data_ptr(), T["dst"].data_ptr(), T["dist"].data_ptr(),
                   T["amin"].data_ptr(), T["amax"].data_ptr(), T["i0"].data_ptr(),
                   T["iN"].data_ptr(), T["valid"].data_ptr())
    counts = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    st = _core.stream(dev)
    call("vg_siddons_count", ctypes.byref(R), counts.data_ptr(), err.data_ptr(), st)
    if int(err.item()) != 0:
        raise ValueError(f"siddons: {int(err.item())} rays produce voxel indices outside the grid "
                         "(the reference raises in ravel_multi_index)")
    off = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    off[1:] = torch.cumsum(counts[:n].to(torch.int64), 0)
    total = int(off[-1].item())
    if total >= 2 ** 31:
        raise VirGpuError("siddons", 1, "more than 2^31 entries")
    off32 = off.to(torch.int32)
    ind = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    ln = torch.empty(max(total, 1), dtype=torch.float32, device=dev)
    call("vg_siddons_fill", ctypes.byref(R), off32.data_ptr(), ind.data_ptr(), ln.data_ptr(), st)
    return ind[:total], ln[:total], off32, shape, grid


def siddons(src, trg, nPixels=128, dPixels=1.0, origin=0.0, ravel=False, flat=False,
            epsilon=1e-5):
    ind, ln, off, shape, grid = siddons_device(src, trg, nPixels, dPixels, origin, epsilon)
    ind, ln, off = ind.cpu().numpy(), ln.cpu().numpy(), off.cpu().numpy()
    if flat:
        return ind, ln, off
    nP = tuple(int(v) for v in grid["n"])
    rays = np.empty(shape, dtype=object)
    flat_rays = rays.reshape(-1)
    for r in range(flat_rays.size):
        a, b = off[r], off[r + 1]
        if a == b:
            continue  # a ray outside the grid stays None, as in the reference
        R, L = ind[a:b], ln[a:b]
        if ravel:
            flat_rays[r] = [R.astype(np.int32), L]
        else:
            x, y, z = np.unravel_index(R, nP)
            flat_rays[r] = [x.astype(np.int32), y.astype(np.int32), z.astype(np.int32), L]
    return rays
