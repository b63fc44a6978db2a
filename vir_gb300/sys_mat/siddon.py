"""Siddon ray lists, drop-in for vir ``sys_mat/siddon.py:siddons``.

``siddons(src, trg, nPixels=128, dPixels=1.0, origin=0.0, ravel=False,
flat=False, epsilon=1e-5)`` returns what the reference returns (siddon.py:636-833):

* ``flat=True``: ``(ind int32, len float32, off int32)``, the CSR form;
* ``ravel=True``: an object array of ``[R int32, L float32]`` per ray;
* otherwise an object array of ``[x_ind, y_ind, z_ind, length]`` per ray;
  rays that miss the grid are ``None``.

The grid planes are vir's float32 boundspace planes, built on the host.  The
per-ray set-up (alpha range, first/last plane index with ``isclose``
rounding: siddon.py:681-751) runs on the GPU (``vg_siddons_setup``, one
thread per ray, each operation in the type numpy gives it, so the values are
bit-identical to the reference's); so does the per-ray loop that sorts the
plane crossings and emits (voxel, length) entries (:754-826, the hot loop;
``vg_siddons_count`` / ``vg_siddons_fill``), in FP32 with the same operation
order.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _core
from .._lib import SiddonRays, SiddonsGrid, VirGpuError, call


def _np3(v, dtype):
    v = np.array(v, dtype=dtype)
    if v.size == 1:
        v = np.repeat(v, 3)
    return v


def _planes(n, d, c):
    # boundspace(n, d, c, dtype=float32) (core_funcs.py:62-81)
    return np.linspace(-n, n, n + 1, dtype=np.float32) * d / 2.0 + c


def setup_device(src, trg, nPixels=128, dPixels=1.0, origin=0.0, epsilon=1e-5, device=None):
    """The per-ray set-up of siddons (siddon.py:681-751) on the device
    (vg_siddons_setup): returns (rays shape, grid, dict of per-ray CUDA
    tensors src, dst, dist, amin, amax, i0, iN, valid).  The grid planes are
    vir's float32 boundspace planes, built on the host."""
    _core.require_cuda()
    dev = device or torch.device("cuda", torch.cuda.current_device())
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
    n = int(np.prod(shape))
    rows = lambda a: np.ascontiguousarray(np.broadcast_to(a, shape + (3,)).reshape(n, 3))
    S = torch.from_numpy(rows(src)).to(dev)
    T = torch.from_numpy(rows(trg)).to(dev)
    f32 = lambda *s: torch.empty(s, dtype=torch.float32, device=dev)
    i32 = lambda *s: torch.empty(s, dtype=torch.int32, device=dev)
    A = dict(src=S, dst=f32(n, 3), dist=f32(n), amin=f32(n), amax=f32(n), i0=i32(n, 3),
             iN=i32(n, 3), valid=torch.empty(n, dtype=torch.uint8, device=dev))
    g = SiddonsGrid(int(nP[0]), int(nP[1]), int(nP[2]), float(dP[0]), float(dP[1]), float(dP[2]),
                    (ctypes.c_float * 3)(Xb[0], Yb[0], Zb[0]),
                    (ctypes.c_float * 3)(Xb[-1], Yb[-1], Zb[-1]), float(epsilon),
                    float(np.float32(epsilon)), 0)
    call("vg_siddons_setup", ctypes.byref(g), n, S.data_ptr(), T.data_ptr(), A["dst"].data_ptr(),
         A["dist"].data_ptr(), A["amin"].data_ptr(), A["amax"].data_ptr(), A["i0"].data_ptr(),
         A["iN"].data_ptr(), A["valid"].data_ptr(), _core.stream(dev))
    grid = dict(n=nP, d=dP, Xb=Xb, Yb=Yb, Zb=Zb)
    return shape, grid, A


def siddons_device(src, trg, nPixels=128, dPixels=1.0, origin=0.0, epsilon=1e-5, device=None):
    """CSR list (ind, len, off) as CUDA tensors, plus the ray shape."""
    _core.require_cuda()
    dev = device or torch.device("cuda", torch.cuda.current_device())
    shape, grid, T = setup_device(src, trg, nPixels, dPixels, origin, epsilon, dev)
    n = int(np.prod(shape))
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
    grid["valid"] = T["valid"]
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
    valid = grid["valid"].cpu().numpy()
    for r in range(flat_rays.size):
        if not valid[r]:
            continue  # a ray that misses the grid stays None, as in the reference
        a, b = off[r], off[r + 1]
        # a ray that enters the grid but keeps no positive length gets empty
        # arrays (siddon.py:758-820 stores them for every such ray)
        R, L = ind[a:b], ln[a:b]
        if ravel:
            flat_rays[r] = [R.astype(np.int32), L]
        else:
            x, y, z = np.unravel_index(R, nP)
            flat_rays[r] = [x.astype(np.int32), y.astype(np.int32), z.astype(np.int32), L]
    return rays


# --- list formats and list algebra (siddon.py:12-633) --------------------------
#
# An sdlist is vir's object array of per-ray voxel lists: [R, L] (raveled,
# R = np.ravel_multi_index((x, y, z), nPixels)) or [X, Y, Z, L] (unraveled),
# None for a ray that misses the grid; the flat form is the CSR triple
# (ind, len, off).  Index bookkeeping stays on the host as in the
# reference; the accumulations (list2array, the ray averages) run on the
# GPU: a scatter-add of the lengths (vg_list_bp) and an ordered compaction
# of the touched voxels (vg_count_nonzero / vg_compact_nonzero).

def ray_ravel(ray, nPixels):
    """siddon.py:592-611"""
    return [np.ravel_multi_index((ray[0], ray[1], ray[2]), tuple(nPixels)).astype(np.int32), ray[3]]


def ray_unravel(ray, nPixels):
    """siddon.py:614-633"""
    x, y, z = np.unravel_index(ray[0], tuple(nPixels))
    return [x.astype(np.int32), y.astype(np.int32), z.astype(np.int32), ray[1]]


def list_ravel(sdlist, nPixels):
    """siddon.py:538-562 (in place)"""
    for i, ray in np.ndenumerate(sdlist):
        if ray is not None:
            sdlist[i] = ray_ravel(ray, nPixels)
    return sdlist


def list_unravel(sdlist, nPixels):
    """siddon.py:565-589 (in place)"""
    for i, ray in np.ndenumerate(sdlist):
        if ray is not None:
            sdlist[i] = ray_unravel(ray, nPixels)
    return sdlist


def list_count_elem(sdlist):
    """siddon.py:166-190"""
    if not isinstance(sdlist, np.ndarray):
        return sdlist[0].size
    count = np.zeros(sdlist.shape, dtype=np.int32)
    for i, ray in np.ndenumerate(sdlist):
        if ray is not None:
            count[i] = ray[0].size
    return count


def list_flatten(sdlist, ravel=False, nPixels=None):
    """siddon.py:490-535: CSR (ind int32 raveled, len float32, off int32)."""
    if not ravel and nPixels is None:
        raise ValueError('nPixels must be provided if ravel=False')
    off = np.insert(np.cumsum(list_count_elem(sdlist)), 0, 0).astype(np.int32)
    ind = np.zeros(off[-1], dtype=np.int32)
    ln = np.zeros(off[-1], dtype=np.float32)
    for r, ray in enumerate(sdlist.flat):
        if ray is not None:
            if not ravel:
                ray = ray_ravel(ray, nPixels)
            ind[off[r]:off[r + 1]] = ray[0]
            ln[off[r]:off[r + 1]] = ray[1]
    return ind, ln, off


def ray_index_shift(ray, shift):
    """siddon.py:251-252"""
    return [ray[0] + shift[0], ray[1] + shift[1], ray[2] + shift[2], ray[3]]


def list_index_shift(sdlist, shift, ravel=False):
    """siddon.py:57-91 (in place; unraveled lists only, as the reference)"""
    shift = np.array(shift, dtype=int)
    if ravel:
        raise ValueError('Cuurently unsuported, ravel must be False')
    for i, ray in np.ndenumerate(sdlist):
        if ray is not None:
            sdlist[i] = ray_index_shift(ray, shift)
    return sdlist


def list_del_ind(sdlist, X_ind, Y_ind, Z_ind, ravel=False):
    """siddon.py:12-54: keep the elements whose x, y and z are listed."""
    if ravel:
        raise ValueError('Cuurently unsuported, ravel must be False')
    for i, ray in np.ndenumerate(sdlist):
        if ray is not None:
            keep = np.isin(ray[0], X_ind) & np.isin(ray[1], Y_ind) & np.isin(ray[2], Z_ind)
            sdlist[i] = [ray[0][keep], ray[1][keep], ray[2][keep], ray[3][keep]]
    return sdlist


def ray_flip(ray, x=None, y=None, z=None, ravel=False, nPixels=None):
    """siddon.py:214-248: reflect indices about x, y, z (2 c - i)."""
    if ravel:
        ray = ray_unravel(ray, nPixels)
    if x:
        ray = [(2 * x - ray[0]).astype(int), ray[1], ray[2], ray[3]]
    if y:
        ray = [ray[0], (2 * y - ray[1]).astype(int), ray[2], ray[3]]
    if z:
        ray = [ray[0], ray[1], (2 * z - ray[2]).astype(int), ray[3]]
    if ravel:
        return [np.ravel_multi_index((ray[0], ray[1], ray[2]), tuple(nPixels)), ray[3]]
    return ray


def list_flip(sdlist, x=None, y=None, z=None, ravel=False, nPixels=None):
    """siddon.py:205-211 (in place)"""
    for i, ray in np.ndenumerate(sdlist):
        if ray is not None:
            sdlist[i] = ray_flip(ray, x=x, y=y, z=z, ravel=ravel, nPixels=nPixels)
    return sdlist


def ray_boundary(ray, nPixels):
    """siddon.py:254-261: drop elements outside the grid."""
    keep = ((ray[0] >= 0) & (ray[0] < nPixels[0]) & (ray[1] >= 0) & (ray[1] < nPixels[1]) &
            (ray[2] >= 0) & (ray[2] < nPixels[2]))
    return [ray[0][keep], ray[1][keep], ray[2][keep], ray[3][keep]]


def list2array_iter_ray(ray, array, ravel=False):
    """siddon.py:94-121: add one ray's lengths into a host array (repeated
    voxels accumulate)."""
    if ravel:
        np.add.at(array.reshape(-1), ray[0], ray[1])
    else:
        np.add.at(array, (ray[0], ray[1], ray[2]), ray[3])


def _csr_device(sdlist, ravel, nPixels, flat, dev):
    if flat:
        ind, ln, off = sdlist[0], sdlist[1], sdlist[2] if len(sdlist) > 2 else None
        if off is None:
            off = np.array([0, np.size(ind)], np.int32)
    else:
        ind, ln, off = list_flatten(sdlist, ravel=ravel, nPixels=nPixels)
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt).to(dev)
    return t(ind, torch.int32), t(ln, torch.float32), t(off, torch.int32)


def _accumulate(sdlist, nPixels, ravel, flat, weights=None):
    """Sum of (weight_r *) lengths per voxel over the rays, on the GPU."""
    from ..projection.proj import list_bp_device
    dev = torch.device("cuda", torch.cuda.current_device())
    _core.require_cuda()
    ind, ln, off = _csr_device(sdlist, ravel, nPixels, flat, dev)
    nrays = off.numel() - 1
    y = (torch.ones(max(nrays, 1), device=dev)[:nrays] if weights is None else
         torch.as_tensor(np.asarray(weights, np.float32).reshape(-1)).to(dev))
    nvox = int(np.prod(nPixels))
    return list_bp_device(y, ind, ln, off, nvox)


def list2array(sdlist, nPixels, ravel=False, flat=False):
    """siddon.py:124-163: per voxel the sum of the rays' intersection lengths."""
    vol = _accumulate(sdlist, nPixels, ravel, flat)
    return vol.reshape(tuple(int(v) for v in nPixels)).cpu().numpy()


def _compact(vol):
    """Indices (increasing) and values of the non-zero entries, on the GPU."""
    L = _core.load()
    n = vol.numel()
    nb = int(L.vg_compact_blocks(n))
    counts = torch.empty(nb, dtype=torch.int32, device=vol.device)
    call("vg_count_nonzero", _core.ptr(vol), n, _core.ptr(counts), _core.stream(vol.device))
    first = torch.zeros(nb + 1, dtype=torch.int64, device=vol.device)
    first[1:] = torch.cumsum(counts.to(torch.int64), 0)
    total = int(first[-1])
    idx = torch.empty(max(total, 1), dtype=torch.int32, device=vol.device)
    val = torch.empty(max(total, 1), dtype=torch.float32, device=vol.device)
    call("vg_compact_nonzero", _core.ptr(vol), n, _core.ptr(first), _core.ptr(idx), _core.ptr(val),
         _core.stream(vol.device))
    return idx[:total].cpu().numpy(), val[:total].cpu().numpy()


def rays_ave(sdlist, ravel=False, flat=False, nPixels=None, nRays=None):
    """siddon.py:432-487: one ray holding every voxel the rays touch, with
    the lengths summed over the rays and divided by their number.  Voxels
    whose summed length is exactly zero are not listed (the reference's
    np.unique keeps them)."""
    if not ravel and nPixels is None:
        raise ValueError('nPixels must be provided if ravel=False')
    if flat and nRays is None:
        raise ValueError('nRays must be provided if flat=True')
    if not flat and nPixels is None:
        raise ValueError('nPixels must be provided if flat=False')
    if not flat:
        nRays = sdlist.size
    nvox = int(np.prod(nPixels)) if nPixels is not None else int(np.max(sdlist[0])) + 1
    idx, val = _compact(_accumulate(sdlist, (nvox,) if nPixels is None else nPixels, ravel, flat))
    if idx.size == 0:
        return None
    val = (val / np.float32(nRays)).astype(np.float32)
    if ravel or flat:
        return [idx, val]
    return ray_unravel([idx, val], nPixels)


def list_ave(sdlist, ravel=False, flat=False, nPixels=None, nRays=None, axis=None):
    """siddon.py:388-429: rays_ave over the given axes of the ray array."""
    if flat and axis is not None:
        raise ValueError('Axis cannot be provided when flat=True')
    if axis is None:
        return rays_ave(sdlist, ravel=ravel, flat=flat, nPixels=nPixels, nRays=nRays)
    out = np.empty(np.delete(sdlist.shape, axis), dtype=object)
    moved = np.moveaxis(sdlist, axis, np.arange(-1 * (np.array(axis).size), 0))
    for i, _ in np.ndenumerate(out):
        out[i] = rays_ave(moved[i], ravel=ravel, flat=flat, nPixels=nPixels, nRays=nRays)
    return out


def rays_weight_ave(sdlist, weights, ravel=False, nPixels=None):
    """siddon.py:350-385: one ray with sum_r weights[r] * lengths per voxel
    (no division)."""
    if not ravel and nPixels is None:
        raise ValueError('nPixels must be provided if ravel=False')
    w = np.asarray(weights, np.float32).reshape(sdlist.shape)
    idx, val = _compact(_accumulate(sdlist, nPixels, ravel, False, weights=w))
    if idx.size == 0:
        return None
    return [idx, val] if ravel else ray_unravel([idx, val], nPixels)


def list_weight_ave(sdlist, weights, ravel=False, nPixels=None, axis=None):
    """siddon.py:328-347"""
    if axis is None:
        return rays_weight_ave(sdlist, weights, ravel=ravel, nPixels=nPixels)
    if len(axis) != weights.ndim:
        raise ValueError('Number of axis must match weights dimensions')
    out = np.empty(np.delete(sdlist.shape, axis), dtype=object)
    moved = np.moveaxis(sdlist, axis, np.arange(-1 * (np.array(axis).size), 0))
    for i, _ in np.ndenumerate(out):
        out[i] = rays_weight_ave(moved[i], weights, ravel=ravel, nPixels=nPixels)
    return out


def list_convole(sdlist, kernel, ravel=False, nPixels=None, axis=None):
    """siddon.py:265-325: each ray replaced by the kernel-weighted
    combination of its neighbours along ``axis`` (kernel renormalised at the
    array's edges)."""
    if len(axis) != kernel.ndim:
        raise ValueError('Number of axis must match kernel dimensions')
    if any(d % 2 == 0 for d in kernel.shape):
        raise ValueError('Kernel must have an odd numer of elements in each dimension')
    out = np.empty(sdlist.shape, dtype=object)
    for ray_idx, _ in np.ndenumerate(sdlist):
        r_sl, k_sl = list(ray_idx), []
        for i, (ax, kd) in enumerate(zip(axis, kernel.shape)):
            s0 = ray_idx[ax] - kd // 2
            k0 = -s0 if s0 < 0 else 0
            s0 = max(s0, 0)
            s1 = ray_idx[ax] + kd // 2 + 1
            k1 = kd - (s1 - sdlist.shape[ax]) if s1 > sdlist.shape[ax] else kd
            s1 = min(s1, sdlist.shape[ax])
            r_sl[ax] = slice(s0, s1)
            k_sl.append(slice(k0, k1))
        k = kernel[tuple(k_sl)]
        kf = kernel.sum() / k.sum()
        out[ray_idx] = rays_weight_ave(sdlist[tuple(r_sl)], kf * k, ravel=ravel, nPixels=nPixels)
    return out
