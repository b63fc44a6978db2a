"""Helical rebinning front-end: vir's ``trajectory.py`` with the sinogram
work on the GPU.

Drop-ins (same names, arguments, shapes and float32 results):

* ``sino_axl2hel(sinoA, nRowsH, ViewsH, nAngsH, pitch, Z=None)`` -- helical
  projections resampled from an axial sinogram (trajectory.py:45-67): each
  helical view's fractional axial view index and z shift are found on the
  host exactly as the reference finds them; the device evaluates
  ``scipy.ndimage.map_coordinates(order=1)`` with scipy's arithmetic
  (``vg_axl2hel``), so the result equals the reference's bit for bit,
  including the 'grid-wrap' branch for views past the last axial angle.
* ``sino_hel2axl(sinoH, geomH, AngsA, Z)``, ``sino_hel2axl180(...)``,
  ``sino_hel2hel(sinoAcq, geomAcq, geomInt, nRowsInt)`` -- axial (or
  helical) sinograms interpolated from a helical acquisition
  (trajectory.py:70-240): the geometry's ``interpZ`` (the caller's object --
  vir's ``core_funcs.Geom`` or :class:`Geom` here) gives each output row's
  two source rows and weights on the host; ``vg_rebin_rows`` gathers them in
  float64 and stores float32, as numpy does (bit-exact).
* ``sino_hel_subset(sino, geomH, nRows, z)`` (trajectory.py:243-254).
* ``forward_project_phantom(phantom, Views, Rows, Cols, Z)`` -- the rotate,
  translate and sum-along-y projector used to simulate helical data
  (trajectory.py:17-42), ``vg_rotsum_fp``; float32 trilinear sampling where
  the reference samples in float64, so it agrees to float32 rounding.

:class:`Geom` restates the trajectory part of vir's ``core_funcs.Geom``
(core_funcs.py:439-730: views, helical z positions, ``updateViews``,
``interpZ``) for callers without vir.

Sinograms may be numpy arrays (results come back as numpy) or torch CUDA
tensors (results stay on the device).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _core
from ._lib import VirGpuError, call


def censpace(n, d=1.0, c=0.0, dtype=float):
    """Sample centres: n values d apart centred at c (core_funcs.py:37-59)."""
    return np.linspace(-n + 1, n - 1, n, dtype=dtype) * d / 2.0 + c


class Geom:
    """The views and helical z positions of vir's core_funcs.Geom
    (core_funcs.py:439-730), with its ``interpZ``."""

    def __init__(self, nViews=512, coverage=2.0 * np.pi, angle0=0.0, pitch=0.0, endpoint=False,
                 src_iso=np.inf, src_det=np.inf, fan_angle=0.0, zTran=0.0):
        self.nViews = int(nViews)
        self.coverage = coverage
        self.angle0 = angle0
        self.pitch = pitch
        self.endpoint = endpoint
        self.src_iso = src_iso
        self.src_det = src_det
        self.fan_angle = fan_angle
        self.zTran = zTran
        self.Views, self.dView = np.linspace(self.angle0, self.angle0 + self.coverage, self.nViews,
                                             endpoint=self.endpoint, retstep=True)
        self.nRotations = coverage / (2.0 * np.pi)
        nAngles = 2 * np.pi / self.dView
        self.nAngles = round(nAngles) if np.isclose(nAngles, round(nAngles)) else nAngles
        if self.fan_angle != 0.0:
            if self.src_iso == np.inf or self.src_det == np.inf:
                raise ValueError("Fanbeam set, src_iso and src_det must be provided")
            self.geom = "Fan beam"
            self.fov = 2.0 * self.src_iso * np.sin(self.fan_angle / 2.0)
        else:
            self.geom = "Parallel beam"
        self.dZ = self.zTran * self.nRotations / self.nViews
        self.Z = censpace(self.nViews, self.dZ)

    def updateViews(self, Views, dView=None, coverage=None, Z=None):
        self.Views = np.array(Views)
        if dView is None:
            self.dView = np.mean(Views[1:] - Views[:-1])
        if coverage is None:
            self.coverage = self.Views[-1] - self.Views[0] + self.dView
        self.nViews = self.Views.size
        self.angle0 = self.Views[0]
        self.nRotations = self.coverage / (2.0 * np.pi)
        self.Z = censpace(self.nViews, self.dZ) if Z is None else Z

    def bins(self, nBins):
        return censpace(nBins, self.fan_angle / nBins * self.src_det)

    def gammas(self, nGammas):
        return censpace(nGammas, self.fan_angle / nGammas)

    def interpZ(self, intZ, angle, nRows, all_views=False):
        """For slices intZ and a projection angle: the views at that angle
        (one per rotation) at or just after (p) and just before (n) it, and in
        each the detector rows just below and above every slice, with their
        z distances; the closest pair by sqrt(dz^2 + (dview/dView)^2)
        (core_funcs.py:574-730).  Returns (idxVp, dVp, idxR_Vp, dR_Vp, idxVn,
        dVn, idxR_Vn, dR_Vn); pairs are (below, above)."""
        intZ = np.array(intZ)
        angle = angle % (2.0 * np.pi)
        angles = np.arange(np.ceil(self.nRotations) + 1) * 2.0 * np.pi + angle
        V = self.Views
        vp = np.searchsorted(V, angles, side='left')
        vp = np.where(np.isclose(V[vp - 1], angles), vp - 1, vp) % self.nViews
        vn = np.where(np.isclose(V[vp], angles), vp, vp - 1) % self.nViews
        if vn[-1] == vn[-2] and vp[-1] == vp[-2]:
            vn, vp, angles = vn[:-1], vp[:-1], angles[:-1]
        rows = censpace(nRows)
        zp = np.add.outer(self.Z[vp], rows)
        zn = np.add.outer(self.Z[vn], rows)
        dVn = np.tile(V[vn] - angles, [intZ.size, 1]).T
        dVp = np.tile(V[vp] - angles, [intZ.size, 1]).T % (2 * np.pi)
        dVn = np.where(np.isclose(dVn, 0.0), 0.0, dVn)
        dVp = np.where(np.isclose(dVp, 0.0), 0.0, dVp)
        dVn = np.where(np.isclose(dVn, 2 * np.pi), 0.0, dVn)
        dVp = np.where(np.isclose(dVp, 2 * np.pi), 0.0, dVp)

        def rows_around(zs):
            lo = np.zeros((zs.shape[0], intZ.size), dtype=int)
            hi = np.zeros((zs.shape[0], intZ.size), dtype=int)
            for i in range(zs.shape[0]):
                up = np.array(np.searchsorted(zs[i], intZ))
                dn = np.where(np.isclose(zs[i, up.clip(0, nRows - 1)], intZ), up, up - 1)
                hi[i] = up.clip(0, nRows - 1)
                lo[i] = dn.clip(0, nRows - 1)
            return lo, hi, np.take_along_axis(zs, lo, 1) - intZ, np.take_along_axis(zs, hi, 1) - intZ

        lo_p, hi_p, dlo_p, dhi_p = rows_around(zp)
        lo_n, hi_n, dlo_n, dhi_n = rows_around(zn)
        if all_views:
            return (vp, dVp, np.stack([lo_p, hi_p], -1), np.stack([dlo_p, dhi_p], -1),
                    vn, dVn, np.stack([lo_n, hi_n], -1), np.stack([dlo_n, dhi_n], -1))
        iz = range(intZ.size)

        def closest(v, dV, lo, hi, dlo, dhi):
            dlo = np.where(dlo <= 0, dlo, -np.inf)
            dhi = np.where(dhi >= 0, dhi, np.inf)
            a = np.sqrt(dlo ** 2 + (dV / self.dView) ** 2).argmin(axis=0)
            b = np.sqrt(dhi ** 2 + (dV / self.dView) ** 2).argmin(axis=0)
            return (np.stack([v[a], v[b]], -1), np.stack([dV[a, iz], dV[b, iz]], -1),
                    np.stack([lo[a, iz], hi[b, iz]], -1), np.stack([dlo[a, iz], dhi[b, iz]], -1))

        return (*closest(vp, dVp, lo_p, hi_p, dlo_p, dhi_p),
                *closest(vn, dVn, lo_n, hi_n, dlo_n, dhi_n))


def _interpZ_batch(geom, intZ, angles, nRows):
    """Geom.interpZ for many angles at once, stacked (angles, slices, 2): the
    same comparisons and arithmetic as one call per angle, broadcast over the
    angles (searchsorted 'left' on a sorted row set is its count of entries
    below the slice; an angle whose last rotation repeats the one before
    excludes it, as interpZ drops it)."""
    intZ = np.array(intZ, dtype=float)
    ang = np.asarray(angles, dtype=float) % (2.0 * np.pi)
    K = int(np.ceil(geom.nRotations)) + 1
    A = np.arange(np.ceil(geom.nRotations) + 1)[None, :] * 2.0 * np.pi + ang[:, None]
    V, nV = geom.Views, geom.nViews
    vp = np.searchsorted(V, A, side='left')
    vp = np.where(np.isclose(V[vp - 1], A), vp - 1, vp) % nV
    vn = np.where(np.isclose(V[vp], A), vp, vp - 1) % nV
    drop = (vn[:, -1] == vn[:, -2]) & (vp[:, -1] == vp[:, -2]) if K > 1 else np.zeros(len(ang), bool)
    rows = censpace(nRows)
    nz = intZ.size

    def dview(v, wrap):
        d = V[v] - A
        if wrap:
            d = d % (2 * np.pi)
        d = np.where(np.isclose(d, 0.0), 0.0, d)
        d = np.where(np.isclose(d, 2 * np.pi), 0.0, d)
        return np.broadcast_to(d[:, :, None], d.shape + (nz,))

    def side(v, dV):
        zs = geom.Z[v][..., None] + rows                                     # (na, K, nRows)
        up = (zs[:, :, None, :] < intZ[None, None, :, None]).sum(-1)           # (na, K, nz)
        upc = up.clip(0, nRows - 1)
        dn = np.where(np.isclose(np.take_along_axis(zs, upc, 2), intZ), up, up - 1)
        hi, lo = upc, dn.clip(0, nRows - 1)
        dlo = np.take_along_axis(zs, lo, 2) - intZ
        dhi = np.take_along_axis(zs, hi, 2) - intZ
        dlo = np.where(dlo <= 0, dlo, -np.inf)
        dhi = np.where(dhi >= 0, dhi, np.inf)
        out = []
        for d, r in ((dlo, lo), (dhi, hi)):
            dist = np.sqrt(d ** 2 + (dV / geom.dView) ** 2)
            dist[drop, -1, :] = np.inf
            k = dist.argmin(axis=1)[:, None, :]                              # (na, 1, nz)
            out.append((np.take_along_axis(np.broadcast_to(v[:, :, None], dist.shape), k, 1)[:, 0],
                        np.take_along_axis(dV, k, 1)[:, 0], np.take_along_axis(r, k, 1)[:, 0],
                        np.take_along_axis(d, k, 1)[:, 0]))
        (va, dva, ra, da), (vb, dvb, rb, db) = out
        return (np.stack([va, vb], -1), np.stack([dva, dvb], -1), np.stack([ra, rb], -1),
                np.stack([da, db], -1))

    return side(vp, dview(vp, True)) + side(vn, dview(vn, False))


def _pair_weights(idxV, idxR, dR):
    """Rows and weights of one interpolated slice set (trajectory.py:84-93)."""
    wR = dR[:, 1] - dR[:, 0]
    with np.errstate(invalid='ignore', divide='ignore'):
        w0 = np.where(wR == 0.0, 0.5, ((wR + dR[:, 0]) / wR))
        w1 = np.where(wR == 0.0, 0.5, ((wR - dR[:, 1]) / wR))
    pairs = np.stack([idxV[:, 0], idxR[:, 0], idxV[:, 1], idxR[:, 1]], -1).astype(np.int32)
    return pairs, np.stack([w0, w1], -1).astype(np.float64)


def _tables(geom, Zs, angs, nRows):
    """(pairs, weights) of the p and n interpolations for every (angle, z)
    row, stacked angle-major.  This package's Geom evaluates all angles of
    one slice set at once; other geometry objects are asked per angle."""
    if isinstance(geom, Geom) and len(Zs) and all(np.array_equal(Zs[0], z) for z in Zs):
        vp, _, rp, drp, vn, _, rn, drn = _interpZ_batch(geom, Zs[0], angs, nRows)
        flat = lambda a: a.reshape(-1, 2)
        a, b = _pair_weights(flat(vp), flat(rp), flat(drp))
        c, d = _pair_weights(flat(vn), flat(rn), flat(drn))
        return a, b, c, d
    pp, wp, pn, wn = [], [], [], []
    for Z, ang in zip(Zs, angs):
        vp, _, rp, drp, vn, _, rn, drn = geom.interpZ(Z, ang, nRows)
        a, b = _pair_weights(vp, rp, drp)
        pp.append(a)
        wp.append(b)
        a, b = _pair_weights(vn, rn, drn)
        pn.append(a)
        wn.append(b)
    return np.concatenate(pp), np.concatenate(wp), np.concatenate(pn), np.concatenate(wn)


def _gather(src, pairs, w, shape, reverse=False):
    dev = src.device
    nv, nr, nc = src.shape
    p = torch.from_numpy(np.ascontiguousarray(pairs)).to(dev)
    ww = torch.from_numpy(np.ascontiguousarray(w)).to(dev)
    out = torch.empty(shape, dtype=torch.float32, device=dev)
    bad = torch.zeros(1, dtype=torch.int64, device=dev)
    n = pairs.shape[0]
    for o0 in range(0, n, 65535):
        o1 = min(n, o0 + 65535)
        call("vg_rebin_rows", _core.ptr(src), nv, nr, nc, _core.ptr(p[o0:o1]), _core.ptr(ww[o0:o1]),
             o1 - o0, int(reverse), _core.ptr(out) + 4 * o0 * nc, _core.ptr(bad),
             _core.stream(dev))
    if int(bad.item()):
        raise IndexError("interpZ returned a view or row index outside the sinogram")
    return out


def _src(sino):
    t = _core.to_device(sino)
    if t.dim() != 3:
        raise ValueError("sinogram must be (views, rows, cols)")
    return t


def sino_hel2axl(sinoH, geomH, AngsA, Z):
    """Two axial sinograms (AngsA, Z, cols) interpolated from the helical
    views at or after (1) and before (2) each angle (trajectory.py:70-105)."""
    src = _src(sinoH)
    AngsA, Z = np.array(AngsA), np.array(Z)
    pp, wp, pn, wn = _tables(geomH, [Z] * AngsA.size, AngsA, src.shape[1])
    shape = (AngsA.size, Z.size, src.shape[2])
    return (_core.to_host_like(_gather(src, pp, wp, shape), sinoH),
            _core.to_host_like(_gather(src, pn, wn, shape), sinoH))


def sino_hel2axl180(sinoH, geomH, AngsA, Z):
    """As sino_hel2axl at each angle and at angle + pi, the latter with the
    columns reversed (trajectory.py:109-170)."""
    src = _src(sinoH)
    AngsA, Z = np.array(AngsA), np.array(Z)
    nr, shape = src.shape[1], (AngsA.size, Z.size, src.shape[2])
    pp, wp, pn, wn = _tables(geomH, [Z] * AngsA.size, AngsA, nr)
    bp, bwp, bn, bwn = _tables(geomH, [Z] * AngsA.size, AngsA + np.pi, nr)
    outs = (_gather(src, pp, wp, shape), _gather(src, pn, wn, shape),
            _gather(src, bp, bwp, shape, reverse=True), _gather(src, bn, bwn, shape, reverse=True))
    return tuple(_core.to_host_like(o, sinoH) for o in outs)


def sino_hel2hel(sinoAcq, geomAcq, geomInt, nRowsInt):
    """Helical sinograms on geomInt's views and z positions (nRowsInt rows
    about each) interpolated from an acquisition (trajectory.py:173-240)."""
    src = _src(sinoAcq)
    Zs = [censpace(nRowsInt, c=z) for z in geomInt.Z]
    pp, wp, pn, wn = _tables(geomAcq, Zs, list(geomInt.Views), src.shape[1])
    shape = (geomInt.nViews, nRowsInt, src.shape[2])
    return (_core.to_host_like(_gather(src, pp, wp, shape), sinoAcq),
            _core.to_host_like(_gather(src, pn, wn, shape), sinoAcq))


def sino_hel_subset(sino, geomH, nRows, z):
    """The views whose rows reach the slices z; restricts geomH to them
    (trajectory.py:243-254)."""
    z = np.array(z)
    lo = np.searchsorted(geomH.Z + (nRows / 2 - .5), z.min() - 1, side='right')
    hi = np.searchsorted(geomH.Z - (nRows / 2 - .5), z.max()) + 1
    geomH.updateViews(geomH.Views[lo:hi], Z=geomH.Z[lo:hi])
    return sino[lo:hi, ...]


def axl2hel_index(nAngsA, nRowsA, nRowsH, ViewsH, nAngsH, pitch, Z=None):
    """Per helical view: the fractional axial view index, the row shift and
    whether the view lies past the last axial angle (trajectory.py:45-67);
    also how many views have a z position."""
    Angs = np.linspace(0, 2 * np.pi, nAngsA + 1, endpoint=True)
    if Z is None:
        dZ = pitch * nRowsH / nAngsH
        Z = censpace(ViewsH.size, c=nRowsA / 2 - nRowsH / 2, d=dZ)
    idx = np.zeros(ViewsH.size)
    wrap = np.zeros(ViewsH.size, np.int32)
    zz = np.zeros(ViewsH.size)
    n_used = min(len(Z), ViewsH.size)  # the reference zips Z with the views
    zz[:n_used] = np.asarray(Z, np.float64)[:n_used]
    for i, view in enumerate(ViewsH[:n_used]):
        view = view % (2 * np.pi)
        k = (np.abs(Angs - view)).argmin()
        idx[i] = np.round(k) if np.isclose(Angs[k], view) else np.interp(view, Angs, np.arange(nAngsA + 1))
        if (view > Angs[-2]) & ~np.isclose(view, Angs[-2]):
            print("Extrapolation warning:", i, view)
            wrap[i] = 1
    return idx, zz, wrap, n_used


def sino_axl2hel(sinoA, nRowsH, ViewsH, nAngsH, pitch, Z=None):
    """Helical sinogram (ViewsH, nRowsH, cols) resampled from an axial one
    (trajectory.py:45-67)."""
    src = _src(sinoA)
    ViewsH = np.asarray(ViewsH)
    nA, nR, nC = src.shape
    idx, zz, wrap, n_used = axl2hel_index(nA, nR, nRowsH, ViewsH, nAngsH, pitch, Z)
    dev = src.device
    out = torch.empty((ViewsH.size, nRowsH, nC), dtype=torch.float32, device=dev)
    ti = torch.from_numpy(idx).to(dev)
    tz = torch.from_numpy(np.ascontiguousarray(zz)).to(dev)
    tw = torch.from_numpy(wrap).to(dev)
    for v0 in range(0, ViewsH.size, 65535):
        v1 = min(ViewsH.size, v0 + 65535)
        call("vg_axl2hel", _core.ptr(src), nA, nR, nC, _core.ptr(ti) + 8 * v0,
             _core.ptr(tz) + 8 * v0, _core.ptr(tw) + 4 * v0, v1 - v0, int(nRowsH),
             _core.ptr(out) + 4 * v0 * nRowsH * nC, _core.stream(dev))
    out[n_used:] = 0  # views without a z position stay zero, as in the reference
    return _core.to_host_like(out, sinoA)


def view_matrices(shape, Views, Z):
    """Per view the first three rows of R_A @ T (trajectory.py:27-37): T moves
    the phantom by -z along the rotation axis, R_A turns it by -view about
    the z axis through the phantom centre; float32 as vir's
    affine_transforms builds them (affine_transforms.py:46-132)."""
    from scipy.spatial import transform
    c = np.array(shape) / 2.0 - 0.5
    Tc = np.identity(4, dtype=np.float32)
    Tc[:3, -1] = c
    out = np.zeros((len(Views), 3, 4), np.float32)
    for i, (z, view) in enumerate(zip(Z, Views)):
        T = np.identity(4, dtype=np.float32)
        T[:3, -1] = (0, 0, -z)
        R = np.identity(4, dtype=np.float32)
        R[:3, :3] = transform.Rotation.from_euler('XYZ', (0, 0, -view)).as_matrix().squeeze() \
            .astype(np.float32)
        RA = Tc @ R @ np.linalg.inv(Tc)
        out[i] = (RA @ T)[:3]
    return out


def forward_project_phantom(phantom, Views, Rows, Cols, Z):
    """Helical projections (views, nZ, nX) of a phantom rotated by -view about
    z and shifted by -z per view, summed along y (trajectory.py:17-42)."""
    vol = _core.to_device(phantom)
    if vol.dim() != 3:
        raise ValueError("phantom must be (nX, nY, nZ)")
    nX, nY, nZ = vol.shape
    Views = np.asarray(Views)
    M = torch.from_numpy(view_matrices((nX, nY, nZ), Views, np.asarray(Z))).to(vol.device)
    out = torch.empty((Views.size, nZ, nX), dtype=torch.float32, device=vol.device)
    for v0 in range(0, Views.size, 65535):
        v1 = min(Views.size, v0 + 65535)
        call("vg_rotsum_fp", _core.ptr(vol), nX, nY, nZ, _core.ptr(M) + 48 * v0, v1 - v0,
             _core.ptr(out) + 4 * v0 * nZ * nX, _core.stream(vol.device))
    return _core.to_host_like(out, phantom)


__all__ = ["Geom", "censpace", "sino_axl2hel", "sino_hel2axl", "sino_hel2axl180", "sino_hel2hel",
           "sino_hel_subset", "forward_project_phantom", "axl2hel_index", "view_matrices"]
