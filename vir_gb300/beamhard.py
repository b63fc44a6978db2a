"""Beam-hardening pre-correction of logged sinograms: vir's
``processing/beamhard.py`` with the per-sample corrections on the GPU.

Drop-ins (same names, arguments and results):

* ``beamhard_cor(line_ints, coefs, mu)`` -- the water polynomial
  ``mu (c0 t^2 + c1 t + c2)``, ``t = line_ints / mu`` (beamhard.py:39-47).
  The result has the dtype numpy gives the reference's expression (float64
  for np.polyfit coefficients) and equals it bit for bit: csrc/beamhard.cu
  replays each operation in numpy's type, separately rounded.
* ``beamhard_cor_table(line_ints, energies, counts, g, atten_eff)`` --
  the spectrum lookup of beamhard.py:16-36: the polyenergetic path length of
  1000 water thicknesses in [0, 80] builds a table that scipy's ``interp1d``
  inverts, evaluated here on the device with interp1d's arithmetic; values
  above the table raise ``ValueError`` as interp1d does.
* ``beamhard_coefs2(energies, counts, g, atten_eff)`` and
  ``beamhard_coefs(energies, counts, det_prob, FocalLength, src_det,
  alpha)`` -- the quadratic fits of beamhard.py:50-113 (host FP64, small).
* ``water_tub_phantom(npixels, dpixel, tub_radius)`` (beamhard.py:116-122).

Also ``beamhard_cor2(line_ints, coefs, mu)``, the lookup-table correction
``line_ints * np.interp(line_ints / mu, linspace(0, 40, 4001), coefs)`` of the
reference's beam-hardening study (tests/Test_Beamhard/beamhard_test.py:26-27).

The reference takes water attenuations from ``xcompy.mixatten('H2O', E)``,
an X-ray attenuation database that is not part of vir and not installed
here: the functions that need it take ``mixatten=`` (a callable with that
signature), defaulting to ``xcompy.mixatten`` when that package imports.  ``beamhard_coefs`` projects the water
tub with ``pj.fan_forwardproject`` of a module outside vir's projector path;
here the default is this package's fan-beam distance-driven projector of the
same geometry (``forward_project=`` takes any other).  In
``beamhard_coefs2`` the parallel-beam branch of the reference cannot run
(``AnalyticSinoParSphere`` reads ``.size`` of the Python list it is given,
intersection_sino.py:98-100); here it computes the chord lengths that branch
intends, 2 sqrt(r^2 - u^2).

Inputs may be numpy arrays (results come back as numpy) or torch tensors
(results stay on the device).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _core
from ._lib import call

MAX_TABLE = 4096  # VG_BH_MAX_TABLE


def _need_mixatten(mixatten, fn):
    if mixatten is None:
        try:  # the reference's database, when the caller's environment has it
            import xcompy
            return xcompy.mixatten
        except ImportError:
            pass
        raise ValueError(
            f"{fn}: water attenuations come from an X-ray attenuation database "
            "(the reference calls xcompy.mixatten('H2O', energies)); pass "
            "mixatten=<callable(material, energies)>")
    return mixatten


def _device_input(line_ints):
    """(device tensor of float32/float64, numpy dtype of the caller's data)."""
    if _core.is_torch(line_ints):
        t = line_ints.detach()
        if t.dtype not in (torch.float32, torch.float64):
            t = t.to(torch.float32)
        dt = np.float32 if t.dtype == torch.float32 else np.float64
        return t.to(_core.device_of(line_ints)).contiguous(), dt
    a = np.asarray(line_ints)
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64)
    return _core.to_device(a, dtype=torch.float32 if a.dtype == np.float32 else torch.float64), a.dtype.type


def _finish(out, like):
    return _core.to_host_like(out, like)


def _poly_types(dt, coefs, mu):
    """Which steps of mu * (c0 t**2 + c1 t + c2), t = x / mu, numpy computes
    in float32 for data of dtype dt: probed on one element with the caller's
    own coefficient and mu objects."""
    x = np.ones(1, dt)
    t = x / mu
    p0 = coefs[0] * t ** 2
    p1 = coefs[1] * t
    s2 = p0 + p1 + coefs[2]
    r = mu * s2
    f32 = [a.dtype == np.float32 for a in (t, p0, p1, s2, r)]
    mask = sum(1 << i for i, b in enumerate(f32) if b)
    return mask, r.dtype.type


def beamhard_cor(line_ints, coefs, mu):
    """vir's beamhard_cor (beamhard.py:39-47) on the device."""
    src, dt = _device_input(line_ints)
    mask, odt = _poly_types(dt, coefs, mu)
    out = torch.empty(src.shape, dtype=torch.float32 if odt == np.float32 else torch.float64,
                      device=src.device)
    if src.numel():
        call("vg_bh_poly", _core.ptr(src), int(src.dtype == torch.float64), _core.ptr(out),
             int(out.dtype == torch.float64), ctypes.c_size_t(src.numel()), float(mu),
             float(coefs[0]), float(coefs[1]), float(coefs[2]), mask, _core.stream(src.device))
    return _finish(out, line_ints)


def _interp_table(x, y, dev, key_f32, round_up):
    """Device table of vg_bh_interp: rows (x_k, y_k, slope_k, 0) with the
    slope of segment k divided as the reference divides it, and the search
    keys (x rounded to float32 toward -inf / +inf when key_f32)."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    m = x.size
    if m < 2 or m > MAX_TABLE:
        raise ValueError(f"lookup table of {m} entries (2..{MAX_TABLE})")
    seg = np.zeros((m, 4))
    seg[:, 0] = x
    seg[:, 1] = y
    seg[:-1, 2] = (y[1:] - y[:-1]) / (x[1:] - x[:-1])
    if key_f32:
        kf = x.astype(np.float32)
        if round_up:
            kf = np.where(kf.astype(np.float64) < x, np.nextafter(kf, np.float32(np.inf)), kf)
        else:
            kf = np.where(kf.astype(np.float64) > x, np.nextafter(kf, np.float32(-np.inf)), kf)
        keys = kf.astype(np.float32)
    else:
        keys = x
    return (torch.from_numpy(np.ascontiguousarray(seg)).to(dev),
            torch.from_numpy(np.ascontiguousarray(keys)).to(dev))


def _interp(line_ints, x, y, mode, mu=1.0):
    src, dt = _device_input(line_ints)
    f32 = src.dtype == torch.float32
    key_f32 = (mode == 0 and f32) or mode == 1
    seg, keys = _interp_table(x, y, src.device, key_f32, round_up=mode != 0)
    out = torch.empty(src.shape, dtype=torch.float64, device=src.device)
    cnt = torch.zeros(1, dtype=torch.int64, device=src.device)
    if src.numel():
        call("vg_bh_interp", _core.ptr(src), int(not f32), _core.ptr(out), 1,
             ctypes.c_size_t(src.numel()), _core.ptr(seg), _core.ptr(keys), int(key_f32),
             int(seg.shape[0]), mode, float(mu), _core.ptr(cnt), _core.stream(src.device))
    return out, int(cnt.item()) if mode == 0 else 0


def spectrum_table(energies, counts, atten_eff, attens):
    """The (x, y) table of beamhard_cor_table (beamhard.py:30-34): x the
    effective-energy line integral of each water thickness in [0, 80], y the
    monoenergetic one, sorted by x as interp1d sorts its abscissae."""
    path_lengths = np.linspace(0, 80, 1000)
    path_lengths_p = -1.0 * np.log(
        np.sum(counts * np.exp(-1.0 * np.outer(path_lengths, attens)), axis=1)
        / np.sum(counts)) / atten_eff
    x = path_lengths_p * atten_eff
    y = path_lengths * atten_eff
    order = np.argsort(x, kind="mergesort")
    return x[order], y[order]


def beamhard_cor_table(line_ints, energies, counts, g, atten_eff, mixatten=None):
    """vir's beamhard_cor_table (beamhard.py:16-36); ``g`` is unused there too."""
    attens = _need_mixatten(mixatten, "beamhard_cor_table")("H2O", energies)
    x, y = spectrum_table(energies, counts, atten_eff, attens)
    out, n_out = _interp(line_ints, x, y, 0)
    if n_out:
        raise ValueError(f"A value in x_new is above the interpolation range's maximum value "
                         f"({x[-1]}): {n_out} of them.")
    return _finish(out, line_ints)


def beamhard_cor2(line_ints, coefs, mu):
    """line_ints * np.interp(line_ints / mu, linspace(0, 40, 4001), coefs)
    (tests/Test_Beamhard/beamhard_test.py:26-27)."""
    coefs = np.asarray(coefs, np.float64)
    xp = np.linspace(0, 40, 4001)
    if coefs.size != xp.size:
        raise ValueError("fp and xp are not of the same length.")
    if _core.is_torch(line_ints):
        dt = np.float64 if line_ints.dtype == torch.float64 else np.float32
    else:
        dt = np.asarray(line_ints).dtype
        dt = dt if dt in (np.float32, np.float64) else np.float64
    f32div = (np.ones(1, dt) / mu).dtype == np.float32
    out, _ = _interp(line_ints, xp, coefs, 1 if f32div else 2, mu)
    return _finish(out, line_ints)


def water_tub_phantom(npixels=512, dpixel=.1, tub_radius=20):
    """Binary disc of radius tub_radius (beamhard.py:116-122)."""
    x, y = np.indices((npixels, npixels))
    return (x - npixels / 2) ** 2 + (y - npixels / 2) ** 2 < (tub_radius / dpixel) ** 2


def _censpace(n, d=1.0, c=0.0):
    return np.linspace(-n + 1, n - 1, n) * d / 2.0 + c


def sphere_chords_fan(radius, gammas, src_iso):
    """Chord lengths of a centred sphere of radius r for fan angles gammas
    at view 0, as intersection_sino.AnalyticSinoFanSphere evaluates them
    (intersection_sino.py:105-121) for S = [0, 0, r]."""
    S = [0, 0, radius]
    xi = src_iso * np.sin(gammas) + 0.0 * np.cos(gammas)
    s = np.sqrt(S[0] ** 2 + S[1] ** 2)
    delta = np.arctan2(S[0], S[1])
    phi = np.add.outer(0, gammas)
    f = S[2] ** 2 * (np.cos(phi) ** 2 + np.sin(phi) ** 2)
    u = xi + s * np.cos(delta - phi)
    return (2. * S[2] ** 2 / f) * np.sqrt((f - u ** 2).clip(0))


def _poly_fit(path_lengths, energies, counts, attens, atten_eff, weights=None, I0=None):
    if weights is None:
        pp = -1.0 * np.log(np.sum(counts * np.exp(-1.0 * np.outer(path_lengths, attens)), axis=1)
                           / np.sum(counts)) / atten_eff
    else:
        pp = -1.0 * np.log(np.trapezoid(counts * np.exp(-1.0 * np.outer(path_lengths, attens))
                                        * weights, x=energies, axis=1) / I0) / atten_eff
    return np.polyfit(pp, path_lengths, 2)


def beamhard_coefs2(energies, counts, g, atten_eff, mixatten=None):
    """vir's beamhard_coefs2 (beamhard.py:50-78): quadratic fit of the
    monoenergetic against the polyenergetic path lengths through a water
    sphere of radius 20, over half of 512 bins.  ``g`` provides ``geom``
    ('Fan beam' / 'Parallel beam'), ``gammas(n)`` and ``src_iso`` as the
    reference's Geom does."""
    attens = _need_mixatten(mixatten, "beamhard_coefs2")("H2O", energies)
    nBins = 512
    if g.geom == 'Fan beam':
        pl = sphere_chords_fan(20, g.gammas(nBins), g.src_iso)
    elif g.geom == 'Parallel beam':
        u = _censpace(nBins, d=0.09756581068603154)
        pl = 2. * np.sqrt((20 * 20 - u * u).clip(0))
    else:
        raise ValueError(f"beamhard_coefs2: unknown geometry {g.geom!r}")
    pl = np.squeeze(pl)[0:int(nBins / 2)]
    return _poly_fit(pl, energies, counts, attens, atten_eff)


def beamhard_coefs(energies, counts, det_prob=1.0, FocalLength=60, src_det=107.255, alpha=0,
                   mixatten=None, forward_project=None):
    """vir's beamhard_coefs (beamhard.py:81-113): the water tub (radius 20,
    512^2 pixels of 0.1) projected over 896 fan bins of 0.1 at one view, half
    of them fitted as in beamhard_coefs2 with the detector's energy weights
    (trapezoidal rule over the spectrum)."""
    mix = _need_mixatten(mixatten, "beamhard_coefs")
    energies = np.asarray(energies, np.float64)
    counts = np.asarray(counts, np.float64)
    energy_weights = det_prob if alpha == 0 else alpha * energies * det_prob
    nCols = 896
    I0 = np.trapezoid(counts * energy_weights, x=energies)
    attens = mix('H2O', energies)
    energy_eff = np.average(energies, weights=counts)
    atten_eff = mix('H2O', [energy_eff])[0]
    phantom = water_tub_phantom()
    if forward_project is None:
        from .sys_mat import dd
        pl = dd.dd_fp_fan_2d(phantom.astype(np.float32), np.zeros(1, np.float32), nCols,
                             float(FocalLength), float(src_det), du=.1, d_pix=.1)
    else:
        pl = forward_project(phantom, FocalLength, src_det, 1, nCols)
    pl = np.squeeze(np.asarray(pl, np.float64))[0:int(nCols / 2)]
    return _poly_fit(pl, energies, counts, attens, atten_eff, weights=energy_weights, I0=I0)


__all__ = ["beamhard_cor", "beamhard_cor_table", "beamhard_cor2", "beamhard_coefs",
           "beamhard_coefs2", "water_tub_phantom", "spectrum_table", "sphere_chords_fan"]
