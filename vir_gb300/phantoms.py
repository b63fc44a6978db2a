"""Seeded random-ellipse / ellipsoid phantoms with analytic line integrals.

These are the synthetic inputs of the tests and the benchmark: sums of
ellipses (2D) or ellipsoids (3D) inside the inscribed field-of-view circle or
sphere, attenuation U(0, vmax) per object, centres and semi-axes uniform in
the field of view, rotation U(0, pi), all drawn from
``numpy.random.default_rng(seed)``.  Line integrals of the continuous objects
are exact (chord length of each quadric times its value), independent of any
projector, so they serve as a second truth beside the oracle.

Coordinates follow vir's distance-driven convention (dd.py:486-494,
527-585): pixel centres d_pix (i + 0.5 - n/2), view direction (cos, sin)
towards the source, detector axis (-sin, cos), bins at
du (j - nu/2 + 0.5 + su).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Ellipses:
    cx: np.ndarray
    cy: np.ndarray
    a: np.ndarray
    b: np.ndarray
    phi: np.ndarray
    val: np.ndarray


def random_ellipses(n_ell=10, fov_radius=1.0, seed=0, vmax=0.02) -> Ellipses:
    rng = np.random.default_rng(seed)
    cx, cy, a, b, phi, val = [], [], [], [], [], []
    while len(cx) < n_ell:
        r = rng.uniform(0, 0.7 * fov_radius)
        t = rng.uniform(0, 2 * np.pi)
        ea, eb = rng.uniform(0.05, 0.4, 2) * fov_radius
        # keep the whole ellipse inside the field of view
        if r + max(ea, eb) > 0.95 * fov_radius:
            continue
        cx.append(r * np.cos(t)); cy.append(r * np.sin(t))
        a.append(ea); b.append(eb)
        phi.append(rng.uniform(0, np.pi)); val.append(rng.uniform(0, vmax))
    return Ellipses(*(np.array(v) for v in (cx, cy, a, b, phi, val)))


def rasterize(e: Ellipses, nx, ny, d_pix=1.0, sub=4) -> np.ndarray:
    """Pixel averages (sub x sub supersampling) as an (nx, ny) float32 image."""
    off = (np.arange(sub) + 0.5) / sub - 0.5
    xs = d_pix * ((np.arange(nx)[:, None] + 0.5 - nx / 2) + off[None, :]).ravel()
    ys = d_pix * ((np.arange(ny)[:, None] + 0.5 - ny / 2) + off[None, :]).ravel()
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    img = np.zeros_like(X)
    for i in range(e.cx.size):
        c, s = np.cos(e.phi[i]), np.sin(e.phi[i])
        xr = (X - e.cx[i]) * c + (Y - e.cy[i]) * s
        yr = -(X - e.cx[i]) * s + (Y - e.cy[i]) * c
        img += e.val[i] * ((xr / e.a[i]) ** 2 + (yr / e.b[i]) ** 2 <= 1.0)
    return img.reshape(nx, sub, ny, sub).mean(axis=(1, 3)).astype(np.float32)


def ellipse_phantom(n=256, n_ell=10, seed=0, d_pix=1.0, vmax=0.02, sub=4):
    """(image, Ellipses) for an n x n grid of pixel width d_pix."""
    e = random_ellipses(n_ell, fov_radius=n * d_pix / 2, seed=seed, vmax=vmax)
    return rasterize(e, n, n, d_pix, sub), e


def _chords(e: Ellipses, px, py, dx, dy):
    """Sum over ellipses of val * chord length of the lines p + t d (|d| = 1)."""
    out = np.zeros(np.broadcast(px, py, dx, dy).shape)
    for i in range(e.cx.size):
        c, s = np.cos(e.phi[i]), np.sin(e.phi[i])
        x0 = (px - e.cx[i]) * c + (py - e.cy[i]) * s
        y0 = -(px - e.cx[i]) * s + (py - e.cy[i]) * c
        ux = dx * c + dy * s
        uy = -dx * s + dy * c
        A = (ux / e.a[i]) ** 2 + (uy / e.b[i]) ** 2
        B = 2 * (x0 * ux / e.a[i] ** 2 + y0 * uy / e.b[i] ** 2)
        C = (x0 / e.a[i]) ** 2 + (y0 / e.b[i]) ** 2 - 1
        disc = B * B - 4 * A * C
        out += e.val[i] * np.sqrt(np.clip(disc, 0, None)) / A
    return out


def sino_par(e: Ellipses, angs, nu, du=1.0, su=0.0):
    """Exact parallel-beam line integrals at bin centres, (na, nu)."""
    a = np.asarray(angs, np.float64)[:, None]
    u = du * (np.arange(nu)[None, :] - nu / 2 + 0.5 + su)
    c, s = np.cos(a), np.sin(a)
    px, py = -s * u, c * u
    return _chords(e, px, py, np.broadcast_to(c, px.shape), np.broadcast_to(s, px.shape))


def sino_fan(e: Ellipses, angs, nu, DSO, DSD, du=1.0, su=0.0):
    """Exact flat-detector fan-beam line integrals at bin centres, (na, nu):
    source at DSO (cos, sin), detector point at (DSO - DSD)(cos, sin) +
    u (-sin, cos)."""
    a = np.asarray(angs, np.float64)[:, None]
    u = du * (np.arange(nu)[None, :] - nu / 2 + 0.5 + su)
    c, s = np.cos(a), np.sin(a)
    sx, sy = DSO * c, DSO * s
    tx = (DSO - DSD) * c - s * u
    ty = (DSO - DSD) * s + c * u
    dx, dy = tx - sx, ty - sy
    n = np.hypot(dx, dy)
    return _chords(e, sx + 0 * u, sy + 0 * u, dx / n, dy / n)


def poisson_noise(p, I0=1e5, seed=0):
    """Transmission noise (tests/Test_SIRT/sirt_test.py:150-153 recipe):
    counts ~ Poisson(I0 exp(-p)), zero counts clamped to 1, y = -ln(counts/I0)."""
    rng = np.random.default_rng(seed)
    counts = rng.poisson(I0 * np.exp(-np.asarray(p, np.float64)))
    counts = np.maximum(counts, 1)
    return (-np.log(counts / I0)).astype(np.float32)


# --- 3D --------------------------------------------------------------------

@dataclass
class Ellipsoids:
    c: np.ndarray      # (n, 3) centres
    ax: np.ndarray     # (n, 3) semi-axes
    R: np.ndarray      # (n, 3, 3) rotations (rows: body axes in world coords)
    val: np.ndarray


def random_ellipsoids(n_obj=20, fov_radius=1.0, seed=0, vmax=0.02) -> Ellipsoids:
    rng = np.random.default_rng(seed)
    cs, axs, Rs, vals = [], [], [], []
    while len(cs) < n_obj:
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        r = rng.uniform(0, 0.6 * fov_radius)
        ax = rng.uniform(0.05, 0.35, 3) * fov_radius
        if r + ax.max() > 0.95 * fov_radius:
            continue
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        cs.append(r * d); axs.append(ax); Rs.append(q.T); vals.append(rng.uniform(0, vmax))
    return Ellipsoids(np.array(cs), np.array(axs), np.array(Rs), np.array(vals))


def rasterize3d(e: Ellipsoids, n, d_pix=1.0, sub=2) -> np.ndarray:
    off = (np.arange(sub) + 0.5) / sub - 0.5
    g = d_pix * ((np.arange(n)[:, None] + 0.5 - n / 2) + off[None, :]).ravel()
    vol = np.zeros((n, n, n), np.float32)
    X, Y = np.meshgrid(g, g, indexing="ij")
    for iz in range(n):
        zs = d_pix * (iz + 0.5 - n / 2 + off)
        acc = np.zeros((n * sub, n * sub), np.float64)
        for z in zs:
            P = np.stack([X, Y, np.full_like(X, z)], -1)
            for i in range(e.val.size):
                q = (P - e.c[i]) @ e.R[i].T / e.ax[i]
                acc += e.val[i] * ((q ** 2).sum(-1) <= 1.0)
        vol[:, :, iz] = (acc / sub).reshape(n, sub, n, sub).mean(axis=(1, 3))
    return vol


def ellipsoid_phantom(n=64, n_obj=20, seed=0, d_pix=1.0, vmax=0.02, sub=2):
    e = random_ellipsoids(n_obj, fov_radius=n * d_pix / 2, seed=seed, vmax=vmax)
    return rasterize3d(e, n, d_pix, sub), e


def rasterize3d_device(e: Ellipsoids, n, d_pix=1.0, device="cuda"):
    """Point-sampled (voxel centres) ellipsoid volume built on the GPU with
    torch, for volumes too large to rasterize on the host (512^3)."""
    import torch
    c = d_pix * (torch.arange(n, device=device, dtype=torch.float32) + 0.5 - n / 2)
    vol = torch.zeros((n, n, n), device=device, dtype=torch.float32)
    step = 16
    for z0 in range(0, n, step):
        X, Y, Z = torch.meshgrid(c, c, c[z0:z0 + step], indexing="ij")
        P = torch.stack([X, Y, Z], -1)
        for i in range(e.val.size):
            R = torch.tensor(e.R[i], device=device, dtype=torch.float32)
            ctr = torch.tensor(e.c[i], device=device, dtype=torch.float32)
            ax = torch.tensor(e.ax[i], device=device, dtype=torch.float32)
            q = ((P - ctr) @ R.T) / ax
            vol[:, :, z0:z0 + step] += float(e.val[i]) * ((q * q).sum(-1) <= 1.0)
    return vol
