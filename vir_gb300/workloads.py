"""Seeded synthetic workloads of the benchmark configurations.

* ``batched_problems(n_problems=64, seed=3)``: the batched-SIRT set --
  image sides drawn uniformly from {128, 256, 512, 1024} (1 mm pixels), view
  counts uniform in 90..1440, detectors of 1.5x the image width (1 mm bins),
  parallel or fan beam (fan: DSO = 1.5 N mm, DSD = 2 DSO), each a random
  ellipse phantom (10 ellipses, attenuation U(0, 0.02)/mm) with exact
  analytic line integrals as the measurement.
"""
from __future__ import annotations

import numpy as np

from . import phantoms as ph


def problem_shapes(n_problems=64, seed=3, sizes=(128, 256, 512, 1024), na_range=(90, 1440)):
    """(side, views, fan) of each problem of the set, without building any
    (the same random draws as batched_problems)."""
    rng = np.random.default_rng(seed)
    out = []
    for p in range(n_problems):
        n = int(rng.choice(sizes))
        na = int(rng.integers(na_range[0], na_range[1] + 1))
        fan = bool(rng.integers(0, 2))
        rng.integers(1 << 30)
        out.append((n, na, fan))
    return out


def batched_problems(n_problems=64, seed=3, sizes=(128, 256, 512, 1024), na_range=(90, 1440),
                     with_truth=False, only=None):
    """The problem set; ``only`` (problem indices) builds just those problems,
    each identical to its entry in the full set."""
    rng = np.random.default_rng(seed)
    out, truth = [], []
    for p in range(n_problems):
        n = int(rng.choice(sizes))
        na = int(rng.integers(na_range[0], na_range[1] + 1))
        fan = bool(rng.integers(0, 2))
        nu = int(round(1.5 * n))
        pseed = int(rng.integers(1 << 30))
        if only is not None and p not in only:
            continue
        img, e = ph.ellipse_phantom(n, 10, seed=pseed, d_pix=1.0, sub=2)
        if fan:
            DSO = 1.5 * n
            DSD = 2.0 * DSO
            angs = np.linspace(0, 2 * np.pi, na, endpoint=False)
            y = ph.sino_fan(e, angs, nu, DSO, DSD, du=1.0).astype(np.float32)
            out.append(dict(sino=y, ang_arr=angs, img_shape=(n, n), geom="fan", DSO=DSO, DSD=DSD,
                            du=1.0, d_pix=1.0))
        else:
            angs = np.linspace(0, np.pi, na, endpoint=False)
            y = ph.sino_par(e, angs, nu, du=1.0).astype(np.float32)
            out.append(dict(sino=y, ang_arr=angs, img_shape=(n, n), geom="par", du=1.0, d_pix=1.0))
        truth.append(img)
    return (out, truth) if with_truth else out
