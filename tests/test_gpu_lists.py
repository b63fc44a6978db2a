"""GPU Siddon lists (siddons) and list projection against the reference's
golden lists, the reference's C list projector and the oracle."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["siddons_edge", "siddons_par", "siddons_cone"])
def test_siddons_flat_bit_exact(vg, golden, case):
    from vir_gb300.sys_mat import siddon
    g = golden[case]
    ind, ln, off = siddon.siddons(g["src"], g["trg"], g["nPixels"], g["dPixels"], flat=True)
    assert np.array_equal(off, g["off"])
    assert np.array_equal(ind, g["ind"])
    assert np.array_equal(ln, g["len"])   # same float32 bits


@pytest.mark.parametrize("case", ["siddons_par", "siddons_edge"])
def test_siddons_object_forms(vg, golden, case):
    """Object forms: None exactly where the reference leaves a ray None (it
    misses the grid); a ray that enters the grid but keeps no positive length
    (the zero-length ray of the edge fixture) holds empty int32 / float32
    arrays, as the reference stores them."""
    from vir_gb300.sys_mat import siddon
    g = golden[case]
    rays = siddon.siddons(g["src"], g["trg"], g["nPixels"], g["dPixels"], ravel=True)
    assert rays.shape == g["src"].shape[:-1]
    flat = rays.reshape(-1)
    none = np.array([r is None for r in flat])
    assert np.array_equal(none, g["obj_none"])
    for r in range(flat.size):
        a, b = g["off"][r], g["off"][r + 1]
        if not none[r]:
            assert flat[r][0].dtype == np.int32 and flat[r][1].dtype == np.float32
            assert np.array_equal(flat[r][0], g["ind"][a:b])
            assert np.array_equal(flat[r][1], g["len"][a:b])
    if case == "siddons_edge":
        assert any(not none[r] and g["off"][r] == g["off"][r + 1] for r in range(flat.size))
    un = siddon.siddons(g["src"], g["trg"], g["nPixels"], g["dPixels"], ravel=False)
    r = next(i for i in range(flat.size) if flat[i] is not None and flat[i][0].size)
    x, y, z = np.unravel_index(flat[r][0], tuple(g["nPixels"]))
    assert np.array_equal(un.reshape(-1)[r][0], x) and np.array_equal(un.reshape(-1)[r][2], z)


def test_list_projection_vs_reference_c(vg, golden):
    """proj.sd_f_proj / sd_b_proj on the GPU against projection_c.c's output."""
    from vir_gb300.projection import proj
    d, c = golden["siddons_cone"], golden["list_c"]
    lst = (d["ind"], d["len"], d["off"])
    fp = proj.sd_f_proj(c["phantom"], lst, flat=True)
    assert np.abs(fp - c["sino"]).max() <= 2e-6 * np.abs(c["sino"]).max()
    bp = proj.sd_b_proj(c["y"], lst, c["phantom"].shape)
    assert np.abs(bp - c["bp"]).max() <= 2e-6 * np.abs(c["bp"]).max()


def c1_rays():
    """The C1 list geometry: 180 parallel views over pi, 367 rays each, a
    256 x 256 x 1 grid of unit voxels; (src, trg, nPixels, dPixels, origin)."""
    dets = np.arange(367) - 183.0
    views = np.linspace(0, np.pi, 180, endpoint=False)
    # proj_geom.geom_circular(..., geom="par") restated: rays along x rotated by each view
    src = np.zeros((180, 367, 3)); trg = np.zeros((180, 367, 3))
    for i, v in enumerate(views):
        c, s = np.cos(v), np.sin(v)
        R = np.array([[c, s], [-s, c]])
        src[i, :, :2] = np.stack([np.full(367, -36700.0), dets], -1) @ R
        trg[i, :, :2] = np.stack([np.full(367, 36700.0), dets], -1) @ R
    return src, trg, (256, 256, 1), 1.0, 0.0


def test_list_c1_scale_vs_oracle(vg, orc):
    """Config C1 geometry through siddons (GPU) and list FP/BP vs the oracle."""
    import torch
    from vir_gb300.projection import proj
    from vir_gb300.sys_mat import siddon
    src, trg, nP, dP, _ = c1_rays()
    ind, ln, off, shape, grid = siddon.siddons_device(src, trg, nP, dP)
    assert off.numel() == 180 * 367 + 1 and ind.numel() > 14_000_000
    x = np.random.default_rng(3).random((256, 256, 1)).astype(np.float32)
    fp = proj.list_fp_device(torch.from_numpy(x).cuda().reshape(-1), ind, ln, off).cpu().numpy()
    ih, lh, oh = ind.cpu().numpy(), ln.cpu().numpy(), off.cpu().numpy()
    fo = orc.list_fp(x, ih, lh, oh)
    assert np.abs(fp - fo).max() <= 2e-6 * np.abs(fo).max()
    y = np.random.default_rng(4).random(fp.size).astype(np.float32)
    bp = proj.list_bp_device(torch.from_numpy(y).cuda(), ind, ln, off, x.size).cpu().numpy()
    bo = orc.list_bp(y, ih, lh, oh, x.size)
    assert np.abs(bp - bo).max() <= 2e-6 * np.abs(bo).max()


class _RaveledRay(ctypes.Structure):   # mpct.RaveledRay layout (mpct.py:103-106)
    _fields_ = [("n", ctypes.c_int), ("R", ctypes.POINTER(ctypes.c_int)),
                ("L", ctypes.POINTER(ctypes.c_float))]


def test_ctypes_list_entry_points(vg, golden):
    """proj_ctype.sd_f_proj_c / sd_b_proj_c accumulate in place like the C."""
    from vir_gb300.projection import proj_ctype
    d, c = golden["siddons_cone"], golden["list_c"]
    nr = d["off"].size - 1
    rays = (_RaveledRay * nr)()
    keep = []
    for r in range(nr):
        a, b = d["off"][r], d["off"][r + 1]
        R = np.ascontiguousarray(d["ind"][a:b], np.int32)
        L = np.ascontiguousarray(d["len"][a:b], np.float32)
        keep += [R, L]
        rays[r].n = int(b - a)
        rays[r].R = R.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        rays[r].L = L.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    sino = np.ones(nr, np.float32)                 # accumulates onto existing contents
    proj_ctype.sd_f_proj_c(c["phantom"].copy(), sino, rays)
    assert np.abs(sino - 1.0 - c["sino"]).max() <= 2e-6 * np.abs(c["sino"]).max()
    ph = np.zeros(c["phantom"].shape, np.float32)
    proj_ctype.sd_b_proj_c(ph, c["y"].copy(), rays)
    assert np.abs(ph - c["bp"]).max() <= 2e-6 * np.abs(c["bp"]).max()


def test_numba_list_entry_points(vg, golden):
    """proj_numba / proj_cuda drop-ins (CSR in, in-place or new sinogram)."""
    from vir_gb300.projection import proj_numba
    d = golden["siddons_cone"]
    c = golden["list_c"]
    nr = d["off"].size - 1
    ref = c["sino"].astype(np.float64)
    for fn in (proj_numba.sd_f_proj_numba, proj_numba.sd_f_proj_numba_p,
               proj_numba.sd_f_proj_numba_g):
        s = fn(c["phantom"], (d["ind"], d["len"], d["off"]), (nr,))
        assert s.dtype == np.float32 and np.abs(s - ref).max() <= 2e-6 * np.abs(ref).max()
    out = np.zeros(nr, np.float32)
    proj_numba.fast_forward_project_p(c["phantom"].ravel(), d["ind"], d["len"], d["off"], out)
    assert np.abs(out - ref).max() <= 2e-6 * np.abs(ref).max()


def test_siddons_setup_device_matches_reference_steps(vg, golden, orc):
    """The device set-up of siddons (vg_siddons_setup) equals the oracle's
    step-by-step restatement of siddon.py:681-751 bit for bit: on the
    reference's golden rays, random rays with zero direction components,
    zero-length rays and integer end points (plane hits), and the C1 list
    geometry.  Plane indices of axes a ray does not move along, and of rays
    that miss the grid, are not read by the kernels; the latter can lie
    beyond the int32 range, whose conversion numpy leaves to the platform
    (INT_MIN on x86, saturation on Arm; the kernel gives INT_MIN)."""
    import warnings
    from vir_gb300.sys_mat import siddon
    rng = np.random.default_rng(17)
    cases = [(golden[c]["src"], golden[c]["trg"], golden[c]["nPixels"], golden[c]["dPixels"], 0.0)
             for c in ("siddons_edge", "siddons_par", "siddons_cone")]
    s, t = rng.uniform(-60, 60, (4000, 3)), rng.uniform(-60, 60, (4000, 3))
    s[::7, 1] = t[::7, 1]
    s[::11, 2] = t[::11, 2]
    s[::13] = t[::13]
    cases.append((s, t, (20, 18, 14), (1.1, 0.9, 1.3), (0.5, -0.3, 0.2)))
    s, t = rng.integers(-30, 30, (3000, 3)).astype(float), rng.integers(-30, 30, (3000, 3)).astype(float)
    cases.append((s, t, (16, 16, 16), 1.0, 0.0))
    # a broadcast source (one point against a detector of targets)
    t = np.stack(np.meshgrid(np.linspace(-40, 40, 61), np.linspace(-9, 9, 7), indexing="ij"), -1)
    t = np.concatenate([np.full(t.shape[:2] + (1,), -80.0), t], -1)
    cases.append((np.array([90.0, 0.3, -0.2]), t, (24, 24, 8), (2.0, 2.0, 1.5), 0.0))
    cases.append(c1_rays())
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for src, trg, nP, dP, oP in cases:
            shape, _, a = siddon.setup_device(src, trg, nP, dP, oP, 1e-5)
            a = {k: v.cpu().numpy() for k, v in a.items()}
            sb = np.broadcast_to(np.asarray(src, np.float32), np.shape(trg)).reshape(-1, 3)
            o = orc.siddons_setup(sb, np.asarray(trg).reshape(-1, 3), nP, dP, oP, 1e-5)
            assert a["amin"].shape == (int(np.prod(shape)),)
            moves = (o["dst"] != 0.0) & o["valid"].astype(bool)[:, None]
            assert np.array_equal(a["dst"].view(np.uint8), np.ascontiguousarray(o["dst"]).view(np.uint8))
            for k in ("amin", "amax", "dist", "valid"):
                assert np.array_equal(a[k].view(np.uint8), np.ascontiguousarray(o[k]).view(np.uint8)), k
            for k in ("i0", "iN"):
                assert np.array_equal(np.where(moves, a[k], 0), np.where(moves, o[k], 0)), k
