"""Siddon list formats and list algebra (siddon.py:12-633) against the
reference's own outputs on the cone fixture's lists.  The index bookkeeping
runs on the host (CPU tests); the accumulating functions run on the GPU."""
import ctypes

import numpy as np
import pytest


def sdlist_from_golden(golden):
    d = golden["siddons_cone"]
    nP = tuple(int(v) for v in d["nPixels"])
    shape = tuple(int(v) for v in golden["list_algebra"]["shape"])
    sdl = np.empty(shape, dtype=object)
    flat = sdl.reshape(-1)
    off = d["off"]
    for r in range(flat.size):
        a, b = off[r], off[r + 1]
        if a == b:
            continue
        x, y, z = np.unravel_index(d["ind"][a:b], nP)
        flat[r] = [x.astype(np.int32), y.astype(np.int32), z.astype(np.int32), d["len"][a:b]]
    return sdl, nP


def check_cat(lst, g, tag, tol=0.0):
    cnt = np.array([0 if r is None else len(r[0]) for r in lst.flat], np.int32)
    assert np.array_equal(cnt, g[f"{tag}_cnt"]), tag
    parts = [r for r in lst.flat if r is not None]
    for k, i in (("X", 0), ("Y", 1), ("Z", 2)):
        assert np.array_equal(np.concatenate([np.asarray(r[i]) for r in parts]), g[f"{tag}_{k}"]), tag
    L = np.concatenate([np.asarray(r[3], np.float64) for r in parts])
    ref = g[f"{tag}_L"].astype(np.float64)
    assert np.abs(L - ref).max() <= tol * np.abs(ref).max(), tag


def test_list_index_algebra_host(golden):
    import copy
    from vir_gb300.sys_mat import siddon as sd
    g = golden["list_algebra"]
    sdl, nP = sdlist_from_golden(golden)
    check_cat(sd.list_flip(copy.deepcopy(sdl), x=5, z=2), g, "flip")
    check_cat(sd.list_index_shift(copy.deepcopy(sdl), (1, -2, 3)), g, "shift")
    check_cat(sd.list_del_ind(copy.deepcopy(sdl), np.arange(2, 9), np.arange(0, 6),
                              np.arange(1, 5)), g, "del")
    # flatten / ravel / unravel round trip, counts
    d = golden["siddons_cone"]
    ind, ln, off = sd.list_flatten(sdl, nPixels=nP)
    assert np.array_equal(ind, d["ind"]) and np.array_equal(ln, d["len"]) and np.array_equal(off, d["off"])
    assert np.array_equal(np.diff(off), sd.list_count_elem(sdl).ravel())
    rav = sd.list_ravel(copy.deepcopy(sdl), nP)
    back = sd.list_unravel(rav, nP)
    for a, b in zip(sdl.flat, back.flat):
        assert (a is None) == (b is None)
        if a is not None:
            assert all(np.array_equal(p, q) for p, q in zip(a, b))
    # ray_boundary keeps the in-grid elements of a shifted ray
    r = sd.ray_index_shift(next(x for x in sdl.flat if x is not None), (10, 0, 0))
    kept = sd.ray_boundary(r, nP)
    assert np.all(kept[0] < nP[0]) and kept[0].size == int((r[0] < nP[0]).sum())


@pytest.mark.gpu
def test_list_accumulations_gpu(vg, golden):
    from vir_gb300.sys_mat import siddon as sd
    g = golden["list_algebra"]
    sdl, nP = sdlist_from_golden(golden)
    l2a = sd.list2array(sdl, nP)
    assert np.abs(l2a - g["l2a"]).max() <= 2e-6 * np.abs(g["l2a"]).max()
    ave = sd.rays_ave(sdl, nPixels=nP)
    for i, k in enumerate(("x", "y", "z")):
        assert np.array_equal(ave[i], g[f"ave_{k}"])
    assert np.abs(ave[3] - g["ave_l"]).max() <= 2e-6 * np.abs(g["ave_l"]).max()
    check_cat(sd.list_ave(sdl, nPixels=nP, axis=(2,)), g, "axave", 2e-6)
    check_cat(sd.list_weight_ave(sdl, g["weights"], nPixels=nP, axis=(2,)), g, "wave", 2e-6)
    check_cat(sd.list_convole(sdl, np.array([0.25, 0.5, 0.25]), nPixels=nP, axis=(2,)), g, "conv",
              2e-6)


@pytest.mark.gpu
def test_csr_ctypes_structures(vg, golden):
    """RaveledRay / UnraveledRay arrays straight from a GPU-made CSR list feed
    the ctypes-list projector like the reference's list_ctypes_object."""
    from vir_gb300 import mpct
    from vir_gb300.projection import proj_ctype
    from vir_gb300.sys_mat import siddon as sd
    d = golden["siddons_cone"]
    nP = tuple(int(v) for v in d["nPixels"])
    ind, ln, off = sd.siddons(d["src"], d["trg"], nP, tuple(d["dPixels"]), flat=True)
    phantom = np.random.default_rng(3).random(nP).astype(np.float32)
    nr = off.size - 1
    want = np.array([(phantom.reshape(-1)[ind[off[r]:off[r + 1]]] * ln[off[r]:off[r + 1]]).sum()
                     for r in range(nr)], np.float64)
    for ravel in (True, False):
        arr = mpct.csr_ctypes(ind, ln, off, ravel=ravel, nPixels=nP)
        sino = np.zeros(nr, np.float32)
        proj_ctype.sd_f_proj_c(phantom, sino, ctypes.byref(arr), ravel=ravel, dims=nP, nRays=nr)
        assert np.abs(sino - want).max() <= 2e-6 * np.abs(want).max()
    sdl, _ = sdlist_from_golden(golden)
    ref_c = mpct.list_ctypes_object(sdl, ravel=False, flat=True)
    sino = np.zeros(nr, np.float32)
    proj_ctype.sd_f_proj_c(phantom, sino, ref_c, ravel=False, dims=nP, nRays=nr)
    assert np.abs(sino - want).max() <= 2e-6 * np.abs(want).max()
