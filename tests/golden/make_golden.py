"""Generates the golden fixtures in this directory by running the reference
(vargasp/vir) itself, imported from its source tree.

Run in a container that holds the vir tree, named by ``--ref`` or by the
VIR_REF environment variable:

    python tests/golden/make_golden.py --ref /path/to/vir

The reference is imported through three shims and nothing else: a ``vir``
symlink to the tree on ``sys.path`` (every module imports ``vir.*``), an
``llvmlite.binding`` stub (``sys_mat/dd.py:11-12`` imports it unconditionally)
and ``dd.prange = range`` (the numba-less fallback of ``dd.py:18-24`` defines
``njit`` but not ``prange``, which the square-geometry loops call).
numba is absent here, so the reference's ``@njit`` functions run as plain
Python through its own fallbacks.  Three modules cannot be imported as modules
(``sys_mat/sp.py`` runs a 128^3 projection at import, ``sirt_dd.py`` and
``sirt_numba.py`` import numba unguarded); for those the named functions' own
source is taken from the file and executed without the module body.

The C list projector is the reference's ``projection/projection_c.c``,
compiled from its source by ``oracle/Makefile`` into ``oracle/_ref``.

Each fixture stores its inputs and the reference's outputs (float32 as the
reference returns them).  Nothing here is used at run time on a GPU machine:
the tests read only the ``.npz`` files.
"""
from __future__ import annotations

import argparse
import ast
import ctypes
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def import_reference(ref_root):
    d = tempfile.mkdtemp(prefix="virref_")
    os.symlink(ref_root, os.path.join(d, "vir"))
    sys.path.insert(0, d)
    llvm = types.ModuleType("llvmlite")
    binding = types.ModuleType("llvmlite.binding")
    binding.set_option = lambda *a, **k: None
    llvm.binding = binding
    sys.modules.setdefault("llvmlite", llvm)
    sys.modules.setdefault("llvmlite.binding", binding)
    import vir  # noqa: F401
    return d


def function_from_source(path, names, extra_globals=None):
    """Executes only the named top-level functions of a reference file."""
    src = open(path).read()
    tree = ast.parse(src)
    keep = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in names]
    mod = ast.Module(body=keep, type_ignores=[])
    g = {"np": np}

    def njit(*a, **k):
        if a and callable(a[0]):
            return a[0]
        return lambda f: f

    g["njit"] = njit
    g["prange"] = range
    if extra_globals:
        g.update(extra_globals)
    exec(compile(mod, path, "exec"), g)
    return {n: g[n] for n in names}


def ellipse_image(n, n_ell, seed, vmax=0.02):
    """Seeded random-ellipse image (x-major, img[ix, iy]) used as fixture input."""
    rng = np.random.default_rng(seed)
    c = np.arange(n) - n / 2 + 0.5
    X, Y = np.meshgrid(c, c, indexing="ij")
    img = np.zeros((n, n), np.float64)
    for _ in range(n_ell):
        r = n / 2 * 0.9
        cx, cy = rng.uniform(-r / 2, r / 2, 2)
        a, b = rng.uniform(0.1 * r, 0.5 * r, 2)
        th = rng.uniform(0, np.pi)
        xr = (X - cx) * np.cos(th) + (Y - cy) * np.sin(th)
        yr = -(X - cx) * np.sin(th) + (Y - cy) * np.cos(th)
        img[(xr / a) ** 2 + (yr / b) ** 2 <= 1] += rng.uniform(0, vmax)
    return img.astype(np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("VIR_REF"),
                    help="the vir source tree (default: $VIR_REF)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give the vir source tree with --ref or VIR_REF")
    ref = args.ref
    import_reference(ref)
    import vir.sys_mat.dd as dd
    dd.prange = range  # dd.py:18-24 binds no prange when numba is absent
    import vir.sys_mat.fp_2d_par as fp2
    import vir.sys_mat.siddon as sd
    import vir.filtration as filt
    import vir.proj_geom as pg
    out = {}

    # --- Siddon 2D parallel (fp_2d_par.siddons_fp_2d) ---------------------
    img = ellipse_image(32, 6, 11, vmax=1.0)
    angs = np.linspace(0, np.pi, 24, endpoint=False)  # includes 0, 45, 90 deg
    out["siddon2d_a"] = dict(img=img, angs=angs, n_dets=np.int32(47), d_det=1.0, d_pix=1.0,
                             sino=fp2.siddons_fp_2d(img, angs, 47, 1.0, 1.0))
    img2 = ellipse_image(24, 4, 12, vmax=1.0)[:, :20].copy()
    angs2 = np.linspace(0, 2 * np.pi, 17, endpoint=False)
    out["siddon2d_b"] = dict(img=img2, angs=angs2, n_dets=np.int32(40), d_det=0.7, d_pix=1.3,
                             sino=fp2.siddons_fp_2d(img2, angs2, 40, 0.7, 1.3))

    # --- separable footprint, parallel rectangle (fp_2d_par) ---------------
    out["sf_par_rect"] = dict(img=img, angs=angs[:12], n_dets=np.int32(47), d_det=1.0,
                              d_pix=1.0,
                              sino=fp2.separable_footprint_fp_2d(img, angs[:12], 47, 1.0, 1.0))

    # --- distance-driven 2D ---------------------------------------------------
    img3 = ellipse_image(32, 6, 13, vmax=1.0)
    a_par = np.linspace(0, np.pi, 24, endpoint=False).astype(np.float32)
    for tag, (nu, du, su, dp) in {"a": (48, 1.0, 0.0, 1.0), "b": (40, 0.8, 0.25, 0.9)}.items():
        sino = dd.dd_fp_par_2d(img3, a_par, nu, du=du, su=su, d_pix=dp)
        y = np.random.default_rng(20).random((a_par.size, nu)).astype(np.float32)
        bp = dd.dd_bp_par_2d(y, a_par, img3.shape, du=du, su=su, d_pix=dp)
        out[f"dd_par_{tag}"] = dict(img=img3, angs=a_par, nu=np.int32(nu), du=du, su=su,
                                    d_pix=dp, sino=sino, y=y, bp=bp)
    a_fan = np.linspace(0, 2 * np.pi, 24, endpoint=False).astype(np.float32)
    for tag, (nu, du, su, dp, DSO, DSD) in {"a": (64, 1.2, 0.0, 0.9, 60.0, 120.0),
                                             "b": (50, 1.0, 0.5, 1.0, 50.0, 90.0)}.items():
        sino = dd.dd_fp_fan_2d(img3, a_fan, nu, DSO, DSD, du=du, su=su, d_pix=dp)
        y = np.random.default_rng(21).random((a_fan.size, nu)).astype(np.float32)
        bp = dd.dd_bp_fan_2d(y, a_fan, img3.shape, DSO, DSD, du=du, su=su, d_pix=dp)
        out[f"dd_fan_{tag}"] = dict(img=img3, angs=a_fan, nu=np.int32(nu), du=du, su=su,
                                    d_pix=dp, DSO=DSO, DSD=DSD, sino=sino, y=y, bp=bp)

    # --- distance-driven cone --------------------------------------------------
    rng = np.random.default_rng(14)
    vol = rng.random((10, 10, 10)).astype(np.float32)  # dd.py:289,388 unpack (nP, nz, no): cubes only
    a_cone = np.linspace(0, 2 * np.pi, 8, endpoint=False).astype(np.float32)
    cone = dict(nu=24, nv=20, DSO=40.0, DSD=80.0, du=1.5, dv=1.4, su=0.25, sv=-0.5, d_pix=1.0)
    kw = {k: cone[k] for k in ("du", "dv", "su", "sv", "d_pix")}
    sino_bug = dd.dd_fp_cone_3d(vol, a_cone, cone["nu"], cone["nv"], cone["DSO"], cone["DSD"], **kw)
    # the same sweep with tmp_u cleared for every (io, iz)
    fixed_src = open(os.path.join(ref, "sys_mat", "dd.py")).read()
    s0 = fixed_src.index("def _dd_fp_cone_sweep")
    s1 = fixed_src.index("@njit", s0)
    body = fixed_src[s0:s1].replace("tmp_u[iu_min:iu_max] = 0.0", "tmp_u[:] = 0.0")
    assert "tmp_u[:] = 0.0" in body
    ns = {"np": np}
    exec(body, ns)
    orig = dd._dd_fp_cone_sweep
    dd._dd_fp_cone_sweep = ns["_dd_fp_cone_sweep"]
    try:
        sino_fix = dd.dd_fp_cone_3d(vol, a_cone, cone["nu"], cone["nv"], cone["DSO"], cone["DSD"], **kw)
    finally:
        dd._dd_fp_cone_sweep = orig
    yc = np.random.default_rng(22).random(sino_fix.shape).astype(np.float32)
    bpc = dd.dd_bp_cone_3d(yc, a_cone, vol.shape, cone["DSO"], cone["DSD"], **kw)
    out["dd_cone"] = dict(vol=vol, angs=a_cone, sino_ref=sino_bug, sino_fixed=sino_fix, y=yc,
                          bp=bpc, **{k: (np.int32(v) if isinstance(v, int) else v)
                                     for k, v in cone.items()})

    # --- separable footprint fan (sp.sf_fp_fan_2d; sp.py not importable) ----
    fns = function_from_source(os.path.join(ref, "sys_mat", "sp.py"), ["sf_fp_fan_2d"])
    img4 = ellipse_image(24, 5, 15, vmax=1.0)
    a_sf = np.linspace(0, 2 * np.pi, 10, endpoint=False)
    out["sf_fan"] = dict(img=img4, angs=a_sf, nu=np.int32(40), DSO=50.0, DSD=100.0, du=1.3,
                         d_pix=1.0,
                         sino=fns["sf_fp_fan_2d"](img4, a_sf, 40, 50.0, 100.0, du=1.3, d_pix=1.0))

    # --- ramp filter (filtration.filter_sino) -----------------------------------
    rs = np.random.default_rng(16).random((5, 37))
    for ft in ("ramp", "hann", "hamming", "blackman", "shepp-logan", "cosine", "gaussian"):
        for rsp in (True, False):
            for cut in (0.5, 0.4):
                key = f"filter_{ft}_{int(rsp)}_{int(cut * 10)}"
                out[key] = dict(sino=rs, du=1.3, cutoff=cut, real_space=rsp,
                                filter_type=np.array(ft),
                                filtered=filt.filter_sino(rs, du=1.3, filter_type=ft, cutoff=cut,
                                                          real_space=rsp))

    # --- Siddon 3D lists (siddon.siddons) -----------------------------------------
    # edge cases of tests/Test_Siddons/siddons_test1.py:20-80 on a 4x4x1 grid
    edge = [([-2.1, .25, .25], [2.0, .25, .25]), ([-2.0, .25, .25], [2.0, .25, .25]),
            ([-1.9, .25, .25], [2.0, .25, .25]), ([-2.0, .25, .25], [1.9, .25, .25]),
            ([-2.0, .25, .25], [2.1, .25, .25]), ([2.1, .25, .25], [-2.0, .25, .25]),
            ([2.0, .25, .25], [-2.0, .25, .25]), ([1.9, .25, .25], [-2.0, .25, .25]),
            ([2.0, .25, .25], [-1.9, .25, .25]), ([2.0, .25, .25], [-2.1, .25, .25]),
            ([.25, 4.0, .25], [.25, 4.0, .25]), ([-4.0, .25, .25], [-4.0, .25, .25]),
            ([2.0, -2.0, 0.0], [-2.0, -2.0, 0.0]), ([2.0, -1.0, 0.0], [-2.0, -1.0, 0.0]),
            ([2.0, 0.0, 0.0], [-2.0, 0.0, 0.0]),
            # a zero-length ray inside the grid: it enters the alpha range but
            # keeps no positive length, so the object forms hold empty arrays
            ([.25, .25, .25], [.25, .25, .25])]
    srcs = np.array([e[0] for e in edge], np.float32)
    trgs = np.array([e[1] for e in edge], np.float32)
    ind, ln, off = sd.siddons(srcs, trgs, (4, 4, 1), 1.0, flat=True)
    # which rays the object form leaves None (rays that miss the grid)
    obj = sd.siddons(srcs, trgs, (4, 4, 1), 1.0, ravel=True).reshape(-1)
    out["siddons_edge"] = dict(src=srcs, trg=trgs, nPixels=np.array([4, 4, 1], np.int32),
                               dPixels=np.array([1.0, 1.0, 1.0]), ind=ind, len=ln, off=off,
                               obj_none=np.array([r is None for r in obj]))
    # a circular parallel geometry (proj_geom.geom_circular) on a 16x16x1 grid
    dets = (np.arange(23) - 11).astype(np.float64) * 0.9
    views = np.linspace(0, np.pi, 12, endpoint=False)
    src, trg = pg.geom_circular(dets, views, geom="par")
    ind, ln, off = sd.siddons(src, trg, (16, 16, 1), 1.0, flat=True)
    obj = sd.siddons(src, trg, (16, 16, 1), 1.0, ravel=True).reshape(-1)
    out["siddons_par"] = dict(src=src.astype(np.float32), trg=trg.astype(np.float32),
                              nPixels=np.array([16, 16, 1], np.int32),
                              dPixels=np.array([1.0, 1.0, 1.0]), ind=ind, len=ln, off=off,
                              obj_none=np.array([r is None for r in obj]))
    # a fan geometry in 3D (cone with one z row offset) on a 12x10x6 grid
    dets = (np.arange(15) - 7).astype(np.float64) * 1.1
    dz = (np.arange(5) - 2).astype(np.float64) * 1.2
    views = np.linspace(0, 2 * np.pi, 7, endpoint=False)
    src, trg = pg.geom_circular(dets, views, geom="cone", src_iso=30.0, det_iso=20.0, DetsZ=dz)
    ind, ln, off = sd.siddons(src, trg, (12, 10, 6), (1.0, 0.8, 1.2), flat=True)
    out["siddons_cone"] = dict(src=src.astype(np.float32), trg=trg.astype(np.float32),
                               nPixels=np.array([12, 10, 6], np.int32),
                               dPixels=np.array([1.0, 0.8, 1.2]), ind=ind, len=ln, off=off)

    # --- the reference C list projector (projection_c.c via its own ctypes) ----
    ref_so = os.path.join(REPO, "oracle", "_ref", "projection.so")
    if os.path.exists(ref_so):
        import vir.mpct as mpct
        so = ctypes.CDLL(ref_so)
        d = out["siddons_cone"]
        nvox = int(np.prod(d["nPixels"]))
        phantom = np.random.default_rng(17).random(tuple(d["nPixels"])).astype(np.float32)
        nr = d["off"].size - 1
        rays = (mpct.RaveledRay * nr)()
        keep = []
        for r in range(nr):
            a, b = d["off"][r], d["off"][r + 1]
            R = np.ascontiguousarray(d["ind"][a:b], np.int32)
            L = np.ascontiguousarray(d["len"][a:b], np.float32)
            keep += [R, L]
            rays[r].n = int(b - a)
            rays[r].R = R.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
            rays[r].L = L.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        sino = np.zeros(nr, np.float32)
        so.forward_proj_ravel_rays_struct(phantom.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                          sino.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                          rays, ctypes.c_int(nr))
        y = np.random.default_rng(18).random(nr).astype(np.float32)
        bp = np.zeros(nvox, np.float32)
        so.back_proj_ravel_rays_struct(bp.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                       y.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                       rays, ctypes.c_int(nr))
        out["list_c"] = dict(phantom=phantom, sino=sino, y=y, bp=bp.reshape(phantom.shape))

    # --- SIRT update rule (sirt_dd.py:23-76) around the reference DD projectors --
    fns = function_from_source(os.path.join(ref, "sys_mat", "sirt_dd.py"),
                               ["fast_divide1", "fast_divide2"])
    img5 = ellipse_image(24, 4, 19, vmax=0.02)
    a5 = np.linspace(0, np.pi, 30, endpoint=False).astype(np.float32)
    y5 = dd.dd_fp_par_2d(img5, a5, 36, du=1.0, d_pix=1.0)
    W_sino = dd.dd_fp_par_2d(np.ones_like(img5), a5, 36, du=1.0, d_pix=1.0)
    W_img = dd.dd_bp_par_2d(np.ones_like(y5), a5, img5.shape, du=1.0, d_pix=1.0)
    x = np.zeros(img5.shape, np.float32) + .00001
    iters = 6
    for _ in range(1, iters):
        est = dd.dd_fp_par_2d(x, a5, 36, du=1.0, d_pix=1.0)
        fns["fast_divide1"](y5, est, W_sino)
        upd = dd.dd_bp_par_2d(est, a5, img5.shape, du=1.0, d_pix=1.0)
        fns["fast_divide2"](upd, W_img)
        x = x + 1.0 * upd
    out["sirt_par"] = dict(img=img5, angs=a5, nu=np.int32(36), sino=y5, W_sino=W_sino,
                           W_img=W_img, iters=np.int32(iters), gamma=1.0, x=x)

    # --- translational square geometry (dd.py:895-1313) and its SIRT ------------
    # (sirt_dd.py:37-76 executed from source around the reference projectors)
    rng = np.random.default_rng(23)
    sq_cases = {
        # detector truncated on both axes, shifted sources and cells
        "a": dict(shape=(8, 8, 6), nu=14, nv=10, nsrc_p=3, nsrc_z=2, DSO=20.0, DSD=36.0,
                  du=1.0, dv=0.9, dsrc_p=0.5, dsrc_z=0.5, su=0.3, sv=4.0, ssrc_p=0.2,
                  ssrc_z=-3.0, d_pix=1.0),
        # source plane inside the object: slab 7 (o_bnd = 3 > DSO) is skipped
        "b": dict(shape=(8, 8, 5), nu=20, nv=12, nsrc_p=2, nsrc_z=3, DSO=2.5, DSD=9.0,
                  du=1.3, dv=1.1, dsrc_p=0.7, dsrc_z=0.4, su=0.0, sv=1.5, ssrc_p=-0.4,
                  ssrc_z=-1.0, d_pix=0.8),
    }
    for tag, c in sq_cases.items():
        vol = rng.random(c["shape"]).astype(np.float32)
        geo = {k: c[k] for k in ("du", "dv", "dsrc_p", "dsrc_z", "su", "sv", "ssrc_p", "ssrc_z",
                                 "d_pix")}
        sino = dd.dd_fp_square(vol, c["nu"], c["nv"], c["nsrc_p"], c["nsrc_z"], c["DSO"],
                               c["DSD"], **geo)
        y = rng.random(sino.shape).astype(np.float32)
        bp = dd.dd_bp_square(y, vol.shape, c["DSO"], c["DSD"], **geo)
        out[f"square_{tag}"] = dict(vol=vol, sino=sino, y=y, bp=bp, **{
            k: (np.int32(v) if isinstance(v, int) else np.asarray(v))
            for k, v in c.items() if k != "shape"})
    fns = function_from_source(os.path.join(ref, "sys_mat", "sirt_dd.py"),
                               ["fast_divide1", "fast_divide2", "sirt"], {"dd": dd})
    c = sq_cases["a"]
    n, nz = c["shape"][0], c["shape"][2]
    vol = np.zeros(c["shape"], np.float32)
    vol[2:6, 3:7, 1:5] = 1.0
    geo = {k: c[k] for k in ("du", "dv", "dsrc_p", "dsrc_z", "su", "sv", "ssrc_p", "ssrc_z",
                             "d_pix")}
    args = (c["nu"], c["nv"], c["nsrc_p"], c["nsrc_z"], c["DSO"], c["DSD"])
    sino = dd.dd_fp_square(vol, *args, **geo)
    W_sino = dd.dd_fp_square(np.ones(c["shape"], np.float32), *args, **geo)
    W_img = dd.dd_bp_square(np.ones(sino.shape, np.float32), c["shape"], c["DSO"], c["DSD"], **geo)
    prms = ((c["DSO"], c["DSD"]), (n, n, nz, c["d_pix"]),
            (c["nsrc_p"], c["nsrc_z"], c["dsrc_p"], c["dsrc_z"], c["ssrc_p"], c["ssrc_z"]),
            (c["nu"], c["nv"], c["du"], c["dv"], c["su"], c["sv"]), (1.0, 5))
    x = fns["sirt"](sino, W_sino, W_img, *prms)
    out["sirt_square"] = dict(vol=vol, sino=sino, W_sino=W_sino, W_img=W_img, x=x,
                              gem_prms=np.array(prms[0]), img_prms=np.array(prms[1]),
                              src_prms=np.array(prms[2]), det_prms=np.array(prms[3]),
                              srt_prms=np.array(prms[4]))

    # --- analytic cone-beam sphere, detector-area averaged (analytic_sino.py:563) --
    # the pin of the separable-footprint cone projector (vir has no working one)
    import vir.sys_mat.analytic_sino as an
    sph = np.array([2.0, -3.0, 1.5, 7.0])
    a_sf = np.linspace(0, 2 * np.pi, 8, endpoint=False)
    nu_s, nv_s, du_s, dv_s, DSO_s, DSD_s = 64, 48, 0.8, 0.8, 60.0, 110.0
    u_s = du_s * (np.arange(nu_s) + 0.5 - nu_s / 2)
    v_s = dv_s * (np.arange(nv_s) + 0.5 - nv_s / 2)
    out["sphere_cone_vol"] = dict(sphere=sph, angs=a_sf, nu=np.int32(nu_s), nv=np.int32(nv_s),
                                  du=du_s, dv=dv_s, DSO=DSO_s, DSD=DSD_s,
                                  proj=an.analytic_sino_sphere_cone_vol(sph, a_sf, u_s, v_s, DSO_s,
                                                                        DSD_s))

    # --- fan FBP parts (processing/reconstruction.py:99-107, proj2.py:580-616) --
    # vir's fan_fbp cannot run; its pre-weight and its Hsieh backprojector can,
    # executed from their own source (the modules' imports are stale)
    rec = function_from_source(os.path.join(ref, "processing", "reconstruction.py"),
                               ["cosine_weighting"])
    p2 = function_from_source(os.path.join(ref, "processing", "proj2.py"),
                              ["fan_backproject_hsieh", "calc_image_arrays"],
                              extra_globals={"sys": types.SimpleNamespace(
                                  stdout=types.SimpleNamespace(write=lambda *a: None,
                                                               flush=lambda: None))})
    p2["fan_backproject_hsieh"].__globals__["calc_image_arrays"] = p2["calc_image_arrays"]
    rng = np.random.default_rng(41)
    sino_w = rng.random((3, 31))
    cols_pos = (np.arange(31) - 15.0) * 1.3
    cols_ang = (np.arange(31) - 15.0) * 0.01
    out["fbp_weights"] = dict(
        sino=sino_w, cols_pos=cols_pos, cols_ang=cols_ang, src_iso=500.0, det_off=1.5,
        equispaced=rec["cosine_weighting"](sino_w, cols_pos, 500.0, detOff=1.5, equispaced=True),
        equiangular=rec["cosine_weighting"](sino_w, cols_ang, 500.0, detOff=1.5, equispaced=False))
    sino_h = rng.random((5, 2, 41))
    views_h = np.linspace(0, 2 * np.pi, 5, endpoint=False) + 0.1
    cols_h = (np.arange(41) - 20.0) * 0.012
    img_h = p2["fan_backproject_hsieh"](sino_h, views_h, cols_h, 60.0, dPixels=(1.1, 1.1),
                                        nPixels=(16, 16), detOff=0.3, pixOff=(0.2, -0.1))
    out["fbp_hsieh"] = dict(sino=sino_h, views=views_h, cols=cols_h, src_iso=60.0,
                            dPixels=np.array([1.1, 1.1]), nPixels=np.array([16, 16], np.int32),
                            detOff=0.3, pixOff=np.array([0.2, -0.1]), img=img_h)

    # --- Siddon list algebra (siddon.py:12-633) on the cone fixture's lists ---
    import copy
    d = out["siddons_cone"]
    nP = (12, 10, 6)
    sdl = sd.siddons(d["src"], d["trg"], nP, (1.0, 0.8, 1.2))

    def cat(lst):
        """object array of unraveled rays -> counts and concatenated X, Y, Z, L"""
        cnt = np.array([0 if r is None else len(r[0]) for r in lst.flat], np.int32)
        parts = [r for r in lst.flat if r is not None]
        if not parts:
            return dict(cnt=cnt)
        return dict(cnt=cnt, X=np.concatenate([r[0] for r in parts]).astype(np.int64),
                    Y=np.concatenate([r[1] for r in parts]).astype(np.int64),
                    Z=np.concatenate([r[2] for r in parts]).astype(np.int64),
                    L=np.concatenate([r[3] for r in parts]).astype(np.float32))

    la = dict(l2a=sd.list2array(sdl, nP), shape=np.array(sdl.shape, np.int32))
    ave = sd.rays_ave(sdl, nPixels=nP)
    la.update(ave_x=ave[0], ave_y=ave[1], ave_z=ave[2], ave_l=ave[3])
    for tag, val in (("axave", sd.list_ave(sdl, nPixels=nP, axis=(2,))),
                     ("wave", sd.list_weight_ave(sdl, np.linspace(0.2, 1.0, sdl.shape[2]),
                                                 nPixels=nP, axis=(2,))),
                     ("conv", sd.list_convole(sdl, np.array([0.25, 0.5, 0.25]), nPixels=nP,
                                              axis=(2,))),
                     ("flip", sd.list_flip(copy.deepcopy(sdl), x=5, z=2)),
                     ("shift", sd.list_index_shift(copy.deepcopy(sdl), (1, -2, 3))),
                     ("del", sd.list_del_ind(copy.deepcopy(sdl), np.arange(2, 9), np.arange(0, 6),
                                             np.arange(1, 5)))):
        for k, v in cat(val).items():
            la[f"{tag}_{k}"] = v
    la["weights"] = np.linspace(0.2, 1.0, sdl.shape[2])
    out["list_algebra"] = la

    # --- ray-driven (rd.py) and pixel-driven (pd.py) projectors --------------
    import vir.sys_mat.rd as rdm
    import vir.sys_mat.pd as pdm
    rng = np.random.default_rng(24)
    img6 = (rng.random((16, 12)) + 0.1).astype(np.float32)   # no zeros (pd.py:335-339)
    a_par6 = np.linspace(0, np.pi, 10, endpoint=False)        # includes 0 and 90 degrees
    a_fan6 = np.linspace(0, 2 * np.pi, 10, endpoint=False)
    vol6 = (rng.random((8, 8, 6)) + 0.1).astype(np.float32)
    a_cone6 = np.linspace(0, 2 * np.pi, 6, endpoint=False)
    for j, tag in ((False, "aw"), (True, "joseph")):
        # nu = 10: every ray inside the image; nu = 14: rays beside it at 0 degrees
        for nu in (10, 14):
            sino = rdm.aw_fp_par_2d(img6, a_par6, nu, du=1.0, su=0.2, d_pix=1.0, joseph=j)
            y = rng.random(sino.shape).astype(np.float32)
            bp = rdm.aw_bp_par_2d(y, a_par6, img6.shape, du=1.0, su=0.2, d_pix=1.0, joseph=j)
            out[f"rd_par_{tag}_{nu}"] = dict(img=img6, angs=a_par6, nu=np.int32(nu), du=1.0,
                                             su=0.2, d_pix=1.0, sino=sino, y=y, bp=bp)
        sino = rdm.aw_fp_fan_2d(img6, a_fan6, 24, 40.0, 80.0, du=1.3, su=0.1, d_pix=1.0, joseph=j)
        y = rng.random(sino.shape).astype(np.float32)
        bp = rdm.aw_bp_fan_2d(y, a_fan6, img6.shape, 40.0, 80.0, du=1.3, su=0.1, d_pix=1.0,
                              joseph=j)
        out[f"rd_fan_{tag}"] = dict(img=img6, angs=a_fan6, nu=np.int32(24), DSO=40.0, DSD=80.0,
                                    du=1.3, su=0.1, d_pix=1.0, sino=sino, y=y, bp=bp)
        # nu == nv: rd.py:688 builds the rows from nu
        sino = rdm.aw_fp_cone_3d(vol6, a_cone6, 10, 10, 30.0, 60.0, du=1.5, dv=1.5, su=0.1,
                                 sv=0.2, d_pix=1.0, joseph=j)
        y = rng.random(sino.shape).astype(np.float32)
        bp = rdm.aw_bp_cone_3d(y, a_cone6, vol6.shape, 30.0, 60.0, du=1.5, dv=1.5, su=0.1,
                               sv=0.2, d_pix=1.0, joseph=j)
        out[f"rd_cone_{tag}"] = dict(vol=vol6, angs=a_cone6, nu=np.int32(10), nv=np.int32(10),
                                     DSO=30.0, DSD=60.0, du=1.5, dv=1.5, su=0.1, sv=0.2,
                                     d_pix=1.0, sino=sino, y=y, bp=bp)
    sino = pdm.pd_fp_par_2d(img6, a_par6, 20, du=1.1, su=0.2, d_pix=1.0)
    y = rng.random(sino.shape).astype(np.float32)
    out["pd_par"] = dict(img=img6, angs=a_par6, nu=np.int32(20), du=1.1, su=0.2, d_pix=1.0,
                         sino=sino, y=y,
                         bp=pdm.pd_bp_par_2d(y, a_par6, img6.shape, du=1.1, su=0.2, d_pix=1.0))
    sino = pdm.pd_fp_fan_2d(img6, a_fan6, 30, 40.0, 80.0, du=1.2, su=0.1, d_pix=1.0)
    y = rng.random(sino.shape).astype(np.float32)
    out["pd_fan"] = dict(img=img6, angs=a_fan6, nu=np.int32(30), DSO=40.0, DSD=80.0, du=1.2,
                         su=0.1, d_pix=1.0, sino=sino, y=y,
                         bp=pdm.pd_bp_fan_2d(y, a_fan6, img6.shape, 40.0, 80.0, du=1.2, su=0.1,
                                             d_pix=1.0))
    sino = pdm.pd_fp_cone_3d(vol6, a_cone6, 14, 12, 30.0, 60.0, du=1.3, dv=1.4, su=0.1, sv=0.2,
                             d_pix=1.0)
    y = rng.random(sino.shape).astype(np.float32)
    out["pd_cone"] = dict(vol=vol6, angs=a_cone6, nu=np.int32(14), nv=np.int32(12), DSO=30.0,
                          DSD=60.0, du=1.3, dv=1.4, su=0.1, sv=0.2, d_pix=1.0, sino=sino, y=y,
                          bp=pdm.pd_bp_cone_3d(y, a_cone6, vol6.shape, 30.0, 60.0, du=1.3, dv=1.4,
                                               su=0.1, sv=0.2, d_pix=1.0))

    # --- TV helpers (tv.py:98-224, executed from source: tv.py imports skimage
    # and a module absent from the tree at import) --------------------------
    fns = function_from_source(os.path.join(ref, "tv.py"),
                               ["pyT", "grad", "div", "grad_abs", "div_abs"])
    rng = np.random.default_rng(25)
    x = rng.normal(size=(9, 7))
    zz = rng.normal(size=(2, 9, 7))
    AA = rng.normal(size=(2, 9, 7))
    AA[:, 0, 0] = [0.3, 0.0]     # a single non-zero component, inside the ball
    AA[:, 0, 1] = [0.0, -2.5]    # a single non-zero component, outside the ball
    out["tv_ops"] = dict(x=x, z=zz, AA=AA, grad=fns["grad"](x), div=fns["div"](zz),
                         grad_abs=fns["grad_abs"](x), div_abs=fns["div_abs"](zz),
                         pyT=fns["pyT"](AA.copy()))

    # --- beam-hardening pre-correction (processing/beamhard.py) -------------
    # beamhard.py imports three modules outside the tree at import: the
    # X-ray attenuation database xcompy (stubbed with a synthetic water curve,
    # mu(E) = 0.17 + 2500 E^-3 per cm, stated here as synthetic), vir's
    # intersection_sino under the name `intersection` (its plotting imports
    # are stubbed when matplotlib is absent), and a projector module
    # `projection` that the fixtures below do not call.
    if "matplotlib" not in sys.modules:  # intersection_sino.py:13-14, plotting only
        mpl = types.ModuleType("matplotlib")
        mpl.pyplot = types.ModuleType("matplotlib.pyplot")
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.pyplot"] = mpl.pyplot
        tk = types.ModuleType("mpl_toolkits")
        tk.mplot3d = types.ModuleType("mpl_toolkits.mplot3d")
        tk.mplot3d.Axes3D = object
        sys.modules["mpl_toolkits"] = tk
        sys.modules["mpl_toolkits.mplot3d"] = tk.mplot3d
    import vir.intersection_sino as inter_mod
    from vir.core import core_funcs as cf

    def mixatten(material, energies):
        e = np.asarray(energies, np.float64)
        return 0.17 + 2500.0 * e ** -3.0

    sys.modules["intersection"] = inter_mod
    sys.modules["projection"] = types.ModuleType("projection")
    xc = types.ModuleType("xcompy")
    xc.mixatten = mixatten
    sys.modules["xcompy"] = xc
    sys.path.insert(0, os.path.join(ref, "processing"))
    import beamhard as bhm
    energies = np.arange(20.0, 121.0)
    counts = np.exp(-0.5 * ((energies - 62.0) / 18.0) ** 2) * 1e6
    atten_eff = float(mixatten("H2O", [np.average(energies, weights=counts)])[0])
    rng = np.random.default_rng(26)
    li = (rng.random((6, 50)) * 8.0).astype(np.float32)
    li[0, :5] = [0.0, 1e-7, 3.5, 7.999, 0.25]
    coefs = np.polyfit(np.linspace(0, 10, 50), np.linspace(0, 10, 50) ** 1.1, 2)
    mu = 0.2
    out["bh_poly"] = dict(line_ints=li, coefs=coefs, mu=mu,
                          cor_f64coefs=bhm.beamhard_cor(li, coefs, mu),
                          cor_pycoefs=bhm.beamhard_cor(li, [float(c) for c in coefs], mu),
                          cor_f64mu=bhm.beamhard_cor(li, coefs, np.float64(mu)),
                          cor_f64in=bhm.beamhard_cor(li.astype(np.float64), coefs, mu))
    li_t = (rng.random((5, 40)) * 6.5 - 0.5).astype(np.float32)  # some negatives: clipped
    out["bh_table"] = dict(line_ints=li_t, energies=energies, counts=counts, atten_eff=atten_eff,
                           attens=mixatten("H2O", energies),
                           cor=bhm.beamhard_cor_table(li_t, energies, counts, None, atten_eff))
    g_fan = cf.Geom(nViews=16, fan_angle=0.6, src_iso=60.0, src_det=107.255)
    out["bh_coefs2_fan"] = dict(energies=energies, counts=counts, atten_eff=atten_eff,
                                fan_angle=0.6, src_iso=60.0, src_det=107.255,
                                coefs=bhm.beamhard_coefs2(energies, counts, g_fan, atten_eff))
    lut = function_from_source(os.path.join(ref, "tests", "Test_Beamhard", "beamhard_test.py"),
                               ["beamhard_cor2"])["beamhard_cor2"]
    coefs_tb = 1.0 + 0.05 * np.sin(np.linspace(0, 3, 4001))
    li_l = (rng.random((4, 30)) * 9.0).astype(np.float32)
    li_l[0, :4] = [0.0, 8.0, 8.2, 8.0000005]   # on, at and past the table's end (mu 0.2: 40)
    out["bh_lut"] = dict(line_ints=li_l, coefs=coefs_tb, mu=0.2, cor=lut(li_l, coefs_tb, 0.2))

    # --- helical rebinning front-end (trajectory.py, core_funcs.Geom) -------
    import vir.trajectory as traj
    rng = np.random.default_rng(27)
    sinoA = rng.random((24, 10, 12)).astype(np.float32)
    viewsH = np.linspace(0.0, 4 * np.pi, 50, endpoint=False)
    viewsH[7] = 2 * np.pi * 23 / 24 + 0.05       # past the last axial angle: grid-wrap branch
    viewsH[8] = 2 * np.pi * 5 / 24                # exactly on an axial angle
    out["traj_axl2hel"] = dict(sinoA=sinoA, nRowsH=np.int32(6), viewsH=viewsH, nAngsH=np.int32(24),
                               pitch=1.0, sinoH=traj.sino_axl2hel(sinoA, 6, viewsH, 24, 1.0))
    zH = np.linspace(-1.0, 5.5, 50)
    out["traj_axl2hel_z"] = dict(sinoA=sinoA, nRowsH=np.int32(6), viewsH=viewsH, nAngsH=np.int32(24),
                                 pitch=1.0, Z=zH,
                                 sinoH=traj.sino_axl2hel(sinoA, 6, viewsH, 24, 1.0, Z=zH))
    gH = cf.Geom(nViews=96, coverage=4 * np.pi, zTran=8.0)
    sinoH = rng.random((96, 6, 10)).astype(np.float32)
    angsA = np.array([0.0, 0.3, 1.0, np.pi, 5.9])
    zA = np.linspace(-3.0, 3.0, 7)
    a1, a2 = traj.sino_hel2axl(sinoH, gH, angsA, zA)
    f1, f2, b1, b2 = traj.sino_hel2axl180(sinoH, gH, angsA, zA)
    gI = cf.Geom(nViews=40, coverage=4 * np.pi, angle0=0.1, zTran=6.0)
    i1, i2 = traj.sino_hel2hel(sinoH, gH, gI, 4)
    out["traj_hel2axl"] = dict(sinoH=sinoH, nViews=np.int32(96), coverage=4 * np.pi, zTran=8.0,
                               angsA=angsA, zA=zA, a1=a1, a2=a2, f1=f1, f2=f2, b1=b1, b2=b2,
                               int_nViews=np.int32(40), int_coverage=4 * np.pi, int_angle0=0.1,
                               int_zTran=6.0, i1=i1, i2=i2, gH_Z=gH.Z, gH_Views=gH.Views)
    iz = gH.interpZ(zA, 1.0, 6)
    out["traj_interpZ"] = dict(zA=zA, angle=1.0, nRows=np.int32(6),
                               **{f"r{k}": np.asarray(v) for k, v in enumerate(iz)})
    gS = cf.Geom(nViews=96, coverage=4 * np.pi, zTran=8.0)
    sub = traj.sino_hel_subset(sinoH, gS, 6, [-1.0, 2.0])
    out["traj_subset"] = dict(z=np.array([-1.0, 2.0]), nRows=np.int32(6), sub=sub,
                              Views=gS.Views, Z=gS.Z)
    ph = rng.random((12, 10, 8)).astype(np.float32)
    vws = np.array([0.0, 0.4, 1.3, np.pi / 2, 2.9, 4.4])
    zz = np.array([0.0, 0.25, -1.5, 2.0, 0.7, -0.3])
    import vir.affine_transforms as aff
    mats = np.stack([(aff.rotateMat((0, 0, -v), center=np.array(ph.shape) / 2.0 - 0.5, seq='XYZ')
                      @ aff.transMat((0, 0, -z)))[:3] for v, z in zip(vws, zz)])
    out["traj_fp_phantom"] = dict(phantom=ph, views=vws, Z=zz, mats=mats,
                                  sino=traj.forward_project_phantom(ph, vws, None, None, zz))

    path = os.path.join(HERE, "golden.npz")
    flat = {}
    for k, d in out.items():
        for kk, v in d.items():
            flat[f"{k}/{kk}"] = np.asarray(v)
    np.savez_compressed(path, **flat)
    print("wrote", path, os.path.getsize(path), "bytes,", len(out), "cases")


if __name__ == "__main__":
    main()
