"""CPU checks of the C-ABI library: it builds for sm_103a, loads, and exports
every entry point include/virgpu.h declares (no compute calls)."""
import ctypes
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(REPO, "include", "virgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vg_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_header():
    from vir_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 8
    for s in syms:
        assert hasattr(lib, s), s
    lib.vg_version.restype = ctypes.c_int
    assert lib.vg_version() >= 100


def test_python_bindings_cover_header():
    from vir_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.exported_symbols())


def test_status_strings():
    from vir_gb300 import build
    lib = ctypes.CDLL(build.build())
    lib.vg_status_string.restype = ctypes.c_char_p
    assert lib.vg_status_string(0) == b"ok"
    assert lib.vg_status_string(1) == b"bad argument"


def test_argument_errors_without_gpu():
    """Invalid sizes are rejected on the host before any launch."""
    from vir_gb300 import _lib
    L = _lib.load()
    g = _lib.DD2DGeom(0, 10, 5, 5, 1.0, 0.0, 1.0, 0.0, 0.0, 0)
    st = L.vg_dd2d_fp(ctypes.byref(g), None, None, None, None, None)
    assert st == 1
    assert b"positive" in L.vg_last_error()


def test_sf3d_workspace_without_gpu():
    """vg_sf3d_workspace_bytes (host only) covers both cone SF calls: the
    forward projection's per-column z sums, nx ny (nz + 1) floats, and the
    back projection's weighted view chunk (at most 256 MiB or one view);
    a forward projection given less is refused before any launch."""
    from vir_gb300 import _lib
    L = _lib.load()
    for (n, nz, na, nu, nv) in ((256, 256, 360, 512, 384), (64, 40, 10, 80, 60), (512, 512, 720, 1024, 768)):
        g = _lib.DD3DGeom(n, n, nz, na, nu, nv, 1.6, 1.6, 0.0, 0.0, 1.0, 600.0, 1100.0)
        fp_need = n * n * (nz + 1) * 4
        chunk = max(1, min(na, (256 << 20) // (nu * nv * 4)))
        bp_need = chunk * nu * nv * 4
        assert L.vg_sf3d_workspace_bytes(ctypes.byref(g)) == max(fp_need, bp_need)
    g = _lib.DD3DGeom(64, 64, 40, 10, 80, 60, 1.6, 1.6, 0.0, 0.0, 1.0, 600.0, 1100.0)
    p = ctypes.c_void_p(256)  # never dereferenced
    st = L.vg_sf3d_fp(ctypes.byref(g), p, p, p, p, 64 * 64 * 41 * 4 - 4, None)
    assert st == 1 and b"workspace" in L.vg_last_error()


def test_sirt_launch_count_without_gpu():
    """vg_dd2d_sirt_launches (host-only): 2 launches per SIRT update when one
    8-warp block holds all bins of a view (the forward projection then writes
    the back projection's tables), 3 otherwise, 0 for a rejected geometry."""
    from vir_gb300 import _lib
    L = _lib.load()
    # the fan SIRT benchmark geometry: 512^2, 720 views, 768 bins (8 warps x 24 bins)
    g = _lib.DD2DGeom(512, 512, 720, 768, 1.2, 0.0, 0.9, 500.0, 1000.0, 1, 0)
    assert L.vg_dd2d_sirt_launches(ctypes.byref(g)) == 2
    # 1024^2 with 1536 bins: 4-warp tiles, the table kernel runs separately
    g = _lib.DD2DGeom(1024, 1024, 90, 1536, 1.0, 0.0, 1.0, 0.0, 0.0, 0, 0)
    assert L.vg_dd2d_sirt_launches(ctypes.byref(g)) == 3
    # an explicit 8-warp variant (6 bins per lane) whose block covers half of the bins
    g = _lib.DD2DGeom(256, 256, 90, 384, 1.0, 0.0, 1.0, 0.0, 0.0, 0, 1)
    assert L.vg_dd2d_sirt_launches(ctypes.byref(g)) == 3
    g = _lib.DD2DGeom(0, 256, 90, 384, 1.0, 0.0, 1.0, 0.0, 0.0, 0, 0)
    assert L.vg_dd2d_sirt_launches(ctypes.byref(g)) == 0


def test_batch_items_without_gpu():
    """vg_sirt2d_batch_items (host-only): per problem na * chunks forward
    projection items (chunks of 192, 384 or 768 bins), na table items and
    (ny / 16) x (nx / 64) back projection tiles, rounded up; every (problem,
    item) pair listed once; null buffers, misaligned workspaces and fan
    detectors reaching the inverse map's pole are refused."""
    import numpy as np
    from vir_gb300 import _lib
    L = _lib.load()
    geoms = [(128, 128, 90, 192, 0), (256, 200, 101, 384, 1), (512, 512, 720, 768, 1),
             (1024, 1024, 40, 1536, 0), (100, 300, 7, 450, 0)]
    P = (_lib.Sirt2DProblem * len(geoms))()
    for i, (nx, ny, na, nu, fan) in enumerate(geoms):
        d = 1.0
        g = _lib.DD2DGeom(nx, ny, na, nu, 1.0, 0.0, d, 2.0 * nx * d if fan else 0.0,
                          4.0 * nx * d if fan else 0.0, fan, 0)
        P[i] = _lib.Sirt2DProblem(g, 16, 16, 16, 16, 16, 16, 16, 256, 1.0, 0)  # never dereferenced
    n = len(geoms)
    nf, nt, nb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert L.vg_sirt2d_batch_items(P, n, None, ctypes.byref(nf), None, ctypes.byref(nt), None,
                                   ctypes.byref(nb)) == 0
    chunk = lambda nu: 192 if nu <= 192 else (384 if nu <= 384 else 768)
    ef = sum(na * -(-nu // chunk(nu)) for _, _, na, nu, _ in geoms)
    et = sum(na for _, _, na, _, _ in geoms)
    eb = sum(-(-ny // 16) * -(-nx // 64) for nx, ny, _, _, _ in geoms)
    assert (nf.value, nt.value, nb.value) == (ef, et, eb)
    fi = np.empty((ef, 2), np.int32)
    ti = np.empty((et, 2), np.int32)
    bi = np.empty((eb, 2), np.int32)
    assert L.vg_sirt2d_batch_items(P, n, fi.ctypes.data, ctypes.byref(nf), ti.ctypes.data,
                                   ctypes.byref(nt), bi.ctypes.data, ctypes.byref(nb)) == 0
    for items, per in ((fi, lambda q: geoms[q][2] * -(-geoms[q][3] // chunk(geoms[q][3]))),
                       (ti, lambda q: geoms[q][2]),
                       (bi, lambda q: -(-geoms[q][1] // 16) * -(-geoms[q][0] // 64))):
        pairs = set(map(tuple, items.tolist()))
        assert len(pairs) == len(items)
        assert pairs == {(q, k) for q in range(n) for k in range(per(q))}
    bad = (_lib.Sirt2DProblem * 1)(P[0])
    bad[0].workspace = 128  # not 256-byte aligned
    assert L.vg_sirt2d_batch_items(bad, 1, None, ctypes.byref(nf), None, ctypes.byref(nt), None,
                                   ctypes.byref(nb)) != 0
    bad[0] = P[0]
    bad[0].y = None
    assert L.vg_sirt2d_batch_items(bad, 1, None, ctypes.byref(nf), None, ctypes.byref(nt), None,
                                   ctypes.byref(nb)) != 0
    bad[0] = P[1]
    bad[0].g.DSD = 0.2 * bad[0].g.nu  # the detector reaches beyond DSD: the pole
    assert L.vg_sirt2d_batch_items(bad, 1, None, ctypes.byref(nf), None, ctypes.byref(nt), None,
                                   ctypes.byref(nb)) != 0


def test_drop_in_table_resolves_and_installs():
    """Every vir function named in the drop-in table exists here, and
    install_into replaces it in an imported vir package (a stand-in tree of
    empty modules, so no GPU and no vir import are needed)."""
    import importlib
    import sys
    import types
    import vir_gb300
    for mod, fns in vir_gb300._DROP_INS.items():
        for name, spec in fns.items():
            m, a = spec.split(":")
            assert callable(getattr(importlib.import_module(m), a)), spec
    root = types.ModuleType("fakevir")
    made = {"fakevir": root}
    for mod in vir_gb300._DROP_INS:
        parts = mod.split(".")
        for i in range(1, len(parts) + 1):
            full = "fakevir." + ".".join(parts[:i])
            if full not in made:
                made[full] = types.ModuleType(full)
    saved = {k: sys.modules.get(k) for k in made}
    sys.modules.update(made)
    try:
        done = vir_gb300.install_into(root)
        assert len(done) == sum(len(f) for f in vir_gb300._DROP_INS.values())
        from vir_gb300.sys_mat import dd
        assert made["fakevir.sys_mat.dd"].dd_fp_fan_2d is dd.dd_fp_fan_2d
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


def _autotune_writer(args):
    path, tag, n = args
    os.environ["VIR_GB300_AUTOTUNE"] = path
    from vir_gb300 import autotune
    for i in range(n):
        with autotune._file_lock():
            c = autotune._read()
            c[f"{tag}-{i}"] = {"variant": i}
            autotune._write(c)
    return tag


def test_autotune_cache_writes_from_two_processes(tmp_path):
    """Two processes updating the autotune cache at once keep each other's
    entries and leave no temporary files behind (file lock around the
    read-modify-write, a private temporary file per write)."""
    import multiprocessing as mp
    path = str(tmp_path / "autotune.json")
    with mp.get_context("spawn").Pool(2) as pool:
        tags = pool.map(_autotune_writer, [(path, "a", 25), (path, "b", 25)])
    assert sorted(tags) == ["a", "b"]
    import json
    with open(path) as fh:
        c = json.load(fh)
    assert len(c) == 50
    assert not [f for f in os.listdir(tmp_path) if f.endswith(".tmp")]
