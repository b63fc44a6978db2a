"""Project-written autotuner for the tile variants of the 2D distance-driven
forward projector (warps x bins per lane, ``vg_dd2d_fp_variants``).

The first time a geometry class is seen, every variant is timed on the
current GPU with CUDA events (on random data of that geometry) and the
fastest is stored in a JSON cache keyed on (kernel, geometry class, GPU
name, library version); later calls read the cache.  The cache lives in
``$VIR_GB300_AUTOTUNE`` or ``~/.cache/vir_gb300/autotune.json``.  Variant 0
(no tuning) uses the library's size heuristic.
"""
from __future__ import annotations

import contextlib
import ctypes
import json
import os
import tempfile
import threading

import numpy as np
import torch

from . import _core
from ._lib import DD2DGeom, call, load

_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("VIR_GB300_AUTOTUNE",
                          os.path.join(os.path.expanduser("~"), ".cache", "vir_gb300",
                                       "autotune.json"))


def _read():
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


@contextlib.contextmanager
def _file_lock():
    """Exclusive lock on a lock file beside the cache, across processes (the
    replica ranks of one job may tune at the same time); the threading lock
    covers the threads of one process."""
    path = cache_path() + ".lock"
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with _lock, open(path, "a") as fh:
        try:
            import fcntl
            fcntl.flock(fh, fcntl.LOCK_EX)
        except (ImportError, OSError):
            pass  # no flock on this platform: the thread lock still holds
        try:
            yield
        finally:
            try:
                fcntl.flock(fh, fcntl.LOCK_UN)
            except (NameError, OSError):
                pass


def _write(d):
    """Write the cache through a temporary file of its own, then rename it
    into place (call with the file lock held)."""
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=os.path.dirname(path), prefix=".autotune.", suffix=".tmp")
    try:
        with os.fdopen(fd, "w") as fh:
            json.dump(d, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except BaseException:
        with contextlib.suppress(OSError):
            os.unlink(tmp)
        raise


def _key(g, dev):
    name = torch.cuda.get_device_name(dev).replace(" ", "_")
    na_class = 1 << max(0, int(np.ceil(np.log2(max(g.na, 1)))))
    return (f"dd2d_fp|fan={g.fan}|nx={g.nx}|ny={g.ny}|nu={g.nu}|na~{na_class}|{name}"
            f"|lib={load().vg_version()}")


def time_fp_variants(g, dev, reps=3):
    """ms per call of each forward-projector variant on this geometry."""
    L = load()
    x = torch.rand((g.nx, g.ny), device=dev)
    xT = x.t().contiguous()
    angs = np.linspace(0, 2 * np.pi, g.na, endpoint=False)
    trig = _core.trig_cache.get(angs, np.float32, dev)
    out = torch.empty((g.na, g.nu), device=dev)
    st = _core.stream(dev)
    res = {}
    for v in range(1, L.vg_dd2d_fp_variants() + 1):
        gv = DD2DGeom(g.nx, g.ny, g.na, g.nu, g.du, g.su, g.d_pix, g.DSO, g.DSD, g.fan, v)
        try:
            call("vg_dd2d_fp", ctypes.byref(gv), x.data_ptr(), xT.data_ptr(), trig.data_ptr(),
                 out.data_ptr(), st)
        except Exception:
            continue  # variant not applicable (e.g. shared memory) for this size
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            call("vg_dd2d_fp", ctypes.byref(gv), x.data_ptr(), xT.data_ptr(), trig.data_ptr(),
                 out.data_ptr(), st)
        e1.record()
        torch.cuda.synchronize(dev)
        res[v] = e0.elapsed_time(e1) / reps
    return res


def best_fp_variant(g, dev=None) -> int:
    """The fastest forward-projector variant for g's geometry class (cached)."""
    dev = dev or torch.device("cuda", torch.cuda.current_device())
    key = _key(g, dev)
    with _file_lock():
        c = _read()
        if key in c:
            return int(c[key]["variant"])
    t = time_fp_variants(g, dev)
    if not t:
        return 0
    best = min(t, key=t.get)
    with _file_lock():  # read-modify-write under the lock: entries of other processes are kept
        c = _read()
        c[key] = {"variant": int(best), "ms": {str(k): round(v, 4) for k, v in t.items()}}
        _write(c)
    return int(best)
