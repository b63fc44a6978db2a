"""Builds libvirgpu.so from csrc/*.cu for sm_103a (GB300), in tree.

    python -m vir_gb300.build        # or vir_gb300.build.build()

Each translation unit is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo) and linked into
vir_gb300/_build/libvirgpu.so.  Only nvcc and the CUDA runtime are needed; no
cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvirgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found (set NVCC or put CUDA's bin on PATH)")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _digest() -> str:
    h = hashlib.sha256()
    files = _sources() + sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + \
        sorted(glob.glob(os.path.join(INCLUDE, "*.h")))
    for f in files:
        h.update(os.path.basename(f).encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, out_dir: str = None,
          defines=()) -> str:
    """Compile (when sources changed) and return the path of libvirgpu.so.

    ``out_dir``/``defines`` build a variant (extra -D macros, e.g. tile
    sizes) into another directory, for tuning sweeps."""
    out_dir = out_dir or OUT_DIR
    lib_path = os.path.join(out_dir, "libvirgpu.so")
    os.makedirs(out_dir, exist_ok=True)
    stamp = os.path.join(out_dir, "libvirgpu.sha256")
    dig = _digest() + "|" + ",".join(defines)
    if not force and os.path.exists(lib_path) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == dig:
                return lib_path
    cc = nvcc()
    dflags = [f"-D{d}" for d in defines]
    objs = []

    def compile_one(src):
        obj = os.path.join(out_dir, os.path.basename(src)[:-3] + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, *dflags, "-I", INCLUDE, "-c", src, "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for obj, log in ex.map(compile_one, _sources()):
            objs.append(obj)
            if verbose and log:
                print(log)
    tmp = lib_path + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib_path)
    with open(stamp, "w") as fh:
        fh.write(dig)
    return lib_path


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
