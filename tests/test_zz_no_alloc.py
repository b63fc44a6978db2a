"""vg_dd2d_bp_noalloc: the backprojection entry point for callers that cannot
allocate device memory when they call (a host that owns a fixed memory
budget, a loop that cannot afford cudaMalloc's implicit synchronisation, a
plugin host that forbids allocation in its callbacks).  It takes its
workspace from a fixed array inside the library instead of from the caller.

Checked through the C ABI against vg_dd2d_bp (caller-provided workspace) on
two different calls in a row, so that leftovers of the first call in the
shared array cannot leak into the second.  Kept in a file of its own that
runs last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_pair(L, g, sino, trig, dev):
    import torch
    from vir_gb300 import _core
    from vir_gb300._lib import dd2d_workspace
    ref = torch.empty((g.nx, g.ny), dtype=torch.float32, device=dev)
    ws = dd2d_workspace(g, dev)
    st = L.vg_dd2d_bp(ctypes.byref(g), ctypes.c_void_p(sino.data_ptr()),
                      ctypes.c_void_p(trig.data_ptr()), ctypes.c_void_p(ref.data_ptr()),
                      ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                      _core.stream(dev))
    assert st == 0, L.vg_last_error()
    out = torch.full((g.nx, g.ny), float("nan"), dtype=torch.float32, device=dev)
    torch.cuda.synchronize(dev)
    before = torch.cuda.memory_allocated(dev)
    # free device bytes as the driver counts them (cudaMemGetInfo): a
    # cudaMalloc inside the library would show here, where torch's own
    # counter cannot see it
    free0 = torch.cuda.mem_get_info(dev)[0]
    st = L.vg_dd2d_bp_noalloc(ctypes.byref(g), ctypes.c_void_p(sino.data_ptr()),
                              ctypes.c_void_p(trig.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                              _core.stream(dev))
    assert st == 0, L.vg_last_error()
    torch.cuda.synchronize(dev)
    assert torch.cuda.memory_allocated(dev) == before
    assert torch.cuda.mem_get_info(dev)[0] == free0
    return ref.cpu().numpy(), out.cpu().numpy()


def test_noalloc_bp_matches_workspace_bp(vg):
    import torch
    from vir_gb300 import _core
    from vir_gb300._lib import DD2DGeom, load
    L = load()
    dev = torch.device("cuda", torch.cuda.current_device())
    rng = np.random.default_rng(31)
    cases = [
        # fan, 720 views x 768 bins onto 512^2 (the benchmark geometry)
        (DD2DGeom(512, 512, 720, 768, 1.2, 0.0, 0.9, 500.0, 1000.0, 1), 2 * np.pi),
        # parallel, different sizes, so the second call rewrites the array differently
        (DD2DGeom(200, 150, 181, 260, 1.0, 0.25, 1.1, 0.0, 0.0, 0), np.pi),
    ]
    # a geometry whose workspace nearly fills the 32 MiB array
    near = DD2DGeom(512, 512, 2800, 1200, 1.2, 0.0, 0.9, 500.0, 1000.0, 1)
    need = L.vg_dd2d_workspace_bytes(ctypes.byref(near))
    cap = L.vg_dd2d_noalloc_scratch_bytes()
    assert 0.9 * cap < need <= cap
    cases.append((near, 2 * np.pi))
    for g, span in cases:
        angs = np.linspace(0, span, g.na, endpoint=False)
        trig = _core.trig_cache.get(angs, np.float32, dev)
        sino = torch.from_numpy(rng.random((g.na, g.nu)).astype(np.float32)).to(dev)
        ref, out = _run_pair(L, g, sino, trig, dev)
        assert np.isfinite(out).all()
        # same kernels on the same inputs: equal to the last bit in practice;
        # the bound is the projector tests' tolerance
        assert np.abs(out - ref).max() <= 1e-6 * np.abs(ref).max()


def test_noalloc_rejects_oversized_geometry(vg):
    from vir_gb300._lib import DD2DGeom, load
    L = load()
    g = DD2DGeom(2048, 2048, 4000, 3072, 1.0, 0.0, 1.0, 0.0, 0.0, 0)
    assert L.vg_dd2d_workspace_bytes(ctypes.byref(g)) > L.vg_dd2d_noalloc_scratch_bytes()
    st = L.vg_dd2d_bp_noalloc(ctypes.byref(g), ctypes.c_void_p(16), ctypes.c_void_p(16),
                              ctypes.c_void_p(16), None)
    assert st == 1
    assert b"scratch" in L.vg_last_error()
