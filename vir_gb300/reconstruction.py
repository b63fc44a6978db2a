"""SIRT and FBP on the GPU distance-driven projectors.

SIRT follows vir's update rule (``sys_mat/sirt_dd.py:23-76``):

    x0 = 1e-5;  for i in range(1, iters):
        r = (y - FP x) / W_sino       (left as FP x where W_sino == 0)
        x = x + gamma * BP(r) / W_img (left as BP r where W_img == 0)

with ``W_sino = FP(1)`` and ``W_img = BP(1)`` computed by the same projector
pair.  The reference runs it around its 4-sided translational geometry; the
same rule wraps the parallel and fan projectors here (as in
``processing/SIRT/sirt.py:34-40``).  On the GPU one update is two fused
kernels (``vg_dd2d_sirt_iter``: residual ratio in the FP epilogue, image
update in the BP epilogue), and a run of updates is captured once as a CUDA
graph and replayed.

FBP (``fbp_2d``) is filter (``filtration.filter_sino``'s 2H, on the GPU) then
a pixel-driven backprojection (``vg_fbp2d_bp``); the fan version pre-weights
rows by DSO / sqrt(DSO^2 + s^2) with s the bin centre scaled to the
isocentre and filters at the isocentre spacing du * DSO / DSD.
"""
from __future__ import annotations

import collections
import ctypes
import threading

import numpy as np
import torch

from . import _core
from ._lib import DD2DGeom, DD3DGeom, call, dd2d_workspace
from .filtration import filter_rows_device


def _initial(x0, shape, dev):
    """vir's start value (a scalar, 1e-5) or an iterate to resume from (an
    image of ``shape``, as ``initial`` of processing/SIRT/sirt.py:15-29):
    (scalar or None, float32 device tensor or None)."""
    if np.ndim(x0) == 0:
        return float(np.float32(float(x0))), None
    t = _core.to_device(x0, dev)
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"x0 has shape {tuple(t.shape)}, the image {tuple(shape)}")
    return None, t


def _geom(nx, ny, na, nu, du, su, d_pix, DSO, DSD, fan, variant=0):
    return DD2DGeom(int(nx), int(ny), int(na), int(nu), _core.f32(du), _core.f32(su),
                    _core.f32(d_pix), _core.f32(DSO), _core.f32(DSD), int(fan), int(variant))


class SIRT2D:
    """Resident SIRT state for one 2D problem on one GPU.

    All buffers live in device memory for the life of the object: the
    measured sinogram ``y``, ``1/W_sino``, ``1/W_img``, the iterate ``x`` and
    its transpose, and the residual scratch ``r``.
    """

    def __init__(self, sino, ang_arr, img_shape, geom="par", DSO=0.0, DSD=0.0, du=1.0, su=0.0,
                 d_pix=1.0, gamma=1.0, x0=1e-5, W_sino=None, W_img=None, device=None,
                 autotune=False):
        _core.require_cuda()
        self.dev = device or _core.device_of(sino)
        self.fan = 1 if geom == "fan" else 0
        self.y = _core.to_device(sino, self.dev)
        self.trig = _core.trig_cache.get(ang_arr, np.float32, self.dev)
        na = self.trig.numel() // 2
        nx, ny = (int(v) for v in img_shape)
        nu = self.y.shape[1]
        if self.y.shape[0] != na:
            raise ValueError("sino rows must equal len(ang_arr)")
        self.g = _geom(nx, ny, na, nu, du, su, d_pix, DSO, DSD, self.fan)
        if autotune:
            from .autotune import best_fp_variant
            self.g.variant = best_fp_variant(self.g, self.dev)
        self.gamma = float(gamma)
        self.ws = dd2d_workspace(self.g, self.dev)
        if W_sino is None:
            ones = torch.ones((nx, ny), dtype=torch.float32, device=self.dev)
            W_sino = self.fp(ones)
        else:
            W_sino = _core.to_device(W_sino, self.dev)
        if W_img is None:
            W_img = self.bp(torch.ones((na, nu), dtype=torch.float32, device=self.dev))
        else:
            W_img = _core.to_device(W_img, self.dev)
        self.inv_ws = torch.where(W_sino != 0, 1.0 / W_sino, torch.zeros_like(W_sino))
        self.inv_wi = torch.where(W_img != 0, 1.0 / W_img, torch.zeros_like(W_img))
        self.x = torch.empty((nx, ny), dtype=torch.float32, device=self.dev)
        self.xT = torch.empty((ny, nx), dtype=torch.float32, device=self.dev)
        self.reset(x0)
        self.r = torch.empty((na, nu), dtype=torch.float32, device=self.dev)
        self._graph = None
        self._graph_n = 0

    def load_sino(self, sino):
        """Copy a new measured sinogram of the same shape into the resident
        ``y`` (asynchronous from pinned host memory; ordered before the next
        update on the current stream)."""
        if _core.is_torch(sino):
            src = sino.detach()
            if src.dtype != torch.float32:
                src = src.float()
        else:
            src = torch.from_numpy(np.ascontiguousarray(np.asarray(sino), dtype=np.float32))
        if tuple(src.shape) != tuple(self.y.shape):
            raise ValueError(f"sino shape {tuple(src.shape)} != {tuple(self.y.shape)}")
        self.y.copy_(src, non_blocking=True)

    # projector pair on this geometry
    def fp(self, img: torch.Tensor) -> torch.Tensor:
        out = torch.empty((self.g.na, self.g.nu), dtype=torch.float32, device=self.dev)
        imgT = img.t().contiguous()
        call("vg_dd2d_fp", ctypes.byref(self.g), _core.ptr(img), _core.ptr(imgT),
             _core.ptr(self.trig), _core.ptr(out), _core.stream(self.dev))
        return out

    def bp(self, sino: torch.Tensor) -> torch.Tensor:
        out = torch.empty((self.g.nx, self.g.ny), dtype=torch.float32, device=self.dev)
        call("vg_dd2d_bp", ctypes.byref(self.g), _core.ptr(sino), _core.ptr(self.trig),
             _core.ptr(out), _core.ptr(self.ws), self.ws.numel(), _core.stream(self.dev))
        return out

    def _iter(self):
        call("vg_dd2d_sirt_iter", ctypes.byref(self.g), _core.ptr(self.y), _core.ptr(self.inv_ws),
             _core.ptr(self.inv_wi), ctypes.c_float(self.gamma), _core.ptr(self.trig),
             _core.ptr(self.x), _core.ptr(self.xT), _core.ptr(self.r), _core.ptr(self.ws),
             self.ws.numel(), _core.stream(self.dev))

    def capture(self, n: int):
        """Capture ``n`` updates as one CUDA graph (replayed by run())."""
        s = torch.cuda.Stream(self.dev)
        s.wait_stream(torch.cuda.current_stream(self.dev))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(n):
                    self._iter()
        torch.cuda.current_stream(self.dev).wait_stream(s)
        self._graph, self._graph_n = g, n
        return g

    def run(self, n_updates: int, graph: bool = True):
        """Apply ``n_updates`` SIRT updates to x (asynchronous)."""
        if n_updates <= 0:
            return self.x
        if graph:
            if self._graph is None or self._graph_n != n_updates:
                self.capture(n_updates)
            self._graph.replay()
        else:
            for _ in range(n_updates):
                self._iter()
        return self.x

    def reset(self, x0=1e-5):
        """Restart from x0: a scalar (vir's 1e-5) or an (nx, ny) iterate to resume from."""
        v, t = _initial(x0, self.x.shape, self.dev)
        if t is None:
            self.x.fill_(v)
            self.xT.fill_(v)
        else:
            self.x.copy_(t)
            self.xT.copy_(t.t())


class SIRT3D:
    """Resident SIRT state for one circular cone-beam problem (the DD cone
    pair of dd_fp_cone_3d / dd_bp_cone_3d) on one GPU: the measured sinogram,
    1/W_sino, 1/W_img, the iterate and the residual scratch stay in device
    memory; one update is vg_dd3d_sirt_iter (residual in the forward
    projection's epilogue, update in the back projection's), and a run of
    updates is captured once as a CUDA graph and replayed."""

    def __init__(self, sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0,
                 d_pix=1.0, gamma=1.0, x0=1e-5, device=None):
        from ._lib import dd3d_workspace
        _core.require_cuda()
        self.dev = device or _core.device_of(sino)
        self.y = _core.to_device(sino, self.dev)
        if self.y.ndim != 3:
            raise ValueError("sino must be (na, nu, nv)")
        self.trig = _core.trig_cache.get(ang_arr, np.float32, self.dev)
        na = self.trig.numel() // 2
        if self.y.shape[0] != na:
            raise ValueError("sino rows must equal len(ang_arr)")
        f = _core.f32
        self.g = DD3DGeom(*(int(v) for v in img_shape), na, int(self.y.shape[1]),
                          int(self.y.shape[2]), f(du), f(dv), f(su), f(sv), f(d_pix), f(DSO), f(DSD))
        self.gamma = float(gamma)
        self.ws = dd3d_workspace(self.g, self.dev)
        shape = tuple(int(v) for v in img_shape)
        W_sino = self._fp(torch.ones(shape, dtype=torch.float32, device=self.dev))
        W_img = self._bp(torch.ones_like(self.y))
        self.inv_ws = torch.where(W_sino != 0, 1.0 / W_sino, torch.zeros_like(W_sino))
        self.inv_wi = torch.where(W_img != 0, 1.0 / W_img, torch.zeros_like(W_img))
        del W_sino, W_img
        self.x = torch.empty(shape, dtype=torch.float32, device=self.dev)
        self.reset(x0)
        self.r = torch.empty_like(self.y)
        self._graph = None
        self._graph_n = 0

    def _fp(self, x):
        out = torch.empty((self.g.na, self.g.nu, self.g.nv), dtype=torch.float32, device=self.dev)
        call("vg_dd3d_fp", ctypes.byref(self.g), _core.ptr(x), _core.ptr(self.trig), _core.ptr(out),
             _core.ptr(self.ws), self.ws.numel() * 4, _core.stream(self.dev))
        return out

    def _bp(self, y):
        out = torch.empty((self.g.nx, self.g.ny, self.g.nz), dtype=torch.float32, device=self.dev)
        call("vg_dd3d_bp", ctypes.byref(self.g), _core.ptr(y), _core.ptr(self.trig), _core.ptr(out),
             _core.ptr(self.ws), self.ws.numel() * 4, _core.stream(self.dev))
        return out

    def _iter(self):
        call("vg_dd3d_sirt_iter", ctypes.byref(self.g), _core.ptr(self.y), _core.ptr(self.inv_ws),
             _core.ptr(self.inv_wi), ctypes.c_float(self.gamma), _core.ptr(self.trig),
             _core.ptr(self.x), _core.ptr(self.r), _core.ptr(self.ws), self.ws.numel() * 4,
             _core.stream(self.dev))

    def capture(self, n: int):
        """Capture ``n`` updates as one CUDA graph (replayed by run())."""
        s = torch.cuda.Stream(self.dev)
        s.wait_stream(torch.cuda.current_stream(self.dev))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(n):
                    self._iter()
        torch.cuda.current_stream(self.dev).wait_stream(s)
        self._graph, self._graph_n = g, n
        return g

    def run(self, n_updates: int, graph: bool = True):
        """Apply ``n_updates`` SIRT updates to x (asynchronous)."""
        if n_updates <= 0:
            return self.x
        if graph:
            if self._graph is None or self._graph_n != n_updates:
                self.capture(n_updates)
            self._graph.replay()
        else:
            for _ in range(n_updates):
                self._iter()
        return self.x

    def reset(self, x0=1e-5):
        """Restart from x0: a scalar (vir's 1e-5) or an (nx, ny, nz) iterate to resume from."""
        v, t = _initial(x0, self.x.shape, self.dev)
        if t is None:
            self.x.fill_(v)
        else:
            self.x.copy_(t)


def sirt_3d(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0,
            gamma=1.0, iters=20, graph=True, x0=1e-5):
    """vir's SIRT (``iters - 1`` updates, x0 = 1e-5) on the cone-beam DD pair;
    ``x0`` may be an iterate to resume from."""
    s = SIRT3D(sino, ang_arr, img_shape, DSO, DSD, du, dv, su, sv, d_pix, gamma, x0=x0)
    x = s.run(int(iters) - 1, graph=graph)
    return _core.to_host_like(x.clone(), sino)


class _PreparedSirt:
    """The prepared SIRT2D states of the last few geometries sirt_2d has
    seen (weights W_sino = FP(1) and W_img = BP(1), device buffers, the
    captured update graph): a call on a geometry seen before copies its
    sinogram into the prepared state and replays the graph, as an FFT
    library reuses a plan.  Each state has its own lock, so concurrent calls
    on one geometry take turns on the host, and an event recorded after each
    call's work, which the next caller's stream waits on, so that their GPU
    work also runs in turn when they use different streams; the states hold
    their device buffers until evicted (at most ``cap``)."""

    def __init__(self, cap=4):
        self._d = collections.OrderedDict()
        self._cap = cap
        self._lock = threading.Lock()

    def get(self, key, make):
        with self._lock:
            e = self._d.get(key)
            if e is not None:
                self._d.move_to_end(key)
                return e
        e = [threading.Lock(), make(), None]  # lock, state, event after the last call's work
        with self._lock:
            self._d[key] = e
            while len(self._d) > self._cap:
                self._d.popitem(last=False)
        return e

    def clear(self):
        with self._lock:
            self._d.clear()


prepared_sirt = _PreparedSirt()


def sirt_2d(sino, ang_arr, img_shape, geom="par", DSO=0.0, DSD=0.0, du=1.0, su=0.0, d_pix=1.0,
            gamma=1.0, iters=100, W_sino=None, W_img=None, graph=True, x0=1e-5):
    """vir's SIRT (``iters - 1`` updates, x0 = 1e-5) on the parallel or fan
    distance-driven pair.  numpy in -> numpy out.  ``x0`` may be an iterate
    to resume from (``initial`` of processing/SIRT/sirt.py).  Without caller
    weights the geometry's prepared state (weights, buffers, update graph) is
    reused across calls (``prepared_sirt``)."""
    if W_sino is not None or W_img is not None:
        s = SIRT2D(sino, ang_arr, img_shape, geom=geom, DSO=DSO, DSD=DSD, du=du, su=su,
                   d_pix=d_pix, gamma=gamma, x0=x0, W_sino=W_sino, W_img=W_img)
        x = s.run(int(iters) - 1, graph=graph)
        return _core.to_host_like(x.clone(), sino)
    dev = _core.device_of(sino)
    a = _core.host_angles(ang_arr)
    f = _core.f32
    key = (str(dev), a.dtype.str, a.shape, a.tobytes(), tuple(int(v) for v in np.shape(sino)),
           tuple(int(v) for v in img_shape), geom, f(DSO), f(DSD), f(du), f(su), f(d_pix),
           float(gamma))
    e = prepared_sirt.get(key, lambda: SIRT2D(sino, ang_arr, img_shape, geom=geom, DSO=DSO,
                                              DSD=DSD, du=du, su=su, d_pix=d_pix, gamma=gamma,
                                              device=dev))
    with e[0]:
        s = e[1]
        cur = torch.cuda.current_stream(s.dev)
        if e[2] is not None:
            cur.wait_event(e[2])  # the previous call's work on this state, on any stream
        s.load_sino(sino)
        s.reset(x0)
        x = s.run(int(iters) - 1, graph=graph).clone()
        e[2] = torch.cuda.Event()
        e[2].record(cur)
    return _core.to_host_like(x, sino)


def fan_preweight(nu, du, su, DSO, DSD):
    """Equispaced cosine pre-weight DSO / sqrt(DSO^2 + s^2) at the bin
    centres scaled to the isocentre (processing/reconstruction.py:99-107)."""
    s = du * (np.arange(nu) - nu / 2.0 + 0.5 + su) * DSO / DSD
    return DSO / np.sqrt(DSO ** 2 + s ** 2)


def fbp_2d(sino, ang_arr, img_shape, geom="par", DSO=0.0, DSD=0.0, du=1.0, su=0.0, d_pix=1.0,
           filter_type="ramp", cutoff=0.5, real_space=True, method="pixel"):
    """Filtered backprojection of a full scan (pi parallel, 2 pi fan).

    method="pixel": the pixel-driven 1/U^2-weighted backprojection
    (vg_fbp2d_bp).  method="dd" (parallel only): vir's working parallel FBP
    over 180 degrees, (pi / 2) dd_bp_par_2d(filter_sino(y)), on the GPU
    distance-driven backprojector."""
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na, nu = y.shape
    fan = 1 if geom == "fan" else 0
    if method == "dd":
        if fan:
            raise ValueError("fbp_2d: method='dd' is vir's parallel-beam route")
        from .sys_mat import dd
        q = filter_rows_device(y, du, filter_type, cutoff, real_space)
        img = dd.dd_bp_par_2d(q, ang_arr, img_shape, du=du, su=su, d_pix=d_pix)
        img.mul_(float(np.pi / 2.0))
        return _core.to_host_like(img, sino)
    if method != "pixel":
        raise ValueError(f"fbp_2d: unknown method {method!r}")
    if fan:
        w = torch.from_numpy(fan_preweight(nu, float(np.float32(du)), float(np.float32(su)),
                                           float(np.float32(DSO)),
                                           float(np.float32(DSD))).astype(np.float32)).to(dev)
        q = filter_rows_device(y, du * DSO / DSD, filter_type, cutoff, real_space, row_weight=w)
    else:
        q = filter_rows_device(y, du, filter_type, cutoff, real_space)
    nx, ny = (int(v) for v in img_shape)
    g = _geom(nx, ny, na, nu, du, su, d_pix, DSO, DSD, fan)
    img = torch.empty((nx, ny), dtype=torch.float32, device=dev)
    call("vg_fbp2d_bp", ctypes.byref(g), _core.ptr(q), _core.ptr(trig), _core.ptr(img),
         _core.stream(dev))
    return _core.to_host_like(img, sino)


def fdk(sino, ang_arr, img_shape, DSO, DSD, du=1.0, dv=1.0, su=0.0, sv=0.0, d_pix=1.0,
        filter_type="ramp", cutoff=0.5, real_space=True):
    """FDK reconstruction of a full circular cone-beam scan (na, nu, nv) on the
    geometry of ``dd_fp_cone_3d``: cosine pre-weight, ramp filter along u at
    the isocentre pitch, 1/U^2-weighted voxel-driven backprojection.  vir has
    no FDK; the weights extend its fan-beam FBP spec (see vg_fdk_* in
    include/virgpu.h)."""
    dev = _core.device_of(sino)
    y = _core.to_device(sino, dev)
    if y.ndim != 3:
        raise ValueError("sino must be (na, nu, nv)")
    trig = _core.trig_cache.get(ang_arr, np.float32, dev)
    na, nu, nv = y.shape
    f = _core.f32
    g = DD3DGeom(int(img_shape[0]), int(img_shape[1]), int(img_shape[2]), na, nu, nv,
                 f(du), f(dv), f(su), f(sv), f(d_pix), f(DSO), f(DSD))
    t = torch.empty((na, nv, nu), dtype=torch.float32, device=dev)
    call("vg_fdk_weight_transpose", ctypes.byref(g), _core.ptr(y), _core.ptr(t), _core.stream(dev))
    qt = filter_rows_device(t.view(na * nv, nu), f(du) * f(DSO) / f(DSD), filter_type, cutoff,
                            real_space)
    q = torch.empty((na, nu, nv), dtype=torch.float32, device=dev)
    call("vg_fdk_transpose_back", ctypes.byref(g), _core.ptr(qt), _core.ptr(q), _core.stream(dev))
    del t, qt
    vol = torch.empty(tuple(int(v) for v in img_shape), dtype=torch.float32, device=dev)
    call("vg_fdk_bp", ctypes.byref(g), _core.ptr(q), _core.ptr(trig), _core.ptr(vol),
         _core.stream(dev))
    return _core.to_host_like(vol, sino)
