"""Batched SIRT: many independent 2D problems (uneven image sizes, view
counts, parallel or fan) iterated together in one CUDA graph.

Each problem keeps its resident state (``reconstruction.SIRT2D``: measured
sinogram, weights, iterate, workspace).  ``BatchedSIRT2D.capture(n)`` records
n SIRT updates of every problem into a single CUDA graph, with the problems
spread over a set of side streams forked from and joined to the capture
stream, so independent problems run concurrently on the GPU and a whole
batch of iterations is one graph launch with no host round trips.  The
update rule is vir's (sys_mat/sirt_dd.py:23-76), via the fused
``vg_dd2d_sirt_iter`` kernels.

``plain(n)`` runs the same updates one problem at a time, one kernel launch
per step (the baseline the batched path is measured against).

``PersistentSIRT2D`` runs the same updates of all problems in ONE persistent
launch (``vg_sirt2d_batch_run``): the resident blocks take work items --
(problem, view, bin chunk) for the forward projection, (problem, view) for
the back projection's tables, (problem, pixel tile) for the back projection
-- from one queue (each kind ordered by decreasing cost), every item waiting
only for the items of its own problem it reads, so that different problems'
updates overlap.  The iterates and/or the measured sinograms may be kept
in bfloat16 (``storage``), arithmetic in float32.  A run stops early, with a
status, when the caller raises ``cancel()`` (pinned host memory the kernel
reads at the start of every update) or when its time budget is spent.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _core
from ._lib import Sirt2DProblem, VirGpuError, call, load
from .reconstruction import SIRT2D

STORAGE = {"fp32": 0, "bf16x": 1, "bf16y": 2, "bf16": 3}
STATUS = {0: "ok", 3: "timeout", 4: "cancelled"}


class BatchedSIRT2D:
    def __init__(self, problems, device=None, n_streams=16, autotune=False):
        """problems: list of dicts with SIRT2D's arguments (sino, ang_arr,
        img_shape, geom, DSO, DSD, du, su, d_pix, gamma)."""
        self.dev = device or torch.device("cuda", torch.cuda.current_device())
        self.items = [SIRT2D(device=self.dev, autotune=autotune, **p) for p in problems]
        self.n_streams = max(1, int(n_streams))
        self._graph = None
        self._n = 0

    def reset(self):
        for it in self.items:
            it.reset()

    def capture(self, n_updates: int):
        cur = torch.cuda.current_stream(self.dev)
        cap = torch.cuda.Stream(self.dev)
        side = [torch.cuda.Stream(self.dev) for _ in range(self.n_streams)]
        cap.wait_stream(cur)
        g = torch.cuda.CUDAGraph()
        # largest problems first so their chains start early
        order = sorted(range(len(self.items)),
                       key=lambda i: -self.items[i].g.na * self.items[i].g.nx * self.items[i].g.ny)
        with torch.cuda.graph(g, stream=cap):
            for s in side:
                s.wait_stream(cap)
            for k, i in enumerate(order):
                s = side[k % self.n_streams]
                with torch.cuda.stream(s):
                    for _ in range(n_updates):
                        self.items[i]._iter()
            for s in side:
                cap.wait_stream(s)
        cur.wait_stream(cap)
        self._graph, self._n = g, n_updates
        return g

    def run(self, n_updates: int):
        if self._graph is None or self._n != n_updates:
            self.capture(n_updates)
        self._graph.replay()

    def plain(self, n_updates: int):
        for it in self.items:
            for _ in range(n_updates):
                it._iter()

    def images(self):
        return [it.x for it in self.items]


class PersistentSIRT2D:
    """All problems' SIRT updates in one persistent launch (see the module
    docstring).  problems: dicts with SIRT2D's arguments."""

    def __init__(self, problems, device=None, storage="fp32"):
        if storage not in STORAGE:
            raise ValueError(f"storage must be one of {sorted(STORAGE)}")
        self.dev = device or torch.device("cuda", torch.cuda.current_device())
        self.storage = storage
        self.items = [SIRT2D(device=self.dev, **p) for p in problems]
        bx, by = STORAGE[storage] & 1, STORAGE[storage] & 2
        self._x = [it.x.to(torch.bfloat16) if bx else it.x for it in self.items]
        self._xT = [it.xT.to(torch.bfloat16) if bx else it.xT for it in self.items]
        self._y = [it.y.to(torch.bfloat16) if by else it.y for it in self.items]
        arr = (Sirt2DProblem * len(self.items))()
        for k, it in enumerate(self.items):
            arr[k] = Sirt2DProblem(it.g, self._y[k].data_ptr(), it.inv_ws.data_ptr(),
                                   it.inv_wi.data_ptr(), it.trig.data_ptr(), self._x[k].data_ptr(),
                                   self._xT[k].data_ptr(), it.r.data_ptr(), it.ws.data_ptr(),
                                   float(np.float32(it.gamma)), 0)
        self._host = arr
        raw = bytes(memoryview(arr).cast("B"))
        self._probs = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(self.dev)
        L = load()
        n = len(self.items)
        nf, nt, nb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        call("vg_sirt2d_batch_items", ctypes.addressof(arr), n, None, ctypes.byref(nf), None,
             ctypes.byref(nt), None, ctypes.byref(nb))
        fp = np.empty((nf.value, 2), np.int32)
        tab = np.empty((nt.value, 2), np.int32)
        bp = np.empty((nb.value, 2), np.int32)
        call("vg_sirt2d_batch_items", ctypes.addressof(arr), n, fp.ctypes.data, ctypes.byref(nf),
             tab.ctypes.data, ctypes.byref(nt), bp.ctypes.data, ctypes.byref(nb))
        # largest items first: forward projection ~ lines x bins, tables ~ bins,
        # back projection tiles ~ views
        g = [it.g for it in self.items]
        cf = np.array([max(g[i].nx, g[i].ny) * min(g[i].nu, 768) for i in fp[:, 0]])
        ct = np.array([g[i].nu for i in tab[:, 0]])
        cb = np.array([g[i].na for i in bp[:, 0]])
        self._fp = torch.from_numpy(fp[np.argsort(-cf, kind="stable")].copy()).to(self.dev)
        self._tab = torch.from_numpy(tab[np.argsort(-ct, kind="stable")].copy()).to(self.dev)
        self._bp = torch.from_numpy(bp[np.argsort(-cb, kind="stable")].copy()).to(self.dev)
        self.max_nd = max(max(x.nx, x.ny) for x in g)
        self._ctrl = torch.zeros(10, dtype=torch.int32, device=self.dev)
        self._counters = torch.zeros(3 * n, dtype=torch.int32, device=self.dev)
        self._cancel = torch.zeros(1, dtype=torch.int32).pin_memory()
        self.grid_blocks = 0
        del L

    def reset(self, x0=1e-5):
        for k, it in enumerate(self.items):
            self._x[k].fill_(float(np.float32(x0)))
            self._xT[k].fill_(float(np.float32(x0)))

    def cancel(self):
        """Ask a running launch to stop at the end of its current update."""
        self._cancel[0] = 1

    def run(self, n_updates: int, budget_s: float = 0.0, wait: bool = True):
        """n_updates SIRT updates of every problem in one launch.  With
        wait, returns (status, updates done) once the run has ended."""
        self._cancel[0] = 0
        gb = ctypes.c_int(0)
        call("vg_sirt2d_batch_run", self._probs.data_ptr(), len(self.items), self.max_nd,
             self._fp.data_ptr(), self._fp.shape[0], self._tab.data_ptr(), self._tab.shape[0],
             self._bp.data_ptr(), self._bp.shape[0], int(n_updates), STORAGE[self.storage],
             self._cancel.data_ptr(), ctypes.c_ulonglong(int(budget_s * 1e9)),
             self._ctrl.data_ptr(), self._counters.data_ptr(), _core.stream(self.dev),
             ctypes.byref(gb))
        self.grid_blocks = gb.value
        if wait:
            return self.result()
        return None

    def result(self):
        """(status name, updates done) of the last run (synchronises)."""
        c = self._ctrl.cpu().numpy()   # (next lo, next hi, status, done, ...)
        return STATUS.get(int(c[2]), str(int(c[2]))), int(c[3])

    def images(self):
        return [x.float() for x in self._x]
