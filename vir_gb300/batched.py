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
"""
from __future__ import annotations

import torch

from .reconstruction import SIRT2D


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
