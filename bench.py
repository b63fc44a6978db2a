"""Benchmark: SIRT iterations/s of the 2D fan-beam distance-driven
reconstruction (512^2 random-ellipse phantom, 720 views over 2 pi, 768 bins of
1.2 mm, DSO 500 mm, DSD 1000 mm, 0.9 mm pixels, Poisson noise at 1e5
photons/ray), one step = 100 SIRT updates of one reconstruction, run as one
CUDA graph.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  Under torchrun with N > 1 every rank runs an
independent replica (the path has no exchange step); value = all ranks'
updates / max-over-ranks time.  `--impl reference` times vir's own CPU
algorithm for the same workload (the FP64 C restatement of dd.py and
sirt_dd.py, all host threads) on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "SIRT iter/s and fwd+back GUPS vs plain FP32 at matched RMSE; % HBM peak"
WORKLOAD = dict(n=512, n_ell=10, seed=2026, d_pix=0.9, na=720, nu=768, du=1.2, DSO=500.0,
                DSD=1000.0, I0=1e5, updates_per_step=100)
L2_FLUSH_BYTES = 256 << 20


def workload_desc():
    w = WORKLOAD
    return (f"2D fan-beam distance-driven SIRT: {w['n']}x{w['n']} random-ellipse phantom "
            f"({w['n_ell']} ellipses, seed {w['seed']}), {w['na']} views over 2pi, {w['nu']} bins "
            f"of {w['du']} mm, DSO {w['DSO']} mm, DSD {w['DSD']} mm, {w['d_pix']} mm pixels, "
            f"Poisson noise {w['I0']:.0e} photons/ray; {w['updates_per_step']} SIRT updates per step")


def make_inputs():
    from vir_gb300 import phantoms as ph
    w = WORKLOAD
    img, e = ph.ellipse_phantom(w["n"], w["n_ell"], seed=w["seed"], d_pix=w["d_pix"])
    angs = np.linspace(0, 2 * np.pi, w["na"], endpoint=False)
    p = ph.sino_fan(e, angs, w["nu"], w["DSO"], w["DSD"], du=w["du"])
    y = ph.poisson_noise(p, w["I0"], seed=w["seed"])
    return img, angs, y


def load_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, burst copy)"
    return 6800.0, "fallback 6.8 TB/s"


def load_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "dd2d_fan_c2.json")
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh)
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def job_rate(local_ms, world, units_per_rank, dist=None, dev=None):
    """Whole-job rate of independent replicas: every rank processes
    units_per_rank units; the job takes the slowest rank's time (max over
    ranks through the process group when there is one).  Returns (max_ms,
    world * units_per_rank / max seconds)."""
    total_ms = float(local_ms)
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        dist.barrier()
    return total_ms, world * units_per_rank / (total_ms / 1e3)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_sirt_iteration_rate(img_shape, angs, y, n_iter=1, want_x=False):
    """vir's algorithm on the host (FP64 C restatement, all threads): seconds
    per SIRT update on the full workload (and the iterate after n_iter
    updates when want_x)."""
    from oracle import oracle as orc
    w = WORKLOAD
    fp = lambda x: orc.dd_fp_fan_2d(x, angs, w["nu"], w["DSO"], w["DSD"], du=w["du"],
                                    d_pix=w["d_pix"])
    bp = lambda s: orc.dd_bp_fan_2d(s, angs, img_shape, w["DSO"], w["DSD"], du=w["du"],
                                    d_pix=w["d_pix"])
    W_sino = fp(np.ones(img_shape, np.float32))
    W_img = bp(np.ones(y.shape, np.float32))
    t0 = time.perf_counter()
    x = orc.sirt(y, fp, bp, img_shape, iters=n_iter + 1, W_sino=W_sino, W_img=W_img)
    dt = time.perf_counter() - t0
    if want_x:
        return dt / n_iter, orc.num_threads(), x
    return dt / n_iter, orc.num_threads()


def arm_config(world):
    """The `config` record both arms print (same keys and values at the same N)."""
    return {"workload": workload_desc(), "parallelism": f"replicas x{world}",
            "l2": "flushed between steps (256 MiB write); inputs 3.3 MB are L2-resident "
                  "within a step", "graph": "100 updates captured as one CUDA graph"}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    img, angs, y = make_inputs()
    for _ in range(args.warmup):
        cpu_sirt_iteration_rate(img.shape, angs, y, 1)
    times = []
    cores = 1
    for _ in range(args.steps):
        dt, cores = cpu_sirt_iteration_rate(img.shape, angs, y, 1)
        times.append(dt)
    sec = statistics.median(times)
    val = 1.0 / sec
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "iter/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": arm_config(world),
            "cpu_baseline": {"value": val, "unit": "iter/s", "cores": cores, "kind": "port",
                             "sample": "1 SIRT update (FP + BP) of the full 512^2 x 720-view "
                                       "workload per step, median over steps"},
            "e2e": {"value": val, "unit": "iter/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_kernels_only(n):
    """Launch the SIRT iteration's kernels n times (for ncu captures)."""
    import torch
    from vir_gb300 import reconstruction as rc
    w = WORKLOAD
    img, angs, y = make_inputs()
    sirt = rc.SIRT2D(y, angs, img.shape, geom="fan", DSO=w["DSO"], DSD=w["DSD"], du=w["du"],
                     d_pix=w["d_pix"])
    for _ in range(n):
        sirt.run(1, graph=False)
    torch.cuda.synchronize()
    print(json.dumps({"kernels_only": n, "ok": True}))
    return 0


# ---- the other configurations (not the default line) -----------------------

EXTRA = {
    "c1": "2D parallel Siddon FP + gather BP: 256x256 random-ellipse phantom, 1 mm pixels, "
          "180 views over pi, 367 bins of 1 mm",
    "c3": "batched SIRT: 64 parallel/fan problems (seed 3), sides in {128,256,512,1024}, "
          "90-1440 views, 1.5x detectors; 50 updates: one persistent launch (work queue, "
          "float32 or bfloat16 storage), one CUDA graph of per-problem chains, one launch per step",
    "c4": "3D cone DD and separable-footprint FP + BP, FDK: 512^3 volume of 20 random "
          "ellipsoids, 0.5 mm voxels, 720 views over 2pi, 1024x768 detector at 0.8 mm, DSO 600 mm, "
          "DSD 1100 mm",
    "c5ad": "differentiable cone projector at C5 (256^3 random ellipsoids, 360 views, 512x384 at "
            "1.6 mm, DSO 600, DSD 1100): 200 Adam steps on ||Ax-y||^2 + 1e-3 TV(x) through "
            "autograd.Project against vir's SIRT rule, compared at matched RMSE",
    "c5": "3D cone DD and separable-footprint FP + BP: 256^3 volume of 20 random ellipsoids, "
          "1 mm voxels, 360 views over 2pi, 512x384 detector at 1.6 mm, DSO 600 mm, DSD 1100 mm",
    "bh": "beam-hardening pre-correction of a 720 x 1024 x 768 float32 logged sinogram (the "
          "C4 detector): water polynomial with np.polyfit coefficients (float64 result) and with "
          "Python-float coefficients (float32 result), 1000-entry spectrum table (interp1d), "
          "4001-entry lookup table (np.interp); each result in numpy's dtype, bit for bit",
    "rows": "projector rows without a workload of their own, at the C2 fan geometry (512^2, "
            "720 views, 768 bins of 1.2 mm, DSO 500, DSD 1000, 0.9 mm pixels), the C1 parallel "
            "geometry (256^2, 180 views, 367 bins) or the C5 cone geometry (256^3, 360 views, "
            "512x384): separable footprint (fan, parallel rectangle), ray-driven AW and Joseph, "
            "pixel-driven, Siddon ray lists (siddons + list FP/BP) and 10 TV-PDHG iterations",
    "helical": "helical rebinning front-end: 1440 helical views (2 rotations, 64 rows x 1024 "
               "columns, 16 rows per rotation of table travel) rebinned to 720 axial angles x "
               "128 slices (sino_hel2axl), the axial sinogram resampled back to the helical views "
               "(sino_axl2hel), and a 128^3 phantom projected over 180 helical views "
               "(forward_project_phantom)",
    "square": "translational square geometry DD FP + BP (dd_fp_square / dd_bp_square) at the "
              "reference's SIRT-script size (64^3, 96x10 sources, 129x64 cells) and at its "
              "nice.py size (250^3, 650x10 sources, 961x121 cells)",
}


def _event_ms(fn, reps, stream):
    import torch
    fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return statistics.median(out)


def orc_mod():
    from oracle import oracle
    return oracle


def _cpu_port_ms(fp, bp):
    """The FP64 C restatement of the same pair on all host threads, once."""
    t0 = time.perf_counter()
    fp()
    t1 = time.perf_counter()
    bp()
    t2 = time.perf_counter()
    return {"fp_ms": (t1 - t0) * 1e3, "bp_ms": (t2 - t1) * 1e3, "cores": orc_mod().num_threads(),
            "kind": "port"}


def _roof(units, ms, peak, compulsory=None):
    """Algorithmic-byte roofline (4 B per voxel-view update); with
    `compulsory` (the launch's unique input + output bytes) also the rate
    and fraction of those, the true lower bound of its traffic."""
    gbs = 4.0 * units / (ms / 1e3) / 1e9
    r = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
         "algorithmic_bytes_per_launch": 4.0 * units}
    if compulsory is not None:
        cg = compulsory / (ms / 1e3) / 1e9
        r["compulsory"] = {"bytes_per_launch": compulsory, "achieved": cg, "frac": cg / peak}
    return r


def storage_error(probs, dev, n_check=2, iters=50):
    """Final-iterate error against the FP64 oracle's SIRT, relative
    (||x - x64|| / ||x64||), for each storage of the persistent batched
    kernel: float32, bfloat16 measured sinogram, bfloat16 iterate, both (the
    kernel reads and writes bfloat16, arithmetic float32).  The smallest
    problems of the set are used so the oracle finishes in seconds."""
    from oracle import oracle as orc
    from vir_gb300.batched import PersistentSIRT2D
    order = sorted(range(len(probs)), key=lambda i: probs[i]["img_shape"][0] * probs[i]["sino"].shape[0])
    out = []
    for i in order[:n_check]:
        p = probs[i]
        kw = dict(du=p["du"], d_pix=p["d_pix"])
        if p["geom"] == "fan":
            fp = lambda x: orc.dd_fp_fan_2d(x, p["ang_arr"], p["sino"].shape[1], p["DSO"], p["DSD"], **kw)
            bp = lambda y: orc.dd_bp_fan_2d(y, p["ang_arr"], p["img_shape"], p["DSO"], p["DSD"], **kw)
        else:
            fp = lambda x: orc.dd_fp_par_2d(x, p["ang_arr"], p["sino"].shape[1], **kw)
            bp = lambda y: orc.dd_bp_par_2d(y, p["ang_arr"], p["img_shape"], **kw)
        x64 = orc.sirt(p["sino"], fp, bp, p["img_shape"], iters=iters)
        nrm = np.linalg.norm(x64)
        rec = {"problem": i, "side": int(p["img_shape"][0]), "views": int(p["sino"].shape[0]),
               "geom": p["geom"], "updates": iters - 1}
        for st in ("fp32", "bf16y", "bf16x", "bf16"):
            b = PersistentSIRT2D([p], device=dev, storage=st)
            b.run(iters - 1)
            x = b.images()[0].cpu().numpy()
            rec[st + "_rel"] = float(np.linalg.norm(x - x64) / nrm)
        out.append(rec)
    return out


def c3_summary(dev, stream, check=True):
    """The batched-SIRT configuration (64 parallel/fan problems of seed 3, 50
    updates): one CUDA graph of per-problem chains, one launch per step (the
    plain FP32 path), one persistent launch in each storage mode; its
    iterates against the graph's, and (check) the final-iterate error of each
    storage mode against the FP64 oracle's SIRT on the two smallest problems."""
    import torch
    from vir_gb300.batched import BatchedSIRT2D, PersistentSIRT2D
    from vir_gb300.workloads import batched_problems
    probs = batched_problems(64, seed=3)
    b = BatchedSIRT2D(probs, n_streams=16)
    res = {}
    for mode in ("graph", "plain"):
        b.reset()
        res[mode] = _event_ms(lambda: b.run(50) if mode == "graph" else b.plain(50), 1, stream)
    b.reset()
    b.run(50)
    xg = [x.clone() for x in b.images()]
    del b
    torch.cuda.empty_cache()
    pers = {}
    for st in ("fp32", "bf16y", "bf16x", "bf16"):
        pb = PersistentSIRT2D(probs, device=dev, storage=st)
        pb.run(1)
        pb.reset()
        pers[st] = _event_ms(lambda: pb.run(50, wait=False), 1, stream)
        if st == "fp32":
            pb.reset()
            status = pb.run(50)
            diff = max(float((a - c).abs().max() / c.abs().max()) for a, c in zip(pb.images(), xg))
            grid = pb.grid_blocks
        del pb
        torch.cuda.empty_cache()
    units = sum(p["sino"].shape[0] * p["img_shape"][0] * p["img_shape"][1] for p in probs)
    return {"metric": "batched SIRT iter/s (50 updates x 64 problems)",
            "graph_ms": res["graph"], "plain_ms": res["plain"],
            "persistent_ms": pers, "persistent_status": status,
            "persistent_grid_blocks": grid,
            "persistent_vs_graph_max_rel_diff": diff,
            "speedup_vs_plain": {"graph": res["plain"] / res["graph"],
                                 **{"persistent_" + k: res["plain"] / v for k, v in pers.items()}},
            "fwd_back_gups_graph": 2 * 50 * units / (res["graph"] / 1e3) / 1e9,
            "fwd_back_gups_persistent": 2 * 50 * units / (pers["fp32"] / 1e3) / 1e9,
            "storage_error": storage_error(probs, dev) if check else None}


def run_workload(args):
    """One JSON line for a configuration other than the default C2 line:
    per-kernel CUDA-event times (median of --steps after --warmup), GUPS and
    the algorithmic-byte roofline.  With --kernels-only N the projector pair
    is just launched N times (for ncu captures): c4 / c5 then also the
    separable-footprint pair, c3 runs N persistent launches of 2 updates."""
    import torch
    from vir_gb300 import phantoms as ph
    from vir_gb300.sys_mat import dd
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    peak, _ = load_peaks()
    reps = max(args.steps, 1)
    wl = args.workload
    line = {"workload": wl, "config": EXTRA[wl], "n_gpus": 1, "dtype": "f32",
            "data": "synthetic"}
    if wl == "c1":
        from vir_gb300.sys_mat import fp_2d_par as f2
        img, _ = ph.ellipse_phantom(256, 10, seed=2025, d_pix=1.0)
        angs = np.linspace(0, np.pi, 180, endpoint=False)
        x = torch.from_numpy(img).to(dev)
        y = f2.siddons_fp_2d(x, angs, 367, 1.0, 1.0)
        fp = lambda: f2.siddons_fp_2d(x, angs, 367, 1.0, 1.0)
        bp = lambda: f2.siddons_bp_2d(y, angs, (256, 256), 1.0, 1.0)
        units = 180 * 256 * 256
        compulsory = 4.0 * (256 * 256 + 180 * 367)  # image + sinogram
        # intersections (kept segments) of the C1 rays, from the walk's trace mode
        from vir_gb300 import _core
        from vir_gb300._lib import call
        trig = _core.trig_cache.get(angs, None, dev)
        cnt = torch.empty((180, 367), dtype=torch.int32, device=dev)
        hsh = torch.empty((180, 367), dtype=torch.int64, device=dev)
        tln = torch.empty((180, 367), dtype=torch.float64, device=dev)
        call("vg_siddon2d_trace", 256, 256, _core.ptr(trig), 180, 367, 1.0, 1.0, _core.ptr(cnt),
             _core.ptr(hsh), _core.ptr(tln), _core.stream(dev))
        n_isect = int(cnt.sum().item())
        yh = y.cpu().numpy()
        line["cpu_port"] = _cpu_port_ms(lambda: orc_mod().siddons_fp_2d(img, angs, 367, 1.0, 1.0),
                                        lambda: orc_mod().siddons_bp_2d(yh, angs, (256, 256), 1.0, 1.0))
    elif wl in ("c4", "c5"):
        n, na, nu, nv, dp, du = ((512, 720, 1024, 768, 0.5, 0.8) if wl == "c4"
                                 else (256, 360, 512, 384, 1.0, 1.6))
        e = ph.random_ellipsoids(20, fov_radius=n * dp / 2, seed=2027)
        x = ph.rasterize3d_device(e, n, dp, device=dev)
        angs = np.linspace(0, 2 * np.pi, na, endpoint=False)
        kw = dict(du=du, dv=du, su=0.0, sv=0.0, d_pix=dp)
        y = dd.dd_fp_cone_3d(x, angs, nu, nv, 600.0, 1100.0, **kw)
        fp = lambda: dd.dd_fp_cone_3d(x, angs, nu, nv, 600.0, 1100.0, **kw)
        bp = lambda: dd.dd_bp_cone_3d(y, angs, (n, n, n), 600.0, 1100.0, **kw)
        units = na * n ** 3
        compulsory = 4.0 * (n ** 3 + na * nu * nv)  # volume + sinogram
    elif wl == "square":
        cases = {"script": (64, 64, 129, 64, 96, 10, 40.0, 72.0,
                            dict(du=1.0, dv=1.0, dsrc_p=0.5, dsrc_z=0.5, su=0.0, sv=32.0,
                                 ssrc_p=0.0, ssrc_z=-27.0, d_pix=1.0)),
                 "nice": (250, 250, 961, 121, 650, 10, 141.381, 261.381,
                          dict(du=2.61381, dv=2.61381, dsrc_p=.48, dsrc_z=.48, su=0.0,
                               sv=158.13554, ssrc_p=0.0, ssrc_z=-74.4, d_pix=.96))}
        out = {}
        if args.kernels_only:  # profiling aid: the script-size case only
            cases = {"script": cases["script"]}
        for name, (n, nz, nu, nv, nsp, nsz, DSO, DSD, kw) in cases.items():
            e = ph.random_ellipsoids(10, fov_radius=n * kw["d_pix"] / 2, seed=2028)
            x = ph.rasterize3d_device(e, n, kw["d_pix"], device=dev)
            y = dd.dd_fp_square(x, nu, nv, nsp, nsz, DSO, DSD, **kw)
            fp = lambda: dd.dd_fp_square(x, nu, nv, nsp, nsz, DSO, DSD, **kw)
            bp = lambda: dd.dd_bp_square(y, (n, n, nz), DSO, DSD, **kw)
            if args.kernels_only:
                for _ in range(args.kernels_only):
                    fp(); bp()
                continue
            r = 1 if name == "nice" else reps
            t_fp, t_bp = _event_ms(fp, r, stream), _event_ms(bp, r, stream)
            units = 4 * nsp * nsz * n * n * nz
            out[name] = {"kernel_ms": {"fp": t_fp, "bp": t_bp},
                         "fwd_back_gups": 2 * units / ((t_fp + t_bp) / 1e3) / 1e9,
                         "roofline_fp": _roof(units, t_fp, peak),
                         "roofline_bp": _roof(units, t_bp, peak)}
            if name == "script":
                xh, yh = x.cpu().numpy(), y.cpu().numpy()
                out[name]["cpu_port"] = _cpu_port_ms(
                    lambda: orc_mod().dd_fp_square(xh, nu, nv, nsp, nsz, DSO, DSD, **kw),
                    lambda: orc_mod().dd_bp_square(yh, (n, n, nz), DSO, DSD, **kw))
            del x, y
            torch.cuda.empty_cache()
        if not args.kernels_only:
            line["cases"] = out
            print(json.dumps(line), flush=True)
        return 0
    elif wl == "bh":
        from vir_gb300 import beamhard as bh
        na, nu, nv = 720, 1024, 768
        g = torch.Generator(device=dev).manual_seed(5)
        li = torch.rand((na, nu, nv), device=dev, generator=g) * 7.0
        e = np.arange(20.0, 121.0)
        cnt = np.exp(-0.5 * ((e - 62.0) / 18.0) ** 2)
        water = lambda m, x: 0.17 + 2500.0 * np.asarray(x, np.float64) ** -3.0  # synthetic
        ae = float(water("H2O", [np.average(e, weights=cnt)])[0])
        coefs = np.polyfit(np.linspace(0, 10, 50), np.linspace(0, 10, 50) ** 1.1, 2)
        lut = 1.0 + 0.05 * np.sin(np.linspace(0, 3, 4001))
        pyc = [float(c) for c in coefs]
        runs = {"poly": lambda: bh.beamhard_cor(li, coefs, 0.2),
                "poly_f32": lambda: bh.beamhard_cor(li, pyc, 0.2),
                "table": lambda: bh.beamhard_cor_table(li, e, cnt, None, ae, mixatten=water),
                "lut": lambda: bh.beamhard_cor2(li, lut, 0.2)}
        n = li.numel()
        out = {}
        sample = li[:8].cpu().numpy()  # 1/90 of the sinogram for the CPU path
        orc = orc_mod()
        cpu = {"poly": lambda: orc.bh_poly(sample, coefs, 0.2),
               "poly_f32": lambda: orc.bh_poly(sample, pyc, 0.2),
               "table": lambda: orc.bh_table(sample, e, cnt, ae, water("H2O", e)),
               "lut": lambda: orc.bh_lut(sample, lut, 0.2)}
        for k, fn in runs.items():
            nbytes = (8.0 if k == "poly_f32" else 12.0) * n  # float32 in; float32 / float64 out
            ms = _event_ms(fn, reps, stream)
            gbs = nbytes / (ms / 1e3) / 1e9
            t0 = time.perf_counter()
            cpu[k]()
            cpu_ms = (time.perf_counter() - t0) * 1e3 * (n / sample.size)
            out[k] = {"ms": ms, "gsamples_per_s": n / (ms / 1e3) / 1e9,
                      # float64 results replay numpy's float64 arithmetic: the FP64 pipe,
                      # not HBM, bounds those cases; the HBM fraction is shown beside it
                      "roofline": {"bound": "hbm" if k == "poly_f32" else "fp64 pipe",
                                   "achieved": gbs, "peak": peak, "unit": "GB/s",
                                   "frac": gbs / peak, "bytes_per_launch": nbytes},
                      "cpu_numpy_ms_full_size": cpu_ms}
        line.update({"cases": out, "cpu_baseline": {
            "kind": "port", "cores": 1,
            "sample": "the oracle's numpy/scipy restatement of beamhard.py:16-47 and "
                      "beamhard_test.py:26-27 on 8 of 720 views, scaled to the full sinogram"}})
        print(json.dumps(line), flush=True)
        return 0
    elif wl == "rows":
        from vir_gb300 import phantoms as ph
        from vir_gb300 import tv
        from vir_gb300.projection import proj
        from vir_gb300.sys_mat import fp_2d_par as f2, pd as pdm, rd, siddon, sp
        orc = orc_mod()
        out = {}

        def case(name, fp, bp, units, cpu_fp, cpu_bp, cpu_scale, sample):
            if args.kernels_only:  # profiling aid: launch the pair, no timing, no CPU port
                for _ in range(args.kernels_only):
                    fp(); bp()
                out[name] = {}
                return
            t_fp, t_bp = _event_ms(fp, reps, stream), _event_ms(bp, reps, stream)
            t0 = time.perf_counter()
            cpu_fp()
            t1 = time.perf_counter()
            cpu_bp()
            t2 = time.perf_counter()
            out[name] = {"kernel_ms": {"fp": t_fp, "bp": t_bp},
                         "fwd_back_gups": 2 * units / ((t_fp + t_bp) / 1e3) / 1e9,
                         "roofline_fp": _roof(units, t_fp, peak), "roofline_bp": _roof(units, t_bp, peak),
                         "cpu_port_ms": {"fp": (t1 - t0) * 1e3 * cpu_scale,
                                         "bp": (t2 - t1) * 1e3 * cpu_scale,
                                         "cores": orc.num_threads(), "sample": sample}}

        # C2 fan geometry
        img, _ = ph.ellipse_phantom(512, 10, seed=2026, d_pix=0.9)
        x2 = torch.from_numpy(img).to(dev)
        a2 = np.linspace(0, 2 * np.pi, 720, endpoint=False)
        geo = (500.0, 1000.0)
        y2 = torch.rand((720, 768), device=dev)
        yh = y2.cpu().numpy()
        s24 = "24 of 720 views, scaled"
        case("sf_fan", lambda: sp.sf_fp_fan_2d(x2, a2, 768, *geo, du=1.2, d_pix=0.9),
             lambda: sp.sf_bp_fan_2d(y2, a2, (512, 512), *geo, du=1.2, d_pix=0.9), 720 * 512 * 512,
             lambda: orc.sf_fp_fan_2d(img, a2[:24], 768, *geo, du=1.2, d_pix=0.9),
             lambda: orc.sf_bp_fan_2d(yh[:24], a2[:24], (512, 512), *geo, du=1.2, d_pix=0.9), 30, s24)
        for tag, jos in (("aw_fan", False), ("joseph_fan", True)):
            case(tag, lambda: rd.aw_fp_fan_2d(x2, a2, 768, *geo, du=1.2, d_pix=0.9, joseph=jos),
                 lambda: rd.aw_bp_fan_2d(y2, a2, (512, 512), *geo, du=1.2, d_pix=0.9, joseph=jos),
                 720 * 512 * 512,
                 lambda: orc.aw_fp_fan_2d(img, a2[:24], 768, *geo, du=1.2, d_pix=0.9, joseph=jos),
                 lambda: orc.aw_bp_fan_2d(yh[:24], a2[:24], (512, 512), *geo, du=1.2, d_pix=0.9,
                                          joseph=jos), 30, s24)
        from vir_gb300 import reconstruction as rcn
        t_fbp = _event_ms(lambda: rcn.fbp_2d(y2, a2, (512, 512), geom="fan", DSO=500.0, DSD=1000.0,
                                             du=1.2, d_pix=0.9), reps, stream)
        out["fbp_fan"] = {"ms": t_fbp, "note": "C2 geometry: cosine weight, ramp filter (FFT "
                                               "route), 1/U^2-weighted back projection"}
        case("pd_fan", lambda: pdm.pd_fp_fan_2d(x2, a2, 768, *geo, du=1.2, d_pix=0.9),
             lambda: pdm.pd_bp_fan_2d(y2, a2, (512, 512), *geo, du=1.2, d_pix=0.9), 720 * 512 * 512,
             lambda: orc.pd_fp_fan_2d(img, a2[:24], 768, *geo, du=1.2, d_pix=0.9),
             lambda: orc.pd_bp_fan_2d(yh[:24], a2[:24], (512, 512), *geo, du=1.2, d_pix=0.9), 30, s24)
        # C1 parallel geometry
        img1, _ = ph.ellipse_phantom(256, 10, seed=2025, d_pix=1.0)
        x1 = torch.from_numpy(img1).to(dev)
        a1 = np.linspace(0, np.pi, 180, endpoint=False)
        y1 = torch.rand((180, 367), device=dev)
        y1h = y1.cpu().numpy()
        case("sf_par_rect", lambda: f2.separable_footprint_fp_2d(x1, a1, 367, 1.0, 1.0),
             lambda: f2.separable_footprint_bp_2d(y1, a1, (256, 256), 1.0, 1.0), 180 * 256 * 256,
             lambda: orc.separable_footprint_fp_2d(img1, a1, 367, 1.0, 1.0),
             lambda: orc.separable_footprint_bp_2d(y1h, a1, (256, 256), 1.0, 1.0), 1,
             "all 180 views")
        # C1 Siddon ray lists: 66,060 rays through a 256 x 256 x 1 grid
        dets = np.arange(367) - 183.0
        src = np.zeros((180, 367, 3))
        trg = np.zeros((180, 367, 3))
        for i, v in enumerate(a1):
            c, s_ = np.cos(v), np.sin(v)
            R = np.array([[c, s_], [-s_, c]])
            src[i, :, :2] = np.stack([np.full(367, -36700.0), dets], -1) @ R
            trg[i, :, :2] = np.stack([np.full(367, 36700.0), dets], -1) @ R
        t_sd = _event_ms(lambda: siddon.siddons_device(src, trg, (256, 256, 1), 1.0), 1, stream)
        ind, ln, off, _, _ = siddon.siddons_device(src, trg, (256, 256, 1), 1.0)
        xv = x1.reshape(-1)
        yl = torch.rand(off.numel() - 1, device=dev)
        ih, lh, oh = ind.cpu().numpy(), ln.cpu().numpy(), off.cpu().numpy()
        case("siddon_lists", lambda: proj.list_fp_device(xv, ind, ln, off),
             lambda: proj.list_bp_device(yl, ind, ln, off, xv.numel()), ind.numel(),
             lambda: orc.list_fp(img1, ih, lh, oh),
             lambda: orc.list_bp(yl.cpu().numpy(), ih, lh, oh, xv.numel()), 1, "the whole list")
        out["siddon_lists"].update({"entries": int(ind.numel()), "rays": int(off.numel() - 1),
                                    "siddons_ms": t_sd,
                                    "units": "list entries (voxel-ray pairs)"})
        # C5 cone geometry
        n, na3, nu3, nv3 = 256, 360, 512, 384
        e3 = ph.random_ellipsoids(20, fov_radius=n / 2, seed=2027)
        x3 = ph.rasterize3d_device(e3, n, 1.0, device=dev)
        a3 = np.linspace(0, 2 * np.pi, na3, endpoint=False)
        kw3 = dict(du=1.6, dv=1.6, su=0.0, sv=0.0, d_pix=1.0)
        y3 = torch.rand((na3, nu3, nv3), device=dev)
        x3h, y3h = x3.cpu().numpy(), y3[:2].cpu().numpy()
        s2 = "2 of 360 views, scaled"
        for tag, jos in (("aw_cone", False), ("joseph_cone", True)):
            case(tag, lambda: rd.aw_fp_cone_3d(x3, a3, nu3, nv3, 600.0, 1100.0, joseph=jos, **kw3),
                 lambda: rd.aw_bp_cone_3d(y3, a3, (n, n, n), 600.0, 1100.0, joseph=jos, **kw3),
                 na3 * n ** 3,
                 lambda: orc.aw_fp_cone_3d(x3h, a3[:2], nu3, nv3, 600.0, 1100.0, joseph=jos, **kw3),
                 lambda: orc.aw_bp_cone_3d(y3h, a3[:2], (n, n, n), 600.0, 1100.0, joseph=jos, **kw3),
                 180, s2)
        case("pd_cone", lambda: pdm.pd_fp_cone_3d(x3, a3, nu3, nv3, 600.0, 1100.0, **kw3),
             lambda: pdm.pd_bp_cone_3d(y3, a3, (n, n, n), 600.0, 1100.0, **kw3), na3 * n ** 3,
             lambda: orc.pd_fp_cone_3d(x3h, a3[:2], nu3, nv3, 600.0, 1100.0, **kw3),
             lambda: orc.pd_bp_cone_3d(y3h, a3[:2], (n, n, n), 600.0, 1100.0, **kw3), 180, s2)
        del x3, y3
        torch.cuda.empty_cache()
        # TV-PDHG on the C2 fan DD pair: 10 iterations (each one FP and one BP)
        from vir_gb300.sys_mat import dd
        yt = dd.dd_fp_fan_2d(x2, a2, 768, *geo, du=1.2, d_pix=0.9)
        fpf = lambda z: dd.dd_fp_fan_2d(z, a2, 768, *geo, du=1.2, d_pix=0.9)
        bpf = lambda z: dd.dd_bp_fan_2d(z, a2, (512, 512), *geo, du=1.2, d_pix=0.9)
        t_tv = _event_ms(lambda: tv.pdhg(yt, fpf, bpf, (512, 512), lam=0.01, iters=10), 1, stream)
        out["tv_pdhg"] = {"ms_10_iterations": t_tv, "iter_per_s": 10 / (t_tv / 1e3),
                          "note": "each iteration: one DD fan FP, one BP and the three fused "
                                  "elementwise kernels; set-up (A1, At1) inside the timed call"}
        line.update({"cases": out})
        print(json.dumps(line), flush=True)
        return 0
    elif wl == "helical":
        from vir_gb300 import _core
        from vir_gb300 import trajectory as tr
        from vir_gb300._lib import call
        g = torch.Generator(device=dev).manual_seed(6)
        nvh, nr, nc = 1440, 64, 1024
        G = tr.Geom(nViews=nvh, coverage=4 * np.pi, zTran=16.0)
        sinoH = torch.rand((nvh, nr, nc), device=dev, generator=g)
        angs = np.linspace(0, 2 * np.pi, 720, endpoint=False)
        Z = np.linspace(-15.5, 15.5, 128)
        pp, wp, pn, wn = tr._tables(G, [Z] * angs.size, angs, nr)
        shape = (angs.size, Z.size, nc)
        out = {}
        ms = _event_ms(lambda: (tr._gather(sinoH, pp, wp, shape), tr._gather(sinoH, pn, wn, shape)),
                       reps, stream)
        n_out = 2 * angs.size * Z.size * nc
        t0 = time.perf_counter()
        tr.sino_hel2axl(sinoH, G, angs, Z)
        torch.cuda.synchronize()
        call_ms = (time.perf_counter() - t0) * 1e3
        gbs = 12.0 * n_out / (ms / 1e3) / 1e9  # two float32 rows read, one written per sample
        hs = sinoH[:, :, :64].cpu().numpy()   # 1/16 of the columns for the CPU path
        t0 = time.perf_counter()
        orc_mod().rebin_rows(hs, pp, wp, shape[:2] + (64,))
        orc_mod().rebin_rows(hs, pn, wn, shape[:2] + (64,))
        cpu_ms = (time.perf_counter() - t0) * 1e3 * nc / 64
        out["hel2axl"] = {"kernel_ms": ms, "call_ms": call_ms, "gsamples_per_s": n_out / ms / 1e6,
                          "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                                       "frac": gbs / peak, "bytes_per_launch": 12.0 * n_out},
                          "cpu_numpy_ms_full_size": cpu_ms}
        sinoA = torch.rand((720, 128, nc), device=dev, generator=g)
        vH = np.linspace(0, 4 * np.pi, nvh, endpoint=False)
        idx, zz, wrap, _ = tr.axl2hel_index(720, 128, nr, vH, 720, 0.5)  # 32 rows per rotation
        ti, tz, tw = (torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in (idx, zz, wrap))
        res = torch.empty((nvh, nr, nc), device=dev)
        ms = _event_ms(lambda: call("vg_axl2hel", _core.ptr(sinoA), 720, 128, nc, _core.ptr(ti),
                                    _core.ptr(tz), _core.ptr(tw), nvh, nr, _core.ptr(res),
                                    _core.stream(dev)), reps, stream)
        n_h = nvh * nr * nc
        gbs = 20.0 * n_h / (ms / 1e3) / 1e9  # four float32 neighbours read, one written
        sa = sinoA[:, :, :64].cpu().numpy()
        t0 = time.perf_counter()
        orc_mod().axl2hel(sa, idx[:90], zz[:90], wrap[:90], nr)
        cpu_ms = (time.perf_counter() - t0) * 1e3 * (nc / 64) * (nvh / 90)
        out["axl2hel"] = {"kernel_ms": ms, "gsamples_per_s": n_h / ms / 1e6,
                          "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                                       "frac": gbs / peak, "bytes_per_launch": 20.0 * n_h},
                          "cpu_scipy_ms_full_size": cpu_ms}
        ph = torch.rand((128, 128, 128), device=dev, generator=g)
        vws = np.linspace(0, 2 * np.pi, 180, endpoint=False)
        zs = np.linspace(-8, 8, 180)
        ms = _event_ms(lambda: tr.forward_project_phantom(ph, vws, None, None, zs), reps, stream)
        n_s = 180 * 128 ** 3
        php = ph.cpu().numpy()
        t0 = time.perf_counter()
        orc_mod().rotsum_fp(php, tr.view_matrices(php.shape, vws[:2], zs[:2]))
        cpu_ms = (time.perf_counter() - t0) * 1e3 * 90
        out["fp_phantom"] = {"kernel_ms": ms, "gsamples_per_s": n_s / ms / 1e6,
                             "note": "trilinear samples (8 L1/L2 reads each) summed along y; "
                                     "bound by the gathers, not by HBM",
                             "cpu_scipy_ms_full_size": cpu_ms}
        line.update({"cases": out, "cpu_baseline": {
            "kind": "port", "cores": 1,
            "sample": "the oracle's numpy / scipy.ndimage restatement of trajectory.py on 1/16 of "
                      "the columns (hel2axl), 90 of 1440 views x 1/16 of the columns (axl2hel), "
                      "2 of 180 views (fp_phantom), scaled to the full workload"}})
        print(json.dumps(line), flush=True)
        return 0
    elif wl == "c5ad":
        from vir_gb300.autograd import ConeGeom, reconstruct_adam, sirt
        n, na, nu, nv = 256, 360, 512, 384
        angs = tuple(np.linspace(0, 2 * np.pi, na, endpoint=False).tolist())
        geom = ConeGeom(angs, (n, n, n), nu, nv, 600.0, 1100.0, du=1.6, dv=1.6, d_pix=1.0)
        e = ph.random_ellipsoids(20, fov_radius=n / 2, seed=2027)
        xt = ph.rasterize3d_device(e, n, 1.0, device=dev)
        y = geom.fp(xt)
        rmse = lambda x: float(((x - xt) ** 2).mean().sqrt())
        # SIRT: 100 updates, RMSE after each (the RMSE evaluation is outside the timing)
        ts, tr = [], []
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

        def cb_s(i, x):
            ev[1].record(stream)
            torch.cuda.synchronize()
            ts.append(ev[0].elapsed_time(ev[1]))
            tr.append(rmse(x))
            ev[0].record(stream)

        ev[0].record(stream)
        sirt(y, geom, iters=101, callback=cb_s)
        ta, ra = [], []

        def cb_a(i, x, L):
            ev[1].record(stream)
            torch.cuda.synchronize()
            ta.append(ev[0].elapsed_time(ev[1]))
            ra.append(rmse(x))
            ev[0].record(stream)

        ev[0].record(stream)
        reconstruct_adam(y, geom, steps=200, lr=3e-3, lam=1e-3, callback=cb_a)
        target = tr[-1]
        k = next((i for i, r in enumerate(ra) if r <= target), None)
        line.update({
            "sirt": {"updates": len(tr), "ms_per_update": statistics.median(ts[1:]),
                     "rmse_every_10": tr[9::10], "path": "unfused projector calls + torch ops; "
                     "the first update also computes W_sino, W_img"},
            "adam": {"steps": len(ra), "ms_per_step": statistics.median(ta[1:]), "lr": 3e-3,
                     "lam": 1e-3, "rmse_every_20": ra[19::20]},
            "matched_rmse": {"rmse": target, "sirt_updates": len(tr),
                             "sirt_ms": float(sum(ts)),
                             "adam_steps": None if k is None else k + 1,
                             "adam_ms": None if k is None else float(sum(ta[:k + 1]))},
            "rmse_zero_image": rmse(torch.zeros_like(xt))})
        print(json.dumps(line), flush=True)
        return 0
    elif wl == "c3":
        if args.kernels_only:  # profiling aid: N persistent launches of 2 updates each
            from vir_gb300.batched import PersistentSIRT2D
            from vir_gb300.workloads import batched_problems
            pb = PersistentSIRT2D(batched_problems(64, seed=3), device=dev)
            for _ in range(args.kernels_only):
                pb.reset()
                pb.run(2)
            print(json.dumps({"kernels_only": args.kernels_only, "workload": wl, "ok": True}))
            return 0
        line.update(c3_summary(dev, stream))
        print(json.dumps(line), flush=True)
        return 0
    if args.kernels_only:
        for _ in range(args.kernels_only):
            fp(); bp()
        if wl in ("c4", "c5"):  # then the separable-footprint pair
            from vir_gb300.sys_mat import sp
            for _ in range(args.kernels_only):
                sp.sf_fp_cone_3d(x, angs, nu, nv, 600.0, 1100.0, **kw)
                sp.sf_bp_cone_3d(y, angs, (n, n, n), 600.0, 1100.0, **kw)
        torch.cuda.synchronize()
        print(json.dumps({"kernels_only": args.kernels_only, "workload": wl, "ok": True}))
        return 0
    t_fp, t_bp = _event_ms(fp, reps, stream), _event_ms(bp, reps, stream)
    line.update({"kernel_ms": {"fp": t_fp, "bp": t_bp},
                 "fwd_back_gups": 2 * units / ((t_fp + t_bp) / 1e3) / 1e9,
                 "roofline_fp": _roof(units, t_fp, peak, compulsory),
                 "roofline_bp": _roof(units, t_bp, peak, compulsory)})
    if wl == "c1":
        line["intersections"] = {"count": n_isect, "per_s_fp": n_isect / (t_fp / 1e3),
                                 "per_s_bp": n_isect / (t_bp / 1e3)}
    if wl in ("c4", "c5"):
        # the separable-footprint pair (SF-TR) on the same cone geometry
        from vir_gb300.sys_mat import sp
        sfp = lambda: sp.sf_fp_cone_3d(x, angs, nu, nv, 600.0, 1100.0, **kw)
        sbp = lambda: sp.sf_bp_cone_3d(y, angs, (n, n, n), 600.0, 1100.0, **kw)
        s_fp, s_bp = _event_ms(sfp, reps, stream), _event_ms(sbp, reps, stream)
        line["sf"] = {"kernel_ms": {"fp": s_fp, "bp": s_bp},
                      "fwd_back_gups": 2 * units / ((s_fp + s_bp) / 1e3) / 1e9,
                      "roofline_fp": _roof(units, s_fp, peak, compulsory),
                      "roofline_bp": _roof(units, s_bp, peak, compulsory),
                      "note": "BP time includes the l_theta weighting of the sinogram"}
    if wl == "c4":
        from vir_gb300 import autograd as ag
        from vir_gb300 import reconstruction as rc
        line["kernel_ms"]["fdk"] = _event_ms(
            lambda: rc.fdk(y, angs, (n, n, n), 600.0, 1100.0, du=du, dv=du, d_pix=dp), 1, stream)
        # 20 SIRT iterations of vir's rule (19 updates) on the cone pair: the
        # fused, graph-captured path (weights at set-up), and the unfused one
        s3 = rc.SIRT3D(y, angs, (n, n, n), 600.0, 1100.0, **kw)
        s3.capture(19)

        def sirt_fused():
            s3.reset()
            s3.run(19)

        t_fused = _event_ms(sirt_fused, 1, stream)
        rmse = float(torch.sqrt(torch.mean((s3.x - x) ** 2)))
        del s3
        torch.cuda.empty_cache()
        geom = ag.ConeGeom(tuple(angs), (n, n, n), nu, nv, 600.0, 1100.0, **kw)
        out = {}

        def sirt20():
            out["x"] = ag.sirt(y, geom, iters=20)

        t_sirt = _event_ms(sirt20, 1, stream)
        rmse_u = float(torch.sqrt(torch.mean((out["x"] - x) ** 2)))
        line["sirt"] = {"iters": 20, "updates": 19, "ms": t_fused,
                        "iter_per_s": 19 / (t_fused / 1e3), "rmse_vs_phantom": rmse,
                        "path": "fused (vg_dd3d_sirt_iter: residual in the FP epilogue, update in "
                                "the BP epilogue), 19 updates as one CUDA graph; weights at set-up",
                        "unfused": {"ms": t_sirt, "iter_per_s": 19 / (t_sirt / 1e3),
                                    "rmse_vs_phantom": rmse_u,
                                    "path": "projector calls + torch elementwise ops, W_sino/W_img "
                                            "inside the timed call"}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c3", action="store_true",
                    help="leave out the batched-SIRT summary (the C3 problem set) of the default line")
    ap.add_argument("--kernels-only", type=int, default=0, metavar="N",
                    help="profiling aid: run the two fused SIRT kernels N times each, no timing")
    ap.add_argument("--workload", default="c2", choices=["c2"] + sorted(EXTRA),
                    help="c2 (default) is the benchmark line; the others print one extra "
                         "JSON line for that configuration")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "c2":
        return run_workload(args)
    if args.kernels_only:
        return run_kernels_only(args.kernels_only)

    import torch
    import torch.distributed as dist
    rank, world, local = dist_info()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import ctypes
    from vir_gb300 import _core
    from vir_gb300._lib import call
    from vir_gb300 import reconstruction as rc

    w = WORKLOAD
    img, angs, y = make_inputs()
    K, Wm, U = args.steps, max(args.warmup, 3), w["updates_per_step"]

    # ---- device-resident SIRT: inputs already in HBM --------------------
    sirt = rc.SIRT2D(y, angs, img.shape, geom="fan", DSO=w["DSO"], DSD=w["DSD"], du=w["du"],
                     d_pix=w["d_pix"], device=dev)
    sirt.capture(U)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(Wm):
        sirt.reset()
        sirt.run(U)
    torch.cuda.synchronize(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(K)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(torch.cuda.current_device()) as clk:
        for i in range(K):
            sirt.reset()
            flush.fill_(float(i))            # L2 flush between timed steps
            ev[i][0].record(stream)
            sirt.run(U)
            ev[i][1].record(stream)
        torch.cuda.synchronize(dev)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms, value = job_rate(sum(step_ms), world, K * U, dist if world > 1 else None, dev)
    x_final = sirt.x.detach().cpu().numpy()
    rmse = float(np.sqrt(np.mean((x_final - img) ** 2)))

    # ---- per-kernel timing of the two halves of the update, launched exactly
    # as the captured graph launches them (the forward projection with its
    # residual / table epilogue, the back projection with its update
    # epilogue), CUDA events on the launch stream between them -------------
    g = sirt.g
    from vir_gb300 import _lib
    launches_per_update = _lib.load().vg_dd2d_sirt_launches(ctypes.byref(g))
    reps = 20
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fp_ms, bp_ms = [], []
    for i in range(reps + 2):
        e[0].record(stream)
        call("vg_dd2d_sirt_residual", ctypes.byref(g), _core.ptr(sirt.y), _core.ptr(sirt.inv_ws),
             _core.ptr(sirt.trig), _core.ptr(sirt.x), _core.ptr(sirt.xT), _core.ptr(sirt.r),
             _core.ptr(sirt.ws), sirt.ws.numel(), _core.stream(dev))
        e[1].record(stream)
        call("vg_dd2d_sirt_update", ctypes.byref(g), _core.ptr(sirt.inv_wi),
             ctypes.c_float(sirt.gamma), _core.ptr(sirt.trig), _core.ptr(sirt.x),
             _core.ptr(sirt.xT), _core.ptr(sirt.r), _core.ptr(sirt.ws), sirt.ws.numel(),
             _core.stream(dev))
        e[2].record(stream)
        torch.cuda.synchronize(dev)
        if i >= 2:
            fp_ms.append(e[0].elapsed_time(e[1]))
            bp_ms.append(e[1].elapsed_time(e[2]))
    t_fp, t_bp = statistics.median(fp_ms), statistics.median(bp_ms)
    in_graph_ms = total_ms / (K * U)
    units = w["na"] * w["n"] * w["n"]                    # voxel-view updates per projector call
    alg_bytes = 4.0 * units
    dom_name, t_dom = ("dd2d_bp_kernel<fan>", t_bp) if t_bp >= t_fp else ("dd2d_fp_kernel<fan>", t_fp)
    peak, peak_src = load_peaks()
    achieved = alg_bytes / (t_dom / 1e3) / 1e9
    comp_bytes = 4.0 * (w["n"] * w["n"] + w["na"] * w["nu"])   # image + sinogram
    traffic = load_traffic()

    # ---- the plain FP32 path: one problem, every op its own launch -------
    # (projector calls of the drop-in API, torch elementwise ratio/update,
    # no fusion, no graph) for the same updates, to state the speed-up of the
    # fused graph path at matched RMSE
    from vir_gb300.autograd import Geom2D, sirt as plain_sirt
    geom = Geom2D(tuple(angs.tolist()), img.shape, w["nu"], du=w["du"], d_pix=w["d_pix"],
                  DSO=w["DSO"], DSD=w["DSD"], fan=True)
    y_dev = torch.from_numpy(y).to(dev)
    W_sino = geom.fp(torch.ones(img.shape, device=dev))
    W_img = geom.bp(torch.ones_like(y_dev))
    plain_sirt(y_dev, geom, iters=4, W_sino=W_sino, W_img=W_img)   # warm-up
    torch.cuda.synchronize(dev)
    pe0, pe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pe0.record(stream)
    x_plain = plain_sirt(y_dev, geom, iters=U + 1, W_sino=W_sino, W_img=W_img)
    pe1.record(stream)
    torch.cuda.synchronize(dev)
    plain_val = U / (pe0.elapsed_time(pe1) / 1e3)
    x_plain = x_plain.cpu().numpy()
    rmse_plain = float(np.sqrt(np.mean((x_plain - img) ** 2)))

    # ---- end to end through the public API with host buffers ----------
    y_pinned = torch.from_numpy(y).pin_memory()
    e2e_ms = []
    for i in range(Wm + K):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        x = rc.sirt_2d(y_pinned, angs, img.shape, geom="fan", DSO=w["DSO"], DSD=w["DSD"],
                       du=w["du"], d_pix=w["d_pix"], iters=U + 1)
        _ = float(x[0, 0])                                # result on the host
        if i >= Wm:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_val = world * U / (statistics.median(e2e_ms) / 1e3)

    line = {
        "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world, "steps": K,
        "warmup": Wm, "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": arm_config(world),
        "fwd_back_gups": 2 * units / ((t_fp + t_bp) / 1e3) / 1e9,
        "kernel_ms": {"dd2d_fp_kernel<fan>": t_fp, "dd2d_bp_kernel<fan>": t_bp,
                      "update_in_graph": in_graph_ms,
                      "note": "each half timed as the graph launches it: the forward "
                              "projection with its residual and table epilogue, the back "
                              "projection with its update epilogue"},
        "rmse_vs_phantom": rmse,
        "plain_fp32": {"value": plain_val, "unit": "iter/s", "rmse_vs_phantom": rmse_plain,
                       "path": "unfused: drop-in FP and BP calls + torch elementwise ops, "
                               "one launch each, no graph",
                       "speedup": value / plain_val,
                       "iterate_rel_diff": float(np.abs(x_final - x_plain).max()
                                                 / np.abs(x_plain).max())},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "kernel": dom_name,
                     "traffic": ((traffic or {}).get("kernels", {}).get(dom_name) or {})
                                .get("dram_bytes_per_launch"),
                     "algorithmic_bytes_per_launch": alg_bytes, "peak_source": peak_src,
                     "compulsory": {"bytes_per_launch": comp_bytes,
                                    "achieved": comp_bytes / (t_dom / 1e3) / 1e9,
                                    "frac": comp_bytes / (t_dom / 1e3) / 1e9 / peak,
                                    "note": "unique inputs + outputs of the launch (image and "
                                            "sinogram); L2-resident, so not a DRAM bound"}},
        "e2e": {"value": e2e_val, "unit": "iter/s", "h2d_bytes_per_step": int(y.nbytes),
                "d2h_bytes_per_step": int(img.nbytes),
                "note": "reconstruction.sirt_2d on a pinned host sinogram: each step copies the "
                        "sinogram in, runs all updates from x0 = 1e-5 and copies the image out; "
                        "the geometry's weights FP(1), BP(1) and its update graph are prepared "
                        "by the first call and reused (reconstruction.prepared_sirt)"},
        "gpu_launches": K * U * launches_per_update,      # library kernels per update (2 or 3)
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        # the whole step on the host cores: the FP64 C restatement of
        # dd.py/sirt_dd.py runs the same 100 updates; its iterate also pins
        # the GPU's against the accuracy criterion (1e-4 relative)
        sec, cores, x_orc = cpu_sirt_iteration_rate(img.shape, angs, y, U, want_x=True)
        line["cpu_baseline"] = {"value": 1.0 / sec, "unit": "iter/s", "cores": cores,
                                "kind": "port",
                                "sample": f"the whole step: {U} SIRT updates (FP + BP) of the full "
                                          "workload, FP64 C restatement of dd.py/sirt_dd.py, "
                                          "OpenMP"}
        r_orc = float(np.sqrt(np.mean((x_orc - img) ** 2)))
        line["oracle_rel"] = {
            "iterate_rel_l2": float(np.linalg.norm(x_final - x_orc) / np.linalg.norm(x_orc)),
            "rmse_vs_phantom_rel": abs(rmse - r_orc) / r_orc,
            "rmse_vs_phantom_oracle": r_orc, "criterion": 1e-4,
            "what": f"the GPU iterate after {U} updates vs the FP64 oracle's"}
    if rank == 0 and world == 1:
        # the FBP half of the configuration: fan FBP of the same noisy
        # sinogram with the Ram-Lak and Hann windows (cosine weight, FFT ramp
        # filter, 1/U^2-weighted back projection), against the phantom and,
        # with the CPU legs, against the FP64 oracle's FBP
        f32 = lambda v: float(np.float32(v))
        y_dev = torch.from_numpy(y).to(dev)
        line["fbp"] = {}
        for filt in ("ramp", "hann"):
            run = lambda: rc.fbp_2d(y_dev, angs, img.shape, geom="fan", DSO=w["DSO"], DSD=w["DSD"],
                                    du=w["du"], d_pix=w["d_pix"], filter_type=filt)
            ms = _event_ms(run, 10, stream)
            rec = run().cpu().numpy()
            rec_f = {"ms": ms, "rmse_vs_phantom": float(np.sqrt(np.mean((rec - img) ** 2)))}
            if not args.no_cpu_baseline:
                from oracle import oracle as orc
                ref = orc.fbp_2d(y, angs, img.shape, fan=True, DSO=f32(w["DSO"]), DSD=f32(w["DSD"]),
                                 du=f32(w["du"]), d_pix=f32(w["d_pix"]), filter_type=filt)
                rec_f["oracle_max_rel"] = float(np.abs(rec - ref).max() / np.abs(ref).max())
                rec_f["oracle_rel_l2"] = float(np.linalg.norm(rec - ref) / np.linalg.norm(ref))
            line["fbp"]["ram-lak" if filt == "ramp" else filt] = rec_f
    if rank == 0 and world == 1 and not args.no_c3:
        # after the timed region: the batched-SIRT configuration, so that its
        # speed-ups over the plain path and its error against the oracle are
        # part of the benchmark record
        line["batched"] = {"workload": EXTRA["c3"],
                           **c3_summary(dev, stream, check=not args.no_cpu_baseline)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
