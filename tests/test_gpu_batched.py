"""Batched SIRT (one CUDA graph over many problems) equals the per-problem
path and the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batched_equals_plain_and_oracle(vg, orc):
    from vir_gb300.batched import BatchedSIRT2D
    from vir_gb300.workloads import batched_problems
    probs = batched_problems(7, seed=11, sizes=(32, 48, 64), na_range=(20, 90))
    b = BatchedSIRT2D(probs, n_streams=3)
    b.run(9)
    got = [x.cpu().numpy() for x in b.images()]
    b.reset()
    b.plain(9)
    ref = [x.cpu().numpy() for x in b.images()]
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)   # same kernels, same order per problem
    for p, g in zip(probs[:3], got[:3]):
        a, n = p["ang_arr"], p["img_shape"]
        nu = p["sino"].shape[1]
        if p["geom"] == "fan":
            fp = lambda x: orc.dd_fp_fan_2d(x, a, nu, p["DSO"], p["DSD"])
            bp = lambda s: orc.dd_bp_fan_2d(s, a, n, p["DSO"], p["DSD"])
        else:
            fp = lambda x: orc.dd_fp_par_2d(x, a, nu)
            bp = lambda s: orc.dd_bp_par_2d(s, a, n)
        xo = orc.sirt(p["sino"], fp, bp, n, iters=10)
        assert np.abs(g - xo).max() <= 2e-4 * np.abs(xo).max()


def test_persistent_equals_per_problem_and_oracle(vg, orc):
    """One persistent launch (vg_sirt2d_batch_run, work queue over all
    problems) gives the per-problem chains' iterates (same kernels per work
    item) and vir's SIRT within the oracle tolerance."""
    from vir_gb300.batched import BatchedSIRT2D, PersistentSIRT2D
    from vir_gb300.workloads import batched_problems
    probs = batched_problems(7, seed=11, sizes=(32, 48, 64), na_range=(20, 90))
    b = BatchedSIRT2D(probs, n_streams=3)
    b.run(9)
    ref = [x.cpu().numpy() for x in b.images()]
    p = PersistentSIRT2D(probs)
    status, done = p.run(9)
    assert (status, done) == ("ok", 9)
    got = [x.cpu().numpy() for x in p.images()]
    for g, r in zip(got, ref):
        assert np.abs(g - r).max() <= 1e-6 * np.abs(r).max()
    for q, g in zip(probs[:3], got[:3]):
        a, n, nu = q["ang_arr"], q["img_shape"], q["sino"].shape[1]
        if q["geom"] == "fan":
            fp = lambda x: orc.dd_fp_fan_2d(x, a, nu, q["DSO"], q["DSD"])
            bp = lambda s: orc.dd_bp_fan_2d(s, a, n, q["DSO"], q["DSD"])
        else:
            fp = lambda x: orc.dd_fp_par_2d(x, a, nu)
            bp = lambda s: orc.dd_bp_par_2d(s, a, n)
        xo = orc.sirt(q["sino"], fp, bp, n, iters=10)
        assert np.abs(g - xo).max() <= 2e-4 * np.abs(xo).max()
    # a second run from the reset iterate repeats the first exactly
    p.reset()
    p.run(9)
    assert all(np.array_equal(x.cpu().numpy(), g) for x, g in zip(p.images(), got))


@pytest.mark.parametrize("storage", ["bf16y", "bf16x", "bf16"])
def test_persistent_bf16_storage_vs_oracle(vg, orc, storage):
    """bfloat16 storage of the measured sinogram, the iterate or both, float32
    arithmetic: the final iterate's error against vir's SIRT in FP64 (relative
    L2) for a 128^2 problem, 49 updates.  Only the sinogram in bfloat16 keeps
    the error near bfloat16's own rounding of the data; rounding the iterate
    at every update costs more."""
    from vir_gb300.batched import PersistentSIRT2D
    from vir_gb300.workloads import batched_problems
    q = batched_problems(1, seed=5, sizes=(128,), na_range=(200, 200))[0]
    a, n, nu = q["ang_arr"], q["img_shape"], q["sino"].shape[1]
    if q["geom"] == "fan":
        fp = lambda x: orc.dd_fp_fan_2d(x, a, nu, q["DSO"], q["DSD"])
        bp = lambda s: orc.dd_bp_fan_2d(s, a, n, q["DSO"], q["DSD"])
    else:
        fp = lambda x: orc.dd_fp_par_2d(x, a, nu)
        bp = lambda s: orc.dd_bp_par_2d(s, a, n)
    xo = orc.sirt(q["sino"], fp, bp, n, iters=50)
    rel = {}
    for st in ("fp32", storage):
        p = PersistentSIRT2D([q], storage=st)
        assert p.run(49) == ("ok", 49)
        x = p.images()[0].cpu().numpy()
        rel[st] = np.linalg.norm(x - xo) / np.linalg.norm(xo)
    assert rel["fp32"] < 1e-5
    bound = {"bf16y": 1e-2, "bf16x": 5e-2, "bf16": 5e-2}[storage]
    assert rel[storage] < bound, rel


def test_persistent_cancel_mid_run(vg):
    """The host raises the cancel flag while a long run is on the GPU: the
    run stops at the end of the current update with status 'cancelled'."""
    import time
    from vir_gb300.batched import PersistentSIRT2D
    from vir_gb300.workloads import batched_problems
    p = PersistentSIRT2D(batched_problems(3, seed=2, sizes=(32,), na_range=(20, 30)))
    p.run(2_000_000, wait=False)
    time.sleep(0.3)
    p.cancel()
    status, done = p.result()
    assert status == "cancelled"
    assert 0 < done < 2_000_000


def test_persistent_time_budget(vg):
    """A time budget shorter than the run stops it with status 'timeout'."""
    from vir_gb300.batched import PersistentSIRT2D
    from vir_gb300.workloads import batched_problems
    p = PersistentSIRT2D(batched_problems(3, seed=2, sizes=(32,), na_range=(20, 30)))
    status, done = p.run(2_000_000, budget_s=0.05)
    assert status == "timeout"
    assert 0 < done < 2_000_000
    # and a run within its budget ends normally
    assert p.run(5, budget_s=30.0) == ("ok", 5)
