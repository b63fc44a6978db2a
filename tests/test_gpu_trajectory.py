"""GPU helical rebinning front-end (trajectory.py) against the reference's
own outputs (golden vectors) and the oracle.  The gathers and the axial to
helical resampling replay numpy's and scipy's float64 arithmetic and are
compared bit for bit (NaN rows included: interpZ yields them where a slice
has no detector row on one side); the rotate-and-sum projector samples in
float32 where scipy samples in float64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def _geoms(h):
    from vir_gb300 import trajectory as tr
    G = tr.Geom(nViews=int(h["nViews"]), coverage=float(h["coverage"]), zTran=float(h["zTran"]))
    GI = tr.Geom(nViews=int(h["int_nViews"]), coverage=float(h["int_coverage"]),
                 angle0=float(h["int_angle0"]), zTran=float(h["int_zTran"]))
    return G, GI


@pytest.mark.parametrize("case", ["traj_axl2hel", "traj_axl2hel_z"])
def test_axl2hel_golden(vg, golden, case):
    from vir_gb300 import trajectory as tr
    a = golden[case]
    got = tr.sino_axl2hel(a["sinoA"], int(a["nRowsH"]), a["viewsH"], int(a["nAngsH"]),
                          float(a["pitch"]), Z=a.get("Z"))
    assert got.dtype == np.float32 and np.array_equal(got, a["sinoH"])


def test_hel2axl_golden(vg, golden):
    from vir_gb300 import trajectory as tr
    h = golden["traj_hel2axl"]
    G, GI = _geoms(h)
    a1, a2 = tr.sino_hel2axl(h["sinoH"], G, h["angsA"], h["zA"])
    assert np.array_equal(a1, h["a1"], equal_nan=True) and np.array_equal(a2, h["a2"], equal_nan=True)
    outs = tr.sino_hel2axl180(h["sinoH"], G, h["angsA"], h["zA"])
    for got, key in zip(outs, ("f1", "f2", "b1", "b2")):
        assert np.array_equal(got, h[key], equal_nan=True), key
    i1, i2 = tr.sino_hel2hel(h["sinoH"], G, GI, 4)
    assert np.array_equal(i1, h["i1"], equal_nan=True) and np.array_equal(i2, h["i2"], equal_nan=True)


def test_fp_phantom_golden(vg, golden):
    from vir_gb300 import trajectory as tr
    f = golden["traj_fp_phantom"]
    got = tr.forward_project_phantom(f["phantom"], f["views"], None, None, f["Z"])
    assert got.shape == f["sino"].shape and rel(got, f["sino"]) < 1e-5


def test_larger_vs_oracle_and_torch(vg, orc):
    """720 helical views of 16 rows x 300 columns (two rotations), rebinned
    to 90 axial angles x 20 slices; 360 axial angles resampled to 500
    helical views; a 40 x 36 x 24 phantom over 30 views; CUDA tensors in."""
    import torch
    from vir_gb300 import trajectory as tr
    rng = np.random.default_rng(41)
    G = tr.Geom(nViews=720, coverage=4 * np.pi, zTran=12.0)
    sinoH = rng.random((720, 16, 300)).astype(np.float32)
    angs = np.linspace(0, 2 * np.pi, 90, endpoint=False)
    Z = np.linspace(-4.0, 4.0, 20)
    a1, a2 = tr.sino_hel2axl(sinoH, G, angs, Z)
    pp, wp, pn, wn = tr._tables(G, [Z] * angs.size, angs, 16)
    sh = (angs.size, Z.size, 300)
    assert np.array_equal(a1, orc.rebin_rows(sinoH, pp, wp, sh), equal_nan=True)
    assert np.array_equal(a2, orc.rebin_rows(sinoH, pn, wn, sh), equal_nan=True)
    t1, _ = tr.sino_hel2axl(torch.from_numpy(sinoH).cuda(), G, angs, Z)
    assert t1.is_cuda and np.array_equal(t1.cpu().numpy(), a1, equal_nan=True)
    sinoA = rng.random((360, 24, 256)).astype(np.float32)
    vH = np.linspace(0, 6 * np.pi, 500, endpoint=False) + 0.013
    got = tr.sino_axl2hel(sinoA, 8, vH, 180, 1.3)
    idx, zz, wrap, _ = tr.axl2hel_index(360, 24, 8, vH, 180, 1.3)
    assert np.array_equal(got, orc.axl2hel(sinoA, idx, zz, wrap, 8))
    ph = rng.random((40, 36, 24)).astype(np.float32)
    vws = np.linspace(0, np.pi, 30)
    zs = np.linspace(-3, 3, 30)
    fp = tr.forward_project_phantom(torch.from_numpy(ph).cuda(), vws, None, None, zs)
    M = tr.view_matrices(ph.shape, vws, zs)
    assert fp.is_cuda and rel(fp.cpu().numpy(), orc.rotsum_fp(ph, M)) < 1e-5
