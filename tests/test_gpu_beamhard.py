"""GPU beam-hardening pre-correction (processing/beamhard.py) against the
reference's own outputs (golden vectors) and the oracle: the device replays
numpy's arithmetic, so the results are equal bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _water(e):
    return 0.17 + 2500.0 * np.asarray(e, np.float64) ** -3.0


def test_poly_golden(vg, golden):
    from vir_gb300 import beamhard as bh
    p = golden["bh_poly"]
    li, coefs, mu = p["line_ints"], p["coefs"], float(p["mu"])
    for got, ref in ((bh.beamhard_cor(li, coefs, mu), p["cor_f64coefs"]),
                     (bh.beamhard_cor(li, [float(c) for c in coefs], mu), p["cor_pycoefs"]),
                     (bh.beamhard_cor(li, coefs, np.float64(mu)), p["cor_f64mu"]),
                     (bh.beamhard_cor(li.astype(np.float64), coefs, mu), p["cor_f64in"])):
        assert got.dtype == ref.dtype and got.shape == ref.shape
        assert np.array_equal(got, ref)


def test_table_golden_and_range(vg, golden, orc):
    """The lookup itself is exact against interp1d on the same host; the
    table (numpy exp/log of the spectrum) may differ in the last bit between
    the machine that wrote the fixture and this one."""
    from vir_gb300 import beamhard as bh
    t = golden["bh_table"]
    got = bh.beamhard_cor_table(t["line_ints"], t["energies"], t["counts"], None,
                                float(t["atten_eff"]), mixatten=lambda m, e: _water(e))
    assert got.dtype == np.float64
    assert np.array_equal(got, orc.bh_table(t["line_ints"], t["energies"], t["counts"],
                                            float(t["atten_eff"]), _water(t["energies"])))
    assert np.allclose(got, t["cor"], rtol=1e-12, atol=0)
    over = t["line_ints"].copy()
    over[1, 3] = 1e3  # beyond the 80-unit water table: interp1d raises
    with pytest.raises(ValueError):
        bh.beamhard_cor_table(over, t["energies"], t["counts"], None, float(t["atten_eff"]),
                              mixatten=lambda m, e: _water(e))


def test_lut_golden(vg, golden):
    from vir_gb300 import beamhard as bh
    lut = golden["bh_lut"]
    got = bh.beamhard_cor2(lut["line_ints"], lut["coefs"], float(lut["mu"]))
    assert got.dtype == np.float64 and np.array_equal(got, lut["cor"])


def test_large_vs_oracle_and_torch(vg, orc):
    """3 M samples (several grid strides per thread), NaN and negative values,
    numpy and CUDA-tensor inputs."""
    import torch
    from vir_gb300 import beamhard as bh
    rng = np.random.default_rng(40)
    li = (rng.random((30, 100, 1000)) * 7.0 - 0.2).astype(np.float32)
    li[0, 0, :3] = [np.nan, -0.0, 0.0]
    coefs = np.polyfit(np.linspace(0, 9, 40), np.linspace(0, 9, 40) ** 1.07, 2)
    ref = orc.bh_poly(li, coefs, 0.19)
    got = bh.beamhard_cor(li, coefs, 0.19)
    assert np.array_equal(got, ref, equal_nan=True)
    gt = bh.beamhard_cor(torch.from_numpy(li).cuda(), coefs, 0.19)
    assert gt.is_cuda and np.array_equal(gt.cpu().numpy(), ref, equal_nan=True)
    e = np.arange(20.0, 121.0)
    cnt = np.exp(-0.5 * ((e - 70.0) / 20.0) ** 2)
    ae = float(_water([np.average(e, weights=cnt)])[0])
    ok = np.nan_to_num(li, nan=1.0)
    ref_t = orc.bh_table(ok, e, cnt, ae, _water(e))
    got_t = bh.beamhard_cor_table(ok, e, cnt, None, ae, mixatten=lambda m, x: _water(x))
    assert np.array_equal(got_t, ref_t)
    coefs_tb = 1.0 + 0.03 * np.cos(np.linspace(0, 5, 4001))
    assert np.array_equal(bh.beamhard_cor2(li, coefs_tb, 0.19), orc.bh_lut(li, coefs_tb, 0.19),
                          equal_nan=True)
