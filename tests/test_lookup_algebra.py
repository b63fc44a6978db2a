"""CPU checks of the index arithmetic behind the 2D distance-driven kernels'
table lookups (vir_gb300/csrc/dd2d.cu), restated in exact integer and FP64
arithmetic:

* the forward projection finds pixel p (-1 .. nd + 1) of a staged line as the
  bit pattern b = 0x4B40000F + (p + 1) of a round-down FMA onto
  1.5 * 2^23 + 15, and its slot as b + (b >> 4) minus a fixed bias;
* the back projection's per-view table holds the sinogram row's running
  integral G in the coordinate t' = (t + 1) / (nu + 2), with sentinel rows
  before and after the detector, read at slot floor(t' (nu + 2)) of the
  saturated t'.
"""
import numpy as np
import pytest

MAGIC = 0x4B400000                      # bits of 1.5 * 2^23
BIAS = MAGIC + (MAGIC >> 4) + 15        # FP_SLOT_BIAS


def fp_slot(p):
    return p + 1 + ((p + 16) >> 4)


def fp_line_entries(nd):
    return fp_slot(nd + 1) + 1


@pytest.mark.parametrize("nd", [1, 7, 8, 15, 16, 17, 131, 512, 1024, 2049])
def test_fp_slot_from_round_down_bits(nd):
    slots = []
    for k in range(nd + 3):                       # floor(t' (nd + 2)) for t' in [0, 1]
        b = MAGIC + 15 + k                         # the FMA result 12582927 + k, exact
        assert np.float32(12582927.0 + k).view(np.uint32) == b
        slot = b + (b >> 4) - BIAS
        assert slot == fp_slot(k - 1)
        slots.append(slot)
    assert slots[0] == 0 and max(slots) < fp_line_entries(nd)
    assert len(set(slots)) == len(slots)          # distinct pixels, distinct slots
    for m0 in range(0, nd, 8):                    # a lane's 8-pixel segment is contiguous
        assert [fp_slot(m0 + i) for i in range(8)] == list(range(fp_slot(m0), fp_slot(m0) + 8))
    # the scan's lanes (8 pixels apart) write 8-byte entries on distinct bank
    # pairs in each half-warp
    for base in range(0, 4 * 256, 256):
        words = [2 * fp_slot(base + 8 * lane) for lane in range(16)]
        assert len({w % 32 for w in words}) == 16


@pytest.mark.parametrize("nu", [1, 7, 768])
def test_bp_table_reproduces_the_running_integral(nu):
    rng = np.random.default_rng(nu)
    du = 1.2
    s = rng.random(nu).astype(np.float32).astype(np.float64)
    run = np.concatenate([[0.0], np.cumsum(s)])      # sum_{i<j} s_i
    # table entries i = j + 1: (T_j - (j + 1) du s_j, du s_j (nu + 2)); sentinels
    x = np.zeros(nu + 3)
    y = np.zeros(nu + 3)
    j = np.arange(nu)
    x[1:nu + 1] = (run[:nu] - (j + 1) * s) * du
    y[1:nu + 1] = du * s * (nu + 2)
    x[nu + 1:] = run[nu] * du
    ts = np.concatenate([np.linspace(-3.0, nu + 3.0, 4 * nu + 97), np.arange(-2, nu + 3, 1.0)])
    for t in ts:
        tq = min(max((t + 1.0) / (nu + 2), 0.0), 1.0)  # the saturating FMA
        slot = int(np.floor(tq * (nu + 2)))           # the round-down FMA's integer
        assert 0 <= slot <= nu + 2
        g = x[slot] + y[slot] * tq
        tc = min(max(t, 0.0), float(nu))
        jj = min(int(np.floor(tc)), nu - 1)
        ref = du * (run[jj] + s[jj] * (tc - jj))
        assert abs(g - ref) <= 1e-12 * max(1.0, run[nu] * du)
