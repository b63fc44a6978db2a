// Beam-hardening pre-correction of logged sinograms (vir's
// processing/beamhard.py), applied elementwise on the device.
//
//  vg_bh_poly: the water polynomial of beamhard_cor (beamhard.py:39-47),
//      out = mu ((c0 t^2 + c1 t) + c2), t = in / mu,
//    in numpy's operation order, each step in the type numpy gives it (a
//    float32 sinogram with Python-float mu keeps t in float32, np.polyfit's
//    float64 coefficients lift the terms to float64, ...: bit i of f32mask
//    says step i is float32, for t (and t^2), c0 t^2, c1 t, the sum with c2
//    and the product with mu).  Every operation is separately rounded (no
//    contraction), so the result equals numpy's bit for bit.
//  vg_bh_interp: piecewise-linear lookup in an increasing table (x_k, y_k),
//    FP64 like the reference's callers:
//      mode 0, scipy interp1d 'linear' as beamhard_cor_table uses it
//        (beamhard.py:16-36): v = max(in, 0); k = searchsorted_left(x, v)
//        clipped to [1, m-1]; out = (y_k - y_k-1)/(x_k - x_k-1) (v - x_k-1)
//        + y_k-1; values outside [x_0, x_m-1] are counted (interp1d raises).
//      mode 1 / 2, np.interp as the lookup-table correction of the
//        reference's beam-hardening study
//        (tests/Test_Beamhard/beamhard_test.py:26-27): v = in / mu, divided
//        in float32 (mode 1: float32 sinogram, Python-float mu) or float64
//        (mode 2); f = y_0 below x_0, y_m-1 above x_m-1, NaN for NaN, y_j at
//        x_j, else slope (v - x_j) + y_j with x_j <= v < x_j+1; out = in f.
//    The search keys live in shared memory; the grid strides over the sinogram.
#include <type_traits>

#include "vg_common.cuh"

namespace {

using namespace vg;

template <typename TI, typename TO>
__global__ void __launch_bounds__(256)
bh_poly_kernel(const TI *__restrict__ in, TO *__restrict__ out, size_t n, double mu, double c0,
               double c1, double c2, int f32mask) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const float muf = (float)mu, c0f = (float)c0, c1f = (float)c1, c2f = (float)c2;
    const bool tf = f32mask & 1, p0f = f32mask & 2, p1f = f32mask & 4, s2f = f32mask & 8,
               rf = f32mask & 16;
    if (f32mask == 31) {  // every step float32 (Python-float coefficients and mu)
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const float t = __fdiv_rn((float)in[i], muf);
            const float s = __fadd_rn(__fadd_rn(__fmul_rn(c0f, __fmul_rn(t, t)), __fmul_rn(c1f, t)),
                                      c2f);
            out[i] = (TO)__fmul_rn(muf, s);
        }
        return;
    }
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float t_f = 0.f, t2_f = 0.f, p0_f = 0.f, p1_f = 0.f, s_f = 0.f;
        double t_d, t2_d, p0_d, p1_d, s_d;
        if (tf) {
            t_f = __fdiv_rn((float)in[i], muf);
            t2_f = __fmul_rn(t_f, t_f);
            t_d = t_f;
            t2_d = t2_f;
        } else {
            t_d = __ddiv_rn((double)in[i], mu);
            t2_d = __dmul_rn(t_d, t_d);
        }
        if (p0f) { p0_f = __fmul_rn(c0f, t2_f); p0_d = p0_f; }
        else p0_d = __dmul_rn(c0, t2_d);
        if (p1f) { p1_f = __fmul_rn(c1f, t_f); p1_d = p1_f; }
        else p1_d = __dmul_rn(c1, t_d);
        if (p0f && p1f) {
            s_f = __fadd_rn(p0_f, p1_f);
            if (s2f) { s_f = __fadd_rn(s_f, c2f); s_d = s_f; }
            else s_d = __dadd_rn((double)s_f, c2);
        } else {
            s_d = __dadd_rn(__dadd_rn(p0_d, p1_d), c2);
        }
        const double r = rf ? (double)__fmul_rn(muf, s_f) : __dmul_rn(mu, s_d);
        out[i] = (TO)r;
    }
}

// first k in [0, m] with key[k] >= v (numpy searchsorted, side 'left')
template <typename K, typename V>
__device__ __forceinline__ int lower_bound(const K *key, int m, V v) {
    int lo = 0, hi = m;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (key[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// first k in [0, m] with key[k] > v (side 'right')
template <typename K, typename V>
__device__ __forceinline__ int upper_bound(const K *key, int m, V v) {
    int lo = 0, hi = m;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (key[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

struct alignas(16) Seg {
    double x, y, s, pad;
};

__device__ __forceinline__ Seg load_seg(const Seg *p) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    return Seg{a.x, a.y, b.x, b.y};
}

// seg[k] = (x_k, y_k, slope_k, 0), slope_k = (y_k+1 - y_k) / (x_k+1 - x_k) as
// the reference divides it (the same IEEE quotient for every sample of the
// segment, so it is computed once on the host).  The binary search runs over
// keys in shared memory: with KF32 the keys are x rounded to float32 toward
// -inf (mode 0, tested with <) or +inf (modes 1 / 2, tested with <=); for a
// sample v that is itself a float32 value, key < v <=> x < v and
// key <= v <=> x <= v exactly, so the float32 search finds numpy's index.
template <typename TI, typename TO, bool KF32>
__global__ void __launch_bounds__(256)
bh_interp_kernel(const TI *__restrict__ in, TO *__restrict__ out, size_t n,
                 const Seg *__restrict__ seg, const void *__restrict__ keys_g, int m,
                 int mode, double mu, unsigned long long *__restrict__ n_out) {
    using K = typename std::conditional<KF32, float, double>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    K *key = reinterpret_cast<K *>(smem_raw);
    for (int k = threadIdx.x; k < m; k += blockDim.x) key[k] = static_cast<const K *>(keys_g)[k];
    __syncthreads();
    const double x0 = seg[0].x, xl = seg[m - 1].x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    unsigned long long outside = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double r;
        if (mode == 0) {
            const TI a = in[i];
            const TI c = a < (TI)0 ? (TI)0 : a;  // line_ints.clip(0); NaN stays
            const double v = (double)c;
            if (v < x0 || v > xl) ++outside;
            int k = KF32 ? lower_bound(key, m, (float)c) : lower_bound(key, m, v);
            k = min(max(k, 1), m - 1);
            const Seg sg = load_seg(seg + (k - 1));
            r = __dadd_rn(__dmul_rn(sg.s, __dsub_rn(v, sg.x)), sg.y);
        } else {
            const float vf = __fdiv_rn((float)in[i], (float)mu);
            const double v = mode == 1 ? (double)vf : __ddiv_rn((double)in[i], mu);
            double f;
            if (v != v) {
                f = v;
            } else if (v > xl) {
                f = seg[m - 1].y;
            } else if (v < x0) {
                f = seg[0].y;
            } else {
                const int j = (KF32 ? upper_bound(key, m, vf) : upper_bound(key, m, v)) - 1;
                const Seg sg = load_seg(seg + j);  // x_j <= v < x_j+1
                if (j == m - 1 || sg.x == v) f = sg.y;
                else f = __dadd_rn(__dmul_rn(sg.s, __dsub_rn(v, sg.x)), sg.y);
            }
            r = __dmul_rn((double)in[i], f);
        }
        out[i] = (TO)r;
    }
    if (n_out && outside) atomicAdd(n_out, outside);
}

int grid_for(size_t n, int per_sm) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t want = (n + 255) / 256;
    const size_t cap = (size_t)sms * per_sm;
    return (int)(want < cap ? (want ? want : 1) : cap);
}

}  // namespace

extern "C" int vg_bh_poly(const void *in, int in_f64, void *out, int out_f64, size_t n, double mu,
                          double c0, double c1, double c2, int f32mask, void *stream) {
    VG_REQUIRE(in && out, "bh_poly: null pointer");
    VG_REQUIRE(n > 0, "bh_poly: empty input");
    const int m = f32mask;
    // float32 steps follow numpy's promotion: a float32 step needs float32 inputs
    VG_REQUIRE(m >= 0 && m < 32 && !((m & 1) && in_f64) && !((m & 2) && !(m & 1)) &&
                   !((m & 4) && !(m & 1)) && !((m & 8) && !((m & 2) && (m & 4))) &&
                   !((m & 16) && !(m & 8)),
               "bh_poly: float32 step mask %d is not a numpy promotion chain", m);
    cudaStream_t st = as_stream(stream);
    const int grid = grid_for(n, 8);
    if (in_f64) {
        if (out_f64) bh_poly_kernel<double, double><<<grid, 256, 0, st>>>((const double *)in, (double *)out, n, mu, c0, c1, c2, m);
        else bh_poly_kernel<double, float><<<grid, 256, 0, st>>>((const double *)in, (float *)out, n, mu, c0, c1, c2, m);
    } else {
        if (out_f64) bh_poly_kernel<float, double><<<grid, 256, 0, st>>>((const float *)in, (double *)out, n, mu, c0, c1, c2, m);
        else bh_poly_kernel<float, float><<<grid, 256, 0, st>>>((const float *)in, (float *)out, n, mu, c0, c1, c2, m);
    }
    return launch_status("bh_poly");
}

extern "C" int vg_bh_interp(const void *in, int in_f64, void *out, int out_f64, size_t n,
                            const double *seg, const void *keys, int key_f32, int m, int mode,
                            double mu, unsigned long long *n_outside, void *stream) {
    VG_REQUIRE(in && out && seg && keys, "bh_interp: null pointer");
    VG_REQUIRE(n > 0, "bh_interp: empty input");
    VG_REQUIRE(m >= 2 && m <= VG_BH_MAX_TABLE, "bh_interp: table of %d entries (2..%d)", m,
               VG_BH_MAX_TABLE);
    VG_REQUIRE(mode >= 0 && mode <= 2, "bh_interp: mode %d (0 interp1d, 1/2 np.interp)", mode);
    VG_REQUIRE(!(mode == 1 && in_f64), "bh_interp: mode 1 divides a float32 sinogram");
    // float32 keys decide exactly only for float32 samples
    VG_REQUIRE(!key_f32 || (mode == 0 && !in_f64) || mode == 1,
               "bh_interp: float32 keys need float32 samples (mode 0 on float32, or mode 1)");
    VG_REQUIRE(((uintptr_t)seg & 15) == 0, "bh_interp: table rows must be 16-byte aligned");
    cudaStream_t st = as_stream(stream);
    const size_t smem = (size_t)m * (key_f32 ? sizeof(float) : sizeof(double));
    const int grid = grid_for(n, 8);
    auto launch = [&](auto kern, auto *ip, auto *op) -> int {
        kern<<<grid, 256, smem, st>>>(ip, op, n, reinterpret_cast<const Seg *>(seg), keys, m,
                                      mode, mu, n_outside);
        return launch_status("bh_interp");
    };
    if (key_f32) {
        if (out_f64) return launch(bh_interp_kernel<float, double, true>, (const float *)in, (double *)out);
        return launch(bh_interp_kernel<float, float, true>, (const float *)in, (float *)out);
    }
    if (in_f64) {
        if (out_f64) return launch(bh_interp_kernel<double, double, false>, (const double *)in, (double *)out);
        return launch(bh_interp_kernel<double, float, false>, (const double *)in, (float *)out);
    }
    if (out_f64) return launch(bh_interp_kernel<float, double, false>, (const float *)in, (double *)out);
    return launch(bh_interp_kernel<float, float, false>, (const float *)in, (float *)out);
}
