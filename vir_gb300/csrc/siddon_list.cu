// Siddon ray lists (sys_mat/siddon.py:636-833) and list projection
// (projection/projection_c.c:126-219, projection/proj.py:56-150).
//
// siddons() does its per-ray set-up vectorised (alpha range, first/last
// plane index with isclose rounding) and spends its time in a per-ray loop
// that sorts all plane crossings and turns consecutive pairs into (voxel,
// length) entries.  siddons_setup_kernel computes the set-up, one thread per
// ray, in the types and operation order of the reference's numpy code; the
// count and fill kernels run the per-ray loop, one thread per ray, in FP32
// with the reference's operation order (every op separately rounded):
//   crossings  (b_i - src)/dST for i in [i0, iN) per axis with dST != 0     (:771-784)
//   Alpha      sort(bounds, crossings); the first/last element dropped when
//              isclose (|a - b| <= 1e-8 + 1e-5 |b| in float32) to its neighbour (:787-793)
//   segment    voxel = trunc((src + (0.5 (a + b)) dST - b_0) / d)            (:796-801)
//              length = float32(distance * (b - a)), kept when > 0            (:803-809)
// The crossing sequences of each axis are monotone in the plane index, so
// the sort is a merge of five sorted sources (3 axes + 2 bounds).
// When a direction component is zero the reference concatenates an empty
// float64 array into Alpha (:774-787), which promotes that ray's sorted list,
// midpoints, isclose tests and lengths to float64; such rays take the FP64
// branch here (the crossing values themselves stay float32 numbers).
// The kernel runs twice: counting entries per ray, then writing them at the
// offsets of an exclusive scan of the counts (CSR: ind, len, off).
#include <type_traits>

#include "vg_common.cuh"

namespace {

using namespace vg;

__device__ __forceinline__ float f_isclose_tol(float y) {
    return __fadd_rn(1e-8f, __fmul_rn(1e-5f, fabsf(y)));
}
__device__ __forceinline__ bool f_isclose(float x, float y) {
    return (fabsf(__fsub_rn(x, y)) <= f_isclose_tol(y) && isfinite(y)) || x == y;
}
__device__ __forceinline__ bool d_isclose(double x, double y) {
    return (fabs(__dsub_rn(x, y)) <= __dadd_rn(1e-8, __dmul_rn(1e-5, fabs(y))) && isfinite(y)) ||
           x == y;
}

// Walks the merged, sorted crossing list of one ray and calls emit(ix, iy,
// iz, len) for every kept segment.  Returns false if a voxel index falls
// outside the grid (the reference raises in ravel_multi_index then).
template <bool F64, typename Emit>
__device__ bool walk_ray(const vg_siddon_rays &R, int r, Emit emit) {
    using T = typename std::conditional<F64, double, float>::type;
    float s[3], d[3];
    int i0[3], iN[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        s[a] = R.src[3 * r + a];
        d[a] = R.dst[3 * r + a];
        i0[a] = R.i0[3 * r + a];
        iN[a] = R.iN[3 * r + a];
    }
    const float *bnd[3] = {R.xb, R.yb, R.zb};
    const int np[3] = {R.nx, R.ny, R.nz};
    const float dp[3] = {R.dx, R.dy, R.dz};
    // per axis: next plane index in increasing-alpha order and remaining count
    int idx[3], left[3], step[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int n = (d[a] != 0.f) ? iN[a] - i0[a] : 0;
        if (n < 0) n = 0;
        left[a] = n;
        step[a] = d[a] > 0.f ? 1 : -1;
        idx[a] = d[a] > 0.f ? i0[a] : iN[a] - 1;
    }
    auto cross = [&](int a) -> float {
        return __fdiv_rn(__fsub_rn(__ldg(bnd[a] + idx[a]), s[a]), d[a]);
    };
    float head[5];
    bool has[5];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        has[a] = left[a] > 0;
        head[a] = has[a] ? cross(a) : 0.f;
    }
    head[3] = R.amin[r]; has[3] = true;
    head[4] = R.amax[r]; has[4] = true;
    const int total = 2 + left[0] + left[1] + left[2];
    const float dist = R.dist[r];
    const float b0[3] = {__ldg(R.xb), __ldg(R.yb), __ldg(R.zb)};

    auto pop = [&]() -> float {
        int best = -1;
        float bv = 0.f;
#pragma unroll
        for (int q = 0; q < 5; ++q)
            if (has[q] && (best < 0 || head[q] < bv)) { best = q; bv = head[q]; }
        if (best < 3) {
            if (--left[best] > 0) { idx[best] += step[best]; head[best] = cross(best); }
            else has[best] = false;
        } else {
            has[best] = false;
        }
        return bv;
    };

    bool ok = true;
    auto segment = [&](float fa0, float fa1) {
        float len;
        int ind[3];
        if (F64) {
            const double a0 = fa0, a1 = fa1;
            const double dA = __dsub_rn(a1, a0);
            const double mA = __dmul_rn(0.5, __dadd_rn(a1, a0));
            len = (float)__dmul_rn((double)dist, dA);
            if (!(len > 0.f)) return;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const double p = __dsub_rn(__dadd_rn((double)s[a], __dmul_rn(mA, (double)d[a])),
                                           (double)b0[a]);
                const double q = __ddiv_rn(p, (double)dp[a]);
                ind[a] = (int)q;
                if (!(q > -1.0) || !(q < (double)np[a])) ok = false;
            }
        } else {
            const float dA = __fsub_rn(fa1, fa0);
            const float mA = __fmul_rn(0.5f, __fadd_rn(fa1, fa0));
            len = __fmul_rn(dist, dA);
            if (!(len > 0.f)) return;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float p = __fsub_rn(__fadd_rn(s[a], __fmul_rn(mA, d[a])), b0[a]);
                const float q = __fdiv_rn(p, dp[a]);
                ind[a] = (int)q;  // truncation toward zero, as astype(np.int32)
                if (!(q > -1.f) || !(q < (float)np[a])) ok = false;
            }
        }
        if (ok) emit(ind[0], ind[1], ind[2], len);
    };
    auto close = [&](float x, float y) { return F64 ? d_isclose(x, y) : f_isclose(x, y); };

    // sorted list A[0..total-1]; drop A[0] if isclose(A[0], A[1]); then drop
    // the last if isclose(A[last], A[last-1]); segments between neighbours.
    float A0 = pop(), A1 = pop();
    int n = total;
    int k = 2;  // elements popped so far
    float prev, cur;
    if (close(A0, A1)) {
        --n;
        prev = A1;
        if (k < total) { cur = pop(); ++k; } else { return ok; }
    } else {
        prev = A0;
        cur = A1;
    }
    // pairs (prev, cur); the final pair is emitted unless the last element is dropped
    while (true) {
        if (k == total) {
            // cur is the last element; prev its predecessor
            if (!close(cur, prev)) segment(prev, cur);
            break;
        }
        const float nxt = pop();
        ++k;
        segment(prev, cur);
        prev = cur;
        cur = nxt;
    }
    (void)n;
    return ok;
}

__device__ __forceinline__ bool has_zero_dir(const vg_siddon_rays &R, int r) {
    return R.dst[3 * r] == 0.f || R.dst[3 * r + 1] == 0.f || R.dst[3 * r + 2] == 0.f;
}

__global__ void siddons_count_kernel(vg_siddon_rays R, int *__restrict__ counts,
                                     int *__restrict__ err) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R.n_rays) return;
    int c = 0;
    if (R.valid[r]) {
        auto cnt = [&](int, int, int, float) { ++c; };
        const bool ok = has_zero_dir(R, r) ? walk_ray<true>(R, r, cnt) : walk_ray<false>(R, r, cnt);
        if (!ok) atomicAdd(err, 1);
    }
    counts[r] = c;
}

__global__ void siddons_fill_kernel(vg_siddon_rays R, const int *__restrict__ off,
                                    int *__restrict__ ind, float *__restrict__ len) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R.n_rays || !R.valid[r]) return;
    int o = off[r];
    const int nyz = R.ny * R.nz;
    auto put = [&](int ix, int iy, int iz, float l) {
        ind[o] = ix * nyz + iy * R.nz + iz;
        len[o] = l;
        ++o;
    };
    if (has_zero_dir(R, r)) walk_ray<true>(R, r, put);
    else walk_ray<false>(R, r, put);
}

// Gather FP over a CSR list, one warp per ray (coalesced ind/len, lane
// partial Kahan sums, shuffle reduction).
__global__ void list_fp_kernel(const float *__restrict__ x, const int *__restrict__ ind,
                               const float *__restrict__ len, const int *__restrict__ off,
                               int nrays, float *__restrict__ sino, int accumulate) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nrays) return;
    const int a = off[warp], b = off[warp + 1];
    Kahan k;
    for (int i = a + lane; i < b; i += 32) k.add(__ldg(x + __ldg(ind + i)) * __ldg(len + i));
    float v = k.s, c = k.c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (lane == 0) sino[warp] = (accumulate ? sino[warp] : 0.f) + (v - c);
}

// Scatter BP: FP64 atomic accumulation (order-independent to far below FP32
// rounding), then one conversion pass.
__global__ void list_bp_scatter_kernel(const float *__restrict__ sino, const int *__restrict__ ind,
                                       const float *__restrict__ len, const int *__restrict__ off,
                                       int nrays, double *__restrict__ acc) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nrays) return;
    const int a = off[warp], b = off[warp + 1];
    const double y = (double)__ldg(sino + warp);
    if (y == 0.0) return;
    for (int i = a + lane; i < b; i += 32)
        atomicAdd(acc + __ldg(ind + i), y * (double)__ldg(len + i));
}

__global__ void list_bp_finish_kernel(const double *__restrict__ acc, int nvox,
                                      float *__restrict__ x, int accumulate) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nvox) return;
    x[i] = (float)((accumulate ? (double)x[i] : 0.0) + acc[i]);
}

// The per-ray set-up of siddons (siddon.py:681-751), each operation in the
// type numpy gives it and separately rounded: float32 throughout, except the
// first plane index (nP + 1) - (pN - a dST - src) / dP, which numpy promotes
// to float64 (an int64 array minus a float32 one); np.isclose(v, round(v),
// atol=epsilon) compares in v's type with atol and rtol = 1e-5 in that type;
// np.max / np.min propagate NaN; the ray length sums the squares left to
// right before the float32 square root, as np.linalg.norm does.
__device__ __forceinline__ bool f_isclose_atol(float x, float y, float atol) {
    return (fabsf(__fsub_rn(x, y)) <= __fadd_rn(atol, __fmul_rn(1e-5f, fabsf(y))) && isfinite(y)) ||
           x == y;
}
__device__ __forceinline__ bool d_isclose_atol(double x, double y, double atol) {
    return (fabs(__dsub_rn(x, y)) <= __dadd_rn(atol, __dmul_rn(1e-5, fabs(y))) && isfinite(y)) ||
           x == y;
}
__device__ __forceinline__ float np_maximum(float a, float b) {
    return (isnan(a) || isnan(b)) ? __int_as_float(0x7fc00000) : fmaxf(a, b);
}
__device__ __forceinline__ float np_minimum(float a, float b) {
    return (isnan(a) || isnan(b)) ? __int_as_float(0x7fc00000) : fminf(a, b);
}
// astype(int32) of an integral value as numpy gives it: values outside the
// int32 range and NaN become INT_MIN (the x86 conversion's result)
__device__ __forceinline__ int np_int32(double v) {
    return (v >= -2147483648.0 && v < 2147483648.0) ? (int)v : (int)0x80000000;
}
// g.Xb[i0:iN] slice bound of an int32 index over n + 1 planes
__device__ __forceinline__ int slice_bound(int i, int L) {
    const long long j = i < 0 ? (long long)i + L : (long long)i;
    return (int)(j < 0 ? 0 : (j > L ? L : j));
}

__global__ void __launch_bounds__(128)
siddons_setup_kernel(vg_siddons_grid G, int n, const float *__restrict__ src,
                     const float *__restrict__ trg, float *__restrict__ dst,
                     float *__restrict__ dist, float *__restrict__ amin_o,
                     float *__restrict__ amax_o, int *__restrict__ i0_o, int *__restrict__ iN_o,
                     unsigned char *__restrict__ valid_o) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int np[3] = {G.nx, G.ny, G.nz};
    const float dp[3] = {G.dx, G.dy, G.dz};
    const float epsf = G.epsilon_f;
    float s[3], d[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        s[a] = src[3 * (size_t)r + a];
        d[a] = __fsub_rn(trg[3 * (size_t)r + a], s[a]);
        dst[3 * (size_t)r + a] = d[a];
    }
    dist[r] = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])),
                                   __fmul_rn(d[2], d[2])));
    // alpha range: m_min = [0, per-axis min], m_max = [1, per-axis max]
    float amin = 0.f, amax = 1.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float den = d[a] != 0.f ? d[a] : epsf;
        const float a0 = __fdiv_rn(__fsub_rn(G.p0[a], s[a]), den);
        const float aN = __fdiv_rn(__fsub_rn(G.pN[a], s[a]), den);
        const bool lt = a0 < aN, gt = a0 > aN;
        amin = np_maximum(amin, lt ? a0 : (gt ? aN : 0.f));
        amax = np_minimum(amax, lt ? aN : (gt ? a0 : 1.f));
    }
    amin_o[r] = amin;
    amax_o[r] = amax;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const bool pos = d[a] > 0.f;
        const float a_lo = pos ? amin : amax, a_hi = pos ? amax : amin;
        const float t = __fdiv_rn(__fsub_rn(__fsub_rn(G.pN[a], __fmul_rn(a_lo, d[a])), s[a]), dp[a]);
        const double v0 = __dsub_rn((double)(np[a] + 1), (double)t);
        const float vN = __fdiv_rn(__fsub_rn(__fadd_rn(s[a], __fmul_rn(a_hi, d[a])), G.p0[a]), dp[a]);
        const double r0 = rint(v0);
        const float rN = rintf(vN);
        const double f0 = d_isclose_atol(v0, r0, G.epsilon) ? r0 : floor(v0);
        const float fN = f_isclose_atol(vN, rN, epsf) ? rN : ceilf(vN);
        const int L = np[a] + 1;
        i0_o[3 * (size_t)r + a] = slice_bound(np_int32(f0), L);
        iN_o[3 * (size_t)r + a] = slice_bound(np_int32((double)fN), L);
    }
    valid_o[r] = (amax > amin) && !f_isclose_atol(amax, amin, epsf);
}

int check_rays(const vg_siddon_rays *R) {
    VG_REQUIRE(R, "siddons: null ray set");
    VG_REQUIRE(R->n_rays >= 0, "siddons: negative ray count");
    VG_REQUIRE(R->nx > 0 && R->ny > 0 && R->nz > 0, "siddons: grid sizes must be positive");
    VG_REQUIRE((long long)R->nx * R->ny * R->nz < (1ll << 31), "siddons: grid above 2^31 voxels");
    VG_REQUIRE(R->xb && R->yb && R->zb && R->src && R->dst && R->dist && R->amin && R->amax &&
               R->i0 && R->iN && R->valid, "siddons: null array");
    return VG_OK;
}

}  // namespace

extern "C" int vg_siddons_setup(const vg_siddons_grid *g, int n, const float *src,
                                const float *trg, float *dst, float *dist, float *amin,
                                float *amax, int *i0, int *iN, unsigned char *valid,
                                void *stream) {
    VG_REQUIRE(g, "siddons_setup: null grid");
    VG_REQUIRE(n >= 0, "siddons_setup: negative ray count");
    VG_REQUIRE(g->nx > 0 && g->ny > 0 && g->nz > 0, "siddons_setup: grid sizes must be positive");
    VG_REQUIRE(n == 0 || (src && trg && dst && dist && amin && amax && i0 && iN && valid),
               "siddons_setup: null array");
    if (n == 0) return VG_OK;
    siddons_setup_kernel<<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(
        *g, n, src, trg, dst, dist, amin, amax, i0, iN, valid);
    return launch_status("siddons_setup");
}

extern "C" int vg_siddons_count(const vg_siddon_rays *R, int *counts, int *err, void *stream) {
    int st = check_rays(R);
    if (st) return st;
    VG_REQUIRE(counts && err, "siddons_count: null pointer");
    if (R->n_rays == 0) return VG_OK;
    siddons_count_kernel<<<ceil_div(R->n_rays, 128), 128, 0, as_stream(stream)>>>(*R, counts, err);
    return launch_status("siddons_count");
}

extern "C" int vg_siddons_fill(const vg_siddon_rays *R, const int *off, int *ind, float *len,
                               void *stream) {
    int st = check_rays(R);
    if (st) return st;
    VG_REQUIRE(off && ind && len, "siddons_fill: null pointer");
    if (R->n_rays == 0) return VG_OK;
    siddons_fill_kernel<<<ceil_div(R->n_rays, 128), 128, 0, as_stream(stream)>>>(*R, off, ind, len);
    return launch_status("siddons_fill");
}

extern "C" int vg_list_fp(const float *x, const int *ind, const float *len, const int *off,
                          int nrays, float *sino, int accumulate, void *stream) {
    VG_REQUIRE(nrays >= 0, "list_fp: negative ray count");
    if (nrays == 0) return VG_OK;
    VG_REQUIRE(x && ind && len && off && sino, "list_fp: null pointer");
    list_fp_kernel<<<ceil_div((long long)nrays * 32, 256), 256, 0, as_stream(stream)>>>(
        x, ind, len, off, nrays, sino, accumulate);
    return launch_status("list_fp");
}

extern "C" size_t vg_list_bp_workspace_bytes(int nvox) {
    return nvox > 0 ? (size_t)nvox * sizeof(double) : 0;
}

extern "C" int vg_list_bp(const float *sino, const int *ind, const float *len, const int *off,
                          int nrays, int nvox, float *x, int accumulate, void *workspace,
                          size_t workspace_bytes, void *stream) {
    VG_REQUIRE(nrays >= 0 && nvox > 0, "list_bp: bad sizes");
    VG_REQUIRE(sino && ind && len && off && x, "list_bp: null pointer");
    VG_REQUIRE(workspace && workspace_bytes >= (size_t)nvox * sizeof(double) &&
                   ((uintptr_t)workspace & 7) == 0,
               "list_bp: workspace of %zu 8-byte-aligned bytes needed", (size_t)nvox * 8);
    cudaStream_t st = as_stream(stream);
    double *acc = reinterpret_cast<double *>(workspace);
    int s = cuda_status(cudaMemsetAsync(acc, 0, (size_t)nvox * sizeof(double), st), "list_bp");
    if (s) return s;
    if (nrays > 0) {
        list_bp_scatter_kernel<<<ceil_div((long long)nrays * 32, 256), 256, 0, st>>>(
            sino, ind, len, off, nrays, acc);
        s = launch_status("list_bp_scatter");
        if (s) return s;
    }
    list_bp_finish_kernel<<<ceil_div(nvox, 256), 256, 0, st>>>(acc, nvox, x, accumulate);
    return launch_status("list_bp_finish");
}
