// Library identity, error plumbing, and the small helpers around the
// projectors: transpose and the row filter used by FBP.
#include <stdarg.h>

#include "vg_common.cuh"

namespace vg {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return VG_OK;
    set_error("%s: %s", where, cudaGetErrorString(e));
    return VG_ERR_CUDA;
}

}  // namespace vg

using namespace vg;

extern "C" int vg_version(void) { return 100; }

extern "C" const char *vg_last_error(void) { return vg::g_err; }

extern "C" const char *vg_status_string(int s) {
    switch (s) {
        case VG_OK: return "ok";
        case VG_ERR_ARG: return "bad argument";
        case VG_ERR_LAUNCH: return "kernel launch failed";
        case VG_ERR_TIMEOUT: return "device wait timed out";
        case VG_ERR_CANCELLED: return "cancelled";
        case VG_ERR_CUDA: return "CUDA error";
        default: return "unknown status";
    }
}

namespace {

// 32x32 tiles through shared memory (padded against bank conflicts).
__global__ void transpose_kernel(const float *__restrict__ in, int rows, int cols,
                                 float *__restrict__ out) {
    __shared__ float tile[32][33];
    int c = blockIdx.x * 32 + threadIdx.x;
    int r0 = blockIdx.y * 32;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        int r = r0 + q;
        if (r < rows && c < cols) tile[q][threadIdx.x] = in[(size_t)r * cols + c];
    }
    __syncthreads();
    int r = r0 + threadIdx.x;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        int cc = blockIdx.x * 32 + q;
        if (r < rows && cc < cols) out[(size_t)cc * rows + r] = tile[threadIdx.x][q];
    }
}

// One block per (256-output chunk, group of FILT_R rows).  The group's
// (weighted) input rows are staged in shared memory; each thread computes
// one output index for all FILT_R rows, so every tap it loads feeds FILT_R
// FMAs.  Sums run in blocks of 64 taps added into a running total (two-level
// summation).  Row groups are walked with a grid stride (any row count).
constexpr int FILT_R = 8;

__global__ void __launch_bounds__(256)
filter_rows_kernel(const float *__restrict__ in, int rows, int nu, const float *__restrict__ taps,
                   const float *__restrict__ row_weight, float *__restrict__ out) {
    extern __shared__ float srow[];  // [FILT_R][nu]
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (int r0 = blockIdx.y * FILT_R; r0 < rows; r0 += gridDim.y * FILT_R) {
        const int nr = min(FILT_R, rows - r0);
        __syncthreads();
        for (int e = threadIdx.x; e < FILT_R * nu; e += blockDim.x) {
            const int r = e / nu, j = e - r * nu;
            float v = 0.f;
            if (r < nr) {
                v = in[(size_t)(r0 + r) * nu + j];
                if (row_weight) v *= row_weight[j];
            }
            srow[e] = v;
        }
        __syncthreads();
        if (i < nu) {
            const float *t = taps + i + nu - 1;  // t[-j] = taps[i - j + nu - 1]
            float tot[FILT_R], blk[FILT_R];
#pragma unroll
            for (int r = 0; r < FILT_R; ++r) tot[r] = 0.f;
            for (int j0 = 0; j0 < nu; j0 += 64) {
#pragma unroll
                for (int r = 0; r < FILT_R; ++r) blk[r] = 0.f;
                const int j1 = min(nu, j0 + 64);
                for (int j = j0; j < j1; ++j) {
                    const float tv = __ldg(t - j);
#pragma unroll
                    for (int r = 0; r < FILT_R; ++r) blk[r] = fmaf(srow[r * nu + j], tv, blk[r]);
                }
#pragma unroll
                for (int r = 0; r < FILT_R; ++r) tot[r] += blk[r];
            }
#pragma unroll
            for (int r = 0; r < FILT_R; ++r)
                if (r < nr) out[(size_t)(r0 + r) * nu + i] = tot[r];
        }
    }
}

// Ordered stream compaction of the non-zero entries of a float array, in two
// launches around a scan of per-block counts: CP_ITEMS entries per block.
constexpr int CP_THREADS = 256, CP_PER = 4, CP_ITEMS = CP_THREADS * CP_PER;

__global__ void __launch_bounds__(CP_THREADS)
count_nonzero_kernel(const float *__restrict__ v, long long n, int *__restrict__ counts) {
    __shared__ int wsum[CP_THREADS / 32];
    const long long base = (long long)blockIdx.x * CP_ITEMS + (long long)threadIdx.x * CP_PER;
    int c = 0;
#pragma unroll
    for (int i = 0; i < CP_PER; ++i) c += (base + i < n && v[base + i] != 0.f) ? 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < CP_THREADS / 32; ++w) t += wsum[w];
        counts[blockIdx.x] = t;
    }
}

// first[b]: number of non-zeros before block b (exclusive scan of counts)
__global__ void __launch_bounds__(CP_THREADS)
compact_nonzero_kernel(const float *__restrict__ v, long long n, const long long *__restrict__ first,
                       int *__restrict__ idx, float *__restrict__ val) {
    __shared__ int wsum[CP_THREADS / 32];
    const long long base = (long long)blockIdx.x * CP_ITEMS + (long long)threadIdx.x * CP_PER;
    float x[CP_PER];
    int c = 0;
#pragma unroll
    for (int i = 0; i < CP_PER; ++i) {
        x[i] = base + i < n ? v[base + i] : 0.f;
        c += x[i] != 0.f ? 1 : 0;
    }
    // exclusive scan of c over the block (warp shuffles, then warp totals)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    long long pos = first[blockIdx.x] + before + inc - c;
#pragma unroll
    for (int i = 0; i < CP_PER; ++i)
        if (x[i] != 0.f) {
            idx[pos] = (int)(base + i);
            val[pos] = x[i];
            ++pos;
        }
}

}  // namespace

extern "C" int vg_compact_blocks(long long n) { return (int)((n + CP_ITEMS - 1) / CP_ITEMS); }

extern "C" int vg_count_nonzero(const float *v, long long n, int *counts, void *stream) {
    VG_REQUIRE(v && counts, "count_nonzero: null pointer");
    VG_REQUIRE(n > 0 && n < (1LL << 31), "count_nonzero: size out of range");
    count_nonzero_kernel<<<vg_compact_blocks(n), CP_THREADS, 0, as_stream(stream)>>>(v, n, counts);
    return launch_status("count_nonzero");
}

extern "C" int vg_compact_nonzero(const float *v, long long n, const long long *first, int *idx,
                                  float *val, void *stream) {
    VG_REQUIRE(v && first && idx && val, "compact_nonzero: null pointer");
    VG_REQUIRE(n > 0 && n < (1LL << 31), "compact_nonzero: size out of range");
    compact_nonzero_kernel<<<vg_compact_blocks(n), CP_THREADS, 0, as_stream(stream)>>>(v, n, first,
                                                                                      idx, val);
    return launch_status("compact_nonzero");
}

extern "C" int vg_transpose(const float *in, int rows, int cols, float *out, void *stream) {
    VG_REQUIRE(in && out, "transpose: null pointer");
    VG_REQUIRE(rows > 0 && cols > 0, "transpose: sizes must be positive");
    VG_REQUIRE(ceil_div(rows, 32) < 65536, "transpose: too many rows");
    dim3 grid(ceil_div(cols, 32), ceil_div(rows, 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(in, rows, cols, out);
    return launch_status("transpose");
}

extern "C" int vg_filter_rows(const float *in, int rows, int nu, const float *taps,
                              const float *row_weight, float *out, void *stream) {
    VG_REQUIRE(in && taps && out, "filter_rows: null pointer");
    VG_REQUIRE(rows > 0 && nu > 0, "filter_rows: bad sizes");
    const size_t smem = (size_t)FILT_R * nu * sizeof(float);
    VG_REQUIRE(smem <= 200 * 1024, "filter_rows: nu above 6400");
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(filter_rows_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_status(e, "filter_rows: shared memory attribute");
    }
    const int groups = ceil_div(rows, FILT_R);
    dim3 grid(ceil_div(nu, 256), groups < 65535 ? groups : 65535);
    filter_rows_kernel<<<grid, 256, smem, as_stream(stream)>>>(in, rows, nu, taps, row_weight,
                                                               out);
    return launch_status("filter_rows");
}
