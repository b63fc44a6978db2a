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

// One block per (row, 256-output chunk).  The (weighted) input row is staged
// in shared memory; taps are read through L1 (consecutive outputs read
// consecutive taps).
__global__ void __launch_bounds__(256)
filter_rows_kernel(const float *__restrict__ in, int nu, const float *__restrict__ taps,
                   const float *__restrict__ row_weight, float *__restrict__ out) {
    extern __shared__ float srow[];
    int r = blockIdx.y;
    const float *src = in + (size_t)r * nu;
    for (int j = threadIdx.x; j < nu; j += blockDim.x)
        srow[j] = row_weight ? src[j] * row_weight[j] : src[j];
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nu) return;
    const float *t = taps + i + nu - 1;  // t[-j] = taps[i - j + nu - 1]
    Kahan acc;
    for (int j = 0; j < nu; ++j) acc.add(srow[j] * __ldg(t - j));
    out[(size_t)r * nu + i] = acc.s;
}

}  // namespace

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
    VG_REQUIRE(rows > 0 && rows < 65536 && nu > 0, "filter_rows: bad sizes");
    VG_REQUIRE(nu <= 48 * 1024 / 4, "filter_rows: nu above 12288");
    dim3 grid(ceil_div(nu, 256), rows);
    filter_rows_kernel<<<grid, 256, nu * sizeof(float), as_stream(stream)>>>(in, nu, taps,
                                                                           row_weight, out);
    return launch_status("filter_rows");
}
