// FDK (Feldkamp-Davis-Kress) reconstruction for the circular cone-beam
// geometry of dd_fp_cone_3d: cosine pre-weight, row ramp filter along u,
// distance-weighted voxel-driven backprojection.
//
// vir has no FDK; the weights extend its fan-beam specification to
// the cone: the equispaced pre-weight of processing/reconstruction.py:99-107
// becomes DSD / sqrt(DSD^2 + u^2 + v^2) on the flat detector, the filter is
// filtration.filter_sino's 2H at the isocentre pitch du DSO / DSD, and the
// backprojection carries the 1/U^2 weight of processing/proj2.py:606-613:
//     f(x, y, z) = pi / (2 na) sum_views Q(u, v) / U^2,
//     o = c x + s y, p = -s x + c y, U = (DSO - o) / DSO,
//     u = DSD p / (DSO - o), v = DSD z / (DSO - o),
// with Q bilinearly interpolated between bin centres (zero outside).
#include "vg_common.cuh"

namespace {

using namespace vg;

// (na, nu, nv) -> weighted (na, nv, nu)
__global__ void fdk_weight_transpose(vg_dd3d_geom g, const float *__restrict__ in,
                                     float *__restrict__ out) {
    __shared__ float tile[32][33];
    const int ia = blockIdx.z;
    const int v0 = blockIdx.x * 32, u0 = blockIdx.y * 32;
    const float *src = in + (size_t)ia * g.nu * g.nv;
    float *dst = out + (size_t)ia * g.nu * g.nv;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int iu = u0 + q, iv = v0 + threadIdx.x;
        if (iu < g.nu && iv < g.nv) {
            const float u = g.du * ((float)iu - 0.5f * g.nu + 0.5f + g.su);
            const float v = g.dv * ((float)iv - 0.5f * g.nv + 0.5f + g.sv);
            const float w = g.DSD * rsqrtf(g.DSD * g.DSD + u * u + v * v);
            tile[q][threadIdx.x] = src[(size_t)iu * g.nv + iv] * w;
        }
    }
    __syncthreads();
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int iv = v0 + q, iu = u0 + threadIdx.x;
        if (iu < g.nu && iv < g.nv) dst[(size_t)iv * g.nu + iu] = tile[threadIdx.x][q];
    }
}

// (na, nv, nu) -> (na, nu, nv)
__global__ void fdk_transpose_back(vg_dd3d_geom g, const float *__restrict__ in,
                                   float *__restrict__ out) {
    __shared__ float tile[32][33];
    const int ia = blockIdx.z;
    const int u0 = blockIdx.x * 32, v0 = blockIdx.y * 32;
    const float *src = in + (size_t)ia * g.nu * g.nv;
    float *dst = out + (size_t)ia * g.nu * g.nv;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int iv = v0 + q, iu = u0 + threadIdx.x;
        if (iu < g.nu && iv < g.nv) tile[q][threadIdx.x] = src[(size_t)iv * g.nu + iu];
    }
    __syncthreads();
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int iu = u0 + q, iv = v0 + threadIdx.x;
        if (iu < g.nu && iv < g.nv) dst[(size_t)iu * g.nv + iv] = tile[threadIdx.x][q];
    }
}

// Thread = FZ consecutive slices of one (x, y) column; the u coordinate,
// 1 / U and the u interpolation are shared by the column's slices.  The
// view table is converted to float once per block into shared memory.
#ifndef VG_FDK_FZ
#define VG_FDK_FZ 4
#endif
constexpr int FZ = VG_FDK_FZ;

__global__ void __launch_bounds__(256)
fdk_bp_kernel(vg_dd3d_geom g, const float *__restrict__ q, const double *__restrict__ trig,
              float scale, float *__restrict__ vol) {
    extern __shared__ float2 cs[];  // (cos, sin) per view
    for (int ia = threadIdx.y * 32 + threadIdx.x; ia < g.na; ia += 256)
        cs[ia] = make_float2((float)__ldg(trig + 2 * ia), (float)__ldg(trig + 2 * ia + 1));
    __syncthreads();
    const int zb = (blockIdx.x * 32 + threadIdx.x) * FZ;
    const int iy = blockIdx.y * 8 + threadIdx.y;
    const int ix = blockIdx.z;
    if (zb >= g.nz || iy >= g.ny) return;
    const float x = g.d_pix * ((float)ix + 0.5f - 0.5f * g.nx);
    const float y = g.d_pix * ((float)iy + 0.5f - 0.5f * g.ny);
    float z[FZ];
#pragma unroll
    for (int t = 0; t < FZ; ++t) z[t] = g.d_pix * ((float)(zb + t) + 0.5f - 0.5f * g.nz);
    const float iu_off = 0.5f * g.nu - 0.5f - g.su, iv_off = 0.5f * g.nv - 0.5f - g.sv;
    const float idu = 1.0f / g.du, idv = 1.0f / g.dv;
    // per-view terms summed in groups of 16 views, the group sums compensated
    Kahan acc[FZ];
    float grp[FZ];
#pragma unroll
    for (int t = 0; t < FZ; ++t) grp[t] = 0.f;
    for (int ia = 0; ia < g.na; ++ia) {
        const float2 t2 = cs[ia];
        const float c = t2.x, s = t2.y;
        const float d = g.DSO - fmaf(c, x, s * y);
        const float r = 1.0f / d;
        const float p = fmaf(-s, x, c * y);
        const float tu = g.DSD * p * r * idu + iu_off;
        const float fu = floorf(tu);
        const int ju = (int)fu;
        const float au = tu - fu;
        const float Ui = g.DSO * r;  // 1 / U
        const float w = Ui * Ui;
        const bool uin = ju >= 0 && ju + 1 < g.nu;
        const float *Qa = q + (size_t)ia * g.nu * g.nv;
        const float zr = g.DSD * r * idv;
#pragma unroll
        for (int t = 0; t < FZ; ++t) {
            const float tv = fmaf(z[t], zr, iv_off);
            const float fv = floorf(tv);
            const int jv = (int)fv;
            const float av = tv - fv;
            float q00, q01, q10, q11;
            if (uin && jv >= 0 && jv + 1 < g.nv) {
                const float *Q = Qa + (size_t)ju * g.nv + jv;
                q00 = __ldg(Q); q01 = __ldg(Q + 1);
                q10 = __ldg(Q + g.nv); q11 = __ldg(Q + g.nv + 1);
            } else {
                auto at = [&](int dj, int k) -> float {
                    const int j = ju + dj;
                    return (j >= 0 && j < g.nu && k >= 0 && k < g.nv) ? __ldg(Qa + (size_t)j * g.nv + k) : 0.f;
                };
                q00 = at(0, jv); q01 = at(0, jv + 1); q10 = at(1, jv); q11 = at(1, jv + 1);
            }
            const float a = fmaf(av, q01 - q00, q00), b = fmaf(av, q11 - q10, q10);
            grp[t] = fmaf(fmaf(au, b - a, a), w, grp[t]);
        }
        if ((ia & 15) == 15) {
#pragma unroll
            for (int t = 0; t < FZ; ++t) { acc[t].add(grp[t]); grp[t] = 0.f; }
        }
    }
#pragma unroll
    for (int t = 0; t < FZ; ++t) {
        acc[t].add(grp[t]);
        if (zb + t < g.nz) vol[((size_t)ix * g.ny + iy) * g.nz + zb + t] = acc[t].s * scale;
    }
}

int check(const vg_dd3d_geom *g) {
    VG_REQUIRE(g && g->nx > 0 && g->ny > 0 && g->nz > 0 && g->na > 0 && g->nu > 0 && g->nv > 0,
               "fdk: sizes must be positive");
    VG_REQUIRE(g->nx < 65536 && g->na < 65536 && ceil_div(g->ny, 8) < 65536 &&
                   ceil_div(g->nu, 32) < 65536, "fdk: sizes too large");
    VG_REQUIRE(g->du > 0.f && g->dv > 0.f && g->d_pix > 0.f && g->DSO > 0.f && g->DSD > 0.f,
               "fdk: pitches and distances must be positive");
    return VG_OK;
}

}  // namespace

extern "C" int vg_fdk_weight_transpose(const vg_dd3d_geom *g, const float *sino, float *out,
                                       void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(sino && out, "fdk_weight_transpose: null pointer");
    dim3 grid(ceil_div(g->nv, 32), ceil_div(g->nu, 32), g->na);
    fdk_weight_transpose<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(*g, sino, out);
    return launch_status("fdk_weight_transpose");
}

extern "C" int vg_fdk_transpose_back(const vg_dd3d_geom *g, const float *in, float *out,
                                     void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(in && out, "fdk_transpose_back: null pointer");
    dim3 grid(ceil_div(g->nu, 32), ceil_div(g->nv, 32), g->na);
    fdk_transpose_back<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(*g, in, out);
    return launch_status("fdk_transpose_back");
}

extern "C" int vg_fdk_bp(const vg_dd3d_geom *g, const float *q, const double *trig, float *vol,
                         void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(q && trig && vol, "fdk_bp: null pointer");
    const float scale = (float)(3.14159265358979323846 / (2.0 * g->na));
    const size_t smem = (size_t)g->na * sizeof(float2);
    VG_REQUIRE(smem <= 200 * 1024, "fdk_bp: more than 25600 views");
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fdk_bp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return cuda_status(e, "fdk_bp: shared memory attribute");
    }
    dim3 grid(ceil_div(g->nz, 32 * FZ), ceil_div(g->ny, 8), g->nx);
    fdk_bp_kernel<<<grid, dim3(32, 8), smem, as_stream(stream)>>>(*g, q, trig, scale, vol);
    return launch_status("fdk_bp");
}
