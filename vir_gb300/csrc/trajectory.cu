// Helical rebinning front-end (vir's trajectory.py) on the device.
//
//  vg_rebin_rows: the row gathers of sino_hel2axl / sino_hel2axl180 /
//    sino_hel2hel (trajectory.py:70-240): output row o (one interpolated
//    slice of one target view) is
//        out[o, c] = float32(src[v0, r0, c] w0 + src[v1, r1, c] w1)
//    in float64 with each operation separately rounded, as numpy evaluates
//    the float32 rows times the float64 weights and stores into float32.
//    The (view, row) pairs and weights come from the geometry's interpZ on
//    the host; `reverse` writes column c to nc - 1 - c (the [..., ::-1] of
//    sino_hel2axl180).
//  vg_axl2hel: sino_axl2hel (trajectory.py:45-67): helical view i samples the
//    axial sinogram at fractional axial view a_i, rows r + z_i and integer
//    columns c with scipy.ndimage.map_coordinates(order=1): per dimension
//    the weights (1 - f, 1 - (1 - f)), each neighbour's value times the
//    weights in dimension order, the 2^3 neighbours summed last dimension
//    fastest, in float64.  mode 'constant' (cval 0): a sample any of whose
//    coordinates lies outside [0, n - 1] is 0; views past the last axial
//    angle (wrap_i) use 'grid-wrap' on rows and columns clipped to the
//    detector, the axial view index wrapping to 0.  The column weights are
//    (1, 0): the zero-weight neighbour is skipped (finite data).
//  vg_rotsum_fp: forward_project_phantom (trajectory.py:17-42): per view the
//    phantom is sampled at M (x, y, z, 1) for every voxel (x, y, z) -- M the
//    view's 3 x 4 float32 affine matrix, each coordinate rounded to 6
//    decimals as np.round does in float32 -- trilinearly with the same
//    weights and cval 0 (in float32), and summed along y:
//    sino[view, z, x] = sum_y.  Lanes run along z (z fastest in the
//    phantom), so a warp's neighbour reads coalesce.
#include "vg_common.cuh"

namespace {

using namespace vg;

__global__ void __launch_bounds__(256)
rebin_rows_kernel(const float *__restrict__ src, int nv, int nr, int nc, const int4 *__restrict__ pairs,
                  const double2 *__restrict__ w, int n_out, int reverse, float *__restrict__ dst,
                  unsigned long long *__restrict__ n_bad) {
    const int o = blockIdx.y;
    const int4 p = pairs[o];
    const double2 ww = w[o];
    const bool ok = p.x >= 0 && p.x < nv && p.y >= 0 && p.y < nr && p.z >= 0 && p.z < nv &&
                    p.w >= 0 && p.w < nr;
    if (!ok) {
        if (n_bad && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(n_bad, 1ull);
        return;
    }
    const float *a = src + ((size_t)p.x * nr + p.y) * nc;
    const float *b = src + ((size_t)p.z * nr + p.w) * nc;
    float *d = dst + (size_t)o * nc;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const double v = __dadd_rn(__dmul_rn((double)__ldg(a + c), ww.x),
                                   __dmul_rn((double)__ldg(b + c), ww.y));
        d[reverse ? nc - 1 - c : c] = (float)v;
    }
}

// map_coordinates order-1 weights of coordinate x in [i, i + 1)
__device__ __forceinline__ void lin_w(double x, int &i, double &w0, double &w1) {
    const double fl = floor(x);
    i = (int)fl;
    const double f = __dsub_rn(x, fl);
    w0 = __dsub_rn(1.0, f);
    w1 = __dsub_rn(1.0, w0);
}

__global__ void __launch_bounds__(256)
axl2hel_kernel(const float *__restrict__ A, int na, int nr, int nc, const double *__restrict__ va,
               const double *__restrict__ vz, const int *__restrict__ wrap, int nrh,
               float *__restrict__ out) {
    const int i = blockIdx.y;                 // helical view
    const double a = va[i], z = vz[i];
    const bool wr = wrap[i] != 0;
    const size_t n = (size_t)nrh * nc;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e / nc), c = (int)(e - (size_t)r * nc);
        double y = __dadd_rn((double)r, z);
        double t = 0.0;
        if (!wr) {
            if (!(a >= 0.0 && a <= (double)(na - 1) && y >= 0.0 && y <= (double)(nr - 1))) {
                out[(size_t)i * n + e] = 0.f;
                continue;
            }
        } else {
            y = fmin(fmax(y, 0.0), (double)(nr - 1));
        }
        int ia, iy;
        double wa0, wa1, wy0, wy1;
        lin_w(a, ia, wa0, wa1);
        lin_w(y, iy, wy0, wy1);
#pragma unroll
        for (int da = 0; da < 2; ++da) {
            int ja = ia + da;
            if (wr) ja = ja >= na ? ja - na : ja;
            const double wa = da ? wa1 : wa0;
#pragma unroll
            for (int dy = 0; dy < 2; ++dy) {
                int jy = iy + dy;
                if (wr) jy = jy >= nr ? jy - nr : jy;
                const double wy = dy ? wy1 : wy0;
                // out-of-range neighbours (weight 0 at the last index) read as cval 0
                const double v = (ja >= 0 && ja < na && jy >= 0 && jy < nr)
                                     ? (double)__ldg(A + ((size_t)ja * nr + jy) * nc + c)
                                     : 0.0;
                t = __dadd_rn(t, __dmul_rn(__dmul_rn(v, wa), wy));  // x column weight 1
            }
        }
        out[(size_t)i * n + e] = (float)t;
    }
}

// np.round(x, 6) of a float32 value: rint(x * 1e6) / 1e6 in float32
__device__ __forceinline__ float round6(float x) {
    return __fdiv_rn(rintf(__fmul_rn(x, 1e6f)), 1e6f);
}

__device__ __forceinline__ void lin_wf(float x, int &i, float &w0, float &w1) {
    const float fl = floorf(x);
    i = (int)fl;
    const float f = __fsub_rn(x, fl);
    w0 = __fsub_rn(1.f, f);
    w1 = __fsub_rn(1.f, w0);
}

// block = 32 z (lanes) x 8 x (warps); grid = (ceil(nz/32), ceil(nx/8), views)
__global__ void __launch_bounds__(256)
rotsum_fp_kernel(const float *__restrict__ vol, int nx, int ny, int nz, const float *__restrict__ M,
                 float *__restrict__ sino) {
    const int iv = blockIdx.z;
    const int z = blockIdx.x * 32 + threadIdx.x, x = blockIdx.y * 8 + threadIdx.y;
    if (z >= nz || x >= nx) return;
    const float *m = M + 12 * iv;
    float acc = 0.f;
    for (int y = 0; y < ny; ++y) {
        float c[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const float *row = m + 4 * r;
            const float s = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(row[0], (float)x),
                                                          __fmul_rn(row[1], (float)y)),
                                                __fmul_rn(row[2], (float)z)),
                                      row[3]);
            c[r] = round6(s);
        }
        if (!(c[0] >= 0.f && c[0] <= (float)(nx - 1) && c[1] >= 0.f && c[1] <= (float)(ny - 1) &&
              c[2] >= 0.f && c[2] <= (float)(nz - 1)))
            continue;  // cval 0
        int i0, i1, i2;
        float a0, a1, b0, b1, d0, d1;
        lin_wf(c[0], i0, a0, a1);
        lin_wf(c[1], i1, b0, b1);
        lin_wf(c[2], i2, d0, d1);
        float t = 0.f;
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const int j0 = i0 + p;
            const float wa = p ? a1 : a0;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int j1 = i1 + q;
                const float wb = q ? b1 : b0;
#pragma unroll
                for (int s = 0; s < 2; ++s) {
                    const int j2 = i2 + s;
                    const float wd = s ? d1 : d0;
                    const float v = (j0 < nx && j1 < ny && j2 < nz)
                                        ? __ldg(vol + ((size_t)j0 * ny + j1) * nz + j2)
                                        : 0.f;
                    t = __fadd_rn(t, __fmul_rn(__fmul_rn(__fmul_rn(v, wa), wb), wd));
                }
            }
        }
        acc = __fadd_rn(acc, t);
    }
    sino[((size_t)iv * nz + z) * nx + x] = acc;
}

}  // namespace

extern "C" int vg_rebin_rows(const float *src, int n_views, int n_rows, int n_cols, const int *pairs,
                             const double *weights, int n_out, int reverse, float *dst,
                             unsigned long long *n_bad, void *stream) {
    VG_REQUIRE(src && pairs && weights && dst, "rebin_rows: null pointer");
    VG_REQUIRE(n_views > 0 && n_rows > 0 && n_cols > 0 && n_out > 0 && n_out < 65536 * 1024,
               "rebin_rows: bad sizes");
    VG_REQUIRE((((uintptr_t)pairs) & 15) == 0 && (((uintptr_t)weights) & 15) == 0,
               "rebin_rows: index and weight tables must be 16-byte aligned");
    VG_REQUIRE(n_out < 65536, "rebin_rows: at most 65535 output rows per call");
    dim3 grid(ceil_div(n_cols, 256) < 8 ? ceil_div(n_cols, 256) : 8, n_out);
    rebin_rows_kernel<<<grid, 256, 0, as_stream(stream)>>>(
        src, n_views, n_rows, n_cols, reinterpret_cast<const int4 *>(pairs),
        reinterpret_cast<const double2 *>(weights), n_out, reverse, dst, n_bad);
    return launch_status("rebin_rows");
}

extern "C" int vg_axl2hel(const float *sinoA, int n_angs, int n_rows, int n_cols,
                          const double *view_index, const double *z_shift, const int *wrap,
                          int n_views_h, int n_rows_h, float *sinoH, void *stream) {
    VG_REQUIRE(sinoA && view_index && z_shift && wrap && sinoH, "axl2hel: null pointer");
    VG_REQUIRE(n_angs > 0 && n_rows > 0 && n_cols > 0 && n_views_h > 0 && n_rows_h > 0,
               "axl2hel: sizes must be positive");
    VG_REQUIRE(n_views_h < 65536, "axl2hel: at most 65535 helical views per call");
    const long long per = (long long)n_rows_h * n_cols;
    const int gx = (int)(ceil_div(per, 256) < 64 ? ceil_div(per, 256) : 64);
    axl2hel_kernel<<<dim3(gx, n_views_h), 256, 0, as_stream(stream)>>>(
        sinoA, n_angs, n_rows, n_cols, view_index, z_shift, wrap, n_rows_h, sinoH);
    return launch_status("axl2hel");
}

extern "C" int vg_rotsum_fp(const float *vol, int nx, int ny, int nz, const float *mats, int n_views,
                            float *sino, void *stream) {
    VG_REQUIRE(vol && mats && sino, "rotsum_fp: null pointer");
    VG_REQUIRE(nx > 0 && ny > 0 && nz > 0 && n_views > 0 && n_views < 65536,
               "rotsum_fp: bad sizes");
    dim3 grid(ceil_div(nz, 32), ceil_div(nx, 8), n_views);
    VG_REQUIRE(grid.y < 65536, "rotsum_fp: nx too large");
    rotsum_fp_kernel<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(vol, nx, ny, nz, mats, sino);
    return launch_status("rotsum_fp");
}
