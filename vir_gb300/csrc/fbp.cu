// Pixel-driven FBP backprojection (parallel and flat-detector fan).
//
// After ramp filtering (filtration.filter_sino, which applies 2H), the
// reconstruction of a full scan (pi parallel or 2 pi either geometry) is
//     f(x, y) = pi / (2 na) * sum_views Q(s(x, y)) / U(x, y)^2
// with, in vir's distance-driven geometry (source direction (cos, sin),
// detector axis (-sin, cos), dd.py:486-494, 527-585):
//     o = cos x + sin y,  p = -sin x + cos y,
//     parallel: s = p, U = 1;
//     fan:      s = DSD p / (DSO - o) on the detector, U = (DSO - o) / DSO,
// Q linearly interpolated between bin centres du (j - nu/2 + 0.5 + su) and
// zero outside the detector.  The fan weights are the equispaced
// (collinear-detector) ones whose pre-weight is the reference's
// cosine_weighting(equispaced=True) (processing/reconstruction.py:99-107) and
// whose distance weight is the 1/U^2 of its Hsieh backprojector
// (processing/proj2.py:606-613).
#include "vg_common.cuh"

namespace {

using namespace vg;

template <bool FAN>
__global__ void fbp2d_bp_kernel(vg_dd2d_geom g, const float *__restrict__ q,
                                const double *__restrict__ trig, float scale,
                                float *__restrict__ img) {
    int iy = blockIdx.x * 32 + threadIdx.x;
    int ix = blockIdx.y * 8 + threadIdx.y;
    if (iy >= g.ny || ix >= g.nx) return;
    float x = g.d_pix * ((float)ix + 0.5f - 0.5f * g.nx);
    float y = g.d_pix * ((float)iy + 0.5f - 0.5f * g.ny);
    float inv_du = 1.0f / g.du;
    float off = 0.5f * g.nu - 0.5f - g.su;  // s -> fractional bin index
    // per-view terms summed in groups of 16 views, the group sums compensated
    Kahan acc;
    float grp = 0.f;
    for (int ia = 0; ia < g.na; ++ia) {
        float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
        float p = -s * x + c * y;
        float w = 1.0f;
        if (FAN) {
            const float r = 1.0f / (g.DSO - (c * x + s * y));  // one division per view
            p = g.DSD * p * r;
            const float Ui = g.DSO * r;                          // 1 / U
            w = Ui * Ui;
        }
        float t = p * inv_du + off;
        float ft = floorf(t);
        int j = (int)ft;
        float a = t - ft;
        const float *row = q + (size_t)ia * g.nu;
        float v0 = (j >= 0 && j < g.nu) ? __ldg(row + j) : 0.f;
        float v1 = (j + 1 >= 0 && j + 1 < g.nu) ? __ldg(row + j + 1) : 0.f;
        grp = fmaf(w, fmaf(a, v1 - v0, v0), grp);
        if ((ia & 15) == 15) {
            acc.add(grp);
            grp = 0.f;
        }
    }
    acc.add(grp);
    img[(size_t)ix * g.ny + iy] = acc.s * scale;
}

}  // namespace

extern "C" int vg_fbp2d_bp(const vg_dd2d_geom *g, const float *q, const double *trig, float *img,
                           void *stream) {
    VG_REQUIRE(g && q && trig && img, "fbp2d_bp: null pointer");
    VG_REQUIRE(g->nx > 0 && g->ny > 0 && g->na > 0 && g->nu > 0, "fbp2d_bp: bad sizes");
    VG_REQUIRE(g->du > 0.f && g->d_pix > 0.f, "fbp2d_bp: du and d_pix must be positive");
    VG_REQUIRE(!g->fan || (g->DSO > 0.f && g->DSD > 0.f), "fbp2d_bp: fan needs DSO, DSD > 0");
    dim3 grid(ceil_div(g->ny, 32), ceil_div(g->nx, 8));
    VG_REQUIRE(grid.y < 65536, "fbp2d_bp: nx too large");
    float scale = (float)(3.14159265358979323846 / (2.0 * g->na));
    if (g->fan)
        fbp2d_bp_kernel<true><<<grid, dim3(32, 8), 0, as_stream(stream)>>>(*g, q, trig, scale, img);
    else
        fbp2d_bp_kernel<false><<<grid, dim3(32, 8), 0, as_stream(stream)>>>(*g, q, trig, scale, img);
    return launch_status("fbp2d_bp");
}
