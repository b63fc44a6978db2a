// 2D separable-footprint projectors and their adjoints, gather form.
//
// Fan (sys_mat/sp.py:12-87): pixel centre (x, y) rotated to xp = c x + s y,
// yp = -s x + c y projects to u0 = DSD xp / (DSO - yp) with footprint half
// width W = DSD d_pix / (DSO - yp); bin iu (centre u_c = du (iu - nu/2 + 0.5))
// receives val * max(0, 1 - |u_c - u0| / W); the result is scaled by d_pix.
// For a fixed (view, bin) the footprint argument
//     t = (u_c - u0) / W = (A x + B y + C) / (DSD d_pix),
//     A = u_c s - DSD c,  B = -(u_c c + DSD s),  C = u_c DSO,
// is linear in (x, y): the FP thread of a bin walks the pixel lines across
// the strip |t| < 1 (one or two pixels per line) with no division.  The BP
// thread of a pixel visits, per view, the bins with |t| < 1.
//
// Parallel rectangle (sys_mat/fp_2d_par.py:67-125): a pixel's footprint is
// the interval of its four corners projected on u = cos y - sin x, half width
// h = d_pix (|cos| + |sin|) / 2 around the projected centre; bin k (edges
// d_det (k - n/2)) receives val * |footprint ∩ bin| / d_det.
#include "vg_common.cuh"

namespace {

using namespace vg;

__device__ __forceinline__ float centre(float d, int i, int n) {
    return d * ((float)i + 0.5f - 0.5f * (float)n);
}

// ---- fan ----------------------------------------------------------------

__global__ void sf_fan_fp_kernel(vg_sf2d_geom g, const float *__restrict__ img,
                                 const float *__restrict__ imgT, const double *__restrict__ trig,
                                 float *__restrict__ sino) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x;
    const int ia = blockIdx.y;
    if (iu >= g.nu) return;
    const double c = __ldg(trig + 2 * ia), s = __ldg(trig + 2 * ia + 1);
    const double uc = (double)g.du * ((double)iu - 0.5 * g.nu + 0.5);
    const double K = (double)g.DSD * g.d_pix;
    // t = a x + b y + c0 (double set-up per bin, float walk)
    const double A = uc * s - g.DSD * c, B = -(uc * c + g.DSD * s), C = uc * g.DSO;
    const float a = (float)(A / K), b = (float)(B / K), c0 = (float)(C / K);
    // the pixel range of a line only has to contain the strip |t| < 1: it is
    // found with the reciprocal pitch (floor / ceil keep it conservative)
    const float idp = 1.0f / g.d_pix;
    // line terms summed in groups of 16 lines, the group sums compensated
    Kahan acc;
    float grp = 0.f;
    if (fabsf(b) >= fabsf(a)) {
        // x lines (column ix): y range of |t| < 1, read img[ix][iy] (contiguous in iy)
        const float ib = 1.0f / b;
        for (int ix = 0; ix < g.nx; ++ix) {
            const float x = centre(g.d_pix, ix, g.nx);
            const float t0 = fmaf(a, x, c0);
            const float y1 = (-1.f - t0) * ib, y2 = (1.f - t0) * ib;
            const float ylo = fminf(y1, y2), yhi = fmaxf(y1, y2);
            const int j0 = max(0, (int)floorf(fmaf(ylo, idp, 0.5f * g.ny - 0.5f)));
            const int j1 = min(g.ny - 1, (int)ceilf(fmaf(yhi, idp, 0.5f * g.ny - 0.5f)));
            for (int iy = j0; iy <= j1; ++iy) {
                const float t = fmaf(b, centre(g.d_pix, iy, g.ny), t0);
                const float w = fmaxf(0.f, 1.f - fabsf(t));
                grp = fmaf(__ldg(img + (size_t)ix * g.ny + iy), w, grp);
            }
            if ((ix & 15) == 15) { acc.add(grp); grp = 0.f; }
        }
    } else {
        const float ia_ = 1.0f / a;
        for (int iy = 0; iy < g.ny; ++iy) {
            const float y = centre(g.d_pix, iy, g.ny);
            const float t0 = fmaf(b, y, c0);
            const float x1 = (-1.f - t0) * ia_, x2 = (1.f - t0) * ia_;
            const float xlo = fminf(x1, x2), xhi = fmaxf(x1, x2);
            const int i0 = max(0, (int)floorf(fmaf(xlo, idp, 0.5f * g.nx - 0.5f)));
            const int i1 = min(g.nx - 1, (int)ceilf(fmaf(xhi, idp, 0.5f * g.nx - 0.5f)));
            for (int ix = i0; ix <= i1; ++ix) {
                const float t = fmaf(a, centre(g.d_pix, ix, g.nx), t0);
                const float w = fmaxf(0.f, 1.f - fabsf(t));
                grp = fmaf(__ldg(imgT + (size_t)iy * g.nx + ix), w, grp);
            }
            if ((iy & 15) == 15) { acc.add(grp); grp = 0.f; }
        }
    }
    acc.add(grp);
    sino[(size_t)ia * g.nu + iu] = acc.s * g.d_pix;
}

__global__ void sf_fan_bp_kernel(vg_sf2d_geom g, const float *__restrict__ sino,
                                 const double *__restrict__ trig, float *__restrict__ img) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iy >= g.ny) return;
    const float x = centre(g.d_pix, ix, g.nx), y = centre(g.d_pix, iy, g.ny);
    const float inv_du = 1.0f / g.du;
    const float iDd = 1.0f / (g.DSD * g.d_pix);
    // view terms summed in groups of 16 views, the group sums compensated
    Kahan acc;
    float grp = 0.f;
    for (int ia = 0; ia < g.na; ++ia) {
        const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
        const float xp = fmaf(c, x, s * y), yp = fmaf(-s, x, c * y);
        const float den = g.DSO - yp;
        const float r = 1.0f / den;  // one division per view
        const float u0 = g.DSD * xp * r, W = g.DSD * g.d_pix * r;
        const float iW = den * iDd;
        // bins with |u_c - u0| < W: u_c = du (iu - nu/2 + 0.5)
        const int k0 = max(0, (int)ceilf((u0 - W) * inv_du + 0.5f * g.nu - 0.5f));
        const int k1 = min(g.nu - 1, (int)floorf((u0 + W) * inv_du + 0.5f * g.nu - 0.5f));
        const float *row = sino + (size_t)ia * g.nu;
        for (int iu = k0; iu <= k1; ++iu) {
            const float uc = g.du * ((float)iu - 0.5f * g.nu + 0.5f);
            const float w = fmaxf(0.f, 1.f - fabsf((uc - u0) * iW));
            grp = fmaf(__ldg(row + iu), w, grp);
        }
        if ((ia & 15) == 15) { acc.add(grp); grp = 0.f; }
    }
    acc.add(grp);
    img[(size_t)ix * g.ny + iy] = acc.s * g.d_pix;
}

// ---- parallel rectangle ------------------------------------------------

__global__ void sf_par_fp_kernel(vg_sf2d_geom g, const float *__restrict__ img,
                                 const float *__restrict__ imgT, const double *__restrict__ trig,
                                 float *__restrict__ sino) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int ia = blockIdx.y;
    if (k >= g.nu) return;
    const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
    const float el = g.du * ((float)k - 0.5f * g.nu), er = el + g.du;
    const float h = 0.5f * g.d_pix * (fabsf(c) + fabsf(s));
    const float inv_det = 1.0f / g.du;
    Kahan acc;
    // footprint centre p = c y - s x; walk lines along the axis with the larger coefficient
    if (fabsf(c) >= fabsf(s)) {
        // x lines: p = c y - s x, y range where |p - bin| overlaps: p in (el - h, er + h)
        const float ic = 1.0f / c;
        for (int ix = 0; ix < g.nx; ++ix) {
            const float x = centre(g.d_pix, ix, g.nx);
            const float sx = s * x;
            const float y1 = (el - h + sx) * ic, y2 = (er + h + sx) * ic;
            const int j0 = max(0, (int)floorf(fminf(y1, y2) / g.d_pix + 0.5f * g.ny - 0.5f));
            const int j1 = min(g.ny - 1, (int)ceilf(fmaxf(y1, y2) / g.d_pix + 0.5f * g.ny - 0.5f));
            float part = 0.f;
            for (int iy = j0; iy <= j1; ++iy) {
                const float p = fmaf(c, centre(g.d_pix, iy, g.ny), -sx);
                const float ov = fminf(p + h, er) - fmaxf(p - h, el);
                if (ov > 0.f) part = fmaf(__ldg(img + (size_t)ix * g.ny + iy), ov, part);
            }
            acc.add(part);
        }
    } else {
        const float is = 1.0f / s;
        for (int iy = 0; iy < g.ny; ++iy) {
            const float y = centre(g.d_pix, iy, g.ny);
            const float cy = c * y;
            // p = cy - s x in (el - h, er + h)  =>  x in ((cy - er - h)/s, (cy - el + h)/s)
            const float x1 = (cy - er - h) * is, x2 = (cy - el + h) * is;
            const int i0 = max(0, (int)floorf(fminf(x1, x2) / g.d_pix + 0.5f * g.nx - 0.5f));
            const int i1 = min(g.nx - 1, (int)ceilf(fmaxf(x1, x2) / g.d_pix + 0.5f * g.nx - 0.5f));
            float part = 0.f;
            for (int ix = i0; ix <= i1; ++ix) {
                const float p = fmaf(-s, centre(g.d_pix, ix, g.nx), cy);
                const float ov = fminf(p + h, er) - fmaxf(p - h, el);
                if (ov > 0.f) part = fmaf(__ldg(imgT + (size_t)iy * g.nx + ix), ov, part);
            }
            acc.add(part);
        }
    }
    sino[(size_t)ia * g.nu + k] = acc.s * inv_det;
}

__global__ void sf_par_bp_kernel(vg_sf2d_geom g, const float *__restrict__ sino,
                                 const double *__restrict__ trig, float *__restrict__ img) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iy >= g.ny) return;
    const float x = centre(g.d_pix, ix, g.nx), y = centre(g.d_pix, iy, g.ny);
    const float inv_det = 1.0f / g.du;
    const float e0 = -0.5f * g.du * g.nu;
    Kahan acc;
    for (int ia = 0; ia < g.na; ++ia) {
        const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
        const float p = fmaf(c, y, -s * x);
        const float h = 0.5f * g.d_pix * (fabsf(c) + fabsf(s));
        const float lo = p - h, hi = p + h;
        int k = max(0, (int)floorf((lo - e0) * inv_det));
        const float *row = sino + (size_t)ia * g.nu;
        float part = 0.f;
        for (; k < g.nu; ++k) {
            const float el = fmaf(g.du, (float)k, e0), er = el + g.du;
            if (el >= hi) break;
            const float ov = fminf(hi, er) - fmaxf(lo, el);
            if (ov > 0.f) part = fmaf(__ldg(row + k), ov, part);
        }
        acc.add(part);
    }
    img[(size_t)ix * g.ny + iy] = acc.s * inv_det;
}

int check(const vg_sf2d_geom *g) {
    VG_REQUIRE(g, "sf2d: null geometry");
    VG_REQUIRE(g->nx > 0 && g->ny > 0 && g->na > 0 && g->na < 65536 && g->nu > 0,
               "sf2d: bad sizes");
    VG_REQUIRE(g->nx < 65536, "sf2d: nx too large");
    VG_REQUIRE(g->du > 0.f && g->d_pix > 0.f, "sf2d: du and d_pix must be positive");
    if (g->fan) {
        const float hx = 0.5f * g->nx * g->d_pix, hy = 0.5f * g->ny * g->d_pix;
        VG_REQUIRE(g->DSD > 0.f && sqrtf(hx * hx + hy * hy) < g->DSO,
                   "sf2d: fan needs DSD > 0 and the image inside the source circle");
    }
    return VG_OK;
}

}  // namespace

extern "C" int vg_sf2d_fp(const vg_sf2d_geom *g, const float *img, const float *imgT,
                          const double *trig, float *sino, void *stream) {
    int st = check(g);
    if (st) return st;
    VG_REQUIRE(img && imgT && trig && sino, "sf2d_fp: null pointer");
    dim3 grid(ceil_div(g->nu, 128), g->na);
    if (g->fan) sf_fan_fp_kernel<<<grid, 128, 0, as_stream(stream)>>>(*g, img, imgT, trig, sino);
    else        sf_par_fp_kernel<<<grid, 128, 0, as_stream(stream)>>>(*g, img, imgT, trig, sino);
    return launch_status("sf2d_fp");
}

extern "C" int vg_sf2d_bp(const vg_sf2d_geom *g, const float *sino, const double *trig,
                          float *img, void *stream) {
    int st = check(g);
    if (st) return st;
    VG_REQUIRE(img && trig && sino, "sf2d_bp: null pointer");
    dim3 grid(ceil_div(g->ny, 128), g->nx);
    if (g->fan) sf_fan_bp_kernel<<<grid, 128, 0, as_stream(stream)>>>(*g, sino, trig, img);
    else        sf_par_bp_kernel<<<grid, 128, 0, as_stream(stream)>>>(*g, sino, trig, img);
    return launch_status("sf2d_bp");
}
