// 2D distance-driven projector pair (parallel and flat-detector fan) in
// gather form.
//
// vir's sweep (sys_mat/dd.py:82-277) walks, per view and per orthogonal
// pixel line, a merge of projected pixel edges with detector edges and adds
// img * overlap * scale into the bin (FP) or the pixel (BP).  The sum it
// computes is, for bin j,
//     sino[j] = sum_io scale(io) sum_k img(k, io) |[P_k, P_k+1] ∩ [u_j, u_j+1]|
// with P_k the projection of driving edge k on line io.  Here each thread
// owns one output element and gathers its terms directly:
//  - FP: a thread per (view, bin) walks the lines; on each it inverts the
//    edge projection to find the 1-3 pixels that overlap its bin;
//  - BP: a thread per pixel walks the views; on each it projects its two
//    driving edges and sums the 1-3 bins they overlap.
// No atomics, no scatter, deterministic.  Geometry per dd.py:
//  - driving axis X when |sin| >= |cos| (dd.py:478, 532);
//  - X-driven: p = -sin*x_edge + cos*y_centre, o = cos*x_edge + sin*y_centre;
//    Y-driven: p = cos*y_edge - sin*x_centre, o = sin*y_edge + cos*x_centre
//    (dd.py:491-494, 507-510, 546-550, 563-567);
//  - fan projection u = DSD p / (DSO - o) (dd.py:50-51);
//  - scale 1/|trig| (parallel) or r / ((DSO - o_c)|trig|), r = |(DSO - o_c, p_c)|
//    for the line centre (dd.py:581-582);
//  - detector edges du (j - nu/2 + su) (dd.py:699);
//  - FP returns sino * d_pix/du, BP returns img / (na d_pix) (dd.py:721-725).
// Pixel edges are d_pix (k - n/2) and line centres their midpoints.
#include "vg_common.cuh"

namespace {

using namespace vg;

struct ViewGeo {
    float pd, od;  // driving-edge coefficients: p = pd*b + cp, o = od*b + co
    float po, oo;  // line-centre coefficients: cp = po*cen, co = oo*cen
    float tabs;    // |sin| (X-driven) or |cos|
    int xdrv;
};

__device__ __forceinline__ ViewGeo view_geo(const double *trig, int ia) {
    ViewGeo v;
    float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
    v.xdrv = fabsf(s) >= fabsf(c);
    if (v.xdrv) { v.pd = -s; v.od = c; v.po = c; v.oo = s; v.tabs = fabsf(s); }
    else        { v.pd = c;  v.od = s; v.po = -s; v.oo = c; v.tabs = fabsf(c); }
    return v;
}

struct Line {
    float cp, co, scl;
};

template <bool FAN>
__device__ __forceinline__ Line line_geo(const vg_dd2d_geom &g, const ViewGeo &v, float cen) {
    Line L;
    L.cp = v.po * cen;
    L.co = v.oo * cen;
    if (FAN) {
        float a = g.DSO - L.co;
        L.scl = sqrtf(a * a + L.cp * L.cp) / (a * v.tabs);
    } else {
        L.scl = 1.0f / v.tabs;
    }
    return L;
}

// projection of driving edge coordinate b on a line
template <bool FAN>
__device__ __forceinline__ float proj(const vg_dd2d_geom &g, const ViewGeo &v, const Line &L,
                                      float b) {
    float p = v.pd * b + L.cp;
    if (!FAN) return p;
    return g.DSD * p / (g.DSO - (v.od * b + L.co));
}

// inverse of proj: driving edge coordinate b whose projection is u
template <bool FAN>
__device__ __forceinline__ float unproj(const vg_dd2d_geom &g, const ViewGeo &v, const Line &L,
                                        float u) {
    if (!FAN) return (u - L.cp) / v.pd;
    return (u * (g.DSO - L.co) - g.DSD * L.cp) / (g.DSD * v.pd + u * v.od);
}

__device__ __forceinline__ float edge_coord(float d_pix, int k, int n) {
    return d_pix * ((float)k - 0.5f * (float)n);
}

__device__ __forceinline__ float centre_coord(float d_pix, int k, int n) {
    return d_pix * ((float)k + 0.5f - 0.5f * (float)n);
}

__device__ __forceinline__ float det_edge(const vg_dd2d_geom &g, int j) {
    return g.du * ((float)j - 0.5f * (float)g.nu + g.su);
}

// Sum over one line of img(k) * overlap(k, [ul, ur]).
template <bool FAN>
__device__ __forceinline__ float line_gather(const vg_dd2d_geom &g, const ViewGeo &v,
                                             const Line &L, const float *__restrict__ row, int nd,
                                             float ul, float ur) {
    float inv = 1.0f / g.d_pix;
    float ka = unproj<FAN>(g, v, L, ul) * inv + 0.5f * nd;
    float kb = unproj<FAN>(g, v, L, ur) * inv + 0.5f * nd;
    float klo = fminf(ka, kb), khi = fmaxf(ka, kb);
    int k0 = max(0, (int)floorf(klo - 1e-3f));
    int k1 = min(nd - 1, (int)floorf(khi + 1e-3f));
    float sum = 0.f;
    if (k0 > k1) return 0.f;
    float pa = proj<FAN>(g, v, L, edge_coord(g.d_pix, k0, nd));
    for (int k = k0; k <= k1; ++k) {
        float pb = proj<FAN>(g, v, L, edge_coord(g.d_pix, k + 1, nd));
        float lo = fminf(pa, pb), hi = fmaxf(pa, pb);
        float ov = fminf(hi, ur) - fmaxf(lo, ul);
        if (ov > 0.f) sum += __ldg(row + k) * ov;
        pa = pb;
    }
    return sum;
}

// mode 0: out = FP;  mode 1 (SIRT residual): out = (y - FP) * inv_w, or FP
// where inv_w == 0.
template <bool FAN>
__global__ void
dd2d_fp_kernel(vg_dd2d_geom g, const float *__restrict__ img, const float *__restrict__ imgT,
               const double *__restrict__ trig, float *__restrict__ out, int mode,
               const float *__restrict__ y, const float *__restrict__ inv_w) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int ia = blockIdx.y;
    if (j >= g.nu) return;
    ViewGeo v = view_geo(trig, ia);
    int nd = v.xdrv ? g.nx : g.ny;
    int no = v.xdrv ? g.ny : g.nx;
    const float *base = v.xdrv ? imgT : img;  // line io is contiguous in k
    float ul = det_edge(g, j), ur = det_edge(g, j + 1);
    Kahan acc;
    for (int io = 0; io < no; ++io) {
        Line L = line_geo<FAN>(g, v, centre_coord(g.d_pix, io, no));
        float s = line_gather<FAN>(g, v, L, base + (size_t)io * nd, nd, ul, ur);
        if (s != 0.f) acc.add(s * L.scl);
    }
    float fp = acc.s * (g.d_pix / g.du);
    size_t o = (size_t)ia * g.nu + j;
    if (mode == 1) {
        float w = inv_w[o];
        fp = (w != 0.f) ? (y[o] - fp) * w : fp;
    }
    out[o] = fp;
}

// Sum over the bins overlapped by [lo, hi] of sino_row(j) * overlap.
__device__ __forceinline__ float bin_gather(const vg_dd2d_geom &g, const float *__restrict__ row,
                                            float lo, float hi) {
    float u0 = det_edge(g, 0);
    float inv_du = 1.0f / g.du;
    int j0 = max(0, (int)floorf((lo - u0) * inv_du - 1e-3f));
    int j1 = min(g.nu - 1, (int)floorf((hi - u0) * inv_du + 1e-3f));
    float sum = 0.f;
    for (int j = j0; j <= j1; ++j) {
        float ov = fminf(hi, det_edge(g, j + 1)) - fmaxf(lo, det_edge(g, j));
        if (ov > 0.f) sum += __ldg(row + j) * ov;
    }
    return sum;
}

// mode 0: img = BP;  mode 1 (SIRT update): x += gamma * BP * inv_w (BP where
// inv_w == 0), written to x and its transpose xT.
template <bool FAN>
__global__ void
dd2d_bp_kernel(vg_dd2d_geom g, const float *__restrict__ sino, const double *__restrict__ trig,
               float *__restrict__ img, int mode, const float *__restrict__ inv_w, float gamma,
               float *__restrict__ xT) {
    int iy = blockIdx.x * 32 + threadIdx.x;
    int ix = blockIdx.y * 8 + threadIdx.y;
    if (iy >= g.ny || ix >= g.nx) return;
    Kahan acc;
    for (int ia = 0; ia < g.na; ++ia) {
        ViewGeo v = view_geo(trig, ia);
        int k, nd, io, no;
        if (v.xdrv) { k = ix; nd = g.nx; io = iy; no = g.ny; }
        else        { k = iy; nd = g.ny; io = ix; no = g.nx; }
        Line L = line_geo<FAN>(g, v, centre_coord(g.d_pix, io, no));
        float pa = proj<FAN>(g, v, L, edge_coord(g.d_pix, k, nd));
        float pb = proj<FAN>(g, v, L, edge_coord(g.d_pix, k + 1, nd));
        float s = bin_gather(g, sino + (size_t)ia * g.nu, fminf(pa, pb), fmaxf(pa, pb));
        if (s != 0.f) acc.add(s * L.scl);
    }
    float bp = acc.s / ((float)g.na * g.d_pix);
    size_t o = (size_t)ix * g.ny + iy;
    if (mode == 1) {
        float w = inv_w[o];
        float upd = (w != 0.f) ? bp * w : bp;
        float xn = img[o] + gamma * upd;
        img[o] = xn;
        xT[(size_t)iy * g.nx + ix] = xn;
    } else {
        img[o] = bp;
    }
}

int check_geom(const vg_dd2d_geom *g) {
    VG_REQUIRE(g, "dd2d: null geometry");
    VG_REQUIRE(g->nx > 0 && g->ny > 0 && g->na > 0 && g->nu > 0, "dd2d: sizes must be positive");
    VG_REQUIRE(g->na < 65536, "dd2d: at most 65535 views per call");
    VG_REQUIRE(g->du > 0.f && g->d_pix > 0.f, "dd2d: du and d_pix must be positive");
    if (g->fan) {
        VG_REQUIRE(g->DSO > 0.f && g->DSD > 0.f, "dd2d: fan needs DSO, DSD > 0");
        // every pixel must lie in front of the source: |corner| < DSO
        float hx = 0.5f * g->nx * g->d_pix, hy = 0.5f * g->ny * g->d_pix;
        VG_REQUIRE(sqrtf(hx * hx + hy * hy) < g->DSO,
                   "dd2d: image half-diagonal must be smaller than DSO");
    }
    return VG_OK;
}

int launch_fp(const vg_dd2d_geom *g, const float *img, const float *imgT, const double *trig,
              float *out, int mode, const float *y, const float *inv_w, cudaStream_t st) {
    dim3 grid(ceil_div(g->nu, 128), g->na);
    if (g->fan)
        dd2d_fp_kernel<true><<<grid, 128, 0, st>>>(*g, img, imgT, trig, out, mode, y, inv_w);
    else
        dd2d_fp_kernel<false><<<grid, 128, 0, st>>>(*g, img, imgT, trig, out, mode, y, inv_w);
    return launch_status("dd2d_fp");
}

int launch_bp(const vg_dd2d_geom *g, const float *sino, const double *trig, float *img, int mode,
              const float *inv_w, float gamma, float *xT, cudaStream_t st) {
    dim3 grid(ceil_div(g->ny, 32), ceil_div(g->nx, 8));
    VG_REQUIRE(grid.y < 65536, "dd2d_bp: nx too large");
    dim3 block(32, 8);
    if (g->fan)
        dd2d_bp_kernel<true><<<grid, block, 0, st>>>(*g, sino, trig, img, mode, inv_w, gamma, xT);
    else
        dd2d_bp_kernel<false><<<grid, block, 0, st>>>(*g, sino, trig, img, mode, inv_w, gamma, xT);
    return launch_status("dd2d_bp");
}

}  // namespace

extern "C" int vg_dd2d_fp(const vg_dd2d_geom *g, const float *img, const float *imgT,
                          const double *trig, float *sino, void *stream) {
    int st = check_geom(g);
    if (st) return st;
    VG_REQUIRE(img && imgT && trig && sino, "dd2d_fp: null pointer");
    return launch_fp(g, img, imgT, trig, sino, 0, nullptr, nullptr, as_stream(stream));
}

extern "C" int vg_dd2d_bp(const vg_dd2d_geom *g, const float *sino, const double *trig,
                          float *img, void *stream) {
    int st = check_geom(g);
    if (st) return st;
    VG_REQUIRE(img && trig && sino, "dd2d_bp: null pointer");
    return launch_bp(g, sino, trig, img, 0, nullptr, 0.f, nullptr, as_stream(stream));
}

extern "C" int vg_dd2d_sirt_iter(const vg_dd2d_geom *g, const float *y, const float *inv_w_sino,
                                 const float *inv_w_img, float gamma, const double *trig,
                                 float *x, float *xT, float *r, void *stream) {
    int st = check_geom(g);
    if (st) return st;
    VG_REQUIRE(y && inv_w_sino && inv_w_img && trig && x && xT && r, "dd2d_sirt_iter: null pointer");
    cudaStream_t s = as_stream(stream);
    st = launch_fp(g, x, xT, trig, r, 1, y, inv_w_sino, s);
    if (st) return st;
    return launch_bp(g, r, trig, x, 1, inv_w_img, gamma, xT, s);
}
