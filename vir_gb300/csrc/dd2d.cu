// 2D distance-driven projector pair (parallel and flat-detector fan) in
// gather form.
//
// vir's sweep (sys_mat/dd.py:82-277) walks, per view and per orthogonal
// pixel line, a merge of projected pixel edges with detector edges and adds
// img * overlap * scale into the bin (FP) or the pixel (BP).  The sum it
// computes is, for bin j,
//     sino[j] = sum_io scale(io) sum_k img(k, io) |[P_k, P_k+1] ∩ [u_j, u_j+1]|
// with P_k the projection of driving edge k on line io.  Here each thread
// owns output elements and gathers their terms; no atomics, deterministic.
//
//  FP (dd2d_fp_kernel): one block per view (x a bin range).  Orthogonal lines
//    are processed in chunks: the block first projects every driving edge of
//    the chunk's lines into shared memory (one division per edge, shared by
//    all bins) and stages the lines' pixels pre-multiplied by the line scale;
//    then each thread walks its bins down the chunk, keeping per bin the
//    index of the pixel under its left edge (it moves by at most a step from
//    one line to the next), and sums the 1-3 overlapping pixels.
//  BP (dd2d_bp_kernel): one block per 32x8 pixel tile.  Views are processed
//    in chunks: the block projects the tile's driving edges for every view of
//    the chunk into shared memory (one division per edge, shared by the two
//    pixels on either side) with the line scales; then each thread sums, per
//    view, the 1-3 bins overlapped by its pixel's projected interval.
//
// Geometry per dd.py:
//  - driving axis X when |sin| >= |cos| (dd.py:478, 532);
//  - X-driven: p = -sin*x_edge + cos*y_centre, o = cos*x_edge + sin*y_centre;
//    Y-driven: p = cos*y_edge - sin*x_centre, o = sin*y_edge + cos*x_centre
//    (dd.py:491-494, 507-510, 546-550, 563-567);
//  - fan projection u = DSD p / (DSO - o) (dd.py:50-51);
//  - scale 1/|trig| (parallel) or r / ((DSO - o_c)|trig|), r = |(DSO - o_c, p_c)|
//    for the line centre (dd.py:581-582);
//  - detector edges du (j - nu/2 + su) (dd.py:699);
//  - FP returns sino * d_pix/du, BP returns img / (na d_pix) (dd.py:721-725).
// Pixel edges are d_pix (k - n/2) and line centres their midpoints.  The
// sweep runs over edges in increasing projection order: when the driving
// coefficient is negative the edge order is reversed, as dd.py:516-518 does.
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

__device__ __forceinline__ ViewGeo vg_of(const float *f, int xdrv) {
    ViewGeo v;
    v.pd = f[0]; v.od = f[1]; v.po = f[2]; v.oo = f[3]; v.tabs = f[4]; v.xdrv = xdrv;
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
__device__ __forceinline__ float proj(const vg_dd2d_geom &g, const ViewGeo &v, float cp, float co,
                                      float b) {
    float p = v.pd * b + cp;
    if (!FAN) return p;
    return g.DSD * p / (g.DSO - (v.od * b + co));
}

// inverse of proj: driving edge coordinate b whose projection is u
template <bool FAN>
__device__ __forceinline__ float unproj(const vg_dd2d_geom &g, const ViewGeo &v, float cp,
                                        float co, float u) {
    if (!FAN) return (u - cp) / v.pd;
    return (u * (g.DSO - co) - g.DSD * cp) / (g.DSD * v.pd + u * v.od);
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

// ---------------------------------------------------------------------------
// Forward projection
// ---------------------------------------------------------------------------

constexpr int FP_THREADS = 256;
constexpr int FP_NB = 4;  // bins per thread (strided by FP_THREADS)
constexpr int FP_MAXL = 32;  // most lines per shared-memory chunk

// Shared memory per chunk line: nd + 1 projected edges and nd scaled pixels.
__host__ __device__ inline int fp_line_floats(int nd) { return 2 * nd + 1; }

// mode 0: out = FP;  mode 1 (SIRT residual): out = (y - FP) * inv_w, or FP
// where inv_w == 0.
template <bool FAN>
__global__ void __launch_bounds__(FP_THREADS, 1)
dd2d_fp_kernel(vg_dd2d_geom g, const float *__restrict__ img, const float *__restrict__ imgT,
               const double *__restrict__ trig, float *__restrict__ out, int mode,
               const float *__restrict__ y, const float *__restrict__ inv_w, int L) {
    extern __shared__ float sm[];
    const int ia = blockIdx.y;
    const ViewGeo v = view_geo(trig, ia);
    const int nd = v.xdrv ? g.nx : g.ny;
    const int no = v.xdrv ? g.ny : g.nx;
    const float *base = v.xdrv ? imgT : img;  // line io is contiguous in k
    const bool rev = v.pd < 0.f;               // edges decreasing in k: sweep reversed
    const int stride = nd + 1;
    float *P = sm;                       // [L][nd + 1] projected edges, sweep order
    float *V = sm + (size_t)L * stride;  // [L][nd] pixel * line scale, sweep order
    __shared__ float Lcp[FP_MAXL], Lco[FP_MAXL], Lsc[FP_MAXL];

    // this thread's bins
    int jb[FP_NB];
    float ul[FP_NB], ur[FP_NB];
    int kk[FP_NB];
    Kahan acc[FP_NB];
#pragma unroll
    for (int i = 0; i < FP_NB; ++i) {
        jb[i] = blockIdx.x * FP_THREADS * FP_NB + i * FP_THREADS + threadIdx.x;
        ul[i] = det_edge(g, jb[i]);
        ur[i] = det_edge(g, jb[i] + 1);
        kk[i] = -1;
    }

    for (int l0 = 0; l0 < no; l0 += L) {
        const int nl = min(L, no - l0);
        __syncthreads();  // previous chunk consumed
        // per-line geometry of lines l0 .. l0 + nl - 1
        for (int l = threadIdx.x; l < nl; l += FP_THREADS) {
            const Line Lg = line_geo<FAN>(g, v, centre_coord(g.d_pix, l0 + l, no));
            Lcp[l] = Lg.cp;
            Lco[l] = Lg.co;
            Lsc[l] = Lg.scl;
        }
        __syncthreads();
        // projected edges and scaled pixels, sweep order
        {
            int l = 0, m = threadIdx.x;
            while (m >= stride) { m -= stride; ++l; }
            while (l < nl) {
                const int io = l0 + l;
                const int kb = rev ? nd - m : m;
                P[l * stride + m] = proj<FAN>(g, v, Lcp[l], Lco[l], edge_coord(g.d_pix, kb, nd));
                if (m < nd) {
                    const int kp = rev ? nd - 1 - m : m;
                    V[l * nd + m] = __ldg(base + (size_t)io * nd + kp) * Lsc[l];
                }
                m += FP_THREADS;
                while (m >= stride) { m -= stride; ++l; }
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < FP_NB; ++i) {
            if (jb[i] >= g.nu) continue;
            const float a = ul[i], b = ur[i];
            int k = kk[i];
            if (k < 0) {
                // first line: invert the edge projection to start near the bin
                const ViewGeo vv = v;
                const float cen = centre_coord(g.d_pix, l0, no);
                const float cp = vv.po * cen, co = vv.oo * cen;
                float kf = unproj<FAN>(g, vv, cp, co, a) / g.d_pix + 0.5f * nd;
                kf = fminf(fmaxf(kf, 0.f), (float)(nd - 1));
                k = (int)kf;
                if (rev) k = nd - 1 - k;
            }
            float part = 0.f;
            for (int l = 0; l < nl; ++l) {
                const float *Pl = P + l * stride;
                const float *Vl = V + l * nd;
                // keep Pl[k] <= a < Pl[k+1] (bounded walks)
                while (k > 0 && Pl[k] > a) --k;
                while (k < nd - 1 && Pl[k + 1] <= a) ++k;
                float pl = Pl[k];
                for (int m = k; m < nd; ++m) {
                    const float pr = Pl[m + 1];
                    const float ov = fminf(pr, b) - fmaxf(pl, a);
                    if (ov > 0.f) part = fmaf(Vl[m], ov, part);
                    if (pr >= b) break;
                    pl = pr;
                }
            }
            acc[i].add(part);
            kk[i] = k;
        }
    }

    const float f = g.d_pix / g.du;
#pragma unroll
    for (int i = 0; i < FP_NB; ++i) {
        if (jb[i] >= g.nu) continue;
        float fp = acc[i].s * f;
        const size_t o = (size_t)ia * g.nu + jb[i];
        if (mode == 1) {
            const float w = inv_w[o];
            fp = (w != 0.f) ? (y[o] - fp) * w : fp;
        }
        out[o] = fp;
    }
}

// ---------------------------------------------------------------------------
// Backprojection
// ---------------------------------------------------------------------------

constexpr int BP_TY = 32;  // pixels along y (threadIdx.x, contiguous in img)
constexpr int BP_TX = 8;   // pixels along x (threadIdx.y)
constexpr int BP_VC = 24;  // views per chunk (static shared memory stays under 48 KiB)
// per view: edges for the tile (X-driven: BP_TY lines x (BP_TX + 1) edges;
// Y-driven: BP_TX lines x (BP_TY + 1) edges) and one scale per line
constexpr int BP_EDGES = (BP_TY * (BP_TX + 1) > BP_TX * (BP_TY + 1)) ? BP_TY * (BP_TX + 1)
                                                                     : BP_TX * (BP_TY + 1);

// mode 0: img = BP;  mode 1 (SIRT update): x += gamma * BP * inv_w (BP where
// inv_w == 0), written to x and its transpose xT.
template <bool FAN>
__global__ void __launch_bounds__(BP_TY * BP_TX)
dd2d_bp_kernel(vg_dd2d_geom g, const float *__restrict__ sino, const double *__restrict__ trig,
               float *__restrict__ img, int mode, const float *__restrict__ inv_w, float gamma,
               float *__restrict__ xT) {
    __shared__ float Ps[BP_VC][BP_EDGES];
    __shared__ float Ss[BP_VC][BP_TY], Lcp[BP_VC][BP_TY], Lco[BP_VC][BP_TY];
    __shared__ float Vg[BP_VC][5];
    __shared__ int Xs[BP_VC];
    const int tid = threadIdx.y * BP_TY + threadIdx.x;
    const int iy0 = blockIdx.x * BP_TY, ix0 = blockIdx.y * BP_TX;
    const int iy = iy0 + threadIdx.x, ix = ix0 + threadIdx.y;
    const bool inside = iy < g.ny && ix < g.nx;
    const float u0 = det_edge(g, 0);
    const float inv_du = 1.0f / g.du;
    Kahan acc;
    for (int a0 = 0; a0 < g.na; a0 += BP_VC) {
        const int nv = min(BP_VC, g.na - a0);
        __syncthreads();
        // stage 1: view geometry of the chunk
        if (tid < nv) {
            const ViewGeo v = view_geo(trig, a0 + tid);
            Vg[tid][0] = v.pd; Vg[tid][1] = v.od; Vg[tid][2] = v.po; Vg[tid][3] = v.oo;
            Vg[tid][4] = v.tabs;
            Xs[tid] = v.xdrv;
        }
        __syncthreads();
        // stage 2: line geometry (X-driven lines are the tile's rows y, else columns x)
        for (int e = tid; e < nv * BP_TY; e += BP_TY * BP_TX) {
            const int vi = e / BP_TY, l = e - vi * BP_TY;
            const ViewGeo v = vg_of(Vg[vi], Xs[vi]);
            const int nl = v.xdrv ? BP_TY : BP_TX;
            const int io = (v.xdrv ? iy0 : ix0) + l, no = v.xdrv ? g.ny : g.nx;
            if (l < nl && io < no) {
                const Line Lg = line_geo<FAN>(g, v, centre_coord(g.d_pix, io, no));
                Lcp[vi][l] = Lg.cp; Lco[vi][l] = Lg.co; Ss[vi][l] = Lg.scl;
            }
        }
        __syncthreads();
        // stage 3: the tile's projected driving edges per view
        for (int e = tid; e < nv * BP_EDGES; e += BP_TY * BP_TX) {
            const int vi = e / BP_EDGES, q = e - vi * BP_EDGES;
            const ViewGeo v = vg_of(Vg[vi], Xs[vi]);
            int nd, no, nl, ne;
            if (v.xdrv) { nl = BP_TY; ne = BP_TX + 1; nd = g.nx; no = g.ny; }
            else        { nl = BP_TX; ne = BP_TY + 1; nd = g.ny; no = g.nx; }
            if (q >= nl * ne) continue;
            const int l = q / ne, b = q - l * ne;
            const int io = (v.xdrv ? iy0 : ix0) + l;
            const int k = (v.xdrv ? ix0 : iy0) + b;
            if (io >= no || k > nd) { Ps[vi][q] = 0.f; continue; }
            Ps[vi][q] = proj<FAN>(g, v, Lcp[vi][l], Lco[vi][l], edge_coord(g.d_pix, k, nd));
        }
        __syncthreads();
        if (inside) {
            for (int vi = 0; vi < nv; ++vi) {
                const bool xd = Xs[vi];
                const int l = xd ? threadIdx.x : threadIdx.y;
                const int b = xd ? threadIdx.y : threadIdx.x;
                const int ne = xd ? BP_TX + 1 : BP_TY + 1;
                const float pa = Ps[vi][l * ne + b], pb = Ps[vi][l * ne + b + 1];
                const float lo = fminf(pa, pb), hi = fmaxf(pa, pb);
                const float *row = sino + (size_t)(a0 + vi) * g.nu;
                int j = max(0, (int)floorf((lo - u0) * inv_du));
                float s = 0.f;
                float el = det_edge(g, j);
                for (; j < g.nu; ++j) {
                    const float er = det_edge(g, j + 1);
                    const float ov = fminf(hi, er) - fmaxf(lo, el);
                    if (ov > 0.f) s = fmaf(__ldg(row + j), ov, s);
                    if (er >= hi) break;
                    el = er;
                }
                acc.add(s * Ss[vi][l]);
            }
        }
    }
    if (!inside) return;
    const float bp = acc.s / ((float)g.na * g.d_pix);
    const size_t o = (size_t)ix * g.ny + iy;
    if (mode == 1) {
        const float w = inv_w[o];
        const float upd = (w != 0.f) ? bp * w : bp;
        const float xn = img[o] + gamma * upd;
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
    VG_REQUIRE(g->nx <= 16384 && g->ny <= 16384, "dd2d: image sides above 16384");
    VG_REQUIRE(g->du > 0.f && g->d_pix > 0.f, "dd2d: du and d_pix must be positive");
    if (g->fan) {
        VG_REQUIRE(g->DSO > 0.f && g->DSD > 0.f, "dd2d: fan needs DSO, DSD > 0");
        // the projections of a line's driving edges are monotone (the sweep's
        // premise, dd.py:516-518) when every line centre is closer to the
        // isocentre than DSO * |trig| >= DSO / sqrt(2)
        float h = 0.5f * (float)(g->nx > g->ny ? g->nx : g->ny) * g->d_pix;
        VG_REQUIRE(h < 0.70710678f * g->DSO,
                   "dd2d: fan geometry needs the image half-width below DSO/sqrt(2)");
    }
    return VG_OK;
}

// Lines per shared-memory chunk of the FP: as many as fit in FP_SMEM bytes.
constexpr int FP_SMEM = 48 * 1024;
int fp_chunk_lines(const vg_dd2d_geom *g) {
    int nd = g->nx > g->ny ? g->nx : g->ny;
    int L = FP_SMEM / (fp_line_floats(nd) * (int)sizeof(float));
    return L < 1 ? 1 : (L > FP_MAXL ? FP_MAXL : L);
}

template <bool FAN>
int set_fp_smem(size_t bytes) {
    static size_t done = 0;
    if (bytes <= 48 * 1024 || bytes <= done) return VG_OK;
    cudaError_t e = cudaFuncSetAttribute(dd2d_fp_kernel<FAN>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return cuda_status(e, "dd2d_fp: shared memory attribute");
    done = bytes;
    return VG_OK;
}

int launch_fp(const vg_dd2d_geom *g, const float *img, const float *imgT, const double *trig,
              float *out, int mode, const float *y, const float *inv_w, cudaStream_t st) {
    const int L = fp_chunk_lines(g);
    const int nd = g->nx > g->ny ? g->nx : g->ny;
    const size_t smem = (size_t)L * fp_line_floats(nd) * sizeof(float);
    VG_REQUIRE(smem <= 200 * 1024, "dd2d_fp: image side too large for one line in shared memory");
    dim3 grid(ceil_div(g->nu, FP_THREADS * FP_NB), g->na);
    int s = g->fan ? set_fp_smem<true>(smem) : set_fp_smem<false>(smem);
    if (s) return s;
    if (g->fan)
        dd2d_fp_kernel<true><<<grid, FP_THREADS, smem, st>>>(*g, img, imgT, trig, out, mode, y,
                                                            inv_w, L);
    else
        dd2d_fp_kernel<false><<<grid, FP_THREADS, smem, st>>>(*g, img, imgT, trig, out, mode, y,
                                                             inv_w, L);
    return launch_status("dd2d_fp");
}

int launch_bp(const vg_dd2d_geom *g, const float *sino, const double *trig, float *img, int mode,
              const float *inv_w, float gamma, float *xT, cudaStream_t st) {
    dim3 grid(ceil_div(g->ny, BP_TY), ceil_div(g->nx, BP_TX));
    VG_REQUIRE(grid.y < 65536, "dd2d_bp: nx too large");
    dim3 block(BP_TY, BP_TX);
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
