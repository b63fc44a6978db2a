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
//  FP (dd2d_fp_kernel): one block per view (x a bin range), one warp per
//    orthogonal line at a time.  The warp projects the line's driving edges
//    (one division per edge), stages the running integral of its pixels in
//    shared memory, and every lane evaluates that integral at the left edges
//    of its bins through the inverse edge map; a bin's term is the
//    difference of the integral at its two edges.
//  BP (dd2d_bp_kernel): one block per 16x64 pixel tile (2x2 per thread).  A
//    per-view table holds the running integral of the sinogram row; each
//    thread projects its patch's driving edges (three per line, shared by
//    neighbouring pixels) and takes differences of the table at them.
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

#include <cuda_bf16.h>

// The forward projection's fused SIRT epilogue also writes the back
// projection's tables (two launches per update; 0 restores the separate
// table kernel).
#ifndef VG_SIRT_FUSED_TABLES
#define VG_SIRT_FUSED_TABLES 1
#endif

// Edge projections and bin positions use approximate reciprocals
// (rcp.approx, about 1 ulp) unless built with -DVG_FAST_DIV=0 (IEEE division).
#ifndef VG_FAST_DIV
#define VG_FAST_DIV 1
#endif

// Both projections find a pixel or bin index as the bit pattern of a
// round-down FMA onto 1.5 * 2^23 (an FMA-pipe operation; exact floor for
// values below 2^22), after saturating the lookup coordinate to [0, 1] in
// the preceding FMA, so that no clamp or float-to-int conversion is needed.

namespace {

using namespace vg;

// Storage types of the image (TX) and the measured sinogram (TY): float, or
// bfloat16 with all arithmetic in float32 (the batched SIRT's bf16 storage).
// COH loads (ld.global.ca) are for data written earlier in the same launch
// (the persistent batched kernel, after an acquire fence); the others use
// the read-only path (ld.global.nc), valid for data no launch writes meanwhile.
template <bool COH = false, typename T> __device__ __forceinline__ T ldro(const T *p) {
    return COH ? __ldca(p) : __ldg(p);
}
template <bool COH = false> __device__ __forceinline__ float ldf(const float *p) { return ldro<COH>(p); }
template <bool COH = false> __device__ __forceinline__ float ldf(const __nv_bfloat16 *p) {
    return __bfloat162float(ldro<COH>(p));
}
__device__ __forceinline__ float ldf_plain(const float *p) { return *p; }
__device__ __forceinline__ float ldf_plain(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
__device__ __forceinline__ void stf(float *p, float v) { *p = v; }
__device__ __forceinline__ void stf(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }
// 8 consecutive values from a 16-byte aligned address (float: two float4
// loads; bfloat16: one 16-byte load)
template <bool COH = false> __device__ __forceinline__ void ld8(const float *p, float *o) {
    const float4 a = ldro<COH>(reinterpret_cast<const float4 *>(p));
    const float4 b = ldro<COH>(reinterpret_cast<const float4 *>(p) + 1);
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
}
template <bool COH = false> __device__ __forceinline__ void ld8(const __nv_bfloat16 *p, float *o) {
    const uint4 a = ldro<COH>(reinterpret_cast<const uint4 *>(p));
    const unsigned w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        o[2 * i] = __uint_as_float(w[i] << 16);
        o[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
    }
}

// A compile-time bool usable in device code (selects a copy of a generic lambda).
template <bool B> struct BoolC {
    __host__ __device__ constexpr operator bool() const { return B; }
};

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
__device__ __forceinline__ float proj(const vg_dd2d_geom &g, const ViewGeo &v, float cp, float co,
                                      float b) {
    float p = v.pd * b + cp;
    if (!FAN) return p;
#if VG_FAST_DIV
    return __fdividef(g.DSD * p, g.DSO - (v.od * b + co));
#else
    return g.DSD * p / (g.DSO - (v.od * b + co));
#endif
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
// Forward projection (integral form, one warp per orthogonal line)
//
// For one view and one orthogonal line, let f(u) be the line's pixels as a
// piecewise-constant function of the detector coordinate (pixel m spans
// [P_m, P_m+1], value V_m = img * line scale) and F(u) its running integral:
//     F(u) = S_k + V_k * (u - P_k),  k the pixel under u,  S_k = sum_{m<k} V_m (P_m+1 - P_m).
// The line's contribution to bin [U_j, U_j+1] -- the sum of img * overlap *
// scale that vir's merge accumulates -- is F(U_j+1) - F(U_j).
//
// A block owns one view and FP_MAXB * 32 bins; each warp walks the lines
// io = warp, warp + nwarps, ...: it stages the line's (P, S, V) in its own
// shared buffer (edges projected once, S by a warp scan; __syncwarp only),
// then every lane evaluates F at the left edges of its bins j = lane + 32 i,
// takes right edges from the neighbouring lane, and accumulates.  The pixel
// k under U comes from the exact inverse of the edge projection (a Moebius
// map whose denominator does not depend on the line: its reciprocal C(U) is
// computed once per view).  Per-warp bin sums are added in a fixed order at
// the end: deterministic, no atomics.
// ---------------------------------------------------------------------------

// Tile variants: WARPS (lines in flight per block) x MAXB (bins per lane,
// strided by 32; a block owns 32 MAXB bins of one view).  vg_dd2d_geom's
// `variant` selects one (1..FP_NVARIANTS), 0 picks by size (fp_variant_for).
// Pixels per lane in the line scan: 8 keeps the 8-warp tiles at 80 registers,
// three blocks per SM (16 needs 128 registers, two blocks, and ran 2 % slower).
#ifndef VG_FP_SEG
#define VG_FP_SEG 8
#endif
constexpr int FP_SEG = VG_FP_SEG;
struct FpVariant { int warps, maxb; };
constexpr FpVariant FP_VARIANTS[] = {{8, 6}, {8, 12}, {8, 24}, {4, 24}, {4, 48}, {2, 48}};
constexpr int FP_NVARIANTS = sizeof(FP_VARIANTS) / sizeof(FP_VARIANTS[0]);

// Line entries are (G_k, V_k) with G_k = S_k - V_k P_k, so F(U) = G_k + V_k U
// for U in pixel k.  Pixel p in -1 .. nd + 1 sits in slot fp_slot(p): p = -1 is
// a zero sentinel for U before the line's first edge (F = 0), p = nd and
// nd + 1 carry the line total (S_nd, 0).  One spare slot every 16 pixels keeps
// the scan's lanes (8 pixels apart) on different shared-memory banks; the
// spare falls between segments, so a lane's 8 pixels (p = 8 m ...) take
// consecutive slots.
__host__ __device__ __forceinline__ int fp_slot(int p) { return p + 1 + ((p + 16) >> 4); }
__host__ __device__ inline int fp_line_entries(int nd) { return fp_slot(nd + 1) + 1; }
// The walk finds pixel p as the bit pattern b = FP_MAGIC_BITS + 16 + p of a
// round-down FMA onto 1.5 * 2^23 + 15; b + (b >> 4) = fp_slot(p) + FP_SLOT_BIAS.
constexpr unsigned FP_MAGIC_BITS = 0x4B400000u;  // 1.5 * 2^23, a multiple of 16
constexpr unsigned FP_SLOT_BIAS = FP_MAGIC_BITS + (FP_MAGIC_BITS >> 4) + 15u;

// Per-view back-projection table: entry i = j + 1 for bin j in -1 .. nu + 1
// holds the running integral G of the sinogram row in the lookup coordinate
// t' = (t + 1) / (nu + 2) (t the position in bins from U_0), G = x + y t':
// (0, 0) before the detector (j = -1), (T_j - (j + 1) du s_j, du s_j (nu + 2))
// on bin j, (T_nu, 0) past it (j = nu, nu + 1).  A lookup saturates t' to
// [0, 1] and takes i = floor(t' (nu + 2)), so it needs no clamps.
__host__ __device__ inline int bp_tab_len(int nu) { return nu + 3; }

struct BpWork {
    float2 *ts;  // [na][nu + 3], see bp_tab_len
    float *scl;  // [na][scl_stride]: signed line scale for the view's driving axis
};

// scale rows hold max(nx, ny) lines, padded to an even count so that a
// pixel patch reads its two lines as one 8-byte load
__host__ __device__ inline int scl_stride(const vg_dd2d_geom &g) {
    const int nm = g.nx > g.ny ? g.nx : g.ny;
    return nm + (nm & 1);
}

__host__ __device__ inline size_t bp_ws_ts_bytes(const vg_dd2d_geom *g) {
    return ((size_t)g->na * bp_tab_len(g->nu) * sizeof(float2) + 255) & ~(size_t)255;
}
size_t bp_ws_bytes(const vg_dd2d_geom *g) {
    return bp_ws_ts_bytes(g) + (((size_t)g->na * scl_stride(*g) * sizeof(float) + 255) & ~(size_t)255);
}
__host__ __device__ inline BpWork bp_ws(const vg_dd2d_geom *g, void *ws) {
    BpWork w;
    w.ts = reinterpret_cast<float2 *>(ws);
    w.scl = reinterpret_cast<float *>(reinterpret_cast<char *>(ws) + bp_ws_ts_bytes(g));
    return w;
}

// Prefix table of view ia's sinogram row (row[j], global or shared memory)
// and the view's line scales, by one block of NT threads (a multiple of 32;
// wsum holds NT / 32 doubles).
template <bool FAN, int NT = 256>
__device__ __forceinline__ void bp_prep_view(const vg_dd2d_geom &g, const float *row, int ia,
                                             const double *__restrict__ trig, BpWork w,
                                             double *wsum) {
    float2 *ts = w.ts + (size_t)ia * bp_tab_len(g.nu);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // contiguous segment per thread
    const int per = (g.nu + NT - 1) / NT;
    const int j0 = threadIdx.x * per;
    double loc = 0.0;
    for (int i = 0; i < per; ++i)
        if (j0 + i < g.nu) loc += (double)row[j0 + i];
    double inc = loc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    double off = 0.0;
    for (int q = 0; q < warp; ++q) off += wsum[q];
    double run = off + inc - loc;
    const double du = (double)g.du;
    const float yk = g.du * (float)(g.nu + 2);
    for (int i = 0; i < per; ++i) {
        const int j = j0 + i;
        if (j < g.nu) {
            const float sv = row[j];
            ts[j + 1] = make_float2((float)((run - (double)(j + 1) * (double)sv) * du), yk * sv);
            run += (double)sv;
        }
    }
    if (threadIdx.x == 0) ts[0] = make_float2(0.f, 0.f);
    if (threadIdx.x == NT - 1) {
        ts[g.nu + 1] = make_float2((float)(run * du), 0.f);
        ts[g.nu + 2] = make_float2((float)(run * du), 0.f);
    }
    // line scales of this view, negated for lines whose edges project in
    // decreasing order (the pixel's interval is then [P(b+1), P(b)])
    const ViewGeo v = view_geo(trig, ia);
    const int no = v.xdrv ? g.ny : g.nx;
    const int nd = v.xdrv ? g.nx : g.ny;
    for (int io = threadIdx.x; io < no; io += NT) {
        const Line L = line_geo<FAN>(g, v, centre_coord(g.d_pix, io, no));
        const float P0 = proj<FAN>(g, v, L.cp, L.co, edge_coord(g.d_pix, 0, nd));
        const float P1 = proj<FAN>(g, v, L.cp, L.co, edge_coord(g.d_pix, nd, nd));
        w.scl[(size_t)ia * scl_stride(g) + io] = P1 >= P0 ? L.scl : -L.scl;
    }
}

// mode 0: out = FP;  mode 1 (SIRT residual): out = (y - FP) * inv_w, or FP
// where inv_w == 0;  mode 2: mode 1, and the block (256 threads, all bins of
// the view) then writes the view's back-projection table and line scales
// into pw, as dd2d_bp_prep would from the residual row.
// One block's work: view ia, bins chunk * 32 FP_MAXB ...  smem2: the line
// buffers (FP_WARPS fp_line_entries(nd) float2, also the warps' bin sums);
// UC: 32 FP_MAXB + 32 float2 of shared memory.
template <bool FAN, int FP_WARPS, int FP_MAXB, bool GUARD, typename TX, typename TY, bool COH = false>
__device__ __forceinline__ void fp_block(const vg_dd2d_geom &g, int ia, int chunk,
                                         const TX *__restrict__ img, const TX *__restrict__ imgT,
                                         const double *__restrict__ trig, float *__restrict__ out,
                                         int mode, const TY *__restrict__ y,
                                         const float *__restrict__ inv_w, BpWork pw, float2 *smem2,
                                         float2 *UC) {
    constexpr int FP_BINS = 32 * FP_MAXB;  // bins per block
    const ViewGeo v = view_geo(trig, ia);
    const int nd = v.xdrv ? g.nx : g.ny;
    const int no = v.xdrv ? g.ny : g.nx;
    const TX *base = v.xdrv ? imgT : img;  // line io is contiguous in k
    const bool rev = v.pd < 0.f;               // edges decreasing in k: sweep reversed
    const int stride = fp_line_entries(nd);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // rows start on 64-byte boundaries when nd % 16 == 0 (and the image is 16-byte aligned)
    const bool vec_rows = (nd % FP_SEG == 0) && ((reinterpret_cast<uintptr_t>(base) & 15) == 0);
    float2 *E = smem2 + (size_t)warp * stride;  // this warp's line buffer
    const int jbase = chunk * FP_BINS;
    const int nb = min(FP_BINS, g.nu - jbase);  // bins of this block
    const float half = 0.5f * (float)nd;
    // The inverse edge map has a pole at U* = -DSD pd / od (rays parallel to
    // the lines).  It lies outside every line's shadow, but a detector wider
    // than 2 DSD can reach it (|U*| >= DSD since |pd| >= |od|): then the
    // GUARD instantiation runs, and a block whose bins contain the pole
    // evaluates F directly as 0 before the line's first projected edge and
    // the line total after its last, instead of trusting the inverse map
    // beyond the pole.
    bool guard = false;
    if (GUARD && FAN && v.od != 0.f) {
        const float Up = -g.DSD * v.pd / v.od;
        const float Ua = det_edge(g, jbase), Ub = det_edge(g, jbase + nb);
        guard = Up >= fminf(Ua, Ub) && Up <= fmaxf(Ua, Ub);
    }

    // Line-independent factor of the inverse map at every bin edge, scaled
    // for the slot lookup: with the sweep index s(U) = (U a_l - b_l) C(U) + nd/2,
    // the walk forms t = sat((s + 1) / (nd + 2)) = sat((U a_l - b_l) C' + h')
    // with C' = C / (nd + 2), h' = (nd/2 + 1) / (nd + 2); floor(t (nd + 2)) - 1
    // is the pixel under U, clamped to -1 .. nd + 1 by the saturation (NaN
    // gives 0, the sentinel).
    const float ndp2 = (float)(nd + 2);
    const float hq = (half + 1.f) / ndp2;
    {
        const float sig = (rev ? -1.f : 1.f) / (g.d_pix * ndp2);
        for (int e = threadIdx.x; e < FP_BINS + 32; e += FP_WARPS * 32) {
            const float U = det_edge(g, jbase + min(e, nb));
            UC[e] = make_float2(U, FAN ? sig / (g.DSD * v.pd + U * v.od) : sig / v.pd);
        }
    }
    __syncthreads();

    float acc[FP_MAXB];
#pragma unroll
    for (int i = 0; i < FP_MAXB; ++i) acc[i] = 0.f;

    // Stages line io into buffer Eb: (G, V) per pixel, the sentinel and the
    // closing edges; returns the line's inverse-map coefficients (la, lb) and,
    // for the guard, its first and last projected edges (Pf <= Pl).  The sweep
    // direction RVC is a compile-time constant in each of the two copies.
    auto stage = [&](auto RVC, int io, float2 *Eb, float &la, float &lb, float &Pf, float &Pl) {
        const bool RV = RVC;
        const Line Lg = line_geo<FAN>(g, v, centre_coord(g.d_pix, io, no));
        la = FAN ? g.DSO - Lg.co : 1.f;       // inverse map numerator U la - lb
        lb = FAN ? g.DSD * Lg.cp : Lg.cp;
        if (GUARD) {
            Pf = proj<FAN>(g, v, Lg.cp, Lg.co, edge_coord(g.d_pix, RV ? nd : 0, nd));
            Pl = proj<FAN>(g, v, Lg.cp, Lg.co, edge_coord(g.d_pix, RV ? 0 : nd, nd));
        }
        const TX *row = base + (size_t)io * nd;
        // lanes own FP_SEG consecutive pixels (edge coordinate b0 + i db along
        // a lane's segment); along the segment the projection's numerator and
        // denominator are affine in the edge number i: P_i = (n0 + i dn) / (d0 + i dd).
        const float db = RV ? -g.d_pix : g.d_pix;
        const float dn = (FAN ? g.DSD : 1.f) * v.pd * db;
        const float dd = -v.od * db;
        float carry = 0.f;
        for (int r0 = 0; r0 < nd; r0 += 32 * FP_SEG) {
            const int m0 = r0 + lane * FP_SEG;
            const float b0 = edge_coord(g.d_pix, RV ? nd - m0 : m0, nd);
            const float n0 = (FAN ? g.DSD : 1.f) * fmaf(v.pd, b0, Lg.cp);
            const float d0 = g.DSO - fmaf(v.od, b0, Lg.co);
            float Pv[FP_SEG + 1], q[FP_SEG];
#pragma unroll
            for (int i = 0; i <= FP_SEG; ++i) {
                const float num = fmaf((float)i, dn, n0);
#if VG_FAST_DIV
                float r;  // approximate reciprocal (as __fdividef, without its range scaling)
                asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(fmaf((float)i, dd, d0)));
                Pv[i] = FAN ? num * r : num;
#else
                Pv[i] = FAN ? num / fmaf((float)i, dd, d0) : num;
#endif
            }
            // pixels m0 .. m0 + FP_SEG - 1 (sweep order): 16-byte loads when
            // the segment is whole and aligned, else element by element
            float tot = 0.f;
            if (vec_rows && m0 + FP_SEG <= nd) {
                static_assert(FP_SEG == 8, "segments of 8 pixels (one 16-byte load of bfloat16)");
                float raw[FP_SEG];
                ld8<COH>(row + (RV ? nd - FP_SEG - m0 : m0), raw);
#pragma unroll
                for (int i = 0; i < FP_SEG; ++i) q[i] = (RV ? raw[FP_SEG - 1 - i] : raw[i]) * Lg.scl;
            } else {
                const TX *px = row + (RV ? nd - 1 - m0 : m0);
                const int step = RV ? -1 : 1;
#pragma unroll
                for (int i = 0; i < FP_SEG; ++i)
                    q[i] = (m0 + i < nd) ? ldf<COH>(px + i * step) * Lg.scl : 0.f;
            }
            float D[FP_SEG];
#pragma unroll
            for (int i = 0; i < FP_SEG; ++i) {
                D[i] = Pv[i + 1] - Pv[i];
                tot = fmaf(q[i], D[i], tot);
            }
            float inc = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += t;
            }
            float run = carry + inc - tot;
            carry += __shfl_sync(0xffffffffu, inc, 31);
            const int lim = nd - m0;  // pixel entries m0 + i with i < lim exist
            float2 *seg = Eb + fp_slot(m0);  // the segment's slots are consecutive
            if (lim >= FP_SEG) {
#pragma unroll
                for (int i = 0; i < FP_SEG; ++i) {
                    seg[i] = make_float2(fmaf(-q[i], Pv[i], run), q[i]);
                    run = fmaf(q[i], D[i], run);
                }
            } else {
#pragma unroll
                for (int i = 0; i < FP_SEG; ++i) {
                    if (i < lim) seg[i] = make_float2(fmaf(-q[i], Pv[i], run), q[i]);
                    run = fmaf(q[i], D[i], run);
                }
            }
        }
        // the sentinel before the first edge and the closing edges (line total)
        if (lane == 0) {
            Eb[fp_slot(-1)] = make_float2(0.f, 0.f);
            Eb[fp_slot(nd)] = make_float2(carry, 0.f);
            Eb[fp_slot(nd + 1)] = make_float2(carry, 0.f);
        }
    };

    // F of a staged line (shared address eb of its slot 0) at detector edge
    // (U, C'(U)): the slot comes from the bit pattern of a round-down FMA of t
    // onto 1.5 * 2^23 + 15 (FP_SLOT_BIAS), without clamps or conversions.
    const unsigned eb = (unsigned)__cvta_generic_to_shared(E) - 8u * FP_SLOT_BIAS;
    auto F = [&](float la, float lb, float Pf, float Pl, float2 uc) {
        float t;
        asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(t) : "f"(fmaf(uc.x, la, -lb)), "f"(uc.y), "f"(hq));
        if (guard) t = uc.x <= Pf ? 0.f : (uc.x >= Pl ? 1.f : t);
        const unsigned b = __float_as_uint(__fmaf_rd(t, ndp2, 12582927.0f));
        float2 e;
        asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];"
                     : "=f"(e.x), "=f"(e.y)
                     : "r"(eb + 8u * (b + (b >> 4))));
        return fmaf(e.y, uc.x, e.x);
    };

    // Each warp stages its lines io = warp, warp + FP_WARPS, ... one at a
    // time and walks the bin edges.  F at the left edge of bin lane + 32 i is
    // streamed: bin i - 1 is finished as soon as edge i is known.  Its right
    // edge is lane + 1's left edge, or for lane 31 lane 0's next one -- one
    // rotation of (lane 0 ? F(edge i) : F(edge i - 1)).
    const int src = (lane + 1) & 31;
    for (int io = warp; io < no; io += FP_WARPS) {
        float la, lb, Pf = 0.f, Pl = 0.f;
        __syncwarp();  // previous line's reads are done
        if (rev) stage(BoolC<true>{}, io, E, la, lb, Pf, Pl);
        else stage(BoolC<false>{}, io, E, la, lb, Pf, Pl);
        __syncwarp();
        float f_prev = 0.f;
#pragma unroll
        for (int i = 0; i <= FP_MAXB; ++i) {
            const float2 uc = UC[lane + 32 * i];  // edges past nb repeat the last one
            const float f_new = F(la, lb, Pf, Pl, uc);
            if (i > 0) {
                const float r = __shfl_sync(0xffffffffu, lane == 0 ? f_new : f_prev, src);
                acc[i - 1] += r - f_prev;
            }
            f_prev = f_new;
        }
    }

    // sum the warps' partial bins in a fixed order
    __syncthreads();
    float *red = reinterpret_cast<float *>(smem2);  // [FP_WARPS][FP_BINS]
#pragma unroll
    for (int i = 0; i < FP_MAXB; ++i) red[warp * FP_BINS + lane + 32 * i] = acc[i];
    __syncthreads();
    const float f = g.d_pix / g.du;
    float *resid = reinterpret_cast<float *>(UC);  // mode 2: the residual row (UC is no longer read)
    for (int e = threadIdx.x; e < nb; e += FP_WARPS * 32) {
        float sum = 0.f;
#pragma unroll
        for (int w = 0; w < FP_WARPS; ++w) sum += red[w * FP_BINS + e];
        float fp = sum * f;
        const size_t o = (size_t)ia * g.nu + jbase + e;
        if (mode >= 1) {
            const float wi = inv_w[o];
            fp = (wi != 0.f) ? (ldf(y + o) - fp) * wi : fp;
        }
        out[o] = fp;
        if (FP_WARPS == 8 && mode == 2) resid[e] = fp;
    }
    if (FP_WARPS == 8 && mode == 2) {
        __shared__ double wsum[8];
        __syncthreads();
        bp_prep_view<FAN>(g, resid, ia, trig, pw, wsum);
    }
}

#ifndef VG_FP_MINB8
#define VG_FP_MINB8 3
#endif
// (the guarded variants of the 24-bin tiles give up occupancy rather than spill)
template <bool FAN, int FP_WARPS, int FP_MAXB, bool GUARD>
__global__ void __launch_bounds__(FP_WARPS * 32, ((FP_MAXB > 24 || (GUARD && FP_MAXB == 24)) ? 1 : (FP_WARPS >= 8 ? (FP_MAXB == 24 ? VG_FP_MINB8 : 2) : 16 / FP_WARPS)))
dd2d_fp_kernel(vg_dd2d_geom g, const float *__restrict__ img, const float *__restrict__ imgT,
               const double *__restrict__ trig, float *__restrict__ out, int mode,
               const float *__restrict__ y, const float *__restrict__ inv_w, BpWork pw) {
    extern __shared__ float2 smem2[];
    __shared__ float2 UC[32 * FP_MAXB + 32];  // per bin edge (U, C'(U)); entries past nb repeat nb
    fp_block<FAN, FP_WARPS, FP_MAXB, GUARD, float, float>(g, blockIdx.y, blockIdx.x, img, imgT, trig,
                                                           out, mode, y, inv_w, pw, smem2, UC);
}

// ---------------------------------------------------------------------------
// Backprojection (integral form)
//
// For one view, let G(u) be the running integral of the sinogram row as a
// piecewise-constant function of u (bin j spans [U_j, U_j+1]):
//     G(u) = T_j + du sino_j (t - j),  t = (u - U_0)/du,  j = floor(t),  T_j = du sum_{i<j} sino_i.
// A pixel whose driving edges project to lo <= hi receives
// scale(line) * (G(hi) - G(lo)) from the view -- the sum of sino * overlap *
// scale that vir's merge distributes.  dd2d_bp_prep writes, per view, the
// table (T_j - j du sino_j, du sino_j) (prefix accumulated in FP64), so that
// G = x_j + y_j t, and the line scales signed by the direction in which the
// line's edges project; the main kernel evaluates G at the two projected
// edges of each pixel.
// ---------------------------------------------------------------------------

// Tile of the back projection: BP_TY x BP_TX patches of 2 x 2 pixels, the
// threads numbered along y first, so that a warp covers 8 x 4 patches
// (16 x 8 pixels) when BP_TY = 8: its table gathers span fewer bins than a
// warp along a 64 x 2 strip (0.213 against 0.233 ms at the fan SIRT size,
// with the view loop unrolled by 4).
#ifndef VG_BP_TY
#define VG_BP_TY 8
#endif
#ifndef VG_BP_TX
#define VG_BP_TX 32
#endif
#ifndef VG_BP_MINB
#define VG_BP_MINB 1
#endif
#ifndef VG_BP_UNROLL
#define VG_BP_UNROLL 4
#endif
constexpr int BP_UNROLL = VG_BP_UNROLL;  // views per unrolled step of the view loop
constexpr int BP_TY = VG_BP_TY;  // patches along y (threadIdx.x, contiguous in img)
constexpr int BP_TX = VG_BP_TX;  // patches along x (threadIdx.y)
constexpr int BP_VC = (BP_TY * BP_TX < 128) ? BP_TY * BP_TX : 128;  // views staged per chunk


// One block per view: prefix table of the sinogram row and line scales.
template <bool FAN>
__global__ void __launch_bounds__(256)
dd2d_bp_prep(vg_dd2d_geom g, const float *__restrict__ sino, const double *__restrict__ trig,
             BpWork w) {
    __shared__ double wsum[8];
    bp_prep_view<FAN>(g, sino + (size_t)blockIdx.x * g.nu, blockIdx.x, trig, w, wsum);
}

__device__ __forceinline__ float rcp_approx(float x) {
#if VG_FAST_DIV
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / x;
#endif
}

// G at the lookup coordinate tq = sat((t + 1) / (nu + 2)) (see bp_tab_len):
// the slot floor(tq (nu + 2)) is the bit pattern of a round-down FMA onto
// 1.5 * 2^23 less that constant's, folded into the address.
template <bool COH = false>
__device__ __forceinline__ float bp_G(const float2 *__restrict__ ts, float nup2, float tq) {
    const unsigned bits = __float_as_uint(__fmaf_rd(tq, nup2, 12582912.0f));
    const float2 *p = reinterpret_cast<const float2 *>(reinterpret_cast<uintptr_t>(ts) +
                                                      8ull * bits - 8ull * 0x4B400000u);
    const float2 e = ldro<COH>(p);
    return fmaf(e.y, tq, e.x);
}

// a b + c saturated to [0, 1] (NaN to 0)
__device__ __forceinline__ float fma_sat(float a, float b, float c) {
    float r;
    asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Each thread owns a 2x2 pixel patch.  A view drives along x (X-driven) or y:
// its two orthogonal lines through the patch share three driving edges each,
// so per view the patch needs 6 edge projections and 6 running-integral
// lookups for its 4 pixels, and the view and line parameters are read once.
// mode 0: img = BP;  mode 1 (SIRT update): x += gamma * BP * inv_w (BP where
// inv_w == 0), written to x and its transpose xT.
// One block's work: the pixel tile (tile_y, tile_x) of BP_TY x BP_TX patches.
template <bool FAN, typename TX, bool COH = false>
__device__ __forceinline__ void bp_block(const vg_dd2d_geom &g, int tile_y, int tile_x, BpWork w,
                                         const double *__restrict__ trig, TX *__restrict__ img,
                                         int mode, const float *__restrict__ inv_w, float gamma,
                                         TX *__restrict__ xT) {
    // per view: fan (DSD pd/du, -od, DSD po/du, -oo), parallel (pd/du, 0, po/du, 0):
    // an edge b on the line through cen lands at bin position
    //   t = (x b + z cen) / (DSO + y b + w cen) + t0   (fan)
    //   t = x b + z cen + t0                           (parallel)
    __shared__ float4 Vs[BP_VC];
    __shared__ int Xs[BP_VC];
    // linear thread index (2D blocks of BP_TY x BP_TX, or 1D blocks of as many)
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int tx = tid % BP_TY, ty = tid / BP_TY;
    const int iy = tile_y * (2 * BP_TY) + 2 * tx;  // patch origin
    const int ix = tile_x * (2 * BP_TX) + 2 * ty;
    const bool inside = iy < g.ny && ix < g.nx;
    const int sstr = scl_stride(g);
    // lookup coordinate tq = (t + 1) / (nu + 2): the view coefficients and the
    // offset carry the factor
    const float nup2 = (float)(g.nu + 2), kq = 1.f / nup2;
    const float t0 = (1.f - det_edge(g, 0) / g.du) * kq;
    const float bx = edge_coord(g.d_pix, ix, g.nx), by = edge_coord(g.d_pix, iy, g.ny);
    const float cx0 = bx + 0.5f * g.d_pix, cy0 = by + 0.5f * g.d_pix;
    const float2 *ts_all = w.ts;
    Kahan acc[2][2];
    for (int a0 = 0; a0 < g.na; a0 += BP_VC) {
        const int nv = min(BP_VC, g.na - a0);
        __syncthreads();
        if (tid < nv) {
            const ViewGeo v = view_geo(trig, a0 + tid);
            const float k = (FAN ? g.DSD : 1.f) / g.du * kq;
            Vs[tid] = FAN ? make_float4(k * v.pd, -v.od, k * v.po, -v.oo)
                          : make_float4(k * v.pd, 0.f, k * v.po, 0.f);
            Xs[tid] = v.xdrv;
        }
        __syncthreads();
        if (!inside) continue;
        float part[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll BP_UNROLL
        for (int vi = 0; vi < nv; ++vi) {
            const float4 q = Vs[vi];
            const bool xd = Xs[vi];
            const float b0 = xd ? bx : by;    // first driving edge of the patch
            const float c0 = xd ? cy0 : cx0;  // centre of the first line
            const int io0 = xd ? iy : ix;
            const int no = xd ? g.ny : g.nx;
            const float2 *ts = ts_all + (size_t)(a0 + vi) * bp_tab_len(g.nu);
            // signed scales of lines io0 and io0 + 1 (io0 is even; rows padded)
            const float2 sc2 = ldro<COH>(reinterpret_cast<const float2 *>(w.scl + (size_t)(a0 + vi) * sstr + io0));
            float cL[2][2];  // [line][position along the driving axis]
#pragma unroll
            for (int L = 0; L < 2; ++L) {
                const float cen = c0 + (float)L * g.d_pix;
                const float nc = FAN ? q.z * cen : fmaf(q.z, cen, t0);
                const float dc = fmaf(q.w, cen, g.DSO);
                float G[3];
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    const float b = fmaf((float)e, g.d_pix, b0);
                    const float tq = FAN ? fma_sat(fmaf(q.x, b, nc), rcp_approx(fmaf(q.y, b, dc)), t0)
                                         : fma_sat(q.x, b, nc);
                    G[e] = bp_G<COH>(ts, nup2, tq);
                }
                const float s = (io0 + L < no) ? (L ? sc2.y : sc2.x) : 0.f;
                cL[L][0] = (G[1] - G[0]) * s;
                cL[L][1] = (G[2] - G[1]) * s;
            }
            // X-driven: line = y offset, position = x offset; Y-driven: the transpose
            part[0][0] += cL[0][0];
            part[1][1] += cL[1][1];
            part[1][0] += xd ? cL[0][1] : cL[1][0];
            part[0][1] += xd ? cL[1][0] : cL[0][1];
        }
#pragma unroll
        for (int dx = 0; dx < 2; ++dx)
#pragma unroll
            for (int dy = 0; dy < 2; ++dy) acc[dx][dy].add(part[dx][dy]);
    }
    if (!inside) return;
    const float f = 1.0f / ((float)g.na * g.d_pix);
#pragma unroll
    for (int dx = 0; dx < 2; ++dx)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            const int px = ix + dx, py = iy + dy;
            if (px >= g.nx || py >= g.ny) continue;
            const float bp = acc[dx][dy].s * f;
            const size_t o = (size_t)px * g.ny + py;
            if (mode == 1) {
                const float wi = inv_w[o];
                const float upd = (wi != 0.f) ? bp * wi : bp;
                const float xn = ldf_plain(img + o) + gamma * upd;
                stf(img + o, xn);
                stf(xT + (size_t)py * g.nx + px, xn);
            } else {
                stf(img + o, bp);
            }
        }
}

template <bool FAN>
__global__ void __launch_bounds__(BP_TY * BP_TX, VG_BP_MINB)
dd2d_bp_kernel(vg_dd2d_geom g, BpWork w, const double *__restrict__ trig,
               float *__restrict__ img, int mode, const float *__restrict__ inv_w, float gamma,
               float *__restrict__ xT) {
    bp_block<FAN, float>(g, blockIdx.x, blockIdx.y, w, trig, img, mode, inv_w, gamma, xT);
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

template <bool FAN, int W, int B>
int launch_fp_t(const vg_dd2d_geom *g, const float *img, const float *imgT, const double *trig,
                float *out, int mode, const float *y, const float *inv_w, cudaStream_t st,
                BpWork pw) {
    const int nd = g->nx > g->ny ? g->nx : g->ny;
    size_t smem = (size_t)W * fp_line_entries(nd) * sizeof(float2);
    const size_t red = (size_t)W * 32 * B * sizeof(float);
    if (smem < red) smem = red;
    VG_REQUIRE(smem <= 200 * 1024, "dd2d_fp: image side too large for this tile variant");
    // the inverse map's pole can reach the detector only when it extends
    // beyond DSD from the centre
    const float ext = fmaxf(fabsf(g->du * (0.f - 0.5f * g->nu + g->su)),
                            fabsf(g->du * ((float)g->nu - 0.5f * g->nu + g->su)));
    const bool guard = FAN && ext >= g->DSD;
    auto kern = guard ? dd2d_fp_kernel<FAN, W, B, true> : dd2d_fp_kernel<FAN, W, B, false>;
    static size_t attr[2] = {0, 0};  // per instantiation: largest dynamic smem already allowed
    if (smem > 48 * 1024 && smem > attr[guard]) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e == cudaSuccess)  // the largest carveout, so that the tile's blocks per SM fit
            e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return cuda_status(e, "dd2d_fp: shared memory attribute");
        attr[guard] = smem;
    }
    dim3 grid(ceil_div(g->nu, 32 * B), g->na);
    kern<<<grid, W * 32, smem, st>>>(*g, img, imgT, trig, out, mode, y, inv_w, pw);
    return launch_status("dd2d_fp");
}

// Size heuristic: the fewest bins per lane covering the detector in one
// block, and fewer warps (line buffers) for long lines.
int fp_variant_for(const vg_dd2d_geom *g) {
    const int nd = g->nx > g->ny ? g->nx : g->ny;
    if (nd > 512) return g->nu > 768 ? 5 : 4;
    if (g->nu <= 192) return 1;
    if (g->nu <= 384) return 2;
    return g->nu <= 768 ? 3 : 5;
}

template <bool FAN>
int launch_fp_fan(int v, const vg_dd2d_geom *g, const float *img, const float *imgT,
                  const double *trig, float *out, int mode, const float *y, const float *inv_w,
                  cudaStream_t st, BpWork pw) {
    switch (v) {
        case 1: return launch_fp_t<FAN, 8, 6>(g, img, imgT, trig, out, mode, y, inv_w, st, pw);
        case 2: return launch_fp_t<FAN, 8, 12>(g, img, imgT, trig, out, mode, y, inv_w, st, pw);
        case 3: return launch_fp_t<FAN, 8, 24>(g, img, imgT, trig, out, mode, y, inv_w, st, pw);
        case 4: return launch_fp_t<FAN, 4, 24>(g, img, imgT, trig, out, mode, y, inv_w, st, pw);
        case 5: return launch_fp_t<FAN, 4, 48>(g, img, imgT, trig, out, mode, y, inv_w, st, pw);
        case 6: return launch_fp_t<FAN, 2, 48>(g, img, imgT, trig, out, mode, y, inv_w, st, pw);
        default: VG_REQUIRE(false, "dd2d_fp: variant %d out of range 0..%d", v, FP_NVARIANTS);
    }
}

// Variant in use: the caller's, else the tile heuristic.
int fp_variant_used(const vg_dd2d_geom *g) { return g->variant ? g->variant : fp_variant_for(g); }

int launch_fp(const vg_dd2d_geom *g, const float *img, const float *imgT, const double *trig,
              float *out, int mode, const float *y, const float *inv_w, cudaStream_t st,
              BpWork pw = BpWork{nullptr, nullptr}) {
    const int v = fp_variant_used(g);
    return g->fan ? launch_fp_fan<true>(v, g, img, imgT, trig, out, mode, y, inv_w, st, pw)
                  : launch_fp_fan<false>(v, g, img, imgT, trig, out, mode, y, inv_w, st, pw);
}

// The SIRT forward projection can also write the back projection's tables
// (mode 2) when one block of 8 warps holds all bins of a view.
bool fp_builds_bp_tables(const vg_dd2d_geom *g) {
    const int v = fp_variant_used(g);
    if (v < 1 || v > FP_NVARIANTS) return false;
    return FP_VARIANTS[v - 1].warps == 8 && 32 * FP_VARIANTS[v - 1].maxb >= g->nu;
}

int launch_bp(const vg_dd2d_geom *g, const float *sino, const double *trig, float *img, int mode,
              const float *inv_w, float gamma, float *xT, void *ws, size_t ws_bytes,
              cudaStream_t st, bool prep = true) {
    VG_REQUIRE(ws != nullptr && ws_bytes >= bp_ws_bytes(g),
               "dd2d_bp: workspace of %zu bytes needed (vg_dd2d_workspace_bytes)", bp_ws_bytes(g));
    VG_REQUIRE(((uintptr_t)ws & 255) == 0, "dd2d_bp: workspace must be 256-byte aligned");
    const BpWork w = bp_ws(g, ws);
    if (prep) {
        if (g->fan) dd2d_bp_prep<true><<<g->na, 256, 0, st>>>(*g, sino, trig, w);
        else        dd2d_bp_prep<false><<<g->na, 256, 0, st>>>(*g, sino, trig, w);
        int s = launch_status("dd2d_bp_prep");
        if (s) return s;
    }
    dim3 grid(ceil_div(g->ny, 2 * BP_TY), ceil_div(g->nx, 2 * BP_TX));
    VG_REQUIRE(grid.y < 65536, "dd2d_bp: nx too large");
    dim3 block(BP_TY, BP_TX);
    if (g->fan)
        dd2d_bp_kernel<true><<<grid, block, 0, st>>>(*g, w, trig, img, mode, inv_w, gamma, xT);
    else
        dd2d_bp_kernel<false><<<grid, block, 0, st>>>(*g, w, trig, img, mode, inv_w, gamma, xT);
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

extern "C" int vg_dd2d_fp_variants(void) { return FP_NVARIANTS; }

extern "C" int vg_dd2d_fp_default_variant(const vg_dd2d_geom *g) {
    return check_geom(g) ? 0 : fp_variant_used(g);
}

extern "C" size_t vg_dd2d_workspace_bytes(const vg_dd2d_geom *g) {
    if (check_geom(g)) return 0;
    return bp_ws_bytes(g);
}

extern "C" int vg_dd2d_bp(const vg_dd2d_geom *g, const float *sino, const double *trig,
                          float *img, void *workspace, size_t workspace_bytes, void *stream) {
    int st = check_geom(g);
    if (st) return st;
    VG_REQUIRE(img && trig && sino, "dd2d_bp: null pointer");
    return launch_bp(g, sino, trig, img, 0, nullptr, 0.f, nullptr, workspace, workspace_bytes,
                     as_stream(stream));
}

namespace {
int check_sirt_ws(const vg_dd2d_geom *g, const void *workspace, size_t workspace_bytes) {
    VG_REQUIRE(workspace != nullptr && workspace_bytes >= bp_ws_bytes(g),
               "dd2d_sirt: workspace of %zu bytes needed (vg_dd2d_workspace_bytes)",
               bp_ws_bytes(g));
    VG_REQUIRE(((uintptr_t)workspace & 255) == 0, "dd2d_sirt: workspace must be 256-byte aligned");
    return VG_OK;
}
// the residual's back-projection tables come from the forward projection's
// epilogue when its block holds whole views (no separate table launch)
bool sirt_fused(const vg_dd2d_geom *g) { return VG_SIRT_FUSED_TABLES && fp_builds_bp_tables(g); }
}  // namespace

extern "C" int vg_dd2d_sirt_residual(const vg_dd2d_geom *g, const float *y,
                                     const float *inv_w_sino, const double *trig, const float *x,
                                     const float *xT, float *r, void *workspace,
                                     size_t workspace_bytes, void *stream) {
    int st = check_geom(g);
    if (st) return st;
    VG_REQUIRE(y && inv_w_sino && trig && x && xT && r, "dd2d_sirt_residual: null pointer");
    st = check_sirt_ws(g, workspace, workspace_bytes);
    if (st) return st;
    return launch_fp(g, x, xT, trig, r, sirt_fused(g) ? 2 : 1, y, inv_w_sino, as_stream(stream),
                     bp_ws(g, workspace));
}

extern "C" int vg_dd2d_sirt_update(const vg_dd2d_geom *g, const float *inv_w_img, float gamma,
                                   const double *trig, float *x, float *xT, const float *r,
                                   void *workspace, size_t workspace_bytes, void *stream) {
    int st = check_geom(g);
    if (st) return st;
    VG_REQUIRE(inv_w_img && trig && x && xT && r, "dd2d_sirt_update: null pointer");
    st = check_sirt_ws(g, workspace, workspace_bytes);
    if (st) return st;
    return launch_bp(g, r, trig, x, 1, inv_w_img, gamma, xT, workspace, workspace_bytes,
                     as_stream(stream), !sirt_fused(g));
}

extern "C" int vg_dd2d_sirt_iter(const vg_dd2d_geom *g, const float *y, const float *inv_w_sino,
                                 const float *inv_w_img, float gamma, const double *trig,
                                 float *x, float *xT, float *r, void *workspace,
                                 size_t workspace_bytes, void *stream) {
    int st = vg_dd2d_sirt_residual(g, y, inv_w_sino, trig, x, xT, r, workspace, workspace_bytes,
                                   stream);
    if (st) return st;
    return vg_dd2d_sirt_update(g, inv_w_img, gamma, trig, x, xT, r, workspace, workspace_bytes,
                               stream);
}

extern "C" int vg_dd2d_sirt_launches(const vg_dd2d_geom *g) {
    if (check_geom(g) != VG_OK) return 0;
    return sirt_fused(g) ? 2 : 3;
}

// ---------------------------------------------------------------------------
// Allocation-free backprojection.
//
// Some callers cannot allocate device memory at call time: a host
// application that hands this library a fixed memory budget and owns every
// allocation itself, code running where cudaMalloc's implicit device
// synchronisation is not acceptable (a real-time acquisition loop), or a
// plugin whose host forbids allocation inside its callbacks.  For them
// vg_dd2d_bp_noalloc does the same backprojection as vg_dd2d_bp with the
// workspace taken from a fixed array in device memory that is part of this
// library (VG_NOALLOC_SCRATCH_BYTES = 32 MiB, held on every device that
// loads the library until the process exits).
//
// - The caller still passes the sinogram and the output image.
// - Geometries whose workspace (vg_dd2d_workspace_bytes) exceeds 32 MiB are
//   rejected with VG_ERR_ARG.
// - The first call in a CUDA context (normally a device's primary context),
//   with that context current, looks up the array's device address
//   (cudaGetSymbolAddress) and caches it under the context's unique id
//   (cuCtxGetId, never reused within a process, so a context created after a
//   device reset or a non-primary context gets its own lookup); make that
//   first call before any stream capture.
// - Every call shares the one array: calls whose executions overlap on the
//   GPU (different streams, or concurrent host threads) race and corrupt
//   each other's results.  Serialise them, e.g. on one stream.
// - Each call rewrites every workspace entry it later reads, so the array's
//   leftover contents from an earlier call do not matter and nothing needs
//   clearing.
// ---------------------------------------------------------------------------

#define VG_NOALLOC_SCRATCH_BYTES (32u << 20)
#define VG_NOALLOC_MAX_CONTEXTS 64

static __device__ __align__(256) unsigned char g_dd2d_scratch[VG_NOALLOC_SCRATCH_BYTES];

#include <mutex>

namespace {
std::mutex g_scratch_mu;
struct ScratchEntry {
    unsigned long long ctx_id;
    void *addr;
};
ScratchEntry g_scratch_cache[VG_NOALLOC_MAX_CONTEXTS] = {};
int g_scratch_n = 0;

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points (the
// library links only the CUDA runtime, so it loads where libcuda is absent).
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Unique id of the current context; with none current yet, the current
// device's primary context is made current first (cudaSetDevice does that).
int current_context_id(unsigned long long *id) {
    cudaError_t e;
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void *f0 = nullptr, *f1 = nullptr;
        cudaDriverEntryPointQueryResult q0, q1;
        e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0);
        if (e != cudaSuccess || q0 != cudaDriverEntryPointSuccess || !f0)
            return cuda_status(e != cudaSuccess ? e : cudaErrorNotSupported,
                               "dd2d_bp_noalloc: cuCtxGetCurrent entry point");
        e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1);
        if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess || !f1)
            return cuda_status(e != cudaSuccess ? e : cudaErrorNotSupported,
                               "dd2d_bp_noalloc: cuCtxGetId entry point");
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f1);
    }
    void *ctx = nullptr;
    VG_REQUIRE(g_ctx_get_current(&ctx) == 0, "dd2d_bp_noalloc: cuCtxGetCurrent failed");
    if (!ctx) {
        int dev = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaSetDevice(dev);
        if (e != cudaSuccess) return cuda_status(e, "dd2d_bp_noalloc: device context");
        VG_REQUIRE(g_ctx_get_current(&ctx) == 0 && ctx, "dd2d_bp_noalloc: no current CUDA context");
    }
    VG_REQUIRE(g_ctx_get_id(ctx, id) == 0, "dd2d_bp_noalloc: cuCtxGetId failed");
    return VG_OK;
}

// Device address of g_dd2d_scratch in the current context (looked up once
// per context, keyed on the context's process-unique id).
int scratch_address(void **out) {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    unsigned long long id = 0;
    int st = current_context_id(&id);
    if (st) return st;
    for (int i = 0; i < g_scratch_n; ++i)
        if (g_scratch_cache[i].ctx_id == id) {
            *out = g_scratch_cache[i].addr;
            return VG_OK;
        }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_dd2d_scratch);
    if (e != cudaSuccess) return cuda_status(e, "dd2d_bp_noalloc: cudaGetSymbolAddress");
    // a full table drops its oldest entry (that context's next call looks up again)
    if (g_scratch_n == VG_NOALLOC_MAX_CONTEXTS) {
        for (int i = 1; i < g_scratch_n; ++i) g_scratch_cache[i - 1] = g_scratch_cache[i];
        --g_scratch_n;
    }
    g_scratch_cache[g_scratch_n++] = ScratchEntry{id, p};
    *out = p;
    return VG_OK;
}
}  // namespace

extern "C" size_t vg_dd2d_noalloc_scratch_bytes(void) { return VG_NOALLOC_SCRATCH_BYTES; }

extern "C" int vg_dd2d_bp_noalloc(const vg_dd2d_geom *g, const float *sino, const double *trig,
                                  float *img, void *stream) {
    int st = check_geom(g);
    if (st) return st;
    VG_REQUIRE(img && trig && sino, "dd2d_bp_noalloc: null pointer");
    const size_t need = bp_ws_bytes(g);
    VG_REQUIRE(need <= VG_NOALLOC_SCRATCH_BYTES,
               "dd2d_bp_noalloc: this geometry needs %zu bytes of workspace, above the fixed "
               "%u-byte scratch; use vg_dd2d_bp with a caller workspace",
               need, (unsigned)VG_NOALLOC_SCRATCH_BYTES);
    void *ws = nullptr;
    st = scratch_address(&ws);
    if (st) return st;
    return launch_bp(g, sino, trig, img, 0, nullptr, 0.f, nullptr, ws, VG_NOALLOC_SCRATCH_BYTES,
                     as_stream(stream));
}

namespace {

using namespace vg;

// ---------------------------------------------------------------------------
// Batched SIRT: many problems in one persistent launch.
//
// The grid (as many blocks of 256 threads as can be resident, launched
// cooperatively so that they all are) runs `iters` SIRT updates of every
// problem.  One update of problem p is three kinds of work items: forward
// projection with the residual epilogue ((p, view, bin chunk)), the back
// projection's tables ((p, view)) and the back projection with the update
// epilogue ((p, pixel tile)).  All items of all updates form one queue,
// update by update and, within an update, forward items, then table items,
// then back-projection items, each kind ordered by the host (largest first);
// blocks take the next item with an atomic counter.  An item waits only for
// the items of its own problem it reads from -- the tables for all of p's
// forward items of this update, the back projection for p's tables, p's next
// forward projection for p's back projection -- counted per problem.  Every
// dependency lies earlier in the queue and is held by a running block, so
// no wait can block forever; waits are still bounded (BATCH_SPIN_LIMIT polls,
// about two seconds), after which the run stops with VG_ERR_TIMEOUT.
//
// The block that takes the first item of an update checks the caller's
// cancel flag (host-mapped memory) and the time budget (nanoseconds of
// %globaltimer since the launch, 0 = none); either stops the run before that
// update (VG_ERR_CANCELLED / VG_ERR_TIMEOUT), and back-projection items of an
// update wait for that check, so a run always ends between updates.  The
// iterates and the measured sinograms may be stored as bfloat16 (arithmetic
// in float32).
// ---------------------------------------------------------------------------

constexpr int BATCH_THREADS = 256;
constexpr long long BATCH_SPIN_LIMIT = 1ll << 25;   // polls of 64 ns sleeps
constexpr int BATCH_UC = 32 * 24 + 32;              // UC entries of the widest tile

struct BatchCtrl {
    unsigned long long next;  // queue head
    int status, done;
    int stop_p;               // 0, or INT_MAX - (the first update not run) once stopped
    int checked;              // updates whose start has been checked
    unsigned exited, pad;
    unsigned long long t0;    // %globaltimer at the first item
};

__device__ __forceinline__ int batch_stop_iter(const BatchCtrl *c, int iters) {
    const int sp = *(const volatile int *)&c->stop_p;
    return sp ? 0x7fffffff - sp : iters;
}
static_assert(sizeof(BatchCtrl) == sizeof(vg_sirt2d_batch_ctrl), "control block layout");

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__host__ __device__ inline int batch_maxb(int nu) { return nu <= 192 ? 6 : (nu <= 384 ? 12 : 24); }
__host__ __device__ inline int batch_nfp(const vg_dd2d_geom &g) {
    const int mb = batch_maxb(g.nu);
    return g.na * ((g.nu + 32 * mb - 1) / (32 * mb));
}
__host__ __device__ inline int batch_nbp(const vg_dd2d_geom &g) {
    return ((g.ny + 2 * BP_TY - 1) / (2 * BP_TY)) * ((g.nx + 2 * BP_TX - 1) / (2 * BP_TX));
}

// thread 0: wait until *cnt >= target (bounded) for an item of update `it`;
// false after a wait that ran out (the run then stops with VG_ERR_TIMEOUT),
// or once the run stops before update `it`
__device__ bool batch_wait(BatchCtrl *c, const int *cnt, long long target, int it, int iters) {
    const volatile int *vcnt = cnt;
    long long n = 0;
    while ((long long)*vcnt < target) {
        const int sp = *(volatile int *)&c->stop_p;
        if (sp == 0 && *(volatile int *)&c->status != 0) return false;  // a wait ran out
        if (it >= batch_stop_iter(c, iters)) return false;
        if (++n > BATCH_SPIN_LIMIT) {
            atomicCAS(&c->status, 0, VG_ERR_TIMEOUT);
            return false;
        }
        __nanosleep(64);
    }
    __threadfence();
    return true;
}

template <bool FAN, int MAXB, typename TX, typename TY>
__device__ __forceinline__ void batch_fp(const vg_sirt2d_problem &p, int view, int chunk, float2 *lines,
                                         float2 *UC) {
    fp_block<FAN, 8, MAXB, false, TX, TY, true>(p.g, view, chunk, static_cast<const TX *>(p.x),
                                          static_cast<const TX *>(p.xT), p.trig, p.r, 1,
                                          static_cast<const TY *>(p.y), p.inv_w_sino,
                                          BpWork{nullptr, nullptr}, lines, UC);
}

// counters: per problem 3 ints (forward, table, back-projection items done)
template <typename TX, typename TY>
__global__ void __launch_bounds__(BATCH_THREADS, 2)
sirt2d_batch_kernel(const vg_sirt2d_problem *__restrict__ P, int nprob,
                    const int2 *__restrict__ fp_items, int n_fp, const int2 *__restrict__ tab_items,
                    int n_tab, const int2 *__restrict__ bp_items, int n_bp, int iters,
                    const volatile int *cancel, unsigned long long budget_ns, BatchCtrl *ctrl,
                    int *counters) {
    extern __shared__ float2 dsm[];
    float2 *UC = dsm, *lines = dsm + BATCH_UC;
    __shared__ long long item_s;
    __shared__ double wsum[BATCH_THREADS / 32];
    const long long total = (long long)n_fp + n_tab + n_bp;
    for (;;) {
        __syncthreads();  // the previous item's shared memory and item_s are no longer read
        if (threadIdx.x == 0) {
            long long k = -1;
            volatile BatchCtrl *vc = ctrl;
            const bool hard = vc->stop_p == 0 && vc->status != 0;  // a wait ran out
            if (!hard) {
                const long long q = (long long)atomicAdd(&ctrl->next, 1ull);
                const int it = (int)(q / total);
                const long long r = q % total;
                if (it < iters && it < batch_stop_iter(ctrl, iters)) {
                    k = q;
                    if (r == 0) {
                        // the start of update `it`: the cancel flag and the time budget
                        if (q == 0) atomicCAS(&ctrl->t0, 0ull, global_ns());
                        int why = 0;
                        const unsigned long long t0 = vc->t0;
                        if (it > 0 && cancel && *cancel) why = VG_ERR_CANCELLED;
                        else if (it > 0 && budget_ns && t0 && global_ns() - t0 > budget_ns)
                            why = VG_ERR_TIMEOUT;
                        if (why) {
                            atomicMax(&ctrl->stop_p, 0x7fffffff - it);
                            atomicCAS(&ctrl->status, 0, why);
                            k = -1;
                        }
                        __threadfence();
                        atomicMax(&ctrl->checked, it + 1);
                    }
                }
            }
            item_s = k;
        }
        __syncthreads();
        const long long k = item_s;
        if (k < 0) break;  // every item of an earlier update is held by a running block
        const int it = (int)(k / total);
        const long long r = k % total;
        int kind, prob, sub;
        if (r < n_fp) { kind = 0; prob = fp_items[r].x; sub = fp_items[r].y; }
        else if (r < n_fp + n_tab) { kind = 1; prob = tab_items[r - n_fp].x; sub = tab_items[r - n_fp].y; }
        else { kind = 2; prob = bp_items[r - n_fp - n_tab].x; sub = bp_items[r - n_fp - n_tab].y; }
        const vg_sirt2d_problem &p = P[prob];
        // the item's inputs: p's back projection of the previous update, p's
        // forward projection or p's tables of this one
        if (threadIdx.x == 0) {
            bool ok;
            if (kind == 0)
                ok = batch_wait(ctrl, counters + 3 * prob + 2, (long long)it * batch_nbp(p.g), it, iters);
            else if (kind == 1)
                ok = batch_wait(ctrl, counters + 3 * prob, (long long)(it + 1) * batch_nfp(p.g), it, iters);
            else
                ok = batch_wait(ctrl, counters + 3 * prob + 1, (long long)(it + 1) * p.g.na, it, iters) &&
                     batch_wait(ctrl, &ctrl->checked, it + 1, it, iters) &&
                     it < batch_stop_iter(ctrl, iters);
            item_s = ok ? k : -1;
        }
        __syncthreads();
        if (item_s < 0) break;
        if (kind == 0) {
            const int mb = batch_maxb(p.g.nu);
            const int nch = (p.g.nu + 32 * mb - 1) / (32 * mb);
            const int view = sub / nch, chunk = sub % nch;
            if (p.g.fan) {
                if (mb == 6) batch_fp<true, 6, TX, TY>(p, view, chunk, lines, UC);
                else if (mb == 12) batch_fp<true, 12, TX, TY>(p, view, chunk, lines, UC);
                else batch_fp<true, 24, TX, TY>(p, view, chunk, lines, UC);
            } else {
                if (mb == 6) batch_fp<false, 6, TX, TY>(p, view, chunk, lines, UC);
                else if (mb == 12) batch_fp<false, 12, TX, TY>(p, view, chunk, lines, UC);
                else batch_fp<false, 24, TX, TY>(p, view, chunk, lines, UC);
            }
        } else if (kind == 1) {
            const BpWork w = bp_ws(&p.g, p.workspace);
            if (p.g.fan) bp_prep_view<true, BATCH_THREADS>(p.g, p.r + (size_t)sub * p.g.nu, sub, p.trig, w, wsum);
            else bp_prep_view<false, BATCH_THREADS>(p.g, p.r + (size_t)sub * p.g.nu, sub, p.trig, w, wsum);
        } else {
            const int nty = (p.g.ny + 2 * BP_TY - 1) / (2 * BP_TY);
            const BpWork w = bp_ws(&p.g, p.workspace);
            if (p.g.fan)
                bp_block<true, TX, true>(p.g, sub % nty, sub / nty, w, p.trig, static_cast<TX *>(p.x), 1,
                                   p.inv_w_img, p.gamma, static_cast<TX *>(p.xT));
            else
                bp_block<false, TX, true>(p.g, sub % nty, sub / nty, w, p.trig, static_cast<TX *>(p.x), 1,
                                    p.inv_w_img, p.gamma, static_cast<TX *>(p.xT));
        }
        __syncthreads();  // the item's writes are done
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(counters + 3 * prob + kind, 1);
        }
    }
    // the last block out records the updates every problem completed
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&ctrl->exited, 1u) == gridDim.x - 1) {
            int done = iters;
            for (int q = 0; q < nprob; ++q) {
                const int d = *(volatile int *)(counters + 3 * q + 2) / batch_nbp(P[q].g);
                done = min(done, d);
            }
            ctrl->done = done;
        }
    }
}

size_t batch_smem(int max_nd) {
    size_t lines = (size_t)8 * fp_line_entries(max_nd) * sizeof(float2);
    const size_t red = (size_t)8 * 32 * 24 * sizeof(float);
    if (lines < red) lines = red;
    return (size_t)BATCH_UC * sizeof(float2) + lines;
}

int batch_check(const vg_sirt2d_problem *p) {
    int st = check_geom(&p->g);
    if (st) return st;
    VG_REQUIRE(p->y && p->inv_w_sino && p->inv_w_img && p->trig && p->x && p->xT && p->r &&
                   p->workspace, "sirt2d_batch: null pointer in a problem");
    VG_REQUIRE(((uintptr_t)p->workspace & 255) == 0, "sirt2d_batch: workspace must be 256-byte aligned");
    const float ext = fmaxf(fabsf(p->g.du * (0.f - 0.5f * p->g.nu + p->g.su)),
                            fabsf(p->g.du * ((float)p->g.nu - 0.5f * p->g.nu + p->g.su)));
    VG_REQUIRE(!p->g.fan || ext < p->g.DSD,
               "sirt2d_batch: a fan detector reaching DSD from its centre is not batched");
    return VG_OK;
}

template <typename TX, typename TY>
int batch_launch(const vg_sirt2d_problem *probs_dev, int nprob, int max_nd, const int *fp, int n_fp,
                 const int *tab, int n_tab, const int *bp, int n_bp, int iters, const int *cancel,
                 unsigned long long budget_ns, void *ctrl, int *counters, cudaStream_t st,
                 int *grid_out) {
    auto kern = sirt2d_batch_kernel<TX, TY>;
    const size_t smem = batch_smem(max_nd);
    VG_REQUIRE(smem <= 200 * 1024, "sirt2d_batch: images above %d pixels a side", max_nd);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "sirt2d_batch: shared memory attribute");
    int dev = 0, nsm = 0, per = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, BATCH_THREADS, smem);
    if (e != cudaSuccess) return cuda_status(e, "sirt2d_batch: occupancy");
    VG_REQUIRE(per > 0, "sirt2d_batch: the kernel does not fit on a multiprocessor");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nsm * per);
    cfg.blockDim = dim3(BATCH_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (grid_out) *grid_out = nsm * per;
    e = cudaLaunchKernelEx(&cfg, kern, probs_dev, nprob, reinterpret_cast<const int2 *>(fp), n_fp,
                           reinterpret_cast<const int2 *>(tab), n_tab,
                           reinterpret_cast<const int2 *>(bp), n_bp, iters,
                           reinterpret_cast<const volatile int *>(cancel), budget_ns,
                           static_cast<BatchCtrl *>(ctrl), counters);
    if (e != cudaSuccess) return cuda_status(e, "sirt2d_batch: launch");
    return launch_status("sirt2d_batch");
}

}  // namespace

extern "C" int vg_sirt2d_batch_items(const vg_sirt2d_problem *probs, int n, int *fp_items,
                                     int *n_fp, int *tab_items, int *n_tab, int *bp_items, int *n_bp) {
    VG_REQUIRE(probs && n > 0 && n_fp && n_tab && n_bp, "sirt2d_batch_items: bad arguments");
    long long cf = 0, ct = 0, cb = 0;
    for (int i = 0; i < n; ++i) {
        int st = batch_check(&probs[i]);
        if (st) return st;
        const vg_dd2d_geom &g = probs[i].g;
        cf += batch_nfp(g);
        ct += g.na;
        cb += batch_nbp(g);
    }
    VG_REQUIRE(cf < (1ll << 30) && cb < (1ll << 30), "sirt2d_batch_items: too many work items");
    if (fp_items && tab_items && bp_items) {
        // items in problem order; the caller may reorder each list freely
        long long a = 0, b = 0, c = 0;
        for (int i = 0; i < n; ++i) {
            const vg_dd2d_geom &g = probs[i].g;
            const int nf = batch_nfp(g), nt = batch_nbp(g);
            for (int k = 0; k < nf; ++k, ++a) { fp_items[2 * a] = i; fp_items[2 * a + 1] = k; }
            for (int k = 0; k < g.na; ++k, ++b) { tab_items[2 * b] = i; tab_items[2 * b + 1] = k; }
            for (int k = 0; k < nt; ++k, ++c) { bp_items[2 * c] = i; bp_items[2 * c + 1] = k; }
        }
    }
    *n_fp = (int)cf;
    *n_tab = (int)ct;
    *n_bp = (int)cb;
    return VG_OK;
}

extern "C" int vg_sirt2d_batch_run(const vg_sirt2d_problem *probs_dev, int n, int max_nd,
                                   const int *fp_items, int n_fp, const int *tab_items, int n_tab,
                                   const int *bp_items, int n_bp, int iters, int storage,
                                   const int *cancel, unsigned long long budget_ns,
                                   vg_sirt2d_batch_ctrl *ctrl, int *counters, void *stream,
                                   int *grid_blocks) {
    VG_REQUIRE(probs_dev && n > 0 && fp_items && tab_items && bp_items && ctrl && counters,
               "sirt2d_batch_run: null pointer");
    VG_REQUIRE((long long)(n_fp + (long long)n_tab + n_bp) * iters < (1ll << 62),
               "sirt2d_batch_run: too many items");
    VG_REQUIRE(n_fp > 0 && n_tab > 0 && n_bp > 0 && iters >= 0 && max_nd > 0,
               "sirt2d_batch_run: bad counts");
    VG_REQUIRE(storage >= 0 && storage <= 3, "sirt2d_batch_run: storage %d not in 0..3", storage);
    cudaStream_t st = as_stream(stream);
    if (cancel) {
        // pinned host memory: its device address (the same pointer under unified addressing)
        void *dp = nullptr;
        if (cudaHostGetDevicePointer(&dp, const_cast<int *>(cancel), 0) == cudaSuccess && dp)
            cancel = static_cast<const int *>(dp);
        else
            cudaGetLastError();  // not registered host memory: used as given
    }
    cudaError_t e = cudaMemsetAsync(ctrl, 0, sizeof(vg_sirt2d_batch_ctrl), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, (size_t)3 * n * sizeof(int), st);
    if (e != cudaSuccess) return cuda_status(e, "sirt2d_batch_run: control block");
    const bool bx = storage & 1, by = storage & 2;
    if (!bx && !by)
        return batch_launch<float, float>(probs_dev, n, max_nd, fp_items, n_fp, tab_items, n_tab,
                                          bp_items, n_bp, iters, cancel, budget_ns, ctrl, counters, st,
                                          grid_blocks);
    if (bx && !by)
        return batch_launch<__nv_bfloat16, float>(probs_dev, n, max_nd, fp_items, n_fp, tab_items,
                                                  n_tab, bp_items, n_bp, iters, cancel, budget_ns, ctrl,
                                                  counters, st, grid_blocks);
    if (!bx && by)
        return batch_launch<float, __nv_bfloat16>(probs_dev, n, max_nd, fp_items, n_fp, tab_items,
                                                  n_tab, bp_items, n_bp, iters, cancel, budget_ns, ctrl,
                                                  counters, st, grid_blocks);
    return batch_launch<__nv_bfloat16, __nv_bfloat16>(probs_dev, n, max_nd, fp_items, n_fp,
                                                      tab_items, n_tab, bp_items, n_bp, iters, cancel,
                                                      budget_ns, ctrl, counters, st, grid_blocks);
}
