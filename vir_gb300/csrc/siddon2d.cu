// 2D parallel-beam Siddon forward projector and its exact gather-form
// adjoint.
//
// Geometry follows sys_mat/fp_2d_par.py:11-64 operation for operation, in
// FP64 with every multiply/add/divide separately rounded (no contraction), so
// the sorted plane-crossing sequence, the segment midpoints and therefore the
// voxel index sequence of every ray are the ones vir's FP64 code produces:
//   edges      X_b[i] = d_pix * (i - nx/2.0)                       (:16-17)
//   detector   det_k  = d_det * ((k - n_dets/2.0) + 0.5)           (:20)
//   origin     (x0, y0) = det_k * (-dy, dx), (dx, dy) = (cos, sin) (:23,29-30)
//   entry/exit t0 = max(min tx, min ty), t1 = min(max tx, max ty)  (:33-43)
//   crossings  all t = (X_b[i] - x0)/dx, (Y_b[j] - y0)/dy in [t0, t1], sorted
//   segments   consecutive pairs a < b, voxel floor((x0 + (0.5(a+b))dx - X_b[0])/d_pix)
// The x- and y-crossing sequences are each monotone in their index, so the
// sort is a two-way merge.  Intersection lengths (b - a) are rounded to FP32
// and the ray sum is Kahan-compensated FP32.
#include "vg_common.cuh"

namespace {

using namespace vg;

struct SidGeom {
    int nx, ny, n_dets;
    double d_det, d_pix, inv_dpix;
    double xb0, xbn, yb0, ybn;
    int dpix_pow2;  // d_pix is a power of two: x / d_pix == x * (1/d_pix) exactly
};

__device__ __forceinline__ double edge(double d_pix, int i, int n) {
    return d_mul(d_pix, (double)i - (double)n * 0.5);
}

__device__ __forceinline__ double div_pix(const SidGeom &g, double v) {
    return g.dpix_pow2 ? d_mul(v, g.inv_dpix) : d_div(v, g.d_pix);
}

// a / b rounded to nearest, given y = RN(1 / b): q0 = RN(a y) is within an
// ulp of a / b, r = a - b q0 is exact (one FMA), and RN(q0 + r y) is the
// correctly rounded quotient (Markstein's theorem; Muller et al., Handbook of
// Floating-Point Arithmetic, division with a fused multiply-add).  Three FP64
// operations per quotient once y is known; finite, normal operands only.
#ifndef VG_SID_RCP
#define VG_SID_RCP 1
#endif
__device__ __forceinline__ double div_by(double a, double b, double y) {
#if VG_SID_RCP
    const double q0 = __dmul_rn(a, y);
    const double r = __fma_rn(-b, q0, a);
    return __fma_rn(r, y, q0);
#else
    return d_div(a, b);
#endif
}

__device__ __forceinline__ double rcp_of(double b) {
#if VG_SID_RCP
    return b != 0.0 ? __drcp_rn(b) : 0.0;
#else
    return 0.0;
#endif
}

struct Ray {
    double x0, y0, t0, t1;
    double rdx, rdy;  // RN(1 / dx), RN(1 / dy)
    bool valid;
};

__device__ __forceinline__ Ray ray_setup(const SidGeom &g, int k, double dx, double dy) {
    Ray r;
    double det = d_mul(g.d_det, d_add((double)k - (double)g.n_dets * 0.5, 0.5));
    r.x0 = d_mul(det, -dy);
    r.y0 = d_mul(det, dx);
    r.rdx = rcp_of(dx);
    r.rdy = rcp_of(dy);
    double tx0 = -INFINITY, txn = INFINITY, ty0 = -INFINITY, tyn = INFINITY;
    if (dx != 0.0) { tx0 = div_by(d_sub(g.xb0, r.x0), dx, r.rdx); txn = div_by(d_sub(g.xbn, r.x0), dx, r.rdx); }
    if (dy != 0.0) { ty0 = div_by(d_sub(g.yb0, r.y0), dy, r.rdy); tyn = div_by(d_sub(g.ybn, r.y0), dy, r.rdy); }
    r.t0 = fmax(fmin(tx0, txn), fmin(ty0, tyn));
    r.t1 = fmin(fmax(tx0, txn), fmax(ty0, tyn));
    r.valid = !(r.t1 <= r.t0 || isinf(r.t0) || isinf(r.t1));
    return r;
}

// Crossing parameter of the j-th plane in traversal order (t non-decreasing
// in j): index i = j when the direction component is positive, n - j else.
// The plane position is edge(d_pix, i, n), read from `et` (a table of the
// same values) when given.
__device__ __forceinline__ double cross_t(double d_pix, int n, int j, bool pos, double o, double d,
                                          double rd, const double *et = nullptr) {
    int i = pos ? j : n - j;
    const double e = et ? et[i] : edge(d_pix, i, n);
    return div_by(d_sub(e, o), d, rd);
}

// The crossings' comparisons run on integers: ord64 maps doubles (no NaN)
// to int64 in the same order, -0 and +0 alike, so x <= y <=> ord64(x) <=
// ord64(y) (FP64 compares use the slow FP64 pipe, integer compares do not).
__device__ __forceinline__ long long ord64(double x) {
    long long b = __double_as_longlong(x);
    if (b == (long long)0x8000000000000000ULL) b = 0;
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

// First traversal index whose crossing is >= t0 (n + 1 when none).
__device__ int first_crossing(double d_pix, int n, bool pos, double o, double d, double rd,
                              double t0, double b0, const double *et = nullptr) {
    double p = d_add(o, d_mul(t0, d));
    double fi = floor((p - b0) / d_pix);
    int j = (int)fmin(fmax(pos ? fi : (double)n - fi, 0.0), (double)(n + 1));
    // settle on the exact boundary (a handful of steps at most)
    for (int it = 0; it < 4 && j > 0 && cross_t(d_pix, n, j - 1, pos, o, d, rd, et) >= t0; ++it) --j;
    while (j > 0 && cross_t(d_pix, n, j - 1, pos, o, d, rd, et) >= t0) --j;
    while (j <= n && cross_t(d_pix, n, j, pos, o, d, rd, et) < t0) ++j;
    return j;
}

// Last traversal index whose crossing is <= t1 (-1 when none).
__device__ int last_crossing(double d_pix, int n, bool pos, double o, double d, double rd,
                             double t1, double b0, const double *et) {
    double p = d_add(o, d_mul(t1, d));
    double fi = floor((p - b0) / d_pix);
    int j = (int)fmin(fmax(pos ? fi : (double)n - fi, -1.0), (double)n);
    while (j >= 0 && cross_t(d_pix, n, j, pos, o, d, rd, et) > t1) --j;
    while (j < n && cross_t(d_pix, n, j + 1, pos, o, d, rd, et) <= t1) ++j;
    return j;
}

// TRACE: instead of the line integral, record per ray the number of
// segments, an order-sensitive hash of their voxel indices and the FP64 sum
// of their lengths (used to check voxel sequences against the oracle).
struct Trace {
    int *count;
    unsigned long long *hash;
    double *len;
};

__device__ __forceinline__ unsigned long long trace_mix(unsigned long long h, unsigned long long v) {
    return (h ^ (v + 0x9E3779B97F4A7C15ull)) * 0x100000001B3ull;
}

// Scatter form of the back projection: each ray of views [ia0, ia0 + nvc)
// writes y * length into a per-(view, pixel) slot reserved for it,
// slot = ray mod S, where S exceeds the number of rays that can cross one
// pixel in one view; a gather pass then sums the slots.
struct Slots {
    const float *y;  // sinogram (na, n_dets)
    float *buf;      // [nvc][nx * ny][S], zeroed
    int S, ia0;
};

// MODE 0: line integrals; 1: trace (count, hash, length); 2: slot scatter.
// P threads (consecutive lanes) share a ray: thread `part` walks the segments
// that start in [tau_part, tau_part+1), the ray's [t0, t1] cut in P equal
// pieces (tau_0 = t0, tau_P = +inf).  Each starts from its first crossings at
// or after tau_part, as the single walk starts from those at or after t0, so
// the parts together visit the single walk's segments, each once.  MODE 0
// adds the parts' sums in part order; the trace needs one walk (P = 1).
#ifndef VG_SID_TAB
#define VG_SID_TAB 1
#endif
#ifndef VG_SID_TAB_MAX
#define VG_SID_TAB_MAX 2048  // plane positions held in shared memory (16 KB)
#endif
#ifndef VG_SID_TRAV
#define VG_SID_TRAV 1
#endif
#ifndef VG_SID_PARTS
#define VG_SID_PARTS 8
#endif
template <int MODE, int P>
__global__ void
siddon2d_fp_kernel(SidGeom g, const float *__restrict__ img, const double *__restrict__ trig,
                   int na, float *__restrict__ sino, Trace tr, Slots sl) {
    static_assert(P == 1 || (MODE != 1 && 32 % P == 0), "parts split rays in MODE 0 and 2");
    constexpr bool TRACE = MODE == 1;
    // the plane positions of both axes, once per block (the same FP64 values
    // edge() computes), when they fit
    __shared__ double etab[VG_SID_TAB_MAX];
    const bool tab = VG_SID_TAB && g.nx + g.ny + 2 <= VG_SID_TAB_MAX;
    if (tab) {
        for (int i = threadIdx.x; i <= g.nx; i += blockDim.x) etab[i] = edge(g.d_pix, i, g.nx);
        for (int i = threadIdx.x; i <= g.ny; i += blockDim.x) etab[g.nx + 1 + i] = edge(g.d_pix, i, g.ny);
    }
    __syncthreads();
    const double *etx = tab ? etab : nullptr, *ety = tab ? etab + g.nx + 1 : nullptr;
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = gid / P, part = gid % P;
    int ia = blockIdx.y + sl.ia0;
    if (k >= g.n_dets || ia >= na) return;  // whole groups of P lanes
    const float yv = MODE == 2 ? __ldg(sl.y + (size_t)ia * g.n_dets + k) : 0.f;
    float *slot = MODE == 2 ? sl.buf + (size_t)blockIdx.y * g.nx * g.ny * sl.S + k % sl.S : nullptr;
    double dx = trig[2 * ia], dy = trig[2 * ia + 1];
    Ray r = ray_setup(g, k, dx, dy);
    Kahan acc;
    int tcount = 0;
    unsigned long long thash = 0xCBF29CE484222325ull;
    double tlen = 0.0;
    if (r.valid) {
        const double INF = INFINITY;
        // this part's range [tbeg, tend) of segment starts
        const double span = d_sub(r.t1, r.t0);
        const double tbeg = part == 0 ? r.t0 : d_add(r.t0, d_mul(span, (double)part / P));
        const double tend = part == P - 1 ? INF : d_add(r.t0, d_mul(span, (double)(part + 1) / P));
        bool px = dx > 0.0, py = dy > 0.0;
        // crossings jx..jx_end of the x planes (and y) lie in [tbeg, t1]
        int jx = 0, jy = 0, jx_end = -1, jy_end = -1;
        double tx = 0.0, ty = 0.0;
        long long ox = 0, oy = 0;  // ord64 of tx, ty
        if (dx != 0.0) {
            jx = first_crossing(g.d_pix, g.nx, px, r.x0, dx, r.rdx, tbeg, g.xb0, etx);
            jx_end = last_crossing(g.d_pix, g.nx, px, r.x0, dx, r.rdx, r.t1, g.xb0, etx);
            if (jx <= jx_end) {
                tx = cross_t(g.d_pix, g.nx, jx, px, r.x0, dx, r.rdx, etx);
                ox = ord64(tx);
            }
        }
        if (dy != 0.0) {
            jy = first_crossing(g.d_pix, g.ny, py, r.y0, dy, r.rdy, tbeg, g.yb0, ety);
            jy_end = last_crossing(g.d_pix, g.ny, py, r.y0, dy, r.rdy, r.t1, g.yb0, ety);
            if (jy <= jy_end) {
                ty = cross_t(g.d_pix, g.ny, jy, py, r.y0, dy, r.rdy, ety);
                oy = ord64(ty);
            }
        }
        bool xa = jx <= jx_end, ya = jy <= jy_end;  // axes with crossings left
        bool have_prev = false;
        double tprev = 0.0;
        long long oprev = 0;
        const long long oend = ord64(tend);
        // A segment's voxel is vir's floor of its midpoint.  The midpoint lies at
        // least h |d| / 2 (h = tn - tprev) from the cell's boundaries along each
        // axis (less the crossings' own rounding), and its computed coordinates
        // are within a few FP64 ulps of L = the ray's largest coordinate or
        // parameter magnitude, so when h |dx| and h |dy| both exceed 1e-9 L the
        // floors are the cell the walk is in: the walk's cell (cx, cy), set from
        // the floors of the first such segment and stepped at every crossing,
        // is used; shorter segments (and rays nearly along an axis) take the
        // floors.
        const double L = 1.0 + fabs(r.t0) + fabs(r.t1) + fabs(r.x0) + fabs(r.y0) + fabs(g.xb0) +
                         fabs(g.yb0);
        const double thr = VG_SID_TRAV ? 1e-9 * L * fmax(fabs(r.rdx), fabs(r.rdy)) : INF;
        int cx = 0, cy = 0;
        bool walk_cell = false;
        const int sx = px ? 1 : -1, sy = py ? 1 : -1;
        // bounded: every step consumes one of nx + ny + 2 crossings
        for (int step = 0; step < g.nx + g.ny + 4; ++step) {
            if (!xa && !ya) break;
            // the earlier crossing; ties take the x plane first
            const bool xcross = xa && (!ya || ox <= oy);
            double tn;
            long long on;
            if (xcross) {
                tn = tx;
                on = ox;
                ++jx;
                xa = jx <= jx_end;
                if (xa) {
                    tx = cross_t(g.d_pix, g.nx, jx, px, r.x0, dx, r.rdx, etx);
                    ox = ord64(tx);
                }
            } else {
                tn = ty;
                on = oy;
                ++jy;
                ya = jy <= jy_end;
                if (ya) {
                    ty = cross_t(g.d_pix, g.ny, jy, py, r.y0, dy, r.rdy, ety);
                    oy = ord64(ty);
                }
            }
            if (have_prev && on > oprev) {
                const double h = d_sub(tn, tprev);
                int ix, iy;
                if (walk_cell && h > thr) {
                    ix = cx;
                    iy = cy;
                } else {
                    double m = d_mul(0.5, d_add(tprev, tn));
                    double fx = floor(div_pix(g, d_sub(d_add(r.x0, d_mul(m, dx)), g.xb0)));
                    double fy = floor(div_pix(g, d_sub(d_add(r.y0, d_mul(m, dy)), g.yb0)));
                    // outside the grid by more than the int range: no voxel
                    ix = fx >= 0.0 && fx < g.nx ? (int)fx : -1;
                    iy = fy >= 0.0 && fy < g.ny ? (int)fy : -1;
                    if (!walk_cell && h > thr) {
                        walk_cell = true;
                        cx = (int)fmax(fmin(fx, 1e9), -1e9);
                        cy = (int)fmax(fmin(fy, 1e9), -1e9);
                    }
                }
                if (ix >= 0 && ix < g.nx && iy >= 0 && iy < g.ny) {
                    size_t pix = (size_t)ix * g.ny + iy;
                    if (TRACE) {
                        ++tcount;
                        thash = trace_mix(thash, pix);
                        tlen = d_add(tlen, h);
                    } else if (MODE == 2) {
                        slot[pix * sl.S] += __fmul_rn(yv, (float)h);
                    } else {
                        float w = (float)h;
                        acc.add(__fmul_rn(__ldg(img + pix), w));
                    }
                }
            }
            // the crossing moves the walk into the next cell along its axis
            if (walk_cell) {
                if (xcross) cx += sx;
                else cy += sy;
            }
            tprev = tn;
            oprev = on;
            have_prev = true;
            if (P > 1 && oprev >= oend) break;  // the next segment starts in the next part
        }
    }
    if (MODE == 0 && P > 1) {
        // the parts' sums, added in part order by the group's first lane
        const unsigned mask = ((1u << P) - 1u) << ((threadIdx.x & 31) & ~(P - 1));
        float ps[P], pc[P];
#pragma unroll
        for (int q = 0; q < P; ++q) {
            ps[q] = __shfl_sync(mask, acc.s, q, P);
            pc[q] = __shfl_sync(mask, acc.c, q, P);
        }
        if (part != 0) return;
        Kahan tot;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            tot.add(ps[q]);
            tot.add(-pc[q]);
        }
        acc = tot;
    }
    size_t o = (size_t)ia * g.n_dets + k;
    if (TRACE) {
        tr.count[o] = tcount;
        tr.hash[o] = thash;
        tr.len[o] = tlen;
    } else if (MODE == 0) {
        sino[o] = acc.s;
    }
}

// Gather of the slot buffer: pixel sums over the chunk's views and slots in
// a fixed order, added to img (first chunk: written).
__global__ void __launch_bounds__(256)
siddon2d_slot_gather(const float *__restrict__ buf, int npix, int S, int nvc, int first,
                     float *__restrict__ img) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    Kahan acc;
    for (int v = 0; v < nvc; ++v) {
        const float *b = buf + ((size_t)v * npix + p) * S;
        float part = 0.f;
        for (int s = 0; s < S; ++s) part += __ldg(b + s);
        acc.add(part);
    }
    img[p] = first ? acc.s : img[p] + acc.s;
}

// Gather-form adjoint.  For pixel (ix, iy) and view ia, the candidate rays
// are the bins whose centre lies within the pixel's projected extent (plus a
// margin).  For each candidate the crossings of the planes around the pixel
// (x planes ix-1..ix+2, y planes iy-1..iy+2) are recomputed with the forward
// projector's arithmetic and filtered to [t0, t1]; every consecutive pair whose
// midpoint voxel (by the forward projector's rule) is (ix, iy) is a segment
// the forward projector assigns to this pixel, with the same FP64 length.
// A segment whose midpoint lies in (ix, iy) has both ends on planes bounding
// this pixel's neighbourhood, so this enumerates exactly the forward
// segments: the pair is an exact transpose, degenerate rays included.
__device__ __forceinline__ int window_crossings(double d_pix, int n, int i_lo, double o, double d,
                                                double rd, double t0, double t1, double *out) {
    int c = 0;
    if (d == 0.0) return 0;
    for (int q = 0; q < 4; ++q) {
        int i = i_lo + q;
        if (i < 0 || i > n) continue;
        double t = div_by(d_sub(edge(d_pix, i, n), o), d, rd);
        if (t0 <= t && t <= t1) out[c++] = t;
    }
    // ascending order (the sequence is monotone in i; reverse when d < 0)
    if (d < 0.0)
        for (int a = 0, b = c - 1; a < b; ++a, --b) { double t = out[a]; out[a] = out[b]; out[b] = t; }
    return c;
}

__global__ void __launch_bounds__(256)
siddon2d_bp_kernel(SidGeom g, const float *__restrict__ sino, const double *__restrict__ trig,
                   int na, float *__restrict__ img) {
    int iy = blockIdx.x * blockDim.x + threadIdx.x;
    int ix = blockIdx.y;
    if (iy >= g.ny || ix >= g.nx) return;
    // pixel centre in FP32 for candidate selection only
    float xc = (float)(g.d_pix * ((double)ix + 0.5 - g.nx * 0.5));
    float yc = (float)(g.d_pix * ((double)iy + 0.5 - g.ny * 0.5));
    float half = 0.5f * (float)g.d_pix;
    float inv_det = (float)(1.0 / g.d_det);
    float koff = 0.5f * g.n_dets - 0.5f;
    Kahan acc;
    for (int ia = 0; ia < na; ++ia) {
        double dx = __ldg(trig + 2 * ia), dy = __ldg(trig + 2 * ia + 1);
        float fdx = (float)dx, fdy = (float)dy;
        float uc = -fdy * xc + fdx * yc;
        float hw = half * (fabsf(fdx) + fabsf(fdy)) + 1e-3f * (float)g.d_det + 1e-5f * fabsf(uc);
        int k_lo = max(0, (int)ceilf((uc - hw) * inv_det + koff));
        int k_hi = min(g.n_dets - 1, (int)floorf((uc + hw) * inv_det + koff));
        for (int k = k_lo; k <= k_hi; ++k) {
            Ray r = ray_setup(g, k, dx, dy);
            if (!r.valid) continue;
            double tx[4], ty[4], t[8];
            int nx_ = window_crossings(g.d_pix, g.nx, ix - 1, r.x0, dx, r.rdx, r.t0, r.t1, tx);
            int ny_ = window_crossings(g.d_pix, g.ny, iy - 1, r.y0, dy, r.rdy, r.t0, r.t1, ty);
            // merge the two ascending lists
            int a = 0, b = 0, n = 0;
            while (a < nx_ || b < ny_) {
                if (b >= ny_ || (a < nx_ && tx[a] <= ty[b])) t[n++] = tx[a++];
                else t[n++] = ty[b++];
            }
            float yv = __ldg(sino + (size_t)ia * g.n_dets + k);
            for (int s = 0; s + 1 < n; ++s) {
                double ta = t[s], tb = t[s + 1];
                if (!(tb > ta)) continue;
                double m = d_mul(0.5, d_add(ta, tb));
                double fx = floor(div_pix(g, d_sub(d_add(r.x0, d_mul(m, dx)), g.xb0)));
                if (fx != (double)ix) continue;
                double fy = floor(div_pix(g, d_sub(d_add(r.y0, d_mul(m, dy)), g.yb0)));
                if (fy != (double)iy) continue;
                acc.add(__fmul_rn(yv, (float)d_sub(tb, ta)));
            }
        }
    }
    img[(size_t)ix * g.ny + iy] = acc.s;
}

int make_geom(SidGeom &g, int nx, int ny, int n_dets, double d_det, double d_pix) {
    VG_REQUIRE(nx > 0 && ny > 0 && n_dets > 0, "siddon2d: sizes must be positive");
    VG_REQUIRE(d_det > 0 && d_pix > 0, "siddon2d: d_det and d_pix must be positive");
    g.nx = nx; g.ny = ny; g.n_dets = n_dets;
    g.d_det = d_det; g.d_pix = d_pix;
    g.inv_dpix = 1.0 / d_pix;
    int e;
    g.dpix_pow2 = frexp(d_pix, &e) == 0.5;
    g.xb0 = d_pix * (0.0 - nx * 0.5);
    g.xbn = d_pix * ((double)nx - nx * 0.5);
    g.yb0 = d_pix * (0.0 - ny * 0.5);
    g.ybn = d_pix * ((double)ny - ny * 0.5);
    return VG_OK;
}

}  // namespace

extern "C" int vg_siddon2d_fp(const float *img, int nx, int ny, const double *trig, int na,
                              int n_dets, double d_det, double d_pix, float *sino, void *stream) {
    SidGeom g;
    int st = make_geom(g, nx, ny, n_dets, d_det, d_pix);
    if (st) return st;
    VG_REQUIRE(na > 0 && na < 65536, "siddon2d_fp: na out of range");
    VG_REQUIRE(img && trig && sino, "siddon2d_fp: null pointer");
    dim3 grid(ceil_div((long long)n_dets * VG_SID_PARTS, 128), na);
    siddon2d_fp_kernel<0, VG_SID_PARTS><<<grid, 128, 0, as_stream(stream)>>>(g, img, trig, na, sino, Trace{},
                                                              Slots{nullptr, nullptr, 1, 0});
    return launch_status("siddon2d_fp");
}

namespace {
__global__ void div_rn_check_kernel(const double *__restrict__ a, const double *__restrict__ b,
                                    size_t n, double *__restrict__ q) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const double bb = b[i];
        q[i] = div_by(a[i], bb, rcp_of(bb));
    }
}
}  // namespace

extern "C" int vg_div_rn_check(const double *a, const double *b, size_t n, double *q, void *stream) {
    VG_REQUIRE(a && b && q, "div_rn_check: null pointer");
    if (n == 0) return VG_OK;
    const int blocks = (int)((n + 255) / 256 < 152 * 32 ? (n + 255) / 256 : 152 * 32);
    div_rn_check_kernel<<<blocks, 256, 0, as_stream(stream)>>>(a, b, n, q);
    return launch_status("div_rn_check");
}

extern "C" int vg_siddon2d_trace(int nx, int ny, const double *trig, int na, int n_dets,
                                 double d_det, double d_pix, int *count,
                                 unsigned long long *hash, double *len, void *stream) {
    SidGeom g;
    int st = make_geom(g, nx, ny, n_dets, d_det, d_pix);
    if (st) return st;
    VG_REQUIRE(na > 0 && na < 65536, "siddon2d_trace: na out of range");
    VG_REQUIRE(trig && count && hash && len, "siddon2d_trace: null pointer");
    dim3 grid(ceil_div(n_dets, 128), na);
    siddon2d_fp_kernel<1, 1><<<grid, 128, 0, as_stream(stream)>>>(g, nullptr, trig, na, nullptr,
                                                              Trace{count, hash, len},
                                                              Slots{nullptr, nullptr, 1, 0});
    return launch_status("siddon2d_trace");
}

extern "C" int vg_siddon2d_bp(const float *sino, int na, int n_dets, const double *trig, int nx,
                              int ny, double d_det, double d_pix, float *img, void *stream) {
    SidGeom g;
    int st = make_geom(g, nx, ny, n_dets, d_det, d_pix);
    if (st) return st;
    VG_REQUIRE(na > 0, "siddon2d_bp: na must be positive");
    VG_REQUIRE(nx < 65536, "siddon2d_bp: nx out of range");
    VG_REQUIRE(img && trig && sino, "siddon2d_bp: null pointer");
    dim3 grid(ceil_div(ny, 256), nx);
    siddon2d_bp_kernel<<<grid, 256, 0, as_stream(stream)>>>(g, sino, trig, na, img);
    return launch_status("siddon2d_bp");
}

// Slots per (view, pixel): more than the rays one pixel can meet in a view
// (its projected width d_pix (|cos| + |sin|) <= d_pix sqrt 2 spans at most
// floor(d_pix sqrt 2 / d_det) + 1 bin centres).
static int siddon_slots(double d_pix, double d_det) {
    return (int)floor(d_pix * 1.4142135623730951 / d_det) + 2;
}

extern "C" size_t vg_siddon2d_bp_workspace_bytes(int nx, int ny, int na, double d_det,
                                                 double d_pix) {
    if (nx <= 0 || ny <= 0 || na <= 0 || !(d_det > 0) || !(d_pix > 0)) return 0;
    const size_t per_view = (size_t)nx * ny * siddon_slots(d_pix, d_det) * sizeof(float);
    size_t views = ((size_t)256 << 20) / per_view;
    if (views < 1) views = 1;
    if (views > (size_t)na) views = na;
    return views * per_view;
}

extern "C" int vg_siddon2d_bp_scatter(const float *sino, int na, int n_dets, const double *trig,
                                      int nx, int ny, double d_det, double d_pix, float *img,
                                      void *workspace, size_t workspace_bytes, void *stream) {
    SidGeom g;
    int st = make_geom(g, nx, ny, n_dets, d_det, d_pix);
    if (st) return st;
    VG_REQUIRE(na > 0 && na < 65536, "siddon2d_bp_scatter: na out of range");
    VG_REQUIRE((long long)nx * ny < (1LL << 31), "siddon2d_bp_scatter: image too large");
    VG_REQUIRE(img && trig && sino && workspace, "siddon2d_bp_scatter: null pointer");
    const int S = siddon_slots(d_pix, d_det);
    const size_t per_view = (size_t)nx * ny * S * sizeof(float);
    VG_REQUIRE(workspace_bytes >= per_view,
               "siddon2d_bp_scatter: workspace of at least %zu bytes needed", per_view);
    VG_REQUIRE(((uintptr_t)workspace & 3) == 0, "siddon2d_bp_scatter: workspace misaligned");
    const int nvc = (int)(workspace_bytes / per_view < (size_t)na ? workspace_bytes / per_view : na);
    cudaStream_t s = as_stream(stream);
    float *buf = static_cast<float *>(workspace);
    const int npix = nx * ny;
    for (int ia0 = 0; ia0 < na; ia0 += nvc) {
        const int nv = na - ia0 < nvc ? na - ia0 : nvc;
        cudaError_t e = cudaMemsetAsync(buf, 0, (size_t)nv * per_view, s);
        if (e != cudaSuccess) return cuda_status(e, "siddon2d_bp_scatter: clear");
        dim3 grid(ceil_div((long long)n_dets * VG_SID_PARTS, 128), nv);
        siddon2d_fp_kernel<2, VG_SID_PARTS><<<grid, 128, 0, s>>>(g, nullptr, trig, na, nullptr, Trace{},
                                                     Slots{sino, buf, S, ia0});
        st = launch_status("siddon2d_bp_scatter");
        if (st) return st;
        siddon2d_slot_gather<<<ceil_div(npix, 256), 256, 0, s>>>(buf, npix, S, nv, ia0 == 0, img);
        st = launch_status("siddon2d_slot_gather");
        if (st) return st;
    }
    return VG_OK;
}
