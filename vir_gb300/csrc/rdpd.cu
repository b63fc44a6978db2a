// Ray-driven (Amanatides-Woo walk, Joseph sampling; sys_mat/rd.py) and
// pixel-driven footprint (sys_mat/pd.py) projector pairs for the parallel
// and fan 2D and circular cone 3D geometries.
//
// Ray-driven: one thread per ray in float32 with the reference's
// formulas.  Parallel rays start at u (-sin, cos) with direction
// (cos, sin) (rd.py:490-499); fan/cone rays run from the source
// DSO (cos, sin, 0) to the detector point -(DSD - DSO)(cos, sin) +
// u (-sin, cos) + v z (rd.py:584-603, 701-730); u = du (iu - (nu/2 - 0.5) +
// su), v the same with nv.  The forward projection gathers along the ray.
// The 2D Amanatides-Woo back projection is a gather over the rays crossing
// each pixel (aw_bp2d_gather, deterministic); the Joseph and cone back
// projections follow vir's own scatter (rd.py:152-176, 357-447) with float
// atomics, so their summation order is not fixed.  Two defects of the
// reference are not reproduced: a ray parallel to an axis is clipped to
// the slab it lies in (the reference's _intersect_bounding never clips
// it, rd.py:52-64, so rays beside the image walk its edge row), and the
// cone's detector rows use nv (rd.py:688 uses nu).  Every walk is bounded
// by an iteration count derived from the volume size.
//
// Pixel-driven: the back projection is a gather, one thread per pixel (2D)
// or one warp per voxel column (cone) over all views; the forward projection
// scatters each pixel's footprint into the 1-4 overlapped bins with float
// atomics, as the reference's loop does (pd.py:56-127), one thread per run of
// pixels along y (2D) or one warp per voxel column and view (cone).  The fan scale 1 / (|cos(a + g)| +
// |sin(a + g)|) with g = atan(u_c / DSD) is evaluated through
// cos(a + g) = (c - s t) / sqrt(1 + t^2), sin(a + g) = (s + c t) /
// sqrt(1 + t^2), t = u_c / DSD, and the cone's 1 / cos(g) as sqrt(1 + t^2).
#include <math.h>

#include "vg_common.cuh"

namespace {

using namespace vg;

constexpr float RD_EPS = 1e-6f;  // rd.py:42

#ifndef VG_JOSEPH_AFFINE
#define VG_JOSEPH_AFFINE 1
#endif

#ifndef VG_PD_CONE_COLUMNS
#define VG_PD_CONE_COLUMNS 1
#endif

struct Ray {
    float o[3], h[3];
};

__device__ __forceinline__ void bounds1(int n, float d, float &lo, float &hi, float &c0) {
    lo = -d * (float)n / 2.f;
    hi = d * (float)n / 2.f;
    c0 = -d * ((float)n / 2.f - 0.5f);
}

// _intersect_bounding with the axis-parallel ray clipped to its slab
__device__ __forceinline__ void slab(float r0, float dr, float lo, float hi, float &t0, float &t1) {
    if (fabsf(dr) > RD_EPS) {
        const float a = (lo - r0) / dr, b = (hi - r0) / dr;
        t0 = fminf(a, b);
        t1 = fmaxf(a, b);
    } else if (r0 >= lo && r0 < hi) {
        t0 = -INFINITY;
        t1 = INFINITY;
    } else {
        t0 = INFINITY;
        t1 = -INFINITY;
    }
}

// Adds corner c of cell cur (its sum slot[c]) into the image when it is
// inside the image and nonzero.
template <int DIM>
__device__ __forceinline__ void flush(int c, const int *cur, float *__restrict__ bimg, const int *n,
                                      size_t sx, size_t sy, const float *slot) {
    if (slot[c] == 0.f) return;
    bool ok = true;
    size_t off = 0;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
        const int i = cur[a] + ((c >> a) & 1);
        ok = ok && i >= 0 && i < n[a];
        off += (size_t)i * (a == 0 ? sx : (a == 1 ? sy : 1));
    }
    if (ok) atomicAdd(bimg + off, slot[c]);
}

// One ray: returns the line integral (BP = false) or adds s times the
// ray's weights into bimg (BP = true).  DIM 2 or 3; img is x-major with
// z fastest.
template <int DIM, bool JOSEPH, bool BP>
__device__ float trace(const Ray &R, const float *__restrict__ img, float *__restrict__ bimg,
                       float s, const int *n, float d) {
    float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f}, c0[3] = {0.f, 0.f, 0.f};
    float te = -INFINITY, tx = INFINITY;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
        float t0, t1;
        bounds1(n[a], d, lo[a], hi[a], c0[a]);
        slab(R.o[a], R.h[a], lo[a], hi[a], t0, t1);
        te = fmaxf(te, t0);
        tx = fminf(tx, t1);
    }
    if (!(tx > te)) return 0.f;
    const size_t sy = DIM == 3 ? (size_t)n[2] : 1, sx = (size_t)n[1] * sy;
    float acc = 0.f;
    if (JOSEPH) {
        const float step = 0.5f;
        // samples at t = te + k / 2 <= tx (the reference's t += step; its float32
        // running sum drifts from te + k / 2 over a ray, this does not)
        const int cap = (int)fminf((tx - te) / step, 4.f * (n[0] + n[1] + (DIM == 3 ? n[2] : 0))) + 2;
        // 2D back projection: the splats of consecutive samples into the
        // corners of the current cell cur are summed in registers (slot c:
        // corner cur + bits of c) and added into the image when the cell moves
        // on, about 1.4 atomics per sample instead of 4.  Neighbouring rays of a
        // warp splat into the same pixels, and those atomics were the 2D
        // kernel's limit.  In 3D the lanes' splats spread along z and their
        // atomics coalesce; there the per-sample splats are kept (the lanes'
        // flushes, at different samples, issue far more atomic instructions).
        int cur[3] = {0, 0, 0};
        float slot[1 << DIM];
#pragma unroll
        for (int c = 0; c < (1 << DIM); ++c) slot[c] = 0.f;
#if VG_JOSEPH_AFFINE
        // sample k's pixel coordinates, (o + t h - c0) / d at t = te + k step,
        // as F0 + k dF (one FMA per axis, no division per sample; within an ulp
        // of |f| of the quotient); the samples are the loop's own: k < cap with
        // te + k step <= tx, a prefix of k found once
        float F0[3], dF[3];
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            F0[a] = (R.o[a] + te * R.h[a] - c0[a]) / d;
            dF[a] = step * R.h[a] / d;
        }
        int kend;
        {
            int k = min((int)floorf((tx - te) / step), cap - 1);
            for (int q = 0; q < 3 && k >= 0 && !(fmaf((float)k, step, te) <= tx); ++q) --k;
            for (int q = 0; q < 3 && k + 1 < cap && fmaf((float)(k + 1), step, te) <= tx; ++q) ++k;
            kend = k + 1;
        }
        for (int it = 0; it < kend; ++it) {
            float f[3];
#pragma unroll
            for (int a = 0; a < DIM; ++a) f[a] = fmaf((float)it, dF[a], F0[a]);
#else
        for (int it = 0; it < cap; ++it) {
            const float t = fmaf((float)it, step, te);
            if (!(t <= tx)) break;
            float f[3];
#pragma unroll
            for (int a = 0; a < DIM; ++a) f[a] = (R.o[a] + t * R.h[a] - c0[a]) / d;
#endif
            if (!BP && DIM == 2) {  // rd.py:269-289: clamped bilinear
                const float fx = fminf(fmaxf(f[0], 0.f), n[0] - 2.f);
                const float fy = fminf(fmaxf(f[1], 0.f), n[1] - 2.f);
                const int ix = (int)fx, iy = (int)fy;
                const float dx = fx - ix, dy = fy - iy;
                const float *b = img + ix * sx + iy;
                acc += (__ldg(b) * (1 - dx) * (1 - dy) + __ldg(b + sx) * dx * (1 - dy) +
                        __ldg(b + 1) * (1 - dx) * dy + __ldg(b + sx + 1) * dx * dy) * step;
            } else if (!BP) {  // rd.py:301-350: truncation, interior cells only
                const int ix = (int)f[0], iy = (int)f[1], iz = (int)f[2];
                if (0 <= ix && ix < n[0] - 1 && 0 <= iy && iy < n[1] - 1 && 0 <= iz && iz < n[2] - 1) {
                    const float dx = f[0] - ix, dy = f[1] - iy, dz = f[2] - iz;
                    const float *b = img + ix * sx + iy * sy + iz;
                    const float c00 = __ldg(b) + dx * (__ldg(b + sx) - __ldg(b));
                    const float c10 = __ldg(b + sy) + dx * (__ldg(b + sx + sy) - __ldg(b + sy));
                    const float c01 = __ldg(b + 1) + dx * (__ldg(b + sx + 1) - __ldg(b + 1));
                    const float c11 = __ldg(b + sy + 1) + dx * (__ldg(b + sx + sy + 1) - __ldg(b + sy + 1));
                    const float c0v = c00 + dy * (c10 - c00), c1v = c01 + dy * (c11 - c01);
                    acc += (c0v + dz * (c1v - c0v)) * step;
                }
            } else {  // rd.py:357-447: floor, splat where in bounds
                int i0[3] = {0, 0, 0};
                float w0[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int a = 0; a < DIM; ++a) {
                    i0[a] = (int)floorf(f[a]);
                    w0[a] = f[a] - i0[a];
                }
                if (DIM == 3) {  // 3D: each splat added at once (see the comment at cur)
#pragma unroll
                    for (int c = 0; c < (1 << DIM); ++c) {
                        float w = s * step;
                        bool ok = true;
                        size_t off = 0;
#pragma unroll
                        for (int a = 0; a < DIM; ++a) {
                            const int bit = (c >> a) & 1, i = i0[a] + bit;
                            ok = ok && i >= 0 && i < n[a];
                            w *= bit ? w0[a] : 1.f - w0[a];
                            off += (size_t)i * (a == 0 ? sx : (a == 1 ? sy : 1));
                        }
                        if (ok) atomicAdd(bimg + off, w);
                    }
                    continue;
                }
                if (it == 0) {
#pragma unroll
                    for (int a = 0; a < DIM; ++a) cur[a] = i0[a];
                }
                // move the corner sums to the sample's cell, one axis at a time:
                // corners the cell leaves are added into the image, the ones it
                // keeps stay, the new ones start at zero
#pragma unroll
                for (int a = 0; a < DIM; ++a) {
                    const int dl = i0[a] - cur[a];
                    if (dl == 0) continue;
                    const int bit = 1 << a;
#pragma unroll
                    for (int c = 0; c < (1 << DIM); ++c) {
                        if (c & bit) continue;
                        // c: the low corner along a, c | bit: the high one
                        if (dl == 1) {
                            flush<DIM>(c, cur, bimg, n, sx, sy, slot);
                            slot[c] = slot[c | bit];
                            slot[c | bit] = 0.f;
                        } else if (dl == -1) {
                            flush<DIM>(c | bit, cur, bimg, n, sx, sy, slot);
                            slot[c | bit] = slot[c];
                            slot[c] = 0.f;
                        } else {
                            flush<DIM>(c, cur, bimg, n, sx, sy, slot);
                            flush<DIM>(c | bit, cur, bimg, n, sx, sy, slot);
                            slot[c] = slot[c | bit] = 0.f;
                        }
                    }
                    cur[a] = i0[a];
                }
                const float sw = s * step;
#pragma unroll
                for (int c = 0; c < (1 << DIM); ++c) {
                    float w = sw;
#pragma unroll
                    for (int a = 0; a < DIM; ++a) w *= ((c >> a) & 1) ? w0[a] : 1.f - w0[a];
                    slot[c] += w;
                }
            }
        }
        if (BP && DIM == 2) {
#pragma unroll
            for (int c = 0; c < (1 << DIM); ++c) flush<DIM>(c, cur, bimg, n, sx, sy, slot);
        }
        return acc;
    }
    int ir[3] = {0, 0, 0}, dir[3] = {0, 0, 0};
    float ts[3] = {INFINITY, INFINITY, INFINITY}, tn[3] = {INFINITY, INFINITY, INFINITY};
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
        // _calc_ir0 and _fp_step_init (rd.py:67-109)
        float r = R.o[a] + te * R.h[a];
        r = fminf(fmaxf(r, lo[a] + RD_EPS), hi[a] - RD_EPS);
        // entry voxel; r - hi may round to 0 in float32 (hi - eps == hi), so the
        // index is clamped to the grid (the reference's walk would stop there)
        ir[a] = min(max((int)floorf((r - lo[a]) / d), 0), n[a] - 1);
        float rn;
        if (R.h[a] > 0) { dir[a] = 1; rn = lo[a] + (ir[a] + 1) * d; }
        else { dir[a] = -1; rn = lo[a] + ir[a] * d; }
        if (fabsf(R.h[a]) > RD_EPS) { ts[a] = d / fabsf(R.h[a]); tn[a] = (rn - R.o[a]) / R.h[a]; }
        if (DIM == 2) tn[a] = fmaxf(tn[a], te);  // rd.py:116-117, 155-156
    }
    float t = te;
    const int cap = n[0] + n[1] + (DIM == 3 ? n[2] : 0) + 4;
    for (int it = 0; it < cap; ++it) {
        // the 2D forward walks while t <= t_exit (rd.py:126), the others while t < t_exit
        if (DIM == 2 && !BP ? !(t <= tx) : !(t < tx)) break;
        bool out = false;
#pragma unroll
        for (int a = 0; a < DIM; ++a) out = out || ir[a] < 0 || ir[a] >= n[a];
        if (out) break;
        // the axis whose boundary comes first (ties to the lower axis), as
        // per-axis flags so that the walk state stays in registers
        bool pick[3];
        if (DIM == 2) {
            pick[0] = tn[0] <= tn[1];
            pick[1] = !pick[0];
            pick[2] = false;
        } else {
            pick[0] = tn[0] <= tn[1] && tn[0] <= tn[2];
            pick[1] = !pick[0] && tn[1] <= tn[2];
            pick[2] = !pick[0] && !pick[1];
        }
        const float tnext = fminf(pick[0] ? tn[0] : (pick[1] ? tn[1] : tn[2]), tx);
        const size_t v = ir[0] * sx + ir[1] * sy + (DIM == 3 ? (size_t)ir[2] : 0);
        if (BP) atomicAdd(bimg + v, s * (tnext - t));
        else acc += __ldg(img + v) * (tnext - t);
        t = tnext;
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            if (pick[a]) {
                tn[a] += ts[a];
                ir[a] += dir[a];
            }
        }
    }
    return acc;
}

__device__ __forceinline__ void make_ray(const vg_ray_geom &g, float c, float s, float u, float v,
                                         Ray &R) {
    if (g.kind == 0) {
        R.o[0] = u * -s; R.o[1] = u * c; R.o[2] = 0.f;
        R.h[0] = c; R.h[1] = s; R.h[2] = 0.f;
        return;
    }
    R.o[0] = g.DSO * c; R.o[1] = g.DSO * s; R.o[2] = 0.f;
    const float vx = -(g.DSD - g.DSO) * c + u * -s - R.o[0];
    const float vy = -(g.DSD - g.DSO) * s + u * c - R.o[1];
    const float vz = g.kind == 2 ? v : 0.f;
    const float m = sqrtf(vx * vx + vy * vy + vz * vz);
    R.h[0] = vx / m; R.h[1] = vy / m; R.h[2] = vz / m;
}

template <int DIM, bool JOSEPH, bool BP>
__global__ void __launch_bounds__(256)
rd_kernel(vg_ray_geom g, const double *__restrict__ trig, const float *__restrict__ in,
          float *__restrict__ out, float bp_scale) {
    const int iv = DIM == 3 ? (int)(blockIdx.x * blockDim.x + threadIdx.x) : 0;
    const int iu = DIM == 3 ? (int)blockIdx.y : (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int ia = DIM == 3 ? (int)blockIdx.z : (int)blockIdx.y;
    const int nv = DIM == 3 ? g.nv : 1;
    if (iu >= g.nu || iv >= nv) return;
    const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
    const float u = g.du * ((float)iu - ((float)g.nu / 2.f - 0.5f) + g.su);
    const float v = g.dv * ((float)iv - ((float)g.nv / 2.f - 0.5f) + g.sv);
    Ray R;
    make_ray(g, c, s, u, v, R);
    const int n[3] = {g.nx, g.ny, g.nz};
    const size_t k = ((size_t)ia * g.nu + iu) * nv + iv;
    if (BP) {
        trace<DIM, JOSEPH, true>(R, nullptr, out, __ldg(in + k) * bp_scale, n, g.d_pix);
    } else {
        float val = trace<DIM, JOSEPH, false>(R, in, nullptr, 0.f, n, g.d_pix);
        if (DIM == 3 && !JOSEPH) val *= g.DSD / sqrtf(g.DSD * g.DSD + u * u + v * v);  // rd.py:782
        out[k] = val;
    }
}

// ---- 2D Amanatides-Woo back projection in gather form ----------------------
//
// The walk's back projection adds s * (t_next - t) to each pixel a ray
// crosses (rd.py:152-176): the length of the ray's chord through the pixel.
// Here a thread owns a 2 x 2 pixel patch and, for every view, sums s times
// the chord of each ray whose detector coordinate falls in the patch's
// shadow (about four rays at 2x magnification and 0.75 bins per pixel): no
// atomics, a fixed summation order.  A chord is the overlap of the ray's
// parameter intervals between the pixel's x planes and between its y planes,
// t_k = A + k B per axis with (A, B) a function of the ray alone, so that
// neighbouring pixels see bit-identical plane crossings and a ray's chords
// telescope as the walk's segments do.  A ray the walk takes as parallel to
// an axis (|h| <= 1e-6, rd.py:58-64, 99-109) never leaves the row or column
// it enters in; those rays (|h| <= 1e-5, a superset) take the walk's own
// set-up (make_ray, slab, the entry index) and are given that row or column.
#ifndef VG_AWG_VS
#define VG_AWG_VS 4
#endif
constexpr int AWG_VS = VG_AWG_VS;              // threads sharing a patch's views
constexpr int AWG_TY = 32;                     // patches along y
constexpr int AWG_TX = 8 / AWG_VS;             // patches along x
constexpr int AWG_VC = 128;  // views staged per chunk
constexpr float AWG_NEAR = 1e-5f;

// Chords of the patch's 4 pixels from the x and y plane parameters (3 each):
// pixel (i, j) spans [tx_i, tx_i+1] and [ty_j, ty_j+1] in either order.
__device__ __forceinline__ void awg_chords(const float *tx, const float *ty, float w,
                                           float (&acc)[2][2]) {
    float ix0[2], ix1[2], iy0[2], iy1[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        ix0[i] = fminf(tx[i], tx[i + 1]);
        ix1[i] = fmaxf(tx[i], tx[i + 1]);
        iy0[i] = fminf(ty[i], ty[i + 1]);
        iy1[i] = fmaxf(ty[i], ty[i + 1]);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float len = fminf(ix1[i], iy1[j]) - fmaxf(ix0[i], iy0[j]);
            acc[i][j] = fmaf(w, fmaxf(len, 0.f), acc[i][j]);
        }
}

// A ray within AWG_NEAR of an axis: the walk's own set-up.  Along an axis
// with |h| > 1e-6 the pixel's planes bound the chord as above (t with the
// unit direction); along the other the ray keeps the entry index the walk
// computes (rd.py:67-74), and only that row or column receives it.  The
// chord is clipped to the walk's [t_entry, t_exit].
__device__ void awg_near(const vg_ray_geom &g, float c, float s, float u, int ix, int iy, float w,
                         float (&acc)[2][2]) {
    Ray R;
    make_ray(g, c, s, u, 0.f, R);
    const int n[2] = {g.nx, g.ny};
    const int k0[2] = {ix, iy};
    float lo[2], hi[2], c0[2], te = -INFINITY, tx = INFINITY;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        float t0, t1;
        bounds1(n[a], g.d_pix, lo[a], hi[a], c0[a]);
        slab(R.o[a], R.h[a], lo[a], hi[a], t0, t1);
        te = fmaxf(te, t0);
        tx = fminf(tx, t1);
    }
    if (!(tx > te)) return;  // the walk does not enter the image
    float in[2][2], out[2][2];  // [axis][pixel offset]: the pixel's t interval along the axis
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        if (fabsf(R.h[a]) > RD_EPS) {
            float tp[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) tp[q] = (lo[a] + (float)(k0[a] + q) * g.d_pix - R.o[a]) / R.h[a];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                in[a][i] = fminf(tp[i], tp[i + 1]);
                out[a][i] = fmaxf(tp[i], tp[i + 1]);
            }
        } else {
            float r = fminf(fmaxf(R.o[a] + te * R.h[a], lo[a] + RD_EPS), hi[a] - RD_EPS);
            const int ir = min(max((int)floorf((r - lo[a]) / g.d_pix), 0), n[a] - 1);
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const bool on = k0[a] + i == ir;
                in[a][i] = on ? -INFINITY : INFINITY;
                out[a][i] = on ? INFINITY : -INFINITY;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float len = fminf(fminf(out[0][i], out[1][j]), tx) - fmaxf(fmaxf(in[0][i], in[1][j]), te);
            if (len > 0.f) acc[i][j] = fmaf(w, len, acc[i][j]);
        }
}

__device__ __forceinline__ float awg_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// One block: AWG_TY x AWG_TX patches (2 AWG_TY x 2 AWG_TX pixels), each
// patch's views split over AWG_VS threads whose sums are added in a fixed
// order at the end.  Per view the block stages the view's constants: fan
// (c, s, -DSD c, -DSD s | lox - DSO c, loy - DSO s); parallel (c, s, d/c, d/s |
// s/c, lox/c, -c/s, loy/s: the plane parameters of the view's common direction).
template <bool FAN>
__global__ void __launch_bounds__(AWG_TY * AWG_TX * AWG_VS)
aw_bp2d_gather(vg_ray_geom g, const double *__restrict__ trig, const float *__restrict__ sino,
               float *__restrict__ img, float sc) {
    __shared__ float4 V1[AWG_VC], V2[AWG_VC];
    __shared__ float red[AWG_VS - 1][AWG_TY * AWG_TX][4];
    const int tid = threadIdx.x;
    const int pt = tid % (AWG_TY * AWG_TX), part = tid / (AWG_TY * AWG_TX);
    const int iy = blockIdx.x * (2 * AWG_TY) + 2 * (pt % AWG_TY);  // patch origin
    const int ix = blockIdx.y * (2 * AWG_TX) + 2 * (pt / AWG_TY);
    const bool inside = ix < g.nx && iy < g.ny;
    const float d = g.d_pix;
    float lox, hix, c0x, loy, hiy, c0y;
    bounds1(g.nx, d, lox, hix, c0x);
    bounds1(g.ny, d, loy, hiy, c0y);
    // the patch's planes x_k = lo + k d, k = ix .. ix + 2 (the walk's grid)
    const float kx = (float)ix, ky = (float)iy;
    const float px0 = lox + kx * d, py0 = loy + ky * d;  // patch corner
    const float uoff = (float)g.nu / 2.f - 0.5f - g.su;    // u = du (iu - uoff)
    const float rdu = 1.f / g.du;
    float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int a0 = 0; a0 < g.na; a0 += AWG_VC) {
        const int nv = min(AWG_VC, g.na - a0);
        __syncthreads();
        for (int k = tid; k < nv; k += AWG_TY * AWG_TX * AWG_VS) {
            const float c = (float)__ldg(trig + 2 * (a0 + k)), s = (float)__ldg(trig + 2 * (a0 + k) + 1);
            if (FAN) {
                V1[k] = make_float4(c, s, -g.DSD * c, -g.DSD * s);
                V2[k] = make_float4(lox - g.DSO * c, loy - g.DSO * s, 0.f, 0.f);
            } else {
                // ray o = u (-s, c), h = (c, s): A_x = (lox + u s) / c, B_x = d / c
                const float rc = awg_rcp(c), rs = awg_rcp(s);
                V1[k] = make_float4(c, s, d * rc, d * rs);
                V2[k] = make_float4(s * rc, lox * rc, -c * rs, loy * rs);  // A = fma(u, .x, .y) ...
            }
        }
        __syncthreads();
        if (!inside) continue;
        for (int vi = part; vi < nv; vi += AWG_VS) {
            const float4 q = V1[vi], q2 = V2[vi];
            const float c = q.x, s = q.y;
            const float *row = sino + (size_t)(a0 + vi) * g.nu;
            // the patch's shadow on the detector, widened by a hundredth of a bin
            float umin, umax;
            {
                const float a00 = fmaf(px0, c, py0 * s), b00 = fmaf(py0, c, -px0 * s);
                const float dax = 2.f * d * c, day = 2.f * d * s;  // corner steps of a, b
                float us[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float ka = (k & 1) ? 1.f : 0.f, kb = (k & 2) ? 1.f : 0.f;
                    const float aa = fmaf(kb, day, fmaf(ka, dax, a00));
                    const float bb = fmaf(kb, dax, fmaf(ka, -day, b00));
                    us[k] = FAN ? g.DSD * bb * awg_rcp(g.DSO - aa) : bb;
                }
                umin = fminf(fminf(us[0], us[1]), fminf(us[2], us[3]));
                umax = fmaxf(fmaxf(us[0], us[1]), fmaxf(us[2], us[3]));
            }
            const int ja = max((int)ceilf(fmaf(umin, rdu, uoff) - 0.01f), 0);
            const int jb = min((int)floorf(fmaf(umax, rdu, uoff) + 0.01f), g.nu - 1);
            if (!FAN && (fabsf(c) <= AWG_NEAR || fabsf(s) <= AWG_NEAR)) {  // taken as axis-parallel
                for (int iu = ja; iu <= jb; ++iu) {
                    const float u = g.du * ((float)iu - ((float)g.nu / 2.f - 0.5f) + g.su);
                    awg_near(g, c, s, u, ix, iy, __ldg(row + iu), acc);
                }
                continue;
            }
            for (int iu = ja; iu <= jb; ++iu) {
                const float sv = __ldg(row + iu);
                const float u = g.du * ((float)iu - ((float)g.nu / 2.f - 0.5f) + g.su);
                float Ax, Bx, Ay, By, w;
                if (FAN) {
                    // direction (vx, vy) from the source, not normalised:
                    // parameters t' = t / m, chords scaled by m
                    const float vx = fmaf(-u, s, q.z), vy = fmaf(u, c, q.w);
                    const float m2 = fmaf(vx, vx, vy * vy);
                    const float m = m2 * rsqrtf(m2);
                    if (fabsf(vx) <= AWG_NEAR * m || fabsf(vy) <= AWG_NEAR * m) {
                        awg_near(g, c, s, u, ix, iy, sv, acc);
                        continue;
                    }
                    const float rvx = awg_rcp(vx), rvy = awg_rcp(vy);
                    Ax = q2.x * rvx; Bx = d * rvx;
                    Ay = q2.y * rvy; By = d * rvy;
                    w = sv * m;
                } else {
                    Ax = fmaf(u, q2.x, q2.y); Bx = q.z;
                    Ay = fmaf(u, q2.z, q2.w); By = q.w;
                    w = sv;
                }
                float tx[3], ty[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    tx[k] = fmaf(kx + (float)k, Bx, Ax);
                    ty[k] = fmaf(ky + (float)k, By, Ay);
                }
                awg_chords(tx, ty, w, acc);
            }
        }
    }
    // the view parts' sums, added in part order
    if (AWG_VS > 1) {
        if (part > 0) {
#pragma unroll
            for (int i = 0; i < 4; ++i) red[part - 1][pt][i] = acc[i >> 1][i & 1];
        }
        __syncthreads();
        if (part > 0) return;
#pragma unroll
        for (int p = 0; p < AWG_VS - 1; ++p)
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[i >> 1][i & 1] += red[p][pt][i];
    }
    if (!inside) return;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
            if (ix + i < g.nx && iy + j < g.ny) img[(size_t)(ix + i) * g.ny + iy + j] = acc[i][j] * sc;
}

// ---- pixel-driven ------------------------------------------------------------

struct Foot {
    float pmin, pmax, scale;  // detector interval and the pixel's weight scale
    float cm;                 // cone: v magnification
};

// The pixel's footprint on the detector for view (c, s) (pd.py:186-206,
// 296-330, 405-445).
__device__ __forceinline__ Foot footprint(const vg_ray_geom &g, float c, float s, int ix, int iy) {
    const float xl = g.d_pix * ((float)ix - g.nx / 2.f), xr = g.d_pix * ((float)(ix + 1) - g.nx / 2.f);
    const float yl = g.d_pix * ((float)iy - g.ny / 2.f), yr = g.d_pix * ((float)(iy + 1) - g.ny / 2.f);
    Foot f;
    f.scale = 1.f / (fabsf(s) + fabsf(c));
    f.cm = 1.f;
    float p[4];
    if (g.kind == 0) {
        p[0] = -s * xl + c * yl; p[1] = -s * xr + c * yl;
        p[2] = -s * xl + c * yr; p[3] = -s * xr + c * yr;
    } else {
        const float xc = 0.5f * (xl + xr), yc = 0.5f * (yl + yr);
        const float oc = c * xc + s * yc;
        const float t = (g.DSD * (-s * xc + c * yc) / (g.DSO - oc)) / g.DSD;  // tan g
        const float sec = sqrtf(1.f + t * t);
        if (g.kind == 1) {
            auto pj = [&](float x, float y) { return g.DSD * (-s * x + c * y) / (g.DSO - (c * x + s * y)); };
            p[0] = pj(xl, yl); p[1] = pj(xr, yl); p[2] = pj(xl, yr); p[3] = pj(xr, yr);
            f.scale = sec / (fabsf(c - s * t) + fabsf(s + c * t));
        } else {
            const float fm = g.DSD / (g.DSO - oc);
            p[0] = fm * (-s * xl + c * yl); p[1] = fm * (-s * xr + c * yl);
            p[2] = fm * (-s * xl + c * yr); p[3] = fm * (-s * xr + c * yr);
            f.cm = fm * sec;
        }
    }
    f.pmin = fminf(fminf(p[0], p[1]), fminf(p[2], p[3]));
    f.pmax = fmaxf(fmaxf(p[0], p[1]), fmaxf(p[2], p[3]));
    return f;
}

__device__ __forceinline__ float ubnd(const vg_ray_geom &g, int k) {
    return g.du * ((float)k - g.nu / 2.f + g.su);
}
__device__ __forceinline__ float vbnd(const vg_ray_geom &g, int k) {
    return g.dv * ((float)k - g.nv / 2.f + g.sv);
}

// FP: thread = (view, pixel column); scatters value * scale * overlap / du
// (* dv overlap / dv) * d_pix.
__global__ void __launch_bounds__(256)
pd_fp_kernel(vg_ray_geom g, const double *__restrict__ trig, const float *__restrict__ img,
             float *__restrict__ sino) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int ia = blockIdx.y;
    if (p >= g.nx * g.ny) return;
    const int ix = p / g.ny, iy = p - ix * g.ny;
    const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
    const Foot f = footprint(g, c, s, ix, iy);
    // cell widths enter as reciprocals (one division per thread, not per cell);
    // the cell ranges are the cells holding the interval's ends, widened by
    // 1e-4 cell against the rounding of the index arithmetic
    const float inv_du = 1.f / g.du, inv_dv = g.kind == 2 ? 1.f / g.dv : 1.f;
    const float u0 = ubnd(g, 0);
    const int iu0 = max(0, (int)floorf(fmaf(f.pmin - u0, inv_du, -1e-4f)));
    const int iu1 = min(g.nu, (int)floorf(fmaf(f.pmax - u0, inv_du, 1e-4f)) + 1);
    if (g.kind < 2) {
        const float val = __ldg(img + p);
        if (val == 0.f) return;
        const float k = val * f.scale * inv_du * g.d_pix;
        for (int iu = iu0; iu < iu1; ++iu) {
            const float l = fmaxf(f.pmin, ubnd(g, iu)), r = fminf(f.pmax, ubnd(g, iu + 1));
            if (r > l) atomicAdd(sino + (size_t)ia * g.nu + iu, k * (r - l));
        }
        return;
    }
    const float kc = f.scale * inv_du * inv_dv * g.d_pix;
    const float *col = img + (size_t)p * g.nz;
    for (int iz = 0; iz < g.nz; ++iz) {
        const float val = __ldg(col + iz);
        if (val == 0.f) continue;
        const float zl = g.d_pix * ((float)iz - g.nz / 2.f), zr = g.d_pix * ((float)(iz + 1) - g.nz / 2.f);
        const float vmin = fminf(f.cm * zl, f.cm * zr), vmax = fmaxf(f.cm * zl, f.cm * zr);
        const int iv0 = max(0, (int)floorf(fmaf(vmin - vbnd(g, 0), inv_dv, -1e-4f)));
        const int iv1 = min(g.nv, (int)floorf(fmaf(vmax - vbnd(g, 0), inv_dv, 1e-4f)) + 1);
        const float kv = val * kc;
        for (int iv = iv0; iv < iv1; ++iv) {
            const float vl = fmaxf(vmin, vbnd(g, iv)), vr = fminf(vmax, vbnd(g, iv + 1));
            if (vr <= vl) continue;
            const float kvv = kv * (vr - vl);
            for (int iu = iu0; iu < iu1; ++iu) {
                const float ul = fmaxf(f.pmin, ubnd(g, iu)), ur = fminf(f.pmax, ubnd(g, iu + 1));
                if (ur > ul) atomicAdd(sino + ((size_t)ia * g.nu + iu) * g.nv + iv, kvv * (ur - ul));
            }
        }
    }
}

// 2D FP with a run of PD_RUN pixels along y per thread: the footprints of
// consecutive pixels move monotonically along u (towards larger u when
// c > 0 (parallel) or c DSO > x (fan), the sign of dp/dy), so the thread
// visits each pixel's bins in that direction and sums consecutive
// contributions to one bin in a register, adding the sum into the sinogram
// when the bin changes.  Each contribution is pd_fp_kernel's.
#ifndef VG_PD_RUN
#define VG_PD_RUN 32
#endif
constexpr int PD_RUN = VG_PD_RUN;

__global__ void __launch_bounds__(256)
pd_fp_run_kernel(vg_ray_geom g, const double *__restrict__ trig, const float *__restrict__ img,
                 float *__restrict__ sino) {
    const int runs = (g.ny + PD_RUN - 1) / PD_RUN;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int ia = blockIdx.y;
    if (q >= g.nx * runs) return;
    const int ix = q / runs, iy0 = (q - ix * runs) * PD_RUN;
    const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
    const float inv_du = 1.f / g.du;
    const float u0 = ubnd(g, 0);
    const float x = g.d_pix * ((float)ix + 0.5f - g.nx / 2.f);
    const bool up = g.kind == 0 ? c >= 0.f : c * g.DSO >= x;
    float *row = sino + (size_t)ia * g.nu;
    int pb = -1;
    float pv = 0.f;
    for (int i = 0; i < PD_RUN; ++i) {
        const int iy = iy0 + i;
        if (iy >= g.ny) break;
        const float val = __ldg(img + (size_t)ix * g.ny + iy);
        if (val == 0.f) continue;
        const Foot f = footprint(g, c, s, ix, iy);
        const int iu0 = max(0, (int)floorf(fmaf(f.pmin - u0, inv_du, -1e-4f)));
        const int iu1 = min(g.nu, (int)floorf(fmaf(f.pmax - u0, inv_du, 1e-4f)) + 1);
        const float k = val * f.scale * inv_du * g.d_pix;
        for (int m = 0; m < iu1 - iu0; ++m) {
            const int iu = up ? iu0 + m : iu1 - 1 - m;
            const float l = fmaxf(f.pmin, ubnd(g, iu)), r = fminf(f.pmax, ubnd(g, iu + 1));
            if (!(r > l)) continue;
            const float w = k * (r - l);
            if (iu == pb) {
                pv += w;
            } else {
                if (pb >= 0) atomicAdd(row + pb, pv);
                pb = iu;
                pv = w;
            }
        }
    }
    if (pb >= 0) atomicAdd(row + pb, pv);
}

// BP: thread = pixel / voxel (lanes along z for the cone), gather over views.
__global__ void __launch_bounds__(256)
pd_bp_kernel(vg_ray_geom g, const double *__restrict__ trig, const float *__restrict__ sino,
             float *__restrict__ img, float scale) {
    const int nz = g.kind == 2 ? g.nz : 1;
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (size_t)g.nx * g.ny * nz) return;
    const int iz = (int)(q % nz);
    const int p = (int)(q / nz), ix = p / g.ny, iy = p - ix * g.ny;
    const float zl = g.d_pix * ((float)iz - g.nz / 2.f), zr = g.d_pix * ((float)(iz + 1) - g.nz / 2.f);
    // cell widths enter as reciprocals (one division per thread, not per cell);
    // the cell ranges are the cells holding the interval's ends, widened by
    // 1e-4 cell against the rounding of the index arithmetic
    const float inv_du = 1.f / g.du, inv_dv = g.kind == 2 ? 1.f / g.dv : 1.f;
    const float u0 = ubnd(g, 0), v0 = g.kind == 2 ? vbnd(g, 0) : 0.f;
    // per-view terms summed in groups of 16 views, the group sums compensated
    Kahan acc;
    float grp = 0.f;
    for (int ia = 0; ia < g.na; ++ia) {
        const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
        const Foot f = footprint(g, c, s, ix, iy);
        const int iu0 = max(0, (int)floorf(fmaf(f.pmin - u0, inv_du, -1e-4f)));
        const int iu1 = min(g.nu, (int)floorf(fmaf(f.pmax - u0, inv_du, 1e-4f)) + 1);
        float part = 0.f;
        if (g.kind < 2) {
            const float *row = sino + (size_t)ia * g.nu;
            const float k = f.scale * inv_du;
            for (int iu = iu0; iu < iu1; ++iu) {
                const float l = fmaxf(f.pmin, ubnd(g, iu)), r = fminf(f.pmax, ubnd(g, iu + 1));
                if (r > l) part = fmaf(__ldg(row + iu), k * (r - l), part);
            }
        } else {
            const float vmin = fminf(f.cm * zl, f.cm * zr), vmax = fmaxf(f.cm * zl, f.cm * zr);
            const int iv0 = max(0, (int)floorf(fmaf(vmin - v0, inv_dv, -1e-4f)));
            const int iv1 = min(g.nv, (int)floorf(fmaf(vmax - v0, inv_dv, 1e-4f)) + 1);
            const float k = f.scale * inv_du * inv_dv;
            const float *col = sino + (size_t)ia * g.nu * g.nv;
            for (int iv = iv0; iv < iv1; ++iv) {
                const float vl = fmaxf(vmin, vbnd(g, iv)), vr = fminf(vmax, vbnd(g, iv + 1));
                if (vr <= vl) continue;
                const float kv = k * (vr - vl);
                for (int iu = iu0; iu < iu1; ++iu) {
                    const float ul = fmaxf(f.pmin, ubnd(g, iu)), ur = fminf(f.pmax, ubnd(g, iu + 1));
                    if (ur > ul) part = fmaf(__ldg(col + (size_t)iu * g.nv + iv), kv * (ur - ul), part);
                }
            }
        }
        grp += part;
        if ((ia & 15) == 15) {
            acc.add(grp);
            grp = 0.f;
        }
    }
    acc.add(grp);
    img[q] = acc.s * scale;
}

#ifndef VG_PD_ZPT
#define VG_PD_ZPT 4
#endif
#ifndef VG_PD_FV
#define VG_PD_FV 3
#endif
constexpr int PD_ZPT = VG_PD_ZPT, PD_FAST = 4, PD_FV = VG_PD_FV;  // fast path: u, v cells

// Cone FP with one warp per (x, y) column and view: lanes hold the voxels
// z = l + 32 m of a z chunk (as pd_bp_cone_kernel), so the warp's atomics
// fall on neighbouring v cells of one u row.  The u overlaps are worked out
// once per column and view; each term is pd_fp_kernel's
// ((value kc) (vr - vl)) (ur - ul), cells of zero overlap and zero voxels add
// nothing.
__global__ void __launch_bounds__(256)
pd_fp_cone_kernel(vg_ray_geom g, const double *__restrict__ trig, const float *__restrict__ img,
                  float *__restrict__ sino, int colx) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int bx = blockIdx.x % colx, by = blockIdx.x / colx;
    const int ix = bx * 2 + (warp >> 2), iy = by * 4 + (warp & 3);
    const int zb = blockIdx.y * 32 * PD_ZPT, ia = blockIdx.z;
    if (ix >= g.nx || iy >= g.ny) return;  // warp-uniform; no barriers below
    const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
    const Foot f = footprint(g, c, s, ix, iy);
    const float inv_du = 1.f / g.du, inv_dv = 1.f / g.dv;
    const float u0 = ubnd(g, 0), v0 = vbnd(g, 0);
    const int iu0 = max(0, (int)floorf(fmaf(f.pmin - u0, inv_du, -1e-4f)));
    const int iu1 = min(g.nu, (int)floorf(fmaf(f.pmax - u0, inv_du, 1e-4f)) + 1);
    const int nuc = iu1 - iu0;
    const float kc = f.scale * inv_du * inv_dv * g.d_pix;
    float *view = sino + (size_t)ia * g.nu * g.nv;
    const float *col = img + ((size_t)ix * g.ny + iy) * g.nz;
    float wu[PD_FAST];
#pragma unroll
    for (int a = 0; a < PD_FAST; ++a) {
        const float ul = fmaxf(f.pmin, ubnd(g, iu0 + a)), ur = fminf(f.pmax, ubnd(g, iu0 + a + 1));
        wu[a] = (a < nuc && ur > ul) ? ur - ul : 0.f;
    }
#pragma unroll
    for (int m = 0; m < PD_ZPT; ++m) {
        const int iz = zb + lane + 32 * m;
        const float val = iz < g.nz ? __ldg(col + iz) : 0.f;
        if (val == 0.f) continue;
        const float zl = g.d_pix * ((float)iz - g.nz / 2.f), zr = g.d_pix * ((float)(iz + 1) - g.nz / 2.f);
        const float vmn = fminf(f.cm * zl, f.cm * zr), vmx = fmaxf(f.cm * zl, f.cm * zr);
        const int iv0 = max(0, (int)floorf(fmaf(vmn - v0, inv_dv, -1e-4f)));
        const int iv1 = min(g.nv, (int)floorf(fmaf(vmx - v0, inv_dv, 1e-4f)) + 1);
        const float kv = val * kc;
        if (nuc <= PD_FAST && iv1 - iv0 <= PD_FV) {
            float wv[PD_FV];
#pragma unroll
            for (int j = 0; j < PD_FV; ++j) {
                const float vl = fmaxf(vmn, vbnd(g, iv0 + j)), vr = fminf(vmx, vbnd(g, iv0 + j + 1));
                wv[j] = (iv0 + j < iv1 && vr > vl) ? kv * (vr - vl) : 0.f;
            }
#pragma unroll
            for (int a = 0; a < PD_FAST; ++a) {
                if (a >= nuc) break;  // warp-uniform
                float *row = view + (size_t)(iu0 + a) * g.nv + iv0;
#pragma unroll
                for (int j = 0; j < PD_FV; ++j)
                    if (wv[j] != 0.f && wu[a] > 0.f) atomicAdd(row + j, wv[j] * wu[a]);
            }
        } else {
            for (int iv = iv0; iv < iv1; ++iv) {
                const float vl = fmaxf(vmn, vbnd(g, iv)), vr = fminf(vmx, vbnd(g, iv + 1));
                if (vr <= vl) continue;
                const float kvv = kv * (vr - vl);
                for (int iu = iu0; iu < iu1; ++iu) {
                    const float ul = fmaxf(f.pmin, ubnd(g, iu)), ur = fminf(f.pmax, ubnd(g, iu + 1));
                    if (ur > ul) atomicAdd(view + (size_t)iu * g.nv + iv, kvv * (ur - ul));
                }
            }
        }
    }
}

// Cone BP with one warp per (x, y) column: the column's u footprint (cells,
// overlaps) is worked out once per view for all its voxels, lane l holding the
// voxels z = l + 32 m, m < PD_ZPT (a z chunk of 32 PD_ZPT voxels per block
// row); the 8 warps of a block are a 2 x 4 patch of neighbouring columns,
// whose footprints share sinogram cells in L1.  When the footprint covers at
// most 4 u and 3 v cells, the u overlaps (ur - ul) and each voxel's
// k (vr - vl) are computed once per view and held in registers; otherwise
// the cells are walked as in pd_bp_kernel.  Each term has pd_bp_kernel's
// weight (k (vr - vl)) (ur - ul), and cells of zero overlap add nothing; per
// view the terms are summed u cells outside, v cells inside.

__global__ void __launch_bounds__(256)
pd_bp_cone_kernel(vg_ray_geom g, const double *__restrict__ trig, const float *__restrict__ sino,
                  float *__restrict__ img, float scale) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ix = blockIdx.x * 2 + (warp >> 2), iy = blockIdx.y * 4 + (warp & 3);
    const int zb = blockIdx.z * 32 * PD_ZPT;
    if (ix >= g.nx || iy >= g.ny) return;  // warp-uniform; no barriers below
    const float inv_du = 1.f / g.du, inv_dv = 1.f / g.dv;
    const float u0 = ubnd(g, 0), v0 = vbnd(g, 0);
    float zl[PD_ZPT], zr[PD_ZPT], grp[PD_ZPT];
    bool in[PD_ZPT];
    Kahan acc[PD_ZPT];
#pragma unroll
    for (int m = 0; m < PD_ZPT; ++m) {
        const int iz = zb + lane + 32 * m;
        in[m] = iz < g.nz;
        zl[m] = g.d_pix * ((float)iz - g.nz / 2.f);
        zr[m] = g.d_pix * ((float)(iz + 1) - g.nz / 2.f);
        grp[m] = 0.f;
    }
    for (int ia = 0; ia < g.na; ++ia) {
        const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
        const Foot f = footprint(g, c, s, ix, iy);
        const int iu0 = max(0, (int)floorf(fmaf(f.pmin - u0, inv_du, -1e-4f)));
        const int iu1 = min(g.nu, (int)floorf(fmaf(f.pmax - u0, inv_du, 1e-4f)) + 1);
        const int nuc = iu1 - iu0;
        const float k = f.scale * inv_du * inv_dv;
        const float *view = sino + (size_t)ia * g.nu * g.nv;
        float wu[PD_FAST];
#pragma unroll
        for (int a = 0; a < PD_FAST; ++a) {
            const float ul = fmaxf(f.pmin, ubnd(g, iu0 + a)), ur = fminf(f.pmax, ubnd(g, iu0 + a + 1));
            wu[a] = (a < nuc && ur > ul) ? ur - ul : 0.f;
        }
#pragma unroll
        for (int m = 0; m < PD_ZPT; ++m) {
            const float vmn = fminf(f.cm * zl[m], f.cm * zr[m]), vmx = fmaxf(f.cm * zl[m], f.cm * zr[m]);
            const int iv0 = in[m] ? max(0, (int)floorf(fmaf(vmn - v0, inv_dv, -1e-4f))) : 0;
            const int iv1 = in[m] ? min(g.nv, (int)floorf(fmaf(vmx - v0, inv_dv, 1e-4f)) + 1) : 0;
            const int nvc = iv1 - iv0;
            float part = 0.f;
            if (nuc <= PD_FAST && nvc <= PD_FV) {
                float wv[PD_FV];
#pragma unroll
                for (int j = 0; j < PD_FV; ++j) {
                    const float vl = fmaxf(vmn, vbnd(g, iv0 + j)), vr = fminf(vmx, vbnd(g, iv0 + j + 1));
                    wv[j] = (j < nvc && vr > vl) ? k * (vr - vl) : 0.f;
                }
#pragma unroll
                for (int a = 0; a < PD_FAST; ++a) {
                    if (a >= nuc) break;  // warp-uniform
                    const float *col = view + (size_t)(iu0 + a) * g.nv + iv0;
#pragma unroll
                    for (int j = 0; j < PD_FV; ++j)
                        if (wv[j] > 0.f && wu[a] > 0.f) part = fmaf(__ldg(col + j), wv[j] * wu[a], part);
                }
            } else {
                for (int iu = iu0; iu < iu1; ++iu) {
                    const float ul = fmaxf(f.pmin, ubnd(g, iu)), ur = fminf(f.pmax, ubnd(g, iu + 1));
                    if (!(ur > ul)) continue;
                    const float *col = view + (size_t)iu * g.nv;
                    for (int iv = iv0; iv < iv1; ++iv) {
                        const float vl = fmaxf(vmn, vbnd(g, iv)), vr = fminf(vmx, vbnd(g, iv + 1));
                        if (vr <= vl) continue;
                        part = fmaf(__ldg(col + iv), (k * (vr - vl)) * (ur - ul), part);
                    }
                }
            }
            grp[m] += part;
        }
        if ((ia & 15) == 15) {
#pragma unroll
            for (int m = 0; m < PD_ZPT; ++m) {
                acc[m].add(grp[m]);
                grp[m] = 0.f;
            }
        }
    }
    float *out = img + ((size_t)ix * g.ny + iy) * g.nz;
#pragma unroll
    for (int m = 0; m < PD_ZPT; ++m) {
        acc[m].add(grp[m]);
        if (in[m]) out[zb + lane + 32 * m] = acc[m].s * scale;
    }
}

int check(const vg_ray_geom *g) {
    VG_REQUIRE(g, "ray/pixel-driven: null geometry");
    VG_REQUIRE(g->kind >= 0 && g->kind <= 2, "ray/pixel-driven: kind must be 0 (par), 1 (fan), 2 (cone)");
    const int nz = g->kind == 2 ? g->nz : 1, nv = g->kind == 2 ? g->nv : 1;
    VG_REQUIRE(g->nx >= 2 && g->ny >= 2 && nz >= 1 && g->na > 0 && g->nu > 0 && nv > 0,
               "ray/pixel-driven: sizes must be positive (image at least 2 x 2)");
    VG_REQUIRE(g->kind < 2 || g->nz >= 2, "ray/pixel-driven: cone volume needs nz >= 2");
    VG_REQUIRE(g->na < 65536 && g->nu < 65536, "ray/pixel-driven: too many views or bins");
    VG_REQUIRE((long long)g->nx * g->ny < (1LL << 31), "ray/pixel-driven: image too large");
    VG_REQUIRE(g->du > 0.f && g->d_pix > 0.f && (g->kind < 2 || g->dv > 0.f),
               "ray/pixel-driven: pitches must be positive");
    VG_REQUIRE(g->kind == 0 || (g->DSO > 0.f && g->DSD > 0.f), "ray/pixel-driven: DSO, DSD must be positive");
    return VG_OK;
}

template <bool JOSEPH, bool BP>
void launch_rd(const vg_ray_geom &g, const double *trig, const float *in, float *out, float sc,
               cudaStream_t st) {
    if (g.kind == 2) {
        dim3 grid(ceil_div(g.nv, 128), g.nu, g.na);
        rd_kernel<3, JOSEPH, BP><<<grid, 128, 0, st>>>(g, trig, in, out, sc);
    } else {
        dim3 grid(ceil_div(g.nu, 128), g.na);
        rd_kernel<2, JOSEPH, BP><<<grid, 128, 0, st>>>(g, trig, in, out, sc);
    }
}

size_t img_count(const vg_ray_geom *g) {
    return (size_t)g->nx * g->ny * (g->kind == 2 ? g->nz : 1);
}
size_t sino_count(const vg_ray_geom *g) {
    return (size_t)g->na * g->nu * (g->kind == 2 ? g->nv : 1);
}

}  // namespace

extern "C" int vg_rd_fp(const vg_ray_geom *g, const float *img, const double *trig, float *sino,
                        void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(img && trig && sino, "rd_fp: null pointer");
    cudaStream_t st = as_stream(stream);
    if (g->joseph) launch_rd<true, false>(*g, trig, img, sino, 1.f, st);
    else launch_rd<false, false>(*g, trig, img, sino, 1.f, st);
    return launch_status("rd_fp");
}

extern "C" int vg_rd_bp(const vg_ray_geom *g, const float *sino, const double *trig, float *img,
                        void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(img && trig && sino, "rd_bp: null pointer");
    cudaStream_t st = as_stream(stream);
    // img / na / d_pix^2 * du (rd.py:538, 646); cone img / na * du * dv (rd.py:786)
    const float sc = g->kind == 2 ? g->du * g->dv / (float)g->na
                                  : g->du / ((float)g->na * g->d_pix * g->d_pix);
    if (g->kind < 2 && !g->joseph) {  // 2D walk: the gather form writes every pixel
        dim3 grid(ceil_div(g->ny, 2 * AWG_TY), ceil_div(g->nx, 2 * AWG_TX));
        VG_REQUIRE(grid.y < 65536, "rd_bp: nx too large");
        const int nt = AWG_TY * AWG_TX * AWG_VS;
        if (g->kind == 1) aw_bp2d_gather<true><<<grid, nt, 0, st>>>(*g, trig, sino, img, sc);
        else aw_bp2d_gather<false><<<grid, nt, 0, st>>>(*g, trig, sino, img, sc);
        return launch_status("rd_bp");
    }
    cudaError_t e = cudaMemsetAsync(img, 0, img_count(g) * sizeof(float), st);
    if (e != cudaSuccess) return cuda_status(e, "rd_bp: clear");
    if (g->joseph) launch_rd<true, true>(*g, trig, sino, img, sc, st);
    else launch_rd<false, true>(*g, trig, sino, img, sc, st);
    return launch_status("rd_bp");
}

extern "C" int vg_pd_fp(const vg_ray_geom *g, const float *img, const double *trig, float *sino,
                        void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(img && trig && sino, "pd_fp: null pointer");
    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(sino, 0, sino_count(g) * sizeof(float), st);
    if (e != cudaSuccess) return cuda_status(e, "pd_fp: clear");
    if (g->kind == 2 && VG_PD_CONE_COLUMNS) {
        const int colx = ceil_div(g->nx, 2);
        dim3 grid(colx * ceil_div(g->ny, 4), ceil_div(g->nz, 32 * PD_ZPT), g->na);
        VG_REQUIRE(grid.y < 65536, "pd_fp: volume too large");
        pd_fp_cone_kernel<<<grid, 256, 0, st>>>(*g, trig, img, sino, colx);
        return launch_status("pd_fp");
    }
    if (g->kind < 2 && PD_RUN > 1) {
        dim3 grid(ceil_div((long long)g->nx * ceil_div(g->ny, PD_RUN), 256), g->na);
        pd_fp_run_kernel<<<grid, 256, 0, st>>>(*g, trig, img, sino);
        return launch_status("pd_fp");
    }
    dim3 grid(ceil_div((long long)g->nx * g->ny, 256), g->na);
    pd_fp_kernel<<<grid, 256, 0, st>>>(*g, trig, img, sino);
    return launch_status("pd_fp");
}

extern "C" int vg_pd_bp(const vg_ray_geom *g, const float *sino, const double *trig, float *img,
                        void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(img && trig && sino, "pd_bp: null pointer");
    // img / na / d_pix * du (pd.py:232); cone * dv (pd.py:479)
    float sc = g->du / ((float)g->na * g->d_pix);
    if (g->kind == 2) sc *= g->dv;
    if (g->kind == 2 && VG_PD_CONE_COLUMNS) {
        dim3 grid(ceil_div(g->nx, 2), ceil_div(g->ny, 4), ceil_div(g->nz, 32 * PD_ZPT));
        VG_REQUIRE(grid.y < 65536 && grid.z < 65536, "pd_bp: volume too large");
        pd_bp_cone_kernel<<<grid, 256, 0, as_stream(stream)>>>(*g, trig, sino, img, sc);
        return launch_status("pd_bp");
    }
    const long long n = (long long)img_count(g);
    VG_REQUIRE(ceil_div(n, 256) < 2147483647LL, "pd_bp: volume too large");
    pd_bp_kernel<<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(*g, trig, sino, img, sc);
    return launch_status("pd_bp");
}
