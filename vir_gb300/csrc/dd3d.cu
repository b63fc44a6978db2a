// 3D cone-beam distance-driven projector pair, gather form.
//
// vir's cone sweep (sys_mat/dd.py:285-468, geometry 589-645, wrappers
// 815-888) weights voxel (k along the driving axis, line io, slice iz) into
// bin (iu, iv) by
//     scale(io) * |[P_k, P_k+1] ∩ [U_iu, U_iu+1]| * |zmag(io) [z_iz, z_iz+1] ∩ [V_iv, V_iv+1]|
// with P the fan projection of the driving edges on line io (as in 2D),
// zmag(io) = DSD / (DSO - o_centre(io)) and z_iz = d_pix (iz - nz/2); FP
// returns sino * d_pix^2 / (du dv), BP returns img / (na d_pix).  The u and v
// factors are separable per line, so each (bin, line) or (voxel, view) pair
// touches only the 1-3 pixels x 1-2 slices (or bins) its intervals overlap.
// (vir's FP reuses a stale u buffer across lines, dd.py:300,335; this is the
// overlap integral that sweep intends.)
//
//  dd3d_prep: per (view, line) the scale and z magnification (workspace).
//  FP: thread = (view, iu, iv), lanes along v; walks the lines; the pixels
//      under a bin come from the exact inverse of the edge projection.
//  BP: thread = voxel, lanes along z; walks the views.
#include "vg_common.cuh"

namespace {

using namespace vg;

struct View3 {
    float pd, od, po, oo, tabs;
    int xdrv;
};

__device__ __forceinline__ View3 view3(const double *trig, int ia) {
    View3 v;
    const float c = (float)__ldg(trig + 2 * ia), s = (float)__ldg(trig + 2 * ia + 1);
    v.xdrv = fabsf(s) >= fabsf(c);
    if (v.xdrv) { v.pd = -s; v.od = c; v.po = c; v.oo = s; v.tabs = fabsf(s); }
    else        { v.pd = c;  v.od = s; v.po = -s; v.oo = c; v.tabs = fabsf(c); }
    return v;
}

__device__ __forceinline__ float cen(float d, int i, int n) { return d * ((float)i + 0.5f - 0.5f * n); }
__device__ __forceinline__ float edg(float d, int i, int n) { return d * ((float)i - 0.5f * n); }

// Pole of the inverse edge map (u of rays parallel to the lines): whether it
// lies in [a, b].  It is outside every line's shadow, but a detector that
// reaches DSD from the centre can contain it; ranges found through the
// inverse map are then not trusted on an interval holding it.
__device__ __forceinline__ bool pole_in(const vg_dd3d_geom &g, const View3 &v, float a, float b) {
    if (v.od == 0.f) return false;
    const float Up = -g.DSD * v.pd / v.od;
    return Up >= fminf(a, b) && Up <= fmaxf(a, b);
}

__device__ __forceinline__ float projU(const vg_dd3d_geom &g, const View3 &v, float cp, float co,
                                       float b) {
    return __fdividef(g.DSD * fmaf(v.pd, b, cp), g.DSO - fmaf(v.od, b, co));
}

// Workspace: tab[na][max(nx, ny)] float2 (scale, zmag) per (view, line),
// then, 16-byte aligned, vf[na][2] float4 per view: (pd, od, po, oo) and
// (|trig|, xdrv, 0, 0), the float view geometry of view3.
size_t tab_bytes(const vg_dd3d_geom *g) {
    const int nm = g->nx > g->ny ? g->nx : g->ny;
    return ((size_t)g->na * nm * 2 * sizeof(float) + 15) & ~(size_t)15;
}

size_t ws_bytes(const vg_dd3d_geom *g) { return tab_bytes(g) + (size_t)g->na * 2 * sizeof(float4); }

__device__ __forceinline__ View3 view_f(const float4 *__restrict__ vf, int ia) {
    const float4 a = vf[2 * ia], b = vf[2 * ia + 1];
    View3 v;
    v.pd = a.x; v.od = a.y; v.po = a.z; v.oo = a.w; v.tabs = b.x; v.xdrv = b.y != 0.f;
    return v;
}

// tab[ia][io] = (scale, zmag); vf[ia] = float view geometry
__global__ void dd3d_prep(vg_dd3d_geom g, const double *__restrict__ trig, float2 *__restrict__ tab,
                          float4 *__restrict__ vf) {
    const int ia = blockIdx.x;
    const View3 v = view3(trig, ia);
    const int no = v.xdrv ? g.ny : g.nx;
    const int nm = g.nx > g.ny ? g.nx : g.ny;
    if (threadIdx.x == 0) {
        vf[2 * ia] = make_float4(v.pd, v.od, v.po, v.oo);
        vf[2 * ia + 1] = make_float4(v.tabs, v.xdrv ? 1.f : 0.f, 0.f, 0.f);
    }
    for (int io = threadIdx.x; io < no; io += blockDim.x) {
        const float c = cen(g.d_pix, io, no);
        const float cp = v.po * c, co = v.oo * c;
        const float a = g.DSO - co;
        tab[(size_t)ia * nm + io] = make_float2(sqrtf(a * a + cp * cp) / (a * v.tabs), g.DSD / a);
    }
}

__device__ __forceinline__ float ufloor_edge(const vg_dd3d_geom &g, int j) {
    return g.du * ((float)j - 0.5f * g.nu + g.su);
}
__device__ __forceinline__ float vfloor_edge(const vg_dd3d_geom &g, int j) {
    return g.dv * ((float)j - 0.5f * g.nv + g.sv);
}

// One cell's share of one line, straight from global memory (any geometry).
__device__ __noinline__ float fp_cell_line(const vg_dd3d_geom &g, const View3 &v, const float *__restrict__ vol,
                              size_t sk, size_t so, int nd, int io, float cp, float co, float zmag,
                              float Ul, float Ur, float Vl, float Vr) {
    const float inv_d = 1.0f / g.d_pix;
    const float rl = 1.0f / (g.DSD * v.pd + Ul * v.od), rr = 1.0f / (g.DSD * v.pd + Ur * v.od);
    const float kl = fmaf(Ul, g.DSO - co, -g.DSD * cp) * rl * inv_d + 0.5f * nd;
    const float kr = fmaf(Ur, g.DSO - co, -g.DSD * cp) * rr * inv_d + 0.5f * nd;
    const bool pole = pole_in(g, v, Ul, Ur);
    const int k0 = pole ? 0 : max(0, (int)floorf(fminf(kl, kr)));
    const int k1 = pole ? nd - 1 : min(nd - 1, (int)floorf(fmaxf(kl, kr)));
    const float izl = Vl / (zmag * g.d_pix) + 0.5f * g.nz;
    const float izr = Vr / (zmag * g.d_pix) + 0.5f * g.nz;
    const int z0 = max(0, (int)floorf(izl)), z1 = min(g.nz - 1, (int)floorf(izr));
    float part = 0.f;
    if (k0 > k1 || z0 > z1) return part;
    float pa = projU(g, v, cp, co, edg(g.d_pix, k0, nd));
    for (int k = k0; k <= k1; ++k) {
        const float pb = projU(g, v, cp, co, edg(g.d_pix, k + 1, nd));
        const float ou = fminf(fmaxf(pa, pb), Ur) - fmaxf(fminf(pa, pb), Ul);
        pa = pb;
        if (ou <= 0.f) continue;
        const float *col = vol + k * sk + io * so;
        float colsum = 0.f;
        for (int iz = z0; iz <= z1; ++iz) {
            const float zl = zmag * edg(g.d_pix, iz, g.nz), zr = zmag * edg(g.d_pix, iz + 1, g.nz);
            const float ov = fminf(zr, Vr) - fmaxf(zl, Vl);
            if (ov > 0.f) colsum = fmaf(__ldg(col + iz), ov, colsum);
        }
        part = fmaf(colsum, ou, part);
    }
    return part;
}

// Forward projection, tiled.  Block = (view, FT_U u-cells x FT_V v-cells);
// thread = 4 adjacent u-cells (warp) x 2 v-cells (lane, lane + 32).  For
// each line io whose shadow meets the tile, the block tabulates in shared
// memory the overlap weights of its cells: per u-cell the first pixel and
// 3 u-overlaps times the line scale, per v-cell the first slice and 3
// v-overlaps (the same float expressions as the backprojector).  Each cell
// then sums 3 x 3 voxels of the line (L1-cached reads; lanes on
// consecutive slices).  Lines where a cell overlaps more than 3 pixels or
// slices take the per-cell global path.  The tables are double-buffered by
// line parity, so one barrier per line suffices.  Line sums are added in
// groups of FT_GROUP lines and the group sums in a second running sum.
constexpr int FT_U = 32, FT_V = 64;
constexpr int FT_GROUP = 16;

struct FpTables {
    float4 uw[2][FT_U];  // per u-cell: weights of pixels k, k+1, k+2 (x line scale)
    int uk[2][FT_U];
    float4 vw[2][FT_V];  // per v-cell: weights of slices z, z+1, z+2
    int vz[2][FT_V];
    int wide[2];
};

// One line's share of a thread's 4 u-cells x 2 v-cells: 1-3 pixel rows
// (trailing rows with zero weight are skipped; the u-cell, hence the branch,
// is the same for the whole warp; a zero row before a weighted one, at the
// volume's far edge, is kept) x NV slices.
template <int NV>
__device__ __forceinline__ void fp_cells(const float4 *uw, const int *uk, const float *line,
                                         size_t sk, float4 wa, float4 wb, int za, int zb,
                                         float part[8]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float4 wu = uw[j];
        const float *r = line + (size_t)uk[j] * sk;
        const int nrow = wu.z != 0.f ? 3 : (wu.y != 0.f ? 2 : 1);
        float ca = 0.f, cb = 0.f;
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            if (t >= nrow) break;
            const float *q = r + t * sk;
            float sa, sb;
            if (NV == 3) {
                sa = fmaf(wa.x, __ldg(q + za), fmaf(wa.y, __ldg(q + za + 1), wa.z * __ldg(q + za + 2)));
                sb = fmaf(wb.x, __ldg(q + zb), fmaf(wb.y, __ldg(q + zb + 1), wb.z * __ldg(q + zb + 2)));
            } else {
                sa = fmaf(wa.x, __ldg(q + za), wa.y * __ldg(q + za + 1));
                sb = fmaf(wb.x, __ldg(q + zb), wb.y * __ldg(q + zb + 1));
            }
            const float wt = t == 0 ? wu.x : (t == 1 ? wu.y : wu.z);
            ca = fmaf(wt, sa, ca);
            cb = fmaf(wt, sb, cb);
        }
        part[2 * j] = ca;
        part[2 * j + 1] = cb;
    }
}

#ifndef VG_CONE_FP_MINB
#define VG_CONE_FP_MINB 3
#endif
template <int MODE>  // 0: projection; 1: SIRT residual epilogue
__global__ void __launch_bounds__(256, VG_CONE_FP_MINB)
dd3d_fp_kernel(vg_dd3d_geom g, const float *__restrict__ vol, const float4 *__restrict__ vf,
               const float2 *__restrict__ tab, float *__restrict__ sino,
               const float *__restrict__ y, const float *__restrict__ inv_w) {
    __shared__ FpTables S;
    const int ia = blockIdx.z;
    const int u0 = blockIdx.y * FT_U, v0 = blockIdx.x * FT_V;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const View3 v = view_f(vf, ia);
    const int nd = v.xdrv ? g.nx : g.ny;
    const int no = v.xdrv ? g.ny : g.nx;
    const int nm = g.nx > g.ny ? g.nx : g.ny;
    const size_t sk = v.xdrv ? (size_t)g.ny * g.nz : (size_t)g.nz;  // stride of k
    const size_t so = v.xdrv ? (size_t)g.nz : (size_t)g.ny * g.nz;  // stride of io
    const float inv_d = 1.0f / g.d_pix;
    const int kmax = nd - 3, zmax = g.nz - 3;
    // the tile's outer edges and their inverse-map denominators
    const float TUl = ufloor_edge(g, u0), TUr = ufloor_edge(g, min(u0 + FT_U, g.nu));
    const float TVl = vfloor_edge(g, v0), TVr = vfloor_edge(g, min(v0 + FT_V, g.nv));
    const float rTl = 1.0f / (g.DSD * v.pd + TUl * v.od), rTr = 1.0f / (g.DSD * v.pd + TUr * v.od);
    const bool tile_pole = pole_in(g, v, TUl, TUr);
    // table threads: tid < FT_U owns u-cell u0 + tid, FT_U <= tid < FT_U + FT_V a v-cell
    const int wu_i = u0 + tid, wv_i = v0 + tid - FT_U;
    const bool is_u = tid < FT_U && wu_i < g.nu;
    const bool is_v = tid >= FT_U && tid < FT_U + FT_V && wv_i < g.nv;
    float cUl = 0.f, cUr = 0.f, crl = 0.f, crr = 0.f, cVl = 0.f, cVr = 0.f;
    if (is_u) {
        cUl = ufloor_edge(g, wu_i); cUr = ufloor_edge(g, wu_i + 1);
        crl = 1.0f / (g.DSD * v.pd + cUl * v.od); crr = 1.0f / (g.DSD * v.pd + cUr * v.od);
    }
    if (is_v) { cVl = vfloor_edge(g, wv_i); cVr = vfloor_edge(g, wv_i + 1); }
    const bool cell_pole = is_u && pole_in(g, v, cUl, cUr);
    const bool small = nd < 3 || g.nz < 3;

    float acc[8], grp[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = grp[c] = 0.f;
    int ngrp = 0, nl = 0;
    // S.wide[b] == io + 1 marks line io for the global path; writers only
    // ever store that marker, so no reset races with them
    if (tid < 2) S.wide[tid] = -1;
    __syncthreads();
    for (int io = 0; io < no; ++io) {
        const float c = cen(g.d_pix, io, no);
        const float cp = v.po * c, co = v.oo * c;
        const float2 sz = __ldg(tab + (size_t)ia * nm + io);
        const float kl = fmaf(TUl, g.DSO - co, -g.DSD * cp) * rTl * inv_d + 0.5f * nd;
        const float kr = fmaf(TUr, g.DSO - co, -g.DSD * cp) * rTr * inv_d + 0.5f * nd;
        const int kA = tile_pole ? 0 : max(0, (int)floorf(fminf(kl, kr)));
        const int kB = tile_pole ? nd - 1 : min(nd - 1, (int)floorf(fmaxf(kl, kr)));
        const float izd = 1.0f / (sz.y * g.d_pix);
        const int zA = max(0, (int)floorf(TVl * izd + 0.5f * g.nz));
        const int zB = min(g.nz - 1, (int)floorf(TVr * izd + 0.5f * g.nz));
        if (kA > kB || zA > zB) continue;  // block-uniform
        const int b = nl++ & 1;
        if (tid < FT_U) {
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            int kb0 = 0;
            if (is_u) {
                const float a = fmaf(cUl, g.DSO - co, -g.DSD * cp) * crl * inv_d + 0.5f * nd;
                const float bb = fmaf(cUr, g.DSO - co, -g.DSD * cp) * crr * inv_d + 0.5f * nd;
                const int ks = (int)floorf(fminf(a, bb)), ke = (int)floorf(fmaxf(a, bb));
                if ((ke - ks > 2 && ke >= 0 && ks < nd) || cell_pole) S.wide[b] = io + 1;
                kb0 = min(max(ks, 0), max(kmax, 0));
                float pa = projU(g, v, cp, co, edg(g.d_pix, kb0, nd));
                float ow[3];
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    const float pb = projU(g, v, cp, co, edg(g.d_pix, kb0 + t + 1, nd));
                    const float o = fminf(fmaxf(pa, pb), cUr) - fmaxf(fminf(pa, pb), cUl);
                    ow[t] = (kb0 + t < nd && o > 0.f) ? o * sz.x : 0.f;
                    pa = pb;
                }
                w = make_float4(ow[0], ow[1], ow[2], 0.f);
            }
            S.uw[b][tid] = w;
            S.uk[b][tid] = kb0;
        } else if (tid < FT_U + FT_V) {
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            int zb0 = 0;
            if (is_v) {
                const int zs = (int)floorf(cVl * izd + 0.5f * g.nz);
                const int ze = (int)floorf(cVr * izd + 0.5f * g.nz);
                if (ze - zs > 2 && ze >= 0 && zs < g.nz) S.wide[b] = io + 1;
                zb0 = min(max(zs, 0), max(zmax, 0));
                float ow[3];
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    const float zl = sz.y * edg(g.d_pix, zb0 + t, g.nz);
                    const float zr = sz.y * edg(g.d_pix, zb0 + t + 1, g.nz);
                    const float o = fminf(zr, cVr) - fmaxf(zl, cVl);
                    ow[t] = (zb0 + t < g.nz && o > 0.f) ? o : 0.f;
                }
                w = make_float4(ow[0], ow[1], ow[2], 0.f);
            }
            S.vw[b][tid - FT_U] = w;
            S.vz[b][tid - FT_U] = zb0;
        }
        __syncthreads();
        float part[8];
        if (S.wide[b] != io + 1 && !small) {
            const float4 wa = S.vw[b][lane], wb = S.vw[b][32 + lane];
            const int za = S.vz[b][lane], zb = S.vz[b][32 + lane];
            const float *line = vol + (size_t)io * so;
            // when no cell of the warp weights a third slice (slices project
            // at least a cell high), the third read and its zero term go
            if (__all_sync(0xffffffffu, wa.z == 0.f && wb.z == 0.f))
                fp_cells<2>(S.uw[b] + 4 * warp, S.uk[b] + 4 * warp, line, sk, wa, wb, za, zb, part);
            else
                fp_cells<3>(S.uw[b] + 4 * warp, S.uk[b] + 4 * warp, line, sk, wa, wb, za, zb, part);
        } else {
#pragma unroll 1
            for (int j = 0; j < 4; ++j) {
                const int iu = u0 + 4 * warp + j;
                const float Ul = ufloor_edge(g, iu), Ur = ufloor_edge(g, iu + 1);
#pragma unroll 1
                for (int h = 0; h < 2; ++h) {
                    const int iv = v0 + 32 * h + lane;
                    part[2 * j + h] = (iu < g.nu && iv < g.nv)
                        ? sz.x * fp_cell_line(g, v, vol, sk, so, nd, io, cp, co, sz.y, Ul, Ur,
                                              vfloor_edge(g, iv), vfloor_edge(g, iv + 1))
                        : 0.f;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) grp[q] += part[q];
        if (++ngrp == FT_GROUP) {
#pragma unroll
            for (int q = 0; q < 8; ++q) { acc[q] += grp[q]; grp[q] = 0.f; }
            ngrp = 0;
        }
    }
    const float f = g.d_pix * g.d_pix / (g.du * g.dv);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int iu = u0 + 4 * warp + j;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int iv = v0 + 32 * h + lane;
            acc[2 * j + h] += grp[2 * j + h];
            if (iu < g.nu && iv < g.nv) {
                const size_t o = ((size_t)ia * g.nu + iu) * g.nv + iv;
                float fp = acc[2 * j + h] * f;
                if (MODE) {  // SIRT residual: (y - FP) / W_sino, FP kept where W_sino == 0
                    const float wi = inv_w[o];
                    fp = (wi != 0.f) ? (y[o] - fp) * wi : fp;
                }
                sino[o] = fp;
            }
        }
    }
}

// Backprojection, tiled.  Block = 8 x 8 columns (x, y) x 32 slices; thread =
// one slice z (lane) of one y row (warp), 8 voxels along x.  Per view the
// block first tabulates in shared memory the overlap weights every voxel
// needs: per column (its pixel on its line) the first detector column and
// 3 u-overlaps times the line scale, per (line, slice) the first detector
// row and 3 v-overlaps -- the same float expressions as the forward
// projector.  Each voxel then sums 3 x 3 sinogram cells (L1-cached reads,
// lanes on consecutive rows of one column).  Views whose voxels overlap more
// than 3 cells along u or v take the per-voxel global path.  The tables are
// double-buffered, so one barrier per view suffices.
constexpr int BT = 8, BZ = 32;

struct BpTables {
    float4 uw[2][BT * BT];  // per column (cx + 8 cy): weights of cells j, j+1, j+2 (x scale)
    int uj[2][BT * BT];
    float4 vw[2][BT][BZ];   // per (line in tile, slice): weights of rows q, q+1, q+2
    int vq[2][BT][BZ];
    int wide[2];
};

__device__ float bp_voxel_view(const vg_dd3d_geom &g, const View3 &v, const float *__restrict__ s,
                               float2 sz, int k, int nd, float cp, float co, int iz) {
    const float u0 = ufloor_edge(g, 0), v0 = vfloor_edge(g, 0);
    const float idu = 1.0f / g.du, idv = 1.0f / g.dv;
    const float pa = projU(g, v, cp, co, edg(g.d_pix, k, nd));
    const float pb = projU(g, v, cp, co, edg(g.d_pix, k + 1, nd));
    const float ulo = fminf(pa, pb), uhi = fmaxf(pa, pb);
    const float vlo = sz.y * edg(g.d_pix, iz, g.nz), vhi = sz.y * edg(g.d_pix, iz + 1, g.nz);
    const int j0 = max(0, (int)floorf((ulo - u0) * idu)), j1 = min(g.nu - 1, (int)floorf((uhi - u0) * idu));
    const int q0 = max(0, (int)floorf((vlo - v0) * idv)), q1 = min(g.nv - 1, (int)floorf((vhi - v0) * idv));
    float part = 0.f;
    for (int j = j0; j <= j1; ++j) {
        const float ou = fminf(uhi, ufloor_edge(g, j + 1)) - fmaxf(ulo, ufloor_edge(g, j));
        if (ou <= 0.f) continue;
        float rs = 0.f;
        for (int q = q0; q <= q1; ++q) {
            const float ov = fminf(vhi, vfloor_edge(g, q + 1)) - fmaxf(vlo, vfloor_edge(g, q));
            if (ov > 0.f) rs = fmaf(__ldg(s + (size_t)j * g.nv + q), ov, rs);
        }
        part = fmaf(rs, ou, part);
    }
    return part * sz.x;
}

#ifndef VG_CONE_BP_MINB
#define VG_CONE_BP_MINB 5
#endif
template <int MODE>  // 0: back projection; 1: SIRT update epilogue
__global__ void __launch_bounds__(256, VG_CONE_BP_MINB)
dd3d_bp_kernel(vg_dd3d_geom g, const float *__restrict__ sino, const float4 *__restrict__ vf,
               const float2 *__restrict__ tab, float *__restrict__ vol,
               const float *__restrict__ inv_w, float gamma) {
    __shared__ BpTables T;
    const int z0 = blockIdx.x * BZ, y0 = blockIdx.y * BT, x0 = blockIdx.z * BT;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int iz = z0 + lane, iy = y0 + warp;  // this thread: voxels (x0 + i, iy, iz), i < 8
    const int nm = g.nx > g.ny ? g.nx : g.ny;
    const float u0 = ufloor_edge(g, 0), v0 = vfloor_edge(g, 0);
    const float idu = 1.0f / g.du, idv = 1.0f / g.dv;
    const int jmax = g.nu - 3, qmax = g.nv - 3;
    Kahan acc[BT];
    float grp[BT];
#pragma unroll
    for (int i = 0; i < BT; ++i) grp[i] = 0.f;
    int ngrp = 0;
    // T.wide[b] == ia + 1 marks view ia for the per-voxel path; writers only
    // ever store that marker, so no reset races with them
    if (tid < 2) T.wide[tid] = -1;
    __syncthreads();
    for (int ia = 0; ia < g.na; ++ia) {
        const int b = ia & 1;
        const View3 v = view_f(vf, ia);
        const int nd = v.xdrv ? g.nx : g.ny, no = v.xdrv ? g.ny : g.nx;
        const int k0 = v.xdrv ? x0 : y0, io0 = v.xdrv ? y0 : x0;  // tile origin in (k, io)
        // v table: thread (line l = warp, slice lane)
        {
            const int io = io0 + warp;
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            int qb = 0;
            if (io < no && iz < g.nz) {
                const float zmag = __ldg(tab + (size_t)ia * nm + io).y;
                const float vlo = zmag * edg(g.d_pix, iz, g.nz), vhi = zmag * edg(g.d_pix, iz + 1, g.nz);
                const int qs = (int)floorf((vlo - v0) * idv), qe = (int)floorf((vhi - v0) * idv);
                if (qe - qs > 2) T.wide[b] = ia + 1;
                qb = min(max(qs, 0), max(qmax, 0));
                float ow[3];
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    const float o = fminf(vhi, vfloor_edge(g, qb + t + 1)) - fmaxf(vlo, vfloor_edge(g, qb + t));
                    ow[t] = (qb + t < g.nv && o > 0.f) ? o : 0.f;
                }
                w = make_float4(ow[0], ow[1], ow[2], 0.f);
            }
            T.vw[b][warp][lane] = w;
            T.vq[b][warp][lane] = qb;
        }
        // u table: thread c < 64 owns column (k0 + c % 8, line io0 + c / 8)
        if (tid < BT * BT) {
            const int k = k0 + (tid & 7), io = io0 + (tid >> 3);
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            int jb = 0;
            if (k < nd && io < no) {
                const float c = cen(g.d_pix, io, no);
                const float cp = v.po * c, co = v.oo * c;
                const float scale = __ldg(tab + (size_t)ia * nm + io).x;
                const float pa = projU(g, v, cp, co, edg(g.d_pix, k, nd));
                const float pb = projU(g, v, cp, co, edg(g.d_pix, k + 1, nd));
                const float ulo = fminf(pa, pb), uhi = fmaxf(pa, pb);
                const int js = (int)floorf((ulo - u0) * idu), je = (int)floorf((uhi - u0) * idu);
                if (je - js > 2) T.wide[b] = ia + 1;
                jb = min(max(js, 0), max(jmax, 0));
                float ow[3];
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    const float o = fminf(uhi, ufloor_edge(g, jb + t + 1)) - fmaxf(ulo, ufloor_edge(g, jb + t));
                    ow[t] = (jb + t < g.nu && o > 0.f) ? o * scale : 0.f;
                }
                w = make_float4(ow[0], ow[1], ow[2], 0.f);
            }
            T.uw[b][tid] = w;
            T.uj[b][tid] = jb;
        }
        __syncthreads();
        const float *s = sino + (size_t)ia * g.nu * g.nv;
        float part[BT];
        if (T.wide[b] != ia + 1 && g.nu >= 3 && g.nv >= 3) {
#pragma unroll
            for (int i = 0; i < BT; ++i) {
                // voxel (x0 + i, iy, iz) is column (k, io) = xdrv ? (x, y) : (y, x)
                const int c = v.xdrv ? (i + BT * warp) : (warp + BT * i);
                const int l = v.xdrv ? warp : i;
                const float4 wu = T.uw[b][c];
                const float4 wv = T.vw[b][l][lane];
                const float *r = s + (size_t)T.uj[b][c] * g.nv + T.vq[b][l][lane];
                // trailing cell rows with zero weight are skipped (the column,
                // hence the branch, is the same for the whole warp; a zero row
                // before a weighted one, at the detector's far edge, is kept)
                const int nrow = wu.z != 0.f ? 3 : (wu.y != 0.f ? 2 : 1);
                float acc3 = wu.x * fmaf(wv.x, __ldg(r), fmaf(wv.y, __ldg(r + 1), wv.z * __ldg(r + 2)));
                if (nrow > 1) {
                    r += g.nv;
                    acc3 = fmaf(wu.y, fmaf(wv.x, __ldg(r), fmaf(wv.y, __ldg(r + 1), wv.z * __ldg(r + 2))), acc3);
                    if (nrow > 2) {
                        r += g.nv;
                        acc3 = fmaf(wu.z, fmaf(wv.x, __ldg(r), fmaf(wv.y, __ldg(r + 1), wv.z * __ldg(r + 2))),
                                    acc3);
                    }
                }
                part[i] = acc3;
            }
        } else {
#pragma unroll 1
            for (int i = 0; i < BT; ++i) {
                const int ix = x0 + i;
                part[i] = 0.f;
                if (ix < g.nx && iy < g.ny && iz < g.nz) {
                    const int k = v.xdrv ? ix : iy, io = v.xdrv ? iy : ix;
                    const float c = cen(g.d_pix, io, no);
                    part[i] = bp_voxel_view(g, v, s, __ldg(tab + (size_t)ia * nm + io), k, nd,
                                            v.po * c, v.oo * c, iz);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < BT; ++i) grp[i] += part[i];
        if (++ngrp == FT_GROUP) {
#pragma unroll
            for (int i = 0; i < BT; ++i) { acc[i].add(grp[i]); grp[i] = 0.f; }
            ngrp = 0;
        }
    }
    const float f = 1.0f / ((float)g.na * g.d_pix);
#pragma unroll
    for (int i = 0; i < BT; ++i) {
        acc[i].add(grp[i]);
        const int ix = x0 + i;
        if (ix < g.nx && iy < g.ny && iz < g.nz) {
            const size_t o = ((size_t)ix * g.ny + iy) * g.nz + iz;
            const float bp = acc[i].s * f;
            if (MODE) {  // SIRT update: x += gamma BP / W_img, BP where W_img == 0
                const float wi = inv_w[o];
                vol[o] += gamma * ((wi != 0.f) ? bp * wi : bp);
            } else {
                vol[o] = bp;
            }
        }
    }
}

int check(const vg_dd3d_geom *g) {
    VG_REQUIRE(g, "dd3d: null geometry");
    VG_REQUIRE(g->nx > 0 && g->ny > 0 && g->nz > 0 && g->na > 0 && g->nu > 0 && g->nv > 0,
               "dd3d: sizes must be positive");
    VG_REQUIRE(g->na < 65536 && g->nx < 65536 && ceil_div(g->nu, 8) < 65536 &&
                   ceil_div(g->ny, 8) < 65536, "dd3d: sizes too large for the grid");
    VG_REQUIRE(g->du > 0.f && g->dv > 0.f && g->d_pix > 0.f && g->DSO > 0.f && g->DSD > 0.f,
               "dd3d: pitches and distances must be positive");
    const float h = 0.5f * (float)(g->nx > g->ny ? g->nx : g->ny) * g->d_pix;
    VG_REQUIRE(h < 0.70710678f * g->DSO, "dd3d: volume half-width must be below DSO/sqrt(2)");
    return VG_OK;
}

int launch_prep(const vg_dd3d_geom *g, const double *trig, void *ws, size_t wsb, cudaStream_t st) {
    VG_REQUIRE(ws && wsb >= ws_bytes(g) && ((uintptr_t)ws & 15) == 0,
               "dd3d: workspace of %zu bytes needed (vg_dd3d_workspace_bytes)", ws_bytes(g));
    dd3d_prep<<<g->na, 256, 0, st>>>(*g, trig, reinterpret_cast<float2 *>(ws),
                                     reinterpret_cast<float4 *>(static_cast<char *>(ws) +
                                                                tab_bytes(g)));
    return launch_status("dd3d_prep");
}

}  // namespace

extern "C" size_t vg_dd3d_workspace_bytes(const vg_dd3d_geom *g) {
    return check(g) ? 0 : ws_bytes(g);
}

extern "C" int vg_dd3d_fp(const vg_dd3d_geom *g, const float *vol, const double *trig,
                          float *sino, void *workspace, size_t workspace_bytes, void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(vol && trig && sino, "dd3d_fp: null pointer");
    cudaStream_t st = as_stream(stream);
    s = launch_prep(g, trig, workspace, workspace_bytes, st);
    if (s) return s;
    dim3 grid(ceil_div(g->nv, FT_V), ceil_div(g->nu, FT_U), g->na);
    dd3d_fp_kernel<0><<<grid, 256, 0, st>>>(
        *g, vol,
        reinterpret_cast<const float4 *>(static_cast<const char *>(workspace) + tab_bytes(g)),
        reinterpret_cast<const float2 *>(workspace), sino, nullptr, nullptr);
    return launch_status("dd3d_fp");
}

extern "C" int vg_dd3d_bp(const vg_dd3d_geom *g, const float *sino, const double *trig,
                          float *vol, void *workspace, size_t workspace_bytes, void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(vol && trig && sino, "dd3d_bp: null pointer");
    cudaStream_t st = as_stream(stream);
    s = launch_prep(g, trig, workspace, workspace_bytes, st);
    if (s) return s;
    dim3 grid(ceil_div(g->nz, BZ), ceil_div(g->ny, BT), ceil_div(g->nx, BT));
    dd3d_bp_kernel<0><<<grid, 256, 0, st>>>(
        *g, sino,
        reinterpret_cast<const float4 *>(static_cast<const char *>(workspace) + tab_bytes(g)),
        reinterpret_cast<const float2 *>(workspace), vol, nullptr, 0.f);
    return launch_status("dd3d_bp");
}

extern "C" int vg_dd3d_sirt_iter(const vg_dd3d_geom *g, const float *y, const float *inv_w_sino,
                                 const float *inv_w_img, float gamma, const double *trig, float *x,
                                 float *r, void *workspace, size_t workspace_bytes, void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(y && inv_w_sino && inv_w_img && trig && x && r, "dd3d_sirt_iter: null pointer");
    cudaStream_t st = as_stream(stream);
    s = launch_prep(g, trig, workspace, workspace_bytes, st);
    if (s) return s;
    const float4 *vf = reinterpret_cast<const float4 *>(static_cast<const char *>(workspace) + tab_bytes(g));
    const float2 *tab = reinterpret_cast<const float2 *>(workspace);
    dim3 gf(ceil_div(g->nv, FT_V), ceil_div(g->nu, FT_U), g->na);
    dd3d_fp_kernel<1><<<gf, 256, 0, st>>>(*g, x, vf, tab, r, y, inv_w_sino);
    s = launch_status("dd3d_fp");
    if (s) return s;
    dim3 gb(ceil_div(g->nz, BZ), ceil_div(g->ny, BT), ceil_div(g->nx, BT));
    dd3d_bp_kernel<1><<<gb, 256, 0, st>>>(*g, r, vf, tab, x, inv_w_img, gamma);
    return launch_status("dd3d_bp");
}
