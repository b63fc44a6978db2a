// 3D cone-beam separable-footprint projector pair (SF-TR, amplitude A2).
//
// vir's sys_mat/sp.py:93-211 (CTGeometry, footprint1D, forward_project,
// back_project) sketches a separable-footprint cone projector without
// rotation angles.  This is the method it stands in for, the trapezoid /
// rectangle separable footprints of Long, Fessler & Balter, "3D forward and
// back-projection for X-ray CT using separable footprints", IEEE TMI 29(11),
// 2010, on vir's circular cone geometry of dd_fp_cone_3d (sys_mat/dd.py:815):
// source at DSO (cos b, sin b), o = c x + s y, p = -s x + c y,
// u = DSD p / (DSO - o), v = DSD z / (DSO - o); cell edges
// U_j = du (j - nu/2 + su), V_l = dv (l - nv/2 + sv); volume (nx, ny, nz) of
// cubic voxels d; sinogram (na, nu, nv), v fastest.  Voxel (x, y, z) adds
//     f * l_phi0 * l_theta(j, l) * F1(j) * F2(l)
// to cell (j, l), where
//   F1(j): the unit trapezoid through the sorted projections tau0..tau3 of
//          the column's four corners (x +- d/2, y +- d/2), averaged over u cell j;
//   F2(l): the rectangle [M (z - d/2), M (z + d/2)], M = DSD / (DSO - o(x, y)),
//          averaged over v cell l;
//   l_phi0 = d |r| / max(|r_x|, |r_y|), r = (x, y) - DSO (c, s): the path
//          length of the transaxial ray through the column centre;
//   l_theta(j, l) = sqrt(1 + v_l^2 / (u_j^2 + DSD^2)) at the cell centre.
// The forward projection returns these line integrals; the back projection
// is its exact adjoint (vir has no back projector for this footprint).
//
//  FP (sf3d_zprefix, sf3d_fp_kernel): the volume's per-column running sums
//    over z are formed first (workspace).  Block = (view, 32 u x 64 v cells),
//    thread = 4 u cells (warp) x 2 v cells (lanes).  For each orthogonal
//    pixel line whose columns reach the tile, the block tabulates in shared
//    memory the columns' footprints, the covering columns and F1 weights of
//    each u cell, and each column's v profile over the tile's v cells
//    g(c, l) = sum_z f(c, z) F2(l; c, z) as the running integral at the 65
//    v edges (the z sums interpolated at the edge's slice coordinate); each
//    cell then adds F1 * l_phi0 * (difference of its edges) over its 1-8
//    covering columns.  Lines where a u cell meets more columns, or the tile
//    more than 64, take a per-cell path.
//  BP (sf3d_bp_kernel): the sinogram is first multiplied by l_theta
//    (sf3d_weight, into the workspace, a chunk of views at a time); block =
//    8 x 8 columns x 32 slices, thread = one slice of 8 columns; per view a
//    table of the columns' u cells and F1 l_phi0 weights (at most 4 u cells
//    per column, else a per-voxel path), then each voxel gathers its 1-3 v
//    cells x 4 u cells.
#include "vg_common.cuh"

namespace {

using namespace vg;

__device__ __forceinline__ float2 view_cs(const double *__restrict__ trig, int ia) {
    return make_float2((float)__ldg(trig + 2 * ia), (float)__ldg(trig + 2 * ia + 1));
}

__device__ __forceinline__ float ucen(const vg_dd3d_geom &g, int j) {
    return g.du * ((float)j + 0.5f - 0.5f * g.nu + g.su);
}
__device__ __forceinline__ float uedge(const vg_dd3d_geom &g, int j) {
    return g.du * ((float)j - 0.5f * g.nu + g.su);
}
__device__ __forceinline__ float vedge(const vg_dd3d_geom &g, int l) {
    return g.dv * ((float)l - 0.5f * g.nv + g.sv);
}
__device__ __forceinline__ float vcen(const vg_dd3d_geom &g, int l) {
    return g.dv * ((float)l + 0.5f - 0.5f * g.nv + g.sv);
}
__device__ __forceinline__ float vox(float d, int i, int n) { return d * ((float)i + 0.5f - 0.5f * n); }

// Footprint of column (x, y): sorted corner projections, l_phi0 and the
// slice height on the detector M d.
struct SfCol {
    float t0, t1, t2, t3, lphi, mz, inv_mz;
};

__device__ __forceinline__ void cswap(float &a, float &b) {
    const float lo = fminf(a, b), hi = fmaxf(a, b);
    a = lo;
    b = hi;
}

__device__ __forceinline__ SfCol sf_col(const vg_dd3d_geom &g, float c, float s, float x, float y) {
    const float h = 0.5f * g.d_pix;
    float u[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float xx = x + ((q & 1) ? h : -h), yy = y + ((q & 2) ? h : -h);
        const float o = fmaf(c, xx, s * yy), p = fmaf(-s, xx, c * yy);
        u[q] = __fdividef(g.DSD * p, g.DSO - o);
    }
    cswap(u[0], u[1]);
    cswap(u[2], u[3]);
    cswap(u[0], u[2]);
    cswap(u[1], u[3]);
    cswap(u[1], u[2]);
    SfCol C;
    C.t0 = u[0]; C.t1 = u[1]; C.t2 = u[2]; C.t3 = u[3];
    const float rx = x - g.DSO * c, ry = y - g.DSO * s;
    C.lphi = __fdividef(g.d_pix * sqrtf(rx * rx + ry * ry), fmaxf(fabsf(rx), fabsf(ry)));
    C.mz = __fdividef(g.DSD * g.d_pix, g.DSO - fmaf(c, x, s * y));
    C.inv_mz = __fdividef(g.DSO - fmaf(c, x, s * y), g.DSD * g.d_pix);
    return C;
}

// Integral of the unit trapezoid (t0, t1, t2, t3) from -inf to u.
__device__ __forceinline__ float trap_cum(float u, const SfCol &C) {
    if (u <= C.t0) return 0.f;
    const float a = 0.5f * (C.t1 - C.t0);
    if (u <= C.t1) {
        const float e = u - C.t0;
        return __fdividef(e * e, 2.f * (C.t1 - C.t0));
    }
    if (u <= C.t2) return a + (u - C.t1);
    const float b = a + (C.t2 - C.t1);
    const float r = 0.5f * (C.t3 - C.t2);
    if (u <= C.t3) {
        const float e = C.t3 - u;
        return b + r - __fdividef(e * e, 2.f * (C.t3 - C.t2));
    }
    return b + r;
}

// F1 averaged over [ua, ub] (cell width du), times l_phi0
__device__ __forceinline__ float uweight(const SfCol &C, float ua, float ub, float inv_du) {
    return (trap_cum(ub, C) - trap_cum(ua, C)) * inv_du * C.lphi;
}

// sum_z f(z) |[M d (z - nz/2), M d (z + 1 - nz/2)] ∩ [va, vb]| / dv for one
// column (f at col, slices contiguous)
__device__ __forceinline__ float vprofile(const vg_dd3d_geom &g, const float *__restrict__ col,
                                          float mz, float inv_mz, float va, float vb, float inv_dv) {
    const float hz = 0.5f * g.nz;
    const float sa = fmaf(va, inv_mz, hz), sb = fmaf(vb, inv_mz, hz);
    const int z0 = max((int)floorf(sa), 0), z1 = min((int)floorf(sb), g.nz - 1);
    float acc = 0.f;
    for (int z = z0; z <= z1; ++z) {
        const float lo = fmaxf(va, mz * ((float)z - hz)), hi = fminf(vb, mz * ((float)z + 1.f - hz));
        const float ov = hi - lo;
        if (ov > 0.f) acc = fmaf(__ldg(col + z), ov, acc);
    }
    return acc * inv_dv;
}

// Fractional pixel index, along the driving axis, of the point of the line
// at orthogonal coordinate `cen` that projects to u (x, y = (b, cen) when
// X-driven, else (cen, b)):  b (DSD pd + u od) = u (DSO - oc) - DSD pc.
__device__ __forceinline__ float unproj_idx(const vg_dd3d_geom &g, float c, float s, bool xdrv,
                                            float cen, float u, int nd) {
    const float pd = xdrv ? -s : c, od = xdrv ? c : s;
    const float pc = xdrv ? c * cen : -s * cen, oc = xdrv ? s * cen : c * cen;
    const float b = __fdividef(u * (g.DSO - oc) - g.DSD * pc, g.DSD * pd + u * od);
    return __fdividef(b, g.d_pix) + 0.5f * nd;
}

// Per-column running sums over z for the forward projection's v profiles:
// zp[c][z] = sum_{z' < z} f(c, z') for z = 0 .. nz (column c = x ny + y),
// accumulated in FP64 and rounded once, so that a profile's edge value
// (an interpolation of zp) and the difference of two of them carry a
// rounding of the column's total, not of its summation.  One warp per column.
__global__ void __launch_bounds__(256)
sf3d_zprefix(vg_dd3d_geom g, const float *__restrict__ vol, float *__restrict__ zp) {
    const size_t col = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (col >= (size_t)g.nx * g.ny) return;
    const float *f = vol + col * g.nz;
    float *p = zp + col * (g.nz + 1);
    if (lane == 0) p[0] = 0.f;
    double carry = 0.0;
    for (int z0 = 0; z0 < g.nz; z0 += 32) {
        const int z = z0 + lane;
        double v = z < g.nz ? (double)__ldg(f + z) : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double t = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += t;
        }
        if (z < g.nz) p[z + 1] = (float)(carry + v);
        carry += __shfl_sync(0xffffffffu, v, 31);
    }
}

// ---------------------------------------------------------------------------
// Forward projection
// ---------------------------------------------------------------------------
constexpr int SU = 32, SV = 64, SCMAX = 64, SKMAX = 8, SLINES = 2048;

// per-line tables, double-buffered by line parity
struct SfFpTab {
    SfCol col[2][SCMAX];
    int poff[2][SCMAX];     // index of (column, z = 0) in the z-prefix array
    int cf[2][SU], cn[2][SU];  // covering columns (table index, count) per u cell
    float w[2][SU][SKMAX];  // F1 l_phi0 weights of those columns
    float gv[2][SCMAX][SV + 1];  // per column: the v profile's running integral at the v edges
    int2 kr[SLINES];        // per line: the range [x, y] of columns that can reach the tile
    float ve[SV + 1];       // the tile's v cell edges
    int wide[2];
};

// one cell's share of one line, straight from global memory (any geometry)
__device__ __noinline__ float sf_cell_line(const vg_dd3d_geom &g, const float *__restrict__ vol,
                                           float c, float s, bool xdrv, int nd, int no, int io,
                                           int kA, int kB, float Ua, float Ub, float Va, float Vb) {
    const float inv_du = 1.0f / g.du, inv_dv = 1.0f / g.dv;
    const float cen = vox(g.d_pix, io, no);
    float part = 0.f;
    for (int k = kA; k <= kB; ++k) {
        const float b = vox(g.d_pix, k, nd);
        const float x = xdrv ? b : cen, y = xdrv ? cen : b;
        const SfCol C = sf_col(g, c, s, x, y);
        if (C.t3 <= Ua || C.t0 >= Ub) continue;
        const float w = uweight(C, Ua, Ub, inv_du);
        if (w == 0.f) continue;
        const int ix = xdrv ? k : io, iy = xdrv ? io : k;
        part = fmaf(w, vprofile(g, vol + ((size_t)ix * g.ny + iy) * g.nz, C.mz, C.inv_mz, Va, Vb, inv_dv),
                    part);
    }
    return part;
}

__global__ void __launch_bounds__(256, 3)
sf3d_fp_kernel(vg_dd3d_geom g, const float *__restrict__ vol, const float *__restrict__ zp,
               const double *__restrict__ trig, float *__restrict__ sino) {
    __shared__ SfFpTab T;
    const int ia = blockIdx.z;
    const int u0 = blockIdx.y * SU, v0 = blockIdx.x * SV;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float2 cs = view_cs(trig, ia);
    const float c = cs.x, s = cs.y;
    const bool xdrv = fabsf(s) >= fabsf(c);
    const int nd = xdrv ? g.nx : g.ny, no = xdrv ? g.ny : g.nx;
    const float inv_du = 1.0f / g.du, inv_dv = 1.0f / g.dv;
    const int nuT = min(SU, g.nu - u0), nvT = min(SV, g.nv - v0);
    const float TUa = uedge(g, u0), TUb = uedge(g, u0 + nuT);
    // the inverse edge map has a pole at u = -DSD pd / od; a tile holding it
    // (or within two cells of it) cannot bound its columns through the map
    const float pd = xdrv ? -s : c, od = xdrv ? c : s;
    bool tile_pole = false;
    if (od != 0.f) {
        const float up = -g.DSD * pd / od;
        tile_pole = up >= TUa - 2.f * g.du && up <= TUb + 2.f * g.du;
    }
    // this thread's (u cell, slot) in the weight table
    const int wu = tid >> 3, wm = tid & 7;
    float acc[8], grp[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = grp[q] = 0.f;
    int ngrp = 0;
    if (tid < 2) T.wide[tid] = -1;
    if (tid <= SV) T.ve[tid] = vedge(g, v0 + tid);
    const float hz = 0.5f * g.nz, nzf = (float)g.nz;
    // columns of every line whose footprints can reach the tile, one line per
    // thread: the map of the tile's u edges (widened by a cell) on both
    // boundaries of the line, one column of margin each side
    for (int jo = tid; jo < no; jo += 256) {
        int kA = 0, kB = nd - 1;
        if (!tile_pole) {
            const float cj = vox(g.d_pix, jo, no), h = 0.5f * g.d_pix;
            const float a0 = unproj_idx(g, c, s, xdrv, cj - h, TUa - g.du, nd);
            const float a1 = unproj_idx(g, c, s, xdrv, cj + h, TUa - g.du, nd);
            const float b0 = unproj_idx(g, c, s, xdrv, cj - h, TUb + g.du, nd);
            const float b1 = unproj_idx(g, c, s, xdrv, cj + h, TUb + g.du, nd);
            const float lo = fminf(fminf(a0, a1), fminf(b0, b1));
            const float hi = fmaxf(fmaxf(a0, a1), fmaxf(b0, b1));
            kA = max((int)floorf(fmaxf(lo, -2.f)) - 1, 0);
            kB = min((int)floorf(fminf(hi, (float)nd + 2.f)) + 1, nd - 1);
        }
        T.kr[jo] = make_int2(kA, kB);
    }
    __syncthreads();
    // phase 1 of a line: its columns' footprints and z-prefix rows into buffer bb
    auto phase1 = [&](int io, int bb) {
        const int2 kr = T.kr[io];
        const int nk = kr.y - kr.x + 1;
        if (nk <= SCMAX && tid < nk) {
            const int k = kr.x + tid;
            const float cen = vox(g.d_pix, io, no), bx = vox(g.d_pix, k, nd);
            T.col[bb][tid] = sf_col(g, c, s, xdrv ? bx : cen, xdrv ? cen : bx);
            const int ix = xdrv ? k : io, iy = xdrv ? io : k;
            T.poff[bb][tid] = (ix * g.ny + iy) * (g.nz + 1);
        }
    };
    auto next_line = [&](int io) {
        do { ++io; } while (io < no && T.kr[io].x > T.kr[io].y);
        return io;
    };
    // One barrier per line: the block builds line io's covering columns,
    // weights and v profiles from buffer b together with the next line's
    // footprints into buffer b ^ 1, then after the barrier each cell adds
    // line io's columns.  Phase 3 of line io reads only phase-2 results of
    // buffer b, which the block next writes two lines later, after the
    // following line's barrier; T.wide[b] holds the index of the last wide
    // line of buffer b (writers only store that index).
    int io = next_line(-1), b = 0;
    if (io < no) phase1(io, 0);
    __syncthreads();
    for (; io < no; b ^= 1) {
        const int2 kr = T.kr[io];
        const int kA = kr.x, kB = kr.y;
        const int nk = kB - kA + 1;
        const bool big = nk > SCMAX;
        const int nxt = next_line(io);
        if (nxt < no) phase1(nxt, b ^ 1);
        if (!big) {
            // phase 2a: covering columns of each u cell (the footprints move
            // monotonically along the line, so they are consecutive; binary
            // searches on the footprints' ends) and their weights, one
            // (u cell, slot) per thread
            if (wu < nuT) {
                const float ua = uedge(g, u0 + wu), ub = uedge(g, u0 + wu + 1);
                const bool inc = T.col[b][nk - 1].t0 >= T.col[b][0].t0;
                // first covering: inc -> first t with t3 > ua; dec -> first t with t0 < ub
                int lo = 0, hi = nk;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    const bool past = inc ? (T.col[b][mid].t3 > ua) : (T.col[b][mid].t0 < ub);
                    if (past) hi = mid; else lo = mid + 1;
                }
                const int first = lo;
                // end (exclusive): inc -> first t with t0 >= ub; dec -> first t with t3 <= ua
                lo = first; hi = nk;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    const bool out = inc ? (T.col[b][mid].t0 >= ub) : (T.col[b][mid].t3 <= ua);
                    if (out) hi = mid; else lo = mid + 1;
                }
                const int n = lo - first;
                if (wm == 0) {
                    T.cf[b][wu] = first;
                    T.cn[b][wu] = min(n, SKMAX);
                    if (n > SKMAX) T.wide[b] = io;
                }
                if (wm < n && wm < SKMAX) T.w[b][wu][wm] = uweight(T.col[b][first + wm], ua, ub, inv_du);
            }
            // phase 2b: per column, the running integral of its v profile at the
            // tile's v edges: the column's z-prefix interpolated at the edge's
            // slice coordinate s = v / (M d) + nz/2, times M d / dv; a cell's
            // profile is the difference of its two edges
            for (int p = tid; p < nk * (SV + 1); p += 256) {
                const int t = p / (SV + 1), l = p - t * (SV + 1);
                float e = 0.f;
                if (l <= nvT) {
                    const float sz = fminf(fmaxf(fmaf(T.ve[l], T.col[b][t].inv_mz, hz), 0.f), nzf);
                    const float zf = fminf(floorf(sz), nzf - 1.f);
                    const float *pc = zp + T.poff[b][t] + (int)zf;
                    const float p0 = __ldg(pc), p1 = __ldg(pc + 1);
                    e = fmaf(p1 - p0, sz - zf, p0) * (T.col[b][t].mz * inv_dv);
                }
                T.gv[b][t][l] = e;
            }
        }
        __syncthreads();
        // phase 3: each cell adds its covering columns' weighted profiles
        float part[8];
        if (!big && T.wide[b] != io) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = 4 * warp + q;
                float pa = 0.f, pb = 0.f;
                if (j < nuT) {
                    const int f0 = T.cf[b][j], n = T.cn[b][j];
                    for (int m = 0; m < n; ++m) {
                        const float w = T.w[b][j][m];
                        const float *gr = T.gv[b][f0 + m];
                        pa = fmaf(w, gr[lane + 1] - gr[lane], pa);
                        pb = fmaf(w, gr[33 + lane] - gr[32 + lane], pb);
                    }
                }
                part[2 * q] = pa;
                part[2 * q + 1] = pb;
            }
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = u0 + 4 * warp + q;
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int l = v0 + 32 * hh + lane;
                    part[2 * q + hh] = (j < g.nu && l < g.nv)
                        ? sf_cell_line(g, vol, c, s, xdrv, nd, no, io, kA, kB, uedge(g, j),
                                       uedge(g, j + 1), vedge(g, l), vedge(g, l + 1))
                        : 0.f;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) grp[q] += part[q];
        if (++ngrp == 16) {
#pragma unroll
            for (int q = 0; q < 8; ++q) { acc[q] += grp[q]; grp[q] = 0.f; }
            ngrp = 0;
        }
        io = nxt;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int j = u0 + 4 * warp + q;
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            const int l = v0 + 32 * hh + lane;
            if (j < g.nu && l < g.nv) {
                const float uc = ucen(g, j), vc = vcen(g, l);
                const float lth = sqrtf(1.f + vc * vc / (uc * uc + g.DSD * g.DSD));
                sino[((size_t)ia * g.nu + j) * g.nv + l] = (acc[2 * q + hh] + grp[2 * q + hh]) * lth;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Back projection
// ---------------------------------------------------------------------------

// out[a - a0] = sino[a] * l_theta, views a0 .. a0 + cnt - 1
__global__ void sf3d_weight(vg_dd3d_geom g, const float *__restrict__ sino, int a0, int cnt,
                            float *__restrict__ out) {
    const size_t n = (size_t)cnt * g.nu * g.nv;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(i % g.nv);
        const int j = (int)((i / g.nv) % g.nu);
        const float uc = ucen(g, j), vc = vcen(g, l);
        const float lth = sqrtf(1.f + vc * vc / (uc * uc + g.DSD * g.DSD));
        out[i] = sino[(size_t)a0 * g.nu * g.nv + i] * lth;
    }
}

constexpr int BT = 8, BZ = 32, BKU = 4;

struct SfBpTab {
    float4 w[2][BT * BT];   // F1 l_phi0 of u cells j0 .. j0 + 3
    int j0[2][BT * BT];
    float mz[2][BT * BT];
    int wide[2];
};

// one voxel, one view, straight from the weighted sinogram (any geometry)
__device__ __noinline__ float sf_voxel_view(const vg_dd3d_geom &g, const float *__restrict__ q,
                                            float c, float s, float x, float y, int iz) {
    const SfCol C = sf_col(g, c, s, x, y);
    const float inv_du = 1.0f / g.du, inv_dv = 1.0f / g.dv;
    const float U0 = uedge(g, 0), V0 = vedge(g, 0);
    const int ja = max((int)floorf((C.t0 - U0) * inv_du), 0);
    const int jb = min((int)floorf((C.t3 - U0) * inv_du), g.nu - 1);
    const float va = C.mz * ((float)iz - 0.5f * g.nz), vb = va + C.mz;
    const int la = max((int)floorf((va - V0) * inv_dv), 0);
    const int lb = min((int)floorf((vb - V0) * inv_dv), g.nv - 1);
    float part = 0.f;
    for (int j = ja; j <= jb; ++j) {
        const float w = uweight(C, uedge(g, j), uedge(g, j + 1), inv_du);
        if (w == 0.f) continue;
        float r = 0.f;
        for (int l = la; l <= lb; ++l) {
            const float ov = fminf(vb, vedge(g, l + 1)) - fmaxf(va, vedge(g, l));
            if (ov > 0.f) r = fmaf(__ldg(q + (size_t)j * g.nv + l), ov, r);
        }
        part = fmaf(w, r, part);
    }
    return part * inv_dv;
}

// the 8 voxels x0 .. x0 + 7 of row iy, slice iz (0 beyond the volume)
__device__ __noinline__ void sf_voxels_view(const vg_dd3d_geom &g, const float *__restrict__ q, float c,
                                            float s, int x0, int iy, int iz, float *out) {
    for (int i = 0; i < BT; ++i) {
        const int ix = x0 + i;
        out[i] = ix < g.nx ? sf_voxel_view(g, q, c, s, vox(g.d_pix, ix, g.nx), vox(g.d_pix, iy, g.ny), iz)
                           : 0.f;
    }
}

__global__ void __launch_bounds__(256, 4)
sf3d_bp_kernel(vg_dd3d_geom g, const float *__restrict__ qw, const double *__restrict__ trig, int a0,
               int cnt, int accumulate, float *__restrict__ vol) {
    __shared__ SfBpTab T;
    const int z0 = blockIdx.x * BZ, y0 = blockIdx.y * BT, x0 = blockIdx.z * BT;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int iz = z0 + lane, iy = y0 + warp;
    const float inv_du = 1.0f / g.du, inv_dv = 1.0f / g.dv;
    const float U0 = uedge(g, 0), V0 = vedge(g, 0);
    const float hz = 0.5f * g.nz;
    Kahan acc[BT];
    float grp[BT];
#pragma unroll
    for (int i = 0; i < BT; ++i) grp[i] = 0.f;
    int ngrp = 0;
    // T.wide[b] == a marks view a for the per-voxel path; writers only ever
    // store that marker, so no reset races with them
    if (tid < 2) T.wide[tid] = -1;
    __syncthreads();
    for (int a = 0; a < cnt; ++a) {
        const int b = a & 1;
        const float2 cs = view_cs(trig, a0 + a);
        if (tid < BT * BT) {
            const int ix = x0 + (tid & 7), jy = y0 + (tid >> 3);
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            int j0 = 0;
            float mz = 1.f;
            if (ix < g.nx && jy < g.ny) {
                const SfCol C = sf_col(g, cs.x, cs.y, vox(g.d_pix, ix, g.nx), vox(g.d_pix, jy, g.ny));
                const int ja = (int)floorf((C.t0 - U0) * inv_du), jb = (int)floorf((C.t3 - U0) * inv_du);
                if (jb - ja >= BKU && jb >= 0 && ja < g.nu) T.wide[b] = a;
                j0 = ja;
                float ww[BKU];
#pragma unroll
                for (int t = 0; t < BKU; ++t) {
                    const int j = ja + t;
                    ww[t] = (j >= 0 && j < g.nu && j <= jb)
                        ? uweight(C, uedge(g, j), uedge(g, j + 1), inv_du) : 0.f;
                }
                w = make_float4(ww[0], ww[1], ww[2], ww[3]);
                mz = C.mz;
            }
            T.w[b][tid] = w;
            T.j0[b][tid] = j0;
            T.mz[b][tid] = mz;
        }
        __syncthreads();
        const float *q = qw + (size_t)a * g.nu * g.nv;
        if (iy < g.ny && iz < g.nz) {
            if (T.wide[b] != a) {
#pragma unroll
                for (int i = 0; i < BT; ++i) {
                    const int col = i + BT * warp;
                    const float mz = T.mz[b][col];
                    const float4 w = T.w[b][col];
                    const int j0 = T.j0[b][col];
                    const float va = mz * ((float)iz - hz), vb = va + mz;
                    const int la = max((int)floorf((va - V0) * inv_dv), 0);
                    const int lb = min((int)floorf((vb - V0) * inv_dv), g.nv - 1);
                    const float wt[BKU] = {w.x, w.y, w.z, w.w};
                    float part = 0.f;
                    for (int l = la; l <= lb; ++l) {
                        const float ov = fminf(vb, vedge(g, l + 1)) - fmaxf(va, vedge(g, l));
                        if (ov <= 0.f) continue;
                        float r = 0.f;
#pragma unroll
                        for (int t = 0; t < BKU; ++t)
                            if (wt[t] != 0.f) r = fmaf(wt[t], __ldg(q + (size_t)(j0 + t) * g.nv + l), r);
                        part = fmaf(r, ov, part);
                    }
                    grp[i] = fmaf(part, inv_dv, grp[i]);
                }
            } else {
                float wv[BT];
                sf_voxels_view(g, q, cs.x, cs.y, x0, iy, iz, wv);
#pragma unroll
                for (int i = 0; i < BT; ++i) grp[i] += wv[i];
            }
        }
        if (++ngrp == 16) {
#pragma unroll
            for (int i = 0; i < BT; ++i) { acc[i].add(grp[i]); grp[i] = 0.f; }
            ngrp = 0;
        }
    }
    if (iy >= g.ny || iz >= g.nz) return;
#pragma unroll
    for (int i = 0; i < BT; ++i) {
        const int ix = x0 + i;
        if (ix >= g.nx) continue;
        acc[i].add(grp[i]);
        float *o = vol + ((size_t)ix * g.ny + iy) * g.nz + iz;
        *o = accumulate ? *o + acc[i].s : acc[i].s;
    }
}

int check(const vg_dd3d_geom *g) {
    VG_REQUIRE(g, "sf3d: null geometry");
    VG_REQUIRE(g->nx > 0 && g->ny > 0 && g->nz > 0 && g->na > 0 && g->nu > 0 && g->nv > 0,
               "sf3d: sizes must be positive");
    VG_REQUIRE(g->na < 65536 && ceil_div(g->nx, BT) < 65536 && ceil_div(g->ny, BT) < 65536 &&
                   ceil_div(g->nu, SU) < 65536, "sf3d: sizes too large");
    VG_REQUIRE(g->nx <= SLINES && g->ny <= SLINES, "sf3d: nx and ny at most %d", SLINES);
    // (nz + 1: the forward projection's z sums index the volume's columns with one extra entry)
    VG_REQUIRE((double)g->nx * g->ny * (g->nz + 1) < 2147483648.0, "sf3d: volume above 2^31 voxels");
    VG_REQUIRE(g->du > 0.f && g->dv > 0.f && g->d_pix > 0.f && g->DSO > 0.f && g->DSD > 0.f,
               "sf3d: pitches and distances must be positive");
    // every voxel in front of the source (its footprint's projections are
    // then finite): the volume's half diagonal in the plane below DSO
    const float hx = 0.5f * g->nx * g->d_pix, hy = 0.5f * g->ny * g->d_pix;
    VG_REQUIRE(hx * hx + hy * hy < g->DSO * g->DSO,
               "sf3d: the volume must lie inside the source circle (half diagonal below DSO)");
    return VG_OK;
}

constexpr size_t SF_CHUNK_BYTES = (size_t)256 << 20;

size_t chunk_views(const vg_dd3d_geom *g) {
    const size_t per = (size_t)g->nu * g->nv * sizeof(float);
    size_t n = SF_CHUNK_BYTES / per;
    if (n < 1) n = 1;
    if (n > (size_t)g->na) n = g->na;
    return n;
}

size_t bp_ws_bytes(const vg_dd3d_geom *g) {
    return chunk_views(g) * (size_t)g->nu * g->nv * sizeof(float);
}

// the forward projection's z-prefix array: nx ny (nz + 1) floats
size_t fp_ws_bytes(const vg_dd3d_geom *g) {
    return (size_t)g->nx * g->ny * (g->nz + 1) * sizeof(float);
}

}  // namespace

extern "C" size_t vg_sf3d_workspace_bytes(const vg_dd3d_geom *g) {
    if (check(g)) return 0;
    const size_t f = fp_ws_bytes(g), b = bp_ws_bytes(g);
    return f > b ? f : b;
}

extern "C" int vg_sf3d_fp(const vg_dd3d_geom *g, const float *vol, const double *trig, float *sino,
                          void *workspace, size_t workspace_bytes, void *stream) {
    int st = check(g);
    if (st) return st;
    VG_REQUIRE(vol && trig && sino, "sf3d_fp: null pointer");
    const size_t need = fp_ws_bytes(g);
    VG_REQUIRE(workspace && workspace_bytes >= need,
               "sf3d_fp: workspace of %zu bytes needed (vg_sf3d_workspace_bytes)", need);
    VG_REQUIRE(((uintptr_t)workspace & 3) == 0, "sf3d_fp: workspace must be 4-byte aligned");
    cudaStream_t s = as_stream(stream);
    float *zp = static_cast<float *>(workspace);
    const size_t ncol = (size_t)g->nx * g->ny;
    sf3d_zprefix<<<ceil_div((long long)ncol * 32, 256), 256, 0, s>>>(*g, vol, zp);
    st = launch_status("sf3d_zprefix");
    if (st) return st;
    dim3 grid(ceil_div(g->nv, SV), ceil_div(g->nu, SU), g->na);
    sf3d_fp_kernel<<<grid, 256, 0, s>>>(*g, vol, zp, trig, sino);
    return launch_status("sf3d_fp");
}

extern "C" int vg_sf3d_bp(const vg_dd3d_geom *g, const float *sino, const double *trig, float *vol,
                          void *workspace, size_t workspace_bytes, void *stream) {
    int st = check(g);
    if (st) return st;
    VG_REQUIRE(sino && trig && vol, "sf3d_bp: null pointer");
    const size_t nch = chunk_views(g);
    const size_t need = bp_ws_bytes(g);
    VG_REQUIRE(workspace && workspace_bytes >= need,
               "sf3d_bp: workspace of %zu bytes needed (vg_sf3d_workspace_bytes)", need);
    cudaStream_t s = as_stream(stream);
    float *qw = static_cast<float *>(workspace);
    dim3 grid(ceil_div(g->nz, BZ), ceil_div(g->ny, BT), ceil_div(g->nx, BT));
    for (int a0 = 0; a0 < g->na; a0 += (int)nch) {
        const int cnt = (int)((size_t)(g->na - a0) < nch ? (size_t)(g->na - a0) : nch);
        sf3d_weight<<<1216, 256, 0, s>>>(*g, sino, a0, cnt, qw);
        st = launch_status("sf3d_weight");
        if (st) return st;
        sf3d_bp_kernel<<<grid, 256, 0, s>>>(*g, qw, trig, a0, cnt, a0 > 0, vol);
        st = launch_status("sf3d_bp");
        if (st) return st;
    }
    return VG_OK;
}
