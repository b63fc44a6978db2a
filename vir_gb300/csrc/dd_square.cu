// Distance-driven projector pair of the translational "square" geometry
// (sys_mat/dd.py:895-1313) and the SIRT iteration around it
// (sys_mat/sirt_dd.py:37-76).
//
// Geometry (dd.py:935-957, 1138-1160).  An n x n x nz object (x, y, z; z
// fastest) with voxel boundaries d_pix (k - n/2) is seen from four sides.
// Each side is a plane of nsrc_p x nsrc_z sources at o = DSO, centres
// dsrc (k - (nsrc - 1)/2) + ssrc, and a flat detector of nu x nv cells with
// boundaries du (k - nu/2) + su + ssrc_p and dv (k - nv/2) + sv + ssrc_z.
// Slab io (the index orthogonal to the side) has the magnification
// M = DSD / (DSO - o_bnd[io]) of its lower boundary (dd.py:972, 1179) and is
// skipped when M <= 0 (dd.py:988, 1185).  Seen from source (sp, sz), the
// parallel boundary p and the height z project to
//     u = M p - (M sp - ssrc_p),    v = M z - (M sz - ssrc_z).
// Side s sees image voxel map_s(io, ip, iz) (dd.py:1004-1007, 1264-1267):
//     s = 0: (io, ip)   1: (n-1-ip, io)   2: (n-1-io, n-1-ip)   3: (ip, n-1-io).
// FP = A * d_pix^2 / (du dv) (dd.py:930); BP = A^T (dd.py:1135).  Both use
// the same float expressions for every boundary, so each (voxel, cell) pair
// gets bit-identical overlap weights in the two directions.
//
// Forward: one thread per detector cell (i_sp, i_sz, iv, iu) and all four
// sides (one float4 of the (nsrc_p, nsrc_z, nv, nu, 4) sinogram), gathering
// over slabs io the voxels whose projected rectangles overlap the cell.  Lanes
// run along iv, so the z-contiguous voxel reads of a warp coalesce; the warp
// shares iu, so the loop over parallel voxels is warp-uniform.  The volume is
// read through L1/L2; the output tile is transposed in shared memory so each
// cell row is written in 128-byte runs.
//
// Back: one thread per voxel of a side's frame (io, ip, iz) and all four
// sides, gathering over sources and overlapping cells (float4 reads, lanes
// along ip so a warp reads consecutive cells of one row).  Sources are taken
// in chunks whose sinogram slice fits in L2; each chunk adds into four FP64
// planes in frame order [io][iz][ip] (the workspace), and a combine kernel
// maps the planes back to image order as (side 0 + side 2) + (side 1 +
// side 3), the imgX + imgY of dd.py:1135, fusing the SIRT update if asked.
#include <math.h>

#include "vg_common.cuh"

#ifndef VG_SQ_TAB_MIN
#define VG_SQ_TAB_MIN 2.f  // cells a voxel spans along u before its slab reads row integrals
#endif

namespace {

using namespace vg;

struct SqGeo {
    int n, nz, nu, nv, nsp, nsz;
    float DSO, DSD, d_pix, du, dv, inv_du, inv_dv;
    float p_b0, z_b0;          // first voxel boundaries: parallel/orthogonal, z
    float u_b0, v_b0;          // first detector boundaries
    float u_end;               // last u boundary, u_b0 + nu du
    float sp0, dsp, sz0, dsz;  // source centres sp0 + k dsp, sz0 + k dsz
    float ssp, ssz;
    float scale;               // d_pix^2 / (du dv)
};

SqGeo make_geo(const vg_dd_square_geom *g) {
    SqGeo q;
    q.n = g->n; q.nz = g->nz; q.nu = g->nu; q.nv = g->nv;
    q.nsp = g->nsrc_p; q.nsz = g->nsrc_z;
    q.DSO = g->DSO; q.DSD = g->DSD; q.d_pix = g->d_pix;
    q.du = g->du; q.dv = g->dv;
    q.inv_du = 1.0f / g->du; q.inv_dv = 1.0f / g->dv;
    // pf.boundspace(n, d, s) = arange(n + 1) d + (s - d n / 2), float32
    q.p_b0 = 0.0f - g->d_pix * ((float)g->n * 0.5f);
    q.z_b0 = 0.0f - g->d_pix * ((float)g->nz * 0.5f);
    q.u_b0 = (g->su + g->ssrc_p) - g->du * ((float)g->nu * 0.5f);
    q.v_b0 = (g->sv + g->ssrc_z) - g->dv * ((float)g->nv * 0.5f);
    q.u_end = fmaf((float)g->nu, g->du, q.u_b0);
    // pf.censpace(n, d, s) = arange(n) d + (s - d (n - 1) / 2)
    q.dsp = g->dsrc_p; q.dsz = g->dsrc_z;
    q.sp0 = g->ssrc_p - g->dsrc_p * ((float)(g->nsrc_p - 1) * 0.5f);
    q.sz0 = g->ssrc_z - g->dsrc_z * ((float)(g->nsrc_z - 1) * 0.5f);
    q.ssp = g->ssrc_p; q.ssz = g->ssrc_z;
    q.scale = g->d_pix * g->d_pix / (g->du * g->dv);
    return q;
}

__device__ __forceinline__ float slab_mag(const SqGeo &g, int io) {
    return g.DSD / (g.DSO - fmaf((float)io, g.d_pix, g.p_b0));
}

__device__ __forceinline__ bool mag_ok(float M) { return M > 0.f && M < INFINITY; }

// First index k in [0, n] of the grid b(k) = b0 + k d whose cell
// [b(k), b(k+1)] can overlap an interval starting at a.  The estimate
// floor((a - b0) / d) is stepped down once when rounding put it past a;
// one too low only costs a zero-weight iteration.
__device__ __forceinline__ int first_cell(float a, float b0, float d, float inv_d, int n) {
    float f = floorf((a - b0) * inv_d);
    f = fminf(fmaxf(f, 0.f), (float)n);
    int k = (int)f;
    if (k > 0 && fmaf((float)k, d, b0) > a) --k;
    return k;
}

// ---- forward ---------------------------------------------------------------

constexpr int FPV = 32;  // cells along v per block (lanes)
constexpr int FPU = 8;   // cells along u per block (warps)

template <bool SIRT>
__global__ void __launch_bounds__(FPV * FPU, 4)
sq_fp_kernel(SqGeo g, const float *__restrict__ vol, float4 *__restrict__ sino,
             const float4 *__restrict__ y, const float4 *__restrict__ w) {
    // per slab: (M d_pix, 1 / (M d_pix), P(0), Q(0)); .x = 0 marks a skipped slab
    extern __shared__ float4 slab[];
    __shared__ float4 stage[FPU][FPV + 1];
    const int isp = blockIdx.z, isz = blockIdx.y;
    const int tiles_v = (g.nv + FPV - 1) / FPV;
    const int v0 = (blockIdx.x % tiles_v) * FPV, u0 = (blockIdx.x / tiles_v) * FPU;
    const int iv = v0 + threadIdx.x, iu = u0 + threadIdx.y;
    const int tid = threadIdx.y * FPV + threadIdx.x;
    const float sp = fmaf((float)isp, g.dsp, g.sp0), sz = fmaf((float)isz, g.dsz, g.sz0);
    for (int io = tid; io < g.n; io += FPV * FPU) {
        const float M = slab_mag(g, io);
        float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
        if (mag_ok(M)) {
            const float md = M * g.d_pix;
            e = make_float4(md, 1.0f / md, fmaf(M, g.p_b0, -fmaf(M, sp, -g.ssp)),
                            fmaf(M, g.z_b0, -fmaf(M, sz, -g.ssz)));
        }
        slab[io] = e;
    }
    __syncthreads();

    Kahan a0, a1, a2, a3;
    if (iv < g.nv && iu < g.nu) {
        const float ul = fmaf((float)iu, g.du, g.u_b0), ur = fmaf((float)(iu + 1), g.du, g.u_b0);
        const float vl = fmaf((float)iv, g.dv, g.v_b0), vr = fmaf((float)(iv + 1), g.dv, g.v_b0);
        const int n = g.n, nz = g.nz;
        for (int io = 0; io < n; ++io) {
            const float4 e = slab[io];
            if (e.x == 0.f) continue;
            int ip = first_cell(ul, e.z, e.x, e.y, n);
            const int iz0 = first_cell(vl, e.w, e.x, e.y, nz);
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
            float pl = fmaf((float)ip, e.x, e.z);
            for (; ip < n && pl < ur; ++ip) {
                const float pr = fmaf((float)(ip + 1), e.x, e.z);
                const float wu = fminf(ur, pr) - fmaxf(ul, pl);
                pl = pr;
                if (wu <= 0.f) continue;
                const float *c0 = vol + ((size_t)io * n + ip) * nz;
                const float *c1 = vol + ((size_t)(n - 1 - ip) * n + io) * nz;
                const float *c2 = vol + ((size_t)(n - 1 - io) * n + (n - 1 - ip)) * nz;
                const float *c3 = vol + ((size_t)ip * n + (n - 1 - io)) * nz;
                float t0 = 0.f, t1 = 0.f, t2 = 0.f, t3 = 0.f;
                float ql = fmaf((float)iz0, e.x, e.w);
                for (int iz = iz0; iz < nz && ql < vr; ++iz) {
                    const float qr = fmaf((float)(iz + 1), e.x, e.w);
                    const float wv = fminf(vr, qr) - fmaxf(vl, ql);
                    ql = qr;
                    if (wv > 0.f) {
                        t0 = fmaf(wv, __ldg(c0 + iz), t0);
                        t1 = fmaf(wv, __ldg(c1 + iz), t1);
                        t2 = fmaf(wv, __ldg(c2 + iz), t2);
                        t3 = fmaf(wv, __ldg(c3 + iz), t3);
                    }
                }
                s0 = fmaf(wu, t0, s0);
                s1 = fmaf(wu, t1, s1);
                s2 = fmaf(wu, t2, s2);
                s3 = fmaf(wu, t3, s3);
            }
            a0.add(s0);
            a1.add(s1);
            a2.add(s2);
            a3.add(s3);
        }
    }
    stage[threadIdx.y][threadIdx.x] =
        make_float4(a0.s * g.scale, a1.s * g.scale, a2.s * g.scale, a3.s * g.scale);
    __syncthreads();
    // write back transposed: consecutive threads take consecutive u cells
    const int ivl = tid / FPU, iul = tid % FPU;
    const int ivw = v0 + ivl, iuw = u0 + iul;
    if (ivw < g.nv && iuw < g.nu) {
        const size_t idx = (((size_t)isp * g.nsz + isz) * g.nv + ivw) * g.nu + iuw;
        float4 r = stage[iul][ivl];
        if (SIRT) {  // sirt_dd.fast_divide1 (sirt_dd.py:23-27)
            const float4 yy = __ldg(y + idx), ww = __ldg(w + idx);
            if (ww.x != 0.f) r.x = (yy.x - r.x) / ww.x;
            if (ww.y != 0.f) r.y = (yy.y - r.y) / ww.y;
            if (ww.z != 0.f) r.z = (yy.z - r.z) / ww.z;
            if (ww.w != 0.f) r.w = (yy.w - r.w) / ww.w;
        }
        sino[idx] = r;
    }
}

// ---- back ------------------------------------------------------------------

constexpr int BPP = 32;  // parallel voxels per block (lanes)
constexpr int BPZ = 8;   // z slices per block (warps)

// Running integrals along u of every detector row (isp, isz, iv) of a chunk
// of sources, for the slabs whose voxels span several cells: with U_j the
// cell boundaries and T_j = du sum_{i<j} c_i (compensated float32 prefix, all
// four sides),
// entry j holds x_j = T_j - c_j U_j and y_j = c_j, so the integral of the row
// from U_0 to u in cell j is G(u) = x_j + y_j u (entry nu: (T_nu, 0)); a
// voxel's u-overlap sum over the row is then G(pr) - G(pl) with both ends
// clamped to the detector.  Table: per row nu + 1 entries of two float4 (x, y).
// compensated float sums (Knuth's TwoSum): (s, c) holds s + c exactly to
// float32 rounding of the compensation
struct CSum {
    float s, c;
};
__device__ __forceinline__ CSum csum_add(CSum a, float v) {
    const float t = __fadd_rn(a.s, v);
    const float bp = __fsub_rn(t, a.s);
    const float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(v, bp));
    return CSum{t, __fadd_rn(a.c, e)};
}
__device__ __forceinline__ CSum csum_add(CSum a, CSum b) {
    CSum r = csum_add(a, b.s);
    r.c = __fadd_rn(r.c, b.c);
    return r;
}

__global__ void __launch_bounds__(256)
sq_bp_prep(SqGeo g, const float4 *__restrict__ sino, int isp0, float4 *__restrict__ tab) {
    __shared__ CSum wsum[8][4];
    const int r = blockIdx.x;  // row within the chunk: (isp - isp0, isz, iv)
    const float4 *c = sino + ((size_t)isp0 * g.nsz * g.nv + r) * g.nu;
    float4 *t = tab + 2 * (size_t)r * (g.nu + 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int per = (g.nu + 255) / 256, j0 = threadIdx.x * per;
    CSum loc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int i = 0; i < per; ++i)
        if (j0 + i < g.nu) {
            const float4 v = __ldg(c + j0 + i);
            loc[0] = csum_add(loc[0], v.x); loc[1] = csum_add(loc[1], v.y);
            loc[2] = csum_add(loc[2], v.z); loc[3] = csum_add(loc[3], v.w);
        }
    CSum inc[4] = {loc[0], loc[1], loc[2], loc[3]};
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const CSum a{__shfl_up_sync(0xffffffffu, inc[q].s, o), __shfl_up_sync(0xffffffffu, inc[q].c, o)};
            if (lane >= o) inc[q] = csum_add(inc[q], a);
        }
    }
    if (lane == 31)
#pragma unroll
        for (int q = 0; q < 4; ++q) wsum[warp][q] = inc[q];
    __syncthreads();
    // exclusive prefix of this thread: earlier warps, earlier lanes of this warp
    CSum run[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        run[q] = CSum{0.f, 0.f};
        for (int w = 0; w < warp; ++w) run[q] = csum_add(run[q], wsum[w][q]);
        const CSum before{__shfl_up_sync(0xffffffffu, inc[q].s, 1), __shfl_up_sync(0xffffffffu, inc[q].c, 1)};
        if (lane > 0) run[q] = csum_add(run[q], before);
    }
    const float du = g.du;
    for (int i = 0; i < per; ++i) {
        const int j = j0 + i;
        if (j < g.nu) {
            const float4 v = __ldg(c + j);
            const float U = fmaf((float)j, g.du, g.u_b0);
            // x_j = T_j - c_j U_j, T_j = du (s + c)
            t[2 * j] = make_float4(fmaf(run[0].s, du, fmaf(-v.x, U, run[0].c * du)),
                                   fmaf(run[1].s, du, fmaf(-v.y, U, run[1].c * du)),
                                   fmaf(run[2].s, du, fmaf(-v.z, U, run[2].c * du)),
                                   fmaf(run[3].s, du, fmaf(-v.w, U, run[3].c * du)));
            t[2 * j + 1] = v;
            run[0] = csum_add(run[0], v.x); run[1] = csum_add(run[1], v.y);
            run[2] = csum_add(run[2], v.z); run[3] = csum_add(run[3], v.w);
        }
    }
    if (threadIdx.x == 255) {
        t[2 * g.nu] = make_float4(fmaf(run[0].s, du, run[0].c * du), fmaf(run[1].s, du, run[1].c * du),
                                  fmaf(run[2].s, du, run[2].c * du), fmaf(run[3].s, du, run[3].c * du));
        t[2 * g.nu + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// G(u) of one table row (see sq_bp_prep), u clamped to the detector
__device__ __forceinline__ float4 sq_G(const float4 *__restrict__ tr, const SqGeo &g, float u) {
    const float uc = fminf(fmaxf(u, g.u_b0), g.u_end);
    const int j = min(max((int)floorf((uc - g.u_b0) * g.inv_du), 0), g.nu);
    const float4 x = __ldg(tr + 2 * j), y = __ldg(tr + 2 * j + 1);
    return make_float4(fmaf(y.x, uc, x.x), fmaf(y.y, uc, x.y), fmaf(y.z, uc, x.z), fmaf(y.w, uc, x.w));
}

// TAB: the slabs of this launch (io0 + blockIdx.y) read the row integrals;
// the host gives them the slabs whose voxels span VG_SQ_TAB_MIN or more cells
// along u (the magnification grows with io), the others a direct launch.
template <bool TAB>
__global__ void __launch_bounds__(BPP * BPZ, 4)
sq_bp_kernel(SqGeo g, const float4 *__restrict__ sino, int isp0, int isp1, int first,
             double *__restrict__ planes, const float4 *__restrict__ tab, int io0) {
    const int io = io0 + blockIdx.y;
    const int tiles_p = (g.n + BPP - 1) / BPP;
    const int ip = (blockIdx.x % tiles_p) * BPP + threadIdx.x;
    const int iz = (blockIdx.x / tiles_p) * BPZ + threadIdx.y;
    if (ip >= g.n || iz >= g.nz) return;
    const float M = slab_mag(g, io);
    Kahan a0, a1, a2, a3;
    if (mag_ok(M)) {
        const float md = M * g.d_pix;
        constexpr bool pref = TAB;
        for (int isp = isp0; isp < isp1; ++isp) {
            const float sp = fmaf((float)isp, g.dsp, g.sp0);
            const float P0 = fmaf(M, g.p_b0, -fmaf(M, sp, -g.ssp));
            const float pl = fmaf((float)ip, md, P0), pr = fmaf((float)(ip + 1), md, P0);
            const int iu0 = first_cell(pl, g.u_b0, g.du, g.inv_du, g.nu);
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
            for (int isz = 0; isz < g.nsz; ++isz) {
                const float sz = fmaf((float)isz, g.dsz, g.sz0);
                const float Q0 = fmaf(M, g.z_b0, -fmaf(M, sz, -g.ssz));
                const float ql = fmaf((float)iz, md, Q0), qr = fmaf((float)(iz + 1), md, Q0);
                int iv = first_cell(ql, g.v_b0, g.dv, g.inv_dv, g.nv);
                const float4 *base = sino + ((size_t)isp * g.nsz + isz) * g.nv * g.nu;
                float vl = fmaf((float)iv, g.dv, g.v_b0);
                for (; iv < g.nv && vl < qr; ++iv) {
                    const float vr = fmaf((float)(iv + 1), g.dv, g.v_b0);
                    const float wv = fminf(vr, qr) - fmaxf(vl, ql);
                    vl = vr;
                    if (wv <= 0.f) continue;
                    const float4 *row = base + (size_t)iv * g.nu;
                    float t0 = 0.f, t1 = 0.f, t2 = 0.f, t3 = 0.f;
                    if (pref) {
                        const float4 *tr = tab + 2 * (((size_t)(isp - isp0) * g.nsz + isz) * g.nv + iv) *
                                                     (size_t)(g.nu + 1);
                        const float4 a = sq_G(tr, g, pl), b = sq_G(tr, g, pr);
                        t0 = b.x - a.x; t1 = b.y - a.y; t2 = b.z - a.z; t3 = b.w - a.w;
                    }
                    float ul = fmaf((float)iu0, g.du, g.u_b0);
                    for (int iu = iu0; !pref && iu < g.nu && ul < pr; ++iu) {
                        const float ur = fmaf((float)(iu + 1), g.du, g.u_b0);
                        const float wu = fminf(ur, pr) - fmaxf(ul, pl);
                        ul = ur;
                        if (wu > 0.f) {
                            const float4 c = __ldg(row + iu);
                            t0 = fmaf(wu, c.x, t0);
                            t1 = fmaf(wu, c.y, t1);
                            t2 = fmaf(wu, c.z, t2);
                            t3 = fmaf(wu, c.w, t3);
                        }
                    }
                    s0 = fmaf(wv, t0, s0);
                    s1 = fmaf(wv, t1, s1);
                    s2 = fmaf(wv, t2, s2);
                    s3 = fmaf(wv, t3, s3);
                }
            }
            a0.add(s0);
            a1.add(s1);
            a2.add(s2);
            a3.add(s3);
        }
    }
    const size_t nvox = (size_t)g.n * g.n * g.nz;
    const size_t f = ((size_t)io * g.nz + iz) * g.n + ip;
    const double v0 = (double)a0.s - (double)a0.c, v1 = (double)a1.s - (double)a1.c;
    const double v2 = (double)a2.s - (double)a2.c, v3 = (double)a3.s - (double)a3.c;
    if (first) {
        planes[f] = v0;
        planes[nvox + f] = v1;
        planes[2 * nvox + f] = v2;
        planes[3 * nvox + f] = v3;
    } else {
        planes[f] += v0;
        planes[nvox + f] += v1;
        planes[2 * nvox + f] += v2;
        planes[3 * nvox + f] += v3;
    }
}

// Frame planes -> image (x, y, z).  Tile of CX x CY x CZ voxels: sides 0 and
// 2 are read with lanes along y, sides 1 and 3 with lanes along x (their
// frame's fastest index), summed in shared memory, written with z fastest.
// The tile strides (1 along z, CZ + 1 along y, CY (CZ + 1) + 1 along x) are
// odd in doubles, so each of the three access patterns is spread over banks.
constexpr int CX = 16, CY = 32, CZ = 8;
constexpr int TSY = CZ + 1, TSX = CY * TSY + 1;

template <bool SIRT>
__global__ void __launch_bounds__(256)
sq_combine_kernel(int n, int nz, const double *__restrict__ planes, float *__restrict__ vol,
                  const float *__restrict__ w, float gamma) {
    __shared__ double tile[CX * TSX];
    const int tiles_z = (nz + CZ - 1) / CZ;
    const int z0 = (blockIdx.x % tiles_z) * CZ, y0 = (blockIdx.x / tiles_z) * CY;
    const int x0 = blockIdx.y * CX;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t nvox = (size_t)n * n * nz;
    const double *p0 = planes, *p1 = planes + nvox, *p2 = planes + 2 * nvox, *p3 = planes + 3 * nvox;
    // sides 0 and 2: frame (io = x, ip = y) and (io = n-1-x, ip = n-1-y)
    for (int r = warp; r < CZ * CX; r += 8) {
        const int zl = r / CX, xl = r % CX;
        const int x = x0 + xl, y = y0 + lane, z = z0 + zl;
        double v = 0.0;
        if (x < n && y < n && z < nz)
            v = p0[((size_t)x * nz + z) * n + y] + p2[((size_t)(n - 1 - x) * nz + z) * n + (n - 1 - y)];
        tile[xl * TSX + lane * TSY + zl] = v;
    }
    __syncthreads();
    // sides 1 and 3: frame (io = y, ip = n-1-x) and (io = n-1-y, ip = x)
    const int xl = threadIdx.x % CX;
    for (int r = threadIdx.x / CX; r < CZ * CY; r += 256 / CX) {
        const int zl = r / CY, yl = r % CY;
        const int x = x0 + xl, y = y0 + yl, z = z0 + zl;
        if (x < n && y < n && z < nz)
            tile[xl * TSX + yl * TSY + zl] += p1[((size_t)y * nz + z) * n + (n - 1 - x)] +
                                              p3[((size_t)(n - 1 - y) * nz + z) * n + x];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < CX * CY * CZ; e += 256) {
        const int zl = e % CZ, yl = (e / CZ) % CY, xl2 = e / (CZ * CY);
        const int x = x0 + xl2, y = y0 + yl, z = z0 + zl;
        if (x < n && y < n && z < nz) {
            const size_t i = ((size_t)x * n + y) * nz + z;
            float u = (float)tile[xl2 * TSX + yl * TSY + zl];
            if (SIRT) {  // sirt_dd.fast_divide2 and the update (sirt_dd.py:30-33, 72)
                const float ww = __ldg(w + i);
                if (ww != 0.f) u = u / ww;
                vol[i] = vol[i] + gamma * u;
            } else {
                vol[i] = u;
            }
        }
    }
}

int check(const vg_dd_square_geom *g) {
    VG_REQUIRE(g, "dd_square: null geometry");
    VG_REQUIRE(g->n > 0 && g->nz > 0 && g->nu > 0 && g->nv > 0 && g->nsrc_p > 0 && g->nsrc_z > 0,
               "dd_square: sizes must be positive");
    VG_REQUIRE(g->n <= 4096, "dd_square: n above 4096");
    VG_REQUIRE(g->nsrc_p < 65536 && g->nsrc_z < 65536, "dd_square: too many sources");
    VG_REQUIRE(g->du > 0.f && g->dv > 0.f && g->d_pix > 0.f,
               "dd_square: pitches must be positive");
    return VG_OK;
}

size_t plane_bytes(const vg_dd_square_geom *g) {
    return (size_t)4 * g->n * g->n * g->nz * sizeof(double);
}

// Sources per back-projection launch with row integrals: their table (two
// float4 per cell boundary) stays within 256 MiB.
int tab_chunk(const vg_dd_square_geom *g) {
    const size_t per_src = (size_t)g->nsrc_z * g->nv * (g->nu + 1) * 2 * sizeof(float4);
    size_t c = ((size_t)256 << 20) / (per_src ? per_src : 1);
    if (c < 1) c = 1;
    if (c > (size_t)g->nsrc_p) c = g->nsrc_p;
    return (int)c;
}

size_t tab_bytes(const vg_dd_square_geom *g) {
    return (size_t)tab_chunk(g) * g->nsrc_z * g->nv * (g->nu + 1) * 2 * sizeof(float4);
}

// workspace: the four FP64 planes, then (256-byte aligned) the row-integral table
size_t ws_bytes(const vg_dd_square_geom *g) {
    return ((plane_bytes(g) + 255) & ~(size_t)255) + tab_bytes(g);
}

int launch_fp(const vg_dd_square_geom *g, const float *vol, float *out, const float *y,
              const float *w, cudaStream_t st) {
    const SqGeo q = make_geo(g);
    const size_t smem = (size_t)g->n * sizeof(float4);
    const long long tiles = (long long)ceil_div(g->nv, FPV) * ceil_div(g->nu, FPU);
    VG_REQUIRE(tiles < 2147483647LL, "dd_square: detector too large");
    dim3 grid((unsigned)tiles, g->nsrc_z, g->nsrc_p);
    if (y) {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(sq_fp_kernel<true>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return cuda_status(e, "dd_square_fp: shared memory attribute");
        }
        sq_fp_kernel<true><<<grid, dim3(FPV, FPU), smem, st>>>(
            q, vol, reinterpret_cast<float4 *>(out), reinterpret_cast<const float4 *>(y),
            reinterpret_cast<const float4 *>(w));
    } else {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(sq_fp_kernel<false>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return cuda_status(e, "dd_square_fp: shared memory attribute");
        }
        sq_fp_kernel<false><<<grid, dim3(FPV, FPU), smem, st>>>(
            q, vol, reinterpret_cast<float4 *>(out), nullptr, nullptr);
    }
    return launch_status("dd_square_fp");
}

// Sources per back-projection launch: the chunk's sinogram slice stays
// within 48 MiB, so the slabs that re-read it find it in L2.
int bp_chunk(const vg_dd_square_geom *g) {
    const size_t per_src = (size_t)g->nsrc_z * g->nv * g->nu * sizeof(float4);
    size_t c = ((size_t)48 << 20) / (per_src ? per_src : 1);
    if (c < 1) c = 1;
    if (c > (size_t)g->nsrc_p) c = g->nsrc_p;
    return (int)c;
}

int launch_bp(const vg_dd_square_geom *g, const float *sino, double *planes, float *vol,
              const float *w, float gamma, cudaStream_t st) {
    const SqGeo q = make_geo(g);
    dim3 grid(ceil_div(g->n, BPP) * ceil_div(g->nz, BPZ), g->n);
    VG_REQUIRE((long long)ceil_div(g->n, BPP) * ceil_div(g->nz, BPZ) < 2147483647LL,
               "dd_square: volume too large");
    // slabs io >= io_tab (magnification, hence the cells a voxel spans,
    // grows with io up to the source plane) read row integrals
    int io_tab = g->n;
    for (int io = 0; io < g->n; ++io) {
        const float M = q.DSD / (q.DSO - fmaf((float)io, q.d_pix, q.p_b0));
        if (M > 0.f && M < INFINITY && M * q.d_pix >= VG_SQ_TAB_MIN * q.du) {
            io_tab = io;
            break;
        }
    }
    const bool use_tab = io_tab < g->n;
    float4 *tab = reinterpret_cast<float4 *>(reinterpret_cast<char *>(planes) +
                                             ((plane_bytes(g) + 255) & ~(size_t)255));
    int chunk = bp_chunk(g);
    if (use_tab && tab_chunk(g) < chunk) chunk = tab_chunk(g);
    for (int s0 = 0; s0 < g->nsrc_p; s0 += chunk) {
        const int s1 = s0 + chunk < g->nsrc_p ? s0 + chunk : g->nsrc_p;
        if (use_tab) {
            const long long rows = (long long)(s1 - s0) * g->nsrc_z * g->nv;
            VG_REQUIRE(rows < 2147483647LL, "dd_square: too many detector rows per chunk");
            sq_bp_prep<<<(unsigned)rows, 256, 0, st>>>(q, reinterpret_cast<const float4 *>(sino), s0,
                                                       tab);
            int s = launch_status("dd_square_bp_prep");
            if (s) return s;
        }
        if (io_tab > 0) {
            dim3 gd(grid.x, io_tab);
            sq_bp_kernel<false><<<gd, dim3(BPP, BPZ), 0, st>>>(
                q, reinterpret_cast<const float4 *>(sino), s0, s1, s0 == 0, planes, nullptr, 0);
            int s = launch_status("dd_square_bp");
            if (s) return s;
        }
        if (use_tab) {
            dim3 gt(grid.x, g->n - io_tab);
            sq_bp_kernel<true><<<gt, dim3(BPP, BPZ), 0, st>>>(
                q, reinterpret_cast<const float4 *>(sino), s0, s1, s0 == 0, planes, tab, io_tab);
            int s = launch_status("dd_square_bp");
            if (s) return s;
        }
    }
    dim3 cgrid(ceil_div(g->nz, CZ) * ceil_div(g->n, CY), ceil_div(g->n, CX));
    if (w)
        sq_combine_kernel<true><<<cgrid, 256, 0, st>>>(g->n, g->nz, planes, vol, w, gamma);
    else
        sq_combine_kernel<false><<<cgrid, 256, 0, st>>>(g->n, g->nz, planes, vol, nullptr, 0.f);
    return launch_status("dd_square_combine");
}

}  // namespace

extern "C" size_t vg_dd_square_workspace_bytes(const vg_dd_square_geom *g) {
    if (check(g)) return 0;
    return ws_bytes(g);
}

extern "C" int vg_dd_square_fp(const vg_dd_square_geom *g, const float *vol, float *sino,
                               void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(vol && sino, "dd_square_fp: null pointer");
    VG_REQUIRE(((uintptr_t)sino & 15) == 0, "dd_square_fp: sinogram not 16-byte aligned");
    return launch_fp(g, vol, sino, nullptr, nullptr, as_stream(stream));
}

extern "C" int vg_dd_square_bp(const vg_dd_square_geom *g, const float *sino, float *vol,
                               void *workspace, size_t workspace_bytes, void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(sino && vol && workspace, "dd_square_bp: null pointer");
    VG_REQUIRE(((uintptr_t)sino & 15) == 0, "dd_square_bp: sinogram not 16-byte aligned");
    VG_REQUIRE(workspace_bytes >= ws_bytes(g), "dd_square_bp: workspace of %zu bytes, %zu needed",
               workspace_bytes, ws_bytes(g));
    VG_REQUIRE(((uintptr_t)workspace & 15) == 0, "dd_square_bp: workspace not 16-byte aligned");
    return launch_bp(g, sino, static_cast<double *>(workspace), vol, nullptr, 0.f,
                     as_stream(stream));
}

extern "C" int vg_dd_square_sirt_iter(const vg_dd_square_geom *g, const float *y,
                                      const float *w_sino, const float *w_vol, float gamma,
                                      float *x, float *r, void *workspace, size_t workspace_bytes,
                                      void *stream) {
    int s = check(g);
    if (s) return s;
    VG_REQUIRE(y && w_sino && w_vol && x && r && workspace, "dd_square_sirt_iter: null pointer");
    VG_REQUIRE(workspace_bytes >= ws_bytes(g),
               "dd_square_sirt_iter: workspace of %zu bytes, %zu needed", workspace_bytes,
               ws_bytes(g));
    VG_REQUIRE(((uintptr_t)workspace & 15) == 0, "dd_square_sirt_iter: workspace not 16-byte aligned");
    VG_REQUIRE((((uintptr_t)y | (uintptr_t)w_sino | (uintptr_t)r) & 15) == 0,
               "dd_square_sirt_iter: sinogram buffers must be 16-byte aligned");
    cudaStream_t st = as_stream(stream);
    s = launch_fp(g, x, r, y, w_sino, st);
    if (s) return s;
    return launch_bp(g, r, static_cast<double *>(workspace), x, w_vol, gamma, st);
}
