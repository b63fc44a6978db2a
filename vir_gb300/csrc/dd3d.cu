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

__device__ __forceinline__ float projU(const vg_dd3d_geom &g, const View3 &v, float cp, float co,
                                       float b) {
    return __fdividef(g.DSD * fmaf(v.pd, b, cp), g.DSO - fmaf(v.od, b, co));
}

size_t ws_bytes(const vg_dd3d_geom *g) {
    const int nm = g->nx > g->ny ? g->nx : g->ny;
    return (size_t)g->na * nm * 2 * sizeof(float);
}

// tab[ia][io] = (scale, zmag)
__global__ void dd3d_prep(vg_dd3d_geom g, const double *__restrict__ trig, float2 *__restrict__ tab) {
    const int ia = blockIdx.x;
    const View3 v = view3(trig, ia);
    const int no = v.xdrv ? g.ny : g.nx;
    const int nm = g.nx > g.ny ? g.nx : g.ny;
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

__global__ void __launch_bounds__(256)
dd3d_fp_kernel(vg_dd3d_geom g, const float *__restrict__ vol, const double *__restrict__ trig,
               const float2 *__restrict__ tab, float *__restrict__ sino) {
    const int iv = blockIdx.x * 32 + threadIdx.x;
    const int iu = blockIdx.y * 8 + threadIdx.y;
    const int ia = blockIdx.z;
    if (iv >= g.nv || iu >= g.nu) return;
    const View3 v = view3(trig, ia);
    const int nd = v.xdrv ? g.nx : g.ny;
    const int no = v.xdrv ? g.ny : g.nx;
    const int nm = g.nx > g.ny ? g.nx : g.ny;
    const float Ul = ufloor_edge(g, iu), Ur = ufloor_edge(g, iu + 1);
    const float Vl = vfloor_edge(g, iv), Vr = vfloor_edge(g, iv + 1);
    // inverse edge map (natural pixel coordinate): b(U) = (U (DSO - co) - DSD cp) / (DSD pd + U od)
    const float rl = 1.0f / (g.DSD * v.pd + Ul * v.od), rr = 1.0f / (g.DSD * v.pd + Ur * v.od);
    const float inv_d = 1.0f / g.d_pix;
    const size_t sk = v.xdrv ? (size_t)g.ny * g.nz : (size_t)g.nz;  // stride of k
    const size_t so = v.xdrv ? (size_t)g.nz : (size_t)g.ny * g.nz;  // stride of io
    Kahan acc;
    for (int io = 0; io < no; ++io) {
        const float c = cen(g.d_pix, io, no);
        const float cp = v.po * c, co = v.oo * c;
        const float2 sz = __ldg(tab + (size_t)ia * nm + io);
        // pixels under [Ul, Ur]
        const float kl = fmaf(Ul, g.DSO - co, -g.DSD * cp) * rl * inv_d + 0.5f * nd;
        const float kr = fmaf(Ur, g.DSO - co, -g.DSD * cp) * rr * inv_d + 0.5f * nd;
        const int k0 = max(0, (int)floorf(fminf(kl, kr)));
        const int k1 = min(nd - 1, (int)floorf(fmaxf(kl, kr)));
        if (k0 > k1) continue;
        // slices under [Vl, Vr]: v edge of slice iz is zmag d (iz - nz/2)
        const float izl = Vl / (sz.y * g.d_pix) + 0.5f * g.nz;
        const float izr = Vr / (sz.y * g.d_pix) + 0.5f * g.nz;
        const int z0 = max(0, (int)floorf(izl)), z1 = min(g.nz - 1, (int)floorf(izr));
        if (z0 > z1) continue;
        float part = 0.f;
        float pa = projU(g, v, cp, co, edg(g.d_pix, k0, nd));
        for (int k = k0; k <= k1; ++k) {
            const float pb = projU(g, v, cp, co, edg(g.d_pix, k + 1, nd));
            const float ou = fminf(fmaxf(pa, pb), Ur) - fmaxf(fminf(pa, pb), Ul);
            pa = pb;
            if (ou <= 0.f) continue;
            const float *col = vol + k * sk + io * so;
            float colsum = 0.f;
            for (int iz = z0; iz <= z1; ++iz) {
                const float zl = sz.y * edg(g.d_pix, iz, g.nz), zr = sz.y * edg(g.d_pix, iz + 1, g.nz);
                const float ov = fminf(zr, Vr) - fmaxf(zl, Vl);
                if (ov > 0.f) colsum = fmaf(__ldg(col + iz), ov, colsum);
            }
            part = fmaf(colsum, ou, part);
        }
        acc.add(part * sz.x);
    }
    sino[((size_t)ia * g.nu + iu) * g.nv + iv] = acc.s * (g.d_pix * g.d_pix / (g.du * g.dv));
}

__global__ void __launch_bounds__(256)
dd3d_bp_kernel(vg_dd3d_geom g, const float *__restrict__ sino, const double *__restrict__ trig,
               const float2 *__restrict__ tab, float *__restrict__ vol) {
    const int iz = blockIdx.x * 32 + threadIdx.x;
    const int iy = blockIdx.y * 8 + threadIdx.y;
    const int ix = blockIdx.z;
    if (iz >= g.nz || iy >= g.ny) return;
    const int nm = g.nx > g.ny ? g.nx : g.ny;
    const float zl0 = edg(g.d_pix, iz, g.nz), zr0 = edg(g.d_pix, iz + 1, g.nz);
    const float u0 = ufloor_edge(g, 0), v0 = vfloor_edge(g, 0);
    const float idu = 1.0f / g.du, idv = 1.0f / g.dv;
    Kahan acc;
    for (int ia = 0; ia < g.na; ++ia) {
        const View3 v = view3(trig, ia);
        int k, nd, io, no;
        if (v.xdrv) { k = ix; nd = g.nx; io = iy; no = g.ny; }
        else        { k = iy; nd = g.ny; io = ix; no = g.nx; }
        const float c = cen(g.d_pix, io, no);
        const float cp = v.po * c, co = v.oo * c;
        const float2 sz = __ldg(tab + (size_t)ia * nm + io);
        const float pa = projU(g, v, cp, co, edg(g.d_pix, k, nd));
        const float pb = projU(g, v, cp, co, edg(g.d_pix, k + 1, nd));
        const float ulo = fminf(pa, pb), uhi = fmaxf(pa, pb);
        const float vlo = sz.y * zl0, vhi = sz.y * zr0;
        const int j0 = max(0, (int)floorf((ulo - u0) * idu)), j1 = min(g.nu - 1, (int)floorf((uhi - u0) * idu));
        const int q0 = max(0, (int)floorf((vlo - v0) * idv)), q1 = min(g.nv - 1, (int)floorf((vhi - v0) * idv));
        if (j0 > j1 || q0 > q1) continue;
        const float *s = sino + (size_t)ia * g.nu * g.nv;
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
        acc.add(part * sz.x);
    }
    vol[((size_t)ix * g.ny + iy) * g.nz + iz] = acc.s / ((float)g.na * g.d_pix);
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
    VG_REQUIRE(ws && wsb >= ws_bytes(g) && ((uintptr_t)ws & 7) == 0,
               "dd3d: workspace of %zu bytes needed (vg_dd3d_workspace_bytes)", ws_bytes(g));
    dd3d_prep<<<g->na, 256, 0, st>>>(*g, trig, reinterpret_cast<float2 *>(ws));
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
    dim3 grid(ceil_div(g->nv, 32), ceil_div(g->nu, 8), g->na);
    dd3d_fp_kernel<<<grid, dim3(32, 8), 0, st>>>(*g, vol, trig,
                                                  reinterpret_cast<const float2 *>(workspace), sino);
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
    dim3 grid(ceil_div(g->nz, 32), ceil_div(g->ny, 8), g->nx);
    dd3d_bp_kernel<<<grid, dim3(32, 8), 0, st>>>(*g, sino, trig,
                                                  reinterpret_cast<const float2 *>(workspace), vol);
    return launch_status("dd3d_bp");
}
