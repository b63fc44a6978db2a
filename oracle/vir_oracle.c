/*
 * vir_oracle.c -- FP64 CPU restatement of vir's projector / backprojector hot
 * path.  TEST INFRASTRUCTURE ONLY: this file is the parity checker used by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.  Nothing in
 * the vir_gb300 package links or calls it.
 *
 * Every function names the reference file:line it restates (paths inside the
 * vargasp/vir tree).  Geometry and accumulation are double precision; inputs
 * (images, sinograms) are float32 as in the reference.  The trig tables
 * (cos, sin per view) are computed by the caller exactly as the reference does
 * (numpy cos/sin of the reference's own angle dtype) and passed in as double,
 * so branch decisions (driving axis, dx == 0) follow the reference's values.
 *
 * Compile: gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC (see Makefile).
 * -ffp-contract=off keeps every a*b+c a separately rounded multiply and add,
 * as numpy evaluates it.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

/* ------------------------------------------------------------------------ */
/* 2D parallel-beam Siddon, sys_mat/fp_2d_par.py:11-64                        */
/* ------------------------------------------------------------------------ */

/* Enumerates the segments of one ray exactly as fp_2d_par.siddons_fp_2d does:
 * image edges d_pix*(i - n/2.0) (:16-17), detector centre
 * d_det*((k - n_dets/2.0) + 0.5) (:20), origin det*(-dy, dx) (:29-30),
 * entry/exit t0/t1 (:33-43), the sorted crossing list filtered to [t0, t1]
 * (:45-53), and per consecutive pair the midpoint voxel by floor (:54-63).
 * Writes (ix, iy, |dt|) of in-image segments; returns their count. */
static int siddon2d_ray_segments(int nx, int ny, double d_pix, double d_det,
                                 int n_dets, int idet, double dx, double dy,
                                 double *scratch, int *oix, int *oiy,
                                 double *olen)
{
    double det = d_det * (((double)idet - n_dets / 2.0) + 0.5);
    double x0 = det * -dy;
    double y0 = det * dx;
    double xb0 = d_pix * (0.0 - nx / 2.0), xbn = d_pix * ((double)nx - nx / 2.0);
    double yb0 = d_pix * (0.0 - ny / 2.0), ybn = d_pix * ((double)ny - ny / 2.0);
    double tx0 = -INFINITY, txn = INFINITY, ty0 = -INFINITY, tyn = INFINITY;
    if (dx != 0.0) { tx0 = (xb0 - x0) / dx; txn = (xbn - x0) / dx; }
    if (dy != 0.0) { ty0 = (yb0 - y0) / dy; tyn = (ybn - y0) / dy; }
    double t0 = fmax(fmin(tx0, txn), fmin(ty0, tyn));
    double t1 = fmin(fmax(tx0, txn), fmax(ty0, tyn));
    if (t1 <= t0 || isinf(t0) || isinf(t1)) return 0;
    int nc = 0;
    if (dx != 0.0)
        for (int i = 0; i <= nx; i++) {
            double t = (d_pix * ((double)i - nx / 2.0) - x0) / dx;
            if (t0 <= t && t <= t1) scratch[nc++] = t;
        }
    if (dy != 0.0)
        for (int i = 0; i <= ny; i++) {
            double t = (d_pix * ((double)i - ny / 2.0) - y0) / dy;
            if (t0 <= t && t <= t1) scratch[nc++] = t;
        }
    if (nc < 2) return 0;
    qsort(scratch, (size_t)nc, sizeof(double), cmp_double);
    int ns = 0;
    for (int s = 0; s + 1 < nc; s++) {
        double a = scratch[s], b = scratch[s + 1];
        if (b <= a) continue;
        double m = 0.5 * (a + b);
        double xc = x0 + m * dx;
        double yc = y0 + m * dy;
        double fx = floor((xc - xb0) / d_pix);
        double fy = floor((yc - yb0) / d_pix);
        if (fx >= 0 && fx < nx && fy >= 0 && fy < ny) {
            oix[ns] = (int)fx;
            oiy[ns] = (int)fy;
            olen[ns] = fabs(b - a);
            ns++;
        }
    }
    return ns;
}

/* Forward projection.  img is (nx, ny) C-order (img[ix*ny+iy]), sino (na,
 * n_dets).  mode 0: FP64 accumulation (the FP64 oracle).  mode 1: each
 * addition rounded to float32 as numpy's `sino[i,j] += img*abs(dt)` on a
 * float32 array does (fp_2d_par.py:63), which reproduces the reference's
 * output bit for bit. */
void orc_siddon_fp_2d(const float *img, int nx, int ny, const double *cosv,
                      const double *sinv, int na, int n_dets, double d_det,
                      double d_pix, int mode, double *sino)
{
#pragma omp parallel
    {
        int cap = nx + ny + 4;
        double *scr = (double *)malloc(sizeof(double) * cap);
        int *ix = (int *)malloc(sizeof(int) * cap);
        int *iy = (int *)malloc(sizeof(int) * cap);
        double *ln = (double *)malloc(sizeof(double) * cap);
#pragma omp for schedule(dynamic)
        for (int ia = 0; ia < na; ia++)
            for (int k = 0; k < n_dets; k++) {
                int ns = siddon2d_ray_segments(nx, ny, d_pix, d_det, n_dets, k,
                                               cosv[ia], sinv[ia], scr, ix, iy, ln);
                double acc = 0.0;
                float acc32 = 0.0f;
                for (int s = 0; s < ns; s++) {
                    double v = (double)img[(size_t)ix[s] * ny + iy[s]] * ln[s];
                    if (mode == 1) acc32 = (float)((double)acc32 + v);
                    else acc += v;
                }
                sino[(size_t)ia * n_dets + k] = mode == 1 ? (double)acc32 : acc;
            }
        free(scr); free(ix); free(iy); free(ln);
    }
}

/* Exact transpose of orc_siddon_fp_2d (mode 0): img[ix,iy] += sino*len over
 * the same segments.  The reference's list backprojector
 * (projection/projection_c.c:176-208) is this operation on a stored list. */
void orc_siddon_bp_2d(const float *sino, int na, int n_dets, const double *cosv,
                      const double *sinv, int nx, int ny, double d_det,
                      double d_pix, double *img)
{
    size_t npx = (size_t)nx * ny;
    memset(img, 0, sizeof(double) * npx);
#pragma omp parallel
    {
        int cap = nx + ny + 4;
        double *scr = (double *)malloc(sizeof(double) * cap);
        int *ix = (int *)malloc(sizeof(int) * cap);
        int *iy = (int *)malloc(sizeof(int) * cap);
        double *ln = (double *)malloc(sizeof(double) * cap);
        double *part = (double *)calloc(npx, sizeof(double));
#pragma omp for schedule(dynamic)
        for (int ia = 0; ia < na; ia++)
            for (int k = 0; k < n_dets; k++) {
                double y = sino[(size_t)ia * n_dets + k];
                int ns = siddon2d_ray_segments(nx, ny, d_pix, d_det, n_dets, k,
                                               cosv[ia], sinv[ia], scr, ix, iy, ln);
                for (int s = 0; s < ns; s++)
                    part[(size_t)ix[s] * ny + iy[s]] += y * ln[s];
            }
#pragma omp critical
        for (size_t i = 0; i < npx; i++) img[i] += part[i];
        free(scr); free(ix); free(iy); free(ln); free(part);
    }
}

/* Per-ray trace for voxel-sequence checks: segment count, order-sensitive
 * hash of voxel indices ix*ny+iy (h = (h ^ (idx + C1)) * C2 from
 * h0 = 0xCBF29CE484222325), and the sum of lengths. */
void orc_siddon_trace_2d(int nx, int ny, const double *cosv, const double *sinv,
                         int na, int n_dets, double d_det, double d_pix,
                         int *count, uint64_t *hash, double *len)
{
#pragma omp parallel
    {
        int cap = nx + ny + 4;
        double *scr = (double *)malloc(sizeof(double) * cap);
        int *ix = (int *)malloc(sizeof(int) * cap);
        int *iy = (int *)malloc(sizeof(int) * cap);
        double *ln = (double *)malloc(sizeof(double) * cap);
#pragma omp for schedule(dynamic)
        for (int ia = 0; ia < na; ia++)
            for (int k = 0; k < n_dets; k++) {
                int ns = siddon2d_ray_segments(nx, ny, d_pix, d_det, n_dets, k,
                                               cosv[ia], sinv[ia], scr, ix, iy, ln);
                uint64_t h = 0xCBF29CE484222325ull;
                double l = 0.0;
                for (int s = 0; s < ns; s++) {
                    uint64_t v = (uint64_t)ix[s] * (uint64_t)ny + (uint64_t)iy[s];
                    h = (h ^ (v + 0x9E3779B97F4A7C15ull)) * 0x100000001B3ull;
                    l += ln[s];
                }
                size_t o = (size_t)ia * n_dets + k;
                count[o] = ns;
                hash[o] = h;
                len[o] = l;
            }
        free(scr); free(ix); free(iy); free(ln);
    }
}

/* Number of nonzero segments per ray (for the intersection count metric). */
long long orc_siddon_count_2d(int nx, int ny, const double *cosv,
                              const double *sinv, int na, int n_dets,
                              double d_det, double d_pix)
{
    long long total = 0;
#pragma omp parallel reduction(+ : total)
    {
        int cap = nx + ny + 4;
        double *scr = (double *)malloc(sizeof(double) * cap);
        int *ix = (int *)malloc(sizeof(int) * cap);
        int *iy = (int *)malloc(sizeof(int) * cap);
        double *ln = (double *)malloc(sizeof(double) * cap);
#pragma omp for schedule(dynamic)
        for (int ia = 0; ia < na; ia++)
            for (int k = 0; k < n_dets; k++)
                total += siddon2d_ray_segments(nx, ny, d_pix, d_det, n_dets, k,
                                               cosv[ia], sinv[ia], scr, ix, iy, ln);
        free(scr); free(ix); free(iy); free(ln);
    }
    return total;
}

/* ------------------------------------------------------------------------ */
/* Distance-driven 2D, sys_mat/dd.py                                         */
/* ------------------------------------------------------------------------ */

/* Per-view geometry of _dd_par_geom (dd.py:472-523) and _dd_fan_geom
 * (dd.py:527-585).  Pixel edges d_pix*(i - n/2) and centres as their
 * midpoints (dd.py:690-695); the view's driving axis is X when
 * |sin| >= |cos|.  Arrays are indexed by the sweep index ip (0..np) after the
 * reversal that makes the projected driving edges increasing (dd.py:516-518);
 * pix(ip, io) gives the flat image index of sweep pixel ip on line io. */
typedef struct {
    int np_, no, xdrv, rev;
    double *p_drv, *o_drv; /* np+1 */
    double *p_orth, *o_orth, *scl; /* no */
} dd_view;

static void dd_view_alloc(dd_view *g, int nx, int ny)
{
    int m = (nx > ny ? nx : ny) + 1;
    g->p_drv = (double *)malloc(sizeof(double) * m);
    g->o_drv = (double *)malloc(sizeof(double) * m);
    g->p_orth = (double *)malloc(sizeof(double) * m);
    g->o_orth = (double *)malloc(sizeof(double) * m);
    g->scl = (double *)malloc(sizeof(double) * m);
}

static void dd_view_free(dd_view *g)
{
    free(g->p_drv); free(g->o_drv); free(g->p_orth); free(g->o_orth); free(g->scl);
}

/* fan == 0: parallel geometry (scale 1/|trig|, o terms unused).
 * fan == 1: fan geometry, scale r / ((DSO - o_orth) |trig|). */
static void dd_view_setup(dd_view *g, int fan, int nx, int ny, double d_pix,
                          double c, double s, double DSO)
{
    double *bnd_d, *cen_o;
    int nd, no;
    double pd, od, po, oo, trig;
    g->xdrv = fabs(s) >= fabs(c);
    if (g->xdrv) { nd = nx; no = ny; pd = -s; od = c; po = c; oo = s; trig = fabs(s); }
    else         { nd = ny; no = nx; pd = c;  od = s; po = -s; oo = c; trig = fabs(c); }
    g->np_ = nd; g->no = no;
    bnd_d = (double *)malloc(sizeof(double) * (nd + 1));
    cen_o = (double *)malloc(sizeof(double) * no);
    for (int i = 0; i <= nd; i++) bnd_d[i] = d_pix * ((double)i - nd / 2.0);
    for (int i = 0; i < no; i++) {
        double l = d_pix * ((double)i - no / 2.0), r = d_pix * ((double)(i + 1) - no / 2.0);
        cen_o[i] = (l + r) / 2.0;
    }
    for (int i = 0; i <= nd; i++) { g->p_drv[i] = pd * bnd_d[i]; g->o_drv[i] = od * bnd_d[i]; }
    g->rev = g->p_drv[1] < g->p_drv[0];
    if (g->rev)
        for (int i = 0, j = nd; i < j; i++, j--) {
            double t = g->p_drv[i]; g->p_drv[i] = g->p_drv[j]; g->p_drv[j] = t;
            t = g->o_drv[i]; g->o_drv[i] = g->o_drv[j]; g->o_drv[j] = t;
        }
    for (int io = 0; io < no; io++) {
        g->p_orth[io] = po * cen_o[io];
        g->o_orth[io] = oo * cen_o[io];
        if (fan) {
            double a = DSO - g->o_orth[io];
            double r = sqrt(a * a + g->p_orth[io] * g->p_orth[io]);
            g->scl[io] = r / (a * trig);
        } else {
            g->scl[io] = 1.0 / trig;
        }
    }
    free(bnd_d); free(cen_o);
}

static inline size_t dd_pix(const dd_view *g, int ip, int io, int nx, int ny)
{
    int k = g->rev ? (g->np_ - 1 - ip) : ip;
    /* X-driven: sweep index along x, line index y; else the transpose. */
    (void)nx;
    return g->xdrv ? (size_t)k * ny + io : (size_t)io * ny + k;
}

static inline double dd_bound(const dd_view *g, int fan, int ip, int io,
                              double DSO, double DSD)
{
    if (!fan) return g->p_drv[ip] + g->p_orth[io];
    /* proj_img2det_fan, dd.py:50-51 */
    return DSD * (g->p_drv[ip] + g->p_orth[io]) / (DSO - (g->o_drv[ip] + g->o_orth[io]));
}

/* One view of the FP sweep (_dd_fp_par_sweep dd.py:82-126,
 * _dd_fp_fan_sweep dd.py:165-221): for each orthogonal line, merge projected
 * pixel edges with detector edges, accumulating img * overlap * scale. */
static void dd2d_fp_view(const dd_view *g, int fan, const float *img, int nx,
                         int ny, const double *u_bnd, int nu, double DSO,
                         double DSD, double *sino_row)
{
    for (int io = 0; io < g->no; io++) {
        double scl = g->scl[io];
        int ip = 0, iu = 0;
        double pl = dd_bound(g, fan, 0, io, DSO, DSD);
        double pr = dd_bound(g, fan, 1, io, DSO, DSD);
        while (ip < g->np_ && iu < nu) {
            double ul = u_bnd[iu], ur = u_bnd[iu + 1];
            double a = pl, b = pr;
            if (b < a) { double t = a; a = b; b = t; }
            double ol = fmax(a, ul), orr = fmin(b, ur);
            if (orr > ol) sino_row[iu] += img[dd_pix(g, ip, io, nx, ny)] * (orr - ol) * scl;
            if (b < ur) {
                ip++;
                if (ip == g->np_) break;
                pl = b; /* the reference carries the (possibly swapped) right edge */
                pr = dd_bound(g, fan, ip + 1, io, DSO, DSD);
            } else {
                iu++;
            }
        }
    }
}

/* One view of the BP sweep (_dd_bp_par_sweep dd.py:130-161,
 * _dd_bp_fan_sweep dd.py:225-277): the same merge, img += sino * overlap *
 * scale.  The BP sweep has no edge swap. */
static void dd2d_bp_view(const dd_view *g, int fan, double *img, int nx, int ny,
                         const float *sino_row, const double *u_bnd, int nu,
                         double DSO, double DSD, int io_lo, int io_hi)
{
    for (int io = io_lo; io < io_hi; io++) {
        double scl = g->scl[io];
        int ip = 0, iu = 0;
        double pl = dd_bound(g, fan, 0, io, DSO, DSD);
        double pr = dd_bound(g, fan, 1, io, DSO, DSD);
        while (ip < g->np_ && iu < nu) {
            double ul = u_bnd[iu], ur = u_bnd[iu + 1];
            double ol = fmax(pl, ul), orr = fmin(pr, ur);
            if (orr > ol) img[dd_pix(g, ip, io, nx, ny)] += sino_row[iu] * (orr - ol) * scl;
            if (pr < ur) {
                ip++;
                if (ip == g->np_) break;
                pl = pr;
                pr = dd_bound(g, fan, ip + 1, io, DSO, DSD);
            } else {
                iu++;
            }
        }
    }
}

static double *dd_u_bounds(int nu, double du, double su)
{
    double *u = (double *)malloc(sizeof(double) * (nu + 1));
    for (int i = 0; i <= nu; i++) u[i] = du * ((double)i - nu / 2.0 + su); /* dd.py:699 */
    return u;
}

/* dd_p_par_2d / dd_p_fan_2d forward branch (dd.py:676-725, 749-803):
 * returns sino * d_pix / du. */
void orc_dd_fp_2d(int fan, const float *img, int nx, int ny, const double *cosv,
                  const double *sinv, int na, int nu, double du, double su,
                  double d_pix, double DSO, double DSD, double *sino)
{
    double *u_bnd = dd_u_bounds(nu, du, su);
#pragma omp parallel
    {
        dd_view g;
        dd_view_alloc(&g, nx, ny);
#pragma omp for schedule(dynamic)
        for (int ia = 0; ia < na; ia++) {
            double *row = sino + (size_t)ia * nu;
            memset(row, 0, sizeof(double) * nu);
            dd_view_setup(&g, fan, nx, ny, d_pix, cosv[ia], sinv[ia], DSO);
            dd2d_fp_view(&g, fan, img, nx, ny, u_bnd, nu, DSO, DSD, row);
            for (int iu = 0; iu < nu; iu++) row[iu] = row[iu] * d_pix / du;
        }
        dd_view_free(&g);
    }
    free(u_bnd);
}

/* dd_p_par_2d / dd_p_fan_2d backward branch: returns img / na / d_pix
 * (dd.py:721-723, 799-801). */
void orc_dd_bp_2d(int fan, const float *sino, int na, int nu, const double *cosv,
                  const double *sinv, int nx, int ny, double du, double su,
                  double d_pix, double DSO, double DSD, double *img)
{
    double *u_bnd = dd_u_bounds(nu, du, su);
    size_t npx = (size_t)nx * ny;
    memset(img, 0, sizeof(double) * npx);
    dd_view g;
    dd_view_alloc(&g, nx, ny);
    for (int ia = 0; ia < na; ia++) {
        dd_view_setup(&g, fan, nx, ny, d_pix, cosv[ia], sinv[ia], DSO);
        /* lines write disjoint pixels, so they run in parallel */
        int no = g.no;
#pragma omp parallel for schedule(static)
        for (int io = 0; io < no; io++)
            dd2d_bp_view(&g, fan, img, nx, ny, sino + (size_t)ia * nu, u_bnd, nu,
                         DSO, DSD, io, io + 1);
    }
    dd_view_free(&g);
    for (size_t i = 0; i < npx; i++) img[i] = img[i] / na / d_pix;
    free(u_bnd);
}

/* ------------------------------------------------------------------------ */
/* Distance-driven 3D cone, sys_mat/dd.py:285-468, 589-645, 815-888          */
/* ------------------------------------------------------------------------ */

/* The volume is (nx, ny, nz) C-order, the sinogram (na, nu, nv) with v
 * fastest.  Per orthogonal line io the driving edges project to u through
 * the fan magnification DSD/(DSO - (o_drv + o_orth)) (dd.py:310-313) and the
 * z edges to v through DSD/(DSO - o_orth) (dd.py:309).  The weight of
 * (voxel, bin) is overlap_u * overlap_v * scale(io) (dd.py:345-379).
 *
 * Deviation, stated: the reference FP reuses one tmp_u buffer for all lines
 * of a view and zeroes only [iu_min, iu_max) of the current line
 * (dd.py:300,335), so sums left by earlier lines outside that range are added
 * again at dd.py:379.  This restatement computes the overlap integral the
 * sweep intends (tmp_u cleared per (io, iz)); with that one change the
 * reference FP and BP form an adjoint pair.  u bins are merged from 0, which
 * is what the iu_min start approximates (dd.py:318-319,338). */
static void cone_line_u(const dd_view *g, int io, double DSO, double DSD,
                        double *pu)
{
    for (int ip = 0; ip <= g->np_; ip++)
        pu[ip] = DSD / (DSO - (g->o_drv[ip] + g->o_orth[io])) * (g->p_drv[ip] + g->p_orth[io]);
}

static inline size_t cone_vox(const dd_view *g, int ip, int io, int iz, int ny, int nz)
{
    int k = g->rev ? (g->np_ - 1 - ip) : ip;
    size_t ix = g->xdrv ? (size_t)k : (size_t)io;
    size_t iy = g->xdrv ? (size_t)io : (size_t)k;
    return (ix * ny + iy) * nz + iz;
}

void orc_dd_fp_cone(const float *vol, int nx, int ny, int nz, const double *cosv,
                    const double *sinv, int na, int nu, int nv, double du,
                    double dv, double su, double sv, double d_pix, double DSO,
                    double DSD, double *sino)
{
    double *u_bnd = dd_u_bounds(nu, du, su);
    double *v_bnd = dd_u_bounds(nv, dv, sv);
    double *z_bnd = (double *)malloc(sizeof(double) * (nz + 1));
    for (int i = 0; i <= nz; i++) z_bnd[i] = d_pix * ((double)i - nz / 2.0);
#pragma omp parallel
    {
        dd_view g;
        dd_view_alloc(&g, nx, ny);
        int m = (nx > ny ? nx : ny) + 1;
        double *pu = (double *)malloc(sizeof(double) * m);
        double *tmp = (double *)malloc(sizeof(double) * nu);
#pragma omp for schedule(dynamic)
        for (int ia = 0; ia < na; ia++) {
            double *s = sino + (size_t)ia * nu * nv;
            memset(s, 0, sizeof(double) * (size_t)nu * nv);
            dd_view_setup(&g, 1, nx, ny, d_pix, cosv[ia], sinv[ia], DSO);
            for (int io = 0; io < g.no; io++) {
                double scl = g.scl[io];
                double zmag = DSD / (DSO - g.o_orth[io]);
                cone_line_u(&g, io, DSO, DSD, pu);
                for (int iz = 0; iz < nz; iz++) {
                    double zl = zmag * z_bnd[iz], zr = zmag * z_bnd[iz + 1];
                    memset(tmp, 0, sizeof(double) * nu);
                    int any = 0;
                    int ip = 0, iu = 0;
                    while (ip < g.np_ && iu < nu) {
                        double ol = fmax(pu[ip], u_bnd[iu]), orr = fmin(pu[ip + 1], u_bnd[iu + 1]);
                        if (orr > ol) { tmp[iu] += vol[cone_vox(&g, ip, io, iz, ny, nz)] * scl * (orr - ol); any = 1; }
                        if (pu[ip + 1] < u_bnd[iu + 1]) ip++; else iu++;
                    }
                    if (!any) continue;
                    for (int iv = 0; iv < nv; iv++) {
                        double ol = fmax(zl, v_bnd[iv]), orr = fmin(zr, v_bnd[iv + 1]);
                        if (orr <= ol) continue;
                        double ov = orr - ol;
                        for (int iu2 = 0; iu2 < nu; iu2++)
                            if (tmp[iu2] != 0.0) s[(size_t)iu2 * nv + iv] += tmp[iu2] * ov;
                    }
                }
            }
            double f = d_pix * d_pix / (du * dv);
            for (size_t i = 0; i < (size_t)nu * nv; i++) s[i] *= f;
        }
        free(pu); free(tmp);
        dd_view_free(&g);
    }
    free(u_bnd); free(v_bnd); free(z_bnd);
}

/* _dd_bp_cone_sweep (dd.py:384-468): per (io, iz, iv) with v overlap, a full
 * u merge distributing sino * overlap_u * overlap_v * scale; returns
 * img / na / d_pix (dd.py:884-886). */
void orc_dd_bp_cone(const float *sino, int na, int nu, int nv, const double *cosv,
                    const double *sinv, int nx, int ny, int nz, double du,
                    double dv, double su, double sv, double d_pix, double DSO,
                    double DSD, double *vol)
{
    double *u_bnd = dd_u_bounds(nu, du, su);
    double *v_bnd = dd_u_bounds(nv, dv, sv);
    double *z_bnd = (double *)malloc(sizeof(double) * (nz + 1));
    for (int i = 0; i <= nz; i++) z_bnd[i] = d_pix * ((double)i - nz / 2.0);
    size_t nvox = (size_t)nx * ny * nz;
    memset(vol, 0, sizeof(double) * nvox);
    dd_view g;
    dd_view_alloc(&g, nx, ny);
    for (int ia = 0; ia < na; ia++) {
        dd_view_setup(&g, 1, nx, ny, d_pix, cosv[ia], sinv[ia], DSO);
        const float *s = sino + (size_t)ia * nu * nv;
        int no = g.no;
#pragma omp parallel
        {
            int m = (nx > ny ? nx : ny) + 1;
            double *pu = (double *)malloc(sizeof(double) * m);
#pragma omp for schedule(dynamic)
            for (int io = 0; io < no; io++) {
                double scl = g.scl[io];
                double zmag = DSD / (DSO - g.o_orth[io]);
                cone_line_u(&g, io, DSO, DSD, pu);
                for (int iz = 0; iz < nz; iz++) {
                    double zl = zmag * z_bnd[iz], zr = zmag * z_bnd[iz + 1];
                    for (int iv = 0; iv < nv; iv++) {
                        double ol = fmax(zl, v_bnd[iv]), orr = fmin(zr, v_bnd[iv + 1]);
                        if (orr <= ol) continue;
                        double ov = orr - ol;
                        int ip = 0, iu = 0;
                        while (ip < g.np_ && iu < nu) {
                            double a = fmax(pu[ip], u_bnd[iu]), b = fmin(pu[ip + 1], u_bnd[iu + 1]);
                            if (b > a) vol[cone_vox(&g, ip, io, iz, ny, nz)] += s[(size_t)iu * nv + iv] * (b - a) * ov * scl;
                            if (pu[ip + 1] < u_bnd[iu + 1]) ip++; else iu++;
                        }
                    }
                }
            }
            free(pu);
        }
    }
    dd_view_free(&g);
    for (size_t i = 0; i < nvox; i++) vol[i] = vol[i] / na / d_pix;
    free(u_bnd); free(v_bnd); free(z_bnd);
}

/* ------------------------------------------------------------------------ */
/* Translational "square" geometry, sys_mat/dd.py:895-1313                   */
/* ------------------------------------------------------------------------ */

/* Geometry of dd_fp_square / dd_bp_square.  prm holds, in this order:
 * DSO, DSD, du, dv, dsrc_p, dsrc_z, su, sv, ssrc_p, ssrc_z, d_pix.
 * Grids follow pf.boundspace / pf.censpace (pf.py:43-56): boundaries
 * d*(k - n/2) + s, centres d*(k - (n-1)/2) + s.  The object is n x n x nz
 * (x, y, z; z fastest); for side s the voxel in the side's frame (io: the
 * orthogonal slab, ip: the parallel index) is the image voxel below
 * (dd.py:1004-1007 + 1042-1045 for the forward, 1264-1267 + 1132-1135 for
 * the back projection: imgX/imgY transposes and their flipped slices). */
typedef struct {
    int n, nz, nu, nv, nsp, nsz;
    double DSO, DSD, du, dv, dsp, dsz, su, sv, ssp, ssz, d_pix;
} sq_geom;

static sq_geom sq_make(const int *dims, const double *prm)
{
    sq_geom g;
    g.n = dims[0]; g.nz = dims[1]; g.nu = dims[2]; g.nv = dims[3];
    g.nsp = dims[4]; g.nsz = dims[5];
    g.DSO = prm[0]; g.DSD = prm[1]; g.du = prm[2]; g.dv = prm[3]; g.dsp = prm[4];
    g.dsz = prm[5]; g.su = prm[6]; g.sv = prm[7]; g.ssp = prm[8]; g.ssz = prm[9];
    g.d_pix = prm[10];
    return g;
}

static inline size_t sq_vox(const sq_geom *g, int side, int io, int ip, int iz)
{
    int n = g->n, ix, iy;
    switch (side) {
    case 0: ix = io; iy = ip; break;                  /* imgY[io, iz, ip]           */
    case 1: ix = n - 1 - ip; iy = io; break;          /* imgX[io, iz, nP-1-ip]      */
    case 2: ix = n - 1 - io; iy = n - 1 - ip; break;  /* imgY[no-1-io, iz, nP-1-ip] */
    default: ix = ip; iy = n - 1 - io; break;         /* imgX[no-1-io, iz, ip]      */
    }
    return ((size_t)ix * n + iy) * g->nz + iz;
}

/* Magnification of slab io: DSD / (DSO - o_bnd[io]), the slab's lower
 * boundary (dd.py:972 and 1179, M_arr indexed by io). */
static inline double sq_mag(const sq_geom *g, int io)
{
    double o = g->d_pix * ((double)io - g->n / 2.0);
    return g->DSD / (g->DSO - o);
}

/* Overlap of [a0, a1] with detector cell k of a boundary grid (b0, d): the
 * index range is widened by one on each side and the overlaps are clamped,
 * so rounding of the estimate cannot drop a cell. */
static inline void sq_range(double a0, double a1, double b0, double d, int n, int *lo, int *hi)
{
    double f0 = floor((a0 - b0) / d) - 1.0, f1 = floor((a1 - b0) / d) + 2.0;
    if (f0 < 0.0) f0 = 0.0;
    if (f1 > n) f1 = n;
    *lo = (int)f0;
    *hi = f1 > f0 ? (int)f1 : (int)f0;
}

/* dd_fp_translational (dd.py:959-1100): per source column i_sp, slab io
 * (skipped when M <= 0, :987-989) and z slice iz, the u overlaps of the
 * projected parallel boundaries M*p_bnd - (M*src_p - ssrc_p) with the u
 * boundaries fill tmp_u[iu][side] (:1028-1059); each source row i_sz then
 * spreads tmp_u over the v overlaps of M*z_bnd - (M*src_z - ssrc_z)
 * (:1061-1098).  Returns sino[i_sp][i_sz][iv][iu][side] * d_pix^2 / (du dv)
 * (dd.py:930). */
void orc_dd_fp_square(const float *img, const int *dims, const double *prm, double *sino)
{
    sq_geom g = sq_make(dims, prm);
    int n = g.n, nz = g.nz, nu = g.nu, nv = g.nv;
    double u0 = g.du * (0.0 - nu / 2.0) + (g.su + g.ssp);
    double v0 = g.dv * (0.0 - nv / 2.0) + (g.sv + g.ssz);
    size_t per_sp = (size_t)g.nsz * nv * nu * 4;
    memset(sino, 0, sizeof(double) * per_sp * g.nsp);
#pragma omp parallel
    {
        double *tmp = (double *)malloc(sizeof(double) * nu * 4);
#pragma omp for schedule(dynamic)
        for (int isp = 0; isp < g.nsp; isp++) {
            double src_p = g.dsp * ((double)isp - (g.nsp - 1) * 0.5) + g.ssp;
            for (int io = 0; io < n; io++) {
                double M = sq_mag(&g, io);
                if (!(M > 0.0)) continue;
                double cp = M * src_p - g.ssp;
                for (int iz = 0; iz < nz; iz++) {
                    memset(tmp, 0, sizeof(double) * nu * 4);
                    for (int ip = 0; ip < n; ip++) {
                        double pl = M * (g.d_pix * ((double)ip - n / 2.0)) - cp;
                        double pr = M * (g.d_pix * ((double)(ip + 1) - n / 2.0)) - cp;
                        int lo, hi;
                        sq_range(pl, pr, u0, g.du, nu, &lo, &hi);
                        double val[4];
                        for (int s = 0; s < 4; s++) val[s] = img[sq_vox(&g, s, io, ip, iz)];
                        for (int iu = lo; iu < hi; iu++) {
                            double ov = fmin(pr, u0 + g.du * (iu + 1)) - fmax(pl, u0 + g.du * iu);
                            if (ov <= 0.0) continue;
                            for (int s = 0; s < 4; s++) tmp[iu * 4 + s] += val[s] * ov;
                        }
                    }
                    for (int isz = 0; isz < g.nsz; isz++) {
                        double src_z = g.dsz * ((double)isz - (g.nsz - 1) * 0.5) + g.ssz;
                        double cz = M * src_z - g.ssz;
                        double zl = M * (g.d_pix * ((double)iz - nz / 2.0)) - cz;
                        double zr = M * (g.d_pix * ((double)(iz + 1) - nz / 2.0)) - cz;
                        int lo, hi;
                        sq_range(zl, zr, v0, g.dv, nv, &lo, &hi);
                        double *base = sino + (size_t)isp * per_sp + (size_t)isz * nv * nu * 4;
                        for (int iv = lo; iv < hi; iv++) {
                            double ov = fmin(zr, v0 + g.dv * (iv + 1)) - fmax(zl, v0 + g.dv * iv);
                            if (ov <= 0.0) continue;
                            double *row = base + (size_t)iv * nu * 4;
                            for (int k = 0; k < nu * 4; k++) row[k] += tmp[k] * ov;
                        }
                    }
                }
            }
        }
        free(tmp);
    }
    double f = g.d_pix * g.d_pix / (g.du * g.dv);
    for (size_t i = 0; i < per_sp * g.nsp; i++) sino[i] *= f;
}

/* dd_bp_translational (dd.py:1164-1313): per slab io (skipped when M <= 0),
 * source column i_sp and z slice iz, tmp_v[iu][side] collects the sinogram
 * rows weighted by their v overlaps over every source row (:1194-1253); each
 * parallel voxel then takes the u-overlap-weighted sum of tmp_v
 * (:1270-1313).  The four sides accumulate in separate planes (one slab per
 * thread, no shared writes) and are summed as (side0 + side2) + (side1 +
 * side3), the imgX + imgY of dd.py:1135.  No output scaling (dd.py:1135). */
void orc_dd_bp_square(const float *sino, const int *dims, const double *prm, double *img)
{
    sq_geom g = sq_make(dims, prm);
    int n = g.n, nz = g.nz, nu = g.nu, nv = g.nv;
    double u0 = g.du * (0.0 - nu / 2.0) + (g.su + g.ssp);
    double v0 = g.dv * (0.0 - nv / 2.0) + (g.sv + g.ssz);
    size_t nvox = (size_t)n * n * nz;
    size_t per_sp = (size_t)g.nsz * nv * nu * 4;
    double *pl4 = (double *)calloc(4 * nvox, sizeof(double));
#pragma omp parallel
    {
        double *tmp = (double *)malloc(sizeof(double) * nu * 4);
#pragma omp for schedule(dynamic)
        for (int io = 0; io < n; io++) {
            double M = sq_mag(&g, io);
            if (!(M > 0.0)) continue;
            for (int isp = 0; isp < g.nsp; isp++) {
                double src_p = g.dsp * ((double)isp - (g.nsp - 1) * 0.5) + g.ssp;
                double cp = M * src_p - g.ssp;
                for (int iz = 0; iz < nz; iz++) {
                    memset(tmp, 0, sizeof(double) * nu * 4);
                    for (int isz = 0; isz < g.nsz; isz++) {
                        double src_z = g.dsz * ((double)isz - (g.nsz - 1) * 0.5) + g.ssz;
                        double cz = M * src_z - g.ssz;
                        double zl = M * (g.d_pix * ((double)iz - nz / 2.0)) - cz;
                        double zr = M * (g.d_pix * ((double)(iz + 1) - nz / 2.0)) - cz;
                        int lo, hi;
                        sq_range(zl, zr, v0, g.dv, nv, &lo, &hi);
                        const float *base = sino + (size_t)isp * per_sp + (size_t)isz * nv * nu * 4;
                        for (int iv = lo; iv < hi; iv++) {
                            double ov = fmin(zr, v0 + g.dv * (iv + 1)) - fmax(zl, v0 + g.dv * iv);
                            if (ov <= 0.0) continue;
                            const float *row = base + (size_t)iv * nu * 4;
                            for (int k = 0; k < nu * 4; k++) tmp[k] += row[k] * ov;
                        }
                    }
                    for (int ip = 0; ip < n; ip++) {
                        double pl = M * (g.d_pix * ((double)ip - n / 2.0)) - cp;
                        double pr = M * (g.d_pix * ((double)(ip + 1) - n / 2.0)) - cp;
                        int lo, hi;
                        sq_range(pl, pr, u0, g.du, nu, &lo, &hi);
                        double acc[4] = {0.0, 0.0, 0.0, 0.0};
                        for (int iu = lo; iu < hi; iu++) {
                            double ov = fmin(pr, u0 + g.du * (iu + 1)) - fmax(pl, u0 + g.du * iu);
                            if (ov <= 0.0) continue;
                            for (int s = 0; s < 4; s++) acc[s] += tmp[iu * 4 + s] * ov;
                        }
                        for (int s = 0; s < 4; s++)
                            pl4[(size_t)s * nvox + sq_vox(&g, s, io, ip, iz)] += acc[s];
                    }
                }
            }
        }
        free(tmp);
    }
    for (size_t i = 0; i < nvox; i++)
        img[i] = (pl4[i] + pl4[2 * nvox + i]) + (pl4[nvox + i] + pl4[3 * nvox + i]);
    free(pl4);
}

/* ------------------------------------------------------------------------ */
/* Separable footprint, sys_mat/sp.py:12-87 and sys_mat/fp_2d_par.py:67-125  */
/* ------------------------------------------------------------------------ */

/* sp.sf_fp_fan_2d: per pixel the linear B-spline footprint of half width
 * DSD*d_pix/(DSO - yp) centred at DSD*xp/(DSO - yp), sampled at bin centres;
 * returns sino * d_pix.  transpose != 0 computes the exact adjoint
 * img[ix,iy] = d_pix * sum sino * w (no counterpart in the reference). */
void orc_sf_fan_2d(int transpose, const float *in, double *out, int nx, int ny,
                   const double *cosv, const double *sinv, int na, int nu,
                   double DSO, double DSD, double du, double d_pix)
{
    if (transpose) memset(out, 0, sizeof(double) * (size_t)nx * ny);
    else memset(out, 0, sizeof(double) * (size_t)na * nu);
    for (int ia = 0; ia < na; ia++) {
        double c = cosv[ia], s = sinv[ia];
#pragma omp parallel for schedule(static)
        for (int ix = 0; ix < nx; ix++) {
            double x = d_pix * ((double)ix - nx / 2.0 + 0.5);
            for (int iy = 0; iy < ny; iy++) {
                double y = d_pix * ((double)iy - ny / 2.0 + 0.5);
                double val = transpose ? 0.0 : in[(size_t)ix * ny + iy];
                if (!transpose && val == 0.0) continue;
                double xp = c * x + s * y, yp = -s * x + c * y;
                double u0 = DSD * xp / (DSO - yp);
                double w_fp = DSD * d_pix / (DSO - yp);
                double umin = u0 - w_fp, umax = u0 + w_fp;
                int iu0 = (int)floor((umin / du) + nu / 2.0);
                int iu1 = (int)ceil((umax / du) + nu / 2.0);
                double acc = 0.0;
                for (int iu = iu0; iu <= iu1; iu++) {
                    if (iu < 0 || iu >= nu) continue;
                    double uc = du * ((double)iu - nu / 2.0 + 0.5);
                    double t = (uc - u0) / w_fp;
                    double w = fmax(0.0, 1.0 - fabs(t));
                    if (transpose) acc += in[(size_t)ia * nu + iu] * w;
                    else {
#pragma omp atomic
                        out[(size_t)ia * nu + iu] += val * w;
                    }
                }
                if (transpose) out[(size_t)ix * ny + iy] += acc;
            }
        }
    }
    size_t n = transpose ? (size_t)nx * ny : (size_t)na * nu;
    for (size_t i = 0; i < n; i++) out[i] *= d_pix;
}

/* fp_2d_par.separable_footprint_fp_2d: each pixel's footprint is the interval
 * spanned by its four projected corners cos*y - sin*x (:105-109); its overlap
 * with each bin, divided by d_det, weights the pixel value (:114-123).
 * transpose != 0 computes the exact adjoint. */
void orc_sf_par_rect_2d(int transpose, const float *in, double *out, int nx,
                        int ny, const double *cosv, const double *sinv, int na,
                        int n_dets, double d_det, double d_pix)
{
    double *db = (double *)malloc(sizeof(double) * (n_dets + 1));
    for (int i = 0; i <= n_dets; i++) db[i] = d_det * ((double)i - n_dets / 2.0);
    if (transpose) memset(out, 0, sizeof(double) * (size_t)nx * ny);
    else memset(out, 0, sizeof(double) * (size_t)na * n_dets);
    for (int ia = 0; ia < na; ia++) {
        double c = cosv[ia], s = sinv[ia];
#pragma omp parallel for schedule(static)
        for (int ix = 0; ix < nx; ix++) {
            double xmin = d_pix * ((double)ix - nx / 2.0), xmax = d_pix * ((double)(ix + 1) - nx / 2.0);
            for (int iy = 0; iy < ny; iy++) {
                double ymin = d_pix * ((double)iy - ny / 2.0), ymax = d_pix * ((double)(iy + 1) - ny / 2.0);
                double val = transpose ? 0.0 : in[(size_t)ix * ny + iy];
                if (!transpose && val == 0.0) continue;
                double cr[4] = {c * ymin - s * xmin, c * ymax - s * xmin,
                                c * ymin - s * xmax, c * ymax - s * xmax};
                double pmin = cr[0], pmax = cr[0];
                for (int q = 1; q < 4; q++) { pmin = fmin(pmin, cr[q]); pmax = fmax(pmax, cr[q]); }
                /* searchsorted(db, pmin, 'right') - 1 and searchsorted(db, pmax, 'left') */
                int i0 = 0;
                while (i0 <= n_dets && db[i0] <= pmin) i0++;
                i0 -= 1;
                int iN = 0;
                while (iN <= n_dets && db[iN] < pmax) iN++;
                double acc = 0.0;
                int lo = i0 > 0 ? i0 : 0, hi = iN < n_dets ? iN : n_dets;
                for (int k = lo; k < hi; k++) {
                    double l = fmax(pmin, db[k]), r = fmin(pmax, db[k + 1]);
                    if (r > l) {
                        double w = (r - l) / d_det;
                        if (transpose) acc += in[(size_t)ia * n_dets + k] * w;
                        else {
#pragma omp atomic
                            out[(size_t)ia * n_dets + k] += val * w;
                        }
                    }
                }
                if (transpose) out[(size_t)ix * ny + iy] += acc;
            }
        }
    }
    free(db);
}

/* ------------------------------------------------------------------------ */
/* Siddon list projection, projection/projection_c.c:126-219                 */
/* ------------------------------------------------------------------------ */

/* Gather FP over a flat CSR list (ind, len, off): sino[r] = sum x[ind]*len. */
void orc_list_fp(const float *x, const int32_t *ind, const float *len,
                 const int32_t *off, int nrays, double *sino)
{
#pragma omp parallel for schedule(dynamic, 256)
    for (int r = 0; r < nrays; r++) {
        double a = 0.0;
        for (int32_t i = off[r]; i < off[r + 1]; i++) a += (double)x[ind[i]] * len[i];
        sino[r] = a;
    }
}

/* Scatter BP over the same list: x[ind] += sino[r]*len (np.add.at semantics,
 * repeated indices accumulate, unlike proj.sd_b_proj's fancy-index +=). */
void orc_list_bp(const float *sino, const int32_t *ind, const float *len,
                 const int32_t *off, int nrays, int nvox, double *x)
{
    memset(x, 0, sizeof(double) * (size_t)nvox);
    for (int r = 0; r < nrays; r++)
        for (int32_t i = off[r]; i < off[r + 1]; i++) x[ind[i]] += (double)sino[r] * len[i];
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
