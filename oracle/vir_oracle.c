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

/* ------------------------------------------------------------------------ */
/* Ray-driven Amanatides-Woo and Joseph, sys_mat/rd.py:40-790                */
/* ------------------------------------------------------------------------ */

#define RD_EPS 1e-6 /* rd.py:42 */

/* _img_bounds (rd.py:46-49): boundaries -+ d n / 2, first centre. */
static void rd_bounds(int n, double d, double *lo, double *hi, double *c0)
{
    *lo = -d * n / 2.0; *hi = d * n / 2.0; *c0 = -d * (n / 2.0 - 0.5);
}

/* _intersect_bounding (rd.py:52-64), with the axis-parallel case fixed: the
 * reference returns (-inf, inf) for a ray parallel to the slab wherever it
 * lies, so rays beside the image walk its edge row (the over-count of
 * axis-aligned views); here such a ray meets the slab only when
 * r_min <= r0 < r_max. */
static void rd_bound(double r0, double dr, double lo, double hi, double *t0, double *t1)
{
    if (fabs(dr) > RD_EPS) {
        double a = (lo - r0) / dr, b = (hi - r0) / dr;
        *t0 = fmin(a, b); *t1 = fmax(a, b);
    } else if (r0 >= lo && r0 < hi) {
        *t0 = -INFINITY; *t1 = INFINITY;
    } else {
        *t0 = INFINITY; *t1 = -INFINITY;
    }
}

/* _calc_ir0 (rd.py:67-74) */
static int rd_ir0(double org, double hat, double t, double lo, double hi, double d)
{
    double r = org + t * hat;
    r = fmin(fmax(r, lo + RD_EPS), hi - RD_EPS);
    return (int)floor((r - lo) / d);
}

/* _fp_step_init (rd.py:77-109) */
static void rd_step(double r0, int ir, double dr, double lo, double d, int *dir, double *ts,
                    double *tn)
{
    double rn;
    if (dr > 0) { *dir = 1; rn = lo + (ir + 1) * d; }
    else { *dir = -1; rn = lo + ir * d; }
    if (fabs(dr) > RD_EPS) { *ts = d / fabs(dr); *tn = (rn - r0) / dr; }
    else { *ts = INFINITY; *tn = INFINITY; }
}

typedef struct { double org[3], hat[3]; } rd_ray;

/* One ray of the 2D (dim 2) or 3D (dim 3) projectors.  joseph = 0: the
 * Amanatides-Woo walk of _aw_{fp,bp}_traverse_{2d,3d} (rd.py:112-248);
 * joseph = 1: the 0.5-step sampling of _joseph_{fp,bp}_{2d,3d}
 * (rd.py:251-447).  bp = 0 returns the line integral of img; bp = 1 adds
 * s_val times the ray's weights into bimg. */
static double rd_trace(int dim, int joseph, const rd_ray *R, const float *img, double *bimg,
                       double s_val, const int *n, double d)
{
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, c0[3] = {0, 0, 0};
    double te = -INFINITY, tx = INFINITY;
    for (int a = 0; a < dim; a++) {
        double t0, t1;
        rd_bounds(n[a], d, &lo[a], &hi[a], &c0[a]);
        rd_bound(R->org[a], R->hat[a], lo[a], hi[a], &t0, &t1);
        te = fmax(te, t0); tx = fmin(tx, t1);
    }
    if (tx <= te) return 0.0;
    size_t sy = dim == 3 ? (size_t)n[2] : 1, sx = (size_t)n[1] * sy;
    double acc = 0.0;
    if (joseph) {
        const double step = 0.5;
        for (double t = te; t <= tx; t += step) {
            double f[3];
            for (int a = 0; a < dim; a++) f[a] = (R->org[a] + t * R->hat[a] - c0[a]) / d;
            if (dim == 2 && !bimg) {               /* rd.py:269-289: clamped bilinear */
                double fx = fmin(fmax(f[0], 0.0), n[0] - 2.0), fy = fmin(fmax(f[1], 0.0), n[1] - 2.0);
                int ix = (int)fx, iy = (int)fy;
                double dx = fx - ix, dy = fy - iy;
                size_t b = ix * sx + iy;
                acc += (img[b] * (1 - dx) * (1 - dy) + img[b + sx] * dx * (1 - dy) +
                        img[b + 1] * (1 - dx) * dy + img[b + sx + 1] * dx * dy) * step;
            } else if (dim == 3 && !bimg) {        /* rd.py:301-350: truncation, interior only */
                int ix = (int)f[0], iy = (int)f[1], iz = (int)f[2];
                if (0 <= ix && ix < n[0] - 1 && 0 <= iy && iy < n[1] - 1 && 0 <= iz && iz < n[2] - 1) {
                    double dx = f[0] - ix, dy = f[1] - iy, dz = f[2] - iz;
                    size_t b = ix * sx + iy * sy + iz;
                    double c00 = img[b] + dx * (img[b + sx] - img[b]);
                    double c10 = img[b + sy] + dx * (img[b + sx + sy] - img[b + sy]);
                    double c01 = img[b + 1] + dx * (img[b + sx + 1] - img[b + 1]);
                    double c11 = img[b + sy + 1] + dx * (img[b + sx + sy + 1] - img[b + sy + 1]);
                    double c0v = c00 + dy * (c10 - c00), c1v = c01 + dy * (c11 - c01);
                    acc += (c0v + dz * (c1v - c0v)) * step;
                }
            } else {                               /* rd.py:357-447: floor, splat in bounds */
                int i0[3] = {0, 0, 0};
                double w0[3] = {1, 1, 1};
                for (int a = 0; a < dim; a++) { i0[a] = (int)floor(f[a]); w0[a] = f[a] - i0[a]; }
                for (int c = 0; c < (1 << dim); c++) {
                    double w = s_val * step;
                    int ok = 1;
                    size_t off = 0;
                    for (int a = 0; a < dim; a++) {
                        int bit = (c >> a) & 1, i = i0[a] + bit;
                        if (i < 0 || i >= n[a]) ok = 0;
                        w *= bit ? w0[a] : 1 - w0[a];
                        off += (size_t)i * (a == 0 ? sx : (a == 1 ? sy : 1));
                    }
                    if (ok) bimg[off] += w;
                }
            }
        }
        return acc;
    }
    int ir[3] = {0, 0, 0}, dir[3] = {0, 0, 0};
    double ts[3] = {INFINITY, INFINITY, INFINITY}, tn[3] = {INFINITY, INFINITY, INFINITY};
    for (int a = 0; a < dim; a++) {
        ir[a] = rd_ir0(R->org[a], R->hat[a], te, lo[a], hi[a], d);
        if (ir[a] < 0) ir[a] = 0;                  /* entry voxel inside the grid */
        if (ir[a] > n[a] - 1) ir[a] = n[a] - 1;
        rd_step(R->org[a], ir[a], R->hat[a], lo[a], d, &dir[a], &ts[a], &tn[a]);
        if (dim == 2) tn[a] = fmax(tn[a], te);     /* rd.py:116-117, 155-156 */
    }
    double t = te;
    /* 2D FP walks while t <= t_exit (rd.py:126), the others while t < t_exit */
    while (dim == 2 && !bimg ? t <= tx : t < tx) {
        int out = 0;
        for (int a = 0; a < dim; a++) out |= ir[a] < 0 || ir[a] >= n[a];
        if (out) break;
        int a = 0;
        if (dim == 2) a = tn[0] <= tn[1] ? 0 : 1;
        else a = (tn[0] <= tn[1] && tn[0] <= tn[2]) ? 0 : (tn[1] <= tn[2] ? 1 : 2);
        double tnext = fmin(tn[a], tx);
        size_t v = ir[0] * sx + ir[1] * sy + (dim == 3 ? (size_t)ir[2] : 0);
        if (bimg) bimg[v] += s_val * (tnext - t);
        else acc += img[v] * (tnext - t);
        t = tnext;
        tn[a] += ts[a];
        ir[a] += dir[a];
    }
    return acc;
}

/* aw_p_par_2d / aw_p_fan_2d (rd.py:473-541, 567-649).  bp = 0: in = img
 * (nx, ny) -> out = sino (na, nu); bp = 1: in = sino -> out = img, scaled
 * img / na / d_pix / d_pix * du (rd.py:538, 646). */
void orc_rd_2d(int fan, int joseph, int bp, const float *in, double *out, int nx, int ny,
               int na, int nu, const double *cosv, const double *sinv, double du, double su,
               double d_pix, double DSO, double DSD)
{
    int n[2] = {nx, ny};
    if (bp) memset(out, 0, sizeof(double) * (size_t)nx * ny);
    for (int ia = 0; ia < na; ia++) {
        double c = cosv[ia], s = sinv[ia];
        for (int iu = 0; iu < nu; iu++) {
            double u = du * ((double)iu - (nu / 2.0 - 0.5) + su);
            rd_ray R;
            if (fan) {
                R.org[0] = DSO * c; R.org[1] = DSO * s;
                double dx = -(DSD - DSO) * c + u * -s - R.org[0];
                double dy = -(DSD - DSO) * s + u * c - R.org[1];
                double m = sqrt(dx * dx + dy * dy);
                R.hat[0] = dx / m; R.hat[1] = dy / m;
            } else {
                R.org[0] = u * -s; R.org[1] = u * c;
                R.hat[0] = c; R.hat[1] = s;
            }
            if (bp) rd_trace(2, joseph, &R, NULL, out, in[(size_t)ia * nu + iu], n, d_pix);
            else out[(size_t)ia * nu + iu] = rd_trace(2, joseph, &R, in, NULL, 0.0, n, d_pix);
        }
    }
    if (bp)
        for (size_t i = 0; i < (size_t)nx * ny; i++) out[i] = out[i] / na / d_pix / d_pix * du;
}

/* aw_p_cone_3d (rd.py:678-790).  The AW forward value is scaled by
 * DSD / sqrt(DSD^2 + u^2 + v^2) (rd.py:782-783); the back projection
 * returns img / na * du * dv (rd.py:786).  Detector rows are
 * dv (iv - (nv/2 - 0.5) + sv): the reference writes nu for nv here
 * (rd.py:688), which shifts the rows whenever nu != nv. */
void orc_rd_cone(int joseph, int bp, const float *in, double *out, int nx, int ny, int nz,
                 int na, int nu, int nv, const double *cosv, const double *sinv, double du,
                 double dv, double su, double sv, double d_pix, double DSO, double DSD)
{
    int n[3] = {nx, ny, nz};
    size_t nvox = (size_t)nx * ny * nz;
    if (bp) memset(out, 0, sizeof(double) * nvox);
    for (int ia = 0; ia < na; ia++) {
        double c = cosv[ia], s = sinv[ia];
        for (int iv = 0; iv < nv; iv++) {
            double v = dv * ((double)iv - (nv / 2.0 - 0.5) + sv);
            for (int iu = 0; iu < nu; iu++) {
                double u = du * ((double)iu - (nu / 2.0 - 0.5) + su);
                rd_ray R;
                R.org[0] = DSO * c; R.org[1] = DSO * s; R.org[2] = 0.0;
                double vx = -(DSD - DSO) * c + u * -s - R.org[0];
                double vy = -(DSD - DSO) * s + u * c - R.org[1];
                double vz = v;
                double m = sqrt(vx * vx + vy * vy + vz * vz);
                R.hat[0] = vx / m; R.hat[1] = vy / m; R.hat[2] = vz / m;
                size_t k = ((size_t)ia * nu + iu) * nv + iv;
                if (bp) {
                    rd_trace(3, joseph, &R, NULL, out, in[k], n, d_pix);
                } else {
                    double val = rd_trace(3, joseph, &R, in, NULL, 0.0, n, d_pix);
                    if (!joseph) val *= DSD / sqrt(DSD * DSD + u * u + v * v);
                    out[k] = val;
                }
            }
        }
    }
    if (bp)
        for (size_t i = 0; i < nvox; i++) out[i] = out[i] / na * du * dv;
}

/* ------------------------------------------------------------------------ */
/* Pixel-driven footprints, sys_mat/pd.py:56-480                             */
/* ------------------------------------------------------------------------ */

/* pd_p_par_2d / pd_p_fan_2d (pd.py:148-235, 256-351): each pixel's four
 * corners are projected (parallel: p = -s x + c y; fan: DSD p / (DSO - o));
 * the bins overlapping [p_min, p_max] get value * overlap / du * scale with
 * scale 1 / (|sin| + |cos|) (parallel) or 1 / (|cos(a+g)| + |sin(a+g)|),
 * g = atan(u_c / DSD) of the pixel centre (fan).  FP returns sino * d_pix,
 * BP img / na / d_pix * du.  The reference's fan FP skips zero pixels
 * without advancing oy_bnd_l (pd.py:335-339), so the centre of the next
 * pixel, and its scale, come out wrong after every zero; here every pixel
 * uses its own centre. */
void orc_pd_2d(int fan, int bp, const float *in, double *out, int nx, int ny, int na, int nu,
               const double *angs, double du, double su, double d_pix, double DSO, double DSD)
{
    size_t npix = (size_t)nx * ny;
    if (bp) memset(out, 0, sizeof(double) * npix);
    else memset(out, 0, sizeof(double) * (size_t)na * nu);
    for (int ia = 0; ia < na; ia++) {
        double c = cos(angs[ia]), s = sin(angs[ia]);
        double pscale = 1.0 / (fabs(s) + fabs(c));
        for (int ix = 0; ix < nx; ix++) {
            double xl = d_pix * (ix - nx / 2.0), xr = d_pix * (ix + 1 - nx / 2.0);
            for (int iy = 0; iy < ny; iy++) {
                double yl = d_pix * (iy - ny / 2.0), yr = d_pix * (iy + 1 - ny / 2.0);
                double xs[2] = {xl, xr}, ys[2] = {yl, yr}, p[4];
                double scale = pscale;
                for (int a = 0; a < 2; a++)
                    for (int b = 0; b < 2; b++) {
                        double pp = -s * xs[a] + c * ys[b];
                        if (fan) pp = DSD * pp / (DSO - (c * xs[a] + s * ys[b]));
                        p[2 * b + a] = pp;
                    }
                if (fan) {
                    double xc = 0.5 * (xl + xr), yc = 0.5 * (yl + yr);
                    double uc = DSD * (-s * xc + c * yc) / (DSO - (c * xc + s * yc));
                    double g = atan(uc / DSD);
                    scale = 1.0 / (fabs(cos(angs[ia] + g)) + fabs(sin(angs[ia] + g)));
                }
                double pmin = fmin(fmin(p[0], p[1]), fmin(p[2], p[3]));
                double pmax = fmax(fmax(p[0], p[1]), fmax(p[2], p[3]));
                int iu0 = (int)floor(pmin / du + nu / 2.0 - su); if (iu0 < 0) iu0 = 0;
                int iu1 = (int)ceil(pmax / du + nu / 2.0 - su); if (iu1 > nu) iu1 = nu;
                size_t q = (size_t)ix * ny + iy;
                if (!bp && in[q] == 0.0f) continue;
                double acc = 0.0;
                for (int iu = iu0; iu < iu1; iu++) {
                    double ub0 = du * (iu - nu / 2.0 + su), ub1 = du * (iu + 1 - nu / 2.0 + su);
                    double l = fmax(pmin, ub0), r = fmin(pmax, ub1);
                    if (r <= l) continue;
                    if (bp) acc += in[(size_t)ia * nu + iu] * (r - l) / du * scale;
                    else out[(size_t)ia * nu + iu] += in[q] * scale * (r - l) / du;
                }
                if (bp) out[q] += acc;
            }
        }
    }
    if (bp) for (size_t i = 0; i < npix; i++) out[i] = out[i] / na / d_pix * du;
    else for (size_t i = 0; i < (size_t)na * nu; i++) out[i] *= d_pix;
}

/* pd_p_cone_3d (pd.py:372-480): per column the fan magnification
 * m = DSD / (DSO - o_c) of its centre projects the four corners to
 * u = m (p corner); slices to v = m / cos(g) z, g = atan(u_c / DSD); cells
 * overlapping [u_min, u_max] x [v_min, v_max] get value * du-overlap / du *
 * dv-overlap / dv / (|sin| + |cos|).  FP returns sino * d_pix, BP
 * img / na / d_pix * du * dv. */
void orc_pd_cone(int bp, const float *in, double *out, int nx, int ny, int nz, int na, int nu,
                 int nv, const double *angs, double du, double dv, double su, double sv,
                 double d_pix, double DSO, double DSD)
{
    size_t nvox = (size_t)nx * ny * nz, nsino = (size_t)na * nu * nv;
    memset(out, 0, sizeof(double) * (bp ? nvox : nsino));
    for (int ia = 0; ia < na; ia++) {
        double c = cos(angs[ia]), s = sin(angs[ia]);
        double pscale = 1.0 / (fabs(s) + fabs(c));
        for (int ix = 0; ix < nx; ix++) {
            double xl = d_pix * (ix - nx / 2.0), xr = d_pix * (ix + 1 - nx / 2.0);
            for (int iy = 0; iy < ny; iy++) {
                double yl = d_pix * (iy - ny / 2.0), yr = d_pix * (iy + 1 - ny / 2.0);
                double xc = 0.5 * (xl + xr), yc = 0.5 * (yl + yr);
                double oc = c * xc + s * yc;
                double uc = DSD * (-s * xc + c * yc) / (DSO - oc);
                double g = atan(uc / DSD);
                double fm = DSD / (DSO - oc), cm = fm / cos(g);
                double uu[4] = {fm * (-s * xl + c * yl), fm * (-s * xr + c * yl),
                                fm * (-s * xl + c * yr), fm * (-s * xr + c * yr)};
                double umin = fmin(fmin(uu[0], uu[1]), fmin(uu[2], uu[3]));
                double umax = fmax(fmax(uu[0], uu[1]), fmax(uu[2], uu[3]));
                int iu0 = (int)floor((umin - du * (-nu / 2.0 + su)) / du) - 1;
                int iu1 = (int)floor((umax - du * (-nu / 2.0 + su)) / du) + 2;
                if (iu0 < 0) iu0 = 0;
                if (iu1 > nu) iu1 = nu;
                for (int iz = 0; iz < nz; iz++) {
                    double zl = d_pix * (iz - nz / 2.0), zr = d_pix * (iz + 1 - nz / 2.0);
                    double vmin = fmin(cm * zl, cm * zr), vmax = fmax(cm * zl, cm * zr);
                    int iv0 = (int)floor((vmin - dv * (-nv / 2.0 + sv)) / dv) - 1;
                    int iv1 = (int)floor((vmax - dv * (-nv / 2.0 + sv)) / dv) + 2;
                    if (iv0 < 0) iv0 = 0;
                    if (iv1 > nv) iv1 = nv;
                    size_t q = ((size_t)ix * ny + iy) * nz + iz;
                    if (!bp && in[q] == 0.0f) continue;
                    double acc = 0.0;
                    for (int iv = iv0; iv < iv1; iv++) {
                        double vl = fmax(vmin, dv * (iv - nv / 2.0 + sv));
                        double vr = fmin(vmax, dv * (iv + 1 - nv / 2.0 + sv));
                        if (vr <= vl) continue;
                        for (int iu = iu0; iu < iu1; iu++) {
                            double ul = fmax(umin, du * (iu - nu / 2.0 + su));
                            double ur = fmin(umax, du * (iu + 1 - nu / 2.0 + su));
                            if (ur <= ul) continue;
                            size_t k = ((size_t)ia * nu + iu) * nv + iv;
                            double w = (ur - ul) / du * (vr - vl) / dv;
                            if (bp) acc += in[k] * w * pscale;
                            else out[k] += in[q] * pscale * w;
                        }
                    }
                    if (bp) out[q] += acc;
                }
            }
        }
    }
    if (bp) for (size_t i = 0; i < nvox; i++) out[i] = out[i] / na / d_pix * du * dv;
    else for (size_t i = 0; i < nsino; i++) out[i] *= d_pix;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
