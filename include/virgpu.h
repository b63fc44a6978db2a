/*
 * virgpu.h -- C ABI of libvirgpu.so, the GB300 (sm_103a) projector /
 * backprojector / reconstruction library behind vir_gb300.
 *
 * Conventions shared by every entry point:
 *  - All array arguments are DEVICE pointers (cudaMalloc'd or torch CUDA
 *    storage), C-contiguous, float32 unless stated.  Images are (nx, ny)
 *    x-major (img[ix*ny + iy]) as in vir; volumes (nx, ny, nz); sinograms
 *    (na, nu) or (na, nu, nv) with v fastest (vir's dd.py layout).
 *  - `trig` is a device array of 2*na doubles (cos0, sin0, cos1, sin1, ...):
 *    the per-view trig table, computed by the caller exactly as vir does
 *    (numpy cos/sin in the reference's own angle dtype, widened to double).
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *    Calls are asynchronous and reentrant per stream; outputs are
 *    overwritten, never accumulated, unless a flag says otherwise.
 *  - Every entry point returns an int status (VG_OK = 0) and never aborts;
 *    vg_last_error() returns a message for the calling thread's last failure.
 *
 * Each declaration names the vir interface it replaces (file:line inside the
 * vargasp/vir tree).
 */
#ifndef VIRGPU_H
#define VIRGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    VG_OK = 0,
    VG_ERR_ARG = 1,       /* bad size, null pointer, misaligned buffer */
    VG_ERR_LAUNCH = 2,    /* kernel launch failed */
    VG_ERR_TIMEOUT = 3,   /* a bounded device wait gave up */
    VG_ERR_CANCELLED = 4, /* the host raised the cancel flag */
    VG_ERR_CUDA = 5       /* another CUDA runtime error */
};

/* Library identity and diagnostics. */
int vg_version(void);
const char *vg_last_error(void);
const char *vg_status_string(int status);

/* ---- 2D parallel-beam Siddon ------------------------------------------- */

/* Forward projection along exact ray paths, one thread per ray, FP64
 * geometry (plane crossings merged in FP64 exactly as vir orders them) and
 * Kahan-compensated FP32 sums.  img (nx, ny) -> sino (na, n_dets).
 * Replaces fp_2d_par.siddons_fp_2d (sys_mat/fp_2d_par.py:11-64). */
int vg_siddon2d_fp(const float *img, int nx, int ny, const double *trig, int na,
                   int n_dets, double d_det, double d_pix, float *sino,
                   void *stream);

/* Exact adjoint of vg_siddon2d_fp in gather form (one thread per pixel, the
 * same FP64 segments recomputed per candidate ray; no atomics).
 * sino (na, n_dets) -> img (nx, ny).  Replaces the list backprojector
 * back_proj_ravel_rays_struct (projection/projection_c.c:200-208) for the
 * same geometry, without a stored list. */
int vg_siddon2d_bp(const float *sino, int na, int n_dets, const double *trig,
                   int nx, int ny, double d_det, double d_pix, float *img,
                   void *stream);

/* The same back projection in scatter form: every ray of a chunk of views
 * retraces its segments exactly as vg_siddon2d_fp does and writes y * length
 * into a (view, pixel) slot reserved for it (ray index mod S, S above the
 * number of rays one pixel can meet in a view), then a gather pass sums the
 * slots per pixel in a fixed order.  Deterministic; the segments and lengths
 * are the forward projector's.  Views are processed in chunks that fit the
 * caller's workspace (vg_siddon2d_bp_workspace_bytes: up to 256 MiB, at
 * least one view). */
size_t vg_siddon2d_bp_workspace_bytes(int nx, int ny, int na, double d_det,
                                      double d_pix);
int vg_siddon2d_bp_scatter(const float *sino, int na, int n_dets,
                           const double *trig, int nx, int ny, double d_det,
                           double d_pix, float *img, void *workspace,
                           size_t workspace_bytes, void *stream);

/* Per-ray trace of vg_siddon2d_fp's path (no image): segment count, an
 * order-sensitive 64-bit hash of the voxel indices (h = (h ^ (idx + C1)) *
 * C2, FNV-style, h0 = 0xCBF29CE484222325) and the FP64 sum of lengths, for
 * checking voxel index sequences ray by ray against an FP64 restatement of
 * fp_2d_par.py:22-63.  Arrays are (na, n_dets). */
int vg_siddon2d_trace(int nx, int ny, const double *trig, int na, int n_dets,
                      double d_det, double d_pix, int *count,
                      unsigned long long *hash, double *len, void *stream);

/* Check of the FP64 quotient the Siddon kernels use for plane crossings:
 * q[i] = a[i] / b[i] from the reciprocal RN(1 / b[i]) and one FMA correction
 * (Markstein), which must equal the correctly rounded quotient bit for bit.
 * Device arrays of n doubles; finite operands, b[i] != 0.  No counterpart in
 * vir (a self-check of this library). */
int vg_div_rn_check(const double *a, const double *b, size_t n, double *q, void *stream);

/* ---- Siddon ray lists (3D) ------------------------------------------------ */

/* Per-ray set-up of sys_mat/siddon.py:siddons (:681-751, computed by
 * vg_siddons_setup) and the grid planes; all arrays are device pointers.  src/dst are (n_rays, 3) float32 source and target-source
 * vectors, dist the float32 ray length, amin/amax the alpha range, i0/iN the
 * per-axis plane index range [i0, iN), valid the rays that cross the grid. */
typedef struct {
    int n_rays;
    int nx, ny, nz;
    float dx, dy, dz;
    const float *xb, *yb, *zb;         /* plane coordinates, n + 1 each */
    const float *src, *dst;            /* (n_rays, 3) */
    const float *dist, *amin, *amax;   /* (n_rays) */
    const int *i0, *iN;                /* (n_rays, 3) */
    const unsigned char *valid;        /* (n_rays) */
} vg_siddon_rays;

/* Grid of the per-ray set-up: sizes, float32 pitches, the first and last
 * plane coordinate of each axis (boundspace's float32 planes,
 * core_funcs.py:62-81), and siddons' epsilon as float64 and float32. */
typedef struct {
    int nx, ny, nz;
    float dx, dy, dz;
    float p0[3], pN[3];
    double epsilon;
    float epsilon_f;
    int pad;
} vg_siddons_grid;

/* The per-ray set-up of siddons (sys_mat/siddon.py:681-751) on the device,
 * one thread per ray, each operation in the type numpy gives it: from
 * src / trg ((n, 3) float32, broadcast by the caller) it writes dst = trg -
 * src, dist (np.linalg.norm), the alpha range amin / amax, the per-axis
 * plane index range [i0, iN) as numpy slice bounds, and valid.  Replaces the
 * reference's vectorised numpy set-up; the outputs feed vg_siddon_rays. */
int vg_siddons_setup(const vg_siddons_grid *g, int n, const float *src, const float *trg,
                     float *dst, float *dist, float *amin, float *amax, int *i0, int *iN,
                     unsigned char *valid, void *stream);

/* Pass 1 of siddons (the per-ray loop, sys_mat/siddon.py:754-826): number
 * of kept (voxel, length) entries per ray into counts (n_rays ints); *err
 * (device int, caller-zeroed) is incremented for every ray with a voxel
 * index outside the grid (where the reference's ravel_multi_index raises). */
int vg_siddons_count(const vg_siddon_rays *r, int *counts, int *err,
                     void *stream);

/* Pass 2: the entries themselves, ray by ray at off[ray] (the exclusive scan
 * of the counts): ind = raveled C-order voxel index (int32), len = float32
 * intersection length -- the flat (ind, len, off) form of siddons(flat=True). */
int vg_siddons_fill(const vg_siddon_rays *r, const int *off, int *ind,
                    float *len, void *stream);

/* List forward projection sino[r] (+)= sum_i x[ind[i]] * len[i] over
 * i in [off[r], off[r+1]): forward_proj_ravel_rays_struct
 * (projection/projection_c.c:150-157) and proj.sd_f_proj (proj.py:56-96).
 * One warp per ray, Kahan sums; accumulate != 0 adds to sino like the C. */
int vg_list_fp(const float *x, const int *ind, const float *len,
               const int *off, int nrays, float *sino, int accumulate,
               void *stream);

/* List backprojection x[ind[i]] (+)= sino[r] * len[i]:
 * back_proj_ravel_rays_struct (projection/projection_c.c:200-208), with
 * repeated voxels accumulated (np.add.at semantics).  FP64 atomics into a
 * workspace of vg_list_bp_workspace_bytes(nvox) bytes, then one rounding. */
size_t vg_list_bp_workspace_bytes(int nvox);
int vg_list_bp(const float *sino, const int *ind, const float *len,
               const int *off, int nrays, int nvox, float *x, int accumulate,
               void *workspace, size_t workspace_bytes, void *stream);

/* ---- 2D distance-driven (parallel and flat-detector fan) --------------- */

/* Geometry of one 2D distance-driven call.  fan = 0: parallel
 * (dd.py:472-523); fan = 1: fan beam with source at distance DSO from the
 * isocentre and a flat detector at DSD (dd.py:527-585). */
typedef struct {
    int nx, ny;      /* image */
    int na, nu;      /* views, detector bins */
    float du, su;    /* bin width, detector shift in bins (dd.py:699) */
    float d_pix;     /* pixel width */
    float DSO, DSD;  /* fan only */
    int fan;
    int variant;     /* forward-projector tile variant, 1..vg_dd2d_fp_variants();
                        0 = chosen from the sizes (vg_dd2d_fp_default_variant) */
} vg_dd2d_geom;

/* Number of forward-projector tile variants, and the one variant 0 maps to
 * for a geometry (the autotuner in vir_gb300/autotune.py times the others). */
int vg_dd2d_fp_variants(void);
int vg_dd2d_fp_default_variant(const vg_dd2d_geom *g);

/* Forward projection, gather form (one thread per bin, pixels of each
 * orthogonal line found directly), returns A x * d_pix / du exactly as
 * dd_fp_par_2d / dd_fp_fan_2d (dd.py:651-661, 725; 730-736, 803).
 * img is (nx, ny); imgT is its transpose (ny, nx) (the caller keeps both so
 * that both driving axes read contiguous lines); sino (na, nu). */
int vg_dd2d_fp(const vg_dd2d_geom *g, const float *img, const float *imgT,
               const double *trig, float *sino, void *stream);

/* Bytes of device workspace vg_dd2d_bp and vg_dd2d_sirt_iter need for this
 * geometry (per-view running integrals of the sinogram rows and line
 * scales); 0 for an invalid geometry. */
size_t vg_dd2d_workspace_bytes(const vg_dd2d_geom *g);

/* Backprojection, gather form (one thread per pixel over all views, no
 * atomics), returns A^T y / (na d_pix) exactly as dd_bp_par_2d /
 * dd_bp_fan_2d (dd.py:666-672, 721-723; 739-745, 799-801).  `workspace` is
 * caller-owned device memory of at least vg_dd2d_workspace_bytes(g) bytes,
 * 256-byte aligned; its contents need no initialisation. */
int vg_dd2d_bp(const vg_dd2d_geom *g, const float *sino, const double *trig,
               float *img, void *workspace, size_t workspace_bytes,
               void *stream);

/* vg_dd2d_bp without a caller workspace, for callers that cannot allocate
 * device memory when they call (a host that owns a fixed memory budget, a
 * loop that cannot afford cudaMalloc's implicit synchronisation, a plugin
 * host that forbids allocation in callbacks).  No counterpart in vir: it is
 * an addition of this library.  The workspace is a fixed 32 MiB array in
 * the library's device memory (vg_dd2d_noalloc_scratch_bytes()), held on
 * every device that loads the library until exit; geometries needing more
 * are rejected with VG_ERR_ARG.  The first call in a CUDA context (that
 * context current; normally a device's primary context) looks the array's
 * address up, caches it under the context's process-unique id (cuCtxGetId),
 * and should come before any stream capture; a context made later (after a
 * device reset, or a non-primary one) gets its own lookup.  All calls share
 * the array: calls that overlap on the GPU race.  Nothing in the array needs
 * clearing between calls. */
int vg_dd2d_bp_noalloc(const vg_dd2d_geom *g, const float *sino,
                       const double *trig, float *img, void *stream);
size_t vg_dd2d_noalloc_scratch_bytes(void);

/* One SIRT update on the same projector pair, both halves fused
 * (sys_mat/sirt_dd.py:51-72):
 *   r   = (y - FP x) * inv_w_sino  (FP x kept where inv_w_sino == 0)
 *   x  += gamma * (BP r) * inv_w_img (BP r kept where inv_w_img == 0)
 * inv_w_* hold 1/W (0 where W == 0).  r is a caller scratch sinogram; x and
 * xT (its transpose) are updated in place. */
int vg_dd2d_sirt_iter(const vg_dd2d_geom *g, const float *y,
                      const float *inv_w_sino, const float *inv_w_img,
                      float gamma, const double *trig, float *x, float *xT,
                      float *r, void *workspace, size_t workspace_bytes,
                      void *stream);

/* The two halves of vg_dd2d_sirt_iter, launched exactly as it launches them
 * (vg_dd2d_sirt_iter is vg_dd2d_sirt_residual then vg_dd2d_sirt_update on
 * the same stream and workspace), for callers that time them or put other
 * work between them:
 *   vg_dd2d_sirt_residual: r = (y - FP x) * inv_w_sino (sirt_dd.py:51-62);
 *     when the forward projection's block holds whole views, it also writes
 *     the back projection's tables of r into the workspace;
 *   vg_dd2d_sirt_update: x += gamma * (BP r) * inv_w_img (sirt_dd.py:64-72),
 *     x and xT in place; it builds r's tables itself where the residual
 *     launch did not. */
int vg_dd2d_sirt_residual(const vg_dd2d_geom *g, const float *y, const float *inv_w_sino,
                          const double *trig, const float *x, const float *xT, float *r,
                          void *workspace, size_t workspace_bytes, void *stream);
int vg_dd2d_sirt_update(const vg_dd2d_geom *g, const float *inv_w_img, float gamma,
                        const double *trig, float *x, float *xT, const float *r,
                        void *workspace, size_t workspace_bytes, void *stream);

/* Kernel launches vg_dd2d_sirt_iter makes per update for this geometry: 2
 * when the forward projection's epilogue writes the back projection's
 * tables (one block of 8 warps holds all bins of a view), else 3; 0 for a
 * geometry vg_dd2d_sirt_iter rejects. */
int vg_dd2d_sirt_launches(const vg_dd2d_geom *g);

/* ---- batched SIRT: many 2D problems in one persistent launch ----------- */

/* One problem of a batch: its geometry and device buffers.  x, xT (the
 * iterate and its transpose, (nx, ny) / (ny, nx)) and y (the measured
 * sinogram) are float32, or bfloat16 when the run's storage flag says so;
 * arithmetic is float32 throughout.  inv_w_* hold 1/W (0 where W == 0), r is
 * a residual scratch (na, nu) float32, workspace has
 * vg_dd2d_workspace_bytes(&g) bytes, 256-byte aligned. */
typedef struct {
    vg_dd2d_geom g;
    const void *y;
    const float *inv_w_sino;
    const float *inv_w_img;
    const double *trig;
    void *x;
    void *xT;
    float *r;
    void *workspace;
    float gamma;
    int pad;
} vg_sirt2d_problem;

/* Device control block of a run (40 bytes, zeroed by vg_sirt2d_batch_run):
 * status (VG_OK, VG_ERR_CANCELLED or VG_ERR_TIMEOUT) and the number of
 * updates every problem completed (done) are valid once the run's stream has
 * reached its end; the other fields are the run's own. */
typedef struct {
    unsigned long long next;
    int status, done;
    int stop_p, checked;
    unsigned exited, pad;
    unsigned long long t0;
} vg_sirt2d_batch_ctrl;

/* Host-only: the work items of a batch (problems on the host): forward
 * projection items (problem, view * chunks + chunk), table items (problem,
 * view) and back projection items (problem, pixel tile), int pairs, in
 * problem order (any order is valid; ordering by decreasing cost balances
 * the blocks).  With null item arrays only the counts are returned. */
int vg_sirt2d_batch_items(const vg_sirt2d_problem *probs, int n, int *fp_items, int *n_fp,
                          int *tab_items, int *n_tab, int *bp_items, int *n_bp);

/* `iters` SIRT updates (sys_mat/sirt_dd.py:51-72, as vg_dd2d_sirt_iter) of
 * all n problems in one persistent, cooperative launch.  Every block takes
 * the next work item from one queue (all items of update 0, then of update
 * 1, ...); an item waits only for the items of its own problem it reads
 * (per-problem counters, 3 n ints of device memory in `counters`), so the
 * updates of different problems overlap.  probs_dev and the item arrays are
 * device memory; max_nd is the largest image side of the batch.  storage:
 * bit 0 stores the iterates, bit 1 the measured sinograms as bfloat16.
 * cancel: NULL, or an int in pinned host memory (or device memory) that the
 * caller may set non-zero at any time; the run then stops at the start of
 * the next update with status VG_ERR_CANCELLED, every problem having the
 * same number of updates.  budget_ns: a time budget (0 = none), checked at
 * the start of every update (VG_ERR_TIMEOUT the same way).  A dependency
 * wait longer than about two seconds stops the run with VG_ERR_TIMEOUT (the
 * iterates are then not all at the same update).  grid_blocks (may be NULL)
 * receives the number of resident blocks launched.  Replaces one
 * vg_dd2d_sirt_iter launch chain per problem; vir has no batching. */
int vg_sirt2d_batch_run(const vg_sirt2d_problem *probs_dev, int n, int max_nd, const int *fp_items,
                        int n_fp, const int *tab_items, int n_tab, const int *bp_items, int n_bp,
                        int iters, int storage, const int *cancel, unsigned long long budget_ns,
                        vg_sirt2d_batch_ctrl *ctrl, int *counters, void *stream, int *grid_blocks);

/* Pixel-driven FBP backprojection of a ramp-filtered sinogram q (na, nu)
 * (filtered by vg_filter_rows, i.e. filtration.filter_sino's 2H):
 *   img(x, y) = pi / (2 na) * sum_views q(s(x, y)) / U(x, y)^2,
 * linear interpolation between bin centres; parallel s = -sin x + cos y,
 * U = 1; fan (flat detector) s = DSD p / (DSO - o), U = (DSO - o) / DSO.
 * The fan weights follow processing/reconstruction.py:99-107 (equispaced
 * cosine pre-weight, applied by the caller through vg_filter_rows'
 * row_weight) and processing/proj2.py:606-613 (1/U^2); vir has no working
 * fan FBP (reconstruction.fan_fbp, :7-67, calls removed interfaces). */
int vg_fbp2d_bp(const vg_dd2d_geom *g, const float *q, const double *trig,
                float *img, void *stream);

/* ---- 3D cone-beam distance-driven --------------------------------------- */

/* Circular cone-beam geometry of dd_fp_cone_3d / dd_bp_cone_3d
 * (sys_mat/dd.py:815-888): volume (nx, ny, nz) of cubic voxels d_pix,
 * detector (nu, nv) with pitches du, dv and shifts su, sv (in bins), source
 * at DSO, flat detector at DSD; sinogram (na, nu, nv), v fastest. */
typedef struct {
    int nx, ny, nz, na, nu, nv;
    float du, dv, su, sv, d_pix, DSO, DSD;
} vg_dd3d_geom;

/* Device workspace (per-view line scales and z magnifications) both cone
 * calls need; 0 for an invalid geometry. */
size_t vg_dd3d_workspace_bytes(const vg_dd3d_geom *g);

/* Forward projection (dd.py:815-825, sweep :285-380 as intended; returns
 * sino * d_pix^2 / (du dv)), one thread per (view, u, v) bin. */
int vg_dd3d_fp(const vg_dd3d_geom *g, const float *vol, const double *trig,
               float *sino, void *workspace, size_t workspace_bytes,
               void *stream);

/* Backprojection (dd.py:829-835, sweep :384-468; returns img / (na d_pix)),
 * one thread per voxel. */
int vg_dd3d_bp(const vg_dd3d_geom *g, const float *sino, const double *trig,
               float *vol, void *workspace, size_t workspace_bytes,
               void *stream);

/* ---- 3D cone-beam separable footprint (SF-TR) --------------------------- */

/* The separable-footprint cone projector that vir's sys_mat/sp.py:93-211
 * (CTGeometry, footprint1D, forward_project, back_project: no rotation
 * angles) sketches: trapezoid transaxial and rectangle axial footprints with
 * the A2 amplitude of Long, Fessler & Balter (IEEE TMI 29(11), 2010), on the
 * circular cone geometry of vg_dd3d_geom (dd_fp_cone_3d, dd.py:815).  Voxel
 * (x, y, z) adds f l_phi0 l_theta F1 F2 to cell (u, v): F1 the unit
 * trapezoid through the projections of the column's four corners, F2 the
 * rectangle [M (z - d/2), M (z + d/2)], M = DSD / (DSO - o), both averaged
 * over the cell; l_phi0 = d |r| / max(|r_x|, |r_y|) for the transaxial ray r
 * through the column centre, l_theta = sqrt(1 + v^2 / (u^2 + DSD^2)) at the
 * cell centre.
 * vg_sf3d_fp: sino (na, nu, nv) = the line integrals above, gather form;
 *   workspace: the volume's per-column running sums over z (nx ny (nz + 1)
 *   floats, FP64-accumulated) from which each column's v profile is read.
 * vg_sf3d_bp: vol = its exact adjoint; workspace: the l_theta-weighted
 *   sinogram of a chunk of views (at most 256 MiB or one view).
 * Both take vg_sf3d_workspace_bytes(g) bytes (the larger need), 4-byte
 * aligned.
 * nx and ny at most 2048.
 * The volume must lie inside the source circle (half diagonal below DSO). */
size_t vg_sf3d_workspace_bytes(const vg_dd3d_geom *g);
int vg_sf3d_fp(const vg_dd3d_geom *g, const float *vol, const double *trig, float *sino,
               void *workspace, size_t workspace_bytes, void *stream);
int vg_sf3d_bp(const vg_dd3d_geom *g, const float *sino, const double *trig, float *vol,
               void *workspace, size_t workspace_bytes, void *stream);

/* One SIRT update on the cone pair, both halves fused (sys_mat/sirt_dd.py:51-72):
 *   r  = (y - FP x) * inv_w_sino   (FP x kept where inv_w_sino == 0)
 *   x += gamma * (BP r) * inv_w_img (BP r kept where inv_w_img == 0)
 * with FP / BP of vg_dd3d_fp / vg_dd3d_bp (vir's scalings); inv_w_* hold
 * 1/W (0 where W == 0); r is a caller scratch sinogram; x is updated in
 * place.  Three launches: the per-view tables, the forward projection with
 * the residual epilogue, the back projection with the update epilogue. */
int vg_dd3d_sirt_iter(const vg_dd3d_geom *g, const float *y, const float *inv_w_sino,
                      const float *inv_w_img, float gamma, const double *trig, float *x,
                      float *r, void *workspace, size_t workspace_bytes, void *stream);

/* ---- translational "square" geometry ------------------------------------ */

/* dd_fp_square / dd_bp_square (sys_mat/dd.py:903, 1104): an n x n x nz
 * object (x, y, z; z fastest) seen from four sides, each a plane of
 * nsrc_p x nsrc_z sources at distance DSO from the centre (centres
 * pf.censpace(nsrc, dsrc, ssrc)) and a flat detector DSD from the sources
 * (cell boundaries pf.boundspace(nu, du, su + ssrc_p) and
 * pf.boundspace(nv, dv, sv + ssrc_z)).  Sinogram (nsrc_p, nsrc_z, nv, nu, 4),
 * the side index fastest, 16-byte aligned. */
typedef struct {
    int n, nz, nu, nv, nsrc_p, nsrc_z;
    float DSO, DSD, du, dv, dsrc_p, dsrc_z, su, sv, ssrc_p, ssrc_z, d_pix;
} vg_dd_square_geom;

/* Device workspace of the backprojection (four FP64 planes of the volume,
 * then the running integrals along u of the detector rows of one chunk of
 * sources; 16-byte aligned); 0 for an invalid geometry. */
size_t vg_dd_square_workspace_bytes(const vg_dd_square_geom *g);

/* Forward projection, dd_fp_square (dd.py:903-930, dd_fp_translational
 * :959-1100): sino = A vol * d_pix^2 / (du dv); slabs whose magnification
 * DSD / (DSO - o) is not positive are skipped (dd.py:988). */
int vg_dd_square_fp(const vg_dd_square_geom *g, const float *vol, float *sino,
                    void *stream);

/* Backprojection, dd_bp_square (dd.py:1104-1135, dd_bp_translational
 * :1164-1313): vol = A^T sino, no scaling. */
int vg_dd_square_bp(const vg_dd_square_geom *g, const float *sino, float *vol,
                    void *workspace, size_t workspace_bytes, void *stream);

/* One update of sirt_dd.sirt (sirt_dd.py:50-72):
 *   r = FP(x); r = (y - r) / w_sino where w_sino != 0 (fast_divide1);
 *   u = BP(r); u = u / w_vol where w_vol != 0 (fast_divide2); x += gamma u.
 * y, w_sino, r: sinogram layout; w_vol, x: volume layout. */
int vg_dd_square_sirt_iter(const vg_dd_square_geom *g, const float *y,
                           const float *w_sino, const float *w_vol, float gamma,
                           float *x, float *r, void *workspace,
                           size_t workspace_bytes, void *stream);

/* ---- ray-driven (rd.py) and pixel-driven (pd.py) projectors ------------- */

/* Geometry of sys_mat/rd.py and sys_mat/pd.py: kind 0 = parallel 2D
 * (image nx x ny), 1 = fan 2D (flat detector at DSD, source at DSO),
 * 2 = circular cone 3D (volume nx x ny x nz, detector nu x nv, v
 * fastest).  joseph selects the Joseph sampling of rd.py instead of its
 * Amanatides-Woo walk (ignored by the pixel-driven pair). */
typedef struct {
    int nx, ny, nz, na, nu, nv;
    float du, dv, su, sv, d_pix, DSO, DSD;
    int kind, joseph;
} vg_ray_geom;

/* aw_fp_par_2d / aw_fp_fan_2d / aw_fp_cone_3d (rd.py:450, 544, 652; the
 * kernels rd.py:112-447): one thread per ray.  trig: float64 (cos, sin) of
 * the float32 angles.  A ray parallel to an axis is clipped to its slab,
 * and cone rows use nv (the reference's rd.py:52-64 and :688 do neither). */
int vg_rd_fp(const vg_ray_geom *g, const float *img, const double *trig,
             float *sino, void *stream);

/* aw_bp_par_2d / aw_bp_fan_2d / aw_bp_cone_3d (rd.py:461, 556, 665),
 * scaled img / na / d_pix^2 * du (2D) or img / na * du * dv (cone).  The 2D
 * Amanatides-Woo back projection gathers, per pixel, s times the chord of
 * every ray crossing it (deterministic; the walk's segment lengths, with
 * rays within 1e-6 of an axis kept in the row or column they enter); the
 * Joseph and cone back projections scatter along each ray (float atomics),
 * as rd.py does. */
int vg_rd_bp(const vg_ray_geom *g, const float *sino, const double *trig,
             float *img, void *stream);

/* pd_fp_par_2d / pd_fp_fan_2d / pd_fp_cone_3d (pd.py:130, 238, 354): each
 * pixel's footprint scattered into the overlapped bins (float atomics),
 * sino * d_pix.  trig: float64 (cos, sin) of the angles as given. */
int vg_pd_fp(const vg_ray_geom *g, const float *img, const double *trig,
             float *sino, void *stream);

/* pd_bp_par_2d / pd_bp_fan_2d / pd_bp_cone_3d (pd.py:138, 246, 363):
 * gather per pixel / voxel over views, img / na / d_pix * du (* dv). */
int vg_pd_bp(const vg_ray_geom *g, const float *sino, const double *trig,
             float *img, void *stream);

/* ---- TV-regularised primal-dual solver (tv.py) ---------------------------- */

/* The fused steps of the preconditioned primal-dual loop of tv.py:262-294
 * for an (nx, ny) image; the projector calls between them are the
 * caller's.  Gradient and divergence are periodic (np.roll, tv.py:207-224).
 *   vg_tv_dual:     z += sigma_z grad(u_bar); z <- z / max(1, |z|) per pixel
 *                   (tv.py:284-285; the projection pyT computes for 2 x 1
 *                   pairs, tv.py:98-184); z is (2, nx, ny).
 *   vg_tv_residual: q += sigma_q (Ax - g); q /= (1 + sigma_q lam) (:287-288).
 *   vg_tv_primal:   u += tau (div z - At q); u_bar = u + theta (u - u_prev)
 *                   (:291-294). */
int vg_tv_dual(const float *u_bar, float *z, int nx, int ny, float sigma_z,
               void *stream);
int vg_tv_residual(float *q, const float *ax, const float *g, const float *sigma_q,
                   float lam, size_t n, void *stream);
int vg_tv_primal(float *u, float *u_bar, const float *z, const float *atq,
                 const float *tau, float theta, int nx, int ny, void *stream);

/* ---- FDK (cone-beam filtered backprojection) ----------------------------- */

/* vir has no FDK; these three steps build it on the cone geometry above.
 * (1) sino (na, nu, nv) -> out (na, nv, nu), each sample times the flat-
 *     detector cosine weight DSD / sqrt(DSD^2 + u^2 + v^2) (the equispaced
 *     pre-weight of processing/reconstruction.py:99-107 in 2D);
 * (2) the caller filters the rows with vg_filter_rows at the isocentre
 *     pitch du DSO / DSD (filtration.filter_sino's 2H);
 * (3) vg_fdk_transpose_back returns to (na, nu, nv) and vg_fdk_bp
 *     backprojects: vol = pi / (2 na) sum_views Q(u, v) / U^2 with
 *     U = (DSO - o) / DSO (processing/proj2.py:606-613), bilinear in (u, v). */
int vg_fdk_weight_transpose(const vg_dd3d_geom *g, const float *sino,
                            float *out, void *stream);
int vg_fdk_transpose_back(const vg_dd3d_geom *g, const float *in, float *out,
                          void *stream);
int vg_fdk_bp(const vg_dd3d_geom *g, const float *q, const double *trig,
              float *vol, void *stream);

/* ---- 2D separable footprint -------------------------------------------- */

/* fan = 1: sys_mat/sp.py:12-87 (sf_fp_fan_2d; bins of width du, source at
 * DSO, detector at DSD); fan = 0: sys_mat/fp_2d_par.py:67-125
 * (separable_footprint_fp_2d; du is the detector pitch d_det). */
typedef struct {
    int nx, ny, na, nu;
    float du, d_pix, DSO, DSD;
    int fan;
} vg_sf2d_geom;

/* Forward projection, gather form (one thread per bin walking the pixel lines
 * across its footprint strip), same output and scale as the reference:
 * sino * d_pix (fan) or overlap / d_det (parallel rectangle).  img (nx, ny)
 * and its transpose imgT (ny, nx). */
int vg_sf2d_fp(const vg_sf2d_geom *g, const float *img, const float *imgT,
               const double *trig, float *sino, void *stream);

/* Its exact adjoint (one thread per pixel over all views); vir has no
 * backprojector for these footprints. */
int vg_sf2d_bp(const vg_sf2d_geom *g, const float *sino, const double *trig,
               float *img, void *stream);

/* ---- elementwise / filter helpers -------------------------------------- */

/* out (cols, rows) = transpose of in (rows, cols). */
int vg_transpose(const float *in, int rows, int cols, float *out, void *stream);

/* Ordered compaction of the non-zero entries of a float array of n < 2^31
 * (the voxel lists of the Siddon list algebra: siddon.py rays_ave and
 * list2array produce them by np.unique / accumulation).  Blocks of
 * 1024 entries: vg_count_nonzero writes each block's count
 * (vg_compact_blocks(n) ints); the caller forms first[b] = the exclusive
 * prefix sum (int64); vg_compact_nonzero then writes the indices and values
 * of the non-zeros in increasing index order. */
int vg_compact_blocks(long long n);
int vg_count_nonzero(const float *v, long long n, int *counts, void *stream);
int vg_compact_nonzero(const float *v, long long n, const long long *first, int *idx,
                       float *val, void *stream);

/* Ramp filtering of each sinogram row as a linear convolution with the
 * spatial kernel of the padded rFFT filter (filtration.filter_sino,
 * filtration.py:238-309): out[r, i] = sum_j in[r, j] * taps[i - j + nu - 1]
 * with taps (2 nu - 1) = irfft(2 H, n=z) reordered to lags -(nu-1)..nu-1.
 * rows x nu in, rows x nu out (any row count, nu <= 6400).  `row_weight`
 * (nu values or NULL) multiplies each input row first (fan-beam cosine
 * pre-weighting). */
int vg_filter_rows(const float *in, int rows, int nu, const float *taps,
                   const float *row_weight, float *out, void *stream);

/* The same filtering by FFT, as filter_sino computes it (filtration.py:238-309):
 * each row (times row_weight when given) zero-padded to z (a power of two,
 * 2 nu <= z <= 32768), rFFT, times spectrum (z/2 + 1 floats: 2H), inverse,
 * first nu samples; float32 in shared memory, one block per row.  twiddles
 * holds z complex values (float pairs) W^m = exp(-2 pi i m / z), m < z. */
int vg_filter_rows_fft(const float *in, int rows, int nu, int z, const float *spectrum,
                       const float *twiddles, const float *row_weight, float *out, void *stream);

/* Beam-hardening pre-correction of logged sinograms (processing/beamhard.py),
 * elementwise over n values; `in` and `out` are float32 or float64
 * (in_f64 / out_f64), computed as numpy computes the reference's
 * expressions, every operation separately rounded.
 *   vg_bh_poly: out = mu ((c0 t^2 + c1 t) + c2), t = in / mu -- beamhard_cor
 *     (beamhard.py:39-47).  Bit i of f32mask makes step i float32 (else
 *     float64), as numpy's promotion of the caller's types decides: 0 t and
 *     t^2, 1 c0 t^2, 2 c1 t, 3 the sum with c2, 4 the product with mu.
 *   vg_bh_interp: piecewise-linear lookup in a table of m (2..VG_BH_MAX_TABLE)
 *     increasing abscissae: seg holds m rows (x_k, y_k, s_k, 0) of float64
 *     (16-byte aligned) with s_k = (y_k+1 - y_k) / (x_k+1 - x_k) (0 for the
 *     last row); keys the m search keys: x_k as float64, or (key_f32, float32
 *     samples only) x_k rounded to float32 toward -inf for mode 0 and toward
 *     +inf for modes 1 / 2.
 *     mode 0: scipy interp1d 'linear' on in.clip(0), as beamhard_cor_table
 *       (beamhard.py:16-36); values outside [x_0, x_m-1] are added to
 *       *n_outside (a device counter, may be NULL; interp1d raises for them).
 *     mode 1 / 2: out = in * np.interp(in / mu, x, y), the lookup-table
 *       correction of tests/Test_Beamhard/beamhard_test.py:26-27, with the
 *       division in float32 (1) or float64 (2). */
#define VG_BH_MAX_TABLE 4096
int vg_bh_poly(const void *in, int in_f64, void *out, int out_f64, size_t n, double mu,
               double c0, double c1, double c2, int f32mask, void *stream);
int vg_bh_interp(const void *in, int in_f64, void *out, int out_f64, size_t n, const double *seg,
                 const void *keys, int key_f32, int m, int mode, double mu,
                 unsigned long long *n_outside, void *stream);

/* Helical rebinning front-end (trajectory.py).
 *   vg_rebin_rows: n_out output rows of n_cols, row o = float32(src[v0, r0, :]
 *     w0 + src[v1, r1, :] w1) in float64 (the gathers of sino_hel2axl,
 *     sino_hel2axl180 and sino_hel2hel, trajectory.py:70-240); src is
 *     (n_views, n_rows, n_cols) float32; pairs (n_out x 4 int32: v0, r0, v1,
 *     r1) and weights (n_out x 2 float64) are 16-byte aligned device tables
 *     built from the geometry's interpZ on the host; reverse != 0 writes the
 *     columns in reverse order; rows with an index out of range are left
 *     unwritten and counted in *n_bad (device counter, may be NULL).
 *   vg_axl2hel: sino_axl2hel (trajectory.py:45-67): helical sinogram
 *     (n_views_h, n_rows_h, n_cols) from the axial (n_angs, n_rows, n_cols),
 *     view i sampled at fractional axial view view_index[i] and rows
 *     r + z_shift[i] with scipy map_coordinates(order=1) arithmetic: mode
 *     'constant' (0 outside [0, n-1]), or 'grid-wrap' on clipped rows and
 *     columns where wrap[i] != 0 (views past the last axial angle).
 *   vg_rotsum_fp: forward_project_phantom (trajectory.py:17-42): sino (n_views,
 *     nz, nx) = sum over y of the (nx, ny, nz) phantom sampled trilinearly
 *     (cval 0) at M_v (x, y, z, 1), each coordinate rounded to 6 decimals;
 *     mats holds n_views row-major 3 x 4 float32 matrices (rows x, y, z of the
 *     view's affine transform). */
int vg_rebin_rows(const float *src, int n_views, int n_rows, int n_cols, const int *pairs,
                  const double *weights, int n_out, int reverse, float *dst,
                  unsigned long long *n_bad, void *stream);
int vg_axl2hel(const float *sinoA, int n_angs, int n_rows, int n_cols, const double *view_index,
               const double *z_shift, const int *wrap, int n_views_h, int n_rows_h, float *sinoH,
               void *stream);
int vg_rotsum_fp(const float *vol, int nx, int ny, int nz, const float *mats, int n_views,
                 float *sino, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* VIRGPU_H */
