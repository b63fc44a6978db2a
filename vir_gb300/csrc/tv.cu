// Fused elementwise steps of the TV-regularised primal-dual (PDHG) solver of
// vir's tv.py (tv.py:200-294): periodic forward-difference gradient and its
// negative adjoint, the divergence (np.roll conventions of tv.py:207-224),
// the projection of each pixel's gradient pair onto the unit ball (what
// tv.py's pyT computes for 2 x 1 pairs, tv.py:98-184), and the
// preconditioned dual and primal updates of the solver loop (tv.py:283-294).
// Images (nx, ny) x-major; the dual field z is (2, nx, ny).
#include "vg_common.cuh"

namespace {

using namespace vg;

// z += sigma_z * grad(u_bar); z <- z / max(1, |z|)
__global__ void tv_dual_kernel(const float *__restrict__ ub, float *__restrict__ z, int nx, int ny,
                               float sigma_z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx * ny) return;
    const int ix = i / ny, iy = i - ix * ny;
    const float c = ub[i];
    const float gx = ub[(ix + 1 == nx ? 0 : ix + 1) * ny + iy] - c;  // roll(x, -1, 0) - x
    const float gy = ub[ix * ny + (iy + 1 == ny ? 0 : iy + 1)] - c;  // roll(x, -1, 1) - x
    const size_t n = (size_t)nx * ny;
    float a = z[i] + sigma_z * gx, b = z[n + i] + sigma_z * gy;
    const float m = sqrtf(a * a + b * b);
    if (m > 1.f) { a /= m; b /= m; }
    z[i] = a;
    z[n + i] = b;
}

// q += sigma_q (Ax - g); q /= (1 + sigma_q lam)
__global__ void tv_residual_kernel(float *__restrict__ q, const float *__restrict__ ax,
                                   const float *__restrict__ g, const float *__restrict__ sq,
                                   float lam, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float s = sq[i];
    q[i] = (q[i] + s * (ax[i] - g[i])) / (1.f + s * lam);
}

// u_prev = u; u += tau (div z - At q); u_bar = u + theta (u - u_prev)
__global__ void tv_primal_kernel(float *__restrict__ u, float *__restrict__ ub,
                                 const float *__restrict__ z, const float *__restrict__ atq,
                                 const float *__restrict__ tau, float theta, int nx, int ny) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx * ny) return;
    const int ix = i / ny, iy = i - ix * ny;
    const size_t n = (size_t)nx * ny;
    // div z = (z0 - roll(z0, 1, 0)) + (z1 - roll(z1, 1, 1))
    const float d = (z[i] - z[(ix == 0 ? nx - 1 : ix - 1) * ny + iy]) +
                    (z[n + i] - z[n + ix * ny + (iy == 0 ? ny - 1 : iy - 1)]);
    const float up = u[i];
    const float un = up + tau[i] * (d - atq[i]);
    u[i] = un;
    ub[i] = un + theta * (un - up);
}

int check2(int nx, int ny) {
    VG_REQUIRE(nx > 0 && ny > 0 && (long long)nx * ny < (1LL << 31), "tv: bad image size");
    return VG_OK;
}

}  // namespace

extern "C" int vg_tv_dual(const float *u_bar, float *z, int nx, int ny, float sigma_z, void *stream) {
    int s = check2(nx, ny);
    if (s) return s;
    VG_REQUIRE(u_bar && z, "tv_dual: null pointer");
    tv_dual_kernel<<<ceil_div((long long)nx * ny, 256), 256, 0, as_stream(stream)>>>(u_bar, z, nx, ny,
                                                                                   sigma_z);
    return launch_status("tv_dual");
}

extern "C" int vg_tv_residual(float *q, const float *ax, const float *g, const float *sigma_q,
                              float lam, size_t n, void *stream) {
    VG_REQUIRE(q && ax && g && sigma_q, "tv_residual: null pointer");
    VG_REQUIRE(n > 0 && ceil_div((long long)n, 256) < 2147483647LL, "tv_residual: bad size");
    tv_residual_kernel<<<ceil_div((long long)n, 256), 256, 0, as_stream(stream)>>>(q, ax, g, sigma_q,
                                                                                 lam, n);
    return launch_status("tv_residual");
}

extern "C" int vg_tv_primal(float *u, float *u_bar, const float *z, const float *atq,
                            const float *tau, float theta, int nx, int ny, void *stream) {
    int s = check2(nx, ny);
    if (s) return s;
    VG_REQUIRE(u && u_bar && z && atq && tau, "tv_primal: null pointer");
    tv_primal_kernel<<<ceil_div((long long)nx * ny, 256), 256, 0, as_stream(stream)>>>(
        u, u_bar, z, atq, tau, theta, nx, ny);
    return launch_status("tv_primal");
}
