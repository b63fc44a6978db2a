// Ramp filtering of sinogram rows by FFT, as vir's filter_sino computes it
// (filtration.py:238-309): each row, zero-padded to z = 2^ceil(log2(2 nu)),
// is transformed (rFFT), multiplied by the real half spectrum S = 2H, and
// transformed back; the first nu samples are kept.
//
// One block per row, in shared memory, float32:
//  - the z real samples are packed as N = z/2 complex points c[n] = x[2n] +
//    i x[2n+1] and transformed by a Stockham FFT (radix-4 ping-pong passes,
//    one radix-2 pass first when log2 N is odd; output in natural order);
//  - the real spectrum is split out, X[k] = E[k] + W^k O[k] with E[k] =
//    (C[k] + conj C[N-k]) / 2, O[k] = (C[k] - conj C[N-k]) / 2i, W =
//    exp(-2 pi i / z), multiplied by S[k], and repacked for the inverse,
//    D[k] = E'[k] + i O'[k], E'[k] = (Y[k] + conj Y[N-k]) / 2, O'[k] =
//    (Y[k] - conj Y[N-k]) W^-k / 2;
//  - the inverse FFT of D gives y[2n] = Re d[n] / N, y[2n+1] = Im d[n] / N.
// Twiddles come from a table of W^m, m = 0..z-1, computed in float64 on the
// host.  O(z log z) per row instead of the O(nu^2) direct convolution.
#include "vg_common.cuh"

namespace {

using namespace vg;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// Stockham autosort FFT of N = 2^L points, unnormalised, forward (W^m =
// exp(-2 pi i m / z), z = 2N) or inverse (conjugate twiddles).  A pass of
// radix R at sub-transform size p (p = 1, then multiplied by each radix)
// takes butterfly i < N/R: k = i mod p, inputs x[i + n N/R] times
// exp(-+2 pi i n k / (R p)) = W^(n k N / (R p / 2)), an R-point DFT, outputs
// at ((i - k) R + k) + m p.  One radix-2 pass when L is odd, then radix-4.
__device__ __forceinline__ float2 tw(const float2 *__restrict__ W, int m, bool inv) {
    float2 w = __ldg(W + m);
    if (inv) w.y = -w.y;
    return w;
}

template <bool INV>
__device__ __forceinline__ float2 *stockham(float2 *a, float2 *b, int N, int L,
                                            const float2 *__restrict__ W) {
    int p = 1, lp = 0;  // p = 2^lp
    if (L & 1) {
        const int half = N >> 1;
        for (int i = threadIdx.x; i < half; i += blockDim.x) {
            const float2 u0 = a[i], u1 = a[i + half];  // p = 1: k = 0, no twiddle
            const int j = i << 1;
            b[j] = make_float2(u0.x + u1.x, u0.y + u1.y);
            b[j + 1] = make_float2(u0.x - u1.x, u0.y - u1.y);
        }
        __syncthreads();
        float2 *t = a; a = b; b = t;
        p = 2;
        lp = 1;
    }
    const int T = N >> 2;
    for (; p < N; p <<= 2, lp += 2) {
        const int sh = L - lp - 1;  // N / (2p) = 2^sh: twiddle index n k 2^sh
        for (int i = threadIdx.x; i < T; i += blockDim.x) {
            const int k = i & (p - 1);
            const float2 u0 = a[i];
            const float2 u1 = cmul(a[i + T], tw(W, k << sh, INV));
            const float2 u2 = cmul(a[i + 2 * T], tw(W, (2 * k) << sh, INV));
            const float2 u3 = cmul(a[i + 3 * T], tw(W, (3 * k) << sh, INV));
            const float2 s02 = make_float2(u0.x + u2.x, u0.y + u2.y);
            const float2 d02 = make_float2(u0.x - u2.x, u0.y - u2.y);
            const float2 s13 = make_float2(u1.x + u3.x, u1.y + u3.y);
            const float2 d13 = make_float2(u1.x - u3.x, u1.y - u3.y);
            // -i d13 (forward) or +i d13 (inverse)
            const float2 r13 = INV ? make_float2(-d13.y, d13.x) : make_float2(d13.y, -d13.x);
            const int j = ((i - k) << 2) + k;
            b[j] = make_float2(s02.x + s13.x, s02.y + s13.y);
            b[j + p] = make_float2(d02.x + r13.x, d02.y + r13.y);
            b[j + 2 * p] = make_float2(s02.x - s13.x, s02.y - s13.y);
            b[j + 3 * p] = make_float2(d02.x - r13.x, d02.y - r13.y);
        }
        __syncthreads();
        float2 *t = a; a = b; b = t;
    }
    return a;
}

__global__ void __launch_bounds__(256)
filter_fft_kernel(const float *__restrict__ in, int nu, int N, int L, const float *__restrict__ S,
                  const float2 *__restrict__ W, const float *__restrict__ row_weight,
                  float *__restrict__ out) {
    extern __shared__ float2 buf[];  // 2 x N complex
    float2 *a = buf, *b = buf + N;
    const size_t r = blockIdx.x;
    const float *x = in + r * nu;
    // pack the zero-padded row: c[n] = x[2n] + i x[2n+1]
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const int j0 = 2 * n, j1 = 2 * n + 1;
        float v0 = j0 < nu ? __ldg(x + j0) : 0.f, v1 = j1 < nu ? __ldg(x + j1) : 0.f;
        if (row_weight) {
            if (j0 < nu) v0 *= __ldg(row_weight + j0);
            if (j1 < nu) v1 *= __ldg(row_weight + j1);
        }
        a[n] = make_float2(v0, v1);
    }
    __syncthreads();
    float2 *C = stockham<false>(a, b, N, L, W);
    float2 *D = C == a ? b : a;
    // split, filter, repack: thread k handles the pair (k, N - k), k <= N/2
    for (int k = threadIdx.x; k <= N / 2; k += blockDim.x) {
        const int km = k == 0 ? 0 : N - k;  // C[N] = C[0]
        const float2 ck = C[k], cm = C[km];
        // X[k] and X[N - k]
        const float2 Ek = make_float2(0.5f * (ck.x + cm.x), 0.5f * (ck.y - cm.y));
        const float2 Ok = make_float2(0.5f * (ck.y + cm.y), -0.5f * (ck.x - cm.x));
        const float2 Em = make_float2(0.5f * (cm.x + ck.x), 0.5f * (cm.y - ck.y));
        const float2 Om = make_float2(0.5f * (cm.y + ck.y), -0.5f * (cm.x - ck.x));
        const float2 wk = __ldg(W + k), wm = __ldg(W + (N - k));  // W^k, W^(N-k)
        float2 Xk = cmul(Ok, wk), Xm = cmul(Om, wm);
        Xk = make_float2(Ek.x + Xk.x, Ek.y + Xk.y);
        Xm = make_float2(Em.x + Xm.x, Em.y + Xm.y);
        const float sk = __ldg(S + k), sm = __ldg(S + (N - k));
        const float2 Yk = make_float2(sk * Xk.x, sk * Xk.y), Ym = make_float2(sm * Xm.x, sm * Xm.y);
        // D[k] from (Y[k], Y[N-k]); D[N-k] from (Y[N-k], Y[k])
        {
            const float2 e = make_float2(0.5f * (Yk.x + Ym.x), 0.5f * (Yk.y - Ym.y));
            const float2 o = cmul(make_float2(0.5f * (Yk.x - Ym.x), 0.5f * (Yk.y + Ym.y)), conjf2(wk));
            D[k] = make_float2(e.x - o.y, e.y + o.x);
        }
        if (k != 0 && k != N / 2) {
            const float2 e = make_float2(0.5f * (Ym.x + Yk.x), 0.5f * (Ym.y - Yk.y));
            const float2 o = cmul(make_float2(0.5f * (Ym.x - Yk.x), 0.5f * (Ym.y + Yk.y)), conjf2(wm));
            D[N - k] = make_float2(e.x - o.y, e.y + o.x);
        }
    }
    __syncthreads();
    float2 *d = stockham<true>(D, C, N, L, W);
    const float inv = 1.f / (float)N;
    float *y = out + r * nu;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const int j0 = 2 * n, j1 = 2 * n + 1;
        const float2 v = d[n];
        if (j0 < nu) y[j0] = v.x * inv;
        if (j1 < nu) y[j1] = v.y * inv;
    }
}

}  // namespace

extern "C" int vg_filter_rows_fft(const float *in, int rows, int nu, int z, const float *spectrum,
                                  const float *twiddles, const float *row_weight, float *out,
                                  void *stream) {
    VG_REQUIRE(in && spectrum && twiddles && out, "filter_rows_fft: null pointer");
    VG_REQUIRE(rows > 0 && nu > 0, "filter_rows_fft: bad sizes");
    VG_REQUIRE(z >= 2 * nu && z >= 4 && (z & (z - 1)) == 0 && z <= (1 << 15),
               "filter_rows_fft: z must be a power of two in [max(2 nu, 4), 32768]");
    const int N = z / 2;
    const size_t smem = (size_t)2 * N * sizeof(float2);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(filter_fft_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_status(e, "filter_rows_fft: shared memory attribute");
    }
    int L = 0;
    while ((1 << L) < N) ++L;
    filter_fft_kernel<<<rows, 256, smem, as_stream(stream)>>>(
        in, nu, N, L, spectrum, reinterpret_cast<const float2 *>(twiddles), row_weight, out);
    return launch_status("filter_rows_fft");
}
