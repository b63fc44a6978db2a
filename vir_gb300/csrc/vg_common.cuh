// Shared helpers of libvirgpu: status/error plumbing and small device
// utilities (compensated sums, FP64 arithmetic without contraction).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/virgpu.h"

namespace vg {

// Last error message of the calling host thread.
void set_error(const char *fmt, ...);

// Turns a CUDA error into a status, recording the message.
int cuda_status(cudaError_t e, const char *where);

// Status of the launch just issued (cudaGetLastError).
inline int launch_status(const char *where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: launch failed: %s", where, cudaGetErrorString(e));
        return VG_ERR_LAUNCH;
    }
    return VG_OK;
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

#define VG_REQUIRE(cond, ...)                  \
    do {                                        \
        if (!(cond)) {                          \
            ::vg::set_error(__VA_ARGS__);       \
            return VG_ERR_ARG;                  \
        }                                       \
    } while (0)

// Kahan-compensated FP32 accumulator (the per-ray / per-pixel sums).
struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        float y = __fsub_rn(v, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
};

// FP64 helpers that keep every operation separately rounded, matching the
// evaluation order of the numpy expressions they restate.
__device__ __forceinline__ double d_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double d_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double d_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double d_div(double a, double b) { return __ddiv_rn(a, b); }

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace vg
