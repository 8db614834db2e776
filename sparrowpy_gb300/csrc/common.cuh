// Shared device helpers for the sparrowpy_gb300 CUDA kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sparrow_gb300.h"

#define SP_PI 3.14159265358979323846

// Exact-order FP64 helpers.  The geometry predicates (visibility, direction
// maps, delays) must reproduce the reference's numpy arithmetic bit for bit,
// so every multiply and add is issued separately with round-to-nearest
// (no fused multiply-add).
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xdiv(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ double xdot3(const double* a, const double* b) {
    return xadd(xadd(xmul(a[0], b[0]), xmul(a[1], b[1])), xmul(a[2], b[2]));
}
__device__ __forceinline__ double xdot2(const double* a, const double* b) {
    return xadd(xmul(a[0], b[0]), xmul(a[1], b[1]));
}
__device__ __forceinline__ double xnorm3(const double* a) { return __dsqrt_rn(xdot3(a, a)); }
__device__ __forceinline__ double xnorm2(const double* a) { return __dsqrt_rn(xdot2(a, a)); }
__device__ __forceinline__ void xcross3(const double* a, const double* b, double* c) {
    c[0] = xsub(xmul(a[1], b[2]), xmul(a[2], b[1]));
    c[1] = xsub(xmul(a[2], b[0]), xmul(a[0], b[2]));
    c[2] = xsub(xmul(a[0], b[1]), xmul(a[1], b[0]));
}

// FP64 -> FP32 by truncating the mantissa with integer operations (the
// conversion instruction runs on GB300's narrow FP64 pipe).  |error| <
// 2^-23 |x|; |x| < 2^-126 gives a signed zero; |x| >= 2^128 gives NaN.
__device__ __forceinline__ float f64_trunc_f32(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    const unsigned sign = hi & 0x80000000u;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(0x7fc00000u);
    return __uint_as_float(sign | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// RadiosityFast.py:1277-1312 `get_scattering_data_receiver_index` (one row)
// and :1359-1390 `get_scattering_data_source`: argmin over a wall's direction
// table of |dir - unit(to - from)|^2, first index on ties.
__device__ __forceinline__ int sp_nearest_dir(const double* from, const double* to, const double* __restrict__ dirs,
                                              int nd) {
    double diff[3] = {xsub(to[0], from[0]), xsub(to[1], from[1]), xsub(to[2], from[2])};
    double nn = xnorm3(diff);
    for (int k = 0; k < 3; ++k) diff[k] = xdiv(diff[k], nn);
    int best = 0;
    double bv = 0.0;
    for (int o = 0; o < nd; ++o) {
        double a = xsub(dirs[3 * o], diff[0]), b = xsub(dirs[3 * o + 1], diff[1]), c = xsub(dirs[3 * o + 2], diff[2]);
        double val = xadd(xadd(xmul(a, a), xmul(b, b)), xmul(c, c));
        if (o == 0 || val < bv) {
            bv = val;
            best = o;
        }
    }
    return best;
}

// Every kernel launch of the library passes its stream through sp_counted(),
// which counts launches (read with sp_kernel_launches()).
void sp_note_launch();
inline cudaStream_t sp_counted(cudaStream_t st) {
    sp_note_launch();
    return st;
}

inline int sp_check_launch() {
    cudaError_t e = cudaGetLastError();
    return (e == cudaSuccess) ? SP_OK : SP_ERR_CUDA;
}

inline unsigned sp_blocks(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (unsigned)b;
}
