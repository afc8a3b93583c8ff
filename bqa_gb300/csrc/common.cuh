// Shared device helpers of the GB300 annealing kernels: complex64 arithmetic on float2,
// block/warp reductions, and the half-ZZ-gate bond coefficients.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bqa_gb300.h"

#define BQA_FULL_MASK 0xffffffffu

namespace bqa {

// ---- complex64 on float2 -----------------------------------------------------------------

__device__ __forceinline__ float2 c_zero() { return make_float2(0.f, 0.f); }
__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float c_abs2(float2 a) { return fmaf(a.x, a.x, a.y * a.y); }

__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// acc + a*b
__device__ __forceinline__ float2 c_fma(float2 a, float2 b, float2 acc) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(-a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(a.y, b.x, acc.y);
    return acc;
}
// acc + conj(a)*b
__device__ __forceinline__ float2 c_fma_conj(float2 a, float2 b, float2 acc) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(-a.y, b.x, acc.y);
    return acc;
}
// a / b
__device__ __forceinline__ float2 c_div(float2 a, float2 b) {
    const float inv = 1.0f / c_abs2(b);
    return make_float2((a.x * b.x + a.y * b.y) * inv, (a.y * b.x - a.x * b.y) * inv);
}

// ---- reductions ----------------------------------------------------------------------------

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(BQA_FULL_MASK, v, o));
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(BQA_FULL_MASK, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(BQA_FULL_MASK, v, o);
    return v;
}

// Block-wide sum of `cnt` floats per thread (cnt <= 8); every thread gets the totals.
// `scratch` needs cnt * 32 floats of shared memory.  Must be called by the whole block.
template <int CNT>
__device__ __forceinline__ void block_sum(float (&v)[CNT], float* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int c = 0; c < CNT; ++c) v[c] = warp_sum(v[c]);
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < CNT; ++c) scratch[c * 32 + warp] = v[c];
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < CNT; ++c) {
        float t = lane < nw ? scratch[c * 32 + lane] : 0.f;
        v[c] = warp_sum(t);
    }
    __syncthreads();
}

__device__ __forceinline__ float block_max(float v, float* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    float t = lane < nw ? scratch[lane] : 0.f;
    v = warp_max(t);
    __syncthreads();
    return v;
}

// max of non-negative floats through their bit patterns (monotone for x >= 0)
__device__ __forceinline__ void atomic_max_nonneg(uint32_t* addr, float v) {
    atomicMax(addr, __float_as_uint(fmaxf(v, 0.f)));
}

// ---- half of exp(-i c Z Z) on one bond -------------------------------------------------------
// The bond of a node is doubled to (e, j), e in {0,1}: block e = 0 carries a0 * I and block
// e = 1 carries a1 * Z on the physical index, a0 = sqrt(cos c), a1 = e^{-i pi/4} sqrt(sin c),
// so a0^2 = cos c and a1^2 = -i sin c (src/bqa/backends.py:20-22,519-526).  The square roots
// are numpy's principal complex square roots of the complex-typed cos/sin, whose zero
// imaginary part carries a sign (-sin(c)*0 for cos, cos(c)*0 for sin); that sign picks the
// branch for a negative argument.  Computed in double, rounded once.
struct HalfZZ {
    float2 a0, a1;
};

__device__ __forceinline__ HalfZZ half_zz(double c) {
    double sc, cc;
    sincos(c, &sc, &cc);
    double r0, i0, r1, i1;
    if (cc >= 0.0) { r0 = sqrt(cc); i0 = 0.0; }
    else { r0 = 0.0; i0 = (sc >= 0.0) ? -sqrt(-cc) : sqrt(-cc); }
    if (sc >= 0.0) { r1 = sqrt(sc); i1 = 0.0; }
    else { r1 = 0.0; i1 = (cc >= 0.0) ? sqrt(-sc) : -sqrt(-sc); }
    // a1 = (1 - i)/sqrt(2) * (r1 + i i1)
    const double h = 0.70710678118654752440;
    HalfZZ out;
    out.a0 = make_float2((float)r0, (float)i0);
    out.a1 = make_float2((float)(h * (r1 + i1)), (float)(h * (i1 - r1)));
    return out;
}

__host__ __device__ __forceinline__ int ipow(int b, int e) {
    int r = 1;
    for (int i = 0; i < e; ++i) r *= b;
    return r;
}

}  // namespace bqa
