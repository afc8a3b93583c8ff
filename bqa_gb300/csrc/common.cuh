// Shared device helpers of the GB300 annealing kernels: complex arithmetic on float2
// (complex64) and double2 (complex128), block/warp reductions, and the half-ZZ-gate bond
// coefficients.  Kernels are templated on the real type R (float or double).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bqa_gb300.h"

#define BQA_FULL_MASK 0xffffffffu

namespace bqa {

template <typename R> struct Cx;
template <> struct Cx<float> { using T = float2; using Bits = uint32_t; };
template <> struct Cx<double> { using T = double2; using Bits = unsigned long long; };

// ---- complex arithmetic ----------------------------------------------------------------------

__device__ __forceinline__ float2 c_make(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ double2 c_make(double x, double y) { return make_double2(x, y); }

template <typename C> __device__ __forceinline__ C c_zero();
template <> __device__ __forceinline__ float2 c_zero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double2 c_zero<double2>() { return make_double2(0.0, 0.0); }

template <typename C> __device__ __forceinline__ C c_add(C a, C b) { return c_make(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C c_sub(C a, C b) { return c_make(a.x - b.x, a.y - b.y); }
template <typename C, typename R> __device__ __forceinline__ C c_scale(C a, R s) { return c_make(a.x * s, a.y * s); }
template <typename C> __device__ __forceinline__ C c_conj(C a) { return c_make(a.x, -a.y); }
template <typename C> __device__ __forceinline__ auto c_abs2(C a) -> decltype(a.x) { return fma(a.x, a.x, a.y * a.y); }

template <typename C> __device__ __forceinline__ C c_mul(C a, C b) {
    return c_make(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// acc + a*b
template <typename C> __device__ __forceinline__ C c_fma(C a, C b, C acc) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
    return acc;
}
// acc + conj(a)*b
template <typename C> __device__ __forceinline__ C c_fma_conj(C a, C b, C acc) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
    return acc;
}
// a / b
template <typename C> __device__ __forceinline__ C c_div(C a, C b) {
    const auto inv = decltype(a.x)(1) / c_abs2(b);
    return c_make((a.x * b.x + a.y * b.y) * inv, (a.y * b.x - a.x * b.y) * inv);
}

// ---- reductions ----------------------------------------------------------------------------

template <typename R> __device__ __forceinline__ R warp_max(R v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(BQA_FULL_MASK, v, o));
    return v;
}
template <typename R> __device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(BQA_FULL_MASK, v, o);
    return v;
}

// Block-wide sum of CNT values per thread; every thread gets the totals.  `scratch` needs
// CNT * 32 values of shared memory.  Must be called by the whole block.
template <int CNT, typename R>
__device__ __forceinline__ void block_sum(R (&v)[CNT], R* scratch) {
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
        R t = lane < nw ? scratch[c * 32 + lane] : R(0);
        v[c] = warp_sum(t);
    }
    __syncthreads();
}

template <typename R>
__device__ __forceinline__ R block_max(R v, R* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    R t = lane < nw ? scratch[lane] : R(0);
    v = warp_max(t);
    __syncthreads();
    return v;
}

// max of non-negative reals through their bit patterns (monotone for x >= 0)
__device__ __forceinline__ void atomic_max_nonneg(uint32_t* addr, float v) {
    atomicMax(addr, __float_as_uint(fmaxf(v, 0.f)));
}
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
    atomicMax(addr, (unsigned long long)__double_as_longlong(fmax(v, 0.0)));
}
__device__ __forceinline__ float bits_to_real(uint32_t b) { return __uint_as_float(b); }
__device__ __forceinline__ double bits_to_real(unsigned long long b) { return __longlong_as_double((long long)b); }

// ---- half of exp(-i c Z Z) on one bond -------------------------------------------------------
// The bond of a node is doubled to (e, j), e in {0,1}: block e = 0 carries a0 * I and block
// e = 1 carries a1 * Z on the physical index, a0 = sqrt(cos c), a1 = e^{-i pi/4} sqrt(sin c),
// so a0^2 = cos c and a1^2 = -i sin c (src/bqa/backends.py:20-22,519-526).  The square roots
// are numpy's principal complex square roots of the complex-typed cos/sin, whose zero
// imaginary part carries a sign (-sin(c)*0 for cos, cos(c)*0 for sin); that sign picks the
// branch for a negative argument.  Computed in double, rounded once to R.
template <typename R>
struct HalfZZ {
    typename Cx<R>::T a0, a1;
};

template <typename R>
__device__ __forceinline__ HalfZZ<R> half_zz(double c) {
    double sc, cc;
    sincos(c, &sc, &cc);
    double r0, i0, r1, i1;
    if (cc >= 0.0) { r0 = sqrt(cc); i0 = 0.0; }
    else { r0 = 0.0; i0 = (sc >= 0.0) ? -sqrt(-cc) : sqrt(-cc); }
    if (sc >= 0.0) { r1 = sqrt(sc); i1 = 0.0; }
    else { r1 = 0.0; i1 = (cc >= 0.0) ? sqrt(-sc) : -sqrt(-sc); }
    // a1 = (1 - i)/sqrt(2) * (r1 + i i1)
    const double h = 0.70710678118654752440;
    HalfZZ<R> out;
    out.a0 = c_make((R)r0, (R)i0);
    out.a1 = c_make((R)(h * (r1 + i1)), (R)(h * (i1 - r1)));
    return out;
}

// half_zz / sincos computed once per warp (lane 0, double precision) and broadcast: the FP64
// pipe is narrow, so per-thread evaluation of the same value dominated the kernels that need
// it.  Every lane of the warp must call these.
template <typename R>
__device__ __forceinline__ HalfZZ<R> half_zz_warp(double c) {
    HalfZZ<R> h;
    if ((threadIdx.x & 31) == 0) h = half_zz<R>(c);
    h.a0.x = __shfl_sync(BQA_FULL_MASK, h.a0.x, 0);
    h.a0.y = __shfl_sync(BQA_FULL_MASK, h.a0.y, 0);
    h.a1.x = __shfl_sync(BQA_FULL_MASK, h.a1.x, 0);
    h.a1.y = __shfl_sync(BQA_FULL_MASK, h.a1.y, 0);
    return h;
}

__device__ __forceinline__ void sincos_warp(double x, double* s, double* c) {
    double sv = 0.0, cv = 0.0;
    if ((threadIdx.x & 31) == 0) sincos(x, &sv, &cv);
    *s = __shfl_sync(BQA_FULL_MASK, sv, 0);
    *c = __shfl_sync(BQA_FULL_MASK, cv, 0);
}

__host__ __device__ __forceinline__ int ipow(int b, int e) {
    int r = 1;
    for (int i = 0; i < e; ++i) r *= b;
    return r;
}

}  // namespace bqa
