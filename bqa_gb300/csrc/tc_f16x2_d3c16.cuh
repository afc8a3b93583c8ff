// Tensor-core (tcgen05) bond products of the degree-3, bond-dim-16 half-node message kernel in
// two FP16 terms (2xFP16), FP32-accurate; closing contractions on the CUDA cores (d3c16::close).
//
// The real GEMM of each product is that of tc_d3c16.cuh (rows r = the two kept bonds, K = the
// interleaved parts of T along bond x, columns n = 2 y + q), with the operand layouts of
// tc_bf16_d3c16.cuh (K-major, 2-byte elements, no swizzle).  Every operand is scaled by a power
// of two 2^k chosen so its largest magnitude lies in [2^14, 2^15) (the node tensor by one
// exponent per half-node, each message by its own), then split v 2^k = hi + lo with hi the
// FP16 rounding of v 2^k and lo the FP16 rounding of the remainder.  Each K step accumulates
// A_lo B_hi + A_hi B_lo + A_hi B_hi in FP32 tensor memory (FP16 x FP16 products are exact); the
// dropped A_lo B_lo and the split residuals are below 2^-21 |v| (11 + 11 significant bits), the
// level of 3xTF32 (tc_d3c16.cuh).  Remainders of elements far below the block maximum fall into
// FP16's subnormal range, where their absolute error stays below 2^-25 of a scaled value that
// is at least 2^14: far below FP32 rounding of the largest element.  The epilogue multiplies
// the accumulators by 2^-(k_T + k_M) (exact) before the closing contractions.
//
// Against 3xTF32 the operands take half the bytes, so the three products' A operands (hi and lo,
// 96 KB) and the messages' B operands (12 KB) are all written at once and the 36 MMAs of a
// half-node run in ONE tensor-core round trip (3xTF32 needs three, rewriting its A space
// between them); FP16 MMAs also run at twice the TF32 rate.
//
// Shared memory (bytes, one region of 110,592): product phase -- A hi of bonds 2, 1, 0 at 0,
// 16 K, 32 K; A lo at 48 K, 64 K, 80 K; B hi of messages 0, 1, 2 at 96 K + 2 K k; B lo at
// 102 K + 2 K k.  Close phase -- V_1, V_2, V_0 (32 KB each, swizzled FP32, tc_d3c16.cuh
// offsets), the two close output buffers and, on the diagonal-message path, the transposed
// messages.  After the region: the mbarrier, the tensor-memory slot and the warps' maxima.
// Tensor memory: V_2, V_1, V_0 at columns [0, 64), [64, 128), [128, 192) of 256.
#pragma once

#include <cuda_fp16.h>

#include "tcgen05.cuh"
#include "tc_d3c16.cuh"
#include "tc_bf16_d3c16.cuh"

namespace bqa {
namespace tch {

constexpr int TH = 256;
constexpr uint32_t A_BYTES = tcb::PA_BYTES, B_BYTES = tcb::PB_BYTES;   // 16,384 and 2,048
constexpr uint32_t A_HI = 0, A_LO = 3 * A_BYTES, B_HI = 6 * A_BYTES, B_LO = B_HI + 3 * B_BYTES;
constexpr uint32_t REGION = B_LO + 3 * B_BYTES;                        // 110,592
// close phase (float2 offsets): V_1, V_2, V_0 at tcd3::X_V*, then the output buffers and messages
constexpr int SP = 3 * 4096, SMT = SP + 2 * 256;
static_assert(8 * (SMT + 3 * 256) <= (int)REGION, "close buffers exceed the region");
static_assert(tcd3::X_V1 == 0 && tcd3::X_V2 == 4096 && tcd3::X_V0 == 8192, "close buffer offsets");
// mbarrier (8 B), tensor-memory slot (4 B), maxima [8 warps][4] (128 B)
constexpr uint32_t SCRATCH = 8 + 4 + 4 * 32;
constexpr uint32_t TMEM_COLS = 256;
constexpr uint32_t IDESC = tc::idesc(tc::FMT_F16, 128, 32);
constexpr uint32_t COL_V2 = tcd3::COL_V2, COL_V1 = tcd3::COL_V1, COL_V0 = tcd3::COL_V0;
constexpr long long WAIT_CYCLES = 2000000000LL;

// bits of |x| (ordered like the magnitudes for finite x)
__device__ __forceinline__ uint32_t mag(float x) { return __float_as_uint(x) & 0x7fffffffu; }

// Exponent k with 2^14 <= m 2^k < 2^15 for the largest magnitude m (bits of m), clamped so that
// 2^k and 2^-k are normal floats; 0 for m = 0.
__device__ __forceinline__ int scale_exp(uint32_t mbits) {
    if (mbits == 0) return 0;
    const int e = (int)(mbits >> 23) - 127;   // floor(log2 m) for normal m, -127 below
    return max(-126, min(126, 14 - e));
}
__device__ __forceinline__ float pow2(int k) { return __uint_as_float((uint32_t)(k + 127) << 23); }

// v 2^k of two values as FP16 hi and lo pairs (the first value at the lower address)
struct Pair {
    uint32_t hi, lo;
};
__device__ __forceinline__ Pair split2(float v0, float v1, float s) {
    const float a = v0 * s, b = v1 * s;
    const __half2 h = __floats2half2_rn(a, b);
    const __half2 l = __floats2half2_rn(a - __low2float(h), b - __high2float(h));
    return {*reinterpret_cast<const uint32_t*>(&h), *reinterpret_cast<const uint32_t*>(&l)};
}

// A operands (hi and lo) of the three products from the share (tcd3::ShareCoord), scaled by s
__device__ __forceinline__ void store_a(const float4 (&v)[8], float s, unsigned char* __restrict__ reg) {
    const tcd3::ShareCoord q(threadIdx.x);
    constexpr uint32_t A2 = 0, A1 = A_BYTES, A0 = 2 * A_BYTES;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int a = q.ap + 2 * m;
        const Pair e0 = split2(v[m].x, v[m].y, s), e1 = split2(v[m].z, v[m].w, s);   // (c0), (c0 + 1)
#pragma unroll
        for (int part = 0; part < 2; ++part) {
            unsigned char* base = reg + (part ? A_LO : A_HI);
            const uint32_t u0 = part ? e0.lo : e0.hi, u1 = part ? e1.lo : e1.hi;
            // bond 2: r = 16 a + b, kk = 2 c + p -- the pair is 8 contiguous bytes
            *reinterpret_cast<uint2*>(base + A2 + tcb::pa_off(16 * a + q.b, 2 * q.c0)) = make_uint2(u0, u1);
            // bond 1: r = 16 a + c, kk = 2 b + p
            *reinterpret_cast<uint32_t*>(base + A1 + tcb::pa_off(16 * a + q.c0, 2 * q.b)) = u0;
            *reinterpret_cast<uint32_t*>(base + A1 + tcb::pa_off(16 * a + q.c0 + 1, 2 * q.b)) = u1;
            // bond 0: r = 16 b + c, kk = 2 a + p
            *reinterpret_cast<uint32_t*>(base + A0 + tcb::pa_off(16 * q.b + q.c0, 2 * a)) = u0;
            *reinterpret_cast<uint32_t*>(base + A0 + tcb::pa_off(16 * q.b + q.c0 + 1, 2 * a)) = u1;
        }
    }
}

// B operands (hi and lo) of the three messages; thread t holds entry (y, x) = (t >> 4, t & 15)
// of message k, M_k[y][x] = m[k], scaled by s[k]:
//     B[2y][2x] = Re, B[2y][2x+1] = -Im, B[2y+1][2x] = Im, B[2y+1][2x+1] = Re.
__device__ __forceinline__ void store_b(const float2 (&m)[3], const float (&s)[3], unsigned char* __restrict__ reg) {
    const int t = threadIdx.x;
    const int y = t >> 4, x = t & 15;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const Pair p0 = split2(m[k].x, -m[k].y, s[k]), p1 = split2(m[k].y, m[k].x, s[k]);
        const uint32_t o0 = k * B_BYTES + tcb::pb_off(2 * y, 2 * x), o1 = k * B_BYTES + tcb::pb_off(2 * y + 1, 2 * x);
        *reinterpret_cast<uint32_t*>(reg + B_HI + o0) = p0.hi;
        *reinterpret_cast<uint32_t*>(reg + B_LO + o0) = p0.lo;
        *reinterpret_cast<uint32_t*>(reg + B_HI + o1) = p1.hi;
        *reinterpret_cast<uint32_t*>(reg + B_LO + o1) = p1.lo;
    }
}

// One thread: the 36 product MMAs (3 products x 2 row tiles x 2 K steps x 3 terms).
__device__ __forceinline__ void issue_products(uint32_t tmem, uint32_t rb) {
    using tcb::PA_LBO;
    using tcb::PA_SBO;
    using tcb::PB_LBO;
    using tcb::PB_SBO;
#pragma unroll
    for (int bond = 0; bond < 3; ++bond) {
        const uint32_t aslot = (2 - bond) * A_BYTES;   // bond 2 at 0, bond 1 at 16 K, bond 0 at 32 K
        const uint32_t col = bond == 2 ? COL_V2 : (bond == 1 ? COL_V1 : COL_V0);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const uint32_t d = tmem + col + 32 * j;
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                const uint32_t ao = rb + aslot + j * 16 * PA_SBO + s * 2 * PA_LBO;
                const uint32_t bo = rb + bond * B_BYTES + s * 2 * PB_LBO;
                const uint64_t ahi = tc::desc_noswz(ao + A_HI, PA_LBO, PA_SBO);
                const uint64_t alo = tc::desc_noswz(ao + A_LO, PA_LBO, PA_SBO);
                const uint64_t bhi = tc::desc_noswz(bo + B_HI, PB_LBO, PB_SBO);
                const uint64_t blo = tc::desc_noswz(bo + B_LO, PB_LBO, PB_SBO);
                tc::mma_f16(d, alo, bhi, IDESC, s ? 1u : 0u);
                tc::mma_f16(d, ahi, blo, IDESC, 1u);
                tc::mma_f16(d, ahi, bhi, IDESC, 1u);
            }
        }
    }
}

}  // namespace tch
}  // namespace bqa
