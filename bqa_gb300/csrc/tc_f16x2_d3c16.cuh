// FP32-accurate tensor-core (tcgen05) parts of the degree-3, bond-dim-16 half-node message
// kernels in two FP16 terms (2xFP16): the bond products (both kernels) and, further down, the
// closing contractions of the all-tensor-core kernel (tcx_half_kernel_d3c16, the default); the
// products-only kernel (tch_half_kernel_d3c16) keeps its closing contractions on the CUDA cores
// (d3c16::close).
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
// is at least 2^14: far below FP32 rounding of the largest element.  The products-only
// kernel's epilogue multiplies the accumulators by 2^-(k_T + k_M) (exact) before the closing
// contractions; the all-tensor-core kernel rescales them into its closing operands instead.
//
// Against 3xTF32 the operands take half the bytes, so the three products' A operands (hi and lo,
// 96 KB) and the messages' B operands (12 KB) are all written at once and the 36 MMAs of a
// half-node run in ONE tensor-core round trip (3xTF32 needs three, rewriting its A space
// between them); FP16 MMAs also run at twice the TF32 rate.
//
// Shared memory (bytes, one region of 110,592): product phase -- A hi of bonds 2, 1, 0 at 0,
// 16 K, 32 K; A lo at 48 K, 64 K, 80 K; B hi of messages 0, 1, 2 at 96 K + 2 K k; B lo at
// 102 K + 2 K k.  Close phase of the products-only kernel -- V_1, V_2, V_0 (32 KB each,
// swizzled FP32, tc_d3c16.cuh offsets), the two close output buffers and, on its
// diagonal-message path, the transposed messages; of the all-tensor-core kernel -- three
// closing-stage buffers (below).  After the region: the mbarrier(s), the tensor-memory slot
// and the warps' maxima.  Tensor memory: V_2, V_1, V_0 at columns [0, 64), [64, 128),
// [128, 192) of 256.
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
// the all-tensor-core kernel: four mbarriers, the slot, the fault word and the maxima
constexpr uint32_t SCRATCH_X = 4 * 8 + 4 + 4 + 4 * 32;
constexpr uint32_t TMEM_COLS = 256;
constexpr uint32_t IDESC = tc::idesc(tc::FMT_F16, 128, 32);
constexpr uint32_t COL_V2 = tcd3::COL_V2, COL_V1 = tcd3::COL_V1, COL_V0 = tcd3::COL_V0;
constexpr long long WAIT_CYCLES = 2000000000LL;

// bits of |x| (ordered like the magnitudes for finite x)
__device__ __forceinline__ uint32_t mag(float x) { return __float_as_uint(x) & 0x7fffffffu; }

// Exponent k with 2^14 <= m 2^k < 2^15 for the largest magnitude m (bits of m), clamped to
// [-50, 50] so that the scales of a product of up to four operands stay normal floats (a block
// beyond 2^36 or below 2^-36 just sits outside [2^14, 2^15)); 0 for m = 0.
__device__ __forceinline__ int scale_exp(uint32_t mbits) {
    if (mbits == 0) return 0;
    const int e = (int)(mbits >> 23) - 127;   // floor(log2 m) for normal m, -127 below
    return max(-50, min(50, 14 - e));
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

// ---------------------------------------------------------------------------------------------
// Closing contractions on the tensor cores too (2xFP16, FP32-accurate).  P[o][o'] =
// sum_kappa conj(X[o, kappa]) R[o', kappa] over the two other bonds kappa is, as in
// tc_bf16_d3c16.cuh, the real GEMM D[(o, p)][(o', q)] = sum_kappa X_p[o, kappa] R_q[o', kappa]
// with Re P = D00 + D11 and Im P = D01 - D10.  Both sides are the products' accumulators times
// 2^-21 (their scaled magnitudes are below 32 x 2^15 x 2^15 = 2^35, so the operands stay below
// 2^14) split into FP16 hi + lo:
//   * X (MN-major, M = 64): row 16 Q + 2 i + l holds X_hi (l = 0) or X_lo (l = 1) of P row
//     8 Q + i (P row = 2 o + p), so both halves of a P row land in neighbouring lanes of the
//     M = 64 accumulator (row m in lane 32 (m / 16) + m % 16) and one shuffle adds them, and the
//     four rows of an open index o (p, l) are 8 contiguous bytes of a core matrix;
//   * R_hi and R_lo (K-major, N = 32): two MMAs per K step into the same accumulator,
// so each K step accumulates all four products X_hi R_hi + X_hi R_lo + X_lo R_hi + X_lo R_lo.
// K (= 256 pairs kappa = (u, v) of the two contracted bonds) is split into two stages by
// parity: stage rho takes the kappa with (u + v) % 2 = rho, at K index 8 u + v / 2, so a thread
// holding a row of the R side (u fixed, v along its registers) writes 16-byte chunks.  The six
// stages (three blocks x two halves) rotate through three 36 KB buffers; both stages of a block
// are written from one read of the accumulators, while the previous block's second stage runs.
// Block accumulators alternate between tensor-memory columns 192 and 224 (the products keep
// [0, 192) until the last block is written).
//
//   block  X side (rows: hi, lo; registers)    R side (rows: hi, lo; registers)   (u, v)
//   P_0    V_1 (o = a, c; b)                   V_2 (o' = a, b; c)                  (b, c)
//   P_2    V_0 (b, o = c; a)                   V_1 (a, o' = c; b)                  (a, b)
//   P_1    V_0 (o = b, c; a)                   V_2 (a, o' = b; c)                  (a, c)
constexpr uint32_t X_LBO = 1152, X_SBO = 144;   // K-chunk and M-group strides (8 groups, padded)
constexpr uint32_t R_LBO = 144, R_SBO = 2304;   // K-chunk (padded) and N-group strides
constexpr uint32_t X_BYTES = 16 * X_LBO;        // 18,432: K = 128
constexpr uint32_t R_BYTES = 4 * R_SBO;         // 9,216
constexpr uint32_t STAGE = X_BYTES + 2 * R_BYTES;
static_assert(3 * STAGE <= REGION, "close stages exceed the region");
constexpr uint32_t COL_C0 = 192, COL_C1 = 224;
constexpr uint32_t ID_CLOSE = tc::idesc(tc::FMT_F16, 64, 32, true, false);
constexpr float OPERAND_SCALE = 1.0f / 2097152.0f;   // 2^-21

__device__ __forceinline__ uint32_t x_off(int m, int k) {   // MN-major
    return (k >> 3) * X_LBO + (m >> 3) * X_SBO + (k & 7) * 16 + (m & 7) * 2;
}
__device__ __forceinline__ uint32_t r_off(int n, int k) {   // K-major
    return (n >> 3) * R_SBO + (k >> 3) * R_LBO + (n & 7) * 16 + (k & 7) * 2;
}

// Operands of both stages of block BLK (half rho into buf[rho]) from the products'
// accumulators: the thread's row r = 16 hi + lo (32 rows a warp, quarter w % 4 of row tile w / 4).
template <int BLK>
__device__ __forceinline__ void write_block(uint32_t tl, int hi, int lo, unsigned char* __restrict__ buf0,
                                            unsigned char* __restrict__ buf1) {
    uint32_t f[32];
    {   // X side: the thread holds open index o and contracted index V; u along the registers
        tc::ld_32x32b_x32(tl + (BLK == 0 ? COL_V1 : COL_V0), f);
        tc::wait_ld();
        const int O = BLK == 1 ? lo : hi, V = BLK == 1 ? hi : lo;
        const int m0 = 16 * (O >> 2) + 4 * (O & 3);   // rows (p, l) = m0 + 2 p + l
#pragma unroll
        for (int rho = 0; rho < 2; ++rho) {
            unsigned char* buf = rho ? buf1 : buf0;
            const bool odd = ((V + rho) & 1) != 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) {   // u = 2 i + odd
                const float x0 = __uint_as_float(odd ? f[4 * i + 2] : f[4 * i]);
                const float x1 = __uint_as_float(odd ? f[4 * i + 3] : f[4 * i + 1]);
                const Pair e = split2(x0, x1, OPERAND_SCALE);
                const int k = 8 * (2 * i + (odd ? 1 : 0)) + (V >> 1);
                *reinterpret_cast<uint2*>(buf + x_off(m0, k)) =
                    make_uint2(__byte_perm(e.hi, e.lo, 0x5410), __byte_perm(e.hi, e.lo, 0x7632));
            }
        }
    }
    {   // R side: the thread holds contracted index U and open index o'; v along the registers
        tc::ld_32x32b_x32(tl + (BLK == 1 ? COL_V1 : COL_V2), f);
        tc::wait_ld();
        const int U = BLK == 0 ? lo : hi, Op = BLK == 0 ? hi : lo;
#pragma unroll
        for (int rho = 0; rho < 2; ++rho) {
            unsigned char* buf = rho ? buf1 : buf0;
            const bool odd = ((U + rho) & 1) != 0;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                uint32_t wh[4], wl[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {   // v = 2 j + odd for j = 2 i, 2 i + 1
                    const float y0 = __uint_as_float(odd ? f[8 * i + 2 + q] : f[8 * i + q]);
                    const float y1 = __uint_as_float(odd ? f[8 * i + 6 + q] : f[8 * i + 4 + q]);
                    const Pair e = split2(y0, y1, OPERAND_SCALE);
                    wh[i] = e.hi;
                    wl[i] = e.lo;
                }
                const uint32_t o = r_off(2 * Op + q, 8 * U);
                *reinterpret_cast<uint4*>(buf + X_BYTES + o) = make_uint4(wh[0], wh[1], wh[2], wh[3]);
                *reinterpret_cast<uint4*>(buf + X_BYTES + R_BYTES + o) = make_uint4(wl[0], wl[1], wl[2], wl[3]);
            }
        }
    }
}

// One thread: the 16 MMAs of a stage (8 K steps x (R_lo, R_hi)) into accumulator d; `acc` 0
// starts the block.
__device__ __forceinline__ void issue_stage(uint32_t d, uint32_t buf, uint32_t acc) {
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const uint64_t x = tc::desc_noswz(buf + s * 2 * X_LBO, X_LBO, X_SBO);
        const uint64_t rh = tc::desc_noswz(buf + X_BYTES + s * 2 * R_LBO, R_LBO, R_SBO);
        const uint64_t rl = tc::desc_noswz(buf + X_BYTES + R_BYTES + s * 2 * R_LBO, R_LBO, R_SBO);
        tc::mma_f16(d, x, rl, ID_CLOSE, (s > 0 || acc) ? 1u : 0u);
        tc::mma_f16(d, x, rh, ID_CLOSE, 1u);
    }
}

// Epilogue of one block by four warps (warp w reading lane quarter w % 4): lanes 2 i and 2 i + 1
// (i < 8) hold the hi and lo rows m = 16 w + 2 i + l of P row 8 w + i; the two are added, lanes
// 2 apart combine the real and imaginary parts, and the even lanes write P row 8 w + lane / 2
// (16 values of part p), scaled by s[0] s[1], to P (global, row-major 16 x 16 complex).
__device__ __forceinline__ void epilogue_block(uint32_t tmem_col, const float (&sc)[2], float* __restrict__ P) {
    const int w = (threadIdx.x >> 5) & 3, lane = threadIdx.x & 31;
    const int pr = 8 * w + ((lane >> 1) & 7), o = pr >> 1, p = pr & 1;
#pragma unroll
    for (int half = 0; half < 2; ++half) {   // columns 2 y + q for y in [8 half, 8 half + 8)
        uint32_t f[16];
        tc::ld_32x32b_x16(tmem_col + ((uint32_t)(32 * w) << 16) + 16 * half, f);
        tc::wait_ld();
#pragma unroll
        for (int y = 0; y < 8; ++y) {
            const float re = __uint_as_float(f[2 * y]), im = __uint_as_float(f[2 * y + 1]);
            const float g0 = re + __shfl_xor_sync(0xffffffffu, re, 1);
            const float g1 = im + __shfl_xor_sync(0xffffffffu, im, 1);
            const float h = __shfl_xor_sync(0xffffffffu, g1, 2);
            const float out = (p ? h - g0 : g0 + h) * sc[0] * sc[1];
            if (lane < 16 && !(lane & 1)) P[2 * (o * 16 + 8 * half + y) + p] = out;
        }
    }
}

}  // namespace tch
}  // namespace bqa
