// BF16 tensor-core (tcgen05) half-node message kernel of degree 3, bond dim 16: bond products
// AND closing contractions on the tensor cores, BF16 operands, FP32 accumulation in tensor
// memory.  The fast sweep of the mixed-precision BP loop (the messages carry BF16 rounding,
// ~1e-3 relative; FP32 sweeps follow it to the stopping tolerance).
//
// A half-node CTA holds T_s[a][b][c] (16^3 complex).  With V_k = T x_k M_k the blocks are
//     P_0 = <V_1|V_2> (open a),  P_2 = <V_0|V_1> (open c),  P_1 = <V_0|V_2> (open b),
// P[o][o'] = sum_kappa conj(X[o, kappa]) R[o', kappa] over the two other bonds kappa.
//
// Products (one MMA chain per product): rows r = the two bonds kept (256), contraction over the
// interleaved (re, im) parts of T along the bond x (32), columns n = 2 y + q over the interleaved
// parts of the result (32) -- the real form of tc_d3c16.cuh with one BF16 term instead of three
// TF32 terms.  Two M = 128 tiles, two K = 16 steps per product.
//
// Closing contractions as real GEMMs with the real/imaginary part in the row index:
//     D[(o, p)][(o', q)] = sum_kappa X_p[o, kappa] R_q[o', kappa]       (M = 64: rows 2 o + p,
//     Re P[o][o'] = D[(o,0),(o',0)] + D[(o,1),(o',1)],                    32 of them used,
//     Im P[o][o'] = D[(o,0),(o',1)] - D[(o,1),(o',0)]                     N = 32, K = 256)
// X (the conjugated side) is stored MN-major, R K-major; kappa orders are chosen so that the
// product whose new index is the fast kappa index writes 16-byte chunks:
//     P_0: X = V_1, R = V_2, kappa = 16 b + c;  P_2: X = V_0, R = V_1, kappa = 16 a + b;
//     P_1: X = V_0, R = V_2, kappa = 16 a + c.
// The 32 rows past the used ones are read from the next operand in shared memory (each K chunk
// of an MN-major operand holds 4 used 8-row groups, and the M stride is a quarter of the K
// stride) and their accumulator rows are ignored.
//
// Shared memory (bytes, one region): product phase -- A operands of the three products
// (K-major, 16 KB each) at 0, 16 K, 32 K, B operands of the three messages (2 KB each) at
// 48 K, the transposed messages at the tail; close phase -- six operands of 18,432 bytes
// (strides padded so the epilogue's stores from tensor memory are at most 2-way bank
// conflicted), written once the products' MMAs have completed.  Tensor memory: products at
// columns [0, 64), [64, 128), [128, 192) (V_2, V_1, V_0); closing contractions at [0, 32),
// [32, 64), [64, 96) once every product column has been read.
#pragma once

#include <cuda_bf16.h>

#include "tcgen05.cuh"
#include "tc_d3c16.cuh"

namespace bqa {
namespace tcb {

constexpr int TH = 256;
// product operands
constexpr uint32_t PA_LBO = 128, PA_SBO = 512, PA_BYTES = 32 * PA_SBO;
constexpr uint32_t PB_LBO = 128, PB_SBO = 512, PB_BYTES = 4 * PB_SBO;
constexpr uint32_t PA2 = 0, PA1 = PA_BYTES, PA0 = 2 * PA_BYTES, PB = 3 * PA_BYTES;
// close operands: X (MN-major) and R (K-major)
constexpr uint32_t CX_LBO = 576, CX_SBO = 144, CR_LBO = 144, CR_SBO = 4608;
constexpr uint32_t COP_BYTES = 32 * CX_LBO;   // = 4 * CR_SBO = 18,432
static_assert(COP_BYTES == 4 * CR_SBO, "close operand sizes");
constexpr uint32_t CX0 = 0, CX2 = COP_BYTES, CX1 = 2 * COP_BYTES;           // X of P_0, P_2, P_1
constexpr uint32_t CR0 = 3 * COP_BYTES, CR2 = 4 * COP_BYTES, CR1 = 5 * COP_BYTES;
constexpr uint32_t REGION = 6 * COP_BYTES + CX_LBO;   // + the last X operand's unused rows
constexpr uint32_t SMT = REGION - 3 * 256 * 8;        // transposed messages (product phase)
static_assert(PB + 3 * PB_BYTES <= SMT, "product operands overlap the messages");
static_assert(3 * 32768 + 2 * 2048 <= SMT, "CUDA-core buffers overlap the messages");
constexpr uint32_t TMEM_COLS = 256;
constexpr uint32_t ID_PROD = tc::idesc(tc::FMT_BF16, 128, 32);
constexpr uint32_t ID_CLOSE = tc::idesc(tc::FMT_BF16, 64, 32, true, false);
constexpr uint32_t COL_V2 = 0, COL_V1 = 64, COL_V0 = 128;
constexpr long long WAIT_CYCLES = 2000000000LL;

__device__ __forceinline__ uint32_t pack(float lo, float hi) {   // two bf16, `lo` at the lower address
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// byte offsets inside the operands
__device__ __forceinline__ uint32_t pa_off(int r, int kk) {
    return (r >> 3) * PA_SBO + (kk >> 3) * PA_LBO + (r & 7) * 16 + (kk & 7) * 2;
}
__device__ __forceinline__ uint32_t pb_off(int n, int kk) {
    return (n >> 3) * PB_SBO + (kk >> 3) * PB_LBO + (n & 7) * 16 + (kk & 7) * 2;
}
__device__ __forceinline__ uint32_t cx_off(int m, int k) {   // MN-major
    return (k >> 3) * CX_LBO + (m >> 3) * CX_SBO + (k & 7) * 16 + (m & 7) * 2;
}
__device__ __forceinline__ uint32_t cr_off(int n, int k) {   // K-major
    return (n >> 3) * CR_SBO + (k >> 3) * CR_LBO + (n & 7) * 16 + (k & 7) * 2;
}

// A operands of the three products from the share (tcd3::ShareCoord), rounded to BF16
__device__ __forceinline__ void store_products_a(const float4 (&v)[8], unsigned char* __restrict__ reg) {
    const tcd3::ShareCoord q(threadIdx.x);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int a = q.ap + 2 * m;
        const uint32_t e0 = pack(v[m].x, v[m].y), e1 = pack(v[m].z, v[m].w);   // (c0), (c0 + 1)
        // bond 2: r = 16 a + b, kk = 2 c + p -- the pair is 8 contiguous bytes
        *reinterpret_cast<uint2*>(reg + PA2 + pa_off(16 * a + q.b, 2 * q.c0)) = make_uint2(e0, e1);
        // bond 1: r = 16 a + c, kk = 2 b + p
        *reinterpret_cast<uint32_t*>(reg + PA1 + pa_off(16 * a + q.c0, 2 * q.b)) = e0;
        *reinterpret_cast<uint32_t*>(reg + PA1 + pa_off(16 * a + q.c0 + 1, 2 * q.b)) = e1;
        // bond 0: r = 16 b + c, kk = 2 a + p
        *reinterpret_cast<uint32_t*>(reg + PA0 + pa_off(16 * q.b + q.c0, 2 * a)) = e0;
        *reinterpret_cast<uint32_t*>(reg + PA0 + pa_off(16 * q.b + q.c0 + 1, 2 * a)) = e1;
    }
}

// B operands of the three messages from the transposed messages Mt[k][x][y] = M_k[y][x]
__device__ __forceinline__ void store_products_b(const float2* __restrict__ Mt, unsigned char* __restrict__ reg) {
    const int t = threadIdx.x;
    const int y = t >> 4, x = t & 15;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float2 m = Mt[k * 256 + x * 16 + y];
        unsigned char* b = reg + PB + k * PB_BYTES;
        *reinterpret_cast<uint32_t*>(b + pb_off(2 * y, 2 * x)) = pack(m.x, -m.y);
        *reinterpret_cast<uint32_t*>(b + pb_off(2 * y + 1, 2 * x)) = pack(m.y, m.x);
    }
}

// One thread: the 12 product MMAs (3 products x 2 row tiles x 2 K steps).
__device__ __forceinline__ void issue_products(uint32_t tmem, uint32_t rb) {
#pragma unroll
    for (int bond = 0; bond < 3; ++bond) {
        const uint32_t a = rb + (bond == 2 ? PA2 : (bond == 1 ? PA1 : PA0));
        const uint32_t b = rb + PB + bond * PB_BYTES;
        const uint32_t col = bond == 2 ? COL_V2 : (bond == 1 ? COL_V1 : COL_V0);
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int s = 0; s < 2; ++s)
                tc::mma_f16(tmem + col + 32 * j, tc::desc_noswz(a + j * 16 * PA_SBO + s * 2 * PA_LBO, PA_LBO, PA_SBO),
                            tc::desc_noswz(b + s * 2 * PB_LBO, PB_LBO, PB_SBO), ID_PROD, s ? 1u : 0u);
    }
}

// One thread: the 48 closing MMAs (3 blocks x 16 K steps), block X into columns 32 slot.
__device__ __forceinline__ void issue_closes(uint32_t tmem, uint32_t rb) {
#pragma unroll
    for (int slot = 0; slot < 3; ++slot) {
        const uint32_t x = rb + (slot == 0 ? CX0 : (slot == 1 ? CX2 : CX1));
        const uint32_t r = rb + (slot == 0 ? CR0 : (slot == 1 ? CR2 : CR1));
#pragma unroll 4
        for (int s = 0; s < 16; ++s)
            tc::mma_f16(tmem + 32 * slot, tc::desc_noswz(x + s * 2 * CX_LBO, CX_LBO, CX_SBO),
                        tc::desc_noswz(r + s * 2 * CR_LBO, CR_LBO, CR_SBO), ID_CLOSE, s ? 1u : 0u);
    }
}

// 8 consecutive values of part q of a row of complex values f (interleaved) as 16 bytes of BF16
__device__ __forceinline__ uint4 part8(const uint32_t (&f)[32], int q, int h) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        w[i] = pack(__uint_as_float(f[2 * (8 * h + 2 * i) + q]), __uint_as_float(f[2 * (8 * h + 2 * i + 1) + q]));
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// Epilogue of the products: every warp takes its 32 rows (quarter w % 4 of row tile w / 4) of
// the three products from tensor memory into the six close operands.
__device__ __forceinline__ void epilogue_products(uint32_t tmem, unsigned char* __restrict__ reg) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j = w >> 2, qd = w & 3;
    const int r = 128 * j + 32 * qd + lane, hi = r >> 4, lo = r & 15;
    const uint32_t tl = tmem + ((uint32_t)(32 * qd) << 16) + 32 * j;
    uint32_t f[32];
    // V_2: r = 16 a + b (a = hi, b = lo), new index c
    tc::ld_32x32b_x32(tl + COL_V2, f);
    tc::wait_ld();
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint4 v = part8(f, q, h);
            *reinterpret_cast<uint4*>(reg + CR0 + cr_off(2 * hi + q, 16 * lo + 8 * h)) = v;   // P_0: o' = a, kappa = 16 b + c
            *reinterpret_cast<uint4*>(reg + CR1 + cr_off(2 * lo + q, 16 * hi + 8 * h)) = v;   // P_1: o' = b, kappa = 16 a + c
        }
    // V_1: r = 16 a + c (a = hi, c = lo), new index b
    tc::ld_32x32b_x32(tl + COL_V1, f);
    tc::wait_ld();
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int h = 0; h < 2; ++h)   // P_2 (R side): o' = c, kappa = 16 a + b
            *reinterpret_cast<uint4*>(reg + CR2 + cr_off(2 * lo + q, 16 * hi + 8 * h)) = part8(f, q, h);
#pragma unroll
    for (int y = 0; y < 16; ++y)      // P_0 (X side): o = a, kappa = 16 b + c
        *reinterpret_cast<uint32_t*>(reg + CX0 + cx_off(2 * hi, 16 * y + lo)) =
            pack(__uint_as_float(f[2 * y]), __uint_as_float(f[2 * y + 1]));
    // V_0: r = 16 b + c (b = hi, c = lo), new index a
    tc::ld_32x32b_x32(tl + COL_V0, f);
    tc::wait_ld();
#pragma unroll
    for (int y = 0; y < 16; ++y) {
        const uint32_t e = pack(__uint_as_float(f[2 * y]), __uint_as_float(f[2 * y + 1]));
        *reinterpret_cast<uint32_t*>(reg + CX2 + cx_off(2 * lo, 16 * y + hi)) = e;   // P_2 (X): o = c, kappa = 16 a + b
        *reinterpret_cast<uint32_t*>(reg + CX1 + cx_off(2 * hi, 16 * y + lo)) = e;   // P_1 (X): o = b, kappa = 16 a + c
    }
}

// Epilogue of one closing contraction (warps with w % 4 in {0, 1}): lanes 0-15 of quarter qd
// hold rows m = 16 qd + lane = 2 o + p of D; lane pairs combine the real and imaginary parts of
// block row o and write them (16 complex values) to P (global, row-major 16 x 16).
__device__ __forceinline__ void epilogue_close(uint32_t tmem, int slot, float* __restrict__ P) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, qd = w & 3;
    uint32_t f[32];
    tc::ld_32x32b_x32(tmem + ((uint32_t)(32 * qd) << 16) + 32 * slot, f);
    tc::wait_ld();
    const int m = 16 * qd + lane, o = m >> 1, p = m & 1;
    float out[16];
#pragma unroll
    for (int y = 0; y < 16; ++y) {
        const float h = __shfl_xor_sync(0xffffffffu, __uint_as_float(f[2 * y + 1]), 1);
        const float own = __uint_as_float(f[2 * y]);
        out[y] = p ? h - own : own + h;
    }
    if (lane < 16) {
#pragma unroll
        for (int y = 0; y < 16; ++y) P[2 * (o * 16 + y) + p] = out[y];
    }
}

}  // namespace tcb
}  // namespace bqa
