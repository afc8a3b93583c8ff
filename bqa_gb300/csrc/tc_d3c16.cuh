// Tensor-core (tcgen05) bond products of the degree-3, bond-dim-16 half-node message kernel.
//
// A half-node CTA holds T_s[a][b][c] (16^3 complex64, s fixed).  With V_k = T x_k M_k the BP
// messages close <V_1|V_2> (bond 0), <V_0|V_1> (bond 2) and <V_0|V_2> (bond 1) (the Hermitian
// split of tiled_node.cuh).  Here the three products run on the tensor cores and the closing
// contractions stay on the CUDA cores (d3c16::close).
//
// Product on bond x as a real GEMM.  Rows r = the two other bond indices (256), contraction
// index kk = 2 x + p over the interleaved (re, im) parts of T (32), columns n = 2 y + q over the
// interleaved parts of the output (32):
//     D[r][n] = sum_kk A[r][kk] B[n][kk],  A[r][2x + p] = part p of T at (r, x),
//     B[2y][2x] = Re M[y][x], B[2y][2x+1] = -Im M[y][x], B[2y+1][2x] = Im M[y][x],
//     B[2y+1][2x+1] = Re M[y][x],
// so row r of D is V_x at (r, y = 0..15), already interleaved.  Per product: two M = 128 tiles,
// N = 32, K = 32 as four K = 8 steps.
//
// FP32 accuracy from TF32 operands (3xTF32): every operand is split as v = hi + lo, hi and lo
// both TF32 (cvt.rna), and each K step accumulates A_lo B_hi + A_hi B_lo + A_hi B_hi in FP32
// tensor memory; the dropped A_lo B_lo and the residual of the split are below 2^-21 |v|.
//
// Operands in shared memory are K-major without swizzle: core matrices of 8 rows x 16 bytes,
// element (r, kk) of a 32-column operand at byte (r/8) SBO + (kk/4) LBO + 16 (r%8) + 4 (kk%4).
// The A operand (T) uses LBO = 128 and SBO = 1056 (= 8 x 128 + 32: each 8-row group starts two
// 16-byte bank groups further on, which makes the three re-layout stores from the threads'
// registers free of bank conflicts); the B operands (messages) use LBO = 144, SBO = 1152 for the
// same reason.  One 96 KB region holds, during the products, A hi/lo (2 x 33 KB) and the three
// messages' B hi/lo (6 x 4.5 KB); the products run one after another through the same A space
// (the next layout of T is written once the previous product's MMAs have completed); after the
// last one the region becomes the three 32 KB close buffers.  The accumulators use 192 of the
// CTA's 256 tensor-memory columns: V_2 at [0, 64), V_1 at [64, 128), V_0 at [128, 192), column
// 32 j for rows [128 j, 128 j + 128).
#pragma once

#include "tcgen05.cuh"
#include "tiled_d3c16.cuh"

namespace bqa {
namespace tcd3 {

constexpr int TH = 256;
constexpr int REGION = 98304;                 // bytes
constexpr uint32_t A_LBO = 128, A_SBO = 1056; // A operand strides (bytes)
constexpr uint32_t B_LBO = 144, B_SBO = 1152; // B operand strides (bytes)
constexpr int A_BYTES = 32 * A_SBO;           // 256 rows
constexpr int B_BYTES = 4 * B_SBO;            // 32 rows
constexpr int A_HI = 0, A_LO = A_BYTES;       // byte offsets of the A operand (product phase)
constexpr int B_OPS = 2 * A_BYTES;            // three messages x (hi, lo)
static_assert(B_OPS + 6 * B_BYTES <= REGION, "product operands exceed the region");
constexpr uint32_t TMEM_COLS = 256;
constexpr uint32_t IDESC = tc::idesc(tc::FMT_TF32, 128, 32);
// close buffers (float2 offsets inside the region): V_1, V_2, V_0
constexpr int X_V1 = 0, X_V2 = 4096, X_V0 = 8192;
constexpr uint32_t COL_V2 = 0, COL_V1 = 64, COL_V0 = 128;
// cycles a wait on the MMA barrier may take before the CTA gives up (~1 s)
constexpr long long WAIT_CYCLES = 2000000000LL;

// float offsets of element (r, kk) in the A and B operands
__device__ __forceinline__ int aoff(int r, int kk) {
    return (r >> 3) * (int)(A_SBO / 4) + (kk >> 2) * (int)(A_LBO / 4) + (r & 7) * 4 + (kk & 3);
}
__device__ __forceinline__ int boff(int n, int kk) {
    return (n >> 3) * (int)(B_SBO / 4) + (kk >> 2) * (int)(B_LBO / 4) + (n & 7) * 4 + (kk & 3);
}

// Thread t's share of T_s: element pairs (a, b, c0), (a, b, c0 + 1) for a = ap + 2 m, m < 8, with
// lane bits 0-1 -> b bits 0-1, lane bit 2 -> ap, lane bits 3-4 -> c0 bits 1-2, and the warp
// index giving b bits 2-3 (warp bits 0-1) and c0 bit 3 (warp bit 2).  A warp reads two values of
// a, four of b and four pairs of c: 64 contiguous bytes of eight rows.
struct ShareCoord {
    int b, c0, ap;
    __device__ __forceinline__ ShareCoord(int t)
        : b((t & 3) + 4 * ((t >> 5) & 3)), c0(2 * (((t >> 3) & 3) + 4 * (t >> 7))), ap((t >> 2) & 1) {}
};

__device__ __forceinline__ void load_share(const float2* __restrict__ ts, float4 (&v)[8]) {
    const ShareCoord q(threadIdx.x);
    const float4* p = reinterpret_cast<const float4*>(ts);
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = p[((q.ap + 2 * m) * 256 + q.b * 16 + q.c0) >> 1];
}

// the share into a swizzled close buffer (layout of tiled_d3c16.cuh)
__device__ __forceinline__ void store_share_swizzled(const float4 (&v)[8], float2* __restrict__ X) {
    const ShareCoord q(threadIdx.x);
#pragma unroll
    for (int m = 0; m < 8; ++m)
        *reinterpret_cast<float4*>(X + (q.ap + 2 * m) * 256 + q.b * 16 + (q.c0 ^ ((q.b & 7) << 1))) = v[m];
}

struct Split {
    float hi, lo;
};
__device__ __forceinline__ Split split(float v) {
    const float h = tc::to_tf32(v);
    return {h, tc::to_tf32(v - h)};
}

// A operand of the product on bond X (2: c, 1: b, 0: a) from the share, hi and lo.  For X = 1, 0
// the two elements of a pair go to different rows; lane bit 1 picks which is stored first, so
// that each 8-byte store instruction of a warp covers all 16 bank pairs twice.
template <int X>
__device__ __forceinline__ void store_a(const float4 (&v)[8], float* __restrict__ ahi, float* __restrict__ alo) {
    const ShareCoord q(threadIdx.x);
    const bool swap = (threadIdx.x >> 1) & 1;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int a = q.ap + 2 * m;
        const Split e0 = split(v[m].x), e1 = split(v[m].y), e2 = split(v[m].z), e3 = split(v[m].w);
        if (X == 2) {   // r = 16 a + b, kk = 2 c + p: the pair is one 16-byte chunk
            const int o = aoff(16 * a + q.b, 2 * q.c0);
            *reinterpret_cast<float4*>(ahi + o) = make_float4(e0.hi, e1.hi, e2.hi, e3.hi);
            *reinterpret_cast<float4*>(alo + o) = make_float4(e0.lo, e1.lo, e2.lo, e3.lo);
        } else {
            // X == 1: r = 16 a + c, kk = 2 b + p;  X == 0: r = 16 b + c, kk = 2 a + p
            const int r0 = X == 1 ? 16 * a + q.c0 : 16 * q.b + q.c0;
            const int kk = X == 1 ? 2 * q.b : 2 * a;
            const int o0 = aoff(r0, kk), o1 = aoff(r0 + 1, kk);
            const int oa = swap ? o1 : o0, ob = swap ? o0 : o1;
            const float2 ha = swap ? make_float2(e2.hi, e3.hi) : make_float2(e0.hi, e1.hi);
            const float2 hb = swap ? make_float2(e0.hi, e1.hi) : make_float2(e2.hi, e3.hi);
            const float2 la = swap ? make_float2(e2.lo, e3.lo) : make_float2(e0.lo, e1.lo);
            const float2 lb = swap ? make_float2(e0.lo, e1.lo) : make_float2(e2.lo, e3.lo);
            *reinterpret_cast<float2*>(ahi + oa) = ha;
            *reinterpret_cast<float2*>(ahi + ob) = hb;
            *reinterpret_cast<float2*>(alo + oa) = la;
            *reinterpret_cast<float2*>(alo + ob) = lb;
        }
    }
}

// B operands of the three messages (message k: hi at bops + k * 2 B_BYTES, lo B_BYTES further;
// byte offsets) from the incoming messages in global memory (M_k[y][x] = m[k][16 y + x]);
// thread t forms entry (y, x) = (t >> 4, t & 15).
__device__ __forceinline__ void store_b(const float2* const (&mg)[3], float* __restrict__ bops) {
    const int t = threadIdx.x;
    const int y = t >> 4, x = t & 15;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float2 m = mg[k][y * 16 + x];
        const Split re = split(m.x), im = split(m.y), nim = split(-m.y);
        float* hi = bops + k * (2 * B_BYTES / 4);
        float* lo = hi + B_BYTES / 4;
        const int o0 = boff(2 * y, 2 * x), o1 = boff(2 * y + 1, 2 * x);
        *reinterpret_cast<float2*>(hi + o0) = make_float2(re.hi, nim.hi);
        *reinterpret_cast<float2*>(lo + o0) = make_float2(re.lo, nim.lo);
        *reinterpret_cast<float2*>(hi + o1) = make_float2(im.hi, re.hi);
        *reinterpret_cast<float2*>(lo + o1) = make_float2(im.lo, re.lo);
    }
}

// One thread: the 24 MMAs of a product (2 row tiles x 4 K steps x 3 terms) into columns col.
__device__ __forceinline__ void issue_product(uint32_t tmem, uint32_t col, uint32_t a_base, uint32_t b_base) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const uint32_t d = tmem + col + 32 * j;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const uint32_t ao = a_base + j * 16 * A_SBO + s * 2 * A_LBO, bo = b_base + s * 2 * B_LBO;
            const uint64_t ahi = tc::desc_noswz(ao + A_HI, A_LBO, A_SBO), alo = tc::desc_noswz(ao + A_LO, A_LBO, A_SBO);
            const uint64_t bhi = tc::desc_noswz(bo, B_LBO, B_SBO), blo = tc::desc_noswz(bo + B_BYTES, B_LBO, B_SBO);
            tc::mma_tf32(d, alo, bhi, IDESC, s > 0 ? 1u : 0u);
            tc::mma_tf32(d, ahi, blo, IDESC, 1u);
            tc::mma_tf32(d, ahi, bhi, IDESC, 1u);
        }
    }
}

// f *= s[0] * s[1] on 32 accumulator words (each factor applied in turn)
__device__ __forceinline__ void scale32(uint32_t (&f)[32], const float (&s)[2]) {
#pragma unroll
    for (int i = 0; i < 32; ++i) f[i] = __float_as_uint(__uint_as_float(f[i]) * s[0] * s[1]);
}

// Epilogue of one warp: its 32 rows (quarter w % 4 of row tile w / 4) of the three products,
// from tensor memory into the swizzled close buffers of the region.  SCALED: the accumulators
// of V_2, V_1, V_0 are multiplied by sc[0][0] sc[0][1], sc[1][0] sc[1][1], sc[2][0] sc[2][1]
// (powers of two that undo the operand scaling of the FP16 products; two factors so that the
// product may leave the float exponent range while each factor stays in it).
template <bool SCALED = false>
__device__ __forceinline__ void epilogue(uint32_t tmem, float2* __restrict__ region, const float (&sc)[3][2] = {}) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j = w >> 2, qd = w & 3;
    const int r = 128 * j + 32 * qd + lane;
    const uint32_t tl = tmem + ((uint32_t)(32 * qd) << 16) + 32 * j;
    uint32_t f[32];
    {   // V_2: r = 16 a + b, columns y -> V_2[a][b][y]
        tc::ld_32x32b_x32(tl + COL_V2, f);
        tc::wait_ld();
        if (SCALED) scale32(f, sc[0]);
        const int a = r >> 4, b = r & 15;
        float2* row = region + X_V2 + a * 256 + b * 16;
#pragma unroll
        for (int u = 0; u < 8; ++u)
            *reinterpret_cast<float4*>(row + ((2 * u) ^ ((b & 7) << 1))) =
                make_float4(__uint_as_float(f[4 * u]), __uint_as_float(f[4 * u + 1]), __uint_as_float(f[4 * u + 2]),
                            __uint_as_float(f[4 * u + 3]));
    }
    {   // V_1: r = 16 a + c, columns y (new b) -> V_1[a][y][c]
        tc::ld_32x32b_x32(tl + COL_V1, f);
        tc::wait_ld();
        if (SCALED) scale32(f, sc[1]);
        const int a = r >> 4, c = r & 15;
        float2* base = region + X_V1 + a * 256;
#pragma unroll
        for (int y = 0; y < 16; ++y)
            base[y * 16 + (c ^ ((y & 7) << 1))] = make_float2(__uint_as_float(f[2 * y]), __uint_as_float(f[2 * y + 1]));
    }
    {   // V_0: r = 16 b + c, columns y (new a) -> V_0[y][b][c]
        tc::ld_32x32b_x32(tl + COL_V0, f);
        tc::wait_ld();
        if (SCALED) scale32(f, sc[2]);
        const int b = r >> 4, c = r & 15;
        float2* base = region + X_V0 + b * 16 + (c ^ ((b & 7) << 1));
#pragma unroll
        for (int y = 0; y < 16; ++y)
            base[y * 256] = make_float2(__uint_as_float(f[2 * y]), __uint_as_float(f[2 * y + 1]));
    }
}

}  // namespace tcd3
}  // namespace bqa
