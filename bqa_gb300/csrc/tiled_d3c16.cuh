// The half-node message kernel's operations specialised to degree 3, bond dim 16 (one CTA of
// 256 threads per (node, s), 16^3 complex per buffer): the products and closing contractions
// of tiled_node.cuh with every swizzled shared-memory address reduced to a per-thread base
// plus a compile-time offset.
//
// A buffer holds element (x0, x1, x2) at x0*256 + x1*16 + (x2 ^ ((x1 & 7) << 1)) (the XOR
// swizzle of tiled_node.cuh: 16-byte chunks of a 128-byte row permuted by the row index).
// In every access pattern below the swizzle term depends on one or two per-thread bits and on
// loop indices that are compile-time after unrolling, so the generic form's three integer
// operations per load disappear; the arithmetic and its order are the generic functions'.
// Each closed form was checked against the generic swizzle for every thread and index.
#pragma once

#include "tiled_node.cuh"

namespace bqa {
namespace tiled {
namespace d3c16 {

constexpr int TH = 256;

// T[s] (16^3 complex) from global memory into a swizzled buffer
__device__ __forceinline__ void load_half(float2* __restrict__ sT, const float4* __restrict__ tg) {
    const int t = threadIdx.x;
    const int base = (2 * t) ^ (((t >> 3) & 7) << 1);
#pragma unroll
    for (int m = 0; m < 8; ++m) *reinterpret_cast<float4*>(sT + base + 512 * m) = tg[t + 256 * m];
}

__device__ __forceinline__ void zero(float2 (&acc)[4][4]) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = make_float2(0.f, 0.f);
}

// Y = X x_1 M (bond 1): thread = tile (a = x0, ig = 4 values of the new x1, bg = 4 values of x2)
__device__ __forceinline__ void prod1(const float2* __restrict__ X, float2* __restrict__ Y,
                                      const float2* __restrict__ Mt) {
    const int t = threadIdx.x;
    const int bg = t & 3, ig = (t >> 2) & 3, a = t >> 4;
    const float2* P[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) P[m] = X + a * 256 + 4 * (bg ^ m);
    const float2* mp = Mt + ig * 4;
    float2 acc[4][4];
    zero(acc);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        float2 x[4], m[4];
        const float2* pj = P[(j >> 1) & 3] + j * 16;
        ld2(pj + 2 * (j & 1), x[0], x[1]);
        ld2(pj + 2 * (1 ^ (j & 1)), x[2], x[3]);
        ld2(mp + j * 16, m[0], m[1]);
        ld2(mp + j * 16 + 2, m[2], m[3]);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = c_fma(m[u], x[v], acc[u][v]);
    }
    float2* Q[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) Q[h] = Y + (a * 16 + ig * 4) * 16 + 4 * (bg ^ (2 * (ig & 1) + h));
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        float2* q = Q[u >> 1] + u * 16;
        st2(q + 2 * (u & 1), acc[u][0], acc[u][1]);
        st2(q + 2 * (1 ^ (u & 1)), acc[u][2], acc[u][3]);
    }
}

// Y = X x_2 M (last bond): thread = tile (4 rows a0.., ig = 4 values of the new x2)
__device__ __forceinline__ void prod2(const float2* __restrict__ X, float2* __restrict__ Y,
                                      const float2* __restrict__ Mt) {
    const int t = threadIdx.x;
    const int ig = t & 3, a0 = (t >> 2) * 4, p = (t >> 2) & 1;
    // rows a0..a0+3 have (row & 7) = 4p + u: the swizzle flips bit 3 of the column when p = 1
    const float2* R0 = X + a0 * 16 + 8 * p;
    const float2* R1 = X + a0 * 16 - 8 * p;
    const float2* mp = Mt + ig * 4;
    float2 acc[4][4];
    zero(acc);
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
        float2 x[4][2], m0[4], m1[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int xo = j ^ (2 * u);
            ld2(((xo & 8) ? R1 : R0) + u * 16 + xo, x[u][0], x[u][1]);
        }
        ld2(mp + j * 16, m0[0], m0[1]);
        ld2(mp + j * 16 + 2, m0[2], m0[3]);
        ld2(mp + (j + 1) * 16, m1[0], m1[1]);
        ld2(mp + (j + 1) * 16 + 2, m1[2], m1[3]);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                acc[u][v] = c_fma(x[u][0], m0[v], acc[u][v]);
                acc[u][v] = c_fma(x[u][1], m1[v], acc[u][v]);
            }
    }
    float2* S[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) S[h] = Y + a0 * 16 + 4 * (ig ^ (2 * p + h));
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        float2* q = S[u >> 1] + u * 16;
        st2(q + 2 * (u & 1), acc[u][0], acc[u][1]);
        st2(q + 2 * (1 ^ (u & 1)), acc[u][2], acc[u][3]);
    }
}

// X <- X x_0 M in place (bond 0): thread = tile (ig = 4 values of the new x0, bg = 4 values of
// (x1, x2)); all reads precede the barrier, all writes follow it
__device__ __forceinline__ void prod0_inplace(float2* X, const float2* __restrict__ Mt) {
    const int t = threadIdx.x;
    const int bg = t & 63, ig = t >> 6;
    const int c = ((bg >> 2) & 7) << 1;
    const int b0 = (bg >> 2) * 16 + ((4 * (bg & 3)) ^ c);
    const int b2 = (bg >> 2) * 16 + ((4 * (bg & 3) + 2) ^ c);
    const float2* mp = Mt + ig * 4;
    float2 acc[4][4];
    zero(acc);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        float2 x[4], m[4];
        ld2(X + b0 + j * 256, x[0], x[1]);
        ld2(X + b2 + j * 256, x[2], x[3]);
        ld2(mp + j * 16, m[0], m[1]);
        ld2(mp + j * 16 + 2, m[2], m[3]);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = c_fma(m[u], x[v], acc[u][v]);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        st2(X + (ig * 4 + u) * 256 + b0, acc[u][0], acc[u][1]);
        st2(X + (ig * 4 + u) * 256 + b2, acc[u][2], acc[u][3]);
    }
}

// P[a][b] = sum conj(X[..]) R[..] over every index but bond IDX; thread = (tile (ag, bg), K-slice ks).
// P is Hermitian: the 10 tiles with ag <= bg (tiled::upper_tile order) run on warps 0-4, warps 5-7
// have no closing work (the block's lower tiles are written as conjugates).
template <int IDX>
__device__ __forceinline__ void close(const float2* __restrict__ X, const float2* __restrict__ R,
                                      float2* __restrict__ P) {
    const int t = threadIdx.x;
    const int ks = t & 15, tile = t >> 4;
    if (tile >= 10) return;
    const int ag = tile < 4 ? 0 : (tile < 7 ? 1 : (tile < 9 ? 2 : 3));
    const int bg = ag + tile - (ag == 0 ? 0 : (ag == 1 ? 4 : (ag == 2 ? 7 : 9)));
    const int b3 = ks >> 3;
    float2 acc[4][4];
    zero(acc);
    if (IDX == 0) {
        // K = (x1, x2) in pairs: y = 2 (ks + 16 it); rows (4ag + u) * 16 + b3 + 2 it
        const int z = (ks & 7) ^ b3;
        const float2* TB[4];
        const float2* RB[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            TB[m] = X + ag * 1024 + b3 * 16 + 2 * (z ^ (2 * m));
            RB[m] = R + bg * 1024 + b3 * 16 + 2 * (z ^ (2 * m));
        }
#pragma unroll
        for (int it = 0; it < 8; ++it) {
            float2 tv[4][2], rv[4][2];
#pragma unroll
            for (int u = 0; u < 4; ++u) ld2(TB[it & 3] + u * 256 + 32 * it, tv[u][0], tv[u][1]);
#pragma unroll
            for (int v = 0; v < 4; ++v) ld2(RB[it & 3] + v * 256 + 32 * it, rv[v][0], rv[v][1]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    acc[u][v] = c_fma_conj(tv[u][0], rv[v][0], acc[u][v]);
                    acc[u][v] = c_fma_conj(tv[u][1], rv[v][1], acc[u][v]);
                }
        }
    } else if (IDX == 1) {
        // K = (x0, x2 pairs): x0 = b3 + 2 it, x2 = 2 (ks & 7); rows x0 * 16 + 4ag + u
        const float2* TB[4];
        const float2* RB[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            TB[u] = X + b3 * 256 + ag * 64 + 2 * ((ks & 7) ^ (4 * (ag & 1) + u)) + u * 16;
            RB[u] = R + b3 * 256 + bg * 64 + 2 * ((ks & 7) ^ (4 * (bg & 1) + u)) + u * 16;
        }
#pragma unroll
        for (int it = 0; it < 8; ++it) {
            float2 tv[4][2], rv[4][2];
#pragma unroll
            for (int u = 0; u < 4; ++u) ld2(TB[u] + 512 * it, tv[u][0], tv[u][1]);
#pragma unroll
            for (int v = 0; v < 4; ++v) ld2(RB[v] + 512 * it, rv[v][0], rv[v][1]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    acc[u][v] = c_fma_conj(tv[u][0], rv[v][0], acc[u][v]);
                    acc[u][v] = c_fma_conj(tv[u][1], rv[v][1], acc[u][v]);
                }
        }
    } else {
        // K = (x0, x1) rows x = ks + 16 it; the open index x2 = 4ag + u (4bg + v)
        const int c = 2 * (ks & 7);
        const float2* T0 = X + ks * 16 + ((4 * ag) ^ c);
        const float2* T2 = X + ks * 16 + ((4 * ag + 2) ^ c);
        const float2* R0 = R + ks * 16 + ((4 * bg) ^ c);
        const float2* R2 = R + ks * 16 + ((4 * bg + 2) ^ c);
#pragma unroll 4
        for (int it = 0; it < 16; ++it) {
            float2 tv[4], rv[4];
            ld2(T0 + 256 * it, tv[0], tv[1]);
            ld2(T2 + 256 * it, tv[2], tv[3]);
            ld2(R0 + 256 * it, rv[0], rv[1]);
            ld2(R2 + 256 * it, rv[2], rv[3]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = c_fma_conj(tv[u], rv[v], acc[u][v]);
        }
    }
    reduce_tile<16, 16>(acc, ks, true, P, ag, bg);
}

}  // namespace d3c16
}  // namespace tiled
}  // namespace bqa
