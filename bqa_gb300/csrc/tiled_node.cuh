// Register-tiled complex64 node contraction for compile-time (degree D, bond dim CHI),
// CHI a multiple of 4.  Same mathematics as node_kernel (node_kernels.cu), organised as
// small GEMMs on shared-memory operands:
//
//   bond product on bond k:   Y[a][i][b] = sum_j M[i][j] X[a][j][b]
//       A = 2 CHI^k rows (s included), B = CHI^(D-1-k) columns.  A thread owns a 4x4 tile of
//       complex accumulators: 4 values of i times 4 of b (B >= 4), or 4 of a times 4 of i on
//       the last bond (B = 1).  Operands come in as 128-bit loads (two complex values) from
//       the tensor and from the transposed message Mt[j][i] = M[i][j].
//   closing contraction for bond idx:
//       P_s[a][b] = sum_{x,y} conj(X[s][x][a][y]) R[s][x][b][y]   (X = T or a product of T)
//       a thread owns a 4x4 tile of (a, b) for one K-slice; the KS slices of a tile sit in
//       adjacent lanes and are summed by recursive halving (reduce_tile).
//
// Tensor buffers in shared memory are XOR-swizzled in 16-byte chunks: element e lives at
// e ^ (((e >> 4) & SW) << 1), SW = 7 for CHI = 16 and 3 for CHI = 8.  A 16-element row is
// 128 bytes, so without the swizzle the same column of consecutive rows falls in one bank
// group; with it, 8 consecutive rows hit 8 distinct groups, and every aligned pair of
// complex values stays contiguous (bit 0 is untouched).
//
// D = 3 splits the two messages of each outgoing message between the two sides of the
// closing contraction.  BP messages are Hermitian (M^H = M), so
//     sum_x conj(T[..x..]) M[x][y] = conj((T x M)[..y..]),
// and with V_k = T x_k M_k the message of bond 0 is the closing contraction of V_1 (conj
// side) with V_2, bond 1 of V_0 with V_2, bond 2 of V_0 with V_1: 3 products and 3 closing
// contractions instead of the reference order's 6 + 3.  V_0 is formed in place over T once T
// has served V_1 and V_2, so three tensor buffers still suffice.  D = 4 shares bond
// products instead: with U = T x_0 M_0 x_1 M_1 the messages of bonds 3 and 2 close U x_2 M_2
// and U x_3 M_3, and V = T x_2 M_2 x_3 M_3 serves bonds 1 and 0: 8 products and 4 closing
// contractions instead of 12 + 4.
#pragma once

#include "common.cuh"

namespace bqa {
namespace tiled {

__host__ __device__ constexpr int cpow(int b, int e) { return e == 0 ? 1 : b * cpow(b, e - 1); }

template <int D, int CHI>
struct Shape {
    static constexpr int PER_S = cpow(CHI, D);
    static constexpr int NT = 2 * PER_S;
    static constexpr int N2 = CHI * CHI;
    static constexpr int PROD_TILES = 2 * (CHI / 4) * (cpow(CHI, D - 1) / 4 > 0 ? cpow(CHI, D - 1) / 4 : 1);
    static constexpr int R32 = ((PROD_TILES + 31) / 32) * 32;
    static constexpr int THREADS = R32 > 512 ? 512 : R32;
    static constexpr int CLOSE_TILES = 2 * (CHI / 4) * (CHI / 4);
    static constexpr int KS_RAW = THREADS / CLOSE_TILES;
    static constexpr int KS = KS_RAW >= 32 ? 32 : (KS_RAW >= 16 ? 16 : (KS_RAW >= 8 ? 8 : (KS_RAW >= 4 ? 4 : (KS_RAW >= 2 ? 2 : 1))));
    static constexpr int SW = CHI == 16 ? 7 : (CHI == 8 ? 3 : 0);
    // shared memory (float2 elements): T, two buffers, D transposed messages, P (2 blocks), scratch
    static constexpr int SMEM_ELEMS = 3 * NT + D * N2 + 2 * N2 + 128;
};

// One CTA per (node, physical index s): the two values of s never mix inside a message
// contraction, so a node splits into two independent halves of half the shared memory.
// The half-node blocks P_s are Hermitian (the message of one physical index), so the closing
// contractions form only the 4x4 tiles on and above the diagonal (NG (NG + 1) / 2 of NG^2) and
// the written block takes the tiles below it as conjugate transposes (write_half_block).
template <int D, int CHI>
struct HalfShape {
    static constexpr int PER_S = cpow(CHI, D);
    static constexpr int N2 = CHI * CHI;
    static constexpr int PROD_TILES = (CHI / 4) * (cpow(CHI, D - 1) / 4 > 0 ? cpow(CHI, D - 1) / 4 : 1);
    static constexpr int R32 = ((PROD_TILES + 31) / 32) * 32;
    static constexpr int THREADS = R32 > 512 ? 512 : R32;
    static constexpr int CLOSE_TILES = (CHI / 4) * (CHI / 4 + 1) / 2;
    static constexpr int KS_RAW = THREADS / CLOSE_TILES;
    static constexpr int KS = KS_RAW >= 32 ? 32 : (KS_RAW >= 16 ? 16 : (KS_RAW >= 8 ? 8 : (KS_RAW >= 4 ? 4 : (KS_RAW >= 2 ? 2 : 1))));
    static constexpr int SW = CHI == 16 ? 7 : (CHI == 8 ? 3 : 0);
    // T_s, two buffers, D transposed messages, P_s (two buffers: the (3, 16) kernel alternates)
    static constexpr int SMEM_ELEMS = 3 * PER_S + D * N2 + 2 * N2;
};

template <int SW>
__device__ __forceinline__ int swz(int e) { return SW ? (e ^ (((e >> 4) & SW) << 1)) : e; }

__device__ __forceinline__ void ld2(const float2* p, float2& a, float2& b) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    a = make_float2(v.x, v.y);
    b = make_float2(v.z, v.w);
}
__device__ __forceinline__ void st2(float2* p, float2 a, float2 b) {
    *reinterpret_cast<float4*>(p) = make_float4(a.x, a.y, b.x, b.y);
}

// Y[a][i][b] = sum_j Mt[j][i] X[a][j][b], B >= 4 (B a multiple of 4)
template <int CHI, int THREADS, int SW>
__device__ __forceinline__ void product_inner(const float2* __restrict__ X, float2* __restrict__ Y,
                                              const float2* __restrict__ Mt, int A, int B) {
    constexpr int NIG = CHI / 4;
    const int nbg = B >> 2;
    const int tiles = A * NIG * nbg;
    for (int t = threadIdx.x; t < tiles; t += THREADS) {
        const int bg = t % nbg;
        const int rest = t / nbg;
        const int ig = rest % NIG;
        const int a = rest / NIG;
        float2 acc[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = make_float2(0.f, 0.f);
        const int xb = a * CHI * B + bg * 4;
        const float2* mp = Mt + ig * 4;
#pragma unroll 4
        for (int j = 0; j < CHI; ++j) {
            float2 x[4], m[4];
            const int e = xb + j * B;
            ld2(X + swz<SW>(e), x[0], x[1]);
            ld2(X + swz<SW>(e + 2), x[2], x[3]);
            ld2(mp + j * CHI, m[0], m[1]);
            ld2(mp + j * CHI + 2, m[2], m[3]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = c_fma(m[u], x[v], acc[u][v]);
        }
        const int yb = (a * CHI + ig * 4) * B + bg * 4;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            st2(Y + swz<SW>(yb + u * B), acc[u][0], acc[u][1]);
            st2(Y + swz<SW>(yb + u * B + 2), acc[u][2], acc[u][3]);
        }
    }
}

// Y[a][i] = sum_j X[a][j] Mt[j][i]  (product on the last bond, B = 1)
template <int CHI, int THREADS, int SW>
__device__ __forceinline__ void product_last(const float2* __restrict__ X, float2* __restrict__ Y,
                                             const float2* __restrict__ Mt, int A) {
    constexpr int NIG = CHI / 4;
    const int tiles = (A >> 2) * NIG;
    for (int t = threadIdx.x; t < tiles; t += THREADS) {
        const int ig = t % NIG;
        const int a0 = (t / NIG) * 4;
        float2 acc[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = make_float2(0.f, 0.f);
        const float2* mp = Mt + ig * 4;
#pragma unroll 2
        for (int j = 0; j < CHI; j += 2) {
            float2 x[4][2], m0[4], m1[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) ld2(X + swz<SW>((a0 + u) * CHI + j), x[u][0], x[u][1]);
            ld2(mp + j * CHI, m0[0], m0[1]);
            ld2(mp + j * CHI + 2, m0[2], m0[3]);
            ld2(mp + (j + 1) * CHI, m1[0], m1[1]);
            ld2(mp + (j + 1) * CHI + 2, m1[2], m1[3]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    acc[u][v] = c_fma(x[u][0], m0[v], acc[u][v]);
                    acc[u][v] = c_fma(x[u][1], m1[v], acc[u][v]);
                }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int yb = (a0 + u) * CHI + ig * 4;
            st2(Y + swz<SW>(yb), acc[u][0], acc[u][1]);
            st2(Y + swz<SW>(yb + 2), acc[u][2], acc[u][3]);
        }
    }
}

// X <- X x_0 M in place (bond 0 of a [NS][CHI]^D buffer): every thread owns at most one
// 4x4 tile, accumulates it from X, and writes it back only after the barrier that follows
// the last read of X by any thread.
template <int D, int CHI, int THREADS, int SW, int NS>
__device__ __forceinline__ void product_first_inplace(float2* X, const float2* __restrict__ Mt) {
    constexpr int NIG = CHI / 4;
    constexpr int B = cpow(CHI, D - 1);
    constexpr int NBG = B / 4;
    constexpr int TILES = NS * NIG * NBG;
    static_assert(TILES <= THREADS, "in-place bond-0 product needs one tile per thread");
    const int t = threadIdx.x;
    const int bg = t % NBG, ig = (t / NBG) % NIG, a = t / (NBG * NIG);
    float2 acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = make_float2(0.f, 0.f);
    if (t < TILES) {
        const int xb = a * CHI * B + bg * 4;
        const float2* mp = Mt + ig * 4;
#pragma unroll 4
        for (int j = 0; j < CHI; ++j) {
            float2 x[4], m[4];
            const int e = xb + j * B;
            ld2(X + swz<SW>(e), x[0], x[1]);
            ld2(X + swz<SW>(e + 2), x[2], x[3]);
            ld2(mp + j * CHI, m[0], m[1]);
            ld2(mp + j * CHI + 2, m[2], m[3]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = c_fma(m[u], x[v], acc[u][v]);
        }
    }
    __syncthreads();
    if (t < TILES) {
        const int yb = (a * CHI + ig * 4) * B + bg * 4;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            st2(X + swz<SW>(yb + u * B), acc[u][0], acc[u][1]);
            st2(X + swz<SW>(yb + u * B + 2), acc[u][2], acc[u][3]);
        }
    }
}

// Bond product on bond k of a [NS][CHI]^D buffer (NS = 2: both values of the physical index,
// NS = 1: one of them).
template <int D, int CHI, int THREADS, int SW, int NS = 2>
__device__ __forceinline__ void product(const float2* X, float2* Y, const float2* Mt, int k) {
    if (k == D - 1)
        product_last<CHI, THREADS, SW>(X, Y, Mt, NS * cpow(CHI, D - 1));
    else
        product_inner<CHI, THREADS, SW>(X, Y, Mt, NS * ipow(CHI, k), ipow(CHI, D - 1 - k));
}

// P[s][a][b] = sum_{x<Ax, y<B} conj(T[s][x][a][y]) R[s][x][b][y]; per s the operands are
// [Ax][CHI][B] with Ax * CHI * B = PER_S.  Result written to P[NS][CHI][CHI].
// Sum a 4x4 complex tile over its KS K-slices (KS adjacent lanes, a power of two <= 32) by
// recursive halving: in the round with lane bit b every lane keeps one half of its values
// and adds the partner's copy of that half, so after log2(KS) rounds lane ks holds the
// 32/KS floats e = ks * (32/KS) + i of the tile (float e = component e & 1 of element e >> 1,
// element q = 4u + v), each summed over all slices.  The lane writes them to P (row stride
// CHI) if the tile is active.  32/KS * (2 - 2/KS) shuffles instead of 32 log2(KS).
template <int KS, int CHI>
__device__ __forceinline__ void reduce_tile(float2 (&acc)[4][4], int ks, bool active, float2* __restrict__ P,
                                            int ag, int bg) {
    float w[32];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        w[2 * q] = acc[q >> 2][q & 3].x;
        w[2 * q + 1] = acc[q >> 2][q & 3].y;
    }
#pragma unroll
    for (int b = KS / 2, n = 32; b > 0; b >>= 1, n >>= 1) {
        const bool up = (ks & b) != 0;
#pragma unroll
        for (int i = 0; i < n / 2; ++i) {
            const float send = up ? w[i] : w[n / 2 + i];
            const float keep = up ? w[n / 2 + i] : w[i];
            w[i] = keep + __shfl_xor_sync(BQA_FULL_MASK, send, b);
        }
    }
    if (active) {
        constexpr int NF = 32 / KS;
        float* pf = reinterpret_cast<float*>(P);
#pragma unroll
        for (int i = 0; i < NF; ++i) {
            const int e = ks * NF + i, q = e >> 1;
            pf[2 * ((ag * 4 + (q >> 2)) * CHI + bg * 4 + (q & 3)) + (e & 1)] = w[i];
        }
    }
}

// Tile k of the upper triangle (row-major, diagonal included) of an NG x NG tile grid.
__device__ __forceinline__ void upper_tile(int k, int NG, int& ag, int& bg) {
    ag = 0;
    int rem = k;
#pragma unroll 1
    while (ag < NG - 1 && rem >= NG - ag) {
        rem -= NG - ag;
        ++ag;
    }
    bg = ag + rem;
}

// HERM (one physical index, NS = 1): only the tiles on and above the diagonal.
template <int CHI, int THREADS, int KS, int PER_S, int SW, int NS = 2, bool HERM = false>
__device__ __forceinline__ void close_tiled(const float2* __restrict__ T, const float2* __restrict__ Rt,
                                            float2* __restrict__ P, int Ax, int B) {
    static_assert(!HERM || NS == 1, "Hermitian closing contractions are per physical index");
    constexpr int NG = CHI / 4;
    constexpr int TILES = HERM ? NG * (NG + 1) / 2 : NS * NG * NG;
    const int t = threadIdx.x;
    const int ks = t % KS;
    const int tile = t / KS;
    const bool active = tile < TILES;
    const int s = (active && !HERM) ? tile / (NG * NG) : 0;
    int ag = (tile / NG) % NG, bg = tile % NG;
    if (HERM) upper_tile(active ? tile : 0, NG, ag, bg);
    float2 acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = make_float2(0.f, 0.f);
    const int tb = s * PER_S + ag * 4 * B;
    const int rb = s * PER_S + bg * 4 * B;
    if (active) {
        if (B >= 2) {
            // K runs over (x, y) in pairs of y
            const int hb = B >> 1;
            const int K2 = Ax * hb;
            for (int p = ks; p < K2; p += KS) {
                const int x = p / hb, y = (p - x * hb) * 2;
                const int off = x * CHI * B + y;
                float2 tv[4][2], rv[4][2];
#pragma unroll
                for (int u = 0; u < 4; ++u) ld2(T + swz<SW>(tb + off + u * B), tv[u][0], tv[u][1]);
#pragma unroll
                for (int v = 0; v < 4; ++v) ld2(Rt + swz<SW>(rb + off + v * B), rv[v][0], rv[v][1]);
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int v = 0; v < 4; ++v) {
                        acc[u][v] = c_fma_conj(tv[u][0], rv[v][0], acc[u][v]);
                        acc[u][v] = c_fma_conj(tv[u][1], rv[v][1], acc[u][v]);
                    }
            }
        } else {
            // last bond: operands [Ax][CHI]; rows x, 4 consecutive a / b per thread
            for (int x = ks; x < Ax; x += KS) {
                float2 tv[4], rv[4];
                ld2(T + swz<SW>(tb + x * CHI), tv[0], tv[1]);
                ld2(T + swz<SW>(tb + x * CHI + 2), tv[2], tv[3]);
                ld2(Rt + swz<SW>(rb + x * CHI), rv[0], rv[1]);
                ld2(Rt + swz<SW>(rb + x * CHI + 2), rv[2], rv[3]);
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int v = 0; v < 4; ++v) acc[u][v] = c_fma_conj(tv[u], rv[v], acc[u][v]);
            }
        }
    }
    // sum the KS slices (adjacent lanes)
    reduce_tile<KS, CHI>(acc, ks, active, P + (size_t)s * CHI * CHI, ag, bg);
}

// Y = X x_k diag(M) for degree 3: Y[e] = M[i][i] X[e], i the bond-k index of element e =
// x0 CHI^2 + x1 CHI + x2 (Mt is the transposed message, its diagonal at i CHI + i).  The dense
// product with a diagonal M adds exact zeros to this one term, so the values are the same.
// Elementwise: X == Y (in place) is allowed.
template <int CHI, int TH, int SW>
__device__ __forceinline__ void diag_scale3(const float2* X, float2* Y, const float2* __restrict__ Mt, int k) {
    constexpr int PS = CHI * CHI * CHI;
    const int div = k == 0 ? CHI * CHI : (k == 1 ? CHI : 1);
    for (int e = threadIdx.x; e < PS; e += TH) {
        const int i = (e / div) % CHI;
        const int p = swz<SW>(e);
        Y[p] = c_fma(Mt[i * CHI + i], X[p], make_float2(0.f, 0.f));
    }
}

// Copy a half-node block P (CHI x CHI, row-major, upper tiles valid) to global memory, the
// tiles below the diagonal as conjugate transposes of those above.
// Threads t0 .. t0 + nt - 1 of the block take part (t = this thread's index among them).
template <int CHI>
__device__ __forceinline__ void write_half_block(const float2* __restrict__ P, float4* __restrict__ og, int t,
                                                 int nt) {
    const float4* sp = reinterpret_cast<const float4*>(P);
    for (int i = t; i < CHI * CHI / 2; i += nt) {
        const int r = (2 * i) / CHI, c = (2 * i) % CHI;
        if ((r >> 2) > (c >> 2)) {
            const float2 x = P[c * CHI + r], y = P[(c + 1) * CHI + r];
            og[i] = make_float4(x.x, -x.y, y.x, -y.y);
        } else {
            og[i] = sp[i];
        }
    }
}

}  // namespace tiled
}  // namespace bqa
