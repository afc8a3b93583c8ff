// Batched one-sided Jacobi SVD (Hestenes) for the truncation step of the simple update.
//
// A segment of W lanes (W = 8, 16 or 32, a power of two >= n) owns one n x n complex
// matrix, zero-padded to W x W: lane j keeps column j of A and column j of V in registers.
// A sweep visits every column pair once: in round r (1 <= r < W) lane j pairs with lane
// j ^ r, which is a perfect matching, and the W-1 rounds cover all pairs.  The pair's
// Gram entries alpha = |a_p|^2, beta = |a_q|^2, gamma = a_p^H a_q are formed by both lanes
// with the SAME operand order, so both make bit-identical rotation decisions; the rotation
//     a_p' = c a_p - s conj(e) a_q,   a_q' = s a_p + c conj(e) a_q,   e = gamma/|gamma|
// with t = sign(zeta)/(|zeta| + sqrt(1+zeta^2)), zeta = (beta-alpha)/(2|gamma|),
// c = 1/sqrt(1+t^2), s = c t, makes the pair orthogonal (the complex form of Hestenes'
// method, Demmel & Veselic 1992).  At convergence A V = U Sigma with sigma_j = |a_j|.
// A pair is rotated only if |gamma| > tol sqrt(alpha beta); sweeps stop when a whole sweep
// rotates nothing in the warp, or at the sweep cap (then a status bit is set).
#include "common.cuh"
#include "internal.h"

namespace bqa {

constexpr int kMaxSweeps = 40;

template <int W>
__device__ __forceinline__ bool jacobi_columns(float2 (&a)[W], float2 (&v)[W], int lane) {
    const float tol = (float)W * 1.2e-7f;
    bool any_rot = true;
    for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
        int rotated = 0;
#pragma unroll 1
        for (int r = 1; r < W; ++r) {
            const bool low = lane < (lane ^ r);
            float2 o[W];
            float alpha = 0.f, beta = 0.f;
            float2 g = c_zero();
#pragma unroll
            for (int i = 0; i < W; ++i) {
                o[i].x = __shfl_xor_sync(BQA_FULL_MASK, a[i].x, r, W);
                o[i].y = __shfl_xor_sync(BQA_FULL_MASK, a[i].y, r, W);
                const float2 p = low ? a[i] : o[i];
                const float2 q = low ? o[i] : a[i];
                alpha = fmaf(p.x, p.x, fmaf(p.y, p.y, alpha));
                beta = fmaf(q.x, q.x, fmaf(q.y, q.y, beta));
                g = c_fma_conj(p, q, g);
            }
            const float gabs = sqrtf(c_abs2(g));
            const bool rot = alpha > 1e-30f && beta > 1e-30f && gabs > tol * sqrtf(alpha) * sqrtf(beta);
            float c = 1.f, s = 0.f;
            float2 eb = make_float2(1.f, 0.f);  // conj(e)
            if (rot) {
                const float zeta = (beta - alpha) / (2.f * gabs);
                const float t = copysignf(1.f, zeta) / (fabsf(zeta) + hypotf(1.f, zeta));
                c = rsqrtf(fmaf(t, t, 1.f));
                s = c * t;
                eb = make_float2(g.x / gabs, -g.y / gabs);
                rotated = 1;
            }
#pragma unroll
            for (int i = 0; i < W; ++i) {
                const float2 p = low ? a[i] : o[i];
                const float2 q = c_mul(eb, low ? o[i] : a[i]);
                a[i] = low ? make_float2(c * p.x - s * q.x, c * p.y - s * q.y)
                           : make_float2(s * p.x + c * q.x, s * p.y + c * q.y);
            }
#pragma unroll
            for (int i = 0; i < W; ++i) {
                float2 ov;
                ov.x = __shfl_xor_sync(BQA_FULL_MASK, v[i].x, r, W);
                ov.y = __shfl_xor_sync(BQA_FULL_MASK, v[i].y, r, W);
                const float2 p = low ? v[i] : ov;
                const float2 q = c_mul(eb, low ? ov : v[i]);
                v[i] = low ? make_float2(c * p.x - s * q.x, c * p.y - s * q.y)
                           : make_float2(s * p.x + c * q.x, s * p.y + c * q.y);
            }
        }
        any_rot = __any_sync(BQA_FULL_MASK, rotated) != 0;
        if (!any_rot) return true;
    }
    return false;
}

template <int W>
__device__ __forceinline__ float seg_sum(float x) {
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) x += __shfl_xor_sync(BQA_FULL_MASK, x, o, W);
    return x;
}

// m = U S Vh per matrix (masked at eps) -> lu = sqrt(S) Vh, ul = U pinv(sqrt(S))
// (src/bqa/backends.py:483-490,709-727).
template <int W>
__global__ void __launch_bounds__(128) env_factor_kernel(const float2* __restrict__ mats, int count, int n,
                                                         float eps, float2* __restrict__ lu,
                                                         float2* __restrict__ ul, int32_t* status) {
    const int lane = threadIdx.x & (W - 1);
    const int mat = (blockIdx.x * blockDim.x + threadIdx.x) / W;
    const bool live = mat < count;
    const size_t base = (size_t)(live ? mat : 0) * n * n;
    float2 a[W], v[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
        a[i] = (live && i < n && lane < n) ? mats[base + (size_t)i * n + lane] : c_zero();
        v[i] = make_float2(i == lane ? 1.f : 0.f, 0.f);
    }
    const bool ok = jacobi_columns<W>(a, v, lane);
    if (!ok && live && lane == 0) atomicOr(status, BQA_STATUS_SVD_NOT_CONVERGED);
    float nrm2 = 0.f;
#pragma unroll
    for (int i = 0; i < W; ++i) nrm2 += c_abs2(a[i]);
    const float sig = sqrtf(nrm2);
    const bool keep = sig > eps;
    const float sq = sqrtf(sig);
    if (!live || lane >= n) return;
    // row `lane` of lu = sqrt(sigma) * conj(v)^T ; column `lane` of ul = a / (sigma sqrt(sigma))
    const float inv = keep ? 1.f / (sig * sq) : 0.f;
    const float sqk = keep ? sq : 0.f;
#pragma unroll
    for (int k = 0; k < W; ++k) {
        if (k < n) {
            lu[base + (size_t)lane * n + k] = make_float2(sqk * v[k].x, -sqk * v[k].y);
            ul[base + (size_t)k * n + lane] = c_scale(a[k], inv);
        }
    }
}

// Per undirected edge p: ker = lu[p] lu[p+h]^T = us s vhs; lambdas; canonicalisers
// (src/bqa/state.py:171-200).
template <int W>
__global__ void __launch_bounds__(128) bond_canon_kernel(const float2* __restrict__ lu, const float2* __restrict__ ul,
                                                         int edges, int n, float eps, float2* __restrict__ canon,
                                                         float* __restrict__ lmbds, uint32_t* colmax,
                                                         int32_t* status) {
    extern __shared__ float4 smem_raw[];
    const int lane = threadIdx.x & (W - 1);
    const int seg = threadIdx.x / W;
    float2* sm = reinterpret_cast<float2*>(smem_raw) + (size_t)seg * W * W;
    const int half = edges / 2;
    const int p = (blockIdx.x * blockDim.x + threadIdx.x) / W;
    const bool live = p < half;
    const int pf = live ? p : 0, pb = pf + half;
    const size_t nn = (size_t)n * n;
    // stage lu_f, then ker[:, lane] = lu_f . lu_b[lane, :]^T
    for (int i = lane; i < n * n; i += W) sm[i] = live ? lu[(size_t)pf * nn + i] : c_zero();
    __syncwarp();
    float2 brow[W];
#pragma unroll
    for (int k = 0; k < W; ++k) brow[k] = (live && lane < n && k < n) ? lu[(size_t)pb * nn + (size_t)lane * n + k] : c_zero();
    float2 a[W], v[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
        float2 acc = c_zero();
        if (i < n) {
#pragma unroll
            for (int k = 0; k < W; ++k)
                if (k < n) acc = c_fma(sm[i * n + k], brow[k], acc);
        }
        a[i] = acc;
        v[i] = make_float2(i == lane ? 1.f : 0.f, 0.f);
    }
    const bool ok = jacobi_columns<W>(a, v, lane);
    if (!ok && live && lane == 0) atomicOr(status, BQA_STATUS_SVD_NOT_CONVERGED);
    float nrm2 = 0.f;
#pragma unroll
    for (int i = 0; i < W; ++i) nrm2 += c_abs2(a[i]);
    const float sig = sqrtf(nrm2);
    const float sk = (lane < n && sig > eps) ? sig : 0.f;
    // descending rank among the segment's columns, ties by column index
    int rank = 0;
#pragma unroll
    for (int k = 0; k < W; ++k) {
        const float o = __shfl_sync(BQA_FULL_MASK, sk, k, W);
        rank += (o > sk) || (o == sk && k < lane);
    }
    const float norm = sqrtf(seg_sum<W>(sk * sk));
    if (live && lane < n) {
        lmbds[(size_t)pf * n + rank] = norm > 0.f ? sk / norm : 0.f;
        if (norm > 0.f) atomic_max_nonneg(colmax + rank, sk / norm);
    }
    const float uinv = sk > 0.f ? 1.f / sig : 0.f;
    // fwd canonicaliser column rank: ul[p] . (a / sigma) -> canon[p + half]
    __syncwarp();
    for (int i = lane; i < n * n; i += W) sm[i] = live ? ul[(size_t)pf * nn + i] : c_zero();
    __syncwarp();
    if (live && lane < n) {
        float2* out = canon + (size_t)pb * nn + rank;
        for (int i = 0; i < n; ++i) {
            float2 acc = c_zero();
#pragma unroll
            for (int k = 0; k < W; ++k)
                if (k < n) acc = c_fma(sm[i * n + k], a[k], acc);
            out[(size_t)i * n] = c_scale(acc, uinv);
        }
    }
    // bwd canonicaliser column rank: ul[p + half] . conj(v)  (vs = vhs^T) -> canon[p]
    __syncwarp();
    for (int i = lane; i < n * n; i += W) sm[i] = live ? ul[(size_t)pb * nn + i] : c_zero();
    __syncwarp();
    if (live && lane < n) {
        const float keep = sk > 0.f ? 1.f : 0.f;
        float2* out = canon + (size_t)pf * nn + rank;
        for (int i = 0; i < n; ++i) {
            float2 acc = c_zero();
#pragma unroll
            for (int k = 0; k < W; ++k)
                if (k < n) acc = c_fma(sm[i * n + k], c_conj(v[k]), acc);
            out[(size_t)i * n] = c_scale(acc, keep);
        }
    }
}

template <int W>
static int launch_env(const float2* m, int count, int n, float eps, float2* lu, float2* ul, int32_t* status,
                      cudaStream_t st) {
    const int per_block = 128 / W;
    const int blocks = (count + per_block - 1) / per_block;
    env_factor_kernel<W><<<blocks, 128, 0, st>>>(m, count, n, eps, lu, ul, status);
    return check_launch("env_factor");
}

template <int W>
static int launch_canon(const float2* lu, const float2* ul, int edges, int n, float eps, float2* canon,
                        float* lmbds, uint32_t* colmax, int32_t* status, cudaStream_t st) {
    const int per_block = 128 / W;
    const int half = edges / 2;
    const int blocks = (half + per_block - 1) / per_block;
    const size_t smem = (size_t)128 * W * sizeof(float2);
    int rc = ensure_smem((const void*)bond_canon_kernel<W>, smem, "bond_canon");
    if (rc) return rc;
    bond_canon_kernel<W><<<blocks, 128, smem, st>>>(lu, ul, edges, n, eps, canon, lmbds, colmax, status);
    return check_launch("bond_canon");
}

}  // namespace bqa

using namespace bqa;

extern "C" {

int32_t bqa_env_factor(const void* mats, int32_t count, int32_t n, float eps, void* lu, void* ul, int32_t* status,
                       void* stream) {
    if (!mats || !lu || !ul || !status || count < 0 || n < 1) return set_error(BQA_ERR_ARG, "bqa_env_factor: bad argument");
    if (count == 0) return BQA_OK;
    auto m = static_cast<const float2*>(mats);
    auto l = static_cast<float2*>(lu);
    auto u = static_cast<float2*>(ul);
    cudaStream_t st = as_stream(stream);
    if (n <= 8) return launch_env<8>(m, count, n, eps, l, u, status, st);
    if (n <= 16) return launch_env<16>(m, count, n, eps, l, u, status, st);
    if (n <= 32) return launch_env<32>(m, count, n, eps, l, u, status, st);
    return set_error(BQA_ERR_UNSUPPORTED, "bqa_env_factor: matrix size %d > 32", n);
}

int32_t bqa_bond_canon(const void* lu, const void* ul, int32_t edges, int32_t n, float eps, void* canon,
                       float* lmbds, uint32_t* colmax, int32_t* status, void* stream) {
    if (!lu || !ul || !canon || !lmbds || !colmax || !status || edges < 2 || n < 1)
        return set_error(BQA_ERR_ARG, "bqa_bond_canon: bad argument");
    auto l = static_cast<const float2*>(lu);
    auto u = static_cast<const float2*>(ul);
    auto c = static_cast<float2*>(canon);
    cudaStream_t st = as_stream(stream);
    if (n <= 8) return launch_canon<8>(l, u, edges, n, eps, c, lmbds, colmax, status, st);
    if (n <= 16) return launch_canon<16>(l, u, edges, n, eps, c, lmbds, colmax, status, st);
    if (n <= 32) return launch_canon<32>(l, u, edges, n, eps, c, lmbds, colmax, status, st);
    return set_error(BQA_ERR_UNSUPPORTED, "bqa_bond_canon: matrix size %d > 32", n);
}

}  // extern "C"
