// Tensor update of one annealing step, fused per node (one CTA per node):
//
//   T'[s, c_0..c_{d-1}] = N * Rx( z_s * sum_j T[s, j_0..j_{d-1}] prod_k W_k^s[j_k, c_k] )
//   W_k^s[j, c] = (a0_k C_k[j, c] + (-1)^s a1_k C_k[chi + j, c]) * sqrt(lambda_k[c])
//
// C_k is the canonicaliser of bond k (first `dim` columns of canon[in_pos[k]]), a0_k, a1_k
// the half-ZZ-gate coefficients of the edge (J_k ztime), z_s = cos(h ztime) -+ i sin(h ztime)
// the Rz gate, Rx mixes s with cos(xtime), -i sin(xtime), and N the per-node L2 normalisation.
// This is, in one pass, the reference's
//   apply_canonicalizers_with_extensions   src/bqa/backends.py:416-432 (state.py:237-246)
//   _apply_z_layer / _apply_x_layer         src/bqa/state.py:142-156, backends.py:506-510
//   _set_to_symmetric_gauge (tensor part)   src/bqa/state.py:219-227, backends.py:450-462
// (all factors are diagonal in s except Rx, which is applied after the bond products).
#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "tiled_node.cuh"
#include "tiled_d3c16.cuh"

namespace bqa {

template <typename R>
struct ApplyArgs {
    using C = typename Cx<R>::T;
    const C* t_in;           // [B][2][chi^d]
    C* t_out;                // [B][2][dim^d]
    const int32_t* in_pos;
    const int32_t* lmbd_pos;
    const double* edge_ampl;
    const double* node_ampl;
    const C* canon;          // [E][n][n], n = 2 chi
    const R* lmbds;          // [E/2][lam_stride]
    int lam_stride;
    int d, chi, dim;
    double ztime;
    R cx, sx;                // cos(xtime), sin(xtime)
};

// Y[s][l][c][r] = sum_j W_s[c][j] X[s][l][j][r]  (same fibre scheme as the message kernels)
template <int CM, typename C>
__device__ __forceinline__ void bond_product(const C* __restrict__ X, C* __restrict__ Y, const C* W0, const C* W1,
                                             int L, int nin, int nout, int Rr) {
    const int per_s = L * Rr;
    for (int f = threadIdx.x; f < 2 * per_s; f += blockDim.x) {
        const int s = f >= per_s;
        const int g = f - s * per_s;
        const int l = g / Rr, r = g - l * Rr;
        const C* xp = X + (size_t)(s * L + l) * nin * Rr + r;
        C x[CM];
#pragma unroll
        for (int j = 0; j < CM; ++j) x[j] = j < nin ? xp[(size_t)j * Rr] : c_zero<C>();
        const C* W = s ? W1 : W0;
        C* yp = Y + (size_t)(s * L + l) * nout * Rr + r;
        for (int c = 0; c < nout; ++c) {
            const C* wr = W + c * nin;
            C acc = c_zero<C>();
#pragma unroll
            for (int j = 0; j < CM; ++j)
                if (j < nin) acc = c_fma(wr[j], x[j], acc);
            yp[(size_t)c * Rr] = acc;
        }
    }
}

// X, Y, the bond matrices, the block reduction's scratch (64), the node's half-ZZ
// coefficients and Rz phase (2d + 1)
__host__ __device__ inline size_t apply_smem_elems(int d, int chi, int dim) {
    const int m = chi > dim ? chi : dim;
    return 2 * (2 * (size_t)ipow(m, d)) + (size_t)d * 2 * dim * chi + 64 + 2 * (size_t)d + 1;
}

// warp 0 evaluates the node's d half-ZZ coefficient pairs and its Rz phase in double precision,
// one lane each, into sC (2d + 1 complex); the caller synchronises before reading them
template <typename R>
__device__ __forceinline__ void node_coefficients(const ApplyArgs<R>& a, int node, typename Cx<R>::T* sC) {
    const int d = a.d;
    if ((int)threadIdx.x < d) {
        const HalfZZ<R> h = half_zz<R>(a.edge_ampl[node * d + threadIdx.x] * a.ztime);
        sC[2 * threadIdx.x] = h.a0;
        sC[2 * threadIdx.x + 1] = h.a1;
    } else if ((int)threadIdx.x == d) {
        double sz, cz;
        sincos(a.node_ampl[node] * a.ztime, &sz, &cz);
        sC[2 * d] = c_make((R)cz, (R)sz);
    }
}

template <int CM, typename R>
__global__ void __launch_bounds__(256) apply_kernel(ApplyArgs<R> a) {
    using C = typename Cx<R>::T;
    extern __shared__ double4_32a smem_raw[];
    C* sm = reinterpret_cast<C*>(smem_raw);
    const int d = a.d, chi = a.chi, dim = a.dim, n = 2 * chi;
    const int m = chi > dim ? chi : dim;
    const size_t buf = 2 * (size_t)ipow(m, d);
    C* sX = sm;
    C* sY = sX + buf;
    C* sW = sY + buf;
    R* sRed = reinterpret_cast<R*>(sW + (size_t)d * 2 * dim * chi);
    C* sC = sW + (size_t)d * 2 * dim * chi + 64;

    const int node = blockIdx.x;
    const int nin = 2 * ipow(chi, d);
    const C* tg = a.t_in + (size_t)node * nin;
    for (int i = threadIdx.x; i < nin; i += blockDim.x) sX[i] = tg[i];
    node_coefficients<R>(a, node, sC);
    __syncthreads();
    for (int k = 0; k < d; ++k) {
        HalfZZ<R> h;
        h.a0 = sC[2 * k];
        h.a1 = sC[2 * k + 1];
        const C* Cc = a.canon + (size_t)a.in_pos[node * d + k] * n * n;
        const R* lam = a.lmbds + (size_t)a.lmbd_pos[node * d + k] * a.lam_stride;
        for (int o = threadIdx.x; o < 2 * dim * chi; o += blockDim.x) {
            const int s = o / (dim * chi);
            const int cj = o - s * dim * chi;
            const int c = cj / chi, j = cj - c * chi;
            const C up = c_mul(h.a0, Cc[(size_t)j * n + c]);
            const C dn = c_mul(h.a1, Cc[(size_t)(chi + j) * n + c]);
            const C w = s ? c_sub(up, dn) : c_add(up, dn);
            sW[(size_t)k * 2 * dim * chi + o] = c_scale(w, sqrt(lam[c]));
        }
    }
    __syncthreads();

    C* cur = sX;
    C* nxt = sY;
    for (int k = 0; k < d; ++k) {
        const C* W0 = sW + (size_t)k * 2 * dim * chi;
        bond_product<CM>(cur, nxt, W0, W0 + dim * chi, ipow(dim, k), chi, dim, ipow(chi, d - 1 - k));
        __syncthreads();
        C* t = cur; cur = nxt; nxt = t;
    }

    // Rz, Rx, norm
    const C z1 = sC[2 * d], z0 = c_conj(z1);
    const int per_s = ipow(dim, d);
    R acc[1] = {0};
    for (int o = threadIdx.x; o < per_s; o += blockDim.x) {
        const C y0 = c_mul(z0, cur[o]), y1 = c_mul(z1, cur[per_s + o]);
        // cos(x) y - i sin(x) X y
        const C t0 = c_make(a.cx * y0.x + a.sx * y1.y, a.cx * y0.y - a.sx * y1.x);
        const C t1 = c_make(a.cx * y1.x + a.sx * y0.y, a.cx * y1.y - a.sx * y0.x);
        cur[o] = t0;
        cur[per_s + o] = t1;
        acc[0] += c_abs2(t0) + c_abs2(t1);
    }
    block_sum<1>(acc, sRed);
    const R inv = R(1) / sqrt(acc[0]);
    C* og = a.t_out + (size_t)node * 2 * per_s;
    for (int o = threadIdx.x; o < 2 * per_s; o += blockDim.x) og[o] = c_scale(cur[o], inv);
}


size_t apply_smem_bytes(int d, int chi, size_t elem_bytes) { return apply_smem_elems(d, chi, chi) * elem_bytes; }

// Node tensors beyond shared memory: the same update with X and Y in a per-CTA slice of
// caller scratch (2 x 2 m^d complex, m = max(chi, dim)); the bond matrices W stay in shared
// memory.  Each CTA walks nodes blockIdx.x, blockIdx.x + gridDim.x, ...
template <int CM, typename R>
__global__ void __launch_bounds__(256) apply_kernel_global(ApplyArgs<R> a, int count, typename Cx<R>::T* scratch) {
    using C = typename Cx<R>::T;
    extern __shared__ double4_32a smem_raw[];
    C* sW = reinterpret_cast<C*>(smem_raw);
    const int d = a.d, chi = a.chi, dim = a.dim, n = 2 * chi;
    const int m = chi > dim ? chi : dim;
    const size_t buf = 2 * (size_t)ipow(m, d);
    R* sRed = reinterpret_cast<R*>(sW + (size_t)d * 2 * dim * chi);
    C* sC = sW + (size_t)d * 2 * dim * chi + 64;
    C* X0 = scratch + (size_t)blockIdx.x * 2 * buf;
    C* Y0 = X0 + buf;
    const int nin = 2 * ipow(chi, d);
    const int per_s = ipow(dim, d);
    for (int node = blockIdx.x; node < count; node += gridDim.x) {
        const C* tg = a.t_in + (size_t)node * nin;
        for (int i = threadIdx.x; i < nin; i += blockDim.x) X0[i] = tg[i];
        node_coefficients<R>(a, node, sC);
        __syncthreads();
        for (int k = 0; k < d; ++k) {
            HalfZZ<R> h;
            h.a0 = sC[2 * k];
            h.a1 = sC[2 * k + 1];
            const C* Cc = a.canon + (size_t)a.in_pos[node * d + k] * n * n;
            const R* lam = a.lmbds + (size_t)a.lmbd_pos[node * d + k] * a.lam_stride;
            for (int o = threadIdx.x; o < 2 * dim * chi; o += blockDim.x) {
                const int s = o / (dim * chi);
                const int cj = o - s * dim * chi;
                const int c = cj / chi, j = cj - c * chi;
                const C up = c_mul(h.a0, Cc[(size_t)j * n + c]);
                const C dn = c_mul(h.a1, Cc[(size_t)(chi + j) * n + c]);
                const C w = s ? c_sub(up, dn) : c_add(up, dn);
                sW[(size_t)k * 2 * dim * chi + o] = c_scale(w, sqrt(lam[c]));
            }
        }
        __syncthreads();
        C* cur = X0;
        C* nxt = Y0;
        for (int k = 0; k < d; ++k) {
            const C* W0 = sW + (size_t)k * 2 * dim * chi;
            bond_product<CM>(cur, nxt, W0, W0 + dim * chi, ipow(dim, k), chi, dim, ipow(chi, d - 1 - k));
            __syncthreads();
            C* t = cur; cur = nxt; nxt = t;
        }
        const C z1 = sC[2 * d], z0 = c_conj(z1);
        R acc[1] = {0};
        for (int o = threadIdx.x; o < per_s; o += blockDim.x) {
            const C y0 = c_mul(z0, cur[o]), y1 = c_mul(z1, cur[per_s + o]);
            const C t0 = c_make(a.cx * y0.x + a.sx * y1.y, a.cx * y0.y - a.sx * y1.x);
            const C t1 = c_make(a.cx * y1.x + a.sx * y0.y, a.cx * y1.y - a.sx * y0.x);
            cur[o] = t0;
            cur[per_s + o] = t1;
            acc[0] += c_abs2(t0) + c_abs2(t1);
        }
        block_sum<1>(acc, sRed);
        const R inv = R(1) / sqrt(acc[0]);
        C* og = a.t_out + (size_t)node * 2 * per_s;
        for (int o = threadIdx.x; o < 2 * per_s; o += blockDim.x) og[o] = c_scale(cur[o], inv);
        __syncthreads();
    }
}

// ---- register-tiled update for dim == chi, complex64 ------------------------------------------
// CTA (node, s) stages T_s and the three s-specific bond matrices W_k^s (with sqrt(lambda) and,
// on bond 0, the Rz phase z_s folded in), runs the d bond products with the tiled GEMM of the
// message kernels and writes z_s-weighted Y_s to tensor_out; apply_rx_norm_kernel then mixes the
// two halves (Rx) and normalises each node.
template <int D, int CHI, bool SPEC_IN>
__global__ void __launch_bounds__(tiled::HalfShape<D, CHI>::THREADS) tiled_apply_half_kernel(ApplyArgs<float> a) {
    using S = tiled::HalfShape<D, CHI>;
    constexpr bool SPEC = SPEC_IN && D == 3 && CHI == 16;
    constexpr int PS = S::PER_S, N2 = S::N2, TH = S::THREADS, SW = S::SW, n = 2 * CHI;
    extern __shared__ double4_32a smem_raw[];
    float2* sX = reinterpret_cast<float2*>(smem_raw);
    float2* sY = sX + PS;
    float2* sW = sY + PS;           // D blocks of [j][c], CHI x CHI
    float2* sC = sW + D * N2;       // half-ZZ coefficients a0, a1 of each bond, then (cos, sin) of Rz
    const int node = blockIdx.x >> 1, s = blockIdx.x & 1;
    {
        const float4* tg = reinterpret_cast<const float4*>(a.t_in + (size_t)node * 2 * PS + (size_t)s * PS);
        for (int i = threadIdx.x; i < PS / 2; i += TH)
            *reinterpret_cast<float4*>(sX + tiled::swz<SW>(2 * i)) = tg[i];
    }
    // the node's D + 1 double-precision trig evaluations, one lane each (one FP64 stream per CTA)
    if (threadIdx.x < D) {
        const HalfZZ<float> h = half_zz<float>(a.edge_ampl[node * D + threadIdx.x] * a.ztime);
        sC[2 * threadIdx.x] = h.a0;
        sC[2 * threadIdx.x + 1] = h.a1;
    } else if (threadIdx.x == D) {
        double sz, cz;
        sincos(a.node_ampl[node] * a.ztime, &sz, &cz);
        sC[2 * D] = make_float2((float)cz, (float)sz);
    }
    __syncthreads();
    const float2 zs = make_float2(sC[2 * D].x, s ? sC[2 * D].y : -sC[2 * D].y);
#pragma unroll
    for (int k = 0; k < D; ++k) {
        HalfZZ<float> h;
        h.a0 = sC[2 * k];
        h.a1 = sC[2 * k + 1];
        const float2* Cc = a.canon + (size_t)a.in_pos[node * D + k] * n * n;
        const float* lam = a.lmbds + (size_t)a.lmbd_pos[node * D + k] * a.lam_stride;
        for (int o = threadIdx.x; o < N2; o += TH) {
            const int j = o / CHI, c = o - j * CHI;
            const float2 up = c_mul(h.a0, Cc[(size_t)j * n + c]);
            const float2 dn = c_mul(h.a1, Cc[(size_t)(CHI + j) * n + c]);
            float2 w = c_scale(s ? c_sub(up, dn) : c_add(up, dn), sqrtf(lam[c]));
            if (k == 0) w = c_mul(zs, w);
            sW[k * N2 + o] = w;
        }
    }
    __syncthreads();
    float2* cur = sX;
    if constexpr (SPEC) {
        // the bond products with the closed-form addresses of the (3, 16) message kernel (the
        // same operations in the same order as tiled::product): bond 0 in place, then 1 and 2
        namespace q = tiled::d3c16;
        q::prod0_inplace(sX, sW);
        __syncthreads();
        q::prod1(sX, sY, sW + N2);
        __syncthreads();
        q::prod2(sY, sX, sW + 2 * N2);
        __syncthreads();
    } else {
        float2* nxt = sY;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            tiled::product<D, CHI, TH, SW, 1>(cur, nxt, sW + k * N2, k);
            __syncthreads();
            float2* t = cur; cur = nxt; nxt = t;
        }
    }
    float4* og = reinterpret_cast<float4*>(a.t_out + (size_t)node * 2 * PS + (size_t)s * PS);
    for (int i = threadIdx.x; i < PS / 2; i += TH) og[i] = *reinterpret_cast<const float4*>(cur + tiled::swz<SW>(2 * i));
}

// T[0] <- cos(x) T[0] - i sin(x) T[1], T[1] <- cos(x) T[1] - i sin(x) T[0], then T /= |T| per node.
__global__ void __launch_bounds__(256) apply_rx_norm_kernel(float2* t, int per_s, float cx, float sx) {
    __shared__ float sRed[32];
    float2* tn = t + (size_t)blockIdx.x * 2 * per_s;
    float acc[1] = {0.f};
    for (int o = threadIdx.x; o < per_s; o += blockDim.x) {
        const float2 y0 = tn[o], y1 = tn[per_s + o];
        const float2 t0 = make_float2(cx * y0.x + sx * y1.y, cx * y0.y - sx * y1.x);
        const float2 t1 = make_float2(cx * y1.x + sx * y0.y, cx * y1.y - sx * y0.x);
        tn[o] = t0;
        tn[per_s + o] = t1;
        acc[0] += c_abs2(t0) + c_abs2(t1);
    }
    block_sum<1>(acc, sRed);
    const float inv = 1.f / sqrtf(acc[0]);
    for (int o = threadIdx.x; o < 2 * per_s; o += blockDim.x) tn[o] = c_scale(tn[o], inv);
}

// BQA_GB300_SPECIALIZED=0 at library load keeps the (3, 16) update on the generic addresses
// too (the two give bit-identical tensors)
static const bool g_apply_specialized = [] {
    const char* v = getenv("BQA_GB300_SPECIALIZED");
    return !(v && v[0] == '0');
}();

template <int D, int CHI>
static int launch_apply_half(const ApplyArgs<float>& a, int count, cudaStream_t st) {
    using S = tiled::HalfShape<D, CHI>;
    const size_t smem = ((size_t)2 * S::PER_S + (size_t)D * S::N2 + 2 * D + 2) * sizeof(float2);
    void (*kern)(ApplyArgs<float>) = tiled_apply_half_kernel<D, CHI, false>;
    if constexpr (D == 3 && CHI == 16)
        if (g_apply_specialized) kern = tiled_apply_half_kernel<D, CHI, true>;
    int rc = ensure_smem((const void*)kern, smem, "tiled apply");
    if (rc) return rc;
    kern<<<2 * count, S::THREADS, smem, st>>>(a);
    rc = check_launch("tiled apply");
    if (rc) return rc;
    apply_rx_norm_kernel<<<count, 256, 0, st>>>(a.t_out, S::PER_S, a.cx, a.sx);
    return check_launch("apply rx norm");
}

// 1 if a tiled update covers (degree, chi == dim) and was launched
static int try_tiled_apply(const ApplyArgs<float>& a, int count, cudaStream_t st, int* rc) {
    if (a.dim != a.chi) return 0;
    const int d = a.d, chi = a.chi;
#define BQA_TAPPLY(DD, CC) \
    if (d == DD && chi == CC) { *rc = launch_apply_half<DD, CC>(a, count, st); return 1; }
    BQA_TAPPLY(2, 8) BQA_TAPPLY(2, 12) BQA_TAPPLY(2, 16)
    BQA_TAPPLY(3, 4) BQA_TAPPLY(3, 8) BQA_TAPPLY(3, 12) BQA_TAPPLY(3, 16)
    BQA_TAPPLY(4, 4) BQA_TAPPLY(4, 8)
#undef BQA_TAPPLY
    return 0;
}

template <typename R>
static int apply_classes(const bqa_class* classes, int n_classes, int chi, int dim, const void* canon,
                         const void* lmbds, int lam_stride, double ztime, double xtime, cudaStream_t st) {
    using C = typename Cx<R>::T;
    const int cm = chi > dim ? chi : dim;
    for (int c = 0; c < n_classes; ++c) {
        const bqa_class& k = classes[c];
        if (k.count <= 0) continue;
        const size_t smem = apply_smem_elems(k.degree, chi, dim) * sizeof(C);
        const bool global = smem > kMaxSmem;
        ApplyArgs<R> a;
        a.t_in = static_cast<const C*>(k.tensor);
        a.t_out = static_cast<C*>(k.tensor_out);
        a.in_pos = k.in_pos;
        a.lmbd_pos = k.lmbd_pos;
        a.edge_ampl = k.edge_ampl;
        a.node_ampl = k.node_ampl;
        a.canon = static_cast<const C*>(canon);
        a.lmbds = static_cast<const R*>(lmbds);
        a.lam_stride = lam_stride;
        a.d = k.degree;
        a.chi = chi;
        a.dim = dim;
        a.ztime = ztime;
        a.cx = (R)cos(xtime);
        a.sx = (R)sin(xtime);
        if (global) {
            const int64_t need = 4 * (int64_t)ipow(cm, k.degree);
            if (!k.scratch || k.scratch_elems < need)
                return set_error(BQA_ERR_UNSUPPORTED,
                                 "apply: degree %d at bond dim %d->%d exceeds shared memory and the class has %lld "
                                 "of the %lld scratch elements a CTA needs (bqa_node_scratch_elems)",
                                 k.degree, chi, dim, (long long)k.scratch_elems, (long long)need);
            const int64_t ctas = std::min<int64_t>((int64_t)k.count, k.scratch_elems / need);
            const size_t gsmem = ((size_t)k.degree * 2 * dim * chi + 64 + 2 * (size_t)k.degree + 1) * sizeof(C);
            void (*gk)(ApplyArgs<R>, int, C*) = nullptr;
            if (chi <= 4) gk = apply_kernel_global<4, R>;
            else if (chi <= 8) gk = apply_kernel_global<8, R>;
            else if (chi <= 16) gk = apply_kernel_global<16, R>;
            else if (chi <= 32) gk = apply_kernel_global<32, R>;
            else return set_error(BQA_ERR_UNSUPPORTED, "apply: bond dim %d > 32", chi);
            int rc = ensure_smem((const void*)gk, gsmem, "apply (global)");
            if (rc) return rc;
            gk<<<(int)ctas, 256, gsmem, st>>>(a, k.count, static_cast<C*>(k.scratch));
            rc = check_launch("apply (global)");
            if (rc) return rc;
            continue;
        }
        if constexpr (sizeof(R) == 4) {
            int trc = BQA_OK;
            if (k.degree >= 2 && try_tiled_apply(a, k.count, st, &trc)) {
                if (trc) return trc;
                continue;
            }
        }
        const int fib = 2 * ipow(cm, k.degree > 0 ? k.degree - 1 : 0);
        int threads = ((fib + 31) / 32) * 32;
        threads = threads < 64 ? 64 : (threads > 256 ? 256 : threads);
        void (*kern)(ApplyArgs<R>) = nullptr;
        if (chi <= 1) kern = apply_kernel<1, R>;
        else if (chi <= 2) kern = apply_kernel<2, R>;
        else if (chi <= 4) kern = apply_kernel<4, R>;
        else if (chi <= 8) kern = apply_kernel<8, R>;
        else if (chi <= 16) kern = apply_kernel<16, R>;
        else if (chi <= 32) kern = apply_kernel<32, R>;
        else return set_error(BQA_ERR_UNSUPPORTED, "apply: bond dim %d > 32", chi);
        int rc = ensure_smem((const void*)kern, smem, "apply");
        if (rc) return rc;
        kern<<<k.count, threads, smem, st>>>(a);
        rc = check_launch("apply");
        if (rc) return rc;
    }
    return BQA_OK;
}

}  // namespace bqa

using namespace bqa;

extern "C" {

int32_t bqa_apply_update(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dim, int32_t dtype,
                         const void* canon, const void* lmbds, int32_t lam_stride, double ztime, double xtime,
                         void* stream) {
    if (!classes || n_classes < 0 || chi < 1 || dim < 1 || !canon || !lmbds || lam_stride < dim)
        return set_error(BQA_ERR_ARG, "bqa_apply_update: bad argument");
    if (dim > 2 * chi) return set_error(BQA_ERR_ARG, "bqa_apply_update: dim %d > 2*chi", dim);
    cudaStream_t st = as_stream(stream);
    if (dtype == BQA_C64)
        return apply_classes<float>(classes, n_classes, chi, dim, canon, lmbds, lam_stride, ztime, xtime, st);
    if (dtype == BQA_C128)
        return apply_classes<double>(classes, n_classes, chi, dim, canon, lmbds, lam_stride, ztime, xtime, st);
    return set_error(BQA_ERR_ARG, "bqa_apply_update: unknown dtype %d", dtype);
}

}  // extern "C"
