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
#include "common.cuh"
#include "internal.h"

namespace bqa {

struct ApplyArgs {
    const float2* t_in;      // [B][2][chi^d]
    float2* t_out;           // [B][2][dim^d]
    const int32_t* in_pos;
    const int32_t* lmbd_pos;
    const double* edge_ampl;
    const double* node_ampl;
    const float2* canon;     // [E][n][n], n = 2 chi
    const float* lmbds;      // [E/2][lam_stride]
    int lam_stride;
    int d, chi, dim;
    double ztime;
    float cx, sx;            // cos(xtime), sin(xtime)
};

// Y[s][l][c][r] = sum_j W_s[c][j] X[s][l][j][r]  (same fibre scheme as the message kernels)
template <int CM>
__device__ __forceinline__ void bond_product(const float2* __restrict__ X, float2* __restrict__ Y,
                                             const float2* W0, const float2* W1, int L, int nin, int nout, int R) {
    const int per_s = L * R;
    for (int f = threadIdx.x; f < 2 * per_s; f += blockDim.x) {
        const int s = f >= per_s;
        const int g = f - s * per_s;
        const int l = g / R, r = g - l * R;
        const float2* xp = X + (size_t)(s * L + l) * nin * R + r;
        float2 x[CM];
#pragma unroll
        for (int j = 0; j < CM; ++j) x[j] = j < nin ? xp[(size_t)j * R] : c_zero();
        const float2* W = s ? W1 : W0;
        float2* yp = Y + (size_t)(s * L + l) * nout * R + r;
        for (int c = 0; c < nout; ++c) {
            const float2* wr = W + c * nin;
            float2 acc = c_zero();
#pragma unroll
            for (int j = 0; j < CM; ++j)
                if (j < nin) acc = c_fma(wr[j], x[j], acc);
            yp[(size_t)c * R] = acc;
        }
    }
}

__host__ __device__ inline size_t apply_smem_floats2(int d, int chi, int dim) {
    const int m = chi > dim ? chi : dim;
    return 2 * (2 * (size_t)ipow(m, d)) + (size_t)d * 2 * dim * chi + 128;
}

template <int CM>
__global__ void __launch_bounds__(256) apply_kernel(ApplyArgs a) {
    extern __shared__ float4 smem_raw[];
    float2* sm = reinterpret_cast<float2*>(smem_raw);
    const int d = a.d, chi = a.chi, dim = a.dim, n = 2 * chi;
    const int m = chi > dim ? chi : dim;
    const size_t buf = 2 * (size_t)ipow(m, d);
    float2* sX = sm;
    float2* sY = sX + buf;
    float2* sW = sY + buf;
    float* sRed = reinterpret_cast<float*>(sW + (size_t)d * 2 * dim * chi);

    const int node = blockIdx.x;
    const int nin = 2 * ipow(chi, d);
    const float2* tg = a.t_in + (size_t)node * nin;
    for (int i = threadIdx.x; i < nin; i += blockDim.x) sX[i] = tg[i];
    for (int k = 0; k < d; ++k) {
        const HalfZZ h = half_zz(a.edge_ampl[node * d + k] * a.ztime);
        const float2* C = a.canon + (size_t)a.in_pos[node * d + k] * n * n;
        const float* lam = a.lmbds + (size_t)a.lmbd_pos[node * d + k] * a.lam_stride;
        for (int o = threadIdx.x; o < 2 * dim * chi; o += blockDim.x) {
            const int s = o / (dim * chi);
            const int cj = o - s * dim * chi;
            const int c = cj / chi, j = cj - c * chi;
            const float2 up = c_mul(h.a0, C[(size_t)j * n + c]);
            const float2 dn = c_mul(h.a1, C[(size_t)(chi + j) * n + c]);
            const float2 w = s ? c_sub(up, dn) : c_add(up, dn);
            sW[(size_t)k * 2 * dim * chi + o] = c_scale(w, sqrtf(lam[c]));
        }
    }
    __syncthreads();

    float2* cur = sX;
    float2* nxt = sY;
    for (int k = 0; k < d; ++k) {
        const float2* W0 = sW + (size_t)k * 2 * dim * chi;
        bond_product<CM>(cur, nxt, W0, W0 + dim * chi, ipow(dim, k), chi, dim, ipow(chi, d - 1 - k));
        __syncthreads();
        float2* t = cur; cur = nxt; nxt = t;
    }

    // Rz, Rx, norm
    double sz, cz;
    sincos(a.node_ampl[node] * a.ztime, &sz, &cz);
    const float2 z0 = make_float2((float)cz, (float)-sz), z1 = make_float2((float)cz, (float)sz);
    const int per_s = ipow(dim, d);
    float acc[1] = {0.f};
    for (int o = threadIdx.x; o < per_s; o += blockDim.x) {
        const float2 y0 = c_mul(z0, cur[o]), y1 = c_mul(z1, cur[per_s + o]);
        // cos(x) y - i sin(x) X y
        const float2 t0 = make_float2(a.cx * y0.x + a.sx * y1.y, a.cx * y0.y - a.sx * y1.x);
        const float2 t1 = make_float2(a.cx * y1.x + a.sx * y0.y, a.cx * y1.y - a.sx * y0.x);
        cur[o] = t0;
        cur[per_s + o] = t1;
        acc[0] += c_abs2(t0) + c_abs2(t1);
    }
    block_sum<1>(acc, sRed);
    const float inv = rsqrtf(acc[0]);
    float2* og = a.t_out + (size_t)node * 2 * per_s;
    for (int o = threadIdx.x; o < 2 * per_s; o += blockDim.x) og[o] = c_scale(cur[o], inv);
}

}  // namespace bqa

using namespace bqa;

extern "C" {

int32_t bqa_apply_update(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dim, const void* canon,
                         const float* lmbds, int32_t lam_stride, double ztime, double xtime, void* stream) {
    if (!classes || n_classes < 0 || chi < 1 || dim < 1 || !canon || !lmbds || lam_stride < dim)
        return set_error(BQA_ERR_ARG, "bqa_apply_update: bad argument");
    if (dim > 2 * chi) return set_error(BQA_ERR_ARG, "bqa_apply_update: dim %d > 2*chi", dim);
    cudaStream_t st = as_stream(stream);
    const int cm = chi > dim ? chi : dim;
    for (int c = 0; c < n_classes; ++c) {
        const bqa_class& k = classes[c];
        if (k.count <= 0) continue;
        const size_t smem = apply_smem_floats2(k.degree, chi, dim) * sizeof(float2);
        if (smem > kMaxSmem)
            return set_error(BQA_ERR_UNSUPPORTED, "apply: degree %d at bond dim %d->%d does not fit shared memory",
                             k.degree, chi, dim);
        ApplyArgs a;
        a.t_in = static_cast<const float2*>(k.tensor);
        a.t_out = static_cast<float2*>(k.tensor_out);
        a.in_pos = k.in_pos;
        a.lmbd_pos = k.lmbd_pos;
        a.edge_ampl = k.edge_ampl;
        a.node_ampl = k.node_ampl;
        a.canon = static_cast<const float2*>(canon);
        a.lmbds = lmbds;
        a.lam_stride = lam_stride;
        a.d = k.degree;
        a.chi = chi;
        a.dim = dim;
        a.ztime = ztime;
        a.cx = (float)cos(xtime);
        a.sx = (float)sin(xtime);
        const int fib = 2 * ipow(cm, k.degree > 0 ? k.degree - 1 : 0);
        int threads = ((fib + 31) / 32) * 32;
        threads = threads < 64 ? 64 : (threads > 256 ? 256 : threads);
        void (*kern)(ApplyArgs) = nullptr;
        if (chi <= 1) kern = apply_kernel<1>;
        else if (chi <= 2) kern = apply_kernel<2>;
        else if (chi <= 4) kern = apply_kernel<4>;
        else if (chi <= 8) kern = apply_kernel<8>;
        else if (chi <= 16) kern = apply_kernel<16>;
        else if (chi <= 32) kern = apply_kernel<32>;
        else return set_error(BQA_ERR_UNSUPPORTED, "apply: bond dim %d > 32", chi);
        int rc = ensure_smem((const void*)kern, smem, "apply");
        if (rc) return rc;
        kern<<<k.count, threads, smem, st>>>(a);
        rc = check_launch("apply");
        if (rc) return rc;
    }
    return BQA_OK;
}

}  // extern "C"
