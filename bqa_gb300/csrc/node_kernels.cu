// Node-contraction kernels: BP messages, extended (ZZ-gate) messages, phys-resolved
// open-bond blocks and per-node densities, plus the BP loop control kernels.
//
// One CTA owns one node.  Its tensor T[2][chi]^d and its d incoming messages are staged in
// shared memory; the other-bond messages are applied by mode products into two ping-pong
// shared buffers, and the closing contraction with conj(T) gives, for bond `idx`,
//     P_s[a][b] = sum_{other bonds} conj(T[s,..a..]) (T x_{k != idx} M_k)[s,..b..]
// for s = 0, 1.  Everything the reference computes per node and bond follows from P_s:
//   BP message (src/bqa/backends.py:393-408):      (P_0 + P_1) / tr
//   extended message (backends.py:396-404,519-526): block (e,f) = conj(a_e) a_f (P_0 + (-1)^(e+f) P_1) / tr
//   <Z_u Z_v> input (no reference counterpart):     P_0, P_1 themselves.
#include <cstdio>

#include "common.cuh"
#include "internal.h"

namespace bqa {

enum NodeMode { MODE_BP = 0, MODE_EXT = 1, MODE_PSPLIT = 2, MODE_DENS = 3 };

struct NodeArgs {
    const float2* tensors;   // [B][2][chi^d]
    const int32_t* in_pos;   // [B][d]
    const int32_t* out_pos;  // [B][d]
    const int32_t* node_ids; // [B]
    const double* edge_ampl; // [B][d]
    int d, chi;
    const float2* msgs_a;    // current messages (BP: buffer a)
    float2* msgs_b;          // BP: buffer b
    float2* out;             // EXT: [E][2chi][2chi]; PSPLIT: [E][2][chi][chi]; DENS: [n][2][2]
    const int32_t* loop_state;
    uint32_t* dist_parts;
    double ztime;
};

// Y[s][l][i][r] = sum_j M_s[i][j] X[s][l][j][r]; X is [2][L][nin][R], Y is [2][L][nout][R],
// M_s row-major nout x nin.  One thread owns one (s, l, r) fibre and keeps it in registers.
template <int CM>
__device__ __forceinline__ void mode_product(const float2* __restrict__ X, float2* __restrict__ Y,
                                             const float2* M0, const float2* M1,
                                             int L, int nin, int nout, int R) {
    const int per_s = L * R;
    for (int f = threadIdx.x; f < 2 * per_s; f += blockDim.x) {
        const int s = f >= per_s;
        const int g = f - s * per_s;
        const int l = g / R, r = g - l * R;
        const float2* xp = X + (size_t)(s * L + l) * nin * R + r;
        float2 x[CM];
#pragma unroll
        for (int j = 0; j < CM; ++j) x[j] = j < nin ? xp[(size_t)j * R] : c_zero();
        const float2* M = s ? M1 : M0;
        float2* yp = Y + (size_t)(s * L + l) * nout * R + r;
        for (int i = 0; i < nout; ++i) {
            const float2* mr = M + i * nin;
            float2 acc = c_zero();
#pragma unroll
            for (int j = 0; j < CM; ++j)
                if (j < nin) acc = c_fma(mr[j], x[j], acc);
            yp[(size_t)i * R] = acc;
        }
    }
}

// P[s][a][b] = sum_{l, r} conj(T[s][l][a][r]) X[s][l][b][r]; T, X are [2][L][n][R].
__device__ __forceinline__ void close_psplit(const float2* __restrict__ T, const float2* __restrict__ X,
                                             float2* __restrict__ P, int L, int n, int R) {
    const int n2 = n * n;
    const size_t per_s = (size_t)L * n * R;
    for (int o = threadIdx.x; o < 2 * n2; o += blockDim.x) {
        const int s = o >= n2;
        const int ab = o - s * n2;
        const int a = ab / n, b = ab - a * n;
        const float2* tp = T + s * per_s + (size_t)a * R;
        const float2* xp = X + s * per_s + (size_t)b * R;
        float2 acc = c_zero();
        for (int l = 0; l < L; ++l) {
            for (int r = 0; r < R; ++r) acc = c_fma_conj(tp[r], xp[r], acc);
            tp += (size_t)n * R;
            xp += (size_t)n * R;
        }
        P[o] = acc;
    }
}

__host__ __device__ inline size_t node_smem_floats2(int d, int chi) {
    const size_t NT = 2 * (size_t)ipow(chi, d);
    return 3 * NT + (size_t)(d + 4) * chi * chi + 128;  // + block_sum scratch (256 floats)
}

template <int CM, int MODE>
__global__ void __launch_bounds__(256) node_kernel(NodeArgs a) {
    extern __shared__ float4 smem_raw[];
    float2* sm = reinterpret_cast<float2*>(smem_raw);
    const int d = a.d, chi = a.chi, n2 = chi * chi;
    const int per_s = ipow(chi, d);
    const int NT = 2 * per_s;
    float2* sT = sm;
    float2* sA = sT + NT;
    float2* sB = sA + NT;
    float2* sM = sB + NT;
    float2* sP = sM + d * n2;
    float* sRed = reinterpret_cast<float*>(sP + 4 * n2);

    const float2* msgs_in = a.msgs_a;
    float2* msgs_out = a.msgs_b;
    if (MODE == MODE_BP && a.loop_state != nullptr) {
        if (a.loop_state[0]) return;                        // BP loop already done
        if (a.loop_state[2]) { msgs_in = a.msgs_b; msgs_out = const_cast<float2*>(a.msgs_a); }
    }

    const int node = blockIdx.x;
    const float2* Tg = a.tensors + (size_t)node * NT;
    for (int i = threadIdx.x; i < NT; i += blockDim.x) sT[i] = Tg[i];
    for (int k = 0; k < d; ++k) {
        const float2* mg = msgs_in + (size_t)a.in_pos[node * d + k] * n2;
        for (int i = threadIdx.x; i < n2; i += blockDim.x) sM[k * n2 + i] = mg[i];
    }
    __syncthreads();

    if (MODE == MODE_DENS) {
        // rho[s][s'] = sum_{bonds} (T x_all M)[s, ..] conj(T[s', ..])  (backends.py:440-448)
        const float2* cur = sT;
        for (int k = 0; k < d; ++k) {
            float2* nxt = (cur == sA) ? sB : sA;
            const float2* M = sM + k * n2;
            mode_product<CM>(cur, nxt, M, M, ipow(chi, k), chi, chi, ipow(chi, d - 1 - k));
            __syncthreads();
            cur = nxt;
        }
        float v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int o = threadIdx.x; o < per_s; o += blockDim.x) {
            const float2 x0 = cur[o], x1 = cur[per_s + o];
            const float2 t0 = sT[o], t1 = sT[per_s + o];
            float2 r00 = c_fma_conj(t0, x0, c_zero()), r01 = c_fma_conj(t1, x0, c_zero());
            float2 r10 = c_fma_conj(t0, x1, c_zero()), r11 = c_fma_conj(t1, x1, c_zero());
            v[0] += r00.x; v[1] += r00.y; v[2] += r01.x; v[3] += r01.y;
            v[4] += r10.x; v[5] += r10.y; v[6] += r11.x; v[7] += r11.y;
        }
        block_sum<8>(v, sRed);
        if (threadIdx.x < 4) {
            const float2 tr = make_float2(v[0] + v[6], v[1] + v[7]);
            const float2 r = make_float2(v[2 * threadIdx.x], v[2 * threadIdx.x + 1]);
            a.out[(size_t)a.node_ids[node] * 4 + threadIdx.x] = c_div(r, tr);
        }
        return;
    }

    float num2 = 0.f, den2 = 0.f;
    for (int idx = 0; idx < d; ++idx) {
        const float2* cur = sT;
        for (int k = 0; k < d; ++k) {
            if (k == idx) continue;
            float2* nxt = (cur == sA) ? sB : sA;
            const float2* M = sM + k * n2;
            mode_product<CM>(cur, nxt, M, M, ipow(chi, k), chi, chi, ipow(chi, d - 1 - k));
            __syncthreads();
            cur = nxt;
        }
        close_psplit(sT, cur, sP, ipow(chi, idx), chi, ipow(chi, d - 1 - idx));
        __syncthreads();

        const int slot = a.out_pos[node * d + idx];
        if (MODE == MODE_PSPLIT) {
            float2* og = a.out + (size_t)slot * 2 * n2;
            for (int i = threadIdx.x; i < 2 * n2; i += blockDim.x) og[i] = sP[i];
        } else {
            float2 tr = c_zero();
            for (int q = 0; q < chi; ++q) tr = c_add(tr, c_add(sP[q * chi + q], sP[n2 + q * chi + q]));
            if (MODE == MODE_BP) {
                const float2* old = msgs_in + (size_t)slot * n2;
                float2* og = msgs_out + (size_t)slot * n2;
                for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                    const float2 m = c_div(c_add(sP[i], sP[n2 + i]), tr);
                    const float2 o = old[i];
                    og[i] = m;
                    num2 = fmaxf(num2, c_abs2(c_sub(m, o)));
                    den2 = fmaxf(den2, c_abs2(c_add(m, o)));
                }
            } else {  // MODE_EXT
                const HalfZZ h = half_zz(a.edge_ampl[node * d + idx] * a.ztime);
                const float2 ae[2] = {h.a0, h.a1};
                const float scale = c_abs2(h.a0) + c_abs2(h.a1);
                const float2 trx = c_scale(tr, scale);
                const int n = 2 * chi;
                float2* og = a.out + (size_t)slot * n * n;
                for (int o = threadIdx.x; o < n * n; o += blockDim.x) {
                    const int row = o / n, col = o - row * n;
                    const int e = row >= chi, f = col >= chi;
                    const int ia = row - e * chi, ib = col - f * chi;
                    const float2 p0 = sP[ia * chi + ib], p1 = sP[n2 + ia * chi + ib];
                    const float2 pe = ((e + f) & 1) ? c_sub(p0, p1) : c_add(p0, p1);
                    const float2 coef = c_mul(c_conj(ae[e]), ae[f]);
                    og[o] = c_div(c_mul(coef, pe), trx);
                }
            }
        }
        __syncthreads();
    }
    if (MODE == MODE_BP) {
        num2 = block_max(num2, sRed);
        den2 = block_max(den2, sRed);
        if (threadIdx.x == 0) {
            atomic_max_nonneg(a.dist_parts, num2);
            atomic_max_nonneg(a.dist_parts + 1, den2);
        }
    }
}

template <int MODE>
static int launch_node_mode(const NodeArgs& args, int count, cudaStream_t st) {
    const int chi = args.chi, d = args.d;
    const size_t smem = node_smem_floats2(d, chi) * sizeof(float2);
    const int fib = 2 * ipow(chi, d > 0 ? d - 1 : 0);
    int threads = ((max(fib, 2 * chi * chi) + 31) / 32) * 32;
    threads = threads < 32 ? 32 : (threads > 256 ? 256 : threads);
    void (*kern)(NodeArgs) = nullptr;
    if (chi <= 1) kern = node_kernel<1, MODE>;
    else if (chi <= 2) kern = node_kernel<2, MODE>;
    else if (chi <= 4) kern = node_kernel<4, MODE>;
    else if (chi <= 8) kern = node_kernel<8, MODE>;
    else if (chi <= 16) kern = node_kernel<16, MODE>;
    else if (chi <= 32) kern = node_kernel<32, MODE>;
    else return set_error(BQA_ERR_UNSUPPORTED, "node kernel: bond dim %d > 32", chi);
    int rc = ensure_smem((const void*)kern, smem, "node kernel");
    if (rc) return rc;
    kern<<<count, threads, smem, st>>>(args);
    return check_launch("node kernel");
}

static int run_classes(int mode, const bqa_class* classes, int n_classes, int chi,
                       const void* msgs_a, void* msgs_b, void* out, uint32_t* dist_parts,
                       const int32_t* loop_state, double ztime, cudaStream_t st) {
    if (!classes || n_classes < 0 || chi < 1) return set_error(BQA_ERR_ARG, "bad class list or bond dim");
    for (int c = 0; c < n_classes; ++c) {
        const bqa_class& k = classes[c];
        if (k.count <= 0) continue;
        if (k.degree == 0 && mode != MODE_DENS) continue;
        if (node_smem_floats2(k.degree, chi) * sizeof(float2) > kMaxSmem)
            return set_error(BQA_ERR_UNSUPPORTED, "degree %d at bond dim %d does not fit shared memory",
                             k.degree, chi);
        NodeArgs a;
        a.tensors = static_cast<const float2*>(k.tensor);
        a.in_pos = k.in_pos;
        a.out_pos = k.out_pos;
        a.node_ids = k.node_ids;
        a.edge_ampl = k.edge_ampl;
        a.d = k.degree;
        a.chi = chi;
        a.msgs_a = static_cast<const float2*>(msgs_a);
        a.msgs_b = static_cast<float2*>(msgs_b);
        a.out = static_cast<float2*>(out);
        a.loop_state = loop_state;
        a.dist_parts = dist_parts;
        a.ztime = ztime;
        int rc = BQA_OK;
        switch (mode) {
            case MODE_BP: rc = launch_node_mode<MODE_BP>(a, k.count, st); break;
            case MODE_EXT: rc = launch_node_mode<MODE_EXT>(a, k.count, st); break;
            case MODE_PSPLIT: rc = launch_node_mode<MODE_PSPLIT>(a, k.count, st); break;
            default: rc = launch_node_mode<MODE_DENS>(a, k.count, st); break;
        }
        if (rc) return rc;
    }
    return BQA_OK;
}

// ---- BP loop control -------------------------------------------------------------------------

__global__ void bp_decide_kernel(uint32_t* parts, int32_t* ls, float eps, float damping, int max_iters) {
    ls[4] = 0;
    if (ls[0]) return;
    const float num = sqrtf(__uint_as_float(parts[0]));
    const float den = sqrtf(__uint_as_float(parts[1]));
    parts[0] = 0u;
    parts[1] = 0u;
    const float dist = num / den;
    const int sweeps = ls[1] + 1;
    ls[1] = sweeps;
    ls[5] = __float_as_int(dist);
    const float best = sweeps == 1 ? dist : fminf(__int_as_float(ls[6]), dist);
    ls[6] = __float_as_int(best);
    if (dist < eps) { ls[0] = 1; return; }                  // keep the sweep's input
    if (sweeps >= max_iters) { ls[0] = 1; ls[3] = 1; ls[2] ^= 1; return; }  // raw last output
    if (damping == 0.f) ls[2] ^= 1;
    else ls[4] = 1;
}

__global__ void bp_damp_kernel(float2* a, float2* b, int64_t n, const int32_t* ls, float damping) {
    if (!ls[4]) return;
    float2* cur = ls[2] ? b : a;
    const float2* nw = ls[2] ? a : b;
    const float keep = damping, take = 1.0f - damping;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 x = cur[i], y = nw[i];
        cur[i] = make_float2(fmaf(take, y.x, keep * x.x), fmaf(take, y.y, keep * x.y));
    }
}

// msgs[e] = diag(lam[e % half][0..dim)) / sum(lam)   (src/bqa/state.py:56-57)
__global__ void msgs_from_lmbds_kernel(const float* lam, int stride, int E, int dim, float2* msgs) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= E) return;
    const float* l = lam + (size_t)(warp % (E / 2)) * stride;
    float s = 0.f;
    for (int i = lane; i < dim; i += 32) s += l[i];
    s = warp_sum(s);
    const float inv = 1.0f / s;
    float2* m = msgs + (size_t)warp * dim * dim;
    for (int o = lane; o < dim * dim; o += 32) {
        const int i = o / dim, j = o - i * dim;
        m[o] = make_float2(i == j ? l[i] * inv : 0.f, 0.f);
    }
}

// <Z_u Z_v> = Re( sum Z^u Z^v / sum S^u S^v ), S = P0 + P1, Z = P0 - P1 (oracle edge_zz)
__global__ void edge_zz_kernel(const float2* pm, int E, int chi, double* zz) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int half = E / 2;
    if (warp >= half) return;
    const int n2 = chi * chi;
    const float2* pu = pm + (size_t)warp * 2 * n2;
    const float2* pv = pm + (size_t)(warp + half) * 2 * n2;
    double nr = 0, ni = 0, dr = 0, di = 0;
    for (int i = lane; i < n2; i += 32) {
        const float2 u0 = pu[i], u1 = pu[n2 + i], v0 = pv[i], v1 = pv[n2 + i];
        const float2 zu = c_sub(u0, u1), zv = c_sub(v0, v1), su = c_add(u0, u1), sv = c_add(v0, v1);
        nr += (double)zu.x * zv.x - (double)zu.y * zv.y;
        ni += (double)zu.x * zv.y + (double)zu.y * zv.x;
        dr += (double)su.x * sv.x - (double)su.y * sv.y;
        di += (double)su.x * sv.y + (double)su.y * sv.x;
    }
    nr = warp_sum_d(nr); ni = warp_sum_d(ni); dr = warp_sum_d(dr); di = warp_sum_d(di);
    if (lane == 0) zz[warp] = (nr * dr + ni * di) / (dr * dr + di * di);
}

}  // namespace bqa

using namespace bqa;

extern "C" {

int32_t bqa_max_bond_dim(int32_t degree) {
    if (degree < 0) return 0;
    int best = 0;
    // message kernels: shared-memory staging; simple update: Jacobi SVD of 2chi x 2chi <= 32
    for (int chi = 1; chi <= 16; ++chi)
        if (node_smem_floats2(degree, chi) * sizeof(float2) <= kMaxSmem) best = chi;
    return best;
}

int32_t bqa_bp_sweep(const bqa_class* classes, int32_t n_classes, int32_t chi, void* msgs_a, void* msgs_b,
                     uint32_t* dist_parts, const int32_t* loop_state, void* stream) {
    if (!msgs_a || !msgs_b || !dist_parts) return set_error(BQA_ERR_ARG, "bqa_bp_sweep: null buffer");
    return run_classes(MODE_BP, classes, n_classes, chi, msgs_a, msgs_b, nullptr, dist_parts, loop_state, 0.0,
                       as_stream(stream));
}

int32_t bqa_bp_finalize(void* msgs_a, void* msgs_b, int64_t msg_elems, uint32_t* dist_parts, int32_t* loop_state,
                        float eps, float damping, int32_t max_iters, void* stream) {
    if (!msgs_a || !msgs_b || !dist_parts || !loop_state || msg_elems < 0 || max_iters < 1)
        return set_error(BQA_ERR_ARG, "bqa_bp_finalize: bad argument");
    cudaStream_t st = as_stream(stream);
    bp_decide_kernel<<<1, 1, 0, st>>>(dist_parts, loop_state, eps, damping, max_iters);
    int rc = check_launch("bp_decide");
    if (rc || damping == 0.f || msg_elems == 0) return rc;
    int blocks = (int)((msg_elems + 255) / 256);
    blocks = blocks > 4 * 152 * 8 ? 4 * 152 * 8 : blocks;
    bp_damp_kernel<<<blocks, 256, 0, st>>>(static_cast<float2*>(msgs_a), static_cast<float2*>(msgs_b), msg_elems,
                                           loop_state, damping);
    return check_launch("bp_damp");
}

int32_t bqa_ext_msgs(const bqa_class* classes, int32_t n_classes, int32_t chi, const void* msgs, void* ext_out,
                     double ztime, void* stream) {
    if (!msgs || !ext_out) return set_error(BQA_ERR_ARG, "bqa_ext_msgs: null buffer");
    return run_classes(MODE_EXT, classes, n_classes, chi, msgs, nullptr, ext_out, nullptr, nullptr, ztime,
                       as_stream(stream));
}

int32_t bqa_psplit(const bqa_class* classes, int32_t n_classes, int32_t chi, const void* msgs, void* pm,
                   void* stream) {
    if (!msgs || !pm) return set_error(BQA_ERR_ARG, "bqa_psplit: null buffer");
    return run_classes(MODE_PSPLIT, classes, n_classes, chi, msgs, nullptr, pm, nullptr, nullptr, 0.0,
                       as_stream(stream));
}

int32_t bqa_densities(const bqa_class* classes, int32_t n_classes, int32_t chi, const void* msgs, void* rho,
                      void* stream) {
    if (!msgs || !rho) return set_error(BQA_ERR_ARG, "bqa_densities: null buffer");
    return run_classes(MODE_DENS, classes, n_classes, chi, msgs, nullptr, rho, nullptr, nullptr, 0.0,
                       as_stream(stream));
}

int32_t bqa_msgs_from_lmbds(const float* lmbds, int32_t lam_stride, int32_t edges, int32_t dim, void* msgs,
                            void* stream) {
    if (!lmbds || !msgs || edges < 2 || dim < 1 || lam_stride < dim)
        return set_error(BQA_ERR_ARG, "bqa_msgs_from_lmbds: bad argument");
    const int blocks = (int)(((int64_t)edges * 32 + 255) / 256);
    msgs_from_lmbds_kernel<<<blocks, 256, 0, as_stream(stream)>>>(lmbds, lam_stride, edges, dim,
                                                                   static_cast<float2*>(msgs));
    return check_launch("msgs_from_lmbds");
}

int32_t bqa_edge_zz(const void* pm, int32_t edges, int32_t chi, double* zz, void* stream) {
    if (!pm || !zz || edges < 2 || chi < 1) return set_error(BQA_ERR_ARG, "bqa_edge_zz: bad argument");
    const int blocks = (int)(((int64_t)(edges / 2) * 32 + 255) / 256);
    edge_zz_kernel<<<blocks, 256, 0, as_stream(stream)>>>(static_cast<const float2*>(pm), edges, chi, zz);
    return check_launch("edge_zz");
}

}  // extern "C"
