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
// All kernels are templated on the real type R: float (complex64 path) or double
// (complex128 path, the reference's BQA_PRECISION=double arithmetic).
#include <cstdlib>
#include <cstring>
#include <new>

#include "common.cuh"
#include "internal.h"
#include "tiled_node.cuh"
#include "tiled_d3c16.cuh"
#include "tc_d3c16.cuh"
#include "tc_bf16_d3c16.cuh"
#include "tc_f16x2_d3c16.cuh"

#include <algorithm>
#include <vector>
#include <type_traits>

namespace bqa {

enum NodeMode { MODE_BP = 0, MODE_EXT = 1, MODE_PSPLIT = 2, MODE_DENS = 3 };

// The register-tiled kernels serve the (degree, chi) pairs they are built for unless the
// environment variable BQA_GB300_TILED=0 is set when the library loads (then every launch
// takes the generic kernel, which tests use to cross-check the two).
static const bool g_use_tiled = [] {
    const char* v = getenv("BQA_GB300_TILED");
    return !(v && v[0] == '0');
}();
// Likewise BQA_GB300_SPECIALIZED=0 keeps the (3, 16) half-node kernel on the generic address
// arithmetic (the two give bit-identical results).
static const bool g_use_specialized = [] {
    const char* v = getenv("BQA_GB300_SPECIALIZED");
    return !(v && v[0] == '0');
}();
// The default (3, 16) half-node kernel is the FP32-accurate tensor-core kernel (2xFP16 bond
// products and closing contractions, tc_f16x2_d3c16.cuh); BQA_GB300_TC=0 set when the library
// loads makes it the CUDA-core kernel.
static const bool g_use_tc = [] {
    const char* v = getenv("BQA_GB300_TC");
    return !(v && v[0] == '0');
}();

// CTAs of the tensor-core kernels whose wait for their MMAs timed out (bqa_tc_faults).
__device__ int32_t g_tc_faults;

template <typename R>
struct NodeArgs {
    using C = typename Cx<R>::T;
    const C* tensors;        // [B][2][chi^d]
    const int32_t* in_pos;   // [B][d]
    const int32_t* out_pos;  // [B][d]
    const int32_t* node_ids; // [B]
    const double* edge_ampl; // [B][d]
    int d, chi;
    const C* msgs_a;         // current messages (BP: buffer a)
    C* msgs_b;               // BP: buffer b
    C* out;                  // EXT: [E][2chi][2chi]; PSPLIT: [E][2][chi][chi]; DENS: [n][2][2]
    const int32_t* loop_state;
    typename Cx<R>::Bits* dist_parts;
    double ztime;
    // mixed-precision BP: 0 = always run; 1 = run only on low-precision sweeps, 2 = only on the
    // others (low_precision_sweep); the two kernels of a mixed sweep share the decision
    int mixed_role = 0;
    float mixed_switch = 0.f;
};

// A sweep of a BP run is a low-precision (BF16) sweep when it is not the run's first and the
// distance of the previous sweep (loop_state[5], float bits) is above the switch.
__device__ __forceinline__ bool low_precision_sweep(const int32_t* ls, float switch_dist) {
    return ls != nullptr && ls[1] >= 1 && __int_as_float(ls[5]) > switch_dist;
}

// ---- packed sweeps (internal.h) ---------------------------------------------------------------

static thread_local PackList* g_pack = nullptr;

void pack_collect(PackList* list) { g_pack = list; }

void PackList::push(const PackEntry& e) {
    if (n == cap) {
        const int nc = cap ? 2 * cap : 64;
        PackEntry* grown = new (std::nothrow) PackEntry[nc];
        if (!grown) {
            error = set_error(BQA_ERR_ARG, "packed sweep: out of host memory");
            return;
        }
        for (int i = 0; i < n; ++i) grown[i] = items[i];
        delete[] items;
        items = grown;
        cap = nc;
    }
    items[n++] = e;
}

// While a PackList collects on this thread, record the launch (launcher, phase, key, nodes,
// arguments) and return true: the caller then returns without launching.
template <typename A>
static bool pack_record(int (*fn)(const PackEntry*, int, cudaStream_t), int phase, int key, int count, const A& args) {
    static_assert(sizeof(A) <= sizeof(PackEntry::args) && std::is_trivially_copyable<A>::value,
                  "packed launch arguments must be a small trivially copyable block");
    if (!g_pack) return false;
    PackEntry e;
    e.launch = fn;
    e.phase = phase;
    e.key = key;
    e.count = count;
    std::memcpy(e.args, &args, sizeof(A));
    g_pack->push(e);
    return true;
}

int pack_execute(const PackList& l, cudaStream_t st) {
    if (l.error) return l.error;
    std::vector<char> issued(l.n, 0);
    std::vector<PackEntry> group;
    for (int phase = 0; phase < 4; ++phase)
        for (int i = 0; i < l.n; ++i) {
            const PackEntry& head = l.items[i];
            if (issued[i] || head.phase != phase) continue;
            group.clear();
            for (int k = i; k < l.n; ++k) {
                const PackEntry& x = l.items[k];
                if (!issued[k] && x.phase == phase && x.launch == head.launch && x.key == head.key) {
                    group.push_back(x);
                    issued[k] = 1;
                }
            }
            const int rc = head.launch(group.data(), (int)group.size(), st);
            if (rc) return rc;
        }
    return BQA_OK;
}

// Y[s][l][i][r] = sum_j M_s[i][j] X[s][l][j][r]; X is [2][L][nin][R], Y is [2][L][nout][R],
// M_s row-major nout x nin.  One thread owns one (s, l, r) fibre and keeps it in registers.
template <int CM, typename C>
__device__ __forceinline__ void mode_product(const C* __restrict__ X, C* __restrict__ Y, const C* M0, const C* M1,
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
        const C* M = s ? M1 : M0;
        C* yp = Y + (size_t)(s * L + l) * nout * Rr + r;
        for (int i = 0; i < nout; ++i) {
            const C* mr = M + i * nin;
            C acc = c_zero<C>();
#pragma unroll
            for (int j = 0; j < CM; ++j)
                if (j < nin) acc = c_fma(mr[j], x[j], acc);
            yp[(size_t)i * Rr] = acc;
        }
    }
}

// Parts of a closing contraction's sum over L * R = chi^(d-1) terms: up to 256 (output, part)
// items, at least 16 terms per part.  A function of the shape only, so a node's outputs do
// not depend on the CTA size.
__host__ __device__ inline int close_parts(int d, int chi) {
    const int outs = 2 * chi * chi;
    const int terms = ipow(chi, d > 0 ? d - 1 : 0);
    int g = 256 / outs;
    if (g > terms / 16) g = terms / 16;
    return g < 1 ? 1 : g;
}

// P[s][a][b] = sum_{l, r} conj(T[s][l][a][r]) X[s][l][b][r]; T, X are [2][L][n][R].  With G > 1
// parts, item (g, o) sums the g-th contiguous chunk of the (l, r) terms of output o into
// scratch[g][o] (G * 2 n^2 elements), and the parts are then added in the order g = 0..G-1.
template <typename C>
__device__ __forceinline__ void close_psplit(const C* __restrict__ T, const C* __restrict__ X, C* __restrict__ P,
                                             int L, int n, int Rr, C* __restrict__ scratch, int G) {
    const int n2 = n * n;
    const size_t per_s = (size_t)L * n * Rr;
    if (G == 1) {
        for (int o = threadIdx.x; o < 2 * n2; o += blockDim.x) {
            const int s = o >= n2;
            const int ab = o - s * n2;
            const int a = ab / n, b = ab - a * n;
            const C* tp = T + s * per_s + (size_t)a * Rr;
            const C* xp = X + s * per_s + (size_t)b * Rr;
            C acc = c_zero<C>();
            for (int l = 0; l < L; ++l) {
                for (int r = 0; r < Rr; ++r) acc = c_fma_conj(tp[r], xp[r], acc);
                tp += (size_t)n * Rr;
                xp += (size_t)n * Rr;
            }
            P[o] = acc;
        }
        return;
    }
    const int terms = L * Rr, chunk = (terms + G - 1) / G;
    for (int w = threadIdx.x; w < 2 * n2 * G; w += blockDim.x) {
        const int g = w / (2 * n2), o = w - g * 2 * n2;
        const int s = o >= n2;
        const int ab = o - s * n2;
        const int a = ab / n, b = ab - a * n;
        const int t0 = g * chunk, t1 = min(terms, t0 + chunk);
        int l = t0 / Rr, r = t0 - l * Rr;
        const C* tp = T + s * per_s + (size_t)a * Rr;
        const C* xp = X + s * per_s + (size_t)b * Rr;
        C acc = c_zero<C>();
        for (int t = t0; t < t1; ++t) {
            const size_t off = (size_t)l * n * Rr + r;
            acc = c_fma_conj(tp[off], xp[off], acc);
            if (++r == Rr) { r = 0; ++l; }
        }
        scratch[w] = acc;
    }
    __syncthreads();
    for (int o = threadIdx.x; o < 2 * n2; o += blockDim.x) {
        C acc = scratch[o];
        for (int g = 1; g < G; ++g) acc = c_add(acc, scratch[g * 2 * n2 + o]);
        P[o] = acc;
    }
}

// shared memory of the node kernel, in complex elements
__host__ __device__ inline size_t node_smem_elems(int d, int chi) {
    const size_t NT = 2 * (size_t)ipow(chi, d);
    return 3 * NT + (size_t)(d + 4) * chi * chi + 128;  // + block-reduction scratch
}

// Outputs of one (node, bond idx) from its open-bond blocks sP = [P_0; P_1]: the BP message
// (plus the dist maxima), the extended message, or the blocks themselves.
template <int MODE, typename R>
__device__ __forceinline__ void write_outputs(const NodeArgs<R>& a, int node, int idx, const typename Cx<R>::T* sP,
                                              const typename Cx<R>::T* msgs_in, typename Cx<R>::T* msgs_out,
                                              R& num2, R& den2) {
    using C = typename Cx<R>::T;
    const int d = a.d, chi = a.chi, n2 = chi * chi;
    const int slot = a.out_pos[node * d + idx];
    if (MODE == MODE_PSPLIT) {
        C* og = a.out + (size_t)slot * 2 * n2;
        for (int i = threadIdx.x; i < 2 * n2; i += blockDim.x) og[i] = sP[i];
    } else {
        C tr = c_zero<C>();
        for (int q = 0; q < chi; ++q) tr = c_add(tr, c_add(sP[q * chi + q], sP[n2 + q * chi + q]));
        if (MODE == MODE_BP) {
            const C* old = msgs_in + (size_t)slot * n2;
            C* og = msgs_out + (size_t)slot * n2;
            for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                const C m = c_div(c_add(sP[i], sP[n2 + i]), tr);
                const C o = old[i];
                og[i] = m;
                num2 = fmax(num2, c_abs2(c_sub(m, o)));
                den2 = fmax(den2, c_abs2(c_add(m, o)));
            }
        } else {  // MODE_EXT
            const HalfZZ<R> h = half_zz_warp<R>(a.edge_ampl[node * d + idx] * a.ztime);
            const R scale = c_abs2(h.a0) + c_abs2(h.a1);
            const C trx = c_scale(tr, scale);
            const int n = 2 * chi;
            C* og = a.out + (size_t)slot * n * n;
            for (int o = threadIdx.x; o < n * n; o += blockDim.x) {
                const int row = o / n, col = o - row * n;
                const int e = row >= chi, f = col >= chi;
                const int ia = row - e * chi, ib = col - f * chi;
                const C p0 = sP[ia * chi + ib], p1 = sP[n2 + ia * chi + ib];
                const C pe = ((e + f) & 1) ? c_sub(p0, p1) : c_add(p0, p1);
                const C coef = c_mul(c_conj(e ? h.a1 : h.a0), f ? h.a1 : h.a0);
                og[o] = c_div(c_mul(coef, pe), trx);
            }
        }
    }
}

template <int CM, int MODE, typename R>
__device__ __forceinline__ void node_body(const NodeArgs<R>& a, int node) {
    using C = typename Cx<R>::T;
    extern __shared__ double4_32a smem_raw[];
    C* sm = reinterpret_cast<C*>(smem_raw);
    const int d = a.d, chi = a.chi, n2 = chi * chi;
    const int per_s = ipow(chi, d);
    const int NT = 2 * per_s;
    C* sT = sm;
    C* sA = sT + NT;
    C* sB = sA + NT;
    C* sM = sB + NT;
    C* sP = sM + d * n2;
    R* sRed = reinterpret_cast<R*>(sP + 4 * n2);

    const C* msgs_in = a.msgs_a;
    C* msgs_out = a.msgs_b;
    if ((MODE == MODE_BP || MODE == MODE_PSPLIT) && a.loop_state != nullptr) {
        if (a.loop_state[0]) return;                        // BP loop already done
        if (a.loop_state[2]) { msgs_in = a.msgs_b; msgs_out = const_cast<C*>(a.msgs_a); }
    }

    const C* Tg = a.tensors + (size_t)node * NT;
    if (MODE == MODE_DENS)
        for (int i = threadIdx.x; i < NT; i += blockDim.x) sT[i] = Tg[i];
    for (int k = 0; k < d; ++k) {
        const C* mg = msgs_in + (size_t)a.in_pos[node * d + k] * n2;
        for (int i = threadIdx.x; i < n2; i += blockDim.x) sM[k * n2 + i] = mg[i];
    }
    __syncthreads();

    if (MODE == MODE_DENS) {
        // rho[s][s'] = sum_{bonds} (T x_all M)[s, ..] conj(T[s', ..])  (backends.py:440-448)
        const C* cur = sT;
        for (int k = 0; k < d; ++k) {
            C* nxt = (cur == sA) ? sB : sA;
            const C* M = sM + k * n2;
            mode_product<CM>(cur, nxt, M, M, ipow(chi, k), chi, chi, ipow(chi, d - 1 - k));
            __syncthreads();
            cur = nxt;
        }
        R v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int o = threadIdx.x; o < per_s; o += blockDim.x) {
            const C x0 = cur[o], x1 = cur[per_s + o];
            const C t0 = sT[o], t1 = sT[per_s + o];
            const C r00 = c_fma_conj(t0, x0, c_zero<C>()), r01 = c_fma_conj(t1, x0, c_zero<C>());
            const C r10 = c_fma_conj(t0, x1, c_zero<C>()), r11 = c_fma_conj(t1, x1, c_zero<C>());
            v[0] += r00.x; v[1] += r00.y; v[2] += r01.x; v[3] += r01.y;
            v[4] += r10.x; v[5] += r10.y; v[6] += r11.x; v[7] += r11.y;
        }
        block_sum<8>(v, sRed);
        if (threadIdx.x < 4) {
            const C tr = c_make(v[0] + v[6], v[1] + v[7]);
            const C r = c_make(v[2 * threadIdx.x], v[2 * threadIdx.x + 1]);
            a.out[(size_t)a.node_ids[node] * 4 + threadIdx.x] = c_div(r, tr);
        }
        return;
    }

    // BP messages, extended messages, open-bond blocks.  Messages are Hermitian, so the block of
    // bond idx is the closing contraction <T x_(A - idx) | T x_B> for idx in A = [0, h) and
    // <T x_A | T x_(B - idx)> for idx in B = [h, d), h = d / 2 (the pairing of the global-memory
    // kernel): |A|^2 + |B|^2 bond products per node instead of d (d - 1), 18 instead of 30 at
    // degree 6.  Every product chain starts from T in global memory (the node's tensor stays in
    // L2 while its CTA works on it); T x_B, later T x_A, is kept in sK (the buffer the densities
    // use for T), the other side's chains run in sA / sB.
    C* sK = sT;
    // T x_k M_k for k in [k0, k1) except skip, the last product written to `last` and the ones
    // before alternating with `other`; T itself (global memory) when the set is empty
    auto chain = [&](int k0, int k1, int skip, C* last, C* other) -> const C* {
        int np = 0;
        for (int k = k0; k < k1; ++k) np += (k != skip);
        const C* cur = Tg;
        int i = 0;
        for (int k = k0; k < k1; ++k) {
            if (k == skip) continue;
            C* nxt = ((np - 1 - i) & 1) ? other : last;
            const C* M = sM + k * n2;
            mode_product<CM>(cur, nxt, M, M, ipow(chi, k), chi, chi, ipow(chi, d - 1 - k));
            __syncthreads();
            cur = nxt;
            ++i;
        }
        return cur;
    };
    const int h = d / 2, G = close_parts(d, chi);
    R num2 = 0, den2 = 0;
    const C* K = h > 0 ? chain(h, d, -1, sK, sA) : Tg;                  // T x_B
    for (int idx = 0; idx < h; ++idx) {
        const C* Y = chain(0, h, idx, sA, sB);                          // T x_(A - idx)
        close_psplit(Y, K, sP, ipow(chi, idx), chi, ipow(chi, d - 1 - idx), sB, G);
        __syncthreads();
        write_outputs<MODE, R>(a, node, idx, sP, msgs_in, msgs_out, num2, den2);
        __syncthreads();
    }
    K = chain(0, h, -1, sK, sA);                                        // T x_A
    for (int idx = h; idx < d; ++idx) {
        const C* Y = chain(h, d, idx, sA, sB);                          // T x_(B - idx)
        close_psplit(K, Y, sP, ipow(chi, idx), chi, ipow(chi, d - 1 - idx), sB, G);
        __syncthreads();
        write_outputs<MODE, R>(a, node, idx, sP, msgs_in, msgs_out, num2, den2);
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

// The generic kernel takes one or several classes (of one job or of several) per launch: CTA b
// belongs to class c with first[c] <= b < first[c + 1] (first counts CTAs).  Shared memory and
// threads are the largest any of the launch's classes needs; each CTA lays out its class's
// buffers in it.  The register-tiled half-node kernels have the same form for packed sweeps.
constexpr int kMaxMergedClasses = 32;   // 32 x 104-byte argument blocks: under 4 KB of parameters
template <typename R>
struct MergedClasses {
    NodeArgs<R> cls[kMaxMergedClasses];
    int first[kMaxMergedClasses + 1];
    int n;
};

// the class of this CTA: the last c with first[c] <= blockIdx.x (classes are never empty)
__device__ __forceinline__ int merged_class(const int* first, int n) {
    int lo = 0, hi = n - 1;
    const int b = (int)blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int CM, int MODE, typename R>
__global__ void __launch_bounds__(256) node_kernel_merged(const __grid_constant__ MergedClasses<R> m) {
    const int c = merged_class(m.first, m.n);
    node_body<CM, MODE, R>(m.cls[c], (int)blockIdx.x - m.first[c]);
}

// The same kernel built for CTAs of up to 1024 threads (BP and open-bond modes, bond dims
// <= 8): for nodes whose shared memory allows one or two CTAs per SM, more warps per node
// hide more latency.  A node's outputs do not depend on the CTA size (every output is formed
// by one thread in a fixed order; the BP maxima are order-free).
template <int CM, int MODE, typename R>
__global__ void __launch_bounds__(1024) node_kernel_merged_wide(const __grid_constant__ MergedClasses<R> m) {
    const int c = merged_class(m.first, m.n);
    node_body<CM, MODE, R>(m.cls[c], (int)blockIdx.x - m.first[c]);
}


// ---- node tensors beyond shared memory --------------------------------------------------------
//
// The same contractions with two work tensors per CTA in a slice of caller scratch (global
// memory); T is read in place from the class buffer; messages, open-bond blocks and the
// closing contraction's staging stay in shared memory.  Each CTA walks nodes blockIdx.x,
// blockIdx.x + gridDim.x, ...  Work tensors are T with a set of messages applied, the
// products running in place: a thread reads its whole fibre into registers before it writes
// it, and fibres are disjoint.

// X[s][l][i][r] <- sum_j M[i][j] X[s][l][j][r] (n x n message, in place)
template <int CM, typename C>
__device__ __forceinline__ void mode_product_inplace(C* X, const C* M, int L, int n, int Rr) {
    const int per_s = L * Rr;
    for (int f = threadIdx.x; f < 2 * per_s; f += blockDim.x) {
        const int s = f >= per_s;
        const int g = f - s * per_s;
        const int l = g / Rr, r = g - l * Rr;
        C* xp = X + (size_t)(s * L + l) * n * Rr + r;
        C x[CM];
#pragma unroll
        for (int j = 0; j < CM; ++j) x[j] = j < n ? xp[(size_t)j * Rr] : c_zero<C>();
        for (int i = 0; i < n; ++i) {
            const C* mr = M + i * n;
            C acc = c_zero<C>();
#pragma unroll
            for (int j = 0; j < CM; ++j)
                if (j < n) acc = c_fma(mr[j], x[j], acc);
            xp[(size_t)i * Rr] = acc;
        }
    }
}

// P[s][a][b] = sum_{l, r} conj(X[s][l][a][r]) Y[s][l][b][r] with X, Y in global memory.  Chunks
// of KC positions k = (l, r) are staged in shared memory (each element read from global memory
// once; rows padded to NP = n rounded up to 4, zero beyond n); thread (s, 4x4 tile of (a, b),
// K-slice sl) accumulates its tile over the slice (8 shared loads per 16 complex FMAs); the
// slices meet in `red` (4096 complex elements).
constexpr int kCloseRed = 4096;
// positions per staged chunk: 64, or 32 above bond dim 16 (keeps complex128 at chi 32 within
// shared memory)
__host__ __device__ inline int close_kc(int n) { return n <= 16 ? 64 : 32; }

template <typename C>
__device__ __forceinline__ void close_global(const C* __restrict__ X, const C* __restrict__ Y, C* __restrict__ P,
                                             C* __restrict__ stage, C* __restrict__ red, int L, int n, int Rr) {
    const int KC = close_kc(n), KP = KC + 1;
    const int K = L * Rr;
    const int NPd = (n + 3) & ~3;
    const int ntile = NPd / 4;
    const int tiles = 2 * ntile * ntile;
    const int SL = (int)blockDim.x / tiles;            // >= 1 for n <= 16 and 256 threads
    const int t = threadIdx.x;
    const int tile = t / SL, sl = t - tile * SL;
    const bool active = tile < tiles;
    const int s = active ? tile / (ntile * ntile) : 0;
    const int ag = active ? (tile / ntile) % ntile : 0, bg = active ? tile % ntile : 0;
    const size_t per_s = (size_t)L * n * Rr;
    C* Xs = stage;                                     // [2][NPd][KP]
    C* Ys = stage + 2 * NPd * KP;
    C acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = c_zero<C>();
    for (int k0 = 0; k0 < K; k0 += KC) {
        const int kc = min(KC, K - k0);
        for (int e = t; e < 2 * NPd * KC; e += blockDim.x) {
            const int sa = e / KC, kk = e - sa * KC;
            const int ss = sa / NPd, aa = sa - ss * NPd;
            C xv = c_zero<C>(), yv = c_zero<C>();
            if (aa < n && kk < kc) {
                const int k = k0 + kk, l = k / Rr, r = k - l * Rr;
                const size_t src = ss * per_s + ((size_t)l * n + aa) * Rr + r;
                xv = X[src];
                yv = Y[src];
            }
            Xs[sa * KP + kk] = xv;
            Ys[sa * KP + kk] = yv;
        }
        __syncthreads();
        if (active) {
            const C* xr = Xs + (s * NPd + ag * 4) * KP;
            const C* yr = Ys + (s * NPd + bg * 4) * KP;
            for (int kk = sl; kk < kc; kk += SL) {
                C xv[4], yv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) xv[u] = xr[u * KP + kk];
#pragma unroll
                for (int v = 0; v < 4; ++v) yv[v] = yr[v * KP + kk];
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int v = 0; v < 4; ++v) acc[u][v] = c_fma_conj(xv[u], yv[v], acc[u][v]);
            }
        }
        __syncthreads();
    }
    // slice partials: red[sl][tile][16]
    if (active) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) red[((size_t)sl * tiles + tile) * 16 + u * 4 + v] = acc[u][v];
    }
    __syncthreads();
    const int n2 = n * n;
    for (int o = t; o < 2 * n2; o += blockDim.x) {
        const int os = o / n2, ab = o - os * n2, a = ab / n, b = ab - a * n;
        const int tl = (os * ntile + a / 4) * ntile + b / 4, q = (a & 3) * 4 + (b & 3);
        C sum = c_zero<C>();
        for (int z = 0; z < SL; ++z) sum = c_add(sum, red[((size_t)z * tiles + tl) * 16 + q]);
        P[o] = sum;
    }
}

// shared memory of the global kernel: messages, P, the close's staging and slice partials, the
// block reductions' scratch (block_sum<8>: 8 x 32 reals fit 128 complex elements)
// (+ d message pointers); messages themselves are read from global memory (L1/L2)
__host__ __device__ inline size_t node_global_smem_elems(int d, int chi, int threads) {
    (void)threads;
    const int n2 = chi * chi;
    const int NPd = (chi + 3) & ~3;
    return 2 * (size_t)n2 + 4 * (size_t)NPd * (close_kc(chi) + 1) + kCloseRed + 128 + (size_t)d;
}

// T x_k M_k for k in [k0, k1) except `skip`, into W: the first product reads T and writes W,
// the others run in place (a plain copy when the set is empty)
template <int CM, typename C>
__device__ __forceinline__ void apply_messages(const C* __restrict__ T, C* W, const C* const* mp, int d, int chi,
                                               size_t NT, int k0, int k1, int skip) {
    bool first = true;
    for (int k = k0; k < k1; ++k) {
        if (k == skip) continue;
        const C* M = mp[k];
        if (first) mode_product<CM>(T, W, M, M, ipow(chi, k), chi, chi, ipow(chi, d - 1 - k));
        else mode_product_inplace<CM>(W, M, ipow(chi, k), chi, ipow(chi, d - 1 - k));
        first = false;
        __syncthreads();
    }
    if (first) {
        for (size_t i = threadIdx.x; i < NT; i += blockDim.x) W[i] = T[i];
        __syncthreads();
    }
}

// Bonds split in A = [0, h) and B = [h, d), h = d / 2.  Messages are Hermitian, so the message
// of bond idx is the closing contraction <T x_(A or B minus idx) | T x_(the other set)>: for
// idx in A, Wa = T x_(A \ idx) against Wb = T x_B (formed once); for idx in B, Wa = T x_A
// (formed once) against Wb = T x_(B \ idx).  |A|^2 + |B|^2 products instead of d (d - 1).
template <int CM, int MODE, typename R>
__global__ void __launch_bounds__(256) node_kernel_global(NodeArgs<R> a, int count, typename Cx<R>::T* scratch) {
    using C = typename Cx<R>::T;
    extern __shared__ double4_32a smem_raw[];
    C* sm = reinterpret_cast<C*>(smem_raw);
    const int d = a.d, chi = a.chi, n2 = chi * chi;
    const int per_s = ipow(chi, d);
    const size_t NT = 2 * (size_t)per_s;
    const int NPd = (chi + 3) & ~3;
    C* sP = sm;
    C* stage = sP + 2 * n2;
    C* red = stage + 4 * (size_t)NPd * (close_kc(chi) + 1);
    R* sRed = reinterpret_cast<R*>(red + kCloseRed);
    const C** mp = reinterpret_cast<const C**>(red + kCloseRed + 128);   // d message pointers
    C* Wa = scratch + (size_t)blockIdx.x * 2 * NT;
    C* Wb = Wa + NT;
    const int h = d / 2;

    const C* msgs_in = a.msgs_a;
    C* msgs_out = a.msgs_b;
    if ((MODE == MODE_BP || MODE == MODE_PSPLIT) && a.loop_state != nullptr) {
        if (a.loop_state[0]) return;
        if (a.loop_state[2]) { msgs_in = a.msgs_b; msgs_out = const_cast<C*>(a.msgs_a); }
    }
    R num2 = 0, den2 = 0;
    for (int node = blockIdx.x; node < count; node += gridDim.x) {
        const C* T = a.tensors + (size_t)node * NT;
        for (int k = threadIdx.x; k < d; k += blockDim.x) mp[k] = msgs_in + (size_t)a.in_pos[node * d + k] * n2;
        __syncthreads();
        if (MODE == MODE_DENS) {
            // rho[s][s'] = sum (T x_all M)[s, ..] conj(T[s', ..]) = sum (T x_B)[s, ..] conj((T x_A)[s', ..])
            apply_messages<CM>(T, Wa, mp, d, chi, NT, 0, h, -1);
            apply_messages<CM>(T, Wb, mp, d, chi, NT, h, d, -1);
            R v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int o = threadIdx.x; o < per_s; o += blockDim.x) {
                const C x0 = Wb[o], x1 = Wb[per_s + o];
                const C t0 = Wa[o], t1 = Wa[per_s + o];
                const C r00 = c_fma_conj(t0, x0, c_zero<C>()), r01 = c_fma_conj(t1, x0, c_zero<C>());
                const C r10 = c_fma_conj(t0, x1, c_zero<C>()), r11 = c_fma_conj(t1, x1, c_zero<C>());
                v[0] += r00.x; v[1] += r00.y; v[2] += r01.x; v[3] += r01.y;
                v[4] += r10.x; v[5] += r10.y; v[6] += r11.x; v[7] += r11.y;
            }
            block_sum<8>(v, sRed);
            if (threadIdx.x < 4) {
                const C tr = c_make(v[0] + v[6], v[1] + v[7]);
                const C r = c_make(v[2 * threadIdx.x], v[2 * threadIdx.x + 1]);
                a.out[(size_t)a.node_ids[node] * 4 + threadIdx.x] = c_div(r, tr);
            }
            __syncthreads();
            continue;
        }
        // idx in A: Wb = T x_B once
        apply_messages<CM>(T, Wb, mp, d, chi, NT, h, d, -1);
        for (int idx = 0; idx < d; ++idx) {
            if (idx == h) apply_messages<CM>(T, Wa, mp, d, chi, NT, 0, h, -1);   // Wa = T x_A for idx in B
            if (idx < h) apply_messages<CM>(T, Wa, mp, d, chi, NT, 0, h, idx);
            else apply_messages<CM>(T, Wb, mp, d, chi, NT, h, d, idx);
            close_global(Wa, Wb, sP, stage, red, ipow(chi, idx), chi, ipow(chi, d - 1 - idx));
            __syncthreads();
            write_outputs<MODE, R>(a, node, idx, sP, msgs_in, msgs_out, num2, den2);
            __syncthreads();
        }
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

template <typename R>
struct GlobalArgs {
    NodeArgs<R> a;
    void* scratch;
    int64_t scratch_elems;
};

template <int MODE, typename R>
static int launch_global_solo(const PackEntry* e, int n, cudaStream_t st);

template <int MODE, typename R>
static int launch_node_global(const NodeArgs<R>& args, int count, void* scratch, int64_t scratch_elems,
                              cudaStream_t st) {
    // packed sweeps issue these one class at a time (a job's classes share its scratch)
    if (pack_record(launch_global_solo<MODE, R>, 0, 0, count, GlobalArgs<R>{args, scratch, scratch_elems}))
        return BQA_OK;
    using C = typename Cx<R>::T;
    const int chi = args.chi, d = args.d;
    const int64_t need = 4 * (int64_t)ipow(chi, d);   // two work tensors
    if (!scratch || scratch_elems < need)
        return set_error(BQA_ERR_UNSUPPORTED,
                         "degree %d at bond dim %d exceeds shared memory and the class has %lld of the %lld "
                         "scratch elements a CTA needs (bqa_node_scratch_elems)",
                         d, chi, (long long)scratch_elems, (long long)need);
    const int64_t ctas = std::min<int64_t>((int64_t)count, scratch_elems / need);
    constexpr int threads = 256;
    const size_t smem = node_global_smem_elems(d, chi, threads) * sizeof(C);
    void (*kern)(NodeArgs<R>, int, C*) = nullptr;
    if (chi <= 4) kern = node_kernel_global<4, MODE, R>;
    else if (chi <= 8) kern = node_kernel_global<8, MODE, R>;
    else if (chi <= 16) kern = node_kernel_global<16, MODE, R>;
    else if (chi <= 32) kern = node_kernel_global<32, MODE, R>;
    else return set_error(BQA_ERR_UNSUPPORTED, "node kernel: bond dim %d > 32", chi);
    int rc = ensure_smem((const void*)kern, smem, "node kernel (global)");
    if (rc) return rc;
    kern<<<(int)ctas, threads, smem, st>>>(args, count, static_cast<C*>(scratch));
    return check_launch("node kernel (global)");
}

template <int MODE, typename R>
static int launch_global_solo(const PackEntry* e, int n, cudaStream_t st) {
    for (int i = 0; i < n; ++i) {
        GlobalArgs<R> g;
        std::memcpy(&g, e[i].args, sizeof(g));
        const int rc = launch_node_global<MODE, R>(g.a, e[i].count, g.scratch, g.scratch_elems, st);
        if (rc) return rc;
    }
    return BQA_OK;
}

// packed sweeps: launches without a merged form, issued one entry at a time through `launch`
template <int (*LAUNCH)(const NodeArgs<float>&, int, cudaStream_t)>
static int launch_solo_f32(const PackEntry* e, int n, cudaStream_t st) {
    for (int i = 0; i < n; ++i) {
        NodeArgs<float> a;
        std::memcpy(&a, e[i].args, sizeof(a));
        const int rc = LAUNCH(a, e[i].count, st);
        if (rc) return rc;
    }
    return BQA_OK;
}

// Register-tiled complex64 kernel for compile-time (D, CHI): BP messages, extended messages,
// densities.
template <int D, int CHI, int MODE>
__global__ void __launch_bounds__(tiled::Shape<D, CHI>::THREADS) tiled_node_kernel(NodeArgs<float> a) {
    using S = tiled::Shape<D, CHI>;
    static_assert(CHI % 4 == 0, "tiled kernel needs chi % 4 == 0");
    static_assert(D >= 2 && D <= 4, "tiled kernel schedules cover degrees 2..4");
    static_assert(S::CLOSE_TILES <= S::THREADS, "close tiles exceed the block");
    constexpr int NT = S::NT, N2 = S::N2, PER_S = S::PER_S, TH = S::THREADS, SW = S::SW;
    extern __shared__ double4_32a smem_raw[];
    float2* sT = reinterpret_cast<float2*>(smem_raw);
    float2* sA = sT + NT;
    float2* sB = sA + NT;
    float2* sMt = sB + NT;
    float2* sP = sMt + D * N2;
    float* sRed = reinterpret_cast<float*>(sP + 2 * N2);

    const float2* msgs_in = a.msgs_a;
    float2* msgs_out = a.msgs_b;
    if (MODE == MODE_BP && a.loop_state != nullptr) {
        if (a.loop_state[0]) return;
        if (a.loop_state[2]) { msgs_in = a.msgs_b; msgs_out = const_cast<float2*>(a.msgs_a); }
    }
    const int node = blockIdx.x;
    {
        const float4* tg = reinterpret_cast<const float4*>(a.tensors + (size_t)node * NT);
        for (int i = threadIdx.x; i < NT / 2; i += TH)
            *reinterpret_cast<float4*>(sT + tiled::swz<SW>(2 * i)) = tg[i];
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const float2* mg = msgs_in + (size_t)a.in_pos[node * D + k] * N2;
        // transpose on the way in; consecutive threads write consecutive shared addresses
        for (int o = threadIdx.x; o < N2; o += TH) {
            const int j = o / CHI, i = o - j * CHI;
            sMt[k * N2 + o] = mg[i * CHI + j];
        }
    }
    __syncthreads();

    float num2 = 0.f, den2 = 0.f;
    auto prod = [&](const float2* X, float2* Y, int k) {
        tiled::product<D, CHI, TH, SW>(X, Y, sMt + k * N2, k);
        __syncthreads();
    };
    // P[a][b] = sum conj(X[..a..]) R[..b..] over every index but bond idx
    auto emit = [&](int idx, const float2* X, const float2* R) {
        tiled::close_tiled<CHI, TH, S::KS, PER_S, SW>(X, R, sP, ipow(CHI, idx), ipow(CHI, D - 1 - idx));
        __syncthreads();
        write_outputs<MODE, float>(a, node, idx, sP, msgs_in, msgs_out, num2, den2);
        __syncthreads();
    };
    if constexpr (MODE == MODE_DENS) {
        // rho[s][s'] = sum (T x_all M)[s, ..] conj(T[s', ..]) (backends.py:440-448): both
        // buffers share one swizzle, so the sum runs over shared positions directly
        const float2* cur = sT;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            float2* nxt = (k & 1) ? sB : sA;
            prod(cur, nxt, k);
            cur = nxt;
        }
        float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int p = threadIdx.x; p < PER_S; p += TH) {
            const float2 x0 = cur[p], x1 = cur[PER_S + p];
            const float2 t0 = sT[p], t1 = sT[PER_S + p];
            const float2 r00 = c_fma_conj(t0, x0, c_zero<float2>()), r01 = c_fma_conj(t1, x0, c_zero<float2>());
            const float2 r10 = c_fma_conj(t0, x1, c_zero<float2>()), r11 = c_fma_conj(t1, x1, c_zero<float2>());
            v[0] += r00.x; v[1] += r00.y; v[2] += r01.x; v[3] += r01.y;
            v[4] += r10.x; v[5] += r10.y; v[6] += r11.x; v[7] += r11.y;
        }
        block_sum<8>(v, sRed);
        if (threadIdx.x < 4) {
            const float2 tr = c_make(v[0] + v[6], v[1] + v[7]);
            const float2 r = c_make(v[2 * threadIdx.x], v[2 * threadIdx.x + 1]);
            a.out[(size_t)a.node_ids[node] * 4 + threadIdx.x] = c_div(r, tr);
        }
        return;
    } else if (D == 2) {
        prod(sT, sA, 1); emit(0, sT, sA);
        prod(sT, sA, 0); emit(1, sT, sA);
    } else if (D == 3) {
        prod(sT, sA, 1);                    // V1 = T x1
        prod(sT, sB, 2);                    // V2 = T x2
        emit(0, sA, sB);
        tiled::product_first_inplace<D, CHI, TH, SW, 2>(sT, sMt);   // V0 = T x0 over T
        __syncthreads();
        emit(2, sT, sA);
        emit(1, sT, sB);
    } else {
        prod(sT, sB, 0); prod(sB, sA, 1);   // U = T x0 x1
        prod(sA, sB, 2); emit(3, sT, sB);
        prod(sA, sB, 3); emit(2, sT, sB);
        prod(sT, sB, 2); prod(sB, sA, 3);   // V = T x2 x3
        prod(sA, sB, 0); emit(1, sT, sB);
        prod(sA, sB, 1); emit(0, sT, sB);
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

template <int D, int CHI, int MODE>
static int launch_tiled(const NodeArgs<float>& args, int count, cudaStream_t st) {
    if (pack_record(launch_solo_f32<launch_tiled<D, CHI, MODE>>, 0, 0, count, args)) return BQA_OK;
    using S = tiled::Shape<D, CHI>;
    const size_t smem = (size_t)S::SMEM_ELEMS * sizeof(float2);
    int rc = ensure_smem((const void*)tiled_node_kernel<D, CHI, MODE>, smem, "tiled node kernel");
    if (rc) return rc;
    tiled_node_kernel<D, CHI, MODE><<<count, S::THREADS, smem, st>>>(args);
    return check_launch("tiled node kernel");
}

// (degree, chi) pairs with a register-tiled complex64 kernel; 1 if launched, 0 if not covered
template <int MODE>
static int try_tiled(const NodeArgs<float>& a, int count, cudaStream_t st, int* rc) {
    const int d = a.d, chi = a.chi;
#define BQA_TILED(DD, CC) \
    if (d == DD && chi == CC) { *rc = launch_tiled<DD, CC, MODE>(a, count, st); return 1; }
    BQA_TILED(2, 8) BQA_TILED(2, 12) BQA_TILED(2, 16)
    BQA_TILED(3, 4) BQA_TILED(3, 8) BQA_TILED(3, 12) BQA_TILED(3, 16)
    BQA_TILED(4, 4) BQA_TILED(4, 8)
#undef BQA_TILED
    return 0;
}


// Half-node register-tiled kernel: CTA (node, s) computes P_s of every bond of the node and
// writes it to pm[slot][s] (the layout of the PSPLIT mode); bp_combine_kernel turns
// P_0 + P_1 into messages.  Same contraction schedules as tiled_node_kernel.
// SPEC: the (3, 16) shape with the address arithmetic of tiled_d3c16.cuh (same operations).
template <int D, int CHI, bool SPEC>
__device__ __forceinline__ void tiled_half_body(const NodeArgs<float>& a, int node, int s) {
    using S = tiled::HalfShape<D, CHI>;
    static_assert(CHI % 4 == 0 && D >= 2 && D <= 4, "half kernel shapes");
    static_assert(!SPEC || (D == 3 && CHI == 16 && S::THREADS == tiled::d3c16::TH && S::KS == 16),
                  "specialised half kernel is built for degree 3, bond dim 16");
    static_assert(S::CLOSE_TILES <= S::THREADS, "close tiles exceed the block");
    constexpr int PS = S::PER_S, N2 = S::N2, TH = S::THREADS, SW = S::SW;
    extern __shared__ double4_32a smem_raw[];
    float2* sT = reinterpret_cast<float2*>(smem_raw);
    float2* sA = sT + PS;
    float2* sB = sA + PS;
    float2* sMt = sB + PS;
    float2* sP = sMt + D * N2;
    const float2* msgs_in = a.msgs_a;
    if (a.loop_state != nullptr) {
        if (a.loop_state[0]) return;
        if (a.loop_state[2]) msgs_in = a.msgs_b;
    }
    if (a.mixed_role == 2 && low_precision_sweep(a.loop_state, a.mixed_switch)) return;
    {
        const float4* tg = reinterpret_cast<const float4*>(a.tensors + (size_t)node * 2 * PS + (size_t)s * PS);
        if constexpr (SPEC) {
            tiled::d3c16::load_half(sT, tg);
        } else {
            for (int i = threadIdx.x; i < PS / 2; i += TH)
                *reinterpret_cast<float4*>(sT + tiled::swz<SW>(2 * i)) = tg[i];
        }
    }
    int offdiag = 0;   // this thread loaded a nonzero off-diagonal message entry
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const float2* mg = msgs_in + (size_t)a.in_pos[node * D + k] * N2;
        // transpose on the way in; consecutive threads write consecutive shared addresses
        for (int o = threadIdx.x; o < N2; o += TH) {
            const int j = o / CHI, i = o - j * CHI;
            const float2 v = mg[i * CHI + j];
            sMt[k * N2 + o] = v;
            offdiag |= (i != j) && (v.x != 0.f || v.y != 0.f);
        }
    }
    // Every incoming message diagonal (the first sweep after a truncation starts from
    // diag(lambda)/tr): the degree-3 bond products are bond scalings (diag_scale3), the same
    // values without the dense products.  NaN counts as nonzero.
    const bool diag = !__syncthreads_or(offdiag);
    auto prod = [&](const float2* X, float2* Y, int k) {
        tiled::product<D, CHI, TH, SW, 1>(X, Y, sMt + k * N2, k);
        __syncthreads();
    };
    auto emit = [&](int idx, const float2* X, const float2* R) {
        tiled::close_tiled<CHI, TH, S::KS, PS, SW, 1, true>(X, R, sP, ipow(CHI, idx), ipow(CHI, D - 1 - idx));
        __syncthreads();
        float4* og = reinterpret_cast<float4*>(a.out + ((size_t)a.out_pos[node * D + idx] * 2 + s) * N2);
        tiled::write_half_block<CHI>(sP, og, threadIdx.x, TH);
        __syncthreads();
    };
    if constexpr (SPEC) {
        namespace q = tiled::d3c16;
        // The closing contractions run on warps 0-4 (the 10 upper tiles); warps 5-7 meanwhile copy
        // the previous block to global memory, so each closing phase ends with one barrier and the
        // blocks alternate between two shared buffers.  The last block is copied at the end.
        constexpr int CT = 160;
        float2* const sPb[2] = {sP, sP + N2};
        int pend = -1, cur = 0;   // bond whose block waits in sPb[cur ^ 1] (-1: none)
        auto out_block = [&](int idx) {
            return reinterpret_cast<float4*>(a.out + ((size_t)a.out_pos[node * D + idx] * 2 + s) * N2);
        };
        auto emit_s = [&](auto idx_tag, const float2* X, const float2* R) {
            constexpr int IDX = decltype(idx_tag)::value;
            if (threadIdx.x < CT) q::close<IDX>(X, R, sPb[cur]);
            else if (pend >= 0) tiled::write_half_block<CHI>(sPb[cur ^ 1], out_block(pend), threadIdx.x - CT, TH - CT);
            __syncthreads();
            pend = IDX;
            cur ^= 1;
        };
        if (diag) {
            tiled::diag_scale3<CHI, TH, SW>(sT, sA, sMt + N2, 1);
            tiled::diag_scale3<CHI, TH, SW>(sT, sB, sMt + 2 * N2, 2);
        } else {
            q::prod1(sT, sA, sMt + N2);
            __syncthreads();
            q::prod2(sT, sB, sMt + 2 * N2);
        }
        __syncthreads();
        emit_s(std::integral_constant<int, 0>{}, sA, sB);
        if (diag) tiled::diag_scale3<CHI, TH, SW>(sT, sT, sMt, 0);
        else q::prod0_inplace(sT, sMt);
        __syncthreads();
        emit_s(std::integral_constant<int, 2>{}, sT, sA);
        emit_s(std::integral_constant<int, 1>{}, sT, sB);
        tiled::write_half_block<CHI>(sPb[cur ^ 1], out_block(pend), threadIdx.x, TH);
    } else if (D == 2) {
        prod(sT, sA, 1); emit(0, sT, sA);
        prod(sT, sA, 0); emit(1, sT, sA);
    } else if (D == 3) {
        if (diag) {
            tiled::diag_scale3<CHI, TH, SW>(sT, sA, sMt + N2, 1);
            tiled::diag_scale3<CHI, TH, SW>(sT, sB, sMt + 2 * N2, 2);
            __syncthreads();
        } else {
            prod(sT, sA, 1);
            prod(sT, sB, 2);
        }
        emit(0, sA, sB);
        if (diag) tiled::diag_scale3<CHI, TH, SW>(sT, sT, sMt, 0);
        else tiled::product_first_inplace<D, CHI, TH, SW, 1>(sT, sMt);
        __syncthreads();
        emit(2, sT, sA);
        emit(1, sT, sB);
    } else {
        prod(sT, sB, 0); prod(sB, sA, 1);
        prod(sA, sB, 2); emit(3, sT, sB);
        prod(sA, sB, 3); emit(2, sT, sB);
        prod(sT, sB, 2); prod(sB, sA, 3);
        prod(sA, sB, 0); emit(1, sT, sB);
        prod(sA, sB, 1); emit(0, sT, sB);
    }
}

template <int D, int CHI, bool SPEC>
__global__ void __launch_bounds__(tiled::HalfShape<D, CHI>::THREADS) tiled_half_kernel(NodeArgs<float> a) {
    tiled_half_body<D, CHI, SPEC>(a, blockIdx.x >> 1, blockIdx.x & 1);
}

// the half-node kernel over several classes (first counts CTAs: two per node)
template <int D, int CHI, bool SPEC>
__global__ void __launch_bounds__(tiled::HalfShape<D, CHI>::THREADS)
    tiled_half_kernel_merged(const __grid_constant__ MergedClasses<float> m) {
    const int c = merged_class(m.first, m.n);
    const int local = (int)blockIdx.x - m.first[c];
    tiled_half_body<D, CHI, SPEC>(m.cls[c], local >> 1, local & 1);
}

template <int D, int CHI, bool SPEC>
static int launch_half_packed(const PackEntry* e, int n, cudaStream_t st);

template <int D, int CHI, bool SPEC>
static int launch_half_k(const NodeArgs<float>& args, int count, cudaStream_t st) {
    if (pack_record(launch_half_packed<D, CHI, SPEC>, 0, 0, count, args)) return BQA_OK;
    using S = tiled::HalfShape<D, CHI>;
    const size_t smem = (size_t)S::SMEM_ELEMS * sizeof(float2);
    int rc = ensure_smem((const void*)tiled_half_kernel<D, CHI, SPEC>, smem, "tiled half kernel");
    if (rc) return rc;
    tiled_half_kernel<D, CHI, SPEC><<<2 * count, S::THREADS, smem, st>>>(args);
    return check_launch("tiled half kernel");
}

template <int D, int CHI, bool SPEC>
static int launch_half_packed(const PackEntry* e, int n, cudaStream_t st) {
    using S = tiled::HalfShape<D, CHI>;
    const size_t smem = (size_t)S::SMEM_ELEMS * sizeof(float2);
    int rc = ensure_smem((const void*)tiled_half_kernel_merged<D, CHI, SPEC>, smem, "tiled half kernel (merged)");
    if (rc) return rc;
    for (int i0 = 0; i0 < n; i0 += kMaxMergedClasses) {
        MergedClasses<float> m;
        m.n = std::min(kMaxMergedClasses, n - i0);
        m.first[0] = 0;
        for (int c = 0; c < m.n; ++c) {
            std::memcpy(&m.cls[c], e[i0 + c].args, sizeof(NodeArgs<float>));
            m.first[c + 1] = m.first[c] + 2 * e[i0 + c].count;
        }
        tiled_half_kernel_merged<D, CHI, SPEC><<<m.first[m.n], S::THREADS, smem, st>>>(m);
        if ((rc = check_launch("tiled half kernel (merged)"))) return rc;
    }
    return BQA_OK;
}

// Half-node kernel of degree 3, bond dim 16 with the bond products on the tensor cores
// (tc_d3c16.cuh) and the closing contractions of the specialised CUDA-core kernel; same inputs,
// outputs and schedule of closes as tiled_half_kernel<3, 16, true>.  Two CTAs of 256 threads and
// 106 KB share an SM (256 tensor-memory columns each).  A CTA whose incoming messages are all
// diagonal applies them as bond scalings on the CUDA cores, as the other half-node kernels do.
__global__ void __launch_bounds__(tcd3::TH, 2) tc_half_kernel_d3c16(NodeArgs<float> a) {
    constexpr int CHI = 16, D = 3, N2 = CHI * CHI, PS = CHI * CHI * CHI, TH = tcd3::TH;
    extern __shared__ double4_32a smem_raw[];
    float2* region = reinterpret_cast<float2*>(smem_raw);
    float2* sMt = region + tcd3::REGION / 8;
    float2* sP = sMt + D * N2;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sP + 2 * N2);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
    float2* const V1 = region + tcd3::X_V1;
    float2* const V2 = region + tcd3::X_V2;
    float2* const V0 = region + tcd3::X_V0;
    const float2* msgs_in = a.msgs_a;
    if (a.loop_state != nullptr) {
        if (a.loop_state[0]) return;
        if (a.loop_state[2]) msgs_in = a.msgs_b;
    }
    const int t = threadIdx.x, warp = t >> 5;
    const int node = blockIdx.x >> 1, s = blockIdx.x & 1;
    float4 tv[8];
    tcd3::load_share(a.tensors + (size_t)node * 2 * PS + (size_t)s * PS, tv);
    int offdiag = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const float2* mg = msgs_in + (size_t)a.in_pos[node * D + k] * N2;
        const int j = t / CHI, i = t - j * CHI;
        const float2 v = mg[i * CHI + j];
        sMt[k * N2 + t] = v;
        offdiag |= (i != j) && (v.x != 0.f || v.y != 0.f);
    }
    const bool diag = !__syncthreads_or(offdiag);
    if (diag) {
        tcd3::store_share_swizzled(tv, V0);
        __syncthreads();
        tiled::diag_scale3<CHI, TH, 7>(V0, V1, sMt + N2, 1);
        tiled::diag_scale3<CHI, TH, 7>(V0, V2, sMt + 2 * N2, 2);
        __syncthreads();
        tiled::diag_scale3<CHI, TH, 7>(V0, V0, sMt, 0);
    } else {
        if (warp == 0) {
            tc::alloc(slot, tcd3::TMEM_COLS);
            tc::relinquish();
        }
        if (t == 0) {
            tc::mbar_init(bar, 1);
            tc::fence_mbar_init();
        }
        float* rf = reinterpret_cast<float*>(region);
        const float2* const mg[3] = {msgs_in + (size_t)a.in_pos[node * D] * N2,
                                     msgs_in + (size_t)a.in_pos[node * D + 1] * N2,
                                     msgs_in + (size_t)a.in_pos[node * D + 2] * N2};
        tcd3::store_b(mg, rf + tcd3::B_OPS / 4);
        tcd3::store_a<2>(tv, rf + tcd3::A_HI / 4, rf + tcd3::A_LO / 4);
        tc::fence_proxy_async();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        const uint32_t tmem = *slot;
        const uint32_t rb = tc::smem_u32(region);
        // V_2 = T x_2 M_2, then V_1, then V_0 through the same A space
        uint32_t parity = 0;
        bool late = false;
#pragma unroll 1
        for (int p = 0; p < 3; ++p) {
            const int bond = 2 - p;
            if (p > 0) {
                if (bond == 1) tcd3::store_a<1>(tv, rf + tcd3::A_HI / 4, rf + tcd3::A_LO / 4);
                else tcd3::store_a<0>(tv, rf + tcd3::A_HI / 4, rf + tcd3::A_LO / 4);
                tc::fence_proxy_async();
                __syncthreads();
            }
            if (t == 0) {
                tc::fence_after();
                const uint32_t col = bond == 2 ? tcd3::COL_V2 : (bond == 1 ? tcd3::COL_V1 : tcd3::COL_V0);
                tcd3::issue_product(tmem, col, rb, rb + tcd3::B_OPS + 2 * tcd3::B_BYTES * bond);
                tc::commit(bar);
            }
            const bool ok = tc::mbar_wait(bar, parity, tcd3::WAIT_CYCLES);
            parity ^= 1;
            if (__syncthreads_or(!ok)) {
                late = true;
                break;
            }
        }
        if (late) {
            // the MMAs did not complete in time: count the fault, give them one more bounded
            // wait, release the tensor memory and leave this CTA's blocks unwritten
            if (t == 0) atomicAdd(&g_tc_faults, 1);
            tc::mbar_wait(bar, parity ^ 1, tcd3::WAIT_CYCLES);
            tc::fence_before();
            __syncthreads();
            if (warp == 0) tc::dealloc(tmem, tcd3::TMEM_COLS);
            return;
        }
        tc::fence_after();
        tcd3::epilogue(tmem, region);
        tc::fence_before();
        __syncthreads();
        if (warp == 0) tc::dealloc(tmem, tcd3::TMEM_COLS);
    }
    __syncthreads();
    // closing contractions on warps 0-4, the previous block copied out by warps 5-7 meanwhile
    namespace q = tiled::d3c16;
    constexpr int CT = 160;
    float2* const sPb[2] = {sP, sP + N2};
    int pend = -1, cur = 0;
    auto out_block = [&](int idx) {
        return reinterpret_cast<float4*>(a.out + ((size_t)a.out_pos[node * D + idx] * 2 + s) * N2);
    };
    auto emit_s = [&](auto idx_tag, const float2* X, const float2* R) {
        constexpr int IDX = decltype(idx_tag)::value;
        if (t < CT) q::close<IDX>(X, R, sPb[cur]);
        else if (pend >= 0) tiled::write_half_block<CHI>(sPb[cur ^ 1], out_block(pend), t - CT, TH - CT);
        __syncthreads();
        pend = IDX;
        cur ^= 1;
    };
    emit_s(std::integral_constant<int, 0>{}, V1, V2);
    emit_s(std::integral_constant<int, 2>{}, V0, V1);
    emit_s(std::integral_constant<int, 1>{}, V0, V2);
    tiled::write_half_block<CHI>(sPb[cur ^ 1], out_block(pend), t, TH);
}

// Half-node kernel of degree 3, bond dim 16 with BF16 tensor-core products and closing
// contractions (tc_bf16_d3c16.cuh).  MIXED: the kernel does the low-precision sweeps of a mixed
// BP run (low_precision_sweep) and returns at once on the others, which the default
// FP32-accurate half-node kernel, launched next with mixed_role 2, does.  Diagonal
// incoming messages take the FP32 bond-scaling path.  Same outputs as the other half-node
// kernels (blocks P_s into pm).
//
// Grid-stride: at most two CTAs per SM walk the `halves` half-nodes (CTA b takes b,
// b + gridDim.x, ...), so a mixed sweep that is not this kernel's returns after a few hundred
// CTAs; tensor memory is allocated once per CTA and the mbarrier runs two phases per half-node.
template <bool MIXED>
__global__ void __launch_bounds__(tcb::TH, 2) tcb_half_kernel_d3c16(NodeArgs<float> a, float switch_dist, int halves) {
    constexpr int CHI = 16, D = 3, N2 = CHI * CHI, PS = CHI * CHI * CHI, TH = tcb::TH;
    extern __shared__ double4_32a smem_raw[];
    unsigned char* reg = reinterpret_cast<unsigned char*>(smem_raw);
    float2* const V1 = reinterpret_cast<float2*>(reg);   // FP32 buffers of the bond-scaling path
    float2* const V2 = V1 + PS;
    float2* const V0 = V1 + 2 * PS;
    float2* const sP = V1 + 3 * PS;
    float2* const sMt = reinterpret_cast<float2*>(reg + tcb::SMT);
    uint64_t* bar = reinterpret_cast<uint64_t*>(reg + tcb::REGION);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
    const float2* msgs_in = a.msgs_a;
    if (a.loop_state != nullptr) {
        if (a.loop_state[0]) return;
        if (a.loop_state[2]) msgs_in = a.msgs_b;
    }
    if (MIXED && !low_precision_sweep(a.loop_state, switch_dist)) return;
    const int t = threadIdx.x, warp = t >> 5;
    if (t == 0) {
        tc::mbar_init(bar, 1);
        tc::fence_mbar_init();
    }
    const uint32_t rb = tc::smem_u32(reg);
    uint32_t tmem = 0;
    bool tmem_held = false;
    namespace q = tiled::d3c16;
    constexpr int CT = 160;
    for (int h = blockIdx.x; h < halves; h += gridDim.x) {
        const int node = h >> 1, s = h & 1;
        float4 tv[8];
        tcd3::load_share(a.tensors + (size_t)node * 2 * PS + (size_t)s * PS, tv);
        int offdiag = 0;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const float2* mg = msgs_in + (size_t)a.in_pos[node * D + k] * N2;
            const int j = t / CHI, i = t - j * CHI;
            const float2 v = mg[i * CHI + j];
            sMt[k * N2 + t] = v;
            offdiag |= (i != j) && (v.x != 0.f || v.y != 0.f);
        }
        const bool diag = !__syncthreads_or(offdiag);
        auto out_block = [&](int idx) { return a.out + ((size_t)a.out_pos[node * D + idx] * 2 + s) * N2; };
        if (!diag) {
            if (!tmem_held) {
                if (warp == 0) {
                    tc::alloc(slot, tcb::TMEM_COLS);
                    tc::relinquish();
                }
                tc::fence_before();
                __syncthreads();
                tc::fence_after();
                tmem = *slot;
                tmem_held = true;
            }
            tcb::store_products_b(sMt, reg);
            tcb::store_products_a(tv, reg);
            tc::fence_proxy_async();
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
            if (t == 0) {
                tcb::issue_products(tmem, rb);
                tc::commit(bar);
            }
            // phase 0: the products; phase 1: the closing contractions
            int late = __syncthreads_or(!tc::mbar_wait(bar, 0, tcb::WAIT_CYCLES)) ? 1 : 0;
            if (!late) {
                tc::fence_after();
                tcb::epilogue_products(tmem, reg);
                tc::fence_proxy_async();
                tc::fence_before();
                __syncthreads();
                if (t == 0) {
                    tc::fence_after();
                    tcb::issue_closes(tmem, rb);
                    tc::commit(bar);
                }
                late = __syncthreads_or(!tc::mbar_wait(bar, 1, tcb::WAIT_CYCLES)) ? 2 : 0;
                if (!late) {
                    tc::fence_after();
                    if ((warp & 3) < 2) {
                        // warps 0, 1: P_0 (columns 0-31) and P_1 (64-95); warps 4, 5: P_2 (32-63)
                        if (warp < 4) {
                            tcb::epilogue_close(tmem, 0, reinterpret_cast<float*>(out_block(0)));
                            tcb::epilogue_close(tmem, 2, reinterpret_cast<float*>(out_block(1)));
                        } else {
                            tcb::epilogue_close(tmem, 1, reinterpret_cast<float*>(out_block(2)));
                        }
                    }
                }
            }
            if (late) {
                // the MMAs did not complete in time: count the fault, give them one more bounded
                // wait and stop this CTA (its remaining blocks stay unwritten)
                if (t == 0) atomicAdd(&g_tc_faults, 1);
                tc::mbar_wait(bar, late - 1, tcb::WAIT_CYCLES);
                break;
            }
            tc::fence_before();   // this half-node's tensor-memory reads precede the next MMAs
            __syncthreads();
            continue;
        }
        // all incoming messages diagonal: bond scalings in FP32, closing contractions on the CUDA cores
        tcd3::store_share_swizzled(tv, V0);
        __syncthreads();
        tiled::diag_scale3<CHI, TH, 7>(V0, V1, sMt + N2, 1);
        tiled::diag_scale3<CHI, TH, 7>(V0, V2, sMt + 2 * N2, 2);
        __syncthreads();
        tiled::diag_scale3<CHI, TH, 7>(V0, V0, sMt, 0);
        __syncthreads();
        float2* const sPb[2] = {sP, sP + N2};
        int pend = -1, cur = 0;
        auto emit_s = [&](auto idx_tag, const float2* X, const float2* R) {
            constexpr int IDX = decltype(idx_tag)::value;
            if (t < CT) q::close<IDX>(X, R, sPb[cur]);
            else if (pend >= 0)
                tiled::write_half_block<CHI>(sPb[cur ^ 1], reinterpret_cast<float4*>(out_block(pend)), t - CT,
                                             TH - CT);
            __syncthreads();
            pend = IDX;
            cur ^= 1;
        };
        emit_s(std::integral_constant<int, 0>{}, V1, V2);
        emit_s(std::integral_constant<int, 2>{}, V0, V1);
        emit_s(std::integral_constant<int, 1>{}, V0, V2);
        tiled::write_half_block<CHI>(sPb[cur ^ 1], reinterpret_cast<float4*>(out_block(pend)), t, TH);
        __syncthreads();
    }
    if (tmem_held) {
        tc::fence_before();
        __syncthreads();
        if (warp == 0) tc::dealloc(tmem, tcb::TMEM_COLS);
    }
}

// Half-node kernel of degree 3, bond dim 16 with 2xFP16 tensor-core bond products (FP32
// accuracy, tc_f16x2_d3c16.cuh) and the closing contractions on the CUDA cores (warps 0-4, the
// previous block copied out by warps 5-7).  Diagonal incoming messages take the FP32
// bond-scaling path.  Same outputs as the other half-node kernels (blocks P_s into pm).
//
// Grid-stride: at most two CTAs per SM walk the `halves` half-nodes; tensor memory is
// allocated once per CTA and the mbarrier runs one phase per half-node with MMAs.
__global__ void __launch_bounds__(tch::TH, 2) tch_half_kernel_d3c16(NodeArgs<float> a, int halves) {
    constexpr int CHI = 16, D = 3, N2 = CHI * CHI, PS = CHI * CHI * CHI, TH = tch::TH;
    extern __shared__ double4_32a smem_raw[];
    unsigned char* reg = reinterpret_cast<unsigned char*>(smem_raw);
    float2* const region = reinterpret_cast<float2*>(smem_raw);
    float2* const V1 = region + tcd3::X_V1;
    float2* const V2 = region + tcd3::X_V2;
    float2* const V0 = region + tcd3::X_V0;
    float2* const sP = region + tch::SP;
    float2* const sMt = region + tch::SMT;
    uint64_t* bar = reinterpret_cast<uint64_t*>(reg + tch::REGION);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
    uint32_t* wmax = slot + 1;   // [warp][|T|, |M_0|, |M_1|, |M_2|]
    const float2* msgs_in = a.msgs_a;
    if (a.loop_state != nullptr) {
        if (a.loop_state[0]) return;
        if (a.loop_state[2]) msgs_in = a.msgs_b;
    }
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    if (t == 0) {
        tc::mbar_init(bar, 1);
        tc::fence_mbar_init();
    }
    const uint32_t rb = tc::smem_u32(reg);
    uint32_t tmem = 0, parity = 0;
    bool tmem_held = false;
    namespace q = tiled::d3c16;
    constexpr int CT = 160;
    for (int h = blockIdx.x; h < halves; h += gridDim.x) {
        const int node = h >> 1, s = h & 1;
        float4 tv[8];
        tcd3::load_share(a.tensors + (size_t)node * 2 * PS + (size_t)s * PS, tv);
        // thread t holds entry (y, x) = (t >> 4, t & 15) of each incoming message
        float2 mv[3];
        int offdiag = 0;
        uint32_t mm[3];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            mv[k] = msgs_in[(size_t)a.in_pos[node * D + k] * N2 + t];
            offdiag |= ((t >> 4) != (t & 15)) && (mv[k].x != 0.f || mv[k].y != 0.f);
            mm[k] = __reduce_max_sync(0xffffffffu, max(tch::mag(mv[k].x), tch::mag(mv[k].y)));
        }
        uint32_t mt = 0;
#pragma unroll
        for (int m = 0; m < 8; ++m)
            mt = max(mt, max(max(tch::mag(tv[m].x), tch::mag(tv[m].y)), max(tch::mag(tv[m].z), tch::mag(tv[m].w))));
        mt = __reduce_max_sync(0xffffffffu, mt);
        if (lane == 0) {
            wmax[4 * warp] = mt;
#pragma unroll
            for (int k = 0; k < D; ++k) wmax[4 * warp + 1 + k] = mm[k];
        }
        const bool diag = !__syncthreads_or(offdiag);
        if (!diag) {
            uint32_t gm[4] = {0, 0, 0, 0};
#pragma unroll
            for (int w = 0; w < TH / 32; ++w)
#pragma unroll
                for (int i = 0; i < 4; ++i) gm[i] = max(gm[i], wmax[4 * w + i]);
            const int kt = tch::scale_exp(gm[0]);
            const int km[3] = {tch::scale_exp(gm[1]), tch::scale_exp(gm[2]), tch::scale_exp(gm[3])};
            if (!tmem_held) {
                if (warp == 0) {
                    tc::alloc(slot, tch::TMEM_COLS);
                    tc::relinquish();
                }
                tc::fence_before();
                __syncthreads();
                tc::fence_after();
                tmem = *slot;
                tmem_held = true;
            }
            const float sm[3] = {tch::pow2(km[0]), tch::pow2(km[1]), tch::pow2(km[2])};
            tch::store_b(mv, sm, reg);
            tch::store_a(tv, tch::pow2(kt), reg);
            tc::fence_proxy_async();
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
            if (t == 0) {
                tch::issue_products(tmem, rb);
                tc::commit(bar);
            }
            const bool ok = tc::mbar_wait(bar, parity, tch::WAIT_CYCLES);
            parity ^= 1;
            if (__syncthreads_or(!ok)) {
                // the MMAs did not complete in time: count the fault, give them one more bounded
                // wait and stop this CTA (its remaining blocks stay unwritten)
                if (t == 0) atomicAdd(&g_tc_faults, 1);
                tc::mbar_wait(bar, parity ^ 1, tch::WAIT_CYCLES);
                break;
            }
            tc::fence_after();
            // V_2, V_1, V_0 carry 2^(kt + km[2]), 2^(kt + km[1]), 2^(kt + km[0])
            const float sc[3][2] = {{tch::pow2(-kt), tch::pow2(-km[2])},
                                    {tch::pow2(-kt), tch::pow2(-km[1])},
                                    {tch::pow2(-kt), tch::pow2(-km[0])}};
            tcd3::epilogue<true>(tmem, region, sc);
            tc::fence_before();
            __syncthreads();
        } else {
            // all incoming messages diagonal: bond scalings in FP32 (sMt[k][16 x + y] = M_k[y][x])
#pragma unroll
            for (int k = 0; k < D; ++k) sMt[k * N2 + 16 * (t & 15) + (t >> 4)] = mv[k];
            tcd3::store_share_swizzled(tv, V0);
            __syncthreads();
            tiled::diag_scale3<CHI, TH, 7>(V0, V1, sMt + N2, 1);
            tiled::diag_scale3<CHI, TH, 7>(V0, V2, sMt + 2 * N2, 2);
            __syncthreads();
            tiled::diag_scale3<CHI, TH, 7>(V0, V0, sMt, 0);
            __syncthreads();
        }
        float2* const sPb[2] = {sP, sP + N2};
        int pend = -1, cur = 0;
        auto out_block = [&](int idx) {
            return reinterpret_cast<float4*>(a.out + ((size_t)a.out_pos[node * D + idx] * 2 + s) * N2);
        };
        auto emit_s = [&](auto idx_tag, const float2* X, const float2* R) {
            constexpr int IDX = decltype(idx_tag)::value;
            if (t < CT) q::close<IDX>(X, R, sPb[cur]);
            else if (pend >= 0) tiled::write_half_block<CHI>(sPb[cur ^ 1], out_block(pend), t - CT, TH - CT);
            __syncthreads();
            pend = IDX;
            cur ^= 1;
        };
        emit_s(std::integral_constant<int, 0>{}, V1, V2);
        emit_s(std::integral_constant<int, 2>{}, V0, V1);
        emit_s(std::integral_constant<int, 1>{}, V0, V2);
        tiled::write_half_block<CHI>(sPb[cur ^ 1], out_block(pend), t, TH);
        __syncthreads();
    }
    if (tmem_held) {
        tc::fence_before();
        __syncthreads();
        if (warp == 0) tc::dealloc(tmem, tch::TMEM_COLS);
    }
}

// Half-node kernel of degree 3, bond dim 16 with the bond products AND the closing
// contractions on the tensor cores, both in 2xFP16 (FP32-accurate; tc_f16x2_d3c16.cuh): one
// product round trip, then six closing stages (three blocks x two halves of the contraction)
// through three shared-memory buffers, a block's two stages written from one read of the
// accumulators while the previous block's MMAs run.  Diagonal incoming messages (the first sweep
// after a truncation) take the same path: a diagonal message is just a sparse B operand, and
// the bond-scaling path with CUDA-core closing contractions measured 13.4 ms against 10.4 ms
// per 100k-node sweep.  Same outputs as the other half-node kernels.
//
// Grid-stride: at most two CTAs per SM walk the `halves` half-nodes; tensor memory is allocated
// once per CTA.  Four mbarriers (products, stage buffers 0-2); every commit is waited for
// exactly once, in order, by every thread, so each wait's parity is its commit count's.  A wait
// that runs out sets the CTA's fault word and the thread carries on (every access stays inside
// its buffers); the CTA stops at the next half-node, after one more bounded wait for its last
// commit, and counts itself in bqa_tc_faults.
__global__ void __launch_bounds__(tch::TH, 2) tcx_half_kernel_d3c16(NodeArgs<float> a, int halves) {
    constexpr int CHI = 16, D = 3, N2 = CHI * CHI, PS = CHI * CHI * CHI, TH = tch::TH;
    extern __shared__ double4_32a smem_raw[];
    unsigned char* reg = reinterpret_cast<unsigned char*>(smem_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(reg + tch::REGION);   // products, buffers 0-2
    uint32_t* slot = reinterpret_cast<uint32_t*>(bars + 4);
    volatile uint32_t* fault = slot + 1;
    uint32_t* wmax = slot + 2;   // [warp][|T|, |M_0|, |M_1|, |M_2|]
    const float2* msgs_in = a.msgs_a;
    if (a.loop_state != nullptr) {
        if (a.loop_state[0]) return;
        if (a.loop_state[2]) msgs_in = a.msgs_b;
    }
    if (a.mixed_role == 2 && low_precision_sweep(a.loop_state, a.mixed_switch)) return;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    if (t == 0) {
        for (int i = 0; i < 4; ++i) tc::mbar_init(bars + i, 1);
        tc::fence_mbar_init();
        *fault = 0;
    }
    const uint32_t rb = tc::smem_u32(reg);
    uint32_t tmem = 0;
    uint32_t commits[4] = {0, 0, 0, 0};
    int last = -1;          // barrier of the latest commit
    uint32_t last_par = 0;  // and the parity of its phase
    bool tmem_held = false;
    // this thread's row of the products' accumulators
    const int prow = 128 * (warp >> 2) + 32 * (warp & 3) + lane, phi = prow >> 4, plo = prow & 15;
    auto wait = [&](int i) {
        if (!tc::mbar_wait(bars + i, (commits[i] - 1) & 1, tch::WAIT_CYCLES)) *fault = 1;
    };
#pragma unroll 1
    for (int h = blockIdx.x; h < halves; h += gridDim.x) {
        const int node = h >> 1, s = h & 1;
        float4 tv[8];
        tcd3::load_share(a.tensors + (size_t)node * 2 * PS + (size_t)s * PS, tv);
        // thread t holds entry (y, x) = (t >> 4, t & 15) of each incoming message
        float2 mv[3];
        uint32_t mm[3];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            mv[k] = msgs_in[(size_t)a.in_pos[node * D + k] * N2 + t];
            mm[k] = __reduce_max_sync(0xffffffffu, max(tch::mag(mv[k].x), tch::mag(mv[k].y)));
        }
        uint32_t mt = 0;
#pragma unroll
        for (int m = 0; m < 8; ++m)
            mt = max(mt, max(max(tch::mag(tv[m].x), tch::mag(tv[m].y)), max(tch::mag(tv[m].z), tch::mag(tv[m].w))));
        mt = __reduce_max_sync(0xffffffffu, mt);
        if (lane == 0) {
            wmax[4 * warp] = mt;
#pragma unroll
            for (int k = 0; k < D; ++k) wmax[4 * warp + 1 + k] = mm[k];
        }
        auto out_block = [&](int idx) { return a.out + ((size_t)a.out_pos[node * D + idx] * 2 + s) * N2; };
        __syncthreads();
        if (*fault) break;
        {
            uint32_t gm[4] = {0, 0, 0, 0};
#pragma unroll
            for (int w = 0; w < TH / 32; ++w)
#pragma unroll
                for (int i = 0; i < 4; ++i) gm[i] = max(gm[i], wmax[4 * w + i]);
            const int kt = tch::scale_exp(gm[0]);
            const int km[3] = {tch::scale_exp(gm[1]), tch::scale_exp(gm[2]), tch::scale_exp(gm[3])};
            if (!tmem_held) {
                if (warp == 0) {
                    tc::alloc(slot, tch::TMEM_COLS);
                    tc::relinquish();
                }
                tc::fence_before();
                __syncthreads();
                tc::fence_after();
                tmem = *slot;
                tmem_held = true;
            }
            const float sm[3] = {tch::pow2(km[0]), tch::pow2(km[1]), tch::pow2(km[2])};
            tch::store_b(mv, sm, reg);
            tch::store_a(tv, tch::pow2(kt), reg);
            tc::fence_proxy_async();
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
            if (t == 0) {
                tch::issue_products(tmem, rb);
                tc::commit(bars);
                // the CTA's next half-node: its tensor and incoming messages into L2 meanwhile
                const int hn = h + gridDim.x;
                if (hn < halves) {
                    const int nn = hn >> 1;
                    tc::prefetch_l2(a.tensors + (size_t)nn * 2 * PS + (size_t)(hn & 1) * PS, PS * sizeof(float2));
#pragma unroll
                    for (int k = 0; k < D; ++k)
                        tc::prefetch_l2(msgs_in + (size_t)a.in_pos[nn * D + k] * N2, N2 * sizeof(float2));
                }
            }
            ++commits[0];
            last = 0;
            last_par = (commits[0] - 1) & 1;
            wait(0);
            tc::fence_after();
            const uint32_t tl = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 32 * (warp >> 2);
            // P = D 2^(42 - 2 kt - km_x - km_r), as two normal factors
            auto unscale = [&](int kx, int kr, float (&sc)[2]) {
                const int e = 42 - 2 * kt - kx - kr, e1 = max(-126, min(126, e));
                sc[0] = tch::pow2(e1);
                sc[1] = tch::pow2(e - e1);
            };
            // block 0: P_0 = <V_1|V_2> (columns C0); 1: P_2 = <V_0|V_1> (C1); 2: P_1 = <V_0|V_2> (C0)
            auto block_epilogue = [&](int blk) {
                float sc[2];
                if (blk == 0) unscale(km[1], km[2], sc);
                else if (blk == 1) unscale(km[0], km[1], sc);
                else unscale(km[0], km[2], sc);
                tch::epilogue_block(tmem + (blk == 1 ? tch::COL_C1 : tch::COL_C0), sc,
                                    reinterpret_cast<float*>(out_block(blk == 0 ? 0 : (blk == 1 ? 2 : 1))));
            };
            // block b's two stages go to buffers (2 b) % 3 and (2 b + 1) % 3: block 1 waits for
            // stage 0 (its buffer 0), block 2 for stages 1 and 2 (buffers 1, 2; block 0's
            // accumulator, which block 2 reuses, is complete then and read first)
            auto block = [&](auto blk_tag) {
                constexpr int BLK = decltype(blk_tag)::value, B0 = (2 * BLK) % 3, B1 = (2 * BLK + 1) % 3;
                if (BLK == 1) {
                    wait(1);
                    tc::fence_after();
                } else if (BLK == 2) {
                    wait(2);
                    wait(3);
                    tc::fence_after();
                    if (warp < 4) block_epilogue(0);
                }
                tch::write_block<BLK>(tl, phi, plo, reg + B0 * tch::STAGE, reg + B1 * tch::STAGE);
                tc::fence_proxy_async();
                tc::fence_before();
                __syncthreads();
                if (t == 0) {
                    tc::fence_after();
                    const uint32_t d = tmem + ((BLK & 1) ? tch::COL_C1 : tch::COL_C0);
                    tch::issue_stage(d, rb + B0 * tch::STAGE, 0);
                    tc::commit(bars + 1 + B0);
                    tch::issue_stage(d, rb + B1 * tch::STAGE, 1);
                    tc::commit(bars + 1 + B1);
                }
                ++commits[1 + B0];
                ++commits[1 + B1];
                last = 1 + B1;
                last_par = (commits[1 + B1] - 1) & 1;
            };
            block(std::integral_constant<int, 0>{});
            block(std::integral_constant<int, 1>{});
            block(std::integral_constant<int, 2>{});
            wait(1);   // stage 3
            wait(2);   // stage 4
            wait(3);   // stage 5
            tc::fence_after();
            block_epilogue(warp < 4 ? 1 : 2);
            tc::fence_before();   // these tensor-memory reads precede the next half-node's MMAs
        }
    }
    tc::fence_before();
    __syncthreads();
    if (*fault) {
        // an MMA wait ran out: give the latest commit one more bounded wait, count the CTA
        if (last >= 0) tc::mbar_wait(bars + last, last_par, tch::WAIT_CYCLES);
        if (t == 0) atomicAdd(&g_tc_faults, 1);
    }
    if (tmem_held && warp == 0) {
        tc::fence_after();
        tc::dealloc(tmem, tch::TMEM_COLS);
    }
}

// BP distance above which the mixed-precision (3, 16) kernel takes its BF16 path; the
// environment variable BQA_GB300_MIXED_SWITCH overrides it when the library loads.
static const float g_mixed_switch = [] {
    const char* v = getenv("BQA_GB300_MIXED_SWITCH");
    return v ? (float)atof(v) : 0.03125f;
}();

// multiprocessors of the current device (cached per device ordinal)
static int sm_count() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 152;
        cache[dev] = n;
    }
    return cache[dev];
}

template <bool MIXED>
static int launch_tcb_half(const NodeArgs<float>& args, int count, cudaStream_t st) {
    if (pack_record(launch_solo_f32<launch_tcb_half<MIXED>>, 0, 0, count, args)) return BQA_OK;
    const size_t smem = (size_t)tcb::REGION + 16;
    int rc = ensure_smem((const void*)tcb_half_kernel_d3c16<MIXED>, smem, "bf16 tensor-core half kernel");
    if (rc) return rc;
    const int halves = 2 * count;
    tcb_half_kernel_d3c16<MIXED><<<std::min(halves, 2 * sm_count()), tcb::TH, smem, st>>>(args, g_mixed_switch,
                                                                                             halves);
    return check_launch("bf16 tensor-core half kernel");
}

static int launch_tcx_half(const NodeArgs<float>& args, int count, cudaStream_t st) {
    const size_t smem = (size_t)tch::REGION + tch::SCRATCH_X;
    int rc = ensure_smem((const void*)tcx_half_kernel_d3c16, smem, "2xFP16 tensor-core half kernel");
    if (rc) return rc;
    const int halves = 2 * count;
    tcx_half_kernel_d3c16<<<std::min(halves, 2 * sm_count()), tch::TH, smem, st>>>(args, halves);
    return check_launch("2xFP16 tensor-core half kernel");
}

static int launch_tch_half(const NodeArgs<float>& args, int count, cudaStream_t st) {
    const size_t smem = (size_t)tch::REGION + tch::SCRATCH;
    int rc = ensure_smem((const void*)tch_half_kernel_d3c16, smem, "2xFP16 tensor-core half kernel");
    if (rc) return rc;
    const int halves = 2 * count;
    tch_half_kernel_d3c16<<<std::min(halves, 2 * sm_count()), tch::TH, smem, st>>>(args, halves);
    return check_launch("2xFP16 tensor-core half kernel");
}

// The FP32-accurate tensor-core kernel, chosen by BQA_GB300_TC_KIND when the library loads:
// products and closing contractions in 2xFP16 (default), "products" for 2xFP16 products with
// the closing contractions on the CUDA cores, "tf32" for 3xTF32 products.
static const int g_tc_kind = [] {
    const char* v = getenv("BQA_GB300_TC_KIND");
    if (v && !strcmp(v, "products")) return 1;
    if (v && !strcmp(v, "tf32")) return 2;
    return 0;
}();

static int launch_tc_half(const NodeArgs<float>& args, int count, cudaStream_t st) {
    if (pack_record(launch_solo_f32<launch_tc_half>, 0, 0, count, args)) return BQA_OK;
    if (g_tc_kind == 0) return launch_tcx_half(args, count, st);
    if (g_tc_kind == 1) return launch_tch_half(args, count, st);
    const size_t smem = (size_t)tcd3::REGION + (3 + 2) * 256 * sizeof(float2) + 16;
    int rc = ensure_smem((const void*)tc_half_kernel_d3c16, smem, "tensor-core half kernel");
    if (rc) return rc;
    tc_half_kernel_d3c16<<<2 * count, tcd3::TH, smem, st>>>(args);
    return check_launch("tensor-core half kernel");
}

template <int D, int CHI>
static int launch_half(const NodeArgs<float>& args, int count, cudaStream_t st) {
    if constexpr (D == 3 && CHI == 16) {
        if (g_use_tc) return launch_tc_half(args, count, st);
        if (g_use_specialized) return launch_half_k<D, CHI, true>(args, count, st);
    }
    return launch_half_k<D, CHI, false>(args, count, st);
}

// 1 if a half-node kernel covers (degree, chi) and was launched
static int try_half(const NodeArgs<float>& a, int count, cudaStream_t st, int* rc) {
    const int d = a.d, chi = a.chi;
#define BQA_HALF(DD, CC) \
    if (d == DD && chi == CC) { *rc = launch_half<DD, CC>(a, count, st); return 1; }
    BQA_HALF(2, 8) BQA_HALF(2, 12) BQA_HALF(2, 16)
    BQA_HALF(3, 4) BQA_HALF(3, 8) BQA_HALF(3, 12) BQA_HALF(3, 16)
    BQA_HALF(4, 4) BQA_HALF(4, 8)
#undef BQA_HALF
    return 0;
}

// Extended messages from the open-bond blocks (the EXT epilogue of write_outputs as a pass of
// its own): block (r, c) of the 2chi x 2chi message of slot e is
// conj(a_r) a_c (P_0 + (-1)^(r+c) P_1) / ((|a_0|^2 + |a_1|^2) tr), a_0, a_1 the half-ZZ
// coefficients of J[e % (E/2)] * ztime (src/bqa/state.py:127-139, backends.py:519-526).
// One warp per slot; every lane forms the trace in the same order as write_outputs, so from
// the same blocks the output equals the one-pass kernel's bit for bit.
template <typename R>
__global__ void __launch_bounds__(256) ext_combine_kernel(const typename Cx<R>::T* __restrict__ pm, int E, int chi,
                                                          const double* __restrict__ edge_j, double ztime,
                                                          typename Cx<R>::T* __restrict__ ext) {
    using C = typename Cx<R>::T;
    const int lane = threadIdx.x & 31;
    const int slot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (slot >= E) return;
    const int n2 = chi * chi, n = 2 * chi;
    const C* p0 = pm + (size_t)slot * 2 * n2;
    const C* p1 = p0 + n2;
    C tr = c_zero<C>();
    for (int q = 0; q < chi; ++q) tr = c_add(tr, c_add(p0[q * chi + q], p1[q * chi + q]));
    const HalfZZ<R> h = half_zz_warp<R>(edge_j[slot % (E / 2)] * ztime);
    const R scale = c_abs2(h.a0) + c_abs2(h.a1);
    const C trx = c_scale(tr, scale);
    C* og = ext + (size_t)slot * n * n;
    for (int o = lane; o < n * n; o += 32) {
        const int row = o / n, col = o - row * n;
        const int e = row >= chi, f = col >= chi;
        const int ia = row - e * chi, ib = col - f * chi;
        const C a0 = p0[ia * chi + ib], a1 = p1[ia * chi + ib];
        const C pe = ((e + f) & 1) ? c_sub(a0, a1) : c_add(a0, a1);
        const C coef = c_mul(c_conj(e ? h.a1 : h.a0), f ? h.a1 : h.a0);
        og[o] = c_div(c_mul(coef, pe), trx);
    }
}

// BP messages from the open-bond blocks: msg[e] = (P_0 + P_1)/tr, with the convergence maxima
// max|new-old|^2 and max|new+old|^2 folded per block into dist_parts.  One warp per slot.
template <typename R>
struct CombineArgs {
    const typename Cx<R>::T* pm;
    int E, chi;
    const typename Cx<R>::T* msgs_a;
    typename Cx<R>::T* msgs_b;
    const int32_t* loop_state;
    typename Cx<R>::Bits* dist_parts;
};

// block `blk` of the combine of one job
template <typename R>
__device__ __forceinline__ void bp_combine_body(const CombineArgs<R>& x, int blk) {
    using C = typename Cx<R>::T;
    __shared__ R sRed[32];
    const C* __restrict__ pm = x.pm;
    const int E = x.E, chi = x.chi;
    const C* msgs_in = x.msgs_a;
    C* msgs_out = x.msgs_b;
    if (x.loop_state != nullptr) {
        if (x.loop_state[0]) return;
        if (x.loop_state[2]) { msgs_in = x.msgs_b; msgs_out = const_cast<C*>(x.msgs_a); }
    }
    typename Cx<R>::Bits* dist_parts = x.dist_parts;
    const int lane = threadIdx.x & 31;
    const int slot = (blk * blockDim.x + threadIdx.x) >> 5;
    const int n2 = chi * chi;
    R num2 = 0, den2 = 0;
    if (slot < E) {
        const C* p0 = pm + (size_t)slot * 2 * n2;
        const C* p1 = p0 + n2;
        C tr = c_zero<C>();
        for (int q = lane; q < chi; q += 32) tr = c_add(tr, c_add(p0[q * chi + q], p1[q * chi + q]));
        tr.x = warp_sum(tr.x);
        tr.y = warp_sum(tr.y);
        const C* old = msgs_in + (size_t)slot * n2;
        C* og = msgs_out + (size_t)slot * n2;
        for (int i = lane; i < n2; i += 32) {
            const C m = c_div(c_add(p0[i], p1[i]), tr);
            const C o = old[i];
            og[i] = m;
            num2 = fmax(num2, c_abs2(c_sub(m, o)));
            den2 = fmax(den2, c_abs2(c_add(m, o)));
        }
    }
    num2 = block_max(num2, sRed);
    den2 = block_max(den2, sRed);
    if (threadIdx.x == 0) {
        atomic_max_nonneg(dist_parts, num2);
        atomic_max_nonneg(dist_parts + 1, den2);
    }
}

template <typename R>
__global__ void __launch_bounds__(256) bp_combine_kernel(const CombineArgs<R> x) {
    bp_combine_body<R>(x, blockIdx.x);
}

// the combines of several jobs in one launch (first counts blocks)
template <typename R>
struct MergedCombine {
    CombineArgs<R> job[kMaxMergedClasses];
    int first[kMaxMergedClasses + 1];
    int n;
};

template <typename R>
__global__ void __launch_bounds__(256) bp_combine_kernel_merged(const __grid_constant__ MergedCombine<R> m) {
    const int c = merged_class(m.first, m.n);
    bp_combine_body<R>(m.job[c], (int)blockIdx.x - m.first[c]);
}

template <typename R>
static int launch_combine_packed(const PackEntry* e, int n, cudaStream_t st) {
    for (int i0 = 0; i0 < n; i0 += kMaxMergedClasses) {
        MergedCombine<R> m;
        m.n = std::min(kMaxMergedClasses, n - i0);
        m.first[0] = 0;
        for (int c = 0; c < m.n; ++c) {
            std::memcpy(&m.job[c], e[i0 + c].args, sizeof(CombineArgs<R>));
            m.first[c + 1] = m.first[c] + e[i0 + c].count;
        }
        bp_combine_kernel_merged<R><<<m.first[m.n], 256, 0, st>>>(m);
        const int rc = check_launch("bp_combine (merged)");
        if (rc) return rc;
    }
    return BQA_OK;
}

// threads of a generic-kernel CTA for degree d at bond dim chi: one per fibre of a mode
// product (or output of a closing contraction), at most 256 -- or, for the BP and open-bond
// passes of nodes whose shared memory leaves room for at most two CTAs per SM, at most 1024
// (bond dims <= 8: the 1024-thread build), so such nodes still run 16-32 warps per SM
static int generic_threads(int d, int chi, int mode, size_t elem_bytes) {
    const int fib = 2 * ipow(chi, d > 0 ? d - 1 : 0);
    int threads = ((max(fib, 2 * chi * chi) + 31) / 32) * 32;
    const size_t smem = node_smem_elems(d, chi) * elem_bytes;
    const bool crowded = (228u * 1024u) / (smem + 1024u) <= 2;
    const int cap = (crowded && chi <= 8 && (mode == MODE_BP || mode == MODE_PSPLIT)) ? 1024 : 256;
    return threads < 32 ? 32 : (threads > cap ? cap : threads);
}

// The generic kernel's build for bond dim chi and CTAs of `threads` threads (0: none).
template <typename A, int MODE, typename R, template <int, int, typename> class Pick>
static void (*generic_build(int chi, int threads))(A) {
    if (threads > 256) {
        if constexpr (MODE == MODE_BP || MODE == MODE_PSPLIT) {
            if (chi <= 1) return Pick<1, MODE, R>::wide;
            if (chi <= 2) return Pick<2, MODE, R>::wide;
            if (chi <= 4) return Pick<4, MODE, R>::wide;
            if (chi <= 8) return Pick<8, MODE, R>::wide;
        }
        return nullptr;
    }
    if (chi <= 1) return Pick<1, MODE, R>::narrow;
    if (chi <= 2) return Pick<2, MODE, R>::narrow;
    if (chi <= 4) return Pick<4, MODE, R>::narrow;
    if (chi <= 8) return Pick<8, MODE, R>::narrow;
    if (chi <= 16) return Pick<16, MODE, R>::narrow;
    if (chi <= 32) return Pick<32, MODE, R>::narrow;
    return nullptr;
}

template <int CM, int MODE, typename R>
struct MergedBuilds {
    static constexpr void (*narrow)(MergedClasses<R>) = node_kernel_merged<CM, MODE, R>;
    static constexpr void (*wide)(MergedClasses<R>) = node_kernel_merged_wide<CM, MODE, R>;
};

static int no_generic_build(int chi, int threads) {
    if (chi > 32) return set_error(BQA_ERR_UNSUPPORTED, "node kernel: bond dim %d > 32", chi);
    return set_error(BQA_ERR_UNSUPPORTED, "node kernel: no %d-thread build at bond dim %d (above 256 threads: bond "
                     "dims <= 8, BP and open-bond passes)", threads, chi);
}

static bool valid_cta(int threads) { return threads >= 32 && threads <= 1024 && threads % 32 == 0; }

// One launch of the generic shared-memory node kernel (any degree and bond dim <= 32 whose
// node fits) over classes args[0..n) (counts[c] nodes each, same bond dim); threads = 0 takes
// the largest generic_threads of the classes.
template <int MODE, typename R>
static int launch_node_generic_merged(const NodeArgs<R>* args, const int* counts, int n, cudaStream_t st,
                                      int threads = 0) {
    const int chi = args[0].chi;
    MergedClasses<R> m;
    m.n = n;
    m.first[0] = 0;
    size_t smem = 0;
    int own = 32;
    for (int c = 0; c < n; ++c) {
        m.cls[c] = args[c];
        m.first[c + 1] = m.first[c] + counts[c];
        smem = std::max(smem, node_smem_elems(args[c].d, chi) * sizeof(typename Cx<R>::T));
        own = std::max(own, generic_threads(args[c].d, chi, MODE, sizeof(typename Cx<R>::T)));
    }
    if (threads == 0) threads = own;
    if (!valid_cta(threads)) return set_error(BQA_ERR_ARG, "node kernel: %d threads per CTA", threads);
    void (*kern)(MergedClasses<R>) = generic_build<MergedClasses<R>, MODE, R, MergedBuilds>(chi, threads);
    if (!kern) return no_generic_build(chi, threads);
    int rc = ensure_smem((const void*)kern, smem, "node kernel");
    if (rc) return rc;
    kern<<<m.first[n], threads, smem, st>>>(m);
    return check_launch("node kernel");
}

// the generic kernel over one class
template <int MODE, typename R>
static int launch_node_generic(const NodeArgs<R>& args, int count, cudaStream_t st, int threads = 0) {
    return launch_node_generic_merged<MODE, R>(&args, &count, 1, st, threads);
}

// the generic kernel's classes of a sweep go out in one launch unless BQA_GB300_MERGE_CLASSES=0
// was set when the library loaded (then one launch per class; the outputs are the same bits)
static const bool g_merge_classes = [] {
    const char* v = getenv("BQA_GB300_MERGE_CLASSES");
    return !(v && v[0] == '0');
}();

// a register-tiled complex64 kernel exists for (d, chi) (the pairs of try_tiled)
static bool tiled_covers(int d, int chi) {
    return (d == 2 && (chi == 8 || chi == 12 || chi == 16)) ||
           (d == 3 && (chi == 4 || chi == 8 || chi == 12 || chi == 16)) || (d == 4 && (chi == 4 || chi == 8));
}

template <int MODE, typename R>
static int launch_node_mode(const NodeArgs<R>& args, int count, cudaStream_t st) {
    if constexpr (sizeof(R) == 4 && (MODE == MODE_BP || MODE == MODE_EXT || MODE == MODE_DENS)) {
        if (g_use_tiled) {
            int rc = BQA_OK;
            if (try_tiled<MODE>(args, count, st, &rc)) return rc;
        }
    }
    return launch_node_generic<MODE, R>(args, count, st);
}

template <int MODE, typename R>
static int launch_merged_mode(const NodeArgs<R>* args, const int* counts, int n, cudaStream_t st, int threads) {
    return launch_node_generic_merged<MODE, R>(args, counts, n, st, threads);
}

// packed sweeps: generic-kernel classes of one (degree, bond dim, CTA size), any jobs
template <int MODE, typename R>
static int launch_generic_packed(const PackEntry* e, int n, cudaStream_t st) {
    NodeArgs<R> a[kMaxMergedClasses];
    int cnt[kMaxMergedClasses];
    const int threads = 32 * (e[0].key >> 16);
    for (int i0 = 0; i0 < n; i0 += kMaxMergedClasses) {
        const int m = std::min(kMaxMergedClasses, n - i0);
        for (int c = 0; c < m; ++c) {
            std::memcpy(&a[c], e[i0 + c].args, sizeof(NodeArgs<R>));
            cnt[c] = e[i0 + c].count;
        }
        const int rc = launch_node_generic_merged<MODE, R>(a, cnt, m, st, threads);
        if (rc) return rc;
    }
    return BQA_OK;
}

// grouping key of a packed generic class: CTA size (warps; 0 = own), degree, bond dim
template <typename R>
static int key_of(const NodeArgs<R>& a, int threads) { return ((threads / 32) << 16) | (a.d << 8) | a.chi; }

// Every class of a sweep (or pass) with the kernel it needs: the global-memory form for node
// tensors beyond shared memory, the register-tiled kernel where one exists (allow_tiled), and
// the generic kernel for the rest -- those in one launch (launch_node_generic_merged).
template <typename R>
static int run_classes(int mode, const bqa_class* classes, int n_classes, int chi, const void* msgs_a, void* msgs_b,
                       void* out, void* dist_parts, const int32_t* loop_state, double ztime, cudaStream_t st,
                       bool allow_tiled = true, const int* cta_threads = nullptr) {
    using C = typename Cx<R>::T;
    if (!classes || n_classes < 0 || chi < 1) return set_error(BQA_ERR_ARG, "bad class list or bond dim");
    NodeArgs<R> gen[kMaxMergedClasses];
    int gen_count[kMaxMergedClasses];
    int n_gen = 0;
    int gen_threads = 0;   // CTA size chosen for the pending classes (0: their own)
    auto flush = [&]() -> int {
        int rc = BQA_OK;
        if (n_gen == 0) return rc;
        switch (mode) {
            case MODE_BP: rc = launch_merged_mode<MODE_BP, R>(gen, gen_count, n_gen, st, gen_threads); break;
            case MODE_EXT: rc = launch_merged_mode<MODE_EXT, R>(gen, gen_count, n_gen, st, gen_threads); break;
            case MODE_PSPLIT: rc = launch_merged_mode<MODE_PSPLIT, R>(gen, gen_count, n_gen, st, gen_threads); break;
            default: rc = launch_merged_mode<MODE_DENS, R>(gen, gen_count, n_gen, st, gen_threads); break;
        }
        n_gen = 0;
        return rc;
    };
    // A class joins the pending launch when that costs no class an extra wave: with the
    // launch's shared memory and threads (the largest of its classes) every class still has
    // its solo occupancy, or its nodes fit in one wave of the merged kernel anyway.  Density
    // passes merge only classes of equal thread counts (their block sums then add in the same
    // order as in a launch of their own).
    const int sms = sm_count();
    auto occupancy = [](size_t smem, int threads) {
        const int by_smem = (int)((228u * 1024u) / (smem + 1024u));
        return std::max(1, std::min(std::min(by_smem, 2048 / threads), 32));
    };
    auto joins = [&](const NodeArgs<R>& a, int count, int want) {
        if (n_gen == 0) return true;
        if (n_gen == kMaxMergedClasses || want != gen_threads) return false;
        auto own = [&](int d) { return want ? want : generic_threads(d, chi, mode, sizeof(C)); };
        const size_t es = sizeof(C);
        size_t smem = node_smem_elems(a.d, chi) * es;
        int threads = own(a.d);
        for (int c = 0; c < n_gen; ++c) {
            if (mode == MODE_DENS && own(gen[c].d) != own(a.d)) return false;
            smem = std::max(smem, node_smem_elems(gen[c].d, chi) * es);
            threads = std::max(threads, own(gen[c].d));
        }
        const int merged = occupancy(smem, threads);
        auto fine = [&](int d, int cnt) {
            return merged >= occupancy(node_smem_elems(d, chi) * es, own(d)) || (int64_t)cnt <= (int64_t)merged * sms;
        };
        if (!fine(a.d, count)) return false;
        for (int c = 0; c < n_gen; ++c)
            if (!fine(gen[c].d, gen_count[c])) return false;
        return true;
    };
    for (int c = 0; c < n_classes; ++c) {
        const bqa_class& k = classes[c];
        if (k.count <= 0) continue;
        if (k.degree == 0 && mode != MODE_DENS) continue;
        const bool global = node_smem_elems(k.degree, chi) * sizeof(C) > kMaxSmem;
        NodeArgs<R> a;
        a.tensors = static_cast<const C*>(k.tensor);
        a.in_pos = k.in_pos;
        a.out_pos = k.out_pos;
        a.node_ids = k.node_ids;
        a.edge_ampl = k.edge_ampl;
        a.d = k.degree;
        a.chi = chi;
        a.msgs_a = static_cast<const C*>(msgs_a);
        a.msgs_b = static_cast<C*>(msgs_b);
        a.out = static_cast<C*>(out);
        a.loop_state = loop_state;
        a.dist_parts = static_cast<typename Cx<R>::Bits*>(dist_parts);
        a.ztime = ztime;
        int rc = BQA_OK;
        const int want = cta_threads ? cta_threads[c] : 0;   // generic kernel's CTA size (0: its own)
        const bool tiled = allow_tiled && sizeof(R) == 4 && g_use_tiled && mode != MODE_PSPLIT &&
                           tiled_covers(k.degree, chi);
        if (global) {
            switch (mode) {
                case MODE_BP: rc = launch_node_global<MODE_BP>(a, k.count, k.scratch, k.scratch_elems, st); break;
                case MODE_EXT: rc = launch_node_global<MODE_EXT>(a, k.count, k.scratch, k.scratch_elems, st); break;
                case MODE_PSPLIT:
                    rc = launch_node_global<MODE_PSPLIT>(a, k.count, k.scratch, k.scratch_elems, st);
                    break;
                default: rc = launch_node_global<MODE_DENS>(a, k.count, k.scratch, k.scratch_elems, st); break;
            }
        } else if (tiled) {
            switch (mode) {
                case MODE_BP: rc = launch_node_mode<MODE_BP>(a, k.count, st); break;
                case MODE_EXT: rc = launch_node_mode<MODE_EXT>(a, k.count, st); break;
                default: rc = launch_node_mode<MODE_DENS>(a, k.count, st); break;
            }
        } else if (g_pack) {   // packed sweep: merged with the same (degree, bond dim, CTA size) of other jobs
            const int key = key_of(a, want);
            switch (mode) {
                case MODE_BP: pack_record(launch_generic_packed<MODE_BP, R>, 0, key, k.count, a); break;
                case MODE_EXT: pack_record(launch_generic_packed<MODE_EXT, R>, 0, key, k.count, a); break;
                case MODE_PSPLIT: pack_record(launch_generic_packed<MODE_PSPLIT, R>, 0, key, k.count, a); break;
                default: pack_record(launch_generic_packed<MODE_DENS, R>, 0, key, k.count, a); break;
            }
        } else {
            if (!g_merge_classes || !joins(a, k.count, want)) rc = flush();
            if (rc) return rc;
            gen[n_gen] = a;
            gen_count[n_gen] = k.count;
            gen_threads = want;
            ++n_gen;
        }
        if (rc) return rc;
    }
    return flush();
}

static int run_classes_dt(int dtype, int mode, const bqa_class* classes, int n_classes, int chi, const void* msgs_a,
                          void* msgs_b, void* out, void* dist_parts, const int32_t* loop_state, double ztime,
                          cudaStream_t st, bool allow_tiled = true, const int* cta_threads = nullptr) {
    if (dtype == BQA_C64)
        return run_classes<float>(mode, classes, n_classes, chi, msgs_a, msgs_b, out, dist_parts, loop_state, ztime, st,
                                  allow_tiled, cta_threads);
    if (dtype == BQA_C128)
        return run_classes<double>(mode, classes, n_classes, chi, msgs_a, msgs_b, out, dist_parts, loop_state, ztime, st,
                                   allow_tiled, cta_threads);
    return set_error(BQA_ERR_ARG, "unknown dtype %d", dtype);
}

// ---- BP loop control -------------------------------------------------------------------------

template <typename R>
__device__ __forceinline__ void bp_decide(typename Cx<R>::Bits* parts, int32_t* ls, double eps, double damping,
                                          int max_iters) {
    ls[4] = 0;
    if (ls[0]) return;
    const R num = sqrt(bits_to_real(parts[0]));
    const R den = sqrt(bits_to_real(parts[1]));
    parts[0] = 0;
    parts[1] = 0;
    const R dist = num / den;
    const int sweeps = ls[1] + 1;
    ls[1] = sweeps;
    ls[5] = __float_as_int((float)dist);
    const float best = sweeps == 1 ? (float)dist : fminf(__int_as_float(ls[6]), (float)dist);
    ls[6] = __float_as_int(best);
    if (dist < eps) { ls[0] = 1; return; }                  // keep the sweep's input
    if (sweeps >= max_iters) { ls[0] = 1; ls[3] = 1; ls[2] ^= 1; return; }  // raw last output
    if (damping == 0.0) ls[2] ^= 1;
    else ls[4] = 1;
}

template <typename R>
__global__ void bp_decide_kernel(typename Cx<R>::Bits* parts, int32_t* ls, double eps, double damping, int max_iters) {
    bp_decide<R>(parts, ls, eps, damping, max_iters);
}

template <typename R>
struct DecideArgs {
    typename Cx<R>::Bits* parts;
    int32_t* ls;
    double eps, damping;
    int max_iters;
};

template <typename R>
struct MergedDecide {
    DecideArgs<R> job[kMaxMergedClasses];
    int n;
};

// the decisions of several jobs' BP runs: thread t decides job t
template <typename R>
__global__ void bp_decide_kernel_merged(const __grid_constant__ MergedDecide<R> m) {
    const int t = threadIdx.x;
    if (t < m.n) bp_decide<R>(m.job[t].parts, m.job[t].ls, m.job[t].eps, m.job[t].damping, m.job[t].max_iters);
}

template <typename R>
static int launch_decide_packed(const PackEntry* e, int n, cudaStream_t st) {
    for (int i0 = 0; i0 < n; i0 += kMaxMergedClasses) {
        MergedDecide<R> m;
        m.n = std::min(kMaxMergedClasses, n - i0);
        for (int c = 0; c < m.n; ++c) std::memcpy(&m.job[c], e[i0 + c].args, sizeof(DecideArgs<R>));
        bp_decide_kernel_merged<R><<<1, 32, 0, st>>>(m);
        const int rc = check_launch("bp_decide (merged)");
        if (rc) return rc;
    }
    return BQA_OK;
}

template <typename R>
__global__ void bp_damp_kernel(typename Cx<R>::T* a, typename Cx<R>::T* b, int64_t n, const int32_t* ls, R damping) {
    using C = typename Cx<R>::T;
    if (!ls[4]) return;
    C* cur = ls[2] ? b : a;
    const C* nw = ls[2] ? a : b;
    const R keep = damping, take = R(1) - damping;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const C x = cur[i], y = nw[i];
        cur[i] = c_make(fma(take, y.x, keep * x.x), fma(take, y.y, keep * x.y));
    }
}

// msgs[e] = diag(lam[e % half][0..dim)) / sum(lam)   (src/bqa/state.py:56-57)
template <typename R>
__global__ void msgs_from_lmbds_kernel(const R* lam, int stride, int E, int dim, typename Cx<R>::T* msgs) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= E) return;
    const R* l = lam + (size_t)(warp % (E / 2)) * stride;
    R s = 0;
    for (int i = lane; i < dim; i += 32) s += l[i];
    s = warp_sum(s);
    const R inv = R(1) / s;
    auto* m = msgs + (size_t)warp * dim * dim;
    for (int o = lane; o < dim * dim; o += 32) {
        const int i = o / dim, j = o - i * dim;
        m[o] = c_make(i == j ? l[i] * inv : R(0), R(0));
    }
}

// <Z_u Z_v> = Re( sum Z^u Z^v / sum S^u S^v ), S = P0 + P1, Z = P0 - P1 (oracle edge_zz)
template <typename R>
__global__ void edge_zz_kernel(const typename Cx<R>::T* pm, int E, int chi, double* zz) {
    using C = typename Cx<R>::T;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int half = E / 2;
    if (warp >= half) return;
    const int n2 = chi * chi;
    const C* pu = pm + (size_t)warp * 2 * n2;
    const C* pv = pm + (size_t)(warp + half) * 2 * n2;
    double nr = 0, ni = 0, dr = 0, di = 0;
    for (int i = lane; i < n2; i += 32) {
        const C u0 = pu[i], u1 = pu[n2 + i], v0 = pv[i], v1 = pv[n2 + i];
        const C zu = c_sub(u0, u1), zv = c_sub(v0, v1), su = c_add(u0, u1), sv = c_add(v0, v1);
        nr += (double)zu.x * zv.x - (double)zu.y * zv.y;
        ni += (double)zu.x * zv.y + (double)zu.y * zv.x;
        dr += (double)su.x * sv.x - (double)su.y * sv.y;
        di += (double)su.x * sv.y + (double)su.y * sv.x;
    }
    nr = warp_sum(nr); ni = warp_sum(ni); dr = warp_sum(dr); di = warp_sum(di);
    if (lane == 0) zz[warp] = (nr * dr + ni * di) / (dr * dr + di * di);
}

// lam[row][c] = 0 for dim <= c < stride: drops spectrum columns a truncation removed
template <typename R>
__global__ void lmbds_truncate_kernel(R* lam, int stride, int rows, int dim) {
    const int w = stride - dim;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)rows * w;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / w), c = dim + (int)(i - (int64_t)r * w);
        lam[(size_t)r * stride + c] = R(0);
    }
}

template <typename R>
static int launch_damp(void* a, void* b, int64_t n, const int32_t* ls, double damping, cudaStream_t st) {
    using C = typename Cx<R>::T;
    int blocks = (int)((n + 255) / 256);
    blocks = blocks > 4 * 152 * 8 ? 4 * 152 * 8 : blocks;
    bp_damp_kernel<R><<<blocks, 256, 0, st>>>(static_cast<C*>(a), static_cast<C*>(b), n, ls, (R)damping);
    return check_launch("bp_damp");
}

struct DampArgs {
    void* a;
    void* b;
    int64_t n;
    const int32_t* ls;
    double damping;
};

template <typename R>
static int launch_damp_solo(const PackEntry* e, int n, cudaStream_t st) {
    for (int i = 0; i < n; ++i) {
        DampArgs x;
        std::memcpy(&x, e[i].args, sizeof(x));
        const int rc = launch_damp<R>(x.a, x.b, x.n, x.ls, x.damping, st);
        if (rc) return rc;
    }
    return BQA_OK;
}

template <typename R>
static int finalize(void* a, void* b, int64_t n, void* parts, int32_t* ls, double eps, double damping, int max_iters,
                    cudaStream_t st) {
    using Bits = typename Cx<R>::Bits;
    if (pack_record(launch_decide_packed<R>, 2, 0, 0, DecideArgs<R>{static_cast<Bits*>(parts), ls, eps, damping,
                                                                     max_iters})) {
        if (damping != 0.0 && n != 0) pack_record(launch_damp_solo<R>, 3, 0, 0, DampArgs{a, b, n, ls, damping});
        return BQA_OK;
    }
    bp_decide_kernel<R><<<1, 1, 0, st>>>(static_cast<Bits*>(parts), ls, eps, damping, max_iters);
    int rc = check_launch("bp_decide");
    if (rc || damping == 0.0 || n == 0) return rc;
    return launch_damp<R>(a, b, n, ls, damping, st);
}

template <typename R>
static NodeArgs<R> class_args(const bqa_class& k, int chi, const void* msgs_a, void* msgs_b, void* out,
                              void* dist_parts, const int32_t* loop_state) {
    using C = typename Cx<R>::T;
    NodeArgs<R> a;
    a.tensors = static_cast<const C*>(k.tensor);
    a.in_pos = k.in_pos;
    a.out_pos = k.out_pos;
    a.node_ids = k.node_ids;
    a.edge_ampl = k.edge_ampl;
    a.d = k.degree;
    a.chi = chi;
    a.msgs_a = static_cast<const C*>(msgs_a);
    a.msgs_b = static_cast<C*>(msgs_b);
    a.out = static_cast<C*>(out);
    a.loop_state = loop_state;
    a.dist_parts = static_cast<typename Cx<R>::Bits*>(dist_parts);
    a.ztime = 0.0;
    return a;
}

template <typename R>
static int launch_bp_combine_t(const void* pm, int edges, int chi, void* msgs_a, void* msgs_b,
                               const int32_t* loop_state, void* dist_parts, cudaStream_t st) {
    using C = typename Cx<R>::T;
    const CombineArgs<R> x{static_cast<const C*>(pm), edges, chi, static_cast<const C*>(msgs_a), static_cast<C*>(msgs_b),
                           loop_state, static_cast<typename Cx<R>::Bits*>(dist_parts)};
    const int blocks = (int)(((int64_t)edges * 32 + 255) / 256);
    if (pack_record(launch_combine_packed<R>, 1, 0, blocks, x)) return BQA_OK;
    bp_combine_kernel<R><<<blocks, 256, 0, st>>>(x);
    return check_launch("bp_combine");
}

static int launch_bp_combine(int dtype, const void* pm, int edges, int chi, void* msgs_a, void* msgs_b,
                             const int32_t* loop_state, void* dist_parts, cudaStream_t st) {
    return dtype == BQA_C64
               ? launch_bp_combine_t<float>(pm, edges, chi, msgs_a, msgs_b, loop_state, dist_parts, st)
               : launch_bp_combine_t<double>(pm, edges, chi, msgs_a, msgs_b, loop_state, dist_parts, st);
}

}  // namespace bqa

using namespace bqa;

extern "C" {

int32_t bqa_max_bond_dim(int32_t degree, int32_t dtype) {
    if (degree < 0 || (dtype != BQA_C64 && dtype != BQA_C128)) return 0;
    const size_t el = dtype == BQA_C64 ? 8 : 16;
    int best = 0;
    // the largest bond dim whose node tensors the message kernels hold in shared memory
    // (beyond it they run on caller scratch, see bqa_node_scratch_elems; the simple update's
    // Jacobi SVDs take 2chi <= 64)
    for (int chi = 1; chi <= 32; ++chi)
        if (node_smem_elems(degree, chi) * el <= kMaxSmem) best = chi;
    return best;
}

int64_t bqa_node_scratch_elems(int32_t degree, int32_t chi, int32_t dtype) {
    if (degree < 0 || chi < 1 || (dtype != BQA_C64 && dtype != BQA_C128)) return 0;
    const size_t el = dtype == BQA_C64 ? 8 : 16;
    const bool msg_fits = node_smem_elems(degree, chi) * el <= kMaxSmem;
    const bool upd_fits = apply_smem_bytes(degree, chi, el) <= kMaxSmem;
    if (msg_fits && upd_fits) return 0;
    // message kernels: one work tensor 2 chi^d; update: two 2 chi^d buffers
    return 4 * (int64_t)ipow(chi, degree);
}

int32_t bqa_bp_sweep(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, void* msgs_a,
                     void* msgs_b, void* dist_parts, const int32_t* loop_state, void* stream) {
    if (!msgs_a || !msgs_b || !dist_parts) return set_error(BQA_ERR_ARG, "bqa_bp_sweep: null buffer");
    return run_classes_dt(dtype, MODE_BP, classes, n_classes, chi, msgs_a, msgs_b, nullptr, dist_parts, loop_state, 0.0,
                          as_stream(stream));
}

int32_t bqa_bp_sweep_split(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, void* msgs_a,
                           void* msgs_b, void* pm, int32_t edges, void* dist_parts, const int32_t* loop_state,
                           void* stream) {
    if (!classes || n_classes < 0 || chi < 1 || !msgs_a || !msgs_b || !pm || !dist_parts || edges < 2)
        return set_error(BQA_ERR_ARG, "bqa_bp_sweep_split: bad argument");
    if (dtype != BQA_C64 && dtype != BQA_C128) return set_error(BQA_ERR_ARG, "bqa_bp_sweep_split: unknown dtype %d", dtype);
    cudaStream_t st = as_stream(stream);
    std::vector<bqa_class> rest;
    for (int c = 0; c < n_classes; ++c) {
        const bqa_class& k = classes[c];
        if (k.count <= 0 || k.degree == 0) continue;
        int rc = BQA_OK;
        if (dtype == BQA_C64 && g_use_tiled) {
            NodeArgs<float> a;
            a.tensors = static_cast<const float2*>(k.tensor);
            a.in_pos = k.in_pos; a.out_pos = k.out_pos; a.node_ids = k.node_ids; a.edge_ampl = k.edge_ampl;
            a.d = k.degree; a.chi = chi;
            a.msgs_a = static_cast<const float2*>(msgs_a); a.msgs_b = static_cast<float2*>(msgs_b);
            a.out = static_cast<float2*>(pm); a.loop_state = loop_state; a.dist_parts = nullptr; a.ztime = 0.0;
            if (try_half(a, k.count, st, &rc)) {
                if (rc) return rc;
                continue;
            }
        }
        rest.push_back(k);
    }
    if (!rest.empty()) {   // classes without a half-node kernel: their open-bond blocks in one pass
        const int rc = run_classes_dt(dtype, MODE_PSPLIT, rest.data(), (int)rest.size(), chi, msgs_a, msgs_b, pm,
                                      nullptr, loop_state, 0.0, st);
        if (rc) return rc;
    }
    return launch_bp_combine(dtype, pm, edges, chi, msgs_a, msgs_b, loop_state, dist_parts, st);
}

int32_t bqa_bp_sweep_plan(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype,
                          const int32_t* variants, void* msgs_a, void* msgs_b, void* pm, int32_t edges,
                          void* dist_parts, const int32_t* loop_state, void* stream) {
    if (!variants)
        return pm ? bqa_bp_sweep_split(classes, n_classes, chi, dtype, msgs_a, msgs_b, pm, edges, dist_parts,
                                       loop_state, stream)
                  : bqa_bp_sweep(classes, n_classes, chi, dtype, msgs_a, msgs_b, dist_parts, loop_state, stream);
    if (!classes || n_classes < 0 || chi < 1 || !msgs_a || !msgs_b || !dist_parts || (pm && edges < 2))
        return set_error(BQA_ERR_ARG, "bqa_bp_sweep_plan: bad argument");
    if (dtype != BQA_C64 && dtype != BQA_C128) return set_error(BQA_ERR_ARG, "bqa_bp_sweep_plan: unknown dtype %d", dtype);
    cudaStream_t st = as_stream(stream);
    std::vector<bqa_class> def_rest, gen_rest;   // classes of the generic kernel: one launch each list
    std::vector<int> gen_threads;                 // their CTA sizes (0: the kernel's own)
    for (int c = 0; c < n_classes; ++c) {
        const bqa_class& k = classes[c];
        if (k.count <= 0 || k.degree == 0) continue;
        const int v = variants[c] & 0xff, warps = (variants[c] >> 8) & 0xff;
        if (v < BQA_VARIANT_DEFAULT || v > BQA_VARIANT_MIXED || (variants[c] >> 16) != 0 || warps > 32 ||
            (warps && v != BQA_VARIANT_GENERIC))
            return set_error(BQA_ERR_ARG, "bqa_bp_sweep_plan: unknown variant %d", variants[c]);
        int rc = BQA_OK;
        if (v == BQA_VARIANT_TENSOR || v == BQA_VARIANT_TENSOR_BF16 || v == BQA_VARIANT_MIXED) {
            if (dtype != BQA_C64 || !pm || k.degree != 3 || chi != 16)
                return set_error(BQA_ERR_UNSUPPORTED, "bqa_bp_sweep_plan: the tensor-core kernels serve the two-stage "
                                 "complex64 sweep of degree 3 at bond dim 16 (got degree %d, bond dim %d)", k.degree, chi);
            const NodeArgs<float> ca = class_args<float>(k, chi, msgs_a, msgs_b, pm, nullptr, loop_state);
            if (v == BQA_VARIANT_TENSOR) {
                rc = launch_tc_half(ca, k.count, st);
            } else if (v == BQA_VARIANT_TENSOR_BF16) {
                rc = launch_tcb_half<false>(ca, k.count, st);
            } else {
                // the BF16 kernel takes the low-precision sweeps, the default FP32-accurate kernel
                // (2xFP16 tensor cores, or the CUDA cores with BQA_GB300_TC=0) the others
                rc = launch_tcb_half<true>(ca, k.count, st);
                if (!rc) {
                    NodeArgs<float> cb = ca;
                    cb.mixed_role = 2;
                    cb.mixed_switch = g_mixed_switch;
                    rc = g_use_tc ? launch_tcx_half(cb, k.count, st)
                                  : (g_use_specialized ? launch_half_k<3, 16, true>(cb, k.count, st)
                                                       : launch_half_k<3, 16, false>(cb, k.count, st));
                }
            }
        } else if (v == BQA_VARIANT_TILED && pm && dtype == BQA_C64 && k.degree == 3 && chi == 16) {
            // the CUDA-core half-node kernel, whatever the default (3, 16) kernel is
            rc = g_use_specialized
                     ? launch_half_k<3, 16, true>(class_args<float>(k, chi, msgs_a, msgs_b, pm, nullptr, loop_state),
                                                  k.count, st)
                     : launch_half_k<3, 16, false>(class_args<float>(k, chi, msgs_a, msgs_b, pm, nullptr, loop_state),
                                                   k.count, st);
        } else if (v == BQA_VARIANT_DEFAULT) {
            // the kernel bqa_bp_sweep_split / bqa_bp_sweep would launch for this class
            int hit = 0;
            if (pm && dtype == BQA_C64 && g_use_tiled) {
                NodeArgs<float> a = class_args<float>(k, chi, msgs_a, msgs_b, pm, nullptr, loop_state);
                hit = try_half(a, k.count, st, &rc);
            }
            if (!hit) def_rest.push_back(k);
        } else if (v == BQA_VARIANT_TILED) {
            if (dtype != BQA_C64)
                return set_error(BQA_ERR_UNSUPPORTED, "bqa_bp_sweep_plan: no register-tiled complex128 kernel");
            NodeArgs<float> a = class_args<float>(k, chi, msgs_a, msgs_b, pm, pm ? nullptr : dist_parts, loop_state);
            const int hit = pm ? try_half(a, k.count, st, &rc) : try_tiled<MODE_BP>(a, k.count, st, &rc);
            if (!hit)
                return set_error(BQA_ERR_UNSUPPORTED, "bqa_bp_sweep_plan: no register-tiled kernel for degree %d, "
                                 "bond dim %d", k.degree, chi);
        } else {
            gen_rest.push_back(k);   // the generic kernel (global-memory form beyond shared memory)
            gen_threads.push_back(32 * warps);
        }
        if (rc) return rc;
    }
    const int mode = pm ? MODE_PSPLIT : MODE_BP;
    void* out = pm ? pm : nullptr;
    void* dist = pm ? nullptr : dist_parts;
    if (!def_rest.empty()) {
        const int rc = run_classes_dt(dtype, mode, def_rest.data(), (int)def_rest.size(), chi, msgs_a, msgs_b, out, dist,
                                      loop_state, 0.0, st);
        if (rc) return rc;
    }
    if (!gen_rest.empty()) {
        const int rc = run_classes_dt(dtype, mode, gen_rest.data(), (int)gen_rest.size(), chi, msgs_a, msgs_b, out, dist,
                                      loop_state, 0.0, st, false, gen_threads.data());
        if (rc) return rc;
    }
    return pm ? launch_bp_combine(dtype, pm, edges, chi, msgs_a, msgs_b, loop_state, dist_parts, st) : BQA_OK;
}

int32_t bqa_tc_faults(int32_t* out, int32_t reset, void* stream) {
    if (!out) return set_error(BQA_ERR_ARG, "bqa_tc_faults: null output");
    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaMemcpyFromSymbolAsync(out, g_tc_faults, sizeof(int32_t), 0, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && reset) {
        static const int32_t zero = 0;
        e = cudaMemcpyToSymbolAsync(g_tc_faults, &zero, sizeof(int32_t), 0, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) return set_error(BQA_ERR_CUDA, "bqa_tc_faults: %s", cudaGetErrorString(e));
    return BQA_OK;
}

int32_t bqa_bp_finalize(void* msgs_a, void* msgs_b, int64_t msg_elems, int32_t dtype, void* dist_parts,
                        int32_t* loop_state, double eps, double damping, int32_t max_iters, void* stream) {
    if (!msgs_a || !msgs_b || !dist_parts || !loop_state || msg_elems < 0 || max_iters < 1)
        return set_error(BQA_ERR_ARG, "bqa_bp_finalize: bad argument");
    cudaStream_t st = as_stream(stream);
    if (dtype == BQA_C64) return finalize<float>(msgs_a, msgs_b, msg_elems, dist_parts, loop_state, eps, damping, max_iters, st);
    if (dtype == BQA_C128) return finalize<double>(msgs_a, msgs_b, msg_elems, dist_parts, loop_state, eps, damping, max_iters, st);
    return set_error(BQA_ERR_ARG, "bqa_bp_finalize: unknown dtype %d", dtype);
}

int32_t bqa_ext_msgs(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs,
                     void* ext_out, double ztime, void* stream) {
    if (!msgs || !ext_out) return set_error(BQA_ERR_ARG, "bqa_ext_msgs: null buffer");
    return run_classes_dt(dtype, MODE_EXT, classes, n_classes, chi, msgs, nullptr, ext_out, nullptr, nullptr, ztime,
                          as_stream(stream));
}

int32_t bqa_ext_msgs_split(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs,
                           void* pm, int32_t edges, const double* edge_j, double ztime, void* ext_out, void* stream) {
    if (!classes || n_classes < 0 || chi < 1 || !msgs || !pm || !edge_j || !ext_out || edges < 2 || edges % 2)
        return set_error(BQA_ERR_ARG, "bqa_ext_msgs_split: bad argument");
    if (dtype != BQA_C64 && dtype != BQA_C128) return set_error(BQA_ERR_ARG, "bqa_ext_msgs_split: unknown dtype %d", dtype);
    cudaStream_t st = as_stream(stream);
    std::vector<bqa_class> rest;
    for (int c = 0; c < n_classes; ++c) {
        const bqa_class& k = classes[c];
        if (k.count <= 0 || k.degree == 0) continue;
        int rc = BQA_OK;
        if (dtype == BQA_C64 && g_use_tiled) {
            NodeArgs<float> a;
            a.tensors = static_cast<const float2*>(k.tensor);
            a.in_pos = k.in_pos; a.out_pos = k.out_pos; a.node_ids = k.node_ids; a.edge_ampl = k.edge_ampl;
            a.d = k.degree; a.chi = chi;
            a.msgs_a = static_cast<const float2*>(msgs); a.msgs_b = nullptr;
            a.out = static_cast<float2*>(pm); a.loop_state = nullptr; a.dist_parts = nullptr; a.ztime = 0.0;
            if (try_half(a, k.count, st, &rc)) {
                if (rc) return rc;
                continue;
            }
        }
        rest.push_back(k);
    }
    if (!rest.empty()) {
        const int rc = run_classes_dt(dtype, MODE_PSPLIT, rest.data(), (int)rest.size(), chi, msgs, nullptr, pm,
                                      nullptr, nullptr, 0.0, st);
        if (rc) return rc;
    }
    return bqa_ext_combine(pm, edges, chi, dtype, edge_j, ztime, ext_out, stream);
}

int32_t bqa_ext_combine(const void* pm, int32_t edges, int32_t chi, int32_t dtype, const double* edge_j, double ztime,
                        void* ext_out, void* stream) {
    if (!pm || !edge_j || !ext_out || chi < 1 || edges < 2 || edges % 2)
        return set_error(BQA_ERR_ARG, "bqa_ext_combine: bad argument");
    cudaStream_t st = as_stream(stream);
    const int blocks = (int)(((int64_t)edges * 32 + 255) / 256);
    if (dtype == BQA_C64)
        ext_combine_kernel<float><<<blocks, 256, 0, st>>>(static_cast<const float2*>(pm), edges, chi, edge_j, ztime,
                                                           static_cast<float2*>(ext_out));
    else if (dtype == BQA_C128)
        ext_combine_kernel<double><<<blocks, 256, 0, st>>>(static_cast<const double2*>(pm), edges, chi, edge_j, ztime,
                                                            static_cast<double2*>(ext_out));
    else
        return set_error(BQA_ERR_ARG, "bqa_ext_combine: unknown dtype %d", dtype);
    return check_launch("ext_combine");
}

int32_t bqa_psplit(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs, void* pm,
                   void* stream) {
    if (!msgs || !pm) return set_error(BQA_ERR_ARG, "bqa_psplit: null buffer");
    return run_classes_dt(dtype, MODE_PSPLIT, classes, n_classes, chi, msgs, nullptr, pm, nullptr, nullptr, 0.0,
                          as_stream(stream));
}

int32_t bqa_densities(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs,
                      void* rho, void* stream) {
    if (!msgs || !rho) return set_error(BQA_ERR_ARG, "bqa_densities: null buffer");
    return run_classes_dt(dtype, MODE_DENS, classes, n_classes, chi, msgs, nullptr, rho, nullptr, nullptr, 0.0,
                          as_stream(stream));
}

int32_t bqa_msgs_from_lmbds(const void* lmbds, int32_t lam_stride, int32_t edges, int32_t dim, int32_t dtype,
                            void* msgs, void* stream) {
    if (!lmbds || !msgs || edges < 2 || dim < 1 || lam_stride < dim)
        return set_error(BQA_ERR_ARG, "bqa_msgs_from_lmbds: bad argument");
    const int blocks = (int)(((int64_t)edges * 32 + 255) / 256);
    cudaStream_t st = as_stream(stream);
    if (dtype == BQA_C64)
        msgs_from_lmbds_kernel<float><<<blocks, 256, 0, st>>>(static_cast<const float*>(lmbds), lam_stride, edges, dim,
                                                              static_cast<float2*>(msgs));
    else if (dtype == BQA_C128)
        msgs_from_lmbds_kernel<double><<<blocks, 256, 0, st>>>(static_cast<const double*>(lmbds), lam_stride, edges,
                                                               dim, static_cast<double2*>(msgs));
    else
        return set_error(BQA_ERR_ARG, "bqa_msgs_from_lmbds: unknown dtype %d", dtype);
    return check_launch("msgs_from_lmbds");
}

int32_t bqa_lmbds_truncate(void* lmbds, int32_t stride, int32_t rows, int32_t dim, int32_t dtype, void* stream) {
    if (!lmbds || rows < 0 || dim < 0 || stride < dim) return set_error(BQA_ERR_ARG, "bqa_lmbds_truncate: bad argument");
    if (rows == 0 || stride == dim) return BQA_OK;
    int blocks = (int)(((int64_t)rows * (stride - dim) + 255) / 256);
    blocks = blocks > 4096 ? 4096 : blocks;
    cudaStream_t st = as_stream(stream);
    if (dtype == BQA_C64)
        lmbds_truncate_kernel<float><<<blocks, 256, 0, st>>>(static_cast<float*>(lmbds), stride, rows, dim);
    else if (dtype == BQA_C128)
        lmbds_truncate_kernel<double><<<blocks, 256, 0, st>>>(static_cast<double*>(lmbds), stride, rows, dim);
    else
        return set_error(BQA_ERR_ARG, "bqa_lmbds_truncate: unknown dtype %d", dtype);
    return check_launch("lmbds_truncate");
}

int32_t bqa_edge_zz(const void* pm, int32_t edges, int32_t chi, int32_t dtype, double* zz, void* stream) {
    if (!pm || !zz || edges < 2 || chi < 1) return set_error(BQA_ERR_ARG, "bqa_edge_zz: bad argument");
    const int blocks = (int)(((int64_t)(edges / 2) * 32 + 255) / 256);
    cudaStream_t st = as_stream(stream);
    if (dtype == BQA_C64)
        edge_zz_kernel<float><<<blocks, 256, 0, st>>>(static_cast<const float2*>(pm), edges, chi, zz);
    else if (dtype == BQA_C128)
        edge_zz_kernel<double><<<blocks, 256, 0, st>>>(static_cast<const double2*>(pm), edges, chi, zz);
    else
        return set_error(BQA_ERR_ARG, "bqa_edge_zz: unknown dtype %d", dtype);
    return check_launch("edge_zz");
}

}  // extern "C"
