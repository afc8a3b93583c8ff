// Batched one-sided Jacobi SVD (Hestenes) for the truncation step of the simple update.
//
// A segment of W lanes (W = 8, 16 or 32, a power of two >= n) owns one n x n complex
// matrix, zero-padded to W x W: lane j keeps column j of A in registers; V is in shared
// memory.  A sweep visits every column pair once: in round r (1 <= r < W) lane j pairs with
// lane j ^ r, which is a perfect matching, and the W-1 rounds cover all pairs.  The pair's
// Gram entries alpha = |a_p|^2, beta = |a_q|^2, gamma = a_p^H a_q are the same bits on both
// lanes (each norm comes from its owner, gamma from sums formed with the same operand
// order), so both make the same rotation decision; the unitary rotation
//     a_p' = c a_p - s conj(e) a_q,   a_q' = c a_q + s e a_p,   e = gamma/|gamma|
// with t = sign(zeta)/(|zeta| + sqrt(1+zeta^2)), zeta = (beta-alpha)/(2|gamma|),
// c = 1/sqrt(1+t^2), s = c t, makes the pair orthogonal: a_p'^H a_q' =
// e ((c^2 - s^2)|gamma| - c s (beta - alpha)) = 0 (the complex form of Hestenes' method,
// Demmel & Veselic 1992).  At convergence A V = U Sigma with sigma_j = |a_j|.
// A pair is rotated if |gamma| > tol sqrt(alpha beta).  Sweeps stop when a whole sweep
// rotates no pair of SIGNIFICANT columns in the warp (both above the noise level of the
// matrix, |a|^2 > W eps^2 |A|_F^2), or at the sweep cap (then a status bit is set).
// Columns below that level are rounding noise (the remains of dependent columns): their
// mutual products never pass the relative test, so they would keep the loop going until
// the cap; they are still rotated like every other pair while the loop runs, so the
// orthogonalisation of the significant columns against them is untouched.
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace bqa {

constexpr int kMaxSweeps = 40;

template <typename R> __device__ __forceinline__ R jacobi_eps();
template <> __device__ __forceinline__ float jacobi_eps<float>() { return 1.2e-7f; }
template <> __device__ __forceinline__ double jacobi_eps<double>() { return 2.3e-16; }

template <typename C>
__device__ __forceinline__ C shfl_xor_c(C v, int r, int w) {
    v.x = __shfl_xor_sync(BQA_FULL_MASK, v.x, r, w);
    v.y = __shfl_xor_sync(BQA_FULL_MASK, v.y, r, w);
    return v;
}

// V lives in shared memory: column j of the segment's V at sV + j * VS, VS = W + 2 complex
// elements, so 128-bit loads of 8 lanes' columns hit 8 distinct bank groups.  A rotation
// updates the pair's two V columns in place: the lower lane of the pair rewrites rows
// [0, W/2) of both columns, the higher lane rows [W/2, W), so one block suffices and each
// round reads and writes every V element of a rotated pair once.
template <int W> struct VStride { static constexpr int VS = W + 2; static constexpr int BLOCK = W * VS; };

constexpr int NP = 4;  // partial sums per reduction over a column

template <int N, typename R>
__device__ __forceinline__ R sum_parts(const R (&p)[N]) {
    R s = p[0];
#pragma unroll
    for (int k = 1; k < N; ++k) s += p[k];
    return s;
}

// |a|^2 of this lane's column, in NP interleaved partial sums
template <int W, typename R>
__device__ __forceinline__ R col_norm2(const typename Cx<R>::T (&a)[W]) {
    R p[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) p[k] = R(0);
#pragma unroll
    for (int i = 0; i < W; ++i) p[i % NP] = fma(a[i].x, a[i].x, fma(a[i].y, a[i].y, p[i % NP]));
    return sum_parts<NP>(p);
}

// One-sided Jacobi on the segment's columns.  a: this lane's column (registers); sV: the
// segment's V block (shared), initialised to I here.  Returns whether it converged.
template <int W, typename R>
__device__ __forceinline__ bool jacobi_columns(typename Cx<R>::T (&a)[W], typename Cx<R>::T* sV, int lane) {
    using C = typename Cx<R>::T;
    constexpr int VS = VStride<W>::VS;
    constexpr int H = W / 2;
#pragma unroll
    for (int i = 0; i < W; ++i) sV[lane * VS + i] = c_make(i == lane ? R(1) : R(0), R(0));
    __syncwarp();
    const R tol = (R)W * jacobi_eps<R>();
    // |a_lane|^2, recomputed (same operation order) whenever the column changes; the pair's
    // norms come from their owners, so both lanes of a pair see the same alpha and beta
    R nown = col_norm2<W, R>(a);
    R fro2 = nown;
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) fro2 += __shfl_xor_sync(BQA_FULL_MASK, fro2, o, W);
    const R col_floor = fmax((R)W * jacobi_eps<R>() * jacobi_eps<R>() * fro2, sizeof(R) == 4 ? R(1e-30) : R(1e-280));
    // a sweep whose significant rotations all had |gamma| < sqrt(tol) sqrt(alpha beta) leaves the
    // pairs orthogonal to ~tol relative (the coupling it reintroduces is second order), so the
    // loop also ends after such a sweep instead of running one more sweep that rotates nothing
    const R big_tol = sqrt(tol);
    for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
        int rotated = 0, big = 0;
#pragma unroll 1
        for (int r = 1; r < W; ++r) {
            const int partner = lane ^ r;
            const bool low = lane < partner;
            const R npart = __shfl_xor_sync(BQA_FULL_MASK, nown, r, W);
            // gamma = p^H q (p = column of the lower lane, q = of the higher) from sums both
            // lanes form bit-identically: Sx = sum Re(conj(own) partner) and the cross sums
            // S1 = sum own.x partner.y, S2 = sum own.y partner.x (they swap roles on the
            // other lane; fma(a, b, c) == fma(b, a, c)).
            // NP independent partial sums per quantity (short dependency chains), combined in
            // a fixed order, so both lanes still form identical bits
            R sx[NP], s1[NP], s2[NP];
#pragma unroll
            for (int k = 0; k < NP; ++k) sx[k] = s1[k] = s2[k] = R(0);
#pragma unroll
            for (int i = 0; i < W; ++i) {
                const C o = shfl_xor_c(a[i], r, W);
                sx[i % NP] = fma(a[i].x, o.x, fma(a[i].y, o.y, sx[i % NP]));
                s1[i % NP] = fma(a[i].x, o.y, s1[i % NP]);
                s2[i % NP] = fma(a[i].y, o.x, s2[i % NP]);
            }
            const R sxs = sum_parts<NP>(sx), s1s = sum_parts<NP>(s1), s2s = sum_parts<NP>(s2);
            const R alpha = low ? nown : npart, beta = low ? npart : nown;
            const C g = c_make(sxs, low ? s1s - s2s : s2s - s1s);
            const R gabs = sqrt(c_abs2(g));
            const bool rot = alpha > R(0) && beta > R(0) && gabs > tol * sqrt(alpha) * sqrt(beta);
            if (__any_sync(BQA_FULL_MASK, rot)) {
                // p' = c p - s conj(e) q,  q' = c q + s e p  (wp = -s conj(e), wq = s e);
                // a lane that does not rotate keeps c = 1, w = 0, an exact no-op
                R c = R(1);
                C wp = c_zero<C>(), wq = c_zero<C>();
                if (rot) {
                    const R zeta = (beta - alpha) / (R(2) * gabs);
                    const R t = copysign(R(1), zeta) / (fabs(zeta) + hypot(R(1), zeta));
                    c = R(1) / sqrt(fma(t, t, R(1)));
                    const R sn = c * t;
                    const R ex = g.x / gabs, ey = g.y / gabs;
                    wp = c_make(-sn * ex, sn * ey);
                    wq = c_make(sn * ex, sn * ey);
                    const bool sig = alpha > col_floor && beta > col_floor;
                    rotated |= sig;
                    big |= sig && gabs >= big_tol * sqrt(alpha) * sqrt(beta);
                }
                const C wown = low ? wp : wq;
#pragma unroll
                for (int i = 0; i < W; ++i) {
                    const C o = shfl_xor_c(a[i], r, W);
                    a[i] = c_fma(wown, o, c_scale(a[i], c));
                }
                nown = col_norm2<W, R>(a);
                if (rot) {
                    // own column first, partner's second: in each access the two lanes of a
                    // pair touch different columns, so their half-column offsets (H rows =
                    // 128 bytes in complex64) do not fall in the same bank group
                    const C wpart = low ? wq : wp;
                    C* vo = sV + lane * VS + (low ? 0 : H);
                    C* vx = sV + partner * VS + (low ? 0 : H);
#pragma unroll
                    for (int i = 0; i < H; i += 2) {
                        C o0, o1, x0, x1;
                        if (sizeof(R) == 4) {
                            const float4 u = *reinterpret_cast<const float4*>(vo + i);
                            const float4 v = *reinterpret_cast<const float4*>(vx + i);
                            o0 = c_make((R)u.x, (R)u.y); o1 = c_make((R)u.z, (R)u.w);
                            x0 = c_make((R)v.x, (R)v.y); x1 = c_make((R)v.z, (R)v.w);
                        } else {
                            o0 = vo[i]; o1 = vo[i + 1]; x0 = vx[i]; x1 = vx[i + 1];
                        }
                        const C no0 = c_fma(wown, x0, c_scale(o0, c)), no1 = c_fma(wown, x1, c_scale(o1, c));
                        const C nx0 = c_fma(wpart, o0, c_scale(x0, c)), nx1 = c_fma(wpart, o1, c_scale(x1, c));
                        if (sizeof(R) == 4) {
                            *reinterpret_cast<float4*>(vo + i) = make_float4((float)no0.x, (float)no0.y, (float)no1.x, (float)no1.y);
                            *reinterpret_cast<float4*>(vx + i) = make_float4((float)nx0.x, (float)nx0.y, (float)nx1.x, (float)nx1.y);
                        } else {
                            vo[i] = no0; vo[i + 1] = no1; vx[i] = nx0; vx[i + 1] = nx1;
                        }
                    }
                }
                __syncwarp();
            }
        }
        if (!__any_sync(BQA_FULL_MASK, rotated) || !__any_sync(BQA_FULL_MASK, big)) return true;
    }
    return false;
}

template <int W, typename R>
__device__ __forceinline__ R seg_sum(R x) {
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) x += __shfl_xor_sync(BQA_FULL_MASK, x, o, W);
    return x;
}

// ---- QR preconditioning (Drmac & Veselic 2008: one-sided Jacobi on the triangular factor) ----
//
// One-sided Jacobi converges in far fewer sweeps on R^H, R from a QR factorisation with column
// pivoting of the matrix, than on the matrix itself: the pivoted R is graded (row norms
// decreasing down the diagonal), so R^H's columns are already nearly orthogonal.  For the
// environment matrices of a saturated anneal (spectra over nine decades) a float32 model of
// this kernel needs 4.9 sweeps instead of 10.7, and its eigenvectors are at least as accurate.
//   m = Q R'  (Householder, columns pivoted by their trailing norms; R' = R with its columns in
//              the original order, so m's column j stays in lane j and no columns move),
//   R'^H = m Q  (m is Hermitian), Jacobi: R'^H V_r = A with orthogonal columns, |a_j| = sigma_j,
//   so m (Q V_r) = A: the columns of E = Q V_r are m's eigenvectors and sigma_j its eigenvalues.
// E replaces the rotation accumulator V of the unpreconditioned kernel; being a product of
// unitaries it is unitary to working precision, like V.

// Shared memory of one segment beyond its V block: the Householder vectors u_k (rows k..W-1,
// packed: W(W+1)/2 complex) and their scales tau_k (W reals, padded to W complex).
template <int W> struct QrStride {
    static constexpr int H = W * (W + 1) / 2;
    static constexpr int BLOCK = VStride<W>::BLOCK + H + W;
};
template <int W> __device__ __forceinline__ int qr_off(int k) { return k * W - (k * (k - 1)) / 2; }
// Column remainders at or below this norm count as zero (|x| (|x| + |x_k|) stays a normal number).
template <typename R> __device__ __forceinline__ R qr_tiny();
template <> __device__ __forceinline__ float qr_tiny<float>() { return 1e-18f; }
template <> __device__ __forceinline__ double qr_tiny<double>() { return 1e-150; }

// a_k = this lane's element k (k a runtime index)
template <int W, typename C>
__device__ __forceinline__ C pick(const C (&a)[W], int k) {
    C x = a[0];
#pragma unroll
    for (int i = 1; i < W; ++i)
        if (i == k) x = a[i];
    return x;
}

// Householder QR with column pivoting of the segment's matrix (lane j holds column j in a),
// then the columns of R'^H into the lanes (lane k: conj of row k of R').  sV is used as the
// transposition buffer; sH / sTau receive the Householder vectors for qr_apply_q.
template <int W, typename R>
__device__ __forceinline__ void qr_precondition(typename Cx<R>::T (&a)[W], typename Cx<R>::T* sV,
                                                typename Cx<R>::T* sH, R* sTau, int lane) {
    using C = typename Cx<R>::T;
    constexpr int VS = VStride<W>::VS;
    bool done = false;
#pragma unroll 1
    for (int k = 0; k < W; ++k) {
        // trailing norm^2 of this lane's column (rows k..W-1); the pivot is the largest among the
        // lanes not pivoted yet, ties to the lowest lane, the same choice on every lane
        R t = R(0);
#pragma unroll
        for (int i = 0; i < W; ++i)
            if (i >= k) t = fma(a[i].x, a[i].x, fma(a[i].y, a[i].y, t));
        R best = done ? R(-1) : t;
        int bl = lane;
#pragma unroll
        for (int o = W / 2; o > 0; o >>= 1) {
            const R ob = __shfl_xor_sync(BQA_FULL_MASK, best, o, W);
            const int ol = __shfl_xor_sync(BQA_FULL_MASK, bl, o, W);
            if (ob > best || (ob == best && ol < bl)) { best = ob; bl = ol; }
        }
        C* u = sH + qr_off<W>(k);     // u[i - k], i = k..W-1
        if (lane == bl) {
            // x = column rows k..: alpha = -phase(x_k) |x|, u = (x - alpha e_k) / sqrt(|x| (|x| + |x_k|)),
            // so |u|^2 = 2 and H = I - u u^H (tau = 1).  A remainder below qr_tiny is dropped (tau = 0,
            // the column zeroed): the Jacobi would treat it as noise, and its reflector scale would
            // overflow.
            const R xn = sqrt(t);
            const C xk = pick<W>(a, k);
            const R ak = sqrt(c_abs2(xk));
            const C ph = ak > R(0) ? c_scale(xk, R(1) / ak) : c_make(R(1), R(0));
            const bool keep = xn > qr_tiny<R>();
            const R scale = keep ? R(1) / sqrt(xn * (xn + ak)) : R(0);
#pragma unroll
            for (int i = 0; i < W; ++i)
                if (i > k) u[i - k] = c_scale(a[i], scale);
            u[0] = c_scale(ph, (ak + xn) * scale);
            sTau[k] = keep ? R(1) : R(0);
            // the pivot column becomes alpha e_k
#pragma unroll
            for (int i = 0; i < W; ++i)
                if (i > k) a[i] = c_zero<C>();
            const C alpha = keep ? c_scale(ph, -xn) : c_zero<C>();
#pragma unroll
            for (int i = 0; i < W; ++i)
                if (i == k) a[i] = alpha;
        }
        __syncwarp();
        const R tau = sTau[k];
        if (!done && lane != bl && tau != R(0)) {
            // a <- a - tau u (u^H a)
            C w = c_zero<C>();
#pragma unroll
            for (int i = 0; i < W; ++i)
                if (i >= k) w = c_fma_conj(u[i - k], a[i], w);
            w = c_scale(w, tau);
#pragma unroll
            for (int i = 0; i < W; ++i)
                if (i >= k) a[i] = c_sub(a[i], c_mul(u[i - k], w));
        }
        done = done || lane == bl;
        __syncwarp();
    }
    // R'^H: lane k takes conj(R'[k][j]) for every j
#pragma unroll
    for (int i = 0; i < W; ++i) sV[lane * VS + i] = a[i];
    __syncwarp();
#pragma unroll
    for (int j = 0; j < W; ++j) a[j] = c_conj(sV[j * VS + lane]);
    __syncwarp();
}

// Column `lane` of sV (V_r after the Jacobi) <- Q V_r = H_0 H_1 ... H_{W-1} V_r.
template <int W, typename R>
__device__ __forceinline__ void qr_apply_q(typename Cx<R>::T* sV, const typename Cx<R>::T* sH, const R* sTau,
                                           int lane) {
    using C = typename Cx<R>::T;
    constexpr int VS = VStride<W>::VS;
    C e[W];
    C* col = sV + lane * VS;
#pragma unroll
    for (int i = 0; i < W; ++i) e[i] = col[i];
#pragma unroll 1
    for (int k = W - 1; k >= 0; --k) {
        const R tau = sTau[k];
        if (tau == R(0)) continue;
        const C* u = sH + qr_off<W>(k);
        C w = c_zero<C>();
#pragma unroll
        for (int i = 0; i < W; ++i)
            if (i >= k) w = c_fma_conj(u[i - k], e[i], w);
        w = c_scale(w, tau);
#pragma unroll
        for (int i = 0; i < W; ++i)
            if (i >= k) e[i] = c_sub(e[i], c_mul(u[i - k], w));
    }
#pragma unroll
    for (int i = 0; i < W; ++i) col[i] = e[i];
    __syncwarp();
}

// m = U S Vh per matrix (masked at eps) -> lu = sqrt(S) Vh, ul = U pinv(sqrt(S))
// (src/bqa/backends.py:483-490,709-727).  The messages are Hermitian positive semidefinite,
// so U = V on every singular value above the noise level (the rest are masked); both factors
// are built from the accumulated V, which stays unitary to working precision, while
// a_j / sigma_j carries a relative error eps |m| / sigma_j for small sigma_j.
// QR: Jacobi on the pivoted triangular factor (qr_precondition / qr_apply_q above).
template <int W, typename R, bool QR>
__global__ void __launch_bounds__(128, 4) env_factor_kernel(const typename Cx<R>::T* __restrict__ mats, int count, int n,
                                                         R eps, typename Cx<R>::T* __restrict__ lu,
                                                         typename Cx<R>::T* __restrict__ ul, int32_t* status) {
    using C = typename Cx<R>::T;
    constexpr int VS = VStride<W>::VS;
    constexpr int BLOCK = QR ? QrStride<W>::BLOCK : VStride<W>::BLOCK;
    extern __shared__ double4_32a smem_raw[];
    const int lane = threadIdx.x & (W - 1);
    C* sV = reinterpret_cast<C*>(smem_raw) + (threadIdx.x / W) * BLOCK;
    C* sH = sV + VStride<W>::BLOCK;
    R* sTau = reinterpret_cast<R*>(sH + QrStride<W>::H);
    const int mat = (blockIdx.x * blockDim.x + threadIdx.x) / W;
    const bool live = mat < count;
    const size_t base = (size_t)(live ? mat : 0) * n * n;
    C a[W];
#pragma unroll
    for (int i = 0; i < W; ++i) a[i] = (live && i < n && lane < n) ? mats[base + (size_t)i * n + lane] : c_zero<C>();
    // (a second pass, R1^H = Q2 R2 with the Jacobi on R2^H, saves about one more sweep in the
    // float32 model but measured slower on GB300: 61.4 -> 72.4 ms per 100k-node step)
    if constexpr (QR) qr_precondition<W, R>(a, sV, sH, sTau, lane);
    const bool ok = jacobi_columns<W, R>(a, sV, lane);
    const C* v = sV + lane * VS;
    if (!ok && live && lane == 0) atomicOr(status, BQA_STATUS_SVD_NOT_CONVERGED);
    R nrm2 = 0;
#pragma unroll
    for (int i = 0; i < W; ++i) nrm2 += c_abs2(a[i]);
    const R sig = sqrt(nrm2);
    if constexpr (QR) qr_apply_q<W, R>(sV, sH, sTau, lane);
    const bool keep = sig > eps;
    const R sq = sqrt(sig);
    const R sqk = keep ? sq : R(0);
    const R inv = keep ? R(1) / sq : R(0);
    // row k of lu = sqrt(sigma_k) conj(v_k)^T, v_k = column k of V: written a row at a time, the
    // lanes along the row (coalesced); column `lane` of ul = v / sqrt(sigma)
#pragma unroll
    for (int k = 0; k < W; ++k) {
        const R sk = __shfl_sync(BQA_FULL_MASK, sqk, k, W);
        if (live && k < n && lane < n) {
            const C vk = sV[k * VS + lane];
            lu[base + (size_t)k * n + lane] = c_make(sk * vk.x, -sk * vk.y);
        }
    }
    if (!live || lane >= n) return;
#pragma unroll
    for (int k = 0; k < W; ++k)
        if (k < n) ul[base + (size_t)k * n + lane] = c_scale(v[k], inv);
}

// Per undirected edge p: ker = lu[p] lu[p+h]^T = us s vhs; lambdas; canonicalisers
// (src/bqa/state.py:171-200).
// QR: the Jacobi runs on the pivoted triangular factor of ker^H (qr_precondition): with
// ker^H = Q R', R'^H = ker Q, and R'^H V_r = A (orthogonal columns) gives ker (Q V_r) = A, so
// Q V_r are ker's right singular vectors and A = us s, the same roles as the direct form.  The
// Householder vectors sit in the segment's staging block, idle between the ker product and
// the canonicaliser products.
template <int W, typename R, bool QR>
__global__ void __launch_bounds__(128, 4) bond_canon_kernel(const typename Cx<R>::T* __restrict__ lu,
                                                         const typename Cx<R>::T* __restrict__ ul, int edges, int n,
                                                         R eps, typename Cx<R>::T* __restrict__ canon,
                                                         R* __restrict__ lmbds, typename Cx<R>::Bits* colmax,
                                                         int32_t* status) {
    static_assert(!QR || QrStride<W>::H + W <= W * W, "Householder vectors fit the staging block");
    using C = typename Cx<R>::T;
    extern __shared__ double4_32a smem_raw[];
    constexpr int VS = VStride<W>::VS;
    const int lane = threadIdx.x & (W - 1);
    const int seg = threadIdx.x / W;
    C* sm = reinterpret_cast<C*>(smem_raw) + (size_t)seg * W * W;
    C* sV = reinterpret_cast<C*>(smem_raw) + (size_t)128 * W + (size_t)seg * VStride<W>::BLOCK;
    const int half = edges / 2;
    const int p = (blockIdx.x * blockDim.x + threadIdx.x) / W;
    const bool live = p < half;
    const int pf = live ? p : 0, pb = pf + half;
    const size_t nn = (size_t)n * n;
    // direct: stage lu_f, then ker[:, lane] = lu_f . lu_b[lane, :]^T (row lane of lu_b in registers)
    // QR: stage lu_b, and lu_f in the (still idle) V block at an odd row stride (conflict-free row
    // reads), then ker^H[:, lane] = conj(lu_b . lu_f[lane, :]^T); no row registers (they spilled)
    const size_t staged = QR ? (size_t)pb : (size_t)pf, other = QR ? (size_t)pf : (size_t)pb;
    for (int i = lane; i < n * n; i += W) sm[i] = live ? lu[staged * nn + i] : c_zero<C>();
    constexpr int RS = W + 1;   // row stride of lu_f in the V block (W * RS <= W * VS)
    if constexpr (QR) {
        for (int i = lane; i < n * n; i += W) {
            const int r = i / n, c = i - r * n;
            sV[r * RS + c] = live ? lu[other * nn + i] : c_zero<C>();
        }
    }
    __syncwarp();
    C a[W];
    if constexpr (QR) {
        const C* frow = sV + lane * RS;
#pragma unroll
        for (int i = 0; i < W; ++i) {
            C acc = c_zero<C>();
            if (i < n && lane < n) {
#pragma unroll
                for (int k = 0; k < W; ++k)
                    if (k < n) acc = c_fma(sm[i * n + k], frow[k], acc);
            }
            a[i] = c_conj(acc);
        }
    } else {
        C brow[W];
#pragma unroll
        for (int k = 0; k < W; ++k)
            brow[k] = (live && lane < n && k < n) ? lu[other * nn + (size_t)lane * n + k] : c_zero<C>();
#pragma unroll
        for (int i = 0; i < W; ++i) {
            C acc = c_zero<C>();
            if (i < n) {
#pragma unroll
                for (int k = 0; k < W; ++k)
                    if (k < n) acc = c_fma(sm[i * n + k], brow[k], acc);
            }
            a[i] = acc;
        }
    }
    C* sH = sm;
    R* sTau = reinterpret_cast<R*>(sm + QrStride<W>::H);
    if constexpr (QR) {
        __syncwarp();   // every lane has read the staged factor before the Householder vectors land there
        qr_precondition<W, R>(a, sV, sH, sTau, lane);
    }
    const bool ok = jacobi_columns<W, R>(a, sV, lane);
    const C* v = sV + lane * VS;
    if (!ok && live && lane == 0) atomicOr(status, BQA_STATUS_SVD_NOT_CONVERGED);
    R nrm2 = 0;
#pragma unroll
    for (int i = 0; i < W; ++i) nrm2 += c_abs2(a[i]);
    const R sig = sqrt(nrm2);
    if constexpr (QR) qr_apply_q<W, R>(sV, sH, sTau, lane);
    const R sk = (lane < n && sig > eps) ? sig : R(0);
    // descending rank among the segment's columns, ties by column index
    int rank = 0;
#pragma unroll
    for (int k = 0; k < W; ++k) {
        const R o = __shfl_sync(BQA_FULL_MASK, sk, k, W);
        rank += (o > sk) || (o == sk && k < lane);
    }
    const R norm = sqrt(seg_sum<W>(sk * sk));
    if (live && lane < n) {
        lmbds[(size_t)pf * n + rank] = norm > R(0) ? sk / norm : R(0);
        if (norm > R(0)) atomic_max_nonneg(colmax + rank, sk / norm);
    }
    const R uinv = sk > R(0) ? R(1) / sig : R(0);
    // fwd canonicaliser column rank: ul[p] . (a / sigma) -> canon[p + half]
    __syncwarp();
    for (int i = lane; i < n * n; i += W) sm[i] = live ? ul[(size_t)pf * nn + i] : c_zero<C>();
    __syncwarp();
    if (live && lane < n) {
        C* out = canon + (size_t)pb * nn + rank;
        for (int i = 0; i < n; ++i) {
            C acc = c_zero<C>();
#pragma unroll
            for (int k = 0; k < W; ++k)
                if (k < n) acc = c_fma(sm[i * n + k], a[k], acc);
            out[(size_t)i * n] = c_scale(acc, uinv);
        }
    }
    // bwd canonicaliser column rank: ul[p + half] . conj(v)  (vs = vhs^T) -> canon[p]
    __syncwarp();
    for (int i = lane; i < n * n; i += W) sm[i] = live ? ul[(size_t)pb * nn + i] : c_zero<C>();
    __syncwarp();
    if (live && lane < n) {
        const R keep = sk > R(0) ? R(1) : R(0);
        C* out = canon + (size_t)pf * nn + rank;
        for (int i = 0; i < n; ++i) {
            C acc = c_zero<C>();
#pragma unroll
            for (int k = 0; k < W; ++k)
                if (k < n) acc = c_fma(sm[i * n + k], c_conj(v[k]), acc);
            out[(size_t)i * n] = c_scale(acc, keep);
        }
    }
}

// ---- matrices of size 33..64 (bond dims 17..32): columns in shared memory ----------------------
//
// One warp per matrix.  A and V are kept column-major in shared memory at an odd stride
// (NS = 65 complex elements), so the 32 lanes reading one row of 32 different columns fall in
// distinct 8-byte bank slots two by two.  The xor round-robin ordering is the same (round r
// pairs j with j ^ r, r = 1..63); lane k takes the k-th pair of the round, forms its Gram
// entries, decides and applies the rotation to both columns of A and V, and updates the two
// cached column norms.  Pairs of a round are disjoint, so lanes never touch the same column.
// Decisions, rotation formula, relative test and stopping rule are those of jacobi_columns.
constexpr int kWide = 64;
constexpr int kWideNS = 65;

template <typename R>
__device__ __forceinline__ bool jacobi_wide(typename Cx<R>::T* A, typename Cx<R>::T* V, R* nrm, int lane) {
    using C = typename Cx<R>::T;
    constexpr int W = kWide, NS = kWideNS;
    for (int j = lane; j < W; j += 32) {
        C* v = V + j * NS;
        for (int i = 0; i < W; ++i) v[i] = c_make(i == j ? R(1) : R(0), R(0));
        const C* a = A + j * NS;
        R p[NP] = {};
        for (int i = 0; i < W; ++i) p[i % NP] = fma(a[i].x, a[i].x, fma(a[i].y, a[i].y, p[i % NP]));
        nrm[j] = sum_parts<NP>(p);
    }
    __syncwarp();
    R fro2 = nrm[lane] + nrm[lane + 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) fro2 += __shfl_xor_sync(BQA_FULL_MASK, fro2, o);
    const R tol = (R)W * jacobi_eps<R>();
    const R col_floor = fmax((R)W * jacobi_eps<R>() * jacobi_eps<R>() * fro2, sizeof(R) == 4 ? R(1e-30) : R(1e-280));
    for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
        int rotated = 0;
        for (int r = 1; r < W; ++r) {
            const int h = 31 - __clz(r);
            const int pc = ((lane >> h) << (h + 1)) | (lane & ((1 << h) - 1));   // bit h clear
            const int qc = pc ^ r;
            C* ap = A + pc * NS;
            C* aq = A + qc * NS;
            const R alpha = nrm[pc], beta = nrm[qc];
            R sx[NP] = {}, sy[NP] = {};
            for (int i = 0; i < W; ++i) {
                const C x = ap[i], y = aq[i];
                sx[i % NP] = fma(x.x, y.x, fma(x.y, y.y, sx[i % NP]));
                sy[i % NP] = fma(x.x, y.y, fma(-x.y, y.x, sy[i % NP]));
            }
            const C g = c_make(sum_parts<NP>(sx), sum_parts<NP>(sy));
            const R gabs = sqrt(c_abs2(g));
            const bool rot = alpha > R(0) && beta > R(0) && gabs > tol * sqrt(alpha) * sqrt(beta);
            if (rot) {
                const R zeta = (beta - alpha) / (R(2) * gabs);
                const R t = copysign(R(1), zeta) / (fabs(zeta) + hypot(R(1), zeta));
                const R c = R(1) / sqrt(fma(t, t, R(1)));
                const R sn = c * t;
                const R ex = g.x / gabs, ey = g.y / gabs;
                const C wp = c_make(-sn * ex, sn * ey), wq = c_make(sn * ex, sn * ey);
                R np_[NP] = {}, nq_[NP] = {};
                for (int i = 0; i < W; ++i) {
                    const C x = ap[i], y = aq[i];
                    const C nx = c_fma(wp, y, c_scale(x, c)), ny = c_fma(wq, x, c_scale(y, c));
                    ap[i] = nx;
                    aq[i] = ny;
                    np_[i % NP] = fma(nx.x, nx.x, fma(nx.y, nx.y, np_[i % NP]));
                    nq_[i % NP] = fma(ny.x, ny.x, fma(ny.y, ny.y, nq_[i % NP]));
                }
                nrm[pc] = sum_parts<NP>(np_);
                nrm[qc] = sum_parts<NP>(nq_);
                C* vp = V + pc * NS;
                C* vq = V + qc * NS;
                for (int i = 0; i < W; ++i) {
                    const C x = vp[i], y = vq[i];
                    vp[i] = c_fma(wp, y, c_scale(x, c));
                    vq[i] = c_fma(wq, x, c_scale(y, c));
                }
                rotated |= (alpha > col_floor && beta > col_floor);
            }
            __syncwarp();
        }
        if (!__any_sync(BQA_FULL_MASK, rotated)) return true;
    }
    return false;
}

// A, V, column norms, and (bond canonicalisation) kept singular values and their ranks
template <typename R>
__host__ __device__ constexpr size_t wide_smem_elems() { return 2 * (size_t)kWide * kWideNS + 3 * kWide; }

// bqa_env_factor for 32 < n <= 64: one warp per matrix (mirrors env_factor_kernel)
template <typename R>
__global__ void __launch_bounds__(32) env_factor_wide_kernel(const typename Cx<R>::T* __restrict__ mats, int count,
                                                             int n, R eps, typename Cx<R>::T* __restrict__ lu,
                                                             typename Cx<R>::T* __restrict__ ul, int32_t* status) {
    using C = typename Cx<R>::T;
    constexpr int NS = kWideNS;
    extern __shared__ double4_32a smem_raw[];
    C* A = reinterpret_cast<C*>(smem_raw);
    C* V = A + kWide * NS;
    R* nrm = reinterpret_cast<R*>(V + kWide * NS);
    const int lane = threadIdx.x;
    const int mat = blockIdx.x;
    const size_t base = (size_t)mat * n * n;
    // column j of A = column j of m (zero-padded to 64)
    for (int e = lane; e < kWide * kWide; e += 32) {
        const int j = e / kWide, i = e - j * kWide;
        A[j * NS + i] = (i < n && j < n) ? mats[base + (size_t)i * n + j] : c_zero<C>();
    }
    __syncwarp();
    const bool ok = jacobi_wide<R>(A, V, nrm, lane);
    if (!ok && lane == 0) atomicOr(status, BQA_STATUS_SVD_NOT_CONVERGED);
    // sigma_j = |a_j|; nrm[j] <- sqrt(sigma_j) if kept, else 0
    for (int j = lane; j < kWide; j += 32) {
        const C* a = A + j * NS;
        R s2 = 0;
        for (int i = 0; i < kWide; ++i) s2 += c_abs2(a[i]);
        const R sig = sqrt(s2);
        nrm[j] = sig > eps ? sqrt(sig) : R(0);
    }
    __syncwarp();
    // lu[j][k] = sqrt(sigma_j) conj(V[k][j]), ul[k][j] = V[k][j] / sqrt(sigma_j)
    for (int e = lane; e < n * n; e += 32) {
        const int j = e / n, k = e - j * n;
        const R sq = nrm[j];
        const C vkj = V[j * NS + k];
        lu[base + (size_t)j * n + k] = c_make(sq * vkj.x, -sq * vkj.y);
    }
    for (int e = lane; e < n * n; e += 32) {
        const int k = e / n, j = e - k * n;
        const R inv = nrm[j] > R(0) ? R(1) / nrm[j] : R(0);
        ul[base + (size_t)k * n + j] = c_scale(V[j * NS + k], inv);
    }
}

// bqa_bond_canon for 32 < n <= 64: one warp per undirected edge (mirrors bond_canon_kernel)
template <typename R>
__global__ void __launch_bounds__(32) bond_canon_wide_kernel(const typename Cx<R>::T* __restrict__ lu,
                                                             const typename Cx<R>::T* __restrict__ ul, int edges, int n,
                                                             R eps, typename Cx<R>::T* __restrict__ canon,
                                                             R* __restrict__ lmbds, typename Cx<R>::Bits* colmax,
                                                             int32_t* status) {
    using C = typename Cx<R>::T;
    constexpr int NS = kWideNS;
    extern __shared__ double4_32a smem_raw[];
    C* A = reinterpret_cast<C*>(smem_raw);
    C* V = A + kWide * NS;
    R* nrm = reinterpret_cast<R*>(V + kWide * NS);
    R* s_sig = reinterpret_cast<R*>(V + kWide * NS + kWide);
    int* s_rank = reinterpret_cast<int*>(V + kWide * NS + 2 * kWide);
    const int lane = threadIdx.x;
    const int half = edges / 2;
    const int pf = blockIdx.x, pb = pf + half;
    const size_t nn = (size_t)n * n;
    const C* luf = lu + (size_t)pf * nn;
    const C* lub = lu + (size_t)pb * nn;
    // ker[i][j] = sum_k lu_f[i][k] lu_b[j][k]; column j of A = column j of ker
    for (int e = lane; e < kWide * kWide; e += 32) {
        const int j = e / kWide, i = e - j * kWide;
        C acc = c_zero<C>();
        if (i < n && j < n)
            for (int k = 0; k < n; ++k) acc = c_fma(luf[(size_t)i * n + k], lub[(size_t)j * n + k], acc);
        A[j * NS + i] = acc;
    }
    __syncwarp();
    const bool ok = jacobi_wide<R>(A, V, nrm, lane);
    if (!ok && lane == 0) atomicOr(status, BQA_STATUS_SVD_NOT_CONVERGED);
    for (int j = lane; j < kWide; j += 32) {
        const C* a = A + j * NS;
        R s2 = 0;
        for (int i = 0; i < kWide; ++i) s2 += c_abs2(a[i]);
        const R sig = sqrt(s2);
        s_sig[j] = (j < n && sig > eps) ? sig : R(0);
        nrm[j] = s_sig[j] > R(0) ? R(1) / sig : R(0);      // 1 / sigma_j of the kept columns
    }
    __syncwarp();
    R ss = 0;
    for (int j = lane; j < kWide; j += 32) ss += s_sig[j] * s_sig[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(BQA_FULL_MASK, ss, o);
    const R norm = sqrt(ss);
    for (int j = lane; j < kWide; j += 32) {
        const R sk = s_sig[j];
        int rank = 0;
        for (int k = 0; k < kWide; ++k) rank += (s_sig[k] > sk) || (s_sig[k] == sk && k < j);
        s_rank[j] = rank;
        if (j < n) {
            lmbds[(size_t)pf * n + rank] = norm > R(0) ? sk / norm : R(0);
            if (norm > R(0)) atomic_max_nonneg(colmax + rank, sk / norm);
        }
    }
    __syncwarp();
    // canon[pb][i][rank_j] = ul_f[i] . a_j / sigma_j ; canon[pf][i][rank_j] = ul_b[i] . conj(v_j)
    const C* ulf = ul + (size_t)pf * nn;
    const C* ulb = ul + (size_t)pb * nn;
    for (int e = lane; e < n * n; e += 32) {
        const int i = e / n, j = e - i * n;
        const R sk = s_sig[j];
        const C* a = A + j * NS;
        const C* v = V + j * NS;
        C acc = c_zero<C>(), accv = c_zero<C>();
        for (int k = 0; k < n; ++k) {
            acc = c_fma(ulf[(size_t)i * n + k], a[k], acc);
            accv = c_fma(ulb[(size_t)i * n + k], c_conj(v[k]), accv);
        }
        canon[(size_t)pb * nn + (size_t)i * n + s_rank[j]] = c_scale(acc, nrm[j]);
        canon[(size_t)pf * nn + (size_t)i * n + s_rank[j]] = c_scale(accv, sk > R(0) ? R(1) : R(0));
    }
}

template <typename R>
static int launch_env_wide(const void* m, int count, int n, double eps, void* lu, void* ul, int32_t* status,
                           cudaStream_t st) {
    using C = typename Cx<R>::T;
    const size_t smem = wide_smem_elems<R>() * sizeof(C);
    int rc = ensure_smem((const void*)env_factor_wide_kernel<R>, smem, "env_factor (64)");
    if (rc) return rc;
    env_factor_wide_kernel<R><<<count, 32, smem, st>>>(static_cast<const C*>(m), count, n, (R)eps, static_cast<C*>(lu),
                                                        static_cast<C*>(ul), status);
    return check_launch("env_factor (64)");
}

template <typename R>
static int launch_canon_wide(const void* lu, const void* ul, int edges, int n, double eps, void* canon, void* lmbds,
                             void* colmax, int32_t* status, cudaStream_t st) {
    using C = typename Cx<R>::T;
    const size_t smem = wide_smem_elems<R>() * sizeof(C);
    int rc = ensure_smem((const void*)bond_canon_wide_kernel<R>, smem, "bond_canon (64)");
    if (rc) return rc;
    bond_canon_wide_kernel<R><<<edges / 2, 32, smem, st>>>(static_cast<const C*>(lu), static_cast<const C*>(ul), edges,
                                                            n, (R)eps, static_cast<C*>(canon), static_cast<R*>(lmbds),
                                                            static_cast<typename Cx<R>::Bits*>(colmax), status);
    return check_launch("bond_canon (64)");
}

// The environment factors run QR-preconditioned unless BQA_GB300_JACOBI_QR=0 is set when the
// library loads (then the Jacobi works on the matrices directly; tests cross-check the two).
// Complex128 matrices above 16 columns keep the direct form: there the preconditioner's extra
// registers spill.
static const bool g_jacobi_qr = [] {
    const char* v = getenv("BQA_GB300_JACOBI_QR");
    return !(v && v[0] == '0');
}();

template <int W, typename R, bool QR>
static int launch_env_k(const void* m, int count, int n, double eps, void* lu, void* ul, int32_t* status,
                        cudaStream_t st) {
    using C = typename Cx<R>::T;
    const int per_block = 128 / W;
    const int blocks = (count + per_block - 1) / per_block;
    const size_t smem = (size_t)(128 / W) * (QR ? QrStride<W>::BLOCK : VStride<W>::BLOCK) * sizeof(C);
    int rc = ensure_smem((const void*)env_factor_kernel<W, R, QR>, smem, "env_factor");
    if (rc) return rc;
    env_factor_kernel<W, R, QR><<<blocks, 128, smem, st>>>(static_cast<const C*>(m), count, n, (R)eps,
                                                           static_cast<C*>(lu), static_cast<C*>(ul), status);
    return check_launch("env_factor");
}

template <int W, typename R>
static int launch_env(const void* m, int count, int n, double eps, void* lu, void* ul, int32_t* status, cudaStream_t st) {
    if constexpr (sizeof(R) == 4 || W <= 16) {
        if (g_jacobi_qr) return launch_env_k<W, R, true>(m, count, n, eps, lu, ul, status, st);
    }
    return launch_env_k<W, R, false>(m, count, n, eps, lu, ul, status, st);
}

template <int W, typename R, bool QR>
static int launch_canon_k(const void* lu, const void* ul, int edges, int n, double eps, void* canon, void* lmbds,
                          void* colmax, int32_t* status, cudaStream_t st) {
    using C = typename Cx<R>::T;
    const int per_block = 128 / W;
    const int half = edges / 2;
    const int blocks = (half + per_block - 1) / per_block;
    const size_t smem = ((size_t)128 * W + (size_t)(128 / W) * VStride<W>::BLOCK) * sizeof(C);
    int rc = ensure_smem((const void*)bond_canon_kernel<W, R, QR>, smem, "bond_canon");
    if (rc) return rc;
    bond_canon_kernel<W, R, QR><<<blocks, 128, smem, st>>>(static_cast<const C*>(lu), static_cast<const C*>(ul),
                                                           edges, n, (R)eps, static_cast<C*>(canon),
                                                           static_cast<R*>(lmbds),
                                                           static_cast<typename Cx<R>::Bits*>(colmax), status);
    return check_launch("bond_canon");
}

// The bond canonicalisation's Jacobi works on ker^H's pivoted triangular factor when
// BQA_GB300_CANON_QR=1 is set when the library loads (complex64, and complex128 up to 16
// columns); by default it works on ker directly.
static const bool g_canon_qr = [] {
    const char* v = getenv("BQA_GB300_CANON_QR");
    return v && v[0] == '1';
}();

template <int W, typename R>
static int launch_canon(const void* lu, const void* ul, int edges, int n, double eps, void* canon, void* lmbds,
                        void* colmax, int32_t* status, cudaStream_t st) {
    if constexpr (sizeof(R) == 4 || W <= 16) {
        if (g_canon_qr) return launch_canon_k<W, R, true>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
    }
    return launch_canon_k<W, R, false>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
}

template <typename R>
static int env_dispatch(const void* m, int count, int n, double eps, void* lu, void* ul, int32_t* status,
                        cudaStream_t st) {
    if (n <= 8) return launch_env<8, R>(m, count, n, eps, lu, ul, status, st);
    if (n <= 16) return launch_env<16, R>(m, count, n, eps, lu, ul, status, st);
    if (n <= 32) return launch_env<32, R>(m, count, n, eps, lu, ul, status, st);
    if (n <= kWide) return launch_env_wide<R>(m, count, n, eps, lu, ul, status, st);
    return set_error(BQA_ERR_UNSUPPORTED, "bqa_env_factor: matrix size %d > %d", n, kWide);
}

template <typename R>
static int canon_dispatch(const void* lu, const void* ul, int edges, int n, double eps, void* canon, void* lmbds,
                          void* colmax, int32_t* status, cudaStream_t st) {
    if (n <= 8) return launch_canon<8, R>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
    if (n <= 16) return launch_canon<16, R>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
    if (n <= 32) return launch_canon<32, R>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
    if (n <= kWide) return launch_canon_wide<R>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
    return set_error(BQA_ERR_UNSUPPORTED, "bqa_bond_canon: matrix size %d > %d", n, kWide);
}

}  // namespace bqa

using namespace bqa;

extern "C" {

int32_t bqa_env_factor(const void* mats, int32_t count, int32_t n, int32_t dtype, double eps, void* lu, void* ul,
                       int32_t* status, void* stream) {
    if (!mats || !lu || !ul || !status || count < 0 || n < 1) return set_error(BQA_ERR_ARG, "bqa_env_factor: bad argument");
    if (count == 0) return BQA_OK;
    cudaStream_t st = as_stream(stream);
    if (dtype == BQA_C64) return env_dispatch<float>(mats, count, n, eps, lu, ul, status, st);
    if (dtype == BQA_C128) return env_dispatch<double>(mats, count, n, eps, lu, ul, status, st);
    return set_error(BQA_ERR_ARG, "bqa_env_factor: unknown dtype %d", dtype);
}

int32_t bqa_bond_canon(const void* lu, const void* ul, int32_t edges, int32_t n, int32_t dtype, double eps, void* canon,
                       void* lmbds, void* colmax, int32_t* status, void* stream) {
    if (!lu || !ul || !canon || !lmbds || !colmax || !status || edges < 2 || n < 1)
        return set_error(BQA_ERR_ARG, "bqa_bond_canon: bad argument");
    if (edges & 1) return set_error(BQA_ERR_ARG, "bqa_bond_canon: odd number of directed edges %d", edges);
    cudaStream_t st = as_stream(stream);
    if (dtype == BQA_C64) return canon_dispatch<float>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
    if (dtype == BQA_C128) return canon_dispatch<double>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
    return set_error(BQA_ERR_ARG, "bqa_bond_canon: unknown dtype %d", dtype);
}

}  // extern "C"

// ---- canonicalisation without caller scratch ------------------------------------------------
//
// bqa_canonicalize_noalloc runs the two kernels above (environment factors, then bond
// canonicalisation) with the intermediate factors lu and ul placed in one file-scope device
// array instead of caller-provided buffers.  It exists for callers that cannot allocate
// device memory: host programs whose device heap belongs to an external pool allocator
// (serving runtimes that reserve all free HBM at start-up), and pipelines that must not call
// cudaMalloc/cudaFree because those synchronise the device.  Such a caller passes only the
// inputs and outputs; the factors live in kNoAllocScratchBytes of device memory that every
// GPU which loads this library holds until the process exits.
//
// The array's device address is looked up once per device, on the first call made with that
// device current (cudaGetSymbolAddress; the host-side name of a __device__ array is not a
// device address).  That first call therefore should come before any stream capture.  All
// calls share the array and it keeps the previous call's contents; every element the kernels
// read is written earlier in the same call, and nothing in it must start at zero.  Calls that
// overlap on the GPU (different streams, or different host threads) race on the array.
// The looked-up address is cached per device ordinal for the life of the process: it does not
// survive cudaDeviceReset (or any other teardown of the device's primary context), after which
// the library's module is loaded again at a new address.

namespace bqa {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;   // 64 MiB: lu + ul
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static void* noalloc_scratch_address(int* rc) {
    static std::mutex mu;
    static void* addr[64] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { *rc = set_error(BQA_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e)); return nullptr; }
    if (dev < 0 || dev >= 64) { *rc = set_error(BQA_ERR_UNSUPPORTED, "device ordinal %d >= 64", dev); return nullptr; }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            *rc = set_error(BQA_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
            return nullptr;
        }
        addr[dev] = p;
    }
    *rc = BQA_OK;
    return addr[dev];
}

}  // namespace bqa

extern "C" {

int32_t bqa_canonicalize_noalloc(const void* ext_msgs, int32_t edges, int32_t n, int32_t dtype, double eps,
                                 void* canon, void* lmbds, void* colmax, int32_t* status, void* stream) {
    if (!ext_msgs || !canon || !lmbds || !colmax || !status || edges < 2 || n < 1)
        return set_error(BQA_ERR_ARG, "bqa_canonicalize_noalloc: bad argument");
    if (edges & 1)
        return set_error(BQA_ERR_ARG, "bqa_canonicalize_noalloc: odd number of directed edges %d", edges);
    if (dtype != BQA_C64 && dtype != BQA_C128)
        return set_error(BQA_ERR_ARG, "bqa_canonicalize_noalloc: unknown dtype %d", dtype);
    if (n > 32) return set_error(BQA_ERR_UNSUPPORTED, "bqa_canonicalize_noalloc: matrix size %d > 32", n);
    const size_t el = dtype == BQA_C64 ? 8 : 16;
    const size_t one = (size_t)edges * n * n * el;
    if (2 * one > kNoAllocScratchBytes)
        return set_error(BQA_ERR_UNSUPPORTED,
                         "bqa_canonicalize_noalloc: %d edges at n=%d need %zu bytes of factors, above the "
                         "%zu-byte static scratch; use bqa_env_factor + bqa_bond_canon with caller buffers",
                         edges, n, 2 * one, kNoAllocScratchBytes);
    int rc = BQA_OK;
    unsigned char* base = static_cast<unsigned char*>(noalloc_scratch_address(&rc));
    if (rc) return rc;
    void* lu = base;
    void* ul = base + ((one + 255) & ~size_t(255));
    cudaStream_t st = as_stream(stream);
    const size_t colmax_bytes = (size_t)n * (dtype == BQA_C64 ? 4 : 8);
    cudaError_t e = cudaMemsetAsync(colmax, 0, colmax_bytes, st);
    if (e != cudaSuccess) return set_error(BQA_ERR_CUDA, "bqa_canonicalize_noalloc: %s", cudaGetErrorString(e));
    if (dtype == BQA_C64) {
        rc = env_dispatch<float>(ext_msgs, edges, n, eps, lu, ul, status, st);
        if (rc) return rc;
        return canon_dispatch<float>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
    }
    rc = env_dispatch<double>(ext_msgs, edges, n, eps, lu, ul, status, st);
    if (rc) return rc;
    return canon_dispatch<double>(lu, ul, edges, n, eps, canon, lmbds, colmax, status, st);
}

}  // extern "C"
