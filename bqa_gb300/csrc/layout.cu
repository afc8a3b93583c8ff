// Degree-class compilation on the device: the graph -> batch index maps of the reference's
// _make_degree_to_layout (src/bqa/config/config_canonicalization.py:62-131), built with
// atomics and single-CTA scans instead of a per-node host loop.
//
// Input: the directed edge list in message-slot order, int32 [E][2] (src, dst); slots
// p < E/2 are the user's edges and slot p + E/2 is the reversal of slot p.  Conventions
// (the same as the host compiler, bit-exact):
//   * bond k of node v is the k-th slot, in increasing slot order, whose source is v;
//   * nodes of one degree form a class, in increasing node id; classes are ordered by the
//     lowest node id of each degree (first appearance);
//   * in_pos = (out_pos + E/2) % E, lmbd_pos = out_pos % (E/2).
//
// bqa_layout_degrees: deg[v], start[v] (exclusive scan of deg), order[] (slots grouped by
// source, increasing inside each group), per-degree lowest node id and node count.
// bqa_layout_class: for one degree, node_ids (increasing), position[v] of its nodes and the
// node-major maps [count][d].
#include "common.cuh"
#include "internal.h"

namespace bqa {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;

// Exclusive scan of this thread's kScanItems values within the CTA, plus the CTA total.
__device__ __forceinline__ int cta_exclusive_scan(int v, int* warp_sums, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(BQA_FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(BQA_FULL_MASK, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const int before = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
    *total = warp_sums[31];
    __syncthreads();  // warp_sums is reused by the next chunk
    return before;
}

__global__ void layout_count_kernel(const int32_t* __restrict__ edges, int E, int n, int32_t* deg, int32_t* status) {
    const int half = E / 2;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < E; p += gridDim.x * blockDim.x) {
        const int s = edges[2 * p], t = edges[2 * p + 1];
        if (s < 0 || s >= n || t < 0 || t >= n || s == t) {
            atomicOr(status, BQA_STATUS_LAYOUT_EDGE);
            continue;
        }
        // slot p + E/2 must be the reversal of slot p (the reference's edge dict order)
        if (p < half && (edges[2 * (p + half)] != t || edges[2 * (p + half) + 1] != s))
            atomicOr(status, BQA_STATUS_LAYOUT_EDGE);
        atomicAdd(deg + s, 1);
    }
}

// start = exclusive scan of deg (one CTA)
__global__ void __launch_bounds__(kScanThreads) layout_scan_kernel(const int32_t* __restrict__ deg, int n,
                                                                   int32_t* __restrict__ start) {
    __shared__ int warp_sums[32];
    int carry = 0;
    for (int base = 0; base < n; base += kScanThreads * kScanItems) {
        const int i0 = base + threadIdx.x * kScanItems;
        int v[kScanItems], sum = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            v[k] = (i0 + k < n) ? deg[i0 + k] : 0;
            sum += v[k];
        }
        int total;
        int run = carry + cta_exclusive_scan(sum, warp_sums, &total);
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (i0 + k < n) start[i0 + k] = run;
            run += v[k];
        }
        carry += total;
    }
}

// order[start[s] + k] = slot p for the k-th arrival of source s (arrival order is arbitrary;
// the per-node sort below restores slot order).  fill[] counts arrivals per node.
__global__ void layout_fill_kernel(const int32_t* __restrict__ edges, int E, int n, const int32_t* __restrict__ start,
                                   int32_t* fill, int32_t* __restrict__ order) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < E; p += gridDim.x * blockDim.x) {
        const int s = edges[2 * p], t = edges[2 * p + 1];
        if (s < 0 || s >= n || t < 0 || t >= n || s == t) continue;
        const int k = atomicAdd(fill + s, 1);
        order[start[s] + k] = p;
    }
}

// Per node: sort its slots, record the degree's lowest node id and node count.
__global__ void layout_node_kernel(const int32_t* __restrict__ deg, const int32_t* __restrict__ start, int n,
                                   int max_degree, int32_t* __restrict__ order, int32_t* class_first,
                                   int32_t* class_count, int32_t* status) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int d = deg[v];
        if (d > max_degree) {
            atomicOr(status, BQA_STATUS_LAYOUT_DEGREE);
            continue;
        }
        int32_t* o = order + start[v];
        for (int i = 1; i < d; ++i) {  // insertion sort, d <= max_degree
            const int x = o[i];
            int j = i - 1;
            while (j >= 0 && o[j] > x) {
                o[j + 1] = o[j];
                --j;
            }
            o[j + 1] = x;
        }
        atomicMin(class_first + d, v);
        atomicAdd(class_count + d, 1);
    }
}

// node_ids of one degree in increasing id (stream compaction by one CTA) and their positions
__global__ void __launch_bounds__(kScanThreads) layout_compact_kernel(const int32_t* __restrict__ deg, int n, int d,
                                                                      int count, int32_t* __restrict__ node_ids,
                                                                      int32_t* __restrict__ position) {
    __shared__ int warp_sums[32];
    int carry = 0;
    for (int base = 0; base < n; base += kScanThreads * kScanItems) {
        const int i0 = base + threadIdx.x * kScanItems;
        int hit[kScanItems], sum = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            hit[k] = (i0 + k < n && deg[i0 + k] == d) ? 1 : 0;
            sum += hit[k];
        }
        int total;
        int run = carry + cta_exclusive_scan(sum, warp_sums, &total);
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (hit[k] && run < count) {
                node_ids[run] = i0 + k;
                position[i0 + k] = run;
            }
            run += hit[k];
        }
        carry += total;
    }
}

// node-major maps of one class: entry (i, k) of [count][d]
__global__ void layout_maps_kernel(const int32_t* __restrict__ node_ids, int count, int d,
                                   const int32_t* __restrict__ start, const int32_t* __restrict__ order, int E,
                                   const double* __restrict__ slot_ampl, const double* __restrict__ node_field,
                                   int32_t* __restrict__ in_pos, int32_t* __restrict__ out_pos,
                                   int32_t* __restrict__ lmbd_pos, double* __restrict__ edge_ampl,
                                   double* __restrict__ node_ampl) {
    const int half = E / 2;
    const long long total = (long long)count * (d > 0 ? d : 1);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = d > 0 ? (int)(e / d) : (int)e;
        const int k = d > 0 ? (int)(e - (long long)i * d) : 0;
        const int v = node_ids[i];
        if (k == 0 && node_ampl) node_ampl[i] = node_field ? node_field[v] : 0.0;
        if (d == 0) continue;
        const int p = order[start[v] + k];
        out_pos[e] = p;
        if (in_pos) in_pos[e] = (p + half) % E;
        if (lmbd_pos) lmbd_pos[e] = p % half;
        if (edge_ampl) edge_ampl[e] = slot_ampl ? slot_ampl[p] : 0.0;
    }
}

static int grid_for(long long work, int threads) {
    long long b = (work + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 152 * 16) b = 152 * 16;
    return (int)b;
}

}  // namespace bqa

using namespace bqa;

extern "C" {

int32_t bqa_layout_degrees(const int32_t* edges, int32_t E, int32_t n, int32_t max_degree, int32_t* deg,
                           int32_t* start, int32_t* order, int32_t* fill, int32_t* class_first,
                           int32_t* class_count, int32_t* status, void* stream) {
    if (!edges || !deg || !start || !order || !fill || !class_first || !class_count || !status || E < 2 || E % 2 ||
        n < 1 || max_degree < 0)
        return set_error(BQA_ERR_ARG, "bqa_layout_degrees: bad argument");
    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(deg, 0, sizeof(int32_t) * (size_t)n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(fill, 0, sizeof(int32_t) * (size_t)n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(class_count, 0, sizeof(int32_t) * (size_t)(max_degree + 1), st);
    // class_first starts at 0x7f7f7f7f (> any node id); the host treats counts of 0 as absent
    if (e == cudaSuccess) e = cudaMemsetAsync(class_first, 0x7f, sizeof(int32_t) * (size_t)(max_degree + 1), st);
    if (e != cudaSuccess) return set_error(BQA_ERR_CUDA, "bqa_layout_degrees: %s", cudaGetErrorString(e));
    layout_count_kernel<<<grid_for(E, 256), 256, 0, st>>>(edges, E, n, deg, status);
    int rc = check_launch("layout_count");
    if (rc) return rc;
    layout_scan_kernel<<<1, kScanThreads, 0, st>>>(deg, n, start);
    if ((rc = check_launch("layout_scan"))) return rc;
    layout_fill_kernel<<<grid_for(E, 256), 256, 0, st>>>(edges, E, n, start, fill, order);
    if ((rc = check_launch("layout_fill"))) return rc;
    layout_node_kernel<<<grid_for(n, 256), 256, 0, st>>>(deg, start, n, max_degree, order, class_first, class_count,
                                                         status);
    return check_launch("layout_node");
}

int32_t bqa_layout_class(int32_t degree, int32_t count, const int32_t* deg, const int32_t* start,
                         const int32_t* order, int32_t n, int32_t E, const double* slot_ampl,
                         const double* node_field, int32_t* node_ids, int32_t* position, int32_t* in_pos,
                         int32_t* out_pos, int32_t* lmbd_pos, double* edge_ampl, double* node_ampl, void* stream) {
    if (degree < 0 || count < 0 || !deg || !start || !order || n < 1 || E < 2 || E % 2 || !node_ids || !position ||
        (degree > 0 && !out_pos))
        return set_error(BQA_ERR_ARG, "bqa_layout_class: bad argument");
    if (count == 0) return BQA_OK;
    cudaStream_t st = as_stream(stream);
    layout_compact_kernel<<<1, kScanThreads, 0, st>>>(deg, n, degree, count, node_ids, position);
    int rc = check_launch("layout_compact");
    if (rc) return rc;
    const long long work = (long long)count * (degree > 0 ? degree : 1);
    layout_maps_kernel<<<grid_for(work, 256), 256, 0, st>>>(node_ids, count, degree, start, order, E, slot_ampl,
                                                            node_field, in_pos, out_pos, lmbd_pos, edge_ampl,
                                                            node_ampl);
    return check_launch("layout_maps");
}

}  // extern "C"
