// Projective measurement of listed nodes of one degree class
// (src/bqa/backends.py:730-734, driven by src/bqa/state.py:272-296): the amplitude slice of
// the rejected outcome is zeroed, then the whole class buffer is divided by its L2 norm
// (the reference normalises the class batch by one global norm).
#include "common.cuh"
#include "internal.h"

namespace bqa {

template <typename C>
__global__ void project_kernel(C* t, int node_elems, const int32_t* pos, const int32_t* outcome, int m) {
    const int half = node_elems / 2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)m * half;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(i / half), o = (int)(i - (int64_t)j * half);
        t[(size_t)pos[j] * node_elems + (size_t)(1 - outcome[j]) * half + o] = c_zero<C>();
    }
}

template <typename C>
__global__ void sumsq_kernel(const C* t, int64_t n, double* acc) {
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (double)c_abs2(t[i]);
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, s);
}

template <typename C>
__global__ void scale_kernel(C* t, int64_t n, const double* acc) {
    const auto inv = (decltype(t[0].x))(1.0 / sqrt(*acc));
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        t[i] = c_scale(t[i], inv);
}

template <typename C>
static int project(void* tensors, int count, int node_elems, const int32_t* positions, const int32_t* outcomes, int m,
                   double* norm2, cudaStream_t st) {
    auto t = static_cast<C*>(tensors);
    const int64_t n = (int64_t)count * node_elems;
    int blocks = (int)(((int64_t)m * (node_elems / 2) + 255) / 256);
    blocks = blocks > 4096 ? 4096 : blocks;
    project_kernel<C><<<blocks, 256, 0, st>>>(t, node_elems, positions, outcomes, m);
    int rc = check_launch("project");
    if (rc) return rc;
    cudaError_t e = cudaMemsetAsync(norm2, 0, sizeof(double), st);
    if (e != cudaSuccess) return set_error(BQA_ERR_CUDA, "bqa_project_nodes: %s", cudaGetErrorString(e));
    int rb = (int)((n + 255) / 256);
    rb = rb > 4096 ? 4096 : rb;
    sumsq_kernel<C><<<rb, 256, 0, st>>>(t, n, norm2);
    rc = check_launch("sumsq");
    if (rc) return rc;
    scale_kernel<C><<<rb, 256, 0, st>>>(t, n, norm2);
    return check_launch("scale");
}

}  // namespace bqa

using namespace bqa;

extern "C" {

int32_t bqa_project_nodes(void* tensors, int32_t count, int32_t node_elems, int32_t dtype, const int32_t* positions,
                          const int32_t* outcomes, int32_t m, double* norm2_scratch, void* stream) {
    if (!tensors || !positions || !outcomes || !norm2_scratch || count < 1 || node_elems < 2 || m < 0)
        return set_error(BQA_ERR_ARG, "bqa_project_nodes: bad argument");
    if (m == 0) return BQA_OK;
    cudaStream_t st = as_stream(stream);
    if (dtype == BQA_C64) return project<float2>(tensors, count, node_elems, positions, outcomes, m, norm2_scratch, st);
    if (dtype == BQA_C128) return project<double2>(tensors, count, node_elems, positions, outcomes, m, norm2_scratch, st);
    return set_error(BQA_ERR_ARG, "bqa_project_nodes: unknown dtype %d", dtype);
}

}  // extern "C"
