// FP32 FMA throughput probe: the compute ceiling of the complex64 CUDA-core kernels.
// Every thread runs 16 independent FMA chains (no memory traffic in the loop) and writes one
// sum so the work cannot be removed; FLOPs = 2 * 16 * iters * blocks * 256.
#include "common.cuh"
#include "internal.h"

namespace bqa {

__global__ void __launch_bounds__(256) fma_probe_kernel(float* __restrict__ out, int iters, float s) {
    float a[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) a[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 16; ++i) a[i] = fmaf(a[i], s, 0.5f);
    }
    float r = 0.f;
#pragma unroll
    for (int i = 0; i < 16; ++i) r += a[i];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = r;
}

}  // namespace bqa

extern "C" int32_t bqa_fp32_fma_probe(int32_t blocks, int32_t iters, float* out, void* stream) {
    if (blocks < 1 || iters < 1 || !out) return bqa::set_error(BQA_ERR_ARG, "bqa_fp32_fma_probe: bad argument");
    bqa::fma_probe_kernel<<<blocks, 256, 0, bqa::as_stream(stream)>>>(out, iters, 0.999f);
    return bqa::check_launch("fp32_fma_probe");
}
