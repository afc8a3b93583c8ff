// Measurement-only probes, built into their own library (libbqa_gb300_probes.so, declared in
// include/bqa_gb300_probes.h) so that the backend's ABI holds only the hot path.
//
// FP32 FMA throughput probe: the compute ceiling of the complex64 CUDA-core kernels.
// Every thread runs 16 independent FMA chains (no memory traffic in the loop) and writes one
// sum so the work cannot be removed; FLOPs = 2 * 16 * iters * blocks * 256.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bqa_gb300_probes.h"

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

// Warp-level MMA throughput probe: every warp runs 8 independent accumulator chains of
// mma.sync on register operands (kind 0: m16n8k16 bf16 -> f32, 4096 FLOP each; kind 1:
// m16n8k8 tf32 -> f32, 2048 FLOP each) and each thread writes one sum.  FLOPs =
// flop_per_mma * 8 * iters * blocks * 8 warps.  It gives the legacy tensor path's ceiling next
// to the FP32 one: the ceilings a tensor-core message contraction would run against.
template <int KIND>
__global__ void __launch_bounds__(256) mma_probe_kernel(float* __restrict__ out, int iters) {
    const unsigned a0 = 0x3f803f80u ^ threadIdx.x, a1 = 0x3f803f80u, a2 = 0x3f803f80u, a3 = 0x3f803f80u;
    const unsigned b0 = 0x3c003c00u, b1 = 0x3c003c00u;
    float c[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) c[j][q] = 0.f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if constexpr (KIND == 0)
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};"
                    : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
                    : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
            else
                asm volatile(
                    "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};"
                    : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
                    : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
        }
    }
    float r = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) r += c[j][q];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = r;
}

}  // namespace bqa

static int32_t launch_status() { return cudaGetLastError() == cudaSuccess ? 0 : 3; }

extern "C" int32_t bqa_mma_probe(int32_t kind, int32_t blocks, int32_t iters, float* out, void* stream) {
    if (blocks < 1 || iters < 1 || !out || (kind != 0 && kind != 1)) return 1;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (kind == 0) bqa::mma_probe_kernel<0><<<blocks, 256, 0, st>>>(out, iters);
    else bqa::mma_probe_kernel<1><<<blocks, 256, 0, st>>>(out, iters);
    return launch_status();
}

extern "C" int32_t bqa_fp32_fma_probe(int32_t blocks, int32_t iters, float* out, void* stream) {
    if (blocks < 1 || iters < 1 || !out) return 1;
    bqa::fma_probe_kernel<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(out, iters, 0.999f);
    return launch_status();
}
