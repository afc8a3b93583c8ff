/*
 * bqa_gb300 measurement probes (libbqa_gb300_probes.so) -- not part of the backend's ABI; no
 * counterpart in the reference.  bench.py uses them to report the GPU's FP32 CUDA-core and
 * warp-level tensor-core ceilings next to the kernels' achieved rates.  Return 0 on success,
 * 1 for a bad argument, 3 when the launch failed.
 */
#ifndef BQA_GB300_PROBES_H
#define BQA_GB300_PROBES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/*
 * FP32 FMA throughput: `blocks` CTAs of 256 threads each run 16 independent FMA chains for
 * `iters` iterations, 2 * 16 * iters * blocks * 256 FLOP in all, and write one float per thread
 * to out[blocks * 256].  Timed by the caller, it gives the FP32 CUDA-core peak.
 */
int32_t bqa_fp32_fma_probe(int32_t blocks, int32_t iters, float* out, void* stream);

/*
 * Warp-level tensor-core throughput: `blocks` CTAs of 256 threads, every warp running 8
 * independent mma.sync accumulator chains for `iters` iterations on register operands -- kind 0:
 * m16n8k16 bf16 inputs, f32 accumulate (4096 FLOP per instruction); kind 1: m16n8k8 tf32 (2048
 * FLOP).  FLOPs = per-instruction FLOP * 8 * iters * blocks * 8; one float per thread goes to
 * out[blocks * 256].
 */
int32_t bqa_mma_probe(int32_t kind, int32_t blocks, int32_t iters, float* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* BQA_GB300_PROBES_H */
