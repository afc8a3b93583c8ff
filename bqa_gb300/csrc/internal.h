// Host-side helpers shared by the translation units of libbqa_gb300 (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bqa {

// Record an error message for bqa_last_error() and return `code`.
int set_error(int code, const char* fmt, ...);

// Turn a pending launch error into BQA_ERR_CUDA with the given context.
int check_launch(const char* what);

// Opt a kernel into `bytes` of dynamic shared memory (once per kernel and size bound).
int ensure_smem(const void* kernel, size_t bytes, const char* what);

constexpr size_t kMaxSmem = 227 * 1024;

// shared memory of the generic tensor update at bond dims <= chi, in bytes (update.cu)
size_t apply_smem_bytes(int d, int chi, size_t elem_bytes);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace bqa
