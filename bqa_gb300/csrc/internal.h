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

// ---- packed sweeps ----------------------------------------------------------------------------
//
// While a PackList collects on a host thread, the BP kernels that thread would launch (node
// kernels, combines, decisions, damping) are recorded instead, with their arguments.
// pack_execute then issues the recorded launches phase by phase, and within a phase one launch
// per kernel for all the entries of that kernel (up to the table size), whatever job or class
// they came from.  Each CTA computes what it computes in its own launch, so the outputs are
// the same bits.
struct PackEntry {
    int (*launch)(const PackEntry* entries, int n, cudaStream_t st);   // issues n entries of one kernel
    int phase;   // 0: node kernels, 1: combines, 2: BP decisions, 3: damping
    int key;     // entries of one launcher with the same key share a launch
    int count;   // nodes of the class (node kernels)
    alignas(16) unsigned char args[128];
};

struct PackList {
    PackEntry* items = nullptr;
    int n = 0, cap = 0;
    int error = 0;   // a record that could not be stored (issuing the list then fails with it)
    PackList() = default;
    PackList(const PackList&) = delete;
    PackList& operator=(const PackList&) = delete;
    ~PackList() { delete[] items; }
    void push(const PackEntry& e);
};

// record the launches of this thread into `list` until pack_collect(nullptr)
void pack_collect(PackList* list);
// issue the recorded launches (the list can be issued again: every sweep of a packed BP run)
int pack_execute(const PackList& list, cudaStream_t st);

}  // namespace bqa
