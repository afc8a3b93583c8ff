// Library-wide entry points of the C ABI: version, error text, size limits.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <unordered_map>

#include "internal.h"
#include "../../include/bqa_gb300.h"

namespace bqa {

static thread_local char g_last_error[512] = "";
// kernel launches issued by this library (every launch is followed by check_launch)
static std::atomic<long long> g_launches{0};

int set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

int check_launch(const char* what) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(BQA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return BQA_OK;
}

int ensure_smem(const void* kernel, size_t bytes, const char* what) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> granted;   // (device, kernel) -> bytes
    if (bytes <= 48 * 1024) return BQA_OK;
    if (bytes > kMaxSmem) return set_error(BQA_ERR_UNSUPPORTED, "%s: needs %zu B of shared memory", what, bytes);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(BQA_ERR_CUDA, "%s: cudaGetDevice: %s", what, cudaGetErrorString(e));
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(dev, kernel);
    auto it = granted.find(key);
    if (it != granted.end() && it->second >= bytes) return BQA_OK;
    // the per-block limit covers static and dynamic shared memory together
    cudaFuncAttributes attr;
    e = cudaFuncGetAttributes(&attr, kernel);
    if (e != cudaSuccess) return set_error(BQA_ERR_CUDA, "%s: cudaFuncGetAttributes: %s", what, cudaGetErrorString(e));
    const size_t room = kMaxSmem > attr.sharedSizeBytes ? kMaxSmem - attr.sharedSizeBytes : 0;
    if (bytes > room)
        return set_error(BQA_ERR_UNSUPPORTED, "%s: needs %zu B of dynamic shared memory next to %zu B static",
                         what, bytes, (size_t)attr.sharedSizeBytes);
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)room);
    if (e != cudaSuccess) return set_error(BQA_ERR_CUDA, "%s: cudaFuncSetAttribute: %s", what, cudaGetErrorString(e));
    granted[key] = room;
    return BQA_OK;
}

}  // namespace bqa

extern "C" {

int32_t bqa_abi_version(void) { return 13; }

int64_t bqa_launch_count(void) { return bqa::g_launches.load(std::memory_order_relaxed); }

const char* bqa_last_error(void) { return bqa::g_last_error; }

}  // extern "C"
