// sgb_common.cuh -- shared helpers of libsinogb300.so: status/error plumbing, device
// buffers, launch accounting.  Internal header (the public ABI is include/sinogb300.h).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <atomic>
#include <string>
#include <vector>

#include "sinogb300.h"

namespace sgb {

// Per-thread message of the last failure, returned by sgb_last_error().
void set_error(const char *fmt, ...);
void clear_error();
const std::string &last_error();

extern std::atomic<long long> g_launches;
// device allocations made by the library (DevBuf::reserve is its only cudaMalloc)
extern std::atomic<long long> g_device_allocs;

// Status from a CUDA call; records the failing expression.
#define SGB_CUDA(expr)                                                                        \
    do {                                                                                      \
        cudaError_t _e = (expr);                                                              \
        if (_e != cudaSuccess) {                                                              \
            sgb::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__,  \
                           __LINE__);                                                         \
            return _e == cudaErrorMemoryAllocation ? SGB_ERR_NOMEM : SGB_ERR_CUDA;            \
        }                                                                                     \
    } while (0)

#define SGB_TRY(expr)                 \
    do {                              \
        int _s = (expr);              \
        if (_s != SGB_OK) return _s;  \
    } while (0)

#define SGB_REQUIRE(cond, ...)                 \
    do {                                       \
        if (!(cond)) {                         \
            sgb::set_error(__VA_ARGS__);       \
            return SGB_ERR_ARG;                \
        }                                      \
    } while (0)

// Checks the launch of the kernel just issued and counts it.
inline int after_launch(const char *name) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("launch of %s failed: %s", name, cudaGetErrorString(e));
        return SGB_ERR_CUDA;
    }
    return SGB_OK;
}

// Owning device allocation (stream-ordered free is not needed: callers sync first).
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    // Grows to at least n bytes (keeps the allocation when already large enough).
    int reserve(size_t n) {
        if (n <= bytes && p) return SGB_OK;
        release();
        if (n == 0) return SGB_OK;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            set_error("cudaMalloc(%zu) failed: %s", n, cudaGetErrorString(e));
            return SGB_ERR_NOMEM;
        }
        g_device_allocs.fetch_add(1, std::memory_order_relaxed);
        bytes = n;
        return SGB_OK;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

// Device view of a bulk array that may live on the host: copies in on demand.
inline int stage_in(const void *src, size_t bytes, int flags, DevBuf &tmp, const void **dev,
                    cudaStream_t st) {
    if (flags & SGB_DEVICE_PTRS) {
        *dev = src;
        return SGB_OK;
    }
    SGB_TRY(tmp.reserve(bytes));
    SGB_CUDA(cudaMemcpyAsync(tmp.p, src, bytes, cudaMemcpyHostToDevice, st));
    *dev = tmp.p;
    return SGB_OK;
}

inline int finish(int flags, cudaStream_t st) {
    if ((flags & SGB_ASYNC) && (flags & SGB_DEVICE_PTRS)) return SGB_OK;
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

// Upload a small host vector converted to float.
int upload_f32(const double *src, size_t n, double scale, DevBuf &dst, cudaStream_t st);

inline __host__ __device__ int floor_div_up(int a, int b) { return (a + b - 1) / b; }

#ifdef __CUDACC__
__device__ __forceinline__ float ld_proj(const float *p) { return __ldg(p); }
__device__ __forceinline__ float ld_proj(const __nv_bfloat16 *p) {
    return __bfloat162float(__ldg(p));
}
#endif

}  // namespace sgb
