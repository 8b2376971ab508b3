// common.cuh -- shared plumbing for libpgeof_cuda: status handling, scratch
// memory, launch accounting and the exact-arithmetic helpers that keep device
// results bit-compatible with the reference's float operation order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <string>

#include "pgeof_cuda.h"

namespace pgeof {

// ----------------------------------------------------------------- errors
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
// Wraps a CUDA call: on failure records the message and returns PGEOF_ERR_CUDA
// (or PGEOF_ERR_OUT_OF_MEMORY) from the enclosing function.
#define PGEOF_CUDA_TRY(expr)                                                                     \
    do {                                                                                         \
        cudaError_t _e = (expr);                                                                 \
        if (_e != cudaSuccess) {                                                                 \
            (void)cudaGetLastError();                                                            \
            return ::pgeof::fail(_e == cudaErrorMemoryAllocation ? PGEOF_ERR_OUT_OF_MEMORY       \
                                                                  : PGEOF_ERR_CUDA,              \
                                 std::string(#expr) + ": " + cudaGetErrorString(_e));            \
        }                                                                                        \
    } while (0)

#define PGEOF_TRY(expr)                     \
    do {                                    \
        int _s = (expr);                    \
        if (_s != PGEOF_OK) return _s;      \
    } while (0)

// Device-side data-error bits (see pgeof_take_device_errors).
enum : uint32_t {
    ERR_NN_RANGE = 1u,
    ERR_PTR_RANGE = 2u,
    ERR_INTERNAL = 4u,
};
uint32_t* device_error_word();  // per-device word, zeroed at first use
int noalloc_take_errors(uint32_t* bits);  // reads and clears the no-allocation entry point's word

// ----------------------------------------------------------------- launches
extern std::atomic<uint64_t> g_launch_count;
inline void count_launch(uint64_t n = 1) { g_launch_count.fetch_add(n, std::memory_order_relaxed); }
// device memory allocations made by the library (pool and cudaMalloc)
extern std::atomic<uint64_t> g_device_alloc_count;
inline void count_device_alloc() { g_device_alloc_count.fetch_add(1, std::memory_order_relaxed); }
int check_launch(const char* what);  // cudaGetLastError after a launch

// Brackets the kernel launches of its scope with CUDA events on `s` while
// kernel timing is enabled (pgeof_profile_enable); a no-op otherwise.
extern std::atomic<int> g_profile_on;
struct KernelTimer {
    const char* name;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    KernelTimer(const char* kernel_name, cudaStream_t stream);
    ~KernelTimer();
    KernelTimer(const KernelTimer&) = delete;
    KernelTimer& operator=(const KernelTimer&) = delete;
};

// ----------------------------------------------------------------- device info
struct DeviceInfo {
    int device = -1;
    int sm_count = 0;
    int max_smem_optin = 0;
};
int current_device_info(const DeviceInfo** out);

// Resident blocks per SM of `kernel` at `threads` threads and `smem` bytes of
// dynamic shared memory on the current device, raising the kernel's shared
// memory limit first when smem > 48 KB. Cached per (device, kernel, threads,
// smem), so repeated launches pay no host-side query.
int kernel_blocks_per_sm(const void* kernel, int threads, int smem, int* per_sm);
// Keeps at least 60 KB of each SM's L1 as data cache for `kernel` at this
// launch size: when its resident blocks would fill more than 196 KB of shared
// memory the carveout preference is capped there (fewer resident blocks),
// otherwise the driver's default stands. Random-gather kernels need the data
// cache: every gather in flight holds an L1 sector until it returns, so with
// the 228 KB carveout (28 KB of L1) their throughput halves.
int cap_smem_carveout(const void* kernel, int threads, int smem);

// ----------------------------------------------------------------- scratch
// Stream-ordered scratch allocations from a library-owned memory pool that
// keeps freed blocks cached (no OS round trip per call).
int scratch_alloc(void** p, size_t bytes, cudaStream_t s);
void scratch_free(void* p, cudaStream_t s);

// RAII holder for one scratch block.
struct Scratch {
    void* p = nullptr;
    cudaStream_t s = nullptr;
    Scratch() = default;
    Scratch(const Scratch&) = delete;
    Scratch& operator=(const Scratch&) = delete;
    ~Scratch() { reset(); }
    void reset() {
        if (p) scratch_free(p, s);
        p = nullptr;
    }
    int alloc(size_t bytes, cudaStream_t stream) {
        reset();
        s = stream;
        return scratch_alloc(&p, bytes ? bytes : 16, stream);
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

int eig_order();  // 0 ascending (reference), 1 descending

}  // namespace pgeof

// ----------------------------------------------------------------- exact ops
// The reference runs its float math without FMA contraction (x86-64 Release);
// these keep the same rounding on the device regardless of -fmad.
#define FADD(a, b) __fadd_rn((a), (b))
#define FSUB(a, b) __fsub_rn((a), (b))
#define FMUL(a, b) __fmul_rn((a), (b))
#define FDIV(a, b) __fdiv_rn((a), (b))
#define DADD(a, b) __dadd_rn((a), (b))
#define DSUB(a, b) __dsub_rn((a), (b))
#define DMUL(a, b) __dmul_rn((a), (b))
#define DDIV(a, b) __ddiv_rn((a), (b))

template <typename T>
struct XOps;
template <>
struct XOps<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
};
template <>
struct XOps<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
};

static inline unsigned ceil_div_u(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }
