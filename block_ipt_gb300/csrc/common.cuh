// common.cuh - shared definitions for the GB300 block-IPT library.
//
// Everything here is internal; the exported C ABI lives in abi.cu and is
// declared in include/ipt_cuda.h and include/ipt_block.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <cstddef>

#include "../../include/ipt_cuda.h"

namespace iptgb {

// Launch geometry shared by the element-wise kernels.
constexpr int kThreads = 256;

inline int blocks_for(size_t count, int threads = kThreads)
{
    size_t b = (count + (size_t)threads - 1) / (size_t)threads;
    if (b == 0) {
        b = 1;
    }
    return (int)b;
}

// Error propagation: every internal call returns an IPT_CUDA_* status.
#define IPTGB_CUDA(call)                                                        \
    do {                                                                        \
        cudaError_t iptgb_err_ = (call);                                        \
        if (iptgb_err_ != cudaSuccess) {                                        \
            fprintf(stderr, "ipt_gb300: CUDA error at %s:%d: %s\n", __FILE__,   \
                    __LINE__, cudaGetErrorString(iptgb_err_));                  \
            return IPT_CUDA_CUDA_ERROR;                                         \
        }                                                                       \
    } while (0)

#define IPTGB_CHECK(expr)                                                       \
    do {                                                                        \
        int iptgb_status_ = (expr);                                             \
        if (iptgb_status_ != IPT_CUDA_SUCCESS) {                                \
            return iptgb_status_;                                               \
        }                                                                       \
    } while (0)

// Every kernel launch of the library is followed by IPTGB_LAUNCH(), which
// checks the launch and counts it (ipt_block_launch_count()).
void count_launch();

#define IPTGB_LAUNCH()                                                          \
    do {                                                                        \
        cudaError_t iptgb_err_ = cudaGetLastError();                            \
        if (iptgb_err_ != cudaSuccess) {                                        \
            fprintf(stderr, "ipt_gb300: launch error at %s:%d: %s\n",           \
                    __FILE__, __LINE__, cudaGetErrorString(iptgb_err_));        \
            return IPT_CUDA_CUDA_ERROR;                                         \
        }                                                                       \
        ::iptgb::count_launch();                                                \
    } while (0)

int env_int(const char *name, int default_value);

// Programmatic dependent launch.  A kernel launched by launch_pdl() may start
// while its predecessor in the stream is still running; it calls pdl_wait()
// before it reads anything the predecessor wrote (or writes anything the
// predecessor reads), and pdl_trigger() to let its own successor start early.
// Under a plain launch pdl_wait() returns at once (stream order already
// holds).  Tuning knob IPT_GB300_PDL=0 launches everything in plain order.
__device__ __forceinline__ void pdl_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ void pdl_trigger()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
int launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
               Args &&...args)
{
    static const bool on = env_int("IPT_GB300_PDL", 1) != 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = on ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, static_cast<Args &&>(args)...);
    if (e != cudaSuccess) {
        fprintf(stderr, "ipt_gb300: launch error: %s\n", cudaGetErrorString(e));
        return IPT_CUDA_CUDA_ERROR;
    }
    count_launch();
    return IPT_CUDA_SUCCESS;
}

// Optional per-kernel timing (ipt_block_profile_*): when enabled, the
// instrumented launch sites bracket their kernel with CUDA events on the
// launch stream.  KernelTimerScope records the start in its constructor and
// the stop in its destructor.
enum ProfiledKernel {
    kProfLowpProduct = 0,   // tensor-core / FP32 SIMT block product (low precision)
    kProfLowpUpdate = 1,    // low-precision IPT update
    kProfFp64Product = 2,   // FP64 dense split-K block product
    kProfFp64Update = 3,    // FP64 IPT update / partial sum
    kProfCsrProduct = 4,    // FP64 CSR block product
    kProfSmallEig = 5,      // one-CTA Jacobi eigensolver
    kProfGram = 6,          // FP64 Gram products
    kProfTallGemm = 7,      // FP64 tall-by-small products
    kProfMlp = 8,           // learned-preconditioner kernels
    kProfClusterUpdate = 9, // block-cluster Gauss-Jordan update
    kProfCount = 10
};
bool profile_enabled();
// Phase marks (ipt_block_trace_*): when enabled, a one-thread kernel writes
// the GPU's global timer into the next slot in stream order and the host
// clock at the call is kept beside it, so the gaps where the GPU waits for
// the host show up.  label must be a string literal.
void trace_mark(const char *label, cudaStream_t s);
struct KernelTimerScope {
    int kernel;
    cudaStream_t stream;
    cudaEvent_t start = nullptr;
    KernelTimerScope(int k, cudaStream_t s);
    ~KernelTimerScope();
};

// A device buffer released by its destructor (stream-ordered when possible).
// Keep memory freed to the current device's stream-ordered pool instead of
// returning it to the driver at every synchronisation (the pool's default),
// so repeated solves reuse their scratch; once per device and process.
void retain_pool_memory();

template <typename T>
struct DeviceBuffer {
    T *ptr = nullptr;
    size_t count = 0;
    cudaStream_t stream = nullptr;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    ~DeviceBuffer() { release(); }
    int alloc(size_t n, cudaStream_t s)
    {
        retain_pool_memory();
        release();
        stream = s;
        count = n;
        if (n == 0) {
            return IPT_CUDA_SUCCESS;
        }
        cudaError_t e = cudaMallocAsync((void **)&ptr, n * sizeof(T), s);
        if (e != cudaSuccess) {
            ptr = nullptr;
            count = 0;
            fprintf(stderr, "ipt_gb300: cudaMallocAsync(%zu bytes) failed: %s\n",
                    n * sizeof(T), cudaGetErrorString(e));
            return IPT_CUDA_CUDA_ERROR;
        }
        return IPT_CUDA_SUCCESS;
    }
    void release()
    {
        if (ptr != nullptr) {
            cudaFreeAsync(ptr, stream);
            ptr = nullptr;
            count = 0;
        }
    }
    T *release_ownership()
    {
        T *p = ptr;
        ptr = nullptr;
        count = 0;
        return p;
    }
};

// Environment knobs keep the reference's names and parsing rules
// (IPT_C_GPU/src/ipt_cuda.cu:18-73).
double env_double(const char *name, double default_value);
int env_int(const char *name, int default_value);
int env_flag(const char *name, int default_value);

}  // namespace iptgb
