// profile.cu - launch counter and optional per-kernel event timing.
#include <atomic>
#include <chrono>
#include <mutex>
#include <vector>

#include "common.cuh"

#define IPT_API extern "C" __attribute__((visibility("default")))

namespace iptgb {

namespace {
std::atomic<long long> g_launches{0};
std::atomic<bool> g_profile{false};
std::mutex g_mu;
struct Pending {
    int kernel;
    cudaEvent_t a, b;
};
std::vector<Pending> g_pending;
double g_ms[kProfCount] = {};
long long g_count[kProfCount] = {};
const char *kNames[kProfCount] = {"lowp_product", "lowp_update", "fp64_product", "fp64_update",
                                  "csr_product", "small_eig", "gram", "tall_gemm", "mlp",
                                  "cluster_update"};

void drain_locked()
{
    for (auto &p : g_pending) {
        float ms = 0.0f;
        if (cudaEventSynchronize(p.b) == cudaSuccess &&
            cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            g_ms[p.kernel] += ms;
            g_count[p.kernel] += 1;
        }
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    g_pending.clear();
}
}  // namespace

void count_launch()
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

bool profile_enabled()
{
    return g_profile.load(std::memory_order_relaxed);
}

KernelTimerScope::KernelTimerScope(int k, cudaStream_t s) : kernel(k), stream(s)
{
    if (profile_enabled() && cudaEventCreate(&start) == cudaSuccess) {
        cudaEventRecord(start, stream);
    } else {
        start = nullptr;
    }
}

KernelTimerScope::~KernelTimerScope()
{
    if (start == nullptr) {
        return;
    }
    cudaEvent_t stop = nullptr;
    if (cudaEventCreate(&stop) != cudaSuccess) {
        cudaEventDestroy(start);
        return;
    }
    cudaEventRecord(stop, stream);
    std::lock_guard<std::mutex> lock(g_mu);
    g_pending.push_back({kernel, start, stop});
    if (g_pending.size() > 4096) {
        drain_locked();
    }
}

// ---- phase marks -----------------------------------------------------------
namespace {
constexpr int kTraceSlots = 4096;
std::atomic<bool> g_trace{false};
unsigned long long *g_trace_dev = nullptr;  // kTraceSlots GPU timestamps (ns)
struct TraceMark {
    const char *label;
    long long host_ns;
};
std::vector<TraceMark> g_marks;

long long host_now_ns()
{
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

__global__ void trace_mark_kernel(unsigned long long *slot)
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *slot = t;
}
}  // namespace

void trace_mark(const char *label, cudaStream_t s)
{
    if (!g_trace.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_trace_dev == nullptr || g_marks.size() >= (size_t)kTraceSlots) return;
    g_marks.push_back({label, host_now_ns()});
    trace_mark_kernel<<<1, 1, 0, s>>>(g_trace_dev + (g_marks.size() - 1));
}

}  // namespace iptgb

using namespace iptgb;

IPT_API int ipt_block_trace_enable(int on)
{
    std::lock_guard<std::mutex> lock(g_mu);
    g_marks.clear();
    if (on != 0 && g_trace_dev == nullptr) {
        if (cudaMalloc(&g_trace_dev, kTraceSlots * sizeof(unsigned long long)) != cudaSuccess) {
            g_trace_dev = nullptr;
            return IPT_CUDA_ALLOCATION_FAILED;
        }
    }
    g_trace.store(on != 0);
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_trace_count(void)
{
    std::lock_guard<std::mutex> lock(g_mu);
    return (int)g_marks.size();
}

IPT_API int ipt_block_trace_read(int count, const char **labels, long long *host_ns,
                                 long long *gpu_ns)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (count < 0 || count > (int)g_marks.size() || (count > 0 && g_trace_dev == nullptr)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    std::vector<unsigned long long> t((size_t)count);
    if (count > 0 && cudaMemcpy(t.data(), g_trace_dev, (size_t)count * sizeof(t[0]),
                                cudaMemcpyDeviceToHost) != cudaSuccess) {
        return IPT_CUDA_CUDA_ERROR;
    }
    for (int i = 0; i < count; ++i) {
        if (labels != nullptr) labels[i] = g_marks[(size_t)i].label;
        if (host_ns != nullptr) host_ns[i] = g_marks[(size_t)i].host_ns;
        if (gpu_ns != nullptr) gpu_ns[i] = (long long)t[(size_t)i];
    }
    return IPT_CUDA_SUCCESS;
}

IPT_API long long ipt_block_launch_count(void)
{
    return g_launches.load();
}

IPT_API void ipt_block_profile_enable(int on)
{
    std::lock_guard<std::mutex> lock(g_mu);
    drain_locked();
    g_profile.store(on != 0);
}

IPT_API void ipt_block_profile_reset(void)
{
    std::lock_guard<std::mutex> lock(g_mu);
    drain_locked();
    for (int i = 0; i < kProfCount; ++i) {
        g_ms[i] = 0.0;
        g_count[i] = 0;
    }
}

IPT_API int ipt_block_profile_read(int kernel, const char **name, double *total_ms,
                                   long long *launches)
{
    if (kernel < 0 || kernel >= kProfCount) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    drain_locked();
    if (name != nullptr) *name = kNames[kernel];
    if (total_ms != nullptr) *total_ms = g_ms[kernel];
    if (launches != nullptr) *launches = g_count[kernel];
    return IPT_CUDA_SUCCESS;
}

namespace iptgb {
void retain_pool_memory()
{
    static std::atomic<unsigned long long> done_mask{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    const unsigned long long bit = 1ULL << dev;
    if (done_mask.load(std::memory_order_acquire) & bit) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long threshold = ~0ULL;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
    done_mask.fetch_or(bit, std::memory_order_acq_rel);
}
}  // namespace iptgb

// FP32 FMA throughput of this GPU (same shape as the FP64 probe below); the
// denominator of kernels bound by the FP32 pipe.
__global__ void ffma_probe_kernel(float *out, int iters, float a, float b)
{
    float acc[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c] = (float)(threadIdx.x + c);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < 16; ++c) acc[c] = fmaf(acc[c], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < 16; ++c) s += acc[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

IPT_API int ipt_block_measure_fp32_peak(double *tflops)
{
    if (tflops == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    int dev = 0, sms = 0;
    IPTGB_CUDA(cudaGetDevice(&dev));
    IPTGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = 8 * sms, threads = 256, iters = 65536;
    float *out = nullptr;
    IPTGB_CUDA(cudaMalloc((void **)&out, sizeof(float) * blocks * threads));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    ffma_probe_kernel<<<blocks, threads>>>(out, iters, 0.9999999f, 1e-7f);
    cudaEventRecord(a);
    ffma_probe_kernel<<<blocks, threads>>>(out, iters, 0.9999999f, 1e-7f);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const cudaError_t e = cudaGetLastError();
    cudaFree(out);
    if (e != cudaSuccess || ms <= 0.0f) return IPT_CUDA_CUDA_ERROR;
    count_launch();
    count_launch();
    *tflops = 2.0 * 16.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    return IPT_CUDA_SUCCESS;
}

// FP64 FMA throughput of this GPU: 16 independent DFMA chains per thread,
// 4 blocks of 256 threads per SM.  Used as the FP64 roofline denominator.
__global__ void dfma_probe_kernel(double *out, int iters, double a, double b)
{
    double acc[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c] = (double)(threadIdx.x + c);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < 16; ++c) acc[c] = fma(acc[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 16; ++c) s += acc[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

IPT_API int ipt_block_measure_fp64_peak(double *tflops)
{
    if (tflops == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    int dev = 0, sms = 0;
    IPTGB_CUDA(cudaGetDevice(&dev));
    IPTGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = 4 * sms, threads = 256, iters = 4096;
    double *out = nullptr;
    IPTGB_CUDA(cudaMalloc((void **)&out, sizeof(double) * blocks * threads));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    dfma_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(a);
    dfma_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const cudaError_t e = cudaGetLastError();
    cudaFree(out);
    if (e != cudaSuccess || ms <= 0.0f) return IPT_CUDA_CUDA_ERROR;
    count_launch();
    count_launch();
    *tflops = 2.0 * 16.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    return IPT_CUDA_SUCCESS;
}
