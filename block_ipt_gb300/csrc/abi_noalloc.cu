// abi_noalloc.cu - the FP64 dense IPT solve with no device allocation.
//
// Some callers cannot let a library call cudaMalloc / cudaFree: applications
// that hand all device memory to their own pool or caching allocator and
// budget it up front, services that forbid allocation after start-up so that
// a long-running process cannot fail or fragment mid-flight, and
// asynchronous pipelines in which the device-wide synchronisation implied by
// cudaFree would stall other streams.  ipt_cuda_device_tol_noalloc serves
// them: the caller passes the matrix and the output buffers, and every piece
// of scratch (the second iterate, the diagonal, the split-K partial slices
// of H X and the norm-reduction slots) lives in one file-scope __device__
// array of kNoallocScratchBytes (16 MiB) that every GPU which loads this
// library holds until the process exits.
//
// Host code may not use the array's name as a device address; the address
// is looked up with cudaGetSymbolAddress on every call, with the caller's
// device current (a cheap host call, and it stays valid after a
// cudaDeviceReset reloads the module).  Every iteration reads the two norms
// back and synchronises the stream, so the entry must never be called inside
// a stream capture.  All calls share the one array and it keeps the last
// call's contents: the parts that must start at zero are cleared on every
// call, and calls that overlap on the GPU (two streams, two threads, one
// device) race on the scratch and must be serialised by the caller.
#include <math.h>

#include <climits>

#include "common.cuh"
#include "kernels.cuh"

#define IPT_API extern "C" __attribute__((visibility("default")))

namespace iptgb {
namespace {

constexpr size_t kNoallocScratchBytes = 16u << 20;  // 16 MiB
constexpr size_t kNoallocDoubles = kNoallocScratchBytes / sizeof(double);

__device__ __align__(256) double g_noalloc_scratch[kNoallocDoubles];

// Device address of the scratch array for the current device, looked up on
// every call: a cached address would dangle once cudaDeviceReset has
// reloaded the module.
int scratch_for_current_device(double **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
        fprintf(stderr, "ipt_gb300: cudaGetSymbolAddress(no-alloc scratch) failed: %s\n",
                cudaGetErrorString(e));
        return IPT_CUDA_CUDA_ERROR;
    }
    *out = static_cast<double *>(p);
    return IPT_CUDA_SUCCESS;
}

size_t align_doubles(size_t count)
{
    return (count + 31) & ~(size_t)31;  // keep every carve-out 256-byte aligned
}

}  // namespace
}  // namespace iptgb

using namespace iptgb;

IPT_API int ipt_cuda_device_tol_noalloc(const double *d_matrix_col_major, int n, int k,
                                        double tol, int maxiter, void *stream,
                                        double *d_vectors, double *d_values,
                                        int *iterations_done_out,
                                        double *fixed_point_residual_out)
{
    if (iterations_done_out != nullptr) *iterations_done_out = 0;
    if (fixed_point_residual_out != nullptr) *fixed_point_residual_out = NAN;
    if (d_matrix_col_major == nullptr || d_vectors == nullptr || d_values == nullptr || n <= 0 ||
        k <= 0 || k > n || !(tol > 0.0) || maxiter <= 0) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    const size_t elems = (size_t)n * (size_t)k;
    if (elems > (size_t)INT_MAX) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    // Scratch layout (doubles): second iterate | diagonal | norm slots |
    // ticket counter + two norms | S partial slices of H X.
    const size_t norm_slots = (size_t)blocks_for(elems);
    const size_t fixed = align_doubles(elems) + align_doubles((size_t)n) +
                         align_doubles(2 * norm_slots) + align_doubles(4);
    if (fixed + align_doubles(elems) > kNoallocDoubles) {
        fprintf(stderr,
                "ipt_gb300: ipt_cuda_device_tol_noalloc: n*k = %zu needs more than the %zu-byte "
                "static scratch (limit: 2*n*k + n + n*k/128 doubles, roughly n*k <= 1.0e6)\n",
                elems, kNoallocScratchBytes);
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    int S = dense64_split_for(n, k, 148);
    {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            sms > 0) {
            S = dense64_split_for(n, k, sms);
        }
    }
    const size_t slice = align_doubles(elems);
    const size_t room = (kNoallocDoubles - fixed) / slice;
    if ((size_t)S > room) {
        S = (int)room;  // fewer, deeper K slices: same result up to rounding
    }

    double *base = nullptr;
    IPTGB_CHECK(scratch_for_current_device(&base));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *xb = base;
    double *d = xb + align_doubles(elems);
    double2 *slots = reinterpret_cast<double2 *>(d + align_doubles((size_t)n));
    unsigned int *counter = reinterpret_cast<unsigned int *>(
        reinterpret_cast<double *>(slots) + align_doubles(2 * norm_slots));
    double *norms = reinterpret_cast<double *>(counter) + 2;
    double *P = reinterpret_cast<double *>(counter) + align_doubles(4);

    NormScratch ns;
    ns.partials = slots;
    ns.capacity = (int)norm_slots;
    ns.counter = counter;
    ns.norms = norms;
    // the ticket counter must start at zero (the array keeps the last call's contents)
    IPTGB_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s));
    IPTGB_CHECK(launch_set_identity(d_vectors, n, k, s));
    IPTGB_CHECK(launch_extract_diagonal(d_matrix_col_major, n, n, d, s));

    // The reference's tolerance loop (IPT_C_GPU/src/ipt_cuda.cu:1644-1703),
    // ping-ponging between the caller's output buffer and the scratch iterate.
    double *x = d_vectors;
    double *y = xb;
    int done = 0;
    double fpres = NAN;
    double host_norms[2] = {0.0, 0.0};
    for (int iter = 0; iter < maxiter; ++iter) {
        IPTGB_CHECK(launch_dense64_partial(d_matrix_col_major, n, n, x, n, k, P, S, s));
        IPTGB_CHECK(launch_dense64_update(P, S, n, k, x, d, y, 1, &ns, s));
        done = iter + 1;
        IPTGB_CUDA(cudaMemcpyAsync(host_norms, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                   s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
        if (host_norms[1] <= 0.0 || !isfinite(host_norms[1])) {
            return IPT_CUDA_INVALID_ARGUMENT;
        }
        fpres = host_norms[0] / host_norms[1];
        double *t = x;
        x = y;
        y = t;
        if (fpres <= tol) {
            break;
        }
    }
    if (x != d_vectors) {
        IPTGB_CUDA(cudaMemcpyAsync(d_vectors, x, elems * sizeof(double), cudaMemcpyDeviceToDevice,
                                   s));
    }
    IPTGB_CHECK(launch_dense64_diag_values(d_matrix_col_major, n, n, d_vectors, k, d_values, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    if (iterations_done_out != nullptr) *iterations_done_out = done;
    if (fixed_point_residual_out != nullptr) *fixed_point_residual_out = fpres;
    return IPT_CUDA_SUCCESS;
}
