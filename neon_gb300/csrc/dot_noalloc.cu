// Allocation-free FP64-accumulated dot product.
//
// Some callers cannot allocate device memory at the point where they need a
// reduction: code that runs between the launches of a stream-ordered
// pipeline, where cudaMalloc/cudaFree would synchronise the device, and host
// plug-ins whose device memory is owned and sized by the host application.
// ngb_dot_noalloc serves them: it computes the same FP64-accumulated dot as
// ngb_dot, but keeps its per-CTA partial sums in a fixed array in this
// library's global memory instead of caller scratch, and calls no cudaMalloc,
// cudaFree or allocating library routine.
//
// The array is g_dot_noalloc_scratch below: kNoallocMaxPartials doubles
// (256 KiB) plus one ticket word, held by every GPU that loads the library
// until the process exits. Each CTA reduces one fixed chunk of kChunk
// elements, so n may be at most kNoallocMaxPartials * kChunk = 2^28 elements;
// larger n is rejected with NGB_ERR_RANGE.
//
// All calls share the array and it keeps the last call's contents: the ticket
// word is cleared on the stream before every launch, and two calls whose
// kernels overlap on the GPU (different streams, no ordering) race on it and
// on the partials.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in), so each call looks up the device address with
// cudaGetSymbolAddress in the CUDA context current on the calling thread: the
// array exists once per context (the device's primary context, or a context
// a driver-API host made current), and an address taken in one context is not
// mapped in another, nor after cudaDeviceReset. A call made while its stream
// is being captured cannot do that lookup, so it uses the address that the
// last uncaptured call saw in the same context (kept per context handle). The
// first call in a context may load the module lazily: make it before any
// stream capture in that context.
#include "common.cuh"
#include <cuda.h>
#include <mutex>
#include <utility>
#include <vector>

namespace ngb {
namespace {

constexpr int     kNoallocThreads = 256;
constexpr int     kNoallocPerThread = 32;
constexpr int64_t kChunk = int64_t(kNoallocThreads) * kNoallocPerThread;  // elements per CTA
constexpr int     kNoallocMaxPartials = 32768;
constexpr int64_t kNoallocMaxN = int64_t(kNoallocMaxPartials) * kChunk;    // 2^28

// partials[0 .. kNoallocMaxPartials), then the ticket word in the last slot.
static __device__ __align__(256) double g_dot_noalloc_scratch[kNoallocMaxPartials + 1];

// (context handle, device address) of the lookups made outside stream capture.
std::mutex                                  g_setup_mutex;
std::vector<std::pair<CUcontext, double*>>  g_scratch_addr;
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
CtxGetCurrentFn                             g_ctx_get_current = nullptr;

template <typename T>
__global__ void __launch_bounds__(kNoallocThreads) dot_noalloc_kernel(int64_t n, const T* __restrict__ a, const T* __restrict__ b,
                                                                      double* __restrict__ result, double* scratch)
{
    __shared__ double       red[kNoallocThreads];
    __shared__ unsigned int ticket;
    unsigned int*           tick = reinterpret_cast<unsigned int*>(scratch + kNoallocMaxPartials);
    const int64_t           base = int64_t(blockIdx.x) * kChunk;
    double                  acc = 0.0;
#pragma unroll 4
    for (int k = 0; k < kNoallocPerThread; k++) {
        const int64_t i = base + int64_t(k) * kNoallocThreads + threadIdx.x;
        if (i < n) acc += double(a[i]) * double(b[i]);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kNoallocThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = red[0];
        __threadfence();
        ticket = atomicAdd(tick, 1u);
    }
    __syncthreads();
    if (ticket != gridDim.x - 1) return;  // not the last CTA: done, nothing waits
    __threadfence();
    double s = 0.0;
    for (unsigned c = threadIdx.x; c < gridDim.x; c += kNoallocThreads) s += __ldcg(scratch + c);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kNoallocThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *result = red[0];
        *tick = 0u;
    }
}

// Device address of the scratch array in the calling thread's current
// context. Outside capture: looked up afresh and remembered for the context;
// under capture: the remembered address of the same context.
int scratch_address(cudaStream_t s, double** out)
{
    // first runtime call: binds the device's primary context to the thread
    // unless the caller made another context current
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    NGB_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_ctx_get_current) {
        void*                           fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        NGB_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !fn) {
            set_error("ngb_dot_noalloc: cuCtxGetCurrent not available from the driver");
            return NGB_ERR_CUDA;
        }
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) {
        set_error("ngb_dot_noalloc: no current CUDA context");
        return NGB_ERR_CUDA;
    }
    for (auto& e : g_scratch_addr) {
        if (e.first != ctx) continue;
        if (cap == cudaStreamCaptureStatusNone) {
            void* p = nullptr;
            NGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_dot_noalloc_scratch));
            e.second = static_cast<double*>(p);
        }
        *out = e.second;
        return NGB_OK;
    }
    if (cap != cudaStreamCaptureStatusNone) {
        set_error("ngb_dot_noalloc: first call in this CUDA context made under stream capture; "
                  "call it once outside capture first");
        return NGB_ERR_INVALID;
    }
    void* p = nullptr;
    NGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_dot_noalloc_scratch));
    g_scratch_addr.emplace_back(ctx, static_cast<double*>(p));
    *out = static_cast<double*>(p);
    return NGB_OK;
}

}  // namespace
}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_dot_noalloc(int64_t n, int32_t field, const void* a, const void* b, double* result, void* stream)
{
    NGB_CHECK_ARG(n >= 0, "n < 0");
    NGB_CHECK_ARG(field == NGB_STORE_F32 || field == NGB_STORE_F64, "field must be NGB_STORE_F32 or NGB_STORE_F64");
    NGB_CHECK_ARG(result && (n == 0 || (a && b)), "NULL argument");
    if (n > kNoallocMaxN) {
        set_error("n = %lld exceeds the maximum of %lld elements of ngb_dot_noalloc (its fixed scratch holds %d partial sums)",
                  (long long)n, (long long)kNoallocMaxN, kNoallocMaxPartials);
        return NGB_ERR_RANGE;
    }
    cudaStream_t s = as_stream(stream);
    double*      scratch = nullptr;
    int          rc = scratch_address(s, &scratch);
    if (rc) return rc;
    if (n == 0) {
        NGB_CUDA_TRY(cudaMemsetAsync(result, 0, sizeof(double), s));
        return NGB_OK;
    }
    NGB_CUDA_TRY(cudaMemsetAsync(scratch + kNoallocMaxPartials, 0, sizeof(double), s));  // ticket starts at zero
    const unsigned blocks = unsigned((n + kChunk - 1) / kChunk);
    if (field == NGB_STORE_F64)
        dot_noalloc_kernel<double><<<blocks, kNoallocThreads, 0, s>>>(n, static_cast<const double*>(a),
                                                                      static_cast<const double*>(b), result, scratch);
    else
        dot_noalloc_kernel<float><<<blocks, kNoallocThreads, 0, s>>>(n, static_cast<const float*>(a), static_cast<const float*>(b),
                                                                     result, scratch);
    NGB_LAUNCH_CHECK("dot_noalloc_kernel");
    return NGB_OK;
}

}  // extern "C"
