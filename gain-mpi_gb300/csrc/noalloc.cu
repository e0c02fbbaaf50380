// gain_dot_noalloc: the FP64 dot product of gain_dot for callers that cannot allocate
// device memory.  It is a multi-block variant of the single-block dot kernel: every block
// reduces a fixed chunk of GAIN_DOT_NOALLOC_CHUNK elements into one partial sum, and the
// last block to finish adds the partials in block order.  The partials and the completion
// ticket live in a file-scope device array of fixed size (no cudaMalloc, no library that
// allocates); its address is looked up on the first call on each device, with that device
// current, and again whenever the device's context has changed since (after a
// cudaDeviceReset the module is loaded anew and the array may move).
//
// Zero state: the completion ticket must be zero when a launch starts.  It is cleared by a
// stream-ordered memset before every launch (and the last block leaves it at zero), so a
// launch that did not finish cannot poison the next one.  The partials need no clearing:
// each block writes its own before taking a ticket.
//
// The scratch is shared by every call on a device: calls whose kernels overlap on the GPU
// (e.g. on two streams without ordering between them) race on it.
#include <mutex>
#include <utility>

#include <cuda.h>

#include "gain_internal.h"

namespace gain {
namespace {

constexpr int kThreads = 256;
constexpr int kChunk = GAIN_DOT_NOALLOC_CHUNK;
constexpr int kMaxBlocks = GAIN_DOT_NOALLOC_MAX_N / GAIN_DOT_NOALLOC_CHUNK;
static_assert((long long)kMaxBlocks * kChunk == GAIN_DOT_NOALLOC_MAX_N, "whole chunks");

// [0, kMaxBlocks): per-block partial sums; [kMaxBlocks]: the completion ticket (low 32 bits).
// 16384 partials + 1 ticket slot: 131 KB of device memory per device.
constexpr int kScratchWords = kMaxBlocks + 1;
static __device__ __align__(256) double g_dot_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};   // context id the address belongs to

// Unique id of the calling thread's current context (driver entry points, resolved once; 0
// when they are unavailable, which only disables the change check).
unsigned long long current_context_id() {
    typedef CUresult (*GetCurrentFn)(CUcontext*);
    typedef CUresult (*GetIdFn)(CUcontext, unsigned long long*);
    static const std::pair<GetCurrentFn, GetIdFn> fns = []() {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
            qa != cudaDriverEntryPointSuccess)
            a = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
            qb != cudaDriverEntryPointSuccess)
            b = nullptr;
        return std::make_pair((GetCurrentFn)a, (GetIdFn)b);
    }();
    if (!fns.first || !fns.second) return 0ull;
    CUcontext ctx = nullptr;
    unsigned long long id = 0ull;
    if (fns.first(&ctx) != CUDA_SUCCESS || !ctx || fns.second(ctx, &id) != CUDA_SUCCESS) return 0ull;
    return id;
}

__global__ void __launch_bounds__(kThreads) k_dot_blocks(int n, const double* __restrict__ x,
                                                          const double* __restrict__ y, double* result,
                                                          double* scratch) {
    __shared__ double red[kThreads / 32];
    __shared__ bool last;
    const long begin = (long)blockIdx.x * kChunk;
    const long end = begin + kChunk < (long)n ? begin + kChunk : (long)n;
    double acc = 0.0;
    for (long i = begin + threadIdx.x; i < end; i += kThreads) acc = __fma_rn(x[i], y[i], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    unsigned int* ticket = (unsigned int*)(scratch + kMaxBlocks);
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w];
        scratch[blockIdx.x] = s;
        __threadfence();   // the partial is visible before the ticket is taken
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // last block: every partial is visible (each was fenced before its ticket)
    __threadfence();
    acc = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) acc += __ldcg(&scratch[b]);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w];
        *result = s;
        *ticket = 0u;
    }
}

// Address of this device's scratch: looked up on the first call on each device (the device
// is current), and again when the device's context is no longer the one it was found in.
gain_status scratch_for_current_device(double** out) {
    int dev = 0;
    GAIN_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return set_error(GAIN_ERR_UNSUPPORTED, "gain_dot_noalloc: device ordinal %d", dev);
    GAIN_CUDA(cudaSetDevice(dev));   // initialises the device's primary context if a reset dropped it
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
        void* p = nullptr;
        GAIN_CUDA(cudaGetSymbolAddress(&p, g_dot_scratch));
        g_scratch_ptr[dev] = (double*)p;
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_ptr[dev];
    return GAIN_OK;
}

}  // namespace
}  // namespace gain

using namespace gain;

extern "C" gain_status gain_dot_noalloc(int n, const double* x, const double* y, double* result, void* stream) {
    clear_error();
    if (n < 0 || !result || (n > 0 && (!x || !y))) return set_error(GAIN_ERR_INVALID_ARG, "gain_dot_noalloc: bad argument");
    if ((long long)n > GAIN_DOT_NOALLOC_MAX_N)
        return set_error(GAIN_ERR_INVALID_ARG,
                         "gain_dot_noalloc: n = %d exceeds the scratch capacity (at most %lld elements)", n,
                         (long long)GAIN_DOT_NOALLOC_MAX_N);
    double* scratch = nullptr;
    GAIN_TRY(scratch_for_current_device(&scratch));
    const cudaStream_t st = (cudaStream_t)stream;
    const int blocks = n > 0 ? (int)(((long long)n + kChunk - 1) / kChunk) : 1;
    GAIN_CUDA(cudaMemsetAsync(scratch + kMaxBlocks, 0, sizeof(double), st));
    k_dot_blocks<<<blocks, kThreads, 0, st>>>(n, x, y, result, scratch);
    GAIN_CUDA(cudaGetLastError());
    return GAIN_OK;
}
