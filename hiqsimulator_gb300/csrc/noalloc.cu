// hqs_probability_noalloc: the probability reduction for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc: code running inside another
// framework's memory pool or arena (which owns all device memory and forbids
// raw allocations), code that must not synchronize the device (cudaMalloc /
// cudaFree can), and launch sequences that are recorded once and replayed.
// For them this entry point computes the same sum as hqs_probability without
// any allocation: its per-CTA partial sums live in a fixed, file-scope
// __device__ array (kNoAllocParts doubles = 32 KiB, held by every GPU that
// loads libhqs.so until the process exits), and the caller passes the state
// and a device pointer for the result.
//
// Work split: a grid-stride sum over the matching amplitudes with at most
// min(kNoAllocParts, 8 CTAs per SM) CTAs, so a small query still spreads
// over every SM and a large one never needs more partial sums than the array
// holds. The largest state accepted is 2^40 amplitudes; beyond that the call
// fails with a clear error before any launch.
//
// Sharing: every call on a device uses the same array and the finishing
// kernel reads only the slots that call's sum kernel wrote, so nothing needs
// clearing between calls; calls that overlap on the GPU (different streams,
// or different host threads without ordering) race on the array.
// Set-up: the first call on each device looks the array's device address up
// with cudaGetSymbolAddress (with that device current) and keeps it for the
// process; make that first call before capturing any stream, and do not use
// the entry point on a device after cudaDeviceReset (the kept address would
// belong to the destroyed context).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/hqs.h"
#include "hqs_arith.cuh"
#include "hqs_desc.h"

namespace hqs {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int kNoAllocParts = 4096;
constexpr int kNoAllocMaxQubits = 40;
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocParts];

std::mutex g_setup_mu;
double* g_partials_addr[kMaxDevices] = {nullptr};
int g_sm_count[kMaxDevices] = {0};

struct NoAllocMask {
    uint64_t val;
    int npos;
    uint8_t pos[64];
};

__device__ __forceinline__ uint64_t insert_zero_na(uint64_t v, int p) {
    const uint64_t low = v & ((1ULL << p) - 1ULL);
    return ((v - low) << 1) | low;
}

// CTA b sums matching amplitudes j = b*256 + t, b*256 + t + grid*256, ...
// (j-th amplitude with (i & mask) == val) and writes partials[b].
template <class NA, class S>
__global__ void __launch_bounds__(kThreads) prob_chunk_kernel(const S* __restrict__ state, uint64_t count,
                                                              const __grid_constant__ NoAllocMask m,
                                                              double* __restrict__ partials) {
    __shared__ double red[kThreads / 32];
    NA acc;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count; j += stride) {
        uint64_t i = j;
        for (int b = 0; b < m.npos; ++b) i = insert_zero_na(i, m.pos[b]);
        acc.add(state[i | m.val]);
    }
    double v = acc.value();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w];
        partials[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kThreads) prob_finish_kernel(const double* __restrict__ partials, int nparts,
                                                               double* __restrict__ out) {
    __shared__ double red[kThreads / 32];
    double v = 0.0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) v += partials[p];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w];
        *out = s;
    }
}

int fail(int code, const std::string& msg) {
    hqs::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" int hqs_probability_noalloc(const void* state, int n, int arith, uint64_t mask, uint64_t val,
                                       double* d_out, void* stream) {
    if (!state || !d_out) return fail(HQS_ERR_INVALID, "hqs_probability_noalloc: null state or output pointer");
    if (n < 0 || n > kNoAllocMaxQubits)
        return fail(HQS_ERR_INVALID, "hqs_probability_noalloc: n out of range (states of at most 2^40 amplitudes)");
    if (arith < HQS_ARITH_F64 || arith > HQS_ARITH_TC64)
        return fail(HQS_ERR_INVALID, "hqs_probability_noalloc: unknown arithmetic");
    if ((mask >> n) != 0) return fail(HQS_ERR_INVALID, "hqs_probability_noalloc: mask out of range");
    NoAllocMask m;
    m.val = val & mask;
    m.npos = 0;
    for (int b = 0; b < 64; ++b)
        if ((mask >> b) & 1ULL) m.pos[m.npos++] = (uint8_t)b;
    const uint64_t count = (1ULL << n) >> m.npos;

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(HQS_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(HQS_ERR_INVALID, "hqs_probability_noalloc: device ordinal too large");
    double* partials = nullptr;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_partials_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_partials);
            if (e != cudaSuccess)
                return fail(HQS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            int c = 0;
            e = cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess)
                return fail(HQS_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
            g_sm_count[dev] = c > 0 ? c : 1;
            g_partials_addr[dev] = static_cast<double*>(p);
        }
        partials = g_partials_addr[dev];
        sms = g_sm_count[dev];
    }
    // CTAs: enough for 8 per SM, no more than the array's slots, no more
    // than one per 256 matching amplitudes
    const uint64_t want = (count + kThreads - 1) / kThreads;
    const unsigned grid =
        (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, std::min<uint64_t>((uint64_t)sms * 8, kNoAllocParts)));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (arith == HQS_ARITH_F64)
        prob_chunk_kernel<hqs::NormAccF64, double2><<<grid, kThreads, 0, s>>>((const double2*)state, count, m, partials);
    else if (arith == HQS_ARITH_DF || arith == HQS_ARITH_TC)
        prob_chunk_kernel<hqs::NormAccDF, double2><<<grid, kThreads, 0, s>>>((const double2*)state, count, m, partials);
    else
        prob_chunk_kernel<hqs::NormAccDF, float2><<<grid, kThreads, 0, s>>>((const float2*)state, count, m, partials);
    prob_finish_kernel<<<1, kThreads, 0, s>>>(partials, (int)grid, d_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(HQS_ERR_CUDA, std::string("hqs_probability_noalloc launch: ") + cudaGetErrorString(e));
    return HQS_OK;
}
