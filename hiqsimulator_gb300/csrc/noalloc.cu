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
// Limits and sharing: one CTA sums 2^20 matching amplitudes, so a call covers
// at most kNoAllocParts * 2^20 = 2^32 matching amplitudes (for example a full
// 32-qubit state); larger requests are rejected. Every call on a device uses
// the same array and overwrites only the slots it reads back, so nothing needs
// clearing between calls, but calls that overlap on the GPU (different
// streams, or different host threads without ordering) race on it.
// The first call on each device looks the array's device address up with
// cudaGetSymbolAddress (with that device current); make that first call
// before capturing any stream.
#include <cuda_runtime.h>
#include <stdint.h>

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
constexpr uint64_t kNoAllocChunk = 1ULL << 20;  // matching amplitudes per CTA
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocParts];

std::mutex g_setup_mu;
double* g_partials_addr[kMaxDevices] = {nullptr};

struct NoAllocMask {
    uint64_t val;
    int npos;
    uint8_t pos[64];
};

__device__ __forceinline__ uint64_t insert_zero_na(uint64_t v, int p) {
    const uint64_t low = v & ((1ULL << p) - 1ULL);
    return ((v - low) << 1) | low;
}

template <class NA, class S>
__global__ void __launch_bounds__(kThreads) prob_chunk_kernel(const S* __restrict__ state, uint64_t count,
                                                              const __grid_constant__ NoAllocMask m,
                                                              double* __restrict__ partials) {
    __shared__ double red[kThreads / 32];
    NA acc;
    const uint64_t begin = (uint64_t)blockIdx.x * kNoAllocChunk;
    const uint64_t end = (begin + kNoAllocChunk < count) ? begin + kNoAllocChunk : count;
    for (uint64_t j = begin + threadIdx.x; j < end; j += blockDim.x) {
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
    if (n < 0 || n > 40) return fail(HQS_ERR_INVALID, "hqs_probability_noalloc: n out of range");
    if (arith < HQS_ARITH_F64 || arith > HQS_ARITH_TC64)
        return fail(HQS_ERR_INVALID, "hqs_probability_noalloc: unknown arithmetic");
    if (n < 64 && (mask >> n) != 0) return fail(HQS_ERR_INVALID, "hqs_probability_noalloc: mask out of range");
    NoAllocMask m;
    m.val = val & mask;
    m.npos = 0;
    for (int b = 0; b < 64; ++b)
        if ((mask >> b) & 1ULL) m.pos[m.npos++] = (uint8_t)b;
    const uint64_t count = (1ULL << n) >> m.npos;
    const uint64_t nparts = (count + kNoAllocChunk - 1) / kNoAllocChunk;
    if (nparts > (uint64_t)kNoAllocParts)
        return fail(HQS_ERR_INVALID,
                    "hqs_probability_noalloc: at most 2^32 matching amplitudes per call (4096 partial sums of "
                    "2^20 amplitudes in the static scratch); use hqs_probability for larger states");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(HQS_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(HQS_ERR_INVALID, "hqs_probability_noalloc: device ordinal too large");
    double* partials = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_partials_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_partials);
            if (e != cudaSuccess)
                return fail(HQS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_partials_addr[dev] = static_cast<double*>(p);
        }
        partials = g_partials_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned grid = (unsigned)(nparts ? nparts : 1);
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
