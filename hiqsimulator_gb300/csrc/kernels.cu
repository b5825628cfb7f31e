// State-vector kernels for one GB300 (sm_103a).
//
// Replaces the reference's OpenMP/AVX2 sweeps (src/simulator-mpi/kernels/
// {nointrin,intrin}/kernel1..5.hpp, kernels_diag.hpp) and the reductions of
// src/simulator-mpi/SimulatorMPI.cpp (getProbability_internal :841-870,
// normalize :872-895, calcLocalApproxDistribution :817-839, Entropy :681-694,
// DeallocateLocalQubit :278-322) with tiled, coalesced passes over HBM.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>

#include "hqs_arith.cuh"
#include "hqs_kernels.h"

namespace hqs {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint64_t insert_zero(uint64_t v, int p) {
    const uint64_t low = v & ((1ULL << p) - 1ULL);
    return ((v - low) << 1) | low;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide FP64 sum of NV values per thread; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = warp_sum(v[i]);
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) red[wid * NV + i] = v[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += red[w * NV + i];
            v[i] = s;
        }
    }
    __syncthreads();
}

// Fixed-order sum of per-CTA partials (nparts x NV, strided by kMaxPartials).
template <int NV>
__global__ void finish_partials(const double* __restrict__ partials, int nparts, double* __restrict__ out) {
    __shared__ double red[32 * 4];
    double v[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = 0.0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
#pragma unroll
        for (int i = 0; i < NV; ++i) v[i] += partials[i * kMaxPartials + p];
    }
    block_sum<NV>(v, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) out[i] = v[i];
    }
}

// Reductions stream the state: 8 CTAs per SM keep enough loads in flight to
// cover HBM latency.
int reduce_grid(uint64_t work) {
    const uint64_t want = (work + kThreads - 1) / kThreads;
    int g = device_sm_count() * 8;
    if ((uint64_t)g > want) g = (int)std::max<uint64_t>(want, 1);
    return std::min(g, kMaxPartials);
}

template <int NV>
cudaError_t finish_reduce(int nparts, ReduceScratch& rs, cudaStream_t s, double* out) {
    finish_partials<NV><<<1, kThreads, 0, s>>>(rs.d_partials, nparts, rs.d_result);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(rs.h_result, rs.d_result, NV * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    for (int i = 0; i < NV; ++i) out[i] = rs.h_result[i];
    return cudaSuccess;
}

// ---------------------------------------------------------------- fused pass

// A run of consecutive diagonal and scalar gates [o0, o1) in place: every
// amplitude is loaded once, multiplied by each gate's entry (gates whose
// outer controls this tile fails are skipped) and stored once.
template <class A>
__device__ __forceinline__ void apply_elementwise_run(typename A::comp_t* buf, const typename A::mat_t* pool,
                                                      const PassDesc& d, int o0, int o1, int Q, uint64_t base) {
    for (int L = threadIdx.x; L < Q; L += blockDim.x) {
        typename A::elem_t x = A::elem_load(buf[L]);
        for (int o = o0; o < o1; ++o) {
            const OpDesc& op = d.ops[o];
            if ((base & op.ctrl_outer) != op.ctrl_outer) continue;
            if (op.k == 0) {
                x = A::elem_mul(pool[op.mat_off], x);
                continue;
            }
            if ((L & op.ctrl_local) != op.ctrl_local) continue;
            int r = 0;
            for (int j = 0; j < op.k; ++j) {
                const int sl = op.tslot[j];
                const uint64_t bit = (sl & kOuterSlot) ? (base >> (sl & 63)) : ((uint64_t)L >> sl);
                r |= (int)(bit & 1ULL) << j;
            }
            x = A::elem_mul(pool[op.mat_off + r], x);
        }
        buf[L] = A::elem_store(x);
    }
}

// Dense k-qubit op, tile src -> tile dst. The matrix is stored transposed
// (matT[c * D + r] = M[r][c]). A task is one output row r for up to GPT index
// groups; consecutive threads take consecutive rows of the same groups, so
// every input read is a shared-memory broadcast and the matrix reads of a
// warp are consecutive.
template <class A, int K, int GPT>
__device__ __forceinline__ void apply_dense(const typename A::comp_t* __restrict__ src,
                                            typename A::comp_t* __restrict__ dst,
                                            const typename A::mat_t* __restrict__ matT, const OpDesc& op, int q) {
    using C = typename A::comp_t;
    constexpr int D = 1 << K;
    const int G = 1 << (q - K);
    const int gpt = G < GPT ? G : GPT;
    const int ntask = D * (G / gpt);
    int ss[K];
    uint32_t bitv[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        ss[j] = op.tslot[j];
        bitv[j] = 1u << op.tslot[j];
    }
#pragma unroll
    for (int a = 1; a < K; ++a)
#pragma unroll
        for (int b = K - 1; b >= a; --b)
            if (ss[b - 1] > ss[b]) { const int t = ss[b]; ss[b] = ss[b - 1]; ss[b - 1] = t; }

    for (int task = threadIdx.x; task < ntask; task += blockDim.x) {
        const int r = task & (D - 1);
        const int g0 = (task >> K) * gpt;
        uint32_t orow = 0;
#pragma unroll
        for (int j = 0; j < K; ++j)
            if ((r >> j) & 1) orow |= bitv[j];
        uint32_t Lb[GPT];
        bool ok[GPT];
#pragma unroll
        for (int i = 0; i < GPT; ++i) {
            uint32_t v = (uint32_t)(g0 + (i < gpt ? i : 0));
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const uint32_t low = v & ((1u << ss[j]) - 1u);
                v = ((v - low) << 1) | low;
            }
            Lb[i] = v;
            ok[i] = (i < gpt) && ((v & op.ctrl_local) == op.ctrl_local);
        }
        typename A::acc_t acc[GPT];
#pragma unroll
        for (int i = 0; i < GPT; ++i) A::zero(acc[i]);
#pragma unroll
        for (int c = 0; c < D; ++c) {
            uint32_t oc = 0;
#pragma unroll
            for (int j = 0; j < K; ++j)
                if ((c >> j) & 1) oc |= bitv[j];
            const typename A::mat_t m = matT[c * D + r];
#pragma unroll
            for (int i = 0; i < GPT; ++i)
                if (ok[i]) A::mac(acc[i], m, src[Lb[i] + oc]);
        }
#pragma unroll
        for (int i = 0; i < GPT; ++i) {
            if (i >= gpt) continue;
            dst[Lb[i] + orow] = ok[i] ? A::finish(acc[i]) : src[Lb[i] + orow];
        }
    }
}


// ------------------------------------------------------------ tensor-core gates
//
// A dense k-qubit gate (k = 3..5) on a tile of G = 2^(q-k) index groups is the
// real GEMM  Y[G x 2D] = X[G x 2D] * B[2D x 2D],  D = 2^k, with X holding the
// interleaved real and imaginary parts of each group's inputs (column 2c + p)
// and B the matching real form of the gate (B[2c][2r] = Re M_rc,
// B[2c+1][2r] = -Im M_rc, B[2c][2r+1] = Im M_rc, B[2c+1][2r+1] = Re M_rc). Every entry of X is written as
// 2^E_row * sum_i d_i 2^(-8-10i) with five signed digits |d_i| <= 512 (E_row
// shared by the row, digit_fields5), every entry of B as
// 2^E_col * sum_j e_j 2^(-9-10j) with E_col shared by the column (digits
// computed on the host). Digits are exact in fp16, a product
// of two digits has at most 18 bits and a 2D <= 64 term sum at most 24 bits,
// so the fp32 accumulation of one digit pair is exact. Pairs (i, j) with
// i + j <= 2 get their own accumulators, the pairs of levels 3 and 4 share one
// each, levels >= 5 are dropped (for unitary gates up to 2^-45.5 of the row
// scale, the largest error of the scheme; measured in an exact model). The epilogue
// converts the eight accumulators to integers and re-assembles doubles with
// integer operations.

// The five digits of a complex128 state entry v, as biased 10-bit fields:
// X = round(|v| 2^(48-E_row)) (to nearest, ties to even: ties are frequent
// when few bits are dropped, and rounding them away from zero would grow the
// state's norm) with v's sign, |X| <= 2^48, where |v| < 2^E_row,
// E_row = ebrow - 1022. Y = X + kFieldBias lies in [0, 2^50), and its 10-bit
// fields f_i (most significant first) give balanced digits d_i = f_i - 512
// in [-512, 511] with X = sum_i d_i 2^(10(4-i)): no carries, no sign per digit.
constexpr unsigned long long kFieldBias = 512ULL * (1ULL + (1ULL << 10) + (1ULL << 20) + (1ULL << 30) + (1ULL << 40));
__device__ __forceinline__ void digit_fields5(double v, int ebrow, uint32_t (&f)[kTcDigits]) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const int eb = (int)((u >> 52) & 0x7FFu);
    unsigned long long a = 0;
    const int sh = 5 + ebrow - eb;  // >= 5
    if (eb != 0 && sh < 62) {
        const unsigned long long M = (u & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
        a = (M + (1ULL << (sh - 1)) - 1ULL + ((M >> sh) & 1ULL)) >> sh;
    }
    const unsigned long long Y = ((u >> 63) ? (0ULL - a) : a) + kFieldBias;
    const uint32_t lo = (uint32_t)Y, hi = (uint32_t)(Y >> 32);
    f[0] = hi >> 8;
    f[1] = __funnelshift_r(lo, hi, 30) & 1023u;
    f[2] = (lo >> 20) & 1023u;
    f[3] = (lo >> 10) & 1023u;
    f[4] = lo & 1023u;
}

// fp16 pair (f0 - 512, f1 - 512) of two biased fields
__device__ __forceinline__ uint32_t pack_fields(uint32_t f0, uint32_t f1) {
    const float a = __int_as_float(0x4B3FFE00 + (int)f0) - 12582912.0f;
    const float b = __int_as_float(0x4B3FFE00 + (int)f1) - 12582912.0f;
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// Two digits of an FP32 v on the FP32 pipe. s = 2^(19 - E_row) with
// |v| < 2^E_row (s = 0 flushes rows below 2^-106). Adding 1.5 * 2^23 rounds
// to an integer (to nearest, ties to even): X = rint(v s), |X| <= 2^19, then
// hi = rint(X / 1024) and lo = X - 1024 hi, both in [-512, 512] and exact.
constexpr float kRoundMagic = 12582912.0f;  // 1.5 * 2^23
__device__ __forceinline__ void digits2f(float v, float s, float& hi, float& lo) {
    const float x = __fadd_rn(__fmaf_rn(v, s, kRoundMagic), -kRoundMagic);
    hi = __fadd_rn(__fmaf_rn(x, 1.0f / 1024.0f, kRoundMagic), -kRoundMagic);
    lo = __fmaf_rn(hi, -1024.0f, x);
}

// S * 2^sc as the nearest double (ties away from zero), built from bits.
__device__ __forceinline__ double fixed_to_double(long long S, int sc) {
    if (S == 0) return 0.0;
    const unsigned long long sgn = (S < 0) ? (1ULL << 63) : 0ULL;
    unsigned long long a = (S < 0) ? (unsigned long long)(-S) : (unsigned long long)S;
    int p = 63 - __clzll((long long)a);
    unsigned long long m;
    if (p <= 52) {
        m = a << (52 - p);
    } else {
        const int sh = p - 52;
        m = (a + (1ULL << (sh - 1))) >> sh;
        if (m >> 53) {
            m >>= 1;
            ++p;
        }
    }
    const int biased = p + sc + 1023;
    if (biased <= 0) return __longlong_as_double((long long)sgn);
    return __longlong_as_double((long long)(sgn | ((unsigned long long)biased << 52) | (m & 0xFFFFFFFFFFFFFULL)));
}


__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}

__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const void* p) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
}

__device__ __forceinline__ void mma_f16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// accumulator of digit pair (i, j): one per pair of levels i + j <= 2, one for
// each of levels 3 and 4
__host__ __device__ constexpr int tc_acc(int i, int j) {
    return (i + j == 0) ? 0 : (i + j == 1) ? 1 + i : (i + j == 2) ? 3 + i : (i + j == 3) ? 6 : 7;
}

// Digit counts of each amplitude type (state digits A, gate digits B) and
// the products kept. complex128: five and five, levels 0..4 (above). complex64:
// two state digits, three gate digits, products (0,0), (0,1), (1,0), (0,2) in
// four accumulators: the gate is exact to 2^-29 of its column scale against
// the state's top digit, and the dropped products (up to 2^-17.4 of the row
// scale for unitary 5-qubit gates, measured in an exact model) depend on the
// state's low digit, so they add noise but no systematic change of the norm.
// All digits round to nearest.
template <class V>
struct TcDigits;
template <>
struct TcDigits<double2> {
    static constexpr int kA = kTcDigits, kB = kTcDigits, kAcc = 8;
    __device__ static constexpr bool keep(int i, int j) { return i + j < kTcDigits; }
    __device__ static constexpr int acc(int i, int j) { return tc_acc(i, j); }
};
template <>
struct TcDigits<float2> {
    static constexpr int kA = kTcDigits64, kB = kTcDigits64B, kAcc = 4;
    __device__ static constexpr bool keep(int i, int j) { return i + j <= 1 || (i == 0 && j == 2); }
    __device__ static constexpr int acc(int i, int j) { return i + j == 0 ? 0 : i + j == 1 ? 1 + i : 3; }
};

// Pool layout of a tensor-core gate (bytes): int32 E_col[2D], then NDB digit
// planes of B^T, each 2D rows of (2D + 8) fp16 (row j holds column j of B).
// tab_key names the op whose group/offset tables the scratch holds (the
// tables depend only on the op, so a CTA builds them once per pass when the
// pass has one tensor-core gate); key is this op's identity in the pass.
template <int K, class V>
__device__ __forceinline__ void apply_tc(const V* __restrict__ src, V* __restrict__ dst,
                                         const unsigned char* __restrict__ pool, const OpDesc& op, int q,
                                         unsigned char* __restrict__ scratch, int& tab_key, int key) {
    using TD = TcDigits<V>;
    constexpr bool kC128 = std::is_same<V, double2>::value;
    constexpr int ND = TD::kA;
    constexpr int NDB = TD::kB;
    constexpr int NACC = TD::kAcc;
    constexpr int D = 1 << K;
    constexpr int KK = 2 * D;
    constexpr int RH = KK + 8;  // fp16 per plane row (padded against bank conflicts)
    const int G = 1 << (q - K);
    const int* ecol = reinterpret_cast<const int*>(pool);
    const __half* planeB = reinterpret_cast<const __half*>(pool + 4 * KK);
    // scratch: [ND digit planes of X][erow[G]: row exponents][gbt[G]: first
    // tile index of each group][offt[D]: tile offset of each input]
    __half* planeA = reinterpret_cast<__half*>(scratch);
    int* erow = reinterpret_cast<int*>(scratch + (size_t)ND * G * RH * 2);
    uint32_t* gbt = reinterpret_cast<uint32_t*>(erow + G);
    uint32_t* offt = gbt + G;
    // pool column scales: complex128 int32 E_col; complex64 float 2^(E_col - 19)

    if (tab_key != key) {
        int ss[K];
        uint32_t bitv[K];
#pragma unroll
        for (int j = 0; j < K; ++j) {
            ss[j] = op.tslot[j];
            bitv[j] = 1u << op.tslot[j];
        }
#pragma unroll
        for (int a = 1; a < K; ++a)
#pragma unroll
            for (int b = K - 1; b >= a; --b)
                if (ss[b - 1] > ss[b]) { const int t = ss[b]; ss[b] = ss[b - 1]; ss[b - 1] = t; }
        for (int g = threadIdx.x; g < G; g += blockDim.x) {
            uint32_t v = (uint32_t)g;
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const uint32_t low = v & ((1u << ss[j]) - 1u);
                v = ((v - low) << 1) | low;
            }
            gbt[g] = v;
        }
        for (int c = threadIdx.x; c < D; c += blockDim.x) {
            uint32_t o = 0;
#pragma unroll
            for (int j = 0; j < K; ++j)
                if ((c >> j) & 1) o |= bitv[j];
            offt[c] = o;
        }
        tab_key = key;
    }

    // 1. digit planes of X. Plane column 2c + p holds part p (0 re, 1 im) of
    // input c. A work item is (group g, 4 consecutive inputs); consecutive
    // threads take consecutive groups, so their tile reads are contiguous
    // whenever tile bit 0 is not a target.
    constexpr int CPI = 2;           // complex inputs per item
    constexpr int NCH = D / CPI;     // items per group
    for (int g = threadIdx.x; g < G; g += blockDim.x) erow[g] = 0;
    __syncthreads();
    for (int it = threadIdx.x; it < G * NCH; it += blockDim.x) {
        const int g = it % G, ch = it / G;
        const uint32_t Lb = gbt[g];
        int eb = 0;
#pragma unroll
        for (int u = 0; u < CPI; ++u) {
            const V x = src[Lb + offt[ch * CPI + u]];
            if constexpr (kC128) {
                eb = max(eb, (int)(((unsigned long long)__double_as_longlong(x.x) >> 52) & 0x7FFu));
                eb = max(eb, (int)(((unsigned long long)__double_as_longlong(x.y) >> 52) & 0x7FFu));
            } else {
                eb = max(eb, (int)((__float_as_uint(x.x) >> 23) & 0xFFu));
                eb = max(eb, (int)((__float_as_uint(x.y) >> 23) & 0xFFu));
            }
        }
        if (eb) atomicMax(&erow[g], eb);
    }
    __syncthreads();
    for (int it = threadIdx.x; it < G * NCH; it += blockDim.x) {
        const int g = it % G, ch = it / G;
        const uint32_t Lb = gbt[g];
        const int ebrow = erow[g];
        uint32_t w[ND][CPI];
#pragma unroll
        for (int u = 0; u < CPI; ++u) {
            const V x = src[Lb + offt[ch * CPI + u]];
            if constexpr (kC128) {
                uint32_t fr[ND], fi[ND];
                digit_fields5(x.x, ebrow, fr);
                digit_fields5(x.y, ebrow, fi);
#pragma unroll
                for (int sdx = 0; sdx < ND; ++sdx) w[sdx][u] = pack_fields(fr[sdx], fi[sdx]);
            } else {
                const float s = ebrow >= 20 ? __int_as_float((272 - ebrow) << 23) : 0.f;
                float hr, lr, hi, li;
                digits2f(x.x, s, hr, lr);
                digits2f(x.y, s, hi, li);
                __half2 h0 = __floats2half2_rn(hr, hi), h1 = __floats2half2_rn(lr, li);
                w[0][u] = *reinterpret_cast<uint32_t*>(&h0);
                w[1][u] = *reinterpret_cast<uint32_t*>(&h1);
            }
        }
#pragma unroll
        for (int sdx = 0; sdx < ND; ++sdx)
            *reinterpret_cast<uint2*>(planeA + (size_t)sdx * G * RH + (size_t)g * RH + ch * 2 * CPI) =
                make_uint2(w[sdx][0], w[sdx][1]);
    }
    __syncthreads();

    // 2. MMA: warp task = (16 groups) x (8 output reals)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int mtiles = G / 16;
    constexpr int NT = KK / 8;
    for (int task = warp; task < mtiles * NT; task += nwarps) {
        const int mt = task / NT, nt = task % NT;
        float acc[NACC][4];
#pragma unroll
        for (int a = 0; a < NACC; ++a)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[a][e] = 0.f;
        const int arow = mt * 16 + (lane & 7) + ((lane >> 3) & 1) * 8;
        const int brow = nt * 8 + (lane & 7);
#pragma unroll
        for (int kp = 0; kp < KK / 32 + (KK < 32 ? 1 : 0); ++kp) {
            // two k16 steps per iteration (one when KK == 16): B fragments for
            // both come from one ldmatrix.x4
            uint32_t af[ND][4];
            const int ks0 = kp * 2;
#pragma unroll
            for (int half = 0; half < (KK < 32 ? 1 : 2); ++half) {
                const int ks = ks0 + half;
                const int acol = ks * 16 + (lane >> 4) * 8;
#pragma unroll
                for (int s = 0; s < ND; ++s)
                    ldsm_x4(af[s], planeA + (size_t)s * G * RH + (size_t)arow * RH + acol);
                const int bcol = ks * 16 + ((lane >> 3) & 1) * 8;
#pragma unroll
                for (int j = 0; j < NDB; ++j) {
                    uint32_t bf[2];
                    ldsm_x2(bf, planeB + (size_t)j * KK * RH + (size_t)brow * RH + bcol);
#pragma unroll
                    for (int i = 0; i < ND; ++i)
                        if (TD::keep(i, j)) mma_f16(acc[TD::acc(i, j)], af[i], bf[0], bf[1]);
                }
            }
        }
        // 3. epilogue: rows g0 and g0 + 8; plane columns nt*8 + 2*tig + {0, 1}
        // are the real and imaginary parts of output r = nt*4 + tig
        const int gid = lane >> 2, tig = lane & 3;
        const int r = nt * 4 + tig;
        const uint32_t orow = offt[r];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int g = mt * 16 + gid + h * 8;
            const uint32_t Lb = gbt[g];
            const uint32_t idx = Lb + orow;
            if ((Lb & op.ctrl_local) != op.ctrl_local) {
                dst[idx] = src[idx];
                continue;
            }
            if constexpr (kC128) {
                const int er = erow[g] - 1022;
                double outv[2];
#pragma unroll
                for (int c2 = 0; c2 < 2; ++c2) {
                    // accumulators hold integers: level sums as one fixed-point
                    // int64 S = L0 2^30 + L1 2^20 + L2 2^10 + L3 + L4 2^-10 (< 2^55),
                    // value = S * 2^(E_row + E_col - 47)
                    const int e = h * 2 + c2;
                    const long long L0 = __float2int_rn(acc[0][e]);
                    const long long L1 = (long long)__float2int_rn(acc[1][e]) + __float2int_rn(acc[2][e]);
                    const long long L2 = (long long)__float2int_rn(acc[3][e]) + __float2int_rn(acc[4][e]) +
                                         __float2int_rn(acc[5][e]);
                    const long long L3 = __float2int_rn(acc[6][e]);
                    const long long L4 = __float2int_rn(acc[7][e]);
                    const long long S = (L0 << 30) + (L1 << 20) + (L2 << 10) + L3 + (L4 >> 10);
                    outv[c2] = fixed_to_double(S, er + ecol[nt * 8 + tig * 2 + c2] - 47);
                }
                dst[idx] = make_double2(outv[0], outv[1]);
            } else {
                // accumulators hold exact integers: value = (L0 2^20 + L1 2^10
                // + L2) * 2^(E_row - 19) * 2^(E_col - 19), the last factor
                // stored per column in the pool as a float
                const int eb = erow[g];
                const float rs = eb >= 20 ? __int_as_float((eb - 18) << 23) : 0.f;
                const float* cscale = reinterpret_cast<const float*>(ecol);
                float outv[2];
#pragma unroll
                for (int c2 = 0; c2 < 2; ++c2) {
                    const int e = h * 2 + c2;
                    const float S = __fmaf_rn(acc[0][e], 1048576.0f,
                                              __fmaf_rn(__fadd_rn(acc[1][e], acc[2][e]), 1024.0f, acc[3][e]));
                    outv[c2] = __fmul_rn(__fmul_rn(S, rs), cscale[nt * 8 + tig * 2 + c2]);
                }
                dst[idx] = make_float2(outv[0], outv[1]);
            }
        }
    }
}

// ------------------------------------------------- complex64 3xTF32 gates
//
// A dense k-qubit gate (k = 3..5) on complex64 amplitudes in the same real
// form as apply_tc: a tile's G = 2^(q-k) index groups are the rows of X
// (G x 2D reals, interleaved re/im of the group's D inputs), Y = X B. Each
// FP32 operand x is split into two TF32 parts, hi = rna(x) and
// lo = rna(x - hi) (x - hi is exact in FP32), and Y accumulates
// lo*hi + hi*lo + hi*hi with m16n8k8 TF32 MMAs in FP32; the dropped lo*lo
// term is below 2^-21 of each product. A fragments are read straight from
// the tile buffer; B comes split and in fragment order from the pass pool:
// for k-step ks and n-tile nt, lane l holds float4 {hi b0, hi b1, lo b0,
// lo b1} with b0 = B[8ks + l%4][8nt + l/4], b1 = B[8ks + l%4 + 4][8nt + l/4].

__device__ __forceinline__ uint32_t tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <int K>
__device__ __forceinline__ void apply_tf32(const float2* __restrict__ src, float2* __restrict__ dst,
                                           const float4* __restrict__ frag, const OpDesc& op, int q) {
    constexpr int D = 1 << K;
    constexpr int KK = 2 * D;
    constexpr int NT = KK / 8;              // n-tiles (8 output reals) and k-steps (8 input reals)
    constexpr int NTW = NT < 4 ? NT : 4;    // n-tiles per warp task
    constexpr int NCH = NT / NTW;
    const int G = 1 << (q - K);
    const int MT = G >> 4;

    int ss[K];
    uint32_t bitv[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        ss[j] = op.tslot[j];
        bitv[j] = 1u << op.tslot[j];
    }
#pragma unroll
    for (int a = 1; a < K; ++a)
#pragma unroll
        for (int b = K - 1; b >= a; --b)
            if (ss[b - 1] > ss[b]) { const int t = ss[b]; ss[b] = ss[b - 1]; ss[b - 1] = t; }
    auto group_base = [&](uint32_t g) {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const uint32_t low = g & ((1u << ss[j]) - 1u);
            g = ((g - low) << 1) | low;
        }
        return g;
    };
    auto offset_of = [&](int c) {
        uint32_t o = 0;
#pragma unroll
        for (int j = 0; j < K; ++j)
            if ((c >> j) & 1) o |= bitv[j];
        return o;
    };

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int gid = lane >> 2, tig = lane & 3;
    for (int task = warp; task < MT * NCH; task += nwarps) {
        const int mt = task / NCH, nc = task % NCH;
        const uint32_t Lb0 = group_base(mt * 16 + gid), Lb1 = group_base(mt * 16 + gid + 8);
        // The tensor cores round their FP32 accumulation toward zero, so a
        // long accumulation chain at full scale shrinks every output (the
        // norm drifts down gate after gate). Each k-step's three products
        // go into a zeroed accumulator (one truncation, at the scale of
        // that k-step's partial sum, whose sign varies) and are added to the
        // running sum with a round-to-nearest FADD.
        float acc[NTW][4];
#pragma unroll
        for (int j = 0; j < NTW; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[j][e] = 0.f;
#pragma unroll
        for (int ks = 0; ks < NT; ++ks) {
            // columns tig and tig + 4 of this k-step: part tig & 1 of inputs
            // 4 ks + tig / 2 and 4 ks + 2 + tig / 2
            const uint32_t o0 = offset_of(ks * 4 + (tig >> 1)), o1 = offset_of(ks * 4 + 2 + (tig >> 1));
            const float2 x00 = src[Lb0 + o0], x10 = src[Lb1 + o0], x01 = src[Lb0 + o1], x11 = src[Lb1 + o1];
            const bool im = (tig & 1) != 0;
            const float av[4] = {im ? x00.y : x00.x, im ? x10.y : x10.x, im ? x01.y : x01.x, im ? x11.y : x11.x};
            uint32_t ah[4], al[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                ah[e] = tf32_rna(av[e]);
                al[e] = tf32_rna(av[e] - __uint_as_float(ah[e]));
            }
#pragma unroll
            for (int j = 0; j < NTW; ++j) {
                const float4 b = frag[(ks * NT + nc * NTW + j) * 32 + lane];
                float t[4] = {0.f, 0.f, 0.f, 0.f};
                mma_tf32(t, al, __float_as_uint(b.x), __float_as_uint(b.y));
                mma_tf32(t, ah, __float_as_uint(b.z), __float_as_uint(b.w));
                mma_tf32(t, ah, __float_as_uint(b.x), __float_as_uint(b.y));
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[j][e] = __fadd_rn(acc[j][e], t[e]);
            }
        }
        // columns 2 tig, 2 tig + 1 of n-tile nt: output nt * 4 + tig
        const bool ok0 = (Lb0 & op.ctrl_local) == op.ctrl_local;
        const bool ok1 = (Lb1 & op.ctrl_local) == op.ctrl_local;
#pragma unroll
        for (int j = 0; j < NTW; ++j) {
            const uint32_t orow = offset_of((nc * NTW + j) * 4 + tig);
            dst[Lb0 + orow] = ok0 ? make_float2(acc[j][0], acc[j][1]) : src[Lb0 + orow];
            dst[Lb1 + orow] = ok1 ? make_float2(acc[j][2], acc[j][3]) : src[Lb1 + orow];
        }
    }
}

constexpr int kPassGPT = 4;

// Shared-memory layout of a pass (host and device agree through pass_smem_t):
// [matrix pool][tile A][tile B][high-bit offsets][16-aligned tensor-core scratch]
// [staging tile, raw state elements, when d.prefetch]
template <class A>
struct PassSmem {
    typename A::mat_t* smat;
    typename A::comp_t* bufA;
    typename A::comp_t* bufB;
    uint64_t* hoff;
    unsigned char* tcs;
    typename A::store_t* stage;
    __device__ __forceinline__ PassSmem(unsigned char* smem, const PassDesc& d) {
        const size_t mat_bytes = ((size_t)d.mat_elems * sizeof(typename A::mat_t) + 15) & ~(size_t)15;
        const size_t Q = (size_t)1 << d.q;
        smat = reinterpret_cast<typename A::mat_t*>(smem);
        bufA = reinterpret_cast<typename A::comp_t*>(smem + mat_bytes);
        bufB = bufA + Q;
        hoff = reinterpret_cast<uint64_t*>(bufB + Q);
        tcs = smem + ((mat_bytes + 2 * sizeof(typename A::comp_t) * Q + sizeof(uint64_t) * ((size_t)1 << (d.q - d.w)) +
                       15) & ~(size_t)15);
        stage = reinterpret_cast<typename A::store_t*>(tcs + d.tc_bytes);
    }
};

// Asynchronous global -> shared copies of single state elements (cp.async):
// each thread copies and later reads back only its own staging slots, so
// waiting for its own copies is the only synchronisation the staging needs.
__device__ __forceinline__ void cp_async_elem(double2* sdst, const double2* gsrc) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)),
                 "l"(gsrc)
                 : "memory");
}
__device__ __forceinline__ void cp_async_elem(float2* sdst, const float2* gsrc) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)),
                 "l"(gsrc)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// First state index of tile t: t's bits spread over the positions outside
// the tile and the fixed (control) positions, fixed positions set.
__device__ __forceinline__ uint64_t tile_base(const PassDesc& d, uint64_t t) {
    uint64_t base = t;
    for (int i = 0; i < d.nins; ++i) base = insert_zero(base, d.ins_pos[i]);
    return base | d.fixed_mask;
}

// A CTA's walk over tiles t0, t0 + stride, ...: the base of the next tile is
// the current one plus the deposited stride, added with the carries skipping
// every position outside `spread` (the bits tile numbers are spread over).
struct TileWalk {
    uint64_t spread, step, base, fixed;
    __device__ __forceinline__ TileWalk(const PassDesc& d, uint64_t t0, uint64_t stride) {
        uint64_t ins = 0;
        for (int i = 0; i < d.nins; ++i) ins |= 1ULL << d.ins_pos[i];
        spread = ~ins & (d.n >= 64 ? ~0ULL : ((1ULL << d.n) - 1ULL));
        fixed = d.fixed_mask;
        base = tile_base(d, t0);
        step = tile_base(d, stride) & ~fixed;
    }
    __device__ __forceinline__ uint64_t after(uint64_t b) const {
        return ((((b & spread) | ~spread) + step) & spread) | fixed;
    }
};

// Issue this thread's copies of tile t into buf (its own slots: the same
// L = threadIdx.x + i * blockDim.x as every load, conversion and store).
template <class A>
__device__ __forceinline__ void tile_prefetch_into(const typename A::store_t* __restrict__ state, const PassDesc& d,
                                                   const PassSmem<A>& sm, uint64_t base,
                                                   typename A::store_t* __restrict__ buf) {
    const int Q = 1 << d.q;
    const uint32_t lowmask = (1u << d.w) - 1u;
    for (int L = threadIdx.x; L < Q; L += blockDim.x)
        cp_async_elem(buf + L, state + base + sm.hoff[L >> d.w] + (L & lowmask));
    cp_async_commit();
}

// ... into the staging buffer.
template <class A>
__device__ __forceinline__ void tile_prefetch(const typename A::store_t* __restrict__ state, const PassDesc& d,
                                              const PassSmem<A>& sm, uint64_t base) {
    tile_prefetch_into<A>(state, d, sm, base, sm.stage);
}

// Stage a pass's matrices and tile offsets into shared memory.
template <class A>
__device__ __forceinline__ void pass_setup(const PassSmem<A>& sm, const PassDesc& d,
                                           const typename A::mat_t* __restrict__ mats) {
    const int nh = d.q - d.w;
    for (uint32_t i = threadIdx.x; i < d.mat_elems; i += blockDim.x) sm.smat[i] = mats[i];
    for (int j = threadIdx.x; j < (1 << nh); j += blockDim.x) {
        uint64_t o = 0;
        for (int b = 0; b < nh; ++b)
            if ((j >> b) & 1) o |= 1ULL << d.tile_pos[d.w + b];
        sm.hoff[j] = o;
    }
    __syncthreads();
}

// One tile of a pass: load into b0 (unless the caller already placed the
// tile there), apply the pass's gates in order, store. b1 is the other tile
// buffer (dense gates ping-pong between the two). With d.prefetch == 2 every
// op of the pass works in place on b0 (tensor-core digit gates, diagonal and
// scalar ops), and b1 belongs to the caller.
template <class A>
__device__ __forceinline__ void pass_tile(typename A::store_t* __restrict__ state, const PassDesc& d,
                                          const PassSmem<A>& sm, uint64_t base, int& tab_key, bool loaded = false,
                                          typename A::comp_t* b0 = nullptr, typename A::comp_t* b1 = nullptr) {
    using C = typename A::comp_t;
    const int Q = 1 << d.q;
    const uint32_t lowmask = (1u << d.w) - 1u;
    const bool inplace = d.prefetch == 2;
    C* src = b0 ? b0 : sm.bufA;
    C* dst = b1 ? b1 : sm.bufB;
    if (!loaded) {
        for (int L = threadIdx.x; L < Q; L += blockDim.x)
            src[L] = A::to_comp(state[base + sm.hoff[L >> d.w] + (L & lowmask)]);
        __syncthreads();
    }
    for (int oi = 0; oi < d.nops; ++oi) {
        const OpDesc& op = d.ops[oi];
        if (op.k == 0 || op.diag) {
            // consecutive diagonal / scalar gates act element by element:
            // one sweep over the tile for the whole run, no barrier between them
            int end = oi + 1;
            while (end < d.nops && (d.ops[end].k == 0 || d.ops[end].diag)) ++end;
            apply_elementwise_run<A>(src, sm.smat, d, oi, end, Q, base);
            __syncthreads();
            oi = end - 1;
            continue;
        }
        if ((base & op.ctrl_outer) != op.ctrl_outer) continue;
        if constexpr (A::kId == 5) {
            if (op.tc) {
                const float4* frag = reinterpret_cast<const float4*>(sm.smat + op.mat_off);
                switch (op.k) {
                    case 3: apply_tf32<3>(src, dst, frag, op, d.q); break;
                    case 4: apply_tf32<4>(src, dst, frag, op, d.q); break;
                    default: apply_tf32<5>(src, dst, frag, op, d.q); break;
                }
                __syncthreads();
                C* tmp = src;
                src = dst;
                dst = tmp;
                continue;
            }
        }
        if constexpr (A::kId == 4 || A::kId == 6) {
            if (op.tc) {
                // the digit planes decouple the MMA reads from the tile, so
                // the gate can also write its result over its input
                const unsigned char* pool = reinterpret_cast<const unsigned char*>(sm.smat + op.mat_off);
                C* out = inplace ? src : dst;
                switch (op.k) {
                    case 3: apply_tc<3, C>(src, out, pool, op, d.q, sm.tcs, tab_key, oi); break;
                    case 4: apply_tc<4, C>(src, out, pool, op, d.q, sm.tcs, tab_key, oi); break;
                    default: apply_tc<5, C>(src, out, pool, op, d.q, sm.tcs, tab_key, oi); break;
                }
                __syncthreads();
                if (!inplace) {
                    C* tmp = src;
                    src = dst;
                    dst = tmp;
                }
                continue;
            }
        }
        switch (op.k) {
            case 1: apply_dense<A, 1, kPassGPT>(src, dst, sm.smat + op.mat_off, op, d.q); break;
            case 2: apply_dense<A, 2, kPassGPT>(src, dst, sm.smat + op.mat_off, op, d.q); break;
            case 3: apply_dense<A, 3, kPassGPT>(src, dst, sm.smat + op.mat_off, op, d.q); break;
            case 4: apply_dense<A, 4, kPassGPT>(src, dst, sm.smat + op.mat_off, op, d.q); break;
            default: apply_dense<A, 5, kPassGPT>(src, dst, sm.smat + op.mat_off, op, d.q); break;
        }
        __syncthreads();
        C* tmp = src;
        src = dst;
        dst = tmp;
    }
    for (int L = threadIdx.x; L < Q; L += blockDim.x)
        state[base + sm.hoff[L >> d.w] + (L & lowmask)] = A::from_comp(src[L]);
    __syncthreads();
}

// resident CTAs per SM the pass kernels are compiled for (register cap):
// digit-plane tensor-core passes 3, 3xTF32 passes 2, the rest 4
__host__ __device__ constexpr int pass_min_blocks(int id) { return (id == 4 || id == 6) ? 3 : id == 5 ? 2 : 4; }

template <class A>
__global__ void __launch_bounds__(kThreads, pass_min_blocks(A::kId)) pass_kernel(typename A::store_t* __restrict__ state,
                                                                             const typename A::mat_t* __restrict__ mats,
                                                                             const __grid_constant__ PassDesc d) {
    extern __shared__ __align__(16) unsigned char smem[];
    const PassSmem<A> sm(smem, d);
    pass_setup<A>(sm, d, mats);
    const uint64_t ntiles = 1ULL << (d.n - d.nins);
    if ((uint64_t)blockIdx.x >= ntiles) return;
    const TileWalk walk(d, blockIdx.x, gridDim.x);
    int tab_key = -1;
    if (!d.prefetch) {
        uint64_t base = walk.base;
        for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x, base = walk.after(base))
            pass_tile<A>(state, d, sm, base, tab_key);
        return;
    }
    if constexpr (std::is_same<typename A::comp_t, typename A::store_t>::value) {
        if (d.prefetch == 2) {
            // all ops in place: tile t + gridDim.x streams into the other tile
            // buffer while tile t is computed; the buffers swap every tile
            typename A::comp_t* cur = sm.bufA;
            typename A::comp_t* nxt = sm.bufB;
            uint64_t base = walk.base;
            tile_prefetch_into<A>(state, d, sm, base, cur);
            for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
                const uint64_t next = walk.after(base);
                cp_async_wait_all();
                if (t + gridDim.x < ntiles) tile_prefetch_into<A>(state, d, sm, next, nxt);
                __syncthreads();
                pass_tile<A>(state, d, sm, base, tab_key, true, cur, nxt);
                typename A::comp_t* tmp = cur;
                cur = nxt;
                nxt = tmp;
                base = next;
            }
            return;
        }
    }
    // software pipeline: tile t + gridDim.x streams into the staging buffer
    // while tile t is computed
    const int Q = 1 << d.q;
    uint64_t base = walk.base;
    tile_prefetch<A>(state, d, sm, base);
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint64_t next = walk.after(base);
        cp_async_wait_all();
        for (int L = threadIdx.x; L < Q; L += blockDim.x) sm.bufA[L] = A::to_comp(sm.stage[L]);
        if (t + gridDim.x < ntiles) tile_prefetch<A>(state, d, sm, next);
        __syncthreads();
        pass_tile<A>(state, d, sm, base, tab_key, true);
        base = next;
    }
}

// Many passes (one per independent state) in one launch: global tile index T
// belongs to the item whose tile range contains it; each CTA walks its tiles
// in increasing T and re-stages the pass when it crosses into a new item.
template <class A>
__global__ void __launch_bounds__(kThreads, pass_min_blocks(A::kId)) batch_pass_kernel(const BatchItem* __restrict__ items,
                                                                                   int nitems, uint64_t total_tiles) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ PassDesc sd;
    int cur = -1;
    int tab_key = -1;
    // runs of 8 consecutive tiles, dealt round-robin to the CTAs: a CTA
    // re-stages an item's matrices at most once per run, and every CTA sees
    // a mix of cheap and expensive items
    constexpr uint64_t kRun = 8;
    for (uint64_t T0 = (uint64_t)blockIdx.x * kRun; T0 < total_tiles; T0 += (uint64_t)gridDim.x * kRun)
    for (uint64_t T = T0; T < min(total_tiles, T0 + kRun); ++T) {
        int lo = 0, hi = nitems - 1;
        while (lo < hi) {  // last item with tile_begin <= T
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].tile_begin <= T) lo = mid;
            else hi = mid - 1;
        }
        if (lo != cur) {
            tab_key = -1;
            __syncthreads();
            const uint32_t* srcw = reinterpret_cast<const uint32_t*>(&items[lo].desc);
            uint32_t* dstw = reinterpret_cast<uint32_t*>(&sd);
            for (int w = threadIdx.x; w < (int)(sizeof(PassDesc) / 4); w += blockDim.x) dstw[w] = srcw[w];
            __syncthreads();
            cur = lo;
            pass_setup<A>(PassSmem<A>(smem, sd), sd, reinterpret_cast<const typename A::mat_t*>(items[lo].mats));
        }
        pass_tile<A>(reinterpret_cast<typename A::store_t*>(items[lo].state), sd, PassSmem<A>(smem, sd),
                     tile_base(sd, T - items[lo].tile_begin), tab_key);
    }
}

template <class A>
size_t pass_smem_t(const PassDesc& d) {
    const size_t mat_bytes = ((size_t)d.mat_elems * sizeof(typename A::mat_t) + 15) & ~(size_t)15;
    return ((mat_bytes + 2 * (sizeof(typename A::comp_t) << d.q) + sizeof(uint64_t) * (1u << (d.q - d.w)) + 15) &
            ~(size_t)15) + d.tc_bytes + (d.prefetch == 1 ? (sizeof(typename A::store_t) << d.q) : 0);
}

template <class A>
cudaError_t launch_batch_t(const BatchItem* d_items, int nitems, uint64_t total_tiles, size_t smem, cudaStream_t s) {
    auto kern = batch_pass_kernel<A>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    uint64_t grid = (uint64_t)device_sm_count() * per_sm;
    const uint64_t runs = (total_tiles + 7) / 8;
    if (grid > runs) grid = runs;
    if (grid == 0) return cudaSuccess;
    kern<<<(unsigned)grid, kThreads, smem, s>>>(d_items, nitems, total_tiles);
    return cudaGetLastError();
}

template <class A>
cudaError_t launch_pass_t(void* state, const void* mats, const PassDesc& d, cudaStream_t s) {
    const size_t smem = pass_smem_t<A>(d);
    auto kern = pass_kernel<A>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint64_t ntiles = 1ULL << (d.n - d.nins);
    uint64_t grid = (uint64_t)device_sm_count() * per_sm;
    if (grid > ntiles) grid = ntiles;
    kern<<<(unsigned)grid, kThreads, smem, s>>>(reinterpret_cast<typename A::store_t*>(state),
                                                 reinterpret_cast<const typename A::mat_t*>(mats), d);
    return cudaGetLastError();
}

// ------------------------------------------------------------- reductions

struct MaskSpec {
    uint64_t val;
    int npos;
    uint8_t pos[64];  // sorted positions of mask bits
};

template <class NA, class S>
__global__ void __launch_bounds__(kThreads) probability_kernel(const S* __restrict__ state, uint64_t count,
                                                               const __grid_constant__ MaskSpec m,
                                                               double* __restrict__ partials) {
    __shared__ double red[32];
    NA acc;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    auto index = [&](uint64_t j) {
        for (int b = 0; b < m.npos; ++b) j = insert_zero(j, m.pos[b]);
        return j | m.val;
    };
    uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for (; j + stride < count; j += 2 * stride) {  // two amplitudes in flight per thread
        const S a0 = state[index(j)], a1 = state[index(j + stride)];
        acc.add(a0);
        acc.add(a1);
    }
    if (j < count) acc.add(state[index(j)]);
    double v[1] = {acc.value()};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = v[0];
}

template <class NA, class S>
__global__ void __launch_bounds__(kThreads) bit_probs_kernel(const S* __restrict__ state, uint64_t count, int pos,
                                                             double* __restrict__ partials) {
    __shared__ double red[64];
    NA a0, a1;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for (; i + 3 * stride < count; i += 4 * stride) {  // four amplitudes in flight per thread
        S v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = state[i + u * stride];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (((i + u * stride) >> pos) & 1ULL) a1.add(v[u]);
            else a0.add(v[u]);
        }
    }
    for (; i < count; i += stride) {
        if ((i >> pos) & 1ULL) a1.add(state[i]);
        else a0.add(state[i]);
    }
    double v[2] = {a0.value(), a1.value()};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = v[0];
        partials[kMaxPartials + blockIdx.x] = v[1];
    }
}

template <class NA, class S>
__global__ void __launch_bounds__(kThreads) entropy_kernel(const S* __restrict__ state, uint64_t count,
                                                           double* __restrict__ partials) {
    __shared__ double red[32];
    double e = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x) {
        NA a;
        a.add(state[i]);
        const double p = a.value();
        if (p > 0.0) e += p * log2(p);
    }
    double v[1] = {e};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = v[0];
}

// Block sums for measurement: one CTA per block when blocks are large, one
// thread per block (summing in index order) when they are small.
template <class NA, class S>
__global__ void __launch_bounds__(kThreads) block_sum_cta_kernel(const S* __restrict__ state, uint64_t K,
                                                                 double* __restrict__ out) {
    __shared__ double red[32];
    NA acc;
    const uint64_t b0 = (uint64_t)blockIdx.x * K;
    uint64_t j = threadIdx.x;
    for (; j + 3 * kThreads < K; j += 4 * kThreads) {  // four amplitudes in flight per thread
        S v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = state[b0 + j + u * kThreads];
#pragma unroll
        for (int u = 0; u < 4; ++u) acc.add(v[u]);
    }
    for (; j < K; j += kThreads) acc.add(state[b0 + j]);
    double v[1] = {acc.value()};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) out[blockIdx.x] = v[0];
}

template <class NA, class S>
__global__ void __launch_bounds__(kThreads) block_sum_serial_kernel(const S* __restrict__ state, uint64_t K,
                                                                    uint64_t nblocks, double* __restrict__ out) {
    const uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (b >= nblocks) return;
    double s = 0.0;
    for (uint64_t j = 0; j < K; ++j) {
        NA a;
        a.add(state[b * K + j]);
        s += a.value();
    }
    out[b] = s;
}

// Pauli expectation: sum_t Re(c_t * sum_i conj(a_i) phase_t(j) a_j), j = i ^ x_t,
// phase_t(j) = i^{|Y_t|} (-1)^{popcount(j & (Y_t|Z_t))}.
template <class S>
__device__ __forceinline__ void load_d2(const S* st, uint64_t i, double& re, double& im);
template <>
__device__ __forceinline__ void load_d2<double2>(const double2* st, uint64_t i, double& re, double& im) {
    const double2 v = st[i];
    re = v.x;
    im = v.y;
}
template <>
__device__ __forceinline__ void load_d2<float2>(const float2* st, uint64_t i, double& re, double& im) {
    const float2 v = st[i];
    re = v.x;
    im = v.y;
}

// |a|^2 of one amplitude as a double-float (h, e): complex128 entries split
// exactly into float pairs, squares formed with FMA.
__device__ __forceinline__ void norm2_df(double2 a, float& h, float& e) {
    const DF r = df_split(a.x), m = df_split(a.y);
    const float ph = r.h * r.h, qh = m.h * m.h;
    float pe = fmaf(r.h, r.h, -ph);
    pe = fmaf(2.f * r.h, r.l, pe);
    float qe = fmaf(m.h, m.h, -qh);
    qe = fmaf(2.f * m.h, m.l, qe);
    h = ph + qh;
    const float bb = h - ph;
    e = ((ph - (h - bb)) + (qh - bb)) + pe + qe;
}
__device__ __forceinline__ void norm2_df(float2 a, float& h, float& e) {
    const float ph = a.x * a.x, qh = a.y * a.y;
    const float pe = fmaf(a.x, a.x, -ph), qe = fmaf(a.y, a.y, -qh);
    h = ph + qh;
    const float bb = h - ph;
    e = ((ph - (h - bb)) + (qh - bb)) + pe + qe;
}

// sum_i (-1)^popcount(i & z) |a_i|^2: the expectation of a Z string, one read
// of the state, two amplitudes in flight per thread.
template <class S>
__global__ void __launch_bounds__(kThreads) zparity_kernel(const S* __restrict__ state, uint64_t count, uint64_t z,
                                                           double* __restrict__ partials) {
    __shared__ double red[32];
    float sh = 0.f, sl = 0.f;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    auto acc = [&](uint64_t i, S a) {
        float h, e;
        norm2_df(a, h, e);
        if (__popcll(i & z) & 1) {
            h = -h;
            e = -e;
        }
        const float s = sh + h, bb = s - sh;
        sl += ((sh - (s - bb)) + (h - bb)) + e;
        sh = s;
    };
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for (; i + stride < count; i += 2 * stride) {
        const S a0 = state[i], a1 = state[i + stride];
        acc(i, a0);
        acc(i + stride, a1);
    }
    if (i < count) acc(i, state[i]);
    double v[1] = {(double)sh + (double)sl};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = v[0];
}

// ---- many Z strings in one read of the state
// E_t = sum_i (-1)^popcount(i & z_t) |a_i|^2 for up to kZMulti masks. The
// state is taken in chunks of 2^q consecutive amplitudes (q = min(n, 12));
// per chunk c the Walsh coefficients W_c[m] = sum_lo (-1)^popcount(lo & m)
// |a_(c 2^q + lo)|^2 of all 2^q low masks come from a fast Walsh-Hadamard
// transform in double-float (16 elements per thread: the four stages over
// index bits 8-11 in registers, the others in shared memory), and mask t
// adds (-1)^popcount(c 2^q & z_t) W_c[z_t mod 2^q]. Cost per amplitude: one
// load and q double-float butterflies, whatever the number of masks.
constexpr int kZMulti = 64;

// (a, b) <- (a + b, a - b) in double-float
__device__ __forceinline__ void df_butterfly(float& ah, float& al, float& bh, float& bl) {
    const float sh = ah + bh, sv = sh - ah;
    const float se = (ah - (sh - sv)) + (bh - sv) + al + bl;
    const float dh = ah - bh, dv = dh - ah;
    const float de = (ah - (dh - dv)) + (-bh - dv) + al - bl;
    const float s2 = sh + se, d2 = dh + de;
    ah = s2;
    al = se - (s2 - sh);
    bh = d2;
    bl = de - (d2 - dh);
}

template <class S>
__global__ void __launch_bounds__(kThreads, 4) zparity_multi_kernel(const S* __restrict__ state, int n, int T,
                                                                 const uint64_t* __restrict__ z,
                                                                 double* __restrict__ partials) {
    __shared__ float wh[4096], wl[4096];
    const int q = n < 12 ? n : 12;
    const uint32_t Q = 1u << q;
    const uint64_t nchunks = 1ULL << (n - q);
    const uint64_t zt = (int)threadIdx.x < T ? z[threadIdx.x] : 0;
    float ah = 0.f, al = 0.f;  // mask threadIdx.x's sum (threads < T)
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const S* base = state + (c << q);
        if (q == 12) {
            // element tid + 256 j: j holds index bits 8-11
            float vh[16], vl[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const S a = base[threadIdx.x + 256 * j];
                norm2_df(a, vh[j], vl[j]);
            }
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (!((j >> b) & 1)) df_butterfly(vh[j], vl[j], vh[j | (1 << b)], vl[j | (1 << b)]);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                wh[threadIdx.x + 256 * j] = vh[j];
                wl[threadIdx.x + 256 * j] = vl[j];
            }
        } else {
            for (uint32_t i = threadIdx.x; i < Q; i += kThreads) norm2_df(base[i], wh[i], wl[i]);
        }
        __syncthreads();
        for (int b = 0; b < (q == 12 ? 8 : q); ++b) {
            for (uint32_t k = threadIdx.x; k < Q / 2; k += kThreads) {
                const uint32_t i = ((k >> b) << (b + 1)) | (k & ((1u << b) - 1u));
                const uint32_t j = i | (1u << b);
                float xh = wh[i], xl = wl[i], yh = wh[j], yl = wl[j];
                df_butterfly(xh, xl, yh, yl);
                wh[i] = xh;
                wl[i] = xl;
                wh[j] = yh;
                wl[j] = yl;
            }
            __syncthreads();
        }
        if ((int)threadIdx.x < T) {
            const uint32_t m = (uint32_t)(zt & (Q - 1u));
            float vh = wh[m], vl = wl[m];
            if (__popcll((c << q) & zt) & 1) {
                vh = -vh;
                vl = -vl;
            }
            const float s2 = ah + vh, bb = s2 - ah;
            al += ((ah - (s2 - bb)) + (vh - bb)) + vl;
            ah = s2;
        }
        __syncthreads();
    }
    if ((int)threadIdx.x < T) partials[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = (double)ah + (double)al;
}

// out[t] = the fixed-order FP64 sum of mask t's per-CTA partials
__global__ void finish_multi_kernel(const double* __restrict__ partials, int nparts, double* __restrict__ out) {
    __shared__ double red[32];
    double v[1] = {0.0};
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) v[0] += partials[(size_t)blockIdx.x * nparts + p];
    block_sum<1>(v, red);
    if (threadIdx.x == 0) out[blockIdx.x] = v[0];
}

// One term of a Pauli sum as the expectation kernel uses it: x the flip
// mask, yz the sign mask, h the lowest bit of x (an unordered pair {i, i^x}
// is visited from its member with bit h clear), im whether the pair
// contributes through Im(conj(a_i) a_j) (an odd number of sign bits inside
// x) rather than the real part, k the real weight as a double-float.
struct PauliTermDev {
    uint64_t x, yz;
    float kh, kl;
    int h, im;
};
constexpr int kPauliChunk = 64;

// sum_t Re(w_t sum_i conj(a_i) ph_t(i ^ x_t) a_(i ^ x_t)), ph_t(k) =
// (-1)^popcount(k & (Y_t | Z_t)), w_t = c_t i^|Y_t|, in one read of the
// state per chunk of 64 terms: each amplitude is loaded once, a term with
// x_t = 0 adds Re(w_t) ph_t(i) |a_i|^2, a term with x_t != 0 takes each pair
// {i, j = i ^ x_t} once. With P = conj(a_i) a_j and s_i = ph_t(i), the pair
// adds Re(w (s_j P + s_i conj(P))) = 2 s_i Re(w) Re(P) when s_i = s_j and
// 2 s_i Im(w) Im(P) when s_i = -s_j (s_i s_j = (-1)^popcount(x_t & yz_t)
// is the same for every pair of the term). Products and sums in
// double-float.
template <class S>
__global__ void __launch_bounds__(kThreads) pauli_expect_kernel(const S* __restrict__ state, uint64_t count,
                                                                int nterms, const uint64_t* __restrict__ xm,
                                                                const uint64_t* __restrict__ ym,
                                                                const uint64_t* __restrict__ zm,
                                                                const double* __restrict__ coef,
                                                                double* __restrict__ partials) {
    __shared__ double red[32];
    __shared__ PauliTermDev tm[kPauliChunk];
    float acc_h = 0.f, acc_l = 0.f;
    auto add = [&](float vh, float vl, const PauliTermDev& T, bool neg) {
        // (vh + vl) (kh + kl), negated when the sign is odd, into the accumulator
        float p = vh * T.kh;
        float e = fmaf(vh, T.kh, -p);
        e = fmaf(vh, T.kl, fmaf(vl, T.kh, e));
        if (neg) {
            p = -p;
            e = -e;
        }
        const float s = acc_h + p, bb = s - acc_h;
        acc_l += ((acc_h - (s - bb)) + (p - bb)) + e;
        acc_h = s;
    };
    for (int t0 = 0; t0 < nterms; t0 += kPauliChunk) {
        const int tn = min(kPauliChunk, nterms - t0);
        __syncthreads();
        if (threadIdx.x < tn) {
            const int t = t0 + threadIdx.x;
            PauliTermDev T;
            T.x = xm[t];
            T.yz = ym[t] | zm[t];
            double wr = coef[2 * t], wi = coef[2 * t + 1];
            for (int r = 0; r < (__popcll(ym[t]) & 3); ++r) {  // w = c i^|Y|
                const double tr = -wi;
                wi = wr;
                wr = tr;
            }
            double k = wr;
            T.im = 0;
            T.h = 0;
            if (T.x != 0) {
                T.im = __popcll(T.x & T.yz) & 1;
                k = 2.0 * (T.im ? wi : wr);
                T.h = __ffsll((long long)T.x) - 1;
            }
            const DF kd = df_split(k);
            T.kh = kd.h;
            T.kl = kd.l;
            tm[threadIdx.x] = T;
        }
        __syncthreads();
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
             i += (uint64_t)gridDim.x * blockDim.x) {
            double ar, ai;
            load_d2<S>(state, i, ar, ai);
            const DF arf = df_split(ar), aif = df_split(ai);
            for (int t = 0; t < tn; ++t) {
                const PauliTermDev T = tm[t];
                const bool neg = (__popcll(i & T.yz) & 1) != 0;
                float vh = 0.f, vl = 0.f;
                if (T.x == 0) {
                    df_mac(vh, vl, arf.h, arf.l, arf.h, arf.l);
                    df_mac(vh, vl, aif.h, aif.l, aif.h, aif.l);
                } else {
                    if ((i >> T.h) & 1ULL) continue;
                    double br, bi;
                    load_d2<S>(state, i ^ T.x, br, bi);
                    const DF brf = df_split(br), bif = df_split(bi);
                    if (T.im) {  // Im(conj(a) b) = ar bi - ai br
                        df_mac(vh, vl, arf.h, arf.l, bif.h, bif.l);
                        df_mac(vh, vl, -aif.h, -aif.l, brf.h, brf.l);
                    } else {     // Re(conj(a) b) = ar br + ai bi
                        df_mac(vh, vl, arf.h, arf.l, brf.h, brf.l);
                        df_mac(vh, vl, aif.h, aif.l, bif.h, bif.l);
                    }
                }
                add(vh, vl, T, neg);
            }
        }
    }
    double v[1] = {(double)acc_h + (double)acc_l};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = v[0];
}

// out_i = sum_t c_t phase_t(j) a_j with j = i ^ x_t. coef holds two entries
// per term in the arithmetic's matrix format: c_t i^{|Y_t|} and its negation,
// selected by the parity of j & (Y_t | Z_t).
template <class A>
__global__ void __launch_bounds__(kThreads) pauli_apply_kernel(const typename A::store_t* __restrict__ in,
                                                               typename A::store_t* __restrict__ out, uint64_t count,
                                                               int nterms, const uint64_t* __restrict__ xm,
                                                               const uint64_t* __restrict__ ym,
                                                               const uint64_t* __restrict__ zm,
                                                               const typename A::mat_t* __restrict__ coef) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x) {
        typename A::acc_t acc;
        A::zero(acc);
        for (int t = 0; t < nterms; ++t) {
            const uint64_t j = i ^ xm[t];
            const int neg = __popcll(j & (ym[t] | zm[t])) & 1;
            A::mac(acc, coef[2 * t + neg], A::to_comp(in[j]));
        }
        out[i] = A::from_comp(A::finish(acc));
    }
}

template <class A>
__global__ void __launch_bounds__(kThreads) collapse_kernel(typename A::store_t* __restrict__ state, uint64_t count,
                                                            uint64_t mask, uint64_t val,
                                                            const typename A::mat_t scale) {
    using S = typename A::store_t;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if ((i & mask) != val) {
            S z;
            z.x = 0;
            z.y = 0;
            state[i] = z;
        } else {
            state[i] = A::from_comp(A::mul(scale, A::to_comp(state[i])));
        }
    }
}

template <class S>
__global__ void fill_kernel(S* __restrict__ state, uint64_t count, S v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x)
        state[i] = v;
}

// new[i] = old[src(i)] for i in [lo, hi); sources are disjoint from [lo, hi).
template <class S>
__global__ void drop_bit_kernel(S* __restrict__ state, uint64_t lo, uint64_t hi, int pos, uint64_t keepbit) {
    const uint64_t lowm = (1ULL << pos) - 1ULL;
    for (uint64_t i = lo + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < hi;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t src = ((i & ~lowm) << 1) | (i & lowm) | keepbit;
        state[i] = state[src];
    }
}

struct PermSpec {
    int n, q, w, nins;
    uint8_t tile_pos[kMaxTileBits];
    uint8_t ins_pos[64];
    uint8_t src_slot[kMaxTileBits];  // for destination tile bit j: source tile bit
    uint16_t src_lut[128];           // source tile index of destination bits 0-5 (first 64) and 6-11
};

// Shared-memory slot of tile element L: L with its low bits XORed by a fold
// of its higher bits, so that a quarter-warp of 16-byte elements (a
// half-warp of 8-byte ones) hits distinct bank groups both when it writes
// consecutive elements and when it reads elements whose indices differ only
// in high bits (the moved qubits).
template <class S>
__device__ __forceinline__ int perm_slot(int L) {
    constexpr int b = sizeof(S) == 16 ? 3 : 4;
    constexpr int m = (1 << b) - 1;
    return L ^ (((L >> b) ^ (L >> (2 * b)) ^ (L >> (3 * b)) ^ (L >> (4 * b))) & m);
}

// In-place bit permutation, one tile at a time: every tile maps onto itself.
// A tile is read with coalesced loads (runs of 2^w consecutive amplitudes),
// held in shared memory and written back permuted; the source index of each
// destination element comes from two 64-entry tables.
template <class S>
__global__ void __launch_bounds__(kThreads) permute_kernel(S* __restrict__ state, const __grid_constant__ PermSpec p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int Q = 1 << p.q;
    S* buf = reinterpret_cast<S*>(smem);
    const int nh = p.q - p.w;
    uint64_t* hoff = reinterpret_cast<uint64_t*>(buf + Q);
    uint16_t* lut = reinterpret_cast<uint16_t*>(hoff + (1 << nh));
    const uint32_t lowmask = (1u << p.w) - 1u;
    for (int j = threadIdx.x; j < (1 << nh); j += blockDim.x) {
        uint64_t o = 0;
        for (int b = 0; b < nh; ++b)
            if ((j >> b) & 1) o |= 1ULL << p.tile_pos[p.w + b];
        hoff[j] = o;
    }
    for (int j = threadIdx.x; j < 128; j += blockDim.x) lut[j] = p.src_lut[j];
    __syncthreads();
    const uint64_t ntiles = 1ULL << (p.n - p.nins);
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        uint64_t base = t;
        for (int i = 0; i < p.nins; ++i) base = insert_zero(base, p.ins_pos[i]);
#pragma unroll 4
        for (int L = threadIdx.x; L < Q; L += kThreads)
            buf[perm_slot<S>(L)] = __ldcs(state + base + hoff[L >> p.w] + (L & lowmask));
        __syncthreads();
#pragma unroll 4
        for (int L = threadIdx.x; L < Q; L += kThreads) {
            const int Ls = lut[L & 63] | lut[64 + (L >> 6)];
            __stcs(state + base + hoff[L >> p.w] + (L & lowmask), buf[perm_slot<S>(Ls)]);
        }
        __syncthreads();
    }
}

__global__ void c64_to_c128_kernel(const float2* __restrict__ in, double2* __restrict__ out, uint64_t count) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = make_double2((double)in[i].x, (double)in[i].y);
}
__global__ void c128_to_c64_kernel(const double2* __restrict__ in, float2* __restrict__ out, uint64_t count) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

int stream_grid(uint64_t count) {
    const uint64_t want = (count + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)device_sm_count() * 8;
    return (int)std::max<uint64_t>(1, std::min(want, cap));
}

MaskSpec make_mask_spec(uint64_t mask, uint64_t val) {
    MaskSpec m;
    m.val = val;
    m.npos = 0;
    for (int b = 0; b < 64; ++b)
        if ((mask >> b) & 1ULL) m.pos[m.npos++] = (uint8_t)b;
    return m;
}

}  // namespace

int device_sm_count() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

// Kernels other than the fused pass treat tensor-core modes as their base
// arithmetic: double-float for complex128, FP32 for complex64.
static inline int base_arith(int a) {
    return a == kArithTC ? kArithDF : (a == kArithTF32 || a == kArithTC64) ? kArithF32 : a;
}

int pass_reg_ctas(int arith, const PassDesc& d) {
    const bool tc = pass_has_tc(d);
    switch (arith) {
        case kArithTC: return tc ? pass_min_blocks(ArithDFRaw::kId) : pass_min_blocks(ArithDF::kId);
        case kArithTC64: return tc ? pass_min_blocks(ArithTC64::kId) : pass_min_blocks(ArithF32::kId);
        case kArithTF32: return tc ? pass_min_blocks(ArithTF32::kId) : pass_min_blocks(ArithF32::kId);
        case kArithF64: return pass_min_blocks(ArithF64::kId);
        case kArithDF: return pass_min_blocks(ArithDF::kId);
        default: return pass_min_blocks(ArithF32::kId);
    }
}

size_t pass_smem_bytes(int arith, const PassDesc& d) {
    switch (arith) {
        case kArithF64: return pass_smem_t<ArithF64>(d);
        case kArithDF: return pass_smem_t<ArithDF>(d);
        case kArithTC: return pass_has_tc(d) ? pass_smem_t<ArithDFRaw>(d) : pass_smem_t<ArithDF>(d);
        default: return pass_smem_t<ArithF32>(d);  // F32, TF32, TC64: same tile and pool element
    }
}

cudaError_t launch_pass(int arith, void* state, const void* mats, const PassDesc& d, cudaStream_t s) {
    switch (arith) {
        case kArithF64: return launch_pass_t<ArithF64>(state, mats, d, s);
        case kArithDF: return launch_pass_t<ArithDF>(state, mats, d, s);
        case kArithF32: return launch_pass_t<ArithF32>(state, mats, d, s);
        // passes without tensor-core gates run the double-float kernel (same
        // matrix format, fewer registers, more resident CTAs)
        case kArithTC: return pass_has_tc(d) ? launch_pass_t<ArithDFRaw>(state, mats, d, s)
                                             : launch_pass_t<ArithDF>(state, mats, d, s);
        case kArithTF32: return pass_has_tc(d) ? launch_pass_t<ArithTF32>(state, mats, d, s)
                                               : launch_pass_t<ArithF32>(state, mats, d, s);
        case kArithTC64: return pass_has_tc(d) ? launch_pass_t<ArithTC64>(state, mats, d, s)
                                               : launch_pass_t<ArithF32>(state, mats, d, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_batch(int arith, bool tc, const BatchItem* d_items, int nitems, uint64_t total_tiles, size_t smem,
                         cudaStream_t s) {
    switch (arith) {
        case kArithF64: return launch_batch_t<ArithF64>(d_items, nitems, total_tiles, smem, s);
        case kArithDF: return launch_batch_t<ArithDF>(d_items, nitems, total_tiles, smem, s);
        case kArithF32: return launch_batch_t<ArithF32>(d_items, nitems, total_tiles, smem, s);
        case kArithTC: return tc ? launch_batch_t<ArithDFRaw>(d_items, nitems, total_tiles, smem, s)
                                 : launch_batch_t<ArithDF>(d_items, nitems, total_tiles, smem, s);
        case kArithTF32: return tc ? launch_batch_t<ArithTF32>(d_items, nitems, total_tiles, smem, s)
                                   : launch_batch_t<ArithF32>(d_items, nitems, total_tiles, smem, s);
        case kArithTC64: return tc ? launch_batch_t<ArithTC64>(d_items, nitems, total_tiles, smem, s)
                                   : launch_batch_t<ArithF32>(d_items, nitems, total_tiles, smem, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t reduce_probability(int arith, const void* state, int n, uint64_t mask, uint64_t val,
                               ReduceScratch& rs, cudaStream_t s, double* out) {
    arith = base_arith(arith);
    const MaskSpec m = make_mask_spec(mask, val);
    const uint64_t count = (1ULL << n) >> m.npos;
    const int g = reduce_grid(count);
    if (arith == kArithF64)
        probability_kernel<NormAccF64, double2><<<g, kThreads, 0, s>>>((const double2*)state, count, m, rs.d_partials);
    else if (arith == kArithDF)
        probability_kernel<NormAccDF, double2><<<g, kThreads, 0, s>>>((const double2*)state, count, m, rs.d_partials);
    else
        probability_kernel<NormAccDF, float2><<<g, kThreads, 0, s>>>((const float2*)state, count, m, rs.d_partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return finish_reduce<1>(g, rs, s, out);
}

cudaError_t reduce_bit_probs(int arith, const void* state, int n, int pos, ReduceScratch& rs, cudaStream_t s,
                             double* out2) {
    arith = base_arith(arith);
    const uint64_t count = 1ULL << n;
    const int g = reduce_grid(count);
    if (arith == kArithF64)
        bit_probs_kernel<NormAccF64, double2><<<g, kThreads, 0, s>>>((const double2*)state, count, pos, rs.d_partials);
    else if (arith == kArithDF)
        bit_probs_kernel<NormAccDF, double2><<<g, kThreads, 0, s>>>((const double2*)state, count, pos, rs.d_partials);
    else
        bit_probs_kernel<NormAccDF, float2><<<g, kThreads, 0, s>>>((const float2*)state, count, pos, rs.d_partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return finish_reduce<2>(g, rs, s, out2);
}

cudaError_t reduce_entropy(int arith, const void* state, int n, ReduceScratch& rs, cudaStream_t s, double* out) {
    arith = base_arith(arith);
    const uint64_t count = 1ULL << n;
    const int g = reduce_grid(count);
    if (arith == kArithF64)
        entropy_kernel<NormAccF64, double2><<<g, kThreads, 0, s>>>((const double2*)state, count, rs.d_partials);
    else if (arith == kArithDF)
        entropy_kernel<NormAccDF, double2><<<g, kThreads, 0, s>>>((const double2*)state, count, rs.d_partials);
    else
        entropy_kernel<NormAccDF, float2><<<g, kThreads, 0, s>>>((const float2*)state, count, rs.d_partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = finish_reduce<1>(g, rs, s, out);
    if (e == cudaSuccess) *out = -*out;
    return e;
}

cudaError_t block_sums(int arith, const void* state, int n, uint64_t nblocks, double* d_out, cudaStream_t s) {
    arith = base_arith(arith);
    const uint64_t K = (1ULL << n) / nblocks;
    if (K >= kThreads) {
        if (arith == kArithF64)
            block_sum_cta_kernel<NormAccF64, double2><<<(unsigned)nblocks, kThreads, 0, s>>>((const double2*)state, K, d_out);
        else if (arith == kArithDF)
            block_sum_cta_kernel<NormAccDF, double2><<<(unsigned)nblocks, kThreads, 0, s>>>((const double2*)state, K, d_out);
        else
            block_sum_cta_kernel<NormAccDF, float2><<<(unsigned)nblocks, kThreads, 0, s>>>((const float2*)state, K, d_out);
    } else {
        const unsigned g = (unsigned)((nblocks + kThreads - 1) / kThreads);
        if (arith == kArithF64)
            block_sum_serial_kernel<NormAccF64, double2><<<g, kThreads, 0, s>>>((const double2*)state, K, nblocks, d_out);
        else if (arith == kArithDF)
            block_sum_serial_kernel<NormAccDF, double2><<<g, kThreads, 0, s>>>((const double2*)state, K, nblocks, d_out);
        else
            block_sum_serial_kernel<NormAccDF, float2><<<g, kThreads, 0, s>>>((const float2*)state, K, nblocks, d_out);
    }
    return cudaGetLastError();
}

cudaError_t reduce_zparity_multi(int arith, const void* state, int n, int T, const uint64_t* d_z, double* d_scratch,
                                 cudaStream_t s, double* out) {
    arith = base_arith(arith);
    if (T < 1 || T > kZMulti) return cudaErrorInvalidValue;
    const int q = n < 12 ? n : 12;
    const uint64_t nchunks = 1ULL << (n - q);
    const int g = (int)std::min<uint64_t>(nchunks, (uint64_t)device_sm_count() * 4);
    double* partials = d_scratch;
    double* d_out = d_scratch + (size_t)T * g;
    if (arith == kArithF32)
        zparity_multi_kernel<float2><<<g, kThreads, 0, s>>>((const float2*)state, n, T, d_z, partials);
    else
        zparity_multi_kernel<double2><<<g, kThreads, 0, s>>>((const double2*)state, n, T, d_z, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    finish_multi_kernel<<<T, kThreads, 0, s>>>(partials, g, d_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(out, d_out, (size_t)T * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

size_t zparity_multi_scratch_bytes(int T) {
    return sizeof(double) * ((size_t)T * (size_t)device_sm_count() * 4 + (size_t)T);
}

cudaError_t reduce_pauli_expectation(int arith, const void* state, int n, int nterms, const uint64_t* d_xm,
                                     const uint64_t* d_ym, const uint64_t* d_zm, const double* d_coef,
                                     ReduceScratch& rs, cudaStream_t s, double* out, bool zonly, uint64_t zmask0) {
    arith = base_arith(arith);
    const uint64_t count = 1ULL << n;
    const int g = reduce_grid(count);
    if (zonly && nterms == 1) {
        // one Z string with a real coefficient: a signed norm (coef applied on the host)
        if (arith == kArithF32)
            zparity_kernel<float2><<<g, kThreads, 0, s>>>((const float2*)state, count, zmask0, rs.d_partials);
        else
            zparity_kernel<double2><<<g, kThreads, 0, s>>>((const double2*)state, count, zmask0, rs.d_partials);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        return finish_reduce<1>(g, rs, s, out);
    }
    if (arith == kArithF32)
        pauli_expect_kernel<float2><<<g, kThreads, 0, s>>>((const float2*)state, count, nterms, d_xm, d_ym, d_zm,
                                                           d_coef, rs.d_partials);
    else
        pauli_expect_kernel<double2><<<g, kThreads, 0, s>>>((const double2*)state, count, nterms, d_xm, d_ym, d_zm,
                                                            d_coef, rs.d_partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return finish_reduce<1>(g, rs, s, out);
}

cudaError_t pauli_apply(int arith, const void* in, void* out, int n, int nterms, const uint64_t* d_xm,
                        const uint64_t* d_ym, const uint64_t* d_zm, const double* d_coef, cudaStream_t s) {
    arith = base_arith(arith);
    const uint64_t count = 1ULL << n;
    const int g = stream_grid(count);
    if (arith == kArithF64)
        pauli_apply_kernel<ArithF64><<<g, kThreads, 0, s>>>((const double2*)in, (double2*)out, count, nterms, d_xm,
                                                             d_ym, d_zm, (const double2*)d_coef);  // 2 x double2 per term
    else if (arith == kArithDF)
        pauli_apply_kernel<ArithDF><<<g, kThreads, 0, s>>>((const double2*)in, (double2*)out, count, nterms, d_xm,
                                                            d_ym, d_zm, (const float4*)d_coef);
    else
        pauli_apply_kernel<ArithF32><<<g, kThreads, 0, s>>>((const float2*)in, (float2*)out, count, nterms, d_xm,
                                                             d_ym, d_zm, (const float2*)d_coef);
    return cudaGetLastError();
}

cudaError_t collapse_scale(int arith, void* state, int n, uint64_t mask, uint64_t val, double scale,
                           cudaStream_t s) {
    arith = base_arith(arith);
    const uint64_t count = 1ULL << n;
    const int g = stream_grid(count);
    if (arith == kArithF64) {
        collapse_kernel<ArithF64><<<g, kThreads, 0, s>>>((double2*)state, count, mask, val, make_double2(scale, 0.0));
    } else if (arith == kArithDF) {
        const float h = (float)scale;
        const float l = (float)(scale - (double)h);
        collapse_kernel<ArithDF><<<g, kThreads, 0, s>>>((double2*)state, count, mask, val, make_float4(h, 0.f, l, 0.f));
    } else {
        collapse_kernel<ArithF32><<<g, kThreads, 0, s>>>((float2*)state, count, mask, val,
                                                         make_float2((float)scale, 0.f));
    }
    return cudaGetLastError();
}

cudaError_t fill_value(int arith, void* state, uint64_t count, double re, double im, cudaStream_t s) {
    arith = base_arith(arith);
    const int g = stream_grid(count);
    if (arith == kArithF32)
        fill_kernel<float2><<<g, kThreads, 0, s>>>((float2*)state, count, make_float2((float)re, (float)im));
    else
        fill_kernel<double2><<<g, kThreads, 0, s>>>((double2*)state, count, make_double2(re, im));
    return cudaGetLastError();
}

cudaError_t drop_bit(int arith, void* state, int n, int pos, int keep, cudaStream_t s) {
    arith = base_arith(arith);
    // windows [lo, hi) whose sources lie entirely above hi (see kernel comment)
    const uint64_t keepbit = keep ? (1ULL << pos) : 0ULL;
    const uint64_t half = 1ULL << (n - 1);
    auto run = [&](uint64_t lo, uint64_t hi) -> cudaError_t {
        const int g = stream_grid(hi - lo);
        if (arith == kArithF32) drop_bit_kernel<float2><<<g, kThreads, 0, s>>>((float2*)state, lo, hi, pos, keepbit);
        else drop_bit_kernel<double2><<<g, kThreads, 0, s>>>((double2*)state, lo, hi, pos, keepbit);
        return cudaGetLastError();
    };
    cudaError_t e = cudaSuccess;
    if (keep) e = run(0, std::min<uint64_t>(1ULL << pos, half));
    for (int j = pos; j < n - 1 && e == cudaSuccess; ++j) e = run(1ULL << j, std::min<uint64_t>(1ULL << (j + 1), half));
    return e;
}

cudaError_t permute_bits(int arith, void* state, int n, int m, const uint8_t* oldpos, const uint8_t* newpos,
                         cudaStream_t s) {
    arith = base_arith(arith);
    if (m == 0) return cudaSuccess;
    PermSpec p{};
    p.n = n;
    // tile: the permuted positions plus the lowest other positions, up to 2^10
    // amplitudes (or the whole state)
    uint64_t inset = 0;
    for (int j = 0; j < m; ++j) inset |= 1ULL << oldpos[j];
    // 32 KiB tiles: six CTAs per SM keep enough loads in flight
    const int qmin = arith == kArithF32 ? 12 : 11;
    int q = std::min(n, std::max(m, qmin));
    if (q > kMaxTileBits) return cudaErrorInvalidValue;
    for (int b = 0; b < n && __builtin_popcountll(inset) < q; ++b) inset |= 1ULL << b;
    q = __builtin_popcountll(inset);
    p.q = q;
    int c = 0;
    for (int b = 0; b < n; ++b)
        if ((inset >> b) & 1ULL) p.tile_pos[c++] = (uint8_t)b;
    p.w = 0;
    while (p.w < q && p.tile_pos[p.w] == p.w) ++p.w;
    p.nins = q;
    for (int j = 0; j < q; ++j) p.ins_pos[j] = p.tile_pos[j];
    int slot[64];
    for (int j = 0; j < q; ++j) slot[p.tile_pos[j]] = j;
    for (int j = 0; j < q; ++j) p.src_slot[j] = (uint8_t)j;
    for (int j = 0; j < m; ++j) p.src_slot[slot[newpos[j]]] = (uint8_t)slot[oldpos[j]];
    for (int v = 0; v < 64; ++v) {
        uint32_t lo = 0, hi = 0;
        for (int j = 0; j < 6; ++j) {
            if (((v >> j) & 1) && j < q) lo |= 1u << p.src_slot[j];
            if (((v >> j) & 1) && j + 6 < q) hi |= 1u << p.src_slot[j + 6];
        }
        p.src_lut[v] = (uint16_t)lo;
        p.src_lut[64 + v] = (uint16_t)hi;
    }
    const size_t elem = (arith == kArithF32) ? sizeof(float2) : sizeof(double2);
    const size_t smem = (elem << q) + sizeof(uint64_t) * (1u << (q - p.w)) + 128 * sizeof(uint16_t);
    const uint64_t ntiles = 1ULL << (n - q);
    const int per_sm = std::max(1, std::min(2048 / kThreads, (int)((227u << 10) / (smem + 1024))));
    const unsigned g = (unsigned)std::min<uint64_t>(ntiles, (uint64_t)device_sm_count() * per_sm);
    if (arith == kArithF32) {
        cudaFuncSetAttribute(permute_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        permute_kernel<float2><<<g, kThreads, smem, s>>>((float2*)state, p);
    } else {
        cudaFuncSetAttribute(permute_kernel<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        permute_kernel<double2><<<g, kThreads, smem, s>>>((double2*)state, p);
    }
    return cudaGetLastError();
}

cudaError_t c64_to_c128(const void* in, void* out, uint64_t count, cudaStream_t s) {
    c64_to_c128_kernel<<<stream_grid(count), kThreads, 0, s>>>((const float2*)in, (double2*)out, count);
    return cudaGetLastError();
}
cudaError_t c128_to_c64(const void* in, void* out, uint64_t count, cudaStream_t s) {
    c128_to_c64_kernel<<<stream_grid(count), kThreads, 0, s>>>((const double2*)in, (float2*)out, count);
    return cudaGetLastError();
}

}  // namespace hqs
