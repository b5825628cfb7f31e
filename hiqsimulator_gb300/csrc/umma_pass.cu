// Tensor-memory fused pass on sm_103a: one dense k-qubit gate (k <= 5,
// widened to five targets with identity factors) on the tcgen05 tensor cores,
// plus the runs of diagonal and scalar gates before and after it, in one
// sweep over the state. Replaces, for its pass, the reference's kernelK sweep
// (src/simulator-mpi/kernels/nointrin/kernel5.hpp:1134-1193) and the diagonal
// sweeps (kernels_diag.hpp:20-81). Two instances: complex128 states (below)
// and complex64 states (three digits per state real, four per gate real,
// levels 0-3, all exact; see the complex64 section).
//
// Tile: 4096 amplitudes = 128 index groups x 32 inputs (the five target bits).
// Per tile the gate is the real GEMM Y[128 x 64] = X[128 x 64] B[64 x 64]
// (interleaved re/im of each group's inputs and outputs). Every state real
// is written as six balanced base-2^9 digits relative to its group's largest
// exponent (X' = x 2^(8 - E), |X'| < 2^8), every gate real as six digits
// relative to its column's largest exponent (B' = b 2^(7 - E_c), |B'| < 2^7,
// top digit <= 128). Digits are exact in fp16, and the digit products with
// i + j = L are summed into one fp32 accumulator region per level L = 0..5:
// levels 0-3 stay below 2^24 (exact integers), levels 4-5 carry at most a
// few units of rounding (2^-46 of the row scale). Dropped levels >= 6 are
// below 2^-45 of the row scale for any inputs.
//
// Operands: the state digit planes are MMA operand A (M = 128 groups, K = 64
// reals), planes 0-3 in tensor memory and planes 4-5 in shared memory (128B
// swizzle); the gate's six digit planes are operand B (N = 64 outputs per
// digit, shared memory). X_i times the gate planes j = 0..5-i, placed side by
// side along N, accumulates each (i, j) product directly into the region of
// level i + j: one MMA covers up to four levels (N = 256). A pass that holds
// only the dense gate does the outputs in two halves of 32 instead (level
// regions of 32 columns, the gate's rows ordered by half, one MMA per X_i and
// half), each half's MMAs committed to their own barrier: the compute warps
// assemble the first half's outputs while the second half's MMAs run.
//
// Warps: 0-15 split digits and assemble outputs (CUDA cores; four per warp
// scheduler), warp 16 moves tiles with TMA tensor copies (load into one of
// two tile buffers, store back from it), warp 17 allocates tensor memory and
// issues the MMAs. Every wait is
// bounded; a wait that runs out raises a CTA-wide abort flag, every warp
// leaves its loop, the TMA warp waits (bounded) for its copies in flight, the
// MMA warp for its MMAs, tensor memory is freed and the host sees the error
// word.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "hqs_arith.cuh"
#include "hqs_kernels.h"
#include "hqs_tc05.cuh"

namespace hqs {

namespace {

using namespace tc05;

constexpr int kCompute = 512;  // warps 0..15
constexpr int kTmaWarp = 16, kMmaWarp = 17;
constexpr int kThreadsU = 576;

// Shared memory (relative to a 1024-byte aligned base) and tensor memory of
// the two instances.
template <bool C64>
struct Lay;
template <>
struct Lay<false> {  // complex128
    static constexpr int kDigits = 6;
    static constexpr uint32_t kGate = 0;         // 6 gate digit planes, 64 rows x 128 B each
    static constexpr uint32_t kGateBytes = kUmmaGatePlaneBytes;
    static constexpr uint32_t kPlanes = 49152;   // state digit planes 4 and 5, 128 rows x 128 B each
    static constexpr uint32_t kTile0 = 81920;    // tile buffers, 4096 x double2
    static constexpr uint32_t kTile1 = 147456;
    static constexpr uint32_t kTileBytes = 4096 * 16;
    static constexpr uint32_t kEcol = 212992;
    static constexpr uint32_t kTmPlanes = 384;   // tensor-memory columns: six level regions of 64 (or per output half six of 32), then planes 0-3
    static constexpr uint32_t kTabEntry = 16;    // factor-table entry: double-float complex
};
template <>
struct Lay<true> {  // complex64
    static constexpr int kDigits = 3;
    static constexpr uint32_t kGate = 0;         // 4 gate digit planes, 64 rows x 128 B each
    static constexpr uint32_t kGateBytes = kUmmaGatePlaneBytes64;
    static constexpr uint32_t kPlanes = 0;       // (state planes all in tensor memory)
    static constexpr uint32_t kTile0 = 32768;    // tile buffers, 4096 x float2
    static constexpr uint32_t kTile1 = 65536;
    static constexpr uint32_t kTileBytes = 4096 * 8;
    static constexpr uint32_t kEcol = 98304;
    static constexpr uint32_t kTmPlanes = 256;   // four level regions of 64, then planes 0-2
    static constexpr uint32_t kTabEntry = 8;     // factor-table entry: FP32 complex
};
template <bool C64>
struct Sm : Lay<C64> {
    using L = Lay<C64>;
    static constexpr uint32_t kEcol = L::kEcol;   // int[64]: gate column exponents
    static constexpr uint32_t kErow = kEcol + 256;  // int[128]: group exponents of the current tile
    static constexpr uint32_t kMx = kErow + 512;    // uint32[512]: quarter-group maxima
    static constexpr uint32_t kGb = kMx + 2048;     // uint16[128]: tile index of each group's input 0
    static constexpr uint32_t kOff = kGb + 256;     // uint16[32]: tile offset of each input
    static constexpr uint32_t kBar = kOff + 64;     // 7 mbarriers
    static constexpr uint32_t kMisc = kBar + 64;    // tensor-memory base, abort flag
    static constexpr uint32_t kLut = kMisc + 64;    // uint8[2][2][64]: factor-table index of tile slots 0-5 / 6-11
    static constexpr uint32_t kTab = kLut + 256;    // [2][256] factor tables of the current tile
    static constexpr uint32_t kEw = kTab + 2 * (1u << kUmmaRunBits) * L::kTabEntry;  // element-wise matrices
    static constexpr uint32_t kBytes = kEw + kUmmaEwMaxBytes + 1024;  // + alignment slack
};

constexpr uint32_t kTmemCols = 512;

__device__ __forceinline__ uint64_t insert_zero_u(uint64_t v, int p) {
    const uint64_t low = v & ((1ULL << p) - 1ULL);
    return ((v - low) << 1) | low;
}

// First state index of tile t and the walk to the CTA's next tile (the
// tile's bits deposited over the positions outside the tile and the fixed
// positions; fixed positions set).
struct Walk {
    uint64_t spread, step, base, fixed;
    __device__ Walk(const PassDesc& d, uint64_t t0, uint64_t stride) {
        uint64_t ins = 0;
        for (int i = 0; i < d.nins; ++i) ins |= 1ULL << d.ins_pos[i];
        spread = ~ins & (d.n >= 64 ? ~0ULL : ((1ULL << d.n) - 1ULL));
        fixed = d.fixed_mask;
        base = deposit(d, t0) | fixed;
        step = deposit(d, stride);
    }
    __device__ static uint64_t deposit(const PassDesc& d, uint64_t t) {
        for (int i = 0; i < d.nins; ++i) t = insert_zero_u(t, d.ins_pos[i]);
        return t;
    }
    __device__ uint64_t after(uint64_t b) const { return ((((b & spread) | ~spread) + step) & spread) | fixed; }
};

// TMA box coordinates of copy c of the tile with base index b: the tile
// base's bits of each dimension (zero over the box run), in the last
// dimension of a plan with extra tile bits also the copy's extra bits;
// dimension 0 counts doubles (two per amplitude)
__device__ __forceinline__ void tile_coords(const UmmaDesc& u, uint64_t b, uint32_t c, int32_t (&co)[5]) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        uint64_t v = 0;
        if (i < u.rank) {
            v = (b >> u.dim_pos[i]) & ((1ULL << u.dim_bits[i]) - 1ULL);
            if (u.dim_kind[i] == 2)
                for (int k = 0; k < u.nextra; ++k)
                    if ((c >> k) & 1u) v |= 1ULL << (u.extra_pos[k] - u.dim_pos[i]);
            if (i == 0) v <<= 1;
        }
        co[i] = (int32_t)v;
    }
}

// ------------------------------------------------------------------ digits
constexpr float kMagic0 = 12582912.0f;  // 1.5 * 2^23: rounds to integers
constexpr float kMagic9 = 24576.0f;     // 1.5 * 2^14: rounds to multiples of 2^-9
constexpr float kMagic27 = 0.09375f;    // 1.5 * 2^-4: rounds to multiples of 2^-27

__device__ __forceinline__ float rnd_with(float x, float m) { return __fsub_rn(__fadd_rn(x, m), m); }

// The six balanced base-2^9 digits of X' = v 2^(1030 - Eb) (|X'| < 2^8 for
// every v of the group): X' = sum_i d_i 2^(-9 i) up to 2^-40 (2^-48 of the
// group's scale). X' = H + L splits the double's 53-bit significand into its
// top 24 bits (H) and the remaining 29 bits (L, rounded to 24 bits).
// T0 = H rounded to multiples of 2^-9 carries digits 0-1, T1 (multiples of
// 2^-27) digits 2-3, T2 = the rest digits 4-5. |d_i| <= 256 except d_2,
// whose bound is 260 (H's rounding tie at 2^-10 ignores L, |L| < 2^-16).
__device__ __forceinline__ void digits6(double v, int Eb, float (&dg)[6]) {
    const uint32_t hi = (uint32_t)__double2hiint(v), lo = (uint32_t)__double2loint(v);
    const int eb = (int)((hi >> 20) & 0x7FFu);
    int dH = eb - Eb + 134;
    dH = eb == 0 ? 0 : max(dH, 0);
    const uint32_t sgn = hi & 0x80000000u;
    const uint32_t mant = __funnelshift_l(lo, hi, 3);
    const float H = __uint_as_float((mant & 0x7FFFFFu) | ((uint32_t)dH << 23) | sgn);
    const int dL = max(dH - 52, 0);
    const float L = __fmul_rn(__uint2float_rn(lo & 0x1FFFFFFFu), __uint_as_float(((uint32_t)dL << 23) | sgn));
    const float T0 = rnd_with(H, kMagic9);
    const float R0 = __fsub_rn(H, T0);
    const float R27 = rnd_with(R0, kMagic27);
    const float D = __fadd_rn(__fsub_rn(R0, R27), L);
    const float D27 = rnd_with(D, kMagic27);
    const float T1 = __fadd_rn(R27, D27);
    const float T2 = __fsub_rn(D, D27);
    dg[0] = rnd_with(T0, kMagic0);
    dg[1] = __fmul_rn(__fsub_rn(T0, dg[0]), 512.f);
    const float u2 = __fmul_rn(T1, 262144.f);
    dg[2] = rnd_with(u2, kMagic0);
    dg[3] = __fmul_rn(__fsub_rn(u2, dg[2]), 512.f);
    const float u4 = __fmul_rn(T2, 68719476736.f);
    dg[4] = rnd_with(u4, kMagic0);
    dg[5] = rnd_with(__fmul_rn(__fsub_rn(u4, dg[4]), 512.f), kMagic0);
}

// The same digits for a normalized double-float amplitude (h, l), |l| <=
// ulp(h) / 2 (an amplitude a diagonal run has multiplied in double-float):
// X' = (h + l) 2^(134 - Ef), Ef the largest float exponent of the group's
// high parts, scaled in two exact steps (2^(134 - Ef) can exceed the float
// range), then digits6's cascade from H = h 2^(134 - Ef), L = l 2^(134 - Ef).
__device__ __forceinline__ void digits6_df(float h, float l, int Ef, float (&dg)[6]) {
    const int k = 134 - Ef, k1 = min(k, 127), k2 = k - k1;
    const float s1 = __uint_as_float((uint32_t)(k1 + 127) << 23), s2 = __uint_as_float((uint32_t)(k2 + 127) << 23);
    const float H = __fmul_rn(__fmul_rn(h, s1), s2);
    const float L = __fmul_rn(__fmul_rn(l, s1), s2);
    const float T0 = rnd_with(H, kMagic9);
    const float R0 = __fsub_rn(H, T0);
    const float R27 = rnd_with(R0, kMagic27);
    const float D = __fadd_rn(__fsub_rn(R0, R27), L);
    const float D27 = rnd_with(D, kMagic27);
    const float T1 = __fadd_rn(R27, D27);
    const float T2 = __fsub_rn(D, D27);
    dg[0] = rnd_with(T0, kMagic0);
    dg[1] = __fmul_rn(__fsub_rn(T0, dg[0]), 512.f);
    const float u2 = __fmul_rn(T1, 262144.f);
    dg[2] = rnd_with(u2, kMagic0);
    dg[3] = __fmul_rn(__fsub_rn(u2, dg[2]), 512.f);
    const float u4 = __fmul_rn(T2, 68719476736.f);
    dg[4] = rnd_with(u4, kMagic0);
    dg[5] = rnd_with(__fmul_rn(__fsub_rn(u4, dg[4]), 512.f), kMagic0);
}

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}

// ------------------------------------------------------------------ epilogue
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// Output real from the six level sums: V = sum_L S_L 2^(-9 L) (level sums
// 0-3 exact integers below 2^24, 4-5 within a few units), as a double-float
// (h, l) by three exact fast two-sums (every partial sum lies on a grid that
// keeps them exact).
__device__ __forceinline__ void level_sum_to_df(const float (&S)[6], float& h, float& l) {
    const float b1 = __fmul_rn(S[1], 1.0f / 512.f);
    const float b2 = __fmul_rn(S[2], 1.0f / 262144.f);
    const float b3 = __fmul_rn(S[3], 1.0f / 134217728.f);
    const float f = __fmaf_rn(S[5], 2.8421709430404007e-14f /* 2^-45 */,
                              __fmul_rn(S[4], 1.4551915228366852e-11f /* 2^-36 */));
    float s1, e1, s2, e2, s3, e3;
    fast_two_sum(S[0], b1, s1, e1);
    fast_two_sum(s1, b2, s2, e2);
    fast_two_sum(s2, b3, s3, e3);
    const float t = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(e3, f));
    fast_two_sum(s3, t, h, l);
}

// The double nearest (h + l) 2^off for a normalized double-float, assembled
// with integer operations, without branches (0 for h = 0 and below the
// double range).
__device__ __forceinline__ double df_to_double_scaled(float h, float l, int off) {
    const uint32_t hb = __float_as_uint(h);
    const int eh = (int)((hb >> 23) & 0xFFu);
    const int be = eh + 896 + off;
    const unsigned long long keep = (eh == 0 || be <= 0) ? 0ULL : ~0ULL;
    const uint32_t sg = hb & 0x80000000u;
    const uint32_t whi = ((uint32_t)be << 20) | ((hb & 0x7FFFFFu) >> 3) | sg;
    const uint32_t wlo = hb << 29;
    // l in units of the double's last place (2^(eh - 179)), with h's sign;
    // when h is a power of two and l points toward zero, the result lies in
    // the binade below, whose last place is half as large
    const uint32_t lb = __float_as_uint(l);
    const int below = ((hb & 0x7FFFFFu) == 0u && l != 0.f && ((lb ^ hb) & 0x80000000u)) ? 1 : 0;
    const int se = min(306 - eh + below, 254);
    const int delta = __float2int_rn(__fmul_rn(l, __uint_as_float(((uint32_t)se << 23) | sg)));
    unsigned long long w = ((unsigned long long)whi << 32) | wlo;
    // magnitude bits plus the signed correction, sign bit kept
    w = (w & 0x7FFFFFFFFFFFFFFFULL) + (unsigned long long)(long long)delta;
    w |= (unsigned long long)sg << 32;
    return __longlong_as_double((long long)(w & keep));
}

// ------------------------------------------------------------------ element-wise runs
// A run of diagonal / scalar gates multiplies every amplitude by the product
// of its gates' entries. Within one tile that product depends only on the
// run's target and control slots inside the tile (at most kUmmaRunBits; the
// positions outside the tile are fixed by the tile base), so each tile first
// tabulates it (double-float, one entry per combination of those slots) and
// every amplitude then takes one table entry.

// pext of a 12-bit tile index over the run's slots, from two 64-entry tables
__device__ __forceinline__ uint32_t run_index(const uint8_t* lut, uint32_t L) { return lut[L & 63u] | lut[64 + (L >> 6)]; }

// table entry i: the run's product at the tile index whose run slots hold i
__device__ __forceinline__ float4 run_entry(const float4* __restrict__ pool, const PassDesc& d, int o0, int o1,
                                            uint32_t mask, uint32_t i, uint64_t base) {
    uint32_t L = 0;
    for (int sl = 0; sl < 12; ++sl)
        if ((mask >> sl) & 1u) {
            L |= (i & 1u) << sl;
            i >>= 1;
        }
    float4 x = make_float4(1.f, 0.f, 0.f, 0.f);
    for (int o = o0; o < o1; ++o) {
        const OpDesc& op = d.ops[o];
        if ((base & op.ctrl_outer) != op.ctrl_outer) continue;
        if (op.k == 0) {
            x = ArithDF::mul(pool[op.mat_off], x);
            continue;
        }
        if ((L & op.ctrl_local) != op.ctrl_local) continue;
        int r = 0;
        for (int j = 0; j < op.k; ++j) {
            const int sl = op.tslot[j];
            const uint64_t bit = (sl & kOuterSlot) ? (base >> (sl & 63)) : ((uint64_t)L >> sl);
            r |= (int)(bit & 1ULL) << j;
        }
        x = ArithDF::mul(pool[op.mat_off + r], x);
    }
    return x;
}

__device__ __forceinline__ void run_apply(double2* buf, const float4* tab, const uint8_t* lut) {
    for (int L = threadIdx.x; L < 4096; L += kCompute) {
        const float4 x = ArithDFRaw::elem_load(buf[L]);
        buf[L] = ArithDFRaw::elem_store(ArithDF::mul(tab[run_index(lut, (uint32_t)L)], x));
    }
}

// ------------------------------------------------------------------ complex64
// The complex64 instance writes every state real as three balanced base-2^9
// digits relative to its group's largest float exponent Ef (X' = x 2^k,
// k = min(134 - Ef, 126), |X'| < 2^8: d0 = X' rounded to an integer, then two
// more rounded 9-bit digits, X' to 2^-19, 2^-27 of the group's scale), every
// gate real as four digits relative to its column (|B'| < 2^7, top digit
// <= 128; the gate to 2^-35 of its column's scale). The products with
// i + j = 0..3 go to four FP32 accumulator regions; every level sum stays
// below 2^24 (levels 2 and 3, the largest: 64 (256^2 + 256^2 + 256 * 128)
// and 64 * 3 * 256^2, below 2^23.6), so the accumulators hold exact
// integers and the tensor cores' rounding of their accumulation never
// applies. The dropped levels 4-5 are below 2^-34 of the row-times-column
// scale. The output is sum_L S_L 2^(-9 L) by an FMA chain (error below
// 2^-23 of sum_k |x_k b_kn|), times the column's and the group's scale.

// X' = x 2^k; each digit rounds with the magic-number add folded into an FMA
// (the product by 512 is exact, so the FMA rounds once, to an integer)
__device__ __forceinline__ void digits3(float x, float sk, float (&dg)[3]) {
    const float X = __fmul_rn(x, sk);
    dg[0] = __fsub_rn(__fadd_rn(X, kMagic0), kMagic0);
    const float r = __fsub_rn(X, dg[0]);
    dg[1] = __fsub_rn(__fmaf_rn(r, 512.f, kMagic0), kMagic0);
    const float u = __fmaf_rn(r, 512.f, -dg[1]);
    dg[2] = __fsub_rn(__fmaf_rn(u, 512.f, kMagic0), kMagic0);
}

// sum_L S_L 2^(-9 L) for the four exact level sums
__device__ __forceinline__ float level_sum4(const float (&S)[4]) {
    const float t = __fmaf_rn(S[2], 1.0f / 262144.f, __fmul_rn(S[3], 1.0f / 134217728.f));
    return __fadd_rn(S[0], __fmaf_rn(S[1], 1.0f / 512.f, t));
}

// run_entry for complex64: FP32 complex products of the run's entries
__device__ __forceinline__ float2 run_entry64(const float2* __restrict__ pool, const PassDesc& d, int o0, int o1,
                                              uint32_t mask, uint32_t i, uint64_t base) {
    uint32_t L = 0;
    for (int sl = 0; sl < 12; ++sl)
        if ((mask >> sl) & 1u) {
            L |= (i & 1u) << sl;
            i >>= 1;
        }
    float2 x = make_float2(1.f, 0.f);
    for (int o = o0; o < o1; ++o) {
        const OpDesc& op = d.ops[o];
        if ((base & op.ctrl_outer) != op.ctrl_outer) continue;
        if (op.k == 0) {
            x = ArithF32::mul(pool[op.mat_off], x);
            continue;
        }
        if ((L & op.ctrl_local) != op.ctrl_local) continue;
        int r = 0;
        for (int j = 0; j < op.k; ++j) {
            const int sl = op.tslot[j];
            const uint64_t bit = (sl & kOuterSlot) ? (base >> (sl & 63)) : ((uint64_t)L >> sl);
            r |= (int)(bit & 1ULL) << j;
        }
        x = ArithF32::mul(pool[op.mat_off + r], x);
    }
    return x;
}

__device__ __forceinline__ void run_apply64(float2* buf, const float2* tab, const uint8_t* lut) {
    for (int L = threadIdx.x; L < 4096; L += kCompute) buf[L] = ArithF32::mul(tab[run_index(lut, (uint32_t)L)], buf[L]);
}

// ------------------------------------------------------------------ kernel
template <bool C64>
__global__ void __launch_bounds__(kThreadsU, 1)
    umma_pass_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ UmmaDesc u,
                     const unsigned char* __restrict__ pool, int* __restrict__ err) {
    using S = Sm<C64>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const PassDesc& d = u.d;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + S::kBar);
    uint64_t* full = bars;        // [2] tile loaded
    uint64_t* tdone = bars + 2;   // [2] tile computed
    uint64_t* pbar = bars + 4;    // state digits written
    uint64_t* mbar = bars + 5;    // MMAs complete
    uint64_t* mbar0 = bars + 6;   // output halves: MMAs of outputs 0-31 complete
    uint32_t* tmem_s = reinterpret_cast<uint32_t*>(sm + S::kMisc);
    volatile int* abort = reinterpret_cast<volatile int*>(sm + S::kMisc + 8);
    int* erow = reinterpret_cast<int*>(sm + S::kErow);
    const int* ecol = reinterpret_cast<const int*>(sm + S::kEcol);
    uint32_t* mxs = reinterpret_cast<uint32_t*>(sm + S::kMx);
    uint16_t* gb = reinterpret_cast<uint16_t*>(sm + S::kGb);
    uint16_t* offt = reinterpret_cast<uint16_t*>(sm + S::kOff);
    uint8_t* lut = sm + S::kLut;

    const uint64_t ntiles = 1ULL << (d.n - d.nins);
    const uint64_t my_n = (uint64_t)blockIdx.x < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

    // ---- set-up
    if (threadIdx.x == 0) {
        for (int i = 0; i < 7; ++i) mbar_init(&bars[i], 1);
        *abort = 0;
        mbar_init_fence();
    }
    if (warp == kMmaWarp) tmem_alloc(tmem_s, kTmemCols);
    if (threadIdx.x < kCompute) {
        const uint4* gsrc = reinterpret_cast<const uint4*>(pool + u.gate_off);
        uint4* gdst = reinterpret_cast<uint4*>(sm + S::kGate);
        for (int i = threadIdx.x; i < (int)(S::kGateBytes / 16); i += kCompute) gdst[i] = gsrc[i];
        if (threadIdx.x < 64) {
            const int ec = reinterpret_cast<const int*>(pool + u.gate_off + S::kGateBytes)[threadIdx.x];
            if constexpr (C64) {
                // the column's scale 2^(ec - 1029) as a float (subnormal or 0
                // for columns far below 1; a unitary's columns are not)
                const int e = ec - 1029;
                const uint32_t bits = e >= -126 ? (uint32_t)(e + 127) << 23 : e >= -149 ? 1u << (e + 149) : 0u;
                reinterpret_cast<float*>(sm + S::kEcol)[threadIdx.x] = __uint_as_float(bits);
            } else {
                reinterpret_cast<int*>(sm + S::kEcol)[threadIdx.x] = ec;
            }
        }
        const uint4* esrc = reinterpret_cast<const uint4*>(pool);
        uint4* edst = reinterpret_cast<uint4*>(sm + S::kEw);
        // whole 16-byte chunks (complex64 entries are 8 bytes; the pool's
        // element-wise block is padded to the gate block's 1024-byte offset)
        for (int i = threadIdx.x; i < (int)((u.ew_bytes + 15) / 16); i += kCompute) edst[i] = esrc[i];
        // group g's first tile index: g's bits deposited over the slots that
        // are not targets; input e's offset: e's bits over the target slots
        uint32_t tmask = 0;
        for (int j = 0; j < 5; ++j) tmask |= 1u << u.tslot[j];
        if (threadIdx.x < 128) {
            uint32_t v = 0, g = threadIdx.x;
            for (int s = 0; s < 12; ++s)
                if (!((tmask >> s) & 1u)) {
                    v |= (g & 1u) << s;
                    g >>= 1;
                }
            gb[threadIdx.x] = (uint16_t)v;
        } else if (threadIdx.x < 160) {
            const uint32_t e = threadIdx.x - 128;
            uint32_t v = 0;
            for (int j = 0; j < 5; ++j) v |= ((e >> j) & 1u) << u.tslot[j];
            offt[e] = (uint16_t)v;
        }
        // factor-table index of tile slots 0-5 and 6-11, per run
        for (int t = threadIdx.x; t < 256; t += kCompute) {
            const int r = t >> 7, hi = (t >> 6) & 1;
            const uint32_t v = (uint32_t)(t & 63) << (hi * 6), m = u.run_mask[r];
            uint32_t idx = 0, k = 0;
            for (int sl = 0; sl < 12; ++sl)
                if ((m >> sl) & 1u) {
                    idx |= ((v >> sl) & 1u) << k;
                    ++k;
                }
            lut[t] = (uint8_t)idx;
        }
    }
    fence_proxy_async();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_s;

    if (warp == kTmaWarp) {
        // ---- tile loads and stores
        const uint32_t ncopy = 1u << u.nextra;
        uint32_t issued[2] = {0, 0};
        auto load = [&](uint64_t b, int s) {
            unsigned char* buf = sm + (s ? S::kTile1 : S::kTile0);
            if (lane == 0) {
                mbar_arrive_expect_tx(&full[s], S::kTileBytes);
                for (uint32_t c = 0; c < ncopy; ++c) {
                    int32_t co[5];
                    tile_coords(u, b, c, co);
                    tma_load(buf + (size_t)c * u.box_bytes, &tmap, co, u.rank, &full[s]);
                }
            }
            ++issued[s];
        };
        const Walk walk(d, blockIdx.x, gridDim.x);
        uint64_t lb = walk.base;  // base of the next tile to load
        if (my_n > 0) {
            load(lb, 0);
            lb = walk.after(lb);
        }
        if (my_n > 1) {
            load(lb, 1);
            lb = walk.after(lb);
        }
        uint64_t sb = walk.base;  // base of the next tile to store
        for (uint64_t it = 0; it < my_n; ++it) {
            const int s = (int)(it & 1);
            bool ok = true;
            if (lane == 0) ok = mbar_wait(&tdone[s], (uint32_t)((it >> 1) & 1), abort);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            if (lane == 0) {
                const unsigned char* buf = sm + (s ? S::kTile1 : S::kTile0);
                for (uint32_t c = 0; c < ncopy; ++c) {
                    int32_t co[5];
                    tile_coords(u, sb, c, co);
                    tma_store(&tmap, co, u.rank, buf + (size_t)c * u.box_bytes);
                }
                bulk_commit();
                bulk_wait_read0();
            }
            __syncwarp();
            sb = walk.after(sb);
            if (it + 2 < my_n) {
                load(lb, s);
                lb = walk.after(lb);
            }
        }
        if (lane == 0) {
            bulk_wait0();
            // loads still in flight (a loop left early): wait for them before
            // the CTA's shared memory goes away
            for (int s = 0; s < 2; ++s)
                if (issued[s]) mbar_wait_quiet(&full[s], (issued[s] - 1) & 1u);
        }
        __syncwarp();
    } else if (warp == kMmaWarp) {
        // ---- MMA issue
        const uint32_t idesc256 = idesc_f16(128, 256), idesc192 = idesc_f16(128, 192), idesc160 = idesc_f16(128, 160),
                       idesc128 = idesc_f16(128, 128), idesc96 = idesc_f16(128, 96), idesc64 = idesc_f16(128, 64),
                       idesc32 = idesc_f16(128, 32);
        const uint32_t gate = smem_u32(sm + S::kGate), planes = smem_u32(sm + S::kPlanes);
        // complex128 passes that hold only the dense gate: outputs in two halves
        const bool halves = !C64 && d.nops == 1;
        uint64_t committed = 0;
        for (uint64_t it = 0; it < my_n; ++it) {
            bool ok = true;
            if (lane == 0) ok = mbar_wait(pbar, (uint32_t)(it & 1), abort);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            fence_after_sync();
            if (lane == 0 && halves) {
                // outputs 0-31, then 32-63: per half six level regions of 32
                // columns and the gate rows of the half (six planes of 32
                // rows), so that X_i times gate digits 0..5-i is one MMA
#pragma unroll
                for (int h = 0; h < 2; ++h) {
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks) {
                        const uint64_t g0 = sdesc_sw128(gate + (uint32_t)h * 24576u + (uint32_t)ks * 32u);
                        auto ta = [&](int i) { return tmem + S::kTmPlanes + (uint32_t)i * 32u + (uint32_t)ks * 8u; };
                        auto td = [&](int lev) { return tmem + (uint32_t)h * 192u + (uint32_t)lev * 32u; };
                        mma_ts(td(0), ta(0), g0, idesc192, ks > 0 ? 1u : 0u);  // levels 0-5
                        mma_ts(td(1), ta(1), g0, idesc160, 1u);                // levels 1-5
                        mma_ts(td(2), ta(2), g0, idesc128, 1u);                // levels 2-5
                        mma_ts(td(3), ta(3), g0, idesc96, 1u);                 // levels 3-5
                        mma_ss(td(4), sdesc_sw128(planes + (uint32_t)ks * 32u), g0, idesc64, 1u);           // levels 4-5
                        mma_ss(td(5), sdesc_sw128(planes + 16384u + (uint32_t)ks * 32u), g0, idesc32, 1u);  // level 5
                    }
                    mma_commit(h == 0 ? mbar0 : mbar);
                }
            } else if (lane == 0) {
#pragma unroll
                for (int ks = 0; ks < 4; ++ks) {
                    // X_i times gate digits j0.. accumulates at level region i + j0
                    auto gdesc = [&](int j0) { return sdesc_sw128(gate + (uint32_t)j0 * 8192u + (uint32_t)ks * 32u); };
                    auto ta = [&](int i) { return tmem + S::kTmPlanes + (uint32_t)i * 32u + (uint32_t)ks * 8u; };
                    auto td = [&](int lev) { return tmem + (uint32_t)lev * 64u; };
                    const uint32_t acc0 = ks > 0 ? 1u : 0u;
                    if constexpr (C64) {
                        mma_ts(td(0), ta(0), gdesc(0), idesc256, acc0);  // levels 0-3 (gate digits 0-3)
                        mma_ts(td(1), ta(1), gdesc(0), idesc192, 1u);    // levels 1-3
                        mma_ts(td(2), ta(2), gdesc(0), idesc128, 1u);    // levels 2-3
                    } else {
                        mma_ts(td(0), ta(0), gdesc(0), idesc256, acc0);  // levels 0-3
                        mma_ts(td(4), ta(0), gdesc(4), idesc128, acc0);  // levels 4-5
                        mma_ts(td(1), ta(1), gdesc(0), idesc256, 1u);    // levels 1-4
                        mma_ts(td(5), ta(1), gdesc(4), idesc64, 1u);     // level 5
                        mma_ts(td(2), ta(2), gdesc(0), idesc256, 1u);    // levels 2-5
                        mma_ts(td(3), ta(3), gdesc(0), idesc192, 1u);    // levels 3-5
                        const uint64_t a4 = sdesc_sw128(planes + (uint32_t)ks * 32u);
                        const uint64_t a5 = sdesc_sw128(planes + 16384u + (uint32_t)ks * 32u);
                        mma_ss(td(4), a4, gdesc(0), idesc128, 1u);       // levels 4-5
                        mma_ss(td(5), a5, gdesc(0), idesc64, 1u);        // level 5
                    }
                }
                mma_commit(mbar);
            }
            __syncwarp();
            committed = it + 1;
        }
        if (committed > 0 && lane == 0) {
            // the last MMAs must be complete before tensor memory is freed
            mbar_wait_quiet(mbar, (uint32_t)((committed - 1) & 1));
        }
        __syncwarp();
    } else if constexpr (!C64) {
        // ---- compute warps (complex128): digits, then outputs. The runs' factor tables
        // are built while the MMAs of the tile run: the post-run table of
        // this tile and the pre-run table of the next (the pre-run table of
        // the first tile before the loop). A pre-run is applied while the
        // digits are formed (the amplitudes stay double-floats in
        // registers), a post-run while the outputs are assembled.
        const int q4 = warp & 3, part = warp >> 2, g = q4 * 32 + lane;
        const OpDesc& tc = d.ops[u.tc_op];
        const uint32_t lane_base = (uint32_t)(q4 * 32) << 16;
        const bool pre = u.tc_op > 0, post = u.tc_op + 1 < d.nops, halves = d.nops == 1;
        const int npre = pre ? 1 << __popc(u.run_mask[0]) : 0, npost = post ? 1 << __popc(u.run_mask[1]) : 0;
        float4* tab_pre = reinterpret_cast<float4*>(sm + S::kTab);
        float4* tab_post = tab_pre + (1 << kUmmaRunBits);
        const float4* ewp = reinterpret_cast<const float4*>(sm + S::kEw);
        const uint8_t* lut_pre = lut;
        const uint8_t* lut_post = lut + 128;
        auto build_pre = [&](uint64_t b) {
            for (int i = threadIdx.x; i < npre; i += kCompute)
                tab_pre[i] = run_entry(ewp, d, 0, u.tc_op, u.run_mask[0], (uint32_t)i, b);
        };
        auto build_post = [&](uint64_t b) {
            for (int i = threadIdx.x; i < npost; i += kCompute)
                tab_post[i] = run_entry(ewp, d, u.tc_op + 1, d.nops, u.run_mask[1], (uint32_t)i, b);
        };
        const Walk walk(d, blockIdx.x, gridDim.x);
        uint64_t base = walk.base;
        if (my_n > 0) build_pre(base);
        for (uint64_t it = 0; it < my_n; ++it, base = walk.after(base)) {
            const int s = (int)(it & 1);
            double2* buf = reinterpret_cast<double2*>(sm + (s ? S::kTile1 : S::kTile0));
            mbar_wait(&full[s], (uint32_t)((it >> 1) & 1), abort);
            bar_sync(1, kCompute);
            if (*abort) break;
            const bool act = (base & tc.ctrl_outer) == tc.ctrl_outer;
            const uint32_t gbase = gb[g];
            // a group whose in-tile controls are not all 1 keeps its inputs
            // (with the runs applied)
            const bool write = (gbase & tc.ctrl_local) == tc.ctrl_local;
            if (act) {
                // digit planes of the tile's 128 groups; this thread: group g,
                // inputs 8 part .. 8 part + 7
                uint32_t mx = 0;
                if (pre) {
                    float4 xf[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const uint32_t L = gbase | offt[part * 8 + i];
                        xf[i] = ArithDF::mul(tab_pre[run_index(lut_pre, L)], ArithDFRaw::elem_load(buf[L]));
                        if (!write) buf[L] = ArithDFRaw::elem_store(xf[i]);
                        mx = max(mx, __float_as_uint(xf[i].x) & 0x7FFFFFFFu);
                        mx = max(mx, __float_as_uint(xf[i].y) & 0x7FFFFFFFu);
                    }
                    mxs[threadIdx.x] = mx;
                    bar_sync(1, kCompute);
                    const int Ef = (int)(max(max(mxs[g], mxs[128 + g]), max(mxs[256 + g], mxs[384 + g])) >> 23);
                    if (part == 0) erow[g] = Ef == 0 ? 0 : Ef + 896;
#pragma unroll
                    for (int bt = 0; bt < 2; ++bt) {
                        uint32_t pl[6][4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            float dr[6], di[6];
                            const float4 v = xf[bt * 4 + i];
                            digits6_df(v.x, v.z, Ef, dr);
                            digits6_df(v.y, v.w, Ef, di);
#pragma unroll
                            for (int q = 0; q < 6; ++q) pl[q][i] = pack_h2(dr[q], di[q]);
                        }
                        const uint32_t e0 = (uint32_t)(part * 8 + bt * 4);
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            tmem_st4(tmem + lane_base + S::kTmPlanes + (uint32_t)q * 32u + e0, pl[q][0], pl[q][1], pl[q][2], pl[q][3]);
                        const uint32_t c0 = e0 >> 2;
#pragma unroll
                        for (int q = 4; q < 6; ++q) {
                            unsigned char* row = sm + S::kPlanes + (uint32_t)(q - 4) * 16384u + (uint32_t)g * 128u;
                            *reinterpret_cast<uint4*>(row + ((c0 ^ (g & 7)) << 4)) =
                                make_uint4(pl[q][0], pl[q][1], pl[q][2], pl[q][3]);
                        }
                    }
                } else {
                    double2 x[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        x[i] = buf[gbase | offt[part * 8 + i]];
                        mx = max(mx, (uint32_t)__double2hiint(x[i].x) & 0x7FFFFFFFu);
                        mx = max(mx, (uint32_t)__double2hiint(x[i].y) & 0x7FFFFFFFu);
                    }
                    mxs[threadIdx.x] = mx;
                    bar_sync(1, kCompute);
                    const int Eb = (int)(max(max(mxs[g], mxs[128 + g]), max(mxs[256 + g], mxs[384 + g])) >> 20);
                    if (part == 0) erow[g] = Eb;
#pragma unroll
                    for (int bt = 0; bt < 2; ++bt) {
                        uint32_t pl[6][4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            float dr[6], di[6];
                            digits6(x[bt * 4 + i].x, Eb, dr);
                            digits6(x[bt * 4 + i].y, Eb, di);
#pragma unroll
                            for (int q = 0; q < 6; ++q) pl[q][i] = pack_h2(dr[q], di[q]);
                        }
                        const uint32_t e0 = (uint32_t)(part * 8 + bt * 4);
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            tmem_st4(tmem + lane_base + S::kTmPlanes + (uint32_t)q * 32u + e0, pl[q][0], pl[q][1], pl[q][2], pl[q][3]);
                        const uint32_t c0 = e0 >> 2;
#pragma unroll
                        for (int q = 4; q < 6; ++q) {
                            unsigned char* row = sm + S::kPlanes + (uint32_t)(q - 4) * 16384u + (uint32_t)g * 128u;
                            *reinterpret_cast<uint4*>(row + ((c0 ^ (g & 7)) << 4)) =
                                make_uint4(pl[q][0], pl[q][1], pl[q][2], pl[q][3]);
                        }
                    }
                }
                tmem_st_wait();
                fence_proxy_async();
            } else if (pre) {
                // the dense gate leaves this tile alone: the runs apply as they are
                run_apply(buf, tab_pre, lut_pre);
            }
            fence_before_sync();
            bar_sync(1, kCompute);
            if (threadIdx.x == 0) mbar_arrive(pbar);
            // while the MMAs run: this tile's post-run table, the next tile's pre-run table
            if (post) build_post(base);
            if (pre && it + 1 < my_n) build_pre(walk.after(base));
            if (halves) {
                // output halves (a pass without runs): outputs 0-31 as soon as
                // their MMAs are complete, while the MMAs of outputs 32-63 run,
                // then outputs 32-63
                bool stop = false;
    #pragma unroll 1
                for (int h = 0; h < 2; ++h) {
                    {
                        mbar_wait(h == 0 ? mbar0 : mbar, (uint32_t)(it & 1), abort);
                        bar_sync(1, kCompute);
                        if (*abort) {
                            stop = true;
                            break;
                        }
                        fence_after_sync();
                    }
                    if (!act) continue;
                    // group g, output reals nb = 32 h + 8 part .. nb + 7 in two chunks
                    // of four: the second chunk's loads are in flight while the
                    // first is assembled. Level L of output n lies at column
                    // 192 h + 32 L + n mod 32. The tensor-memory loads are
                    // warp-collective: every thread takes part, also for a group
                    // that keeps its inputs.
                    const int Eb = erow[g];
                    const uint32_t nb = (uint32_t)(h * 32 + part * 8);
                    const uint32_t cb = lane_base + (uint32_t)(h * 192 + part * 8);
                    constexpr uint32_t ls = 32u;
                    uint32_t r[2][6][4];
    #pragma unroll
                    for (int lev = 0; lev < 6; ++lev) tmem_ld4(tmem + cb + (uint32_t)lev * ls, r[0][lev]);
                    tmem_ld_wait_regs(r[0]);
    #pragma unroll
                    for (int ch = 0; ch < 2; ++ch) {
                        const uint32_t n0 = nb + (uint32_t)(ch * 4);
                        if (ch == 0) {
    #pragma unroll
                            for (int lev = 0; lev < 6; ++lev) tmem_ld4(tmem + cb + (uint32_t)lev * ls + 4u, r[1][lev]);
                        }
    #pragma unroll
                        for (int a = 0; a < 2; ++a) {
                            const uint32_t L = gbase | offt[(n0 >> 1) + a];
                            if (!write) {  // the pre-run was stored with the digits
                                if (post)
                                    buf[L] = ArithDFRaw::elem_store(
                                        ArithDF::mul(tab_post[run_index(lut_post, L)], ArithDFRaw::elem_load(buf[L])));
                                continue;
                            }
                            float hh[2], l[2];
    #pragma unroll
                            for (int p = 0; p < 2; ++p) {
                                const int c = a * 2 + p;
                                const float S[6] = {__uint_as_float(r[ch][0][c]), __uint_as_float(r[ch][1][c]),
                                                    __uint_as_float(r[ch][2][c]), __uint_as_float(r[ch][3][c]),
                                                    __uint_as_float(r[ch][4][c]), __uint_as_float(r[ch][5][c])};
                                level_sum_to_df(S, hh[p], l[p]);
                            }
                            if (post) {
                                const float4 v = ArithDF::mul(tab_post[run_index(lut_post, L)], make_float4(hh[0], hh[1], l[0], l[1]));
                                hh[0] = v.x;
                                hh[1] = v.y;
                                l[0] = v.z;
                                l[1] = v.w;
                            }
                            // a zero group (Eb = 0): the offset puts every output below
                            // the double range, so it is 0 (no branch)
                            const int c0 = a * 2, ez = Eb == 0 ? -4096 : 0;
                            buf[L] = make_double2(df_to_double_scaled(hh[0], l[0], Eb + ez + ecol[n0 + c0] - 2059),
                                                  df_to_double_scaled(hh[1], l[1], Eb + ez + ecol[n0 + c0 + 1] - 2059));
                        }
                        if (ch == 0) tmem_ld_wait_regs(r[1]);
                    }
                }
                if (stop) break;
            } else {
                mbar_wait(mbar, (uint32_t)(it & 1), abort);
                bar_sync(1, kCompute);
                if (*abort) break;
                fence_after_sync();
                if (act) {
                    // outputs: group g, output reals 16 part .. 16 part + 15. The
                    // tensor-memory loads are warp-collective: every thread takes
                    // part, also for a group that keeps its inputs.
                    const int Eb = erow[g];
                    // four chunks of four output reals; the next chunk's loads are
                    // in flight while the current one is assembled
                    uint32_t r[4][6][4];
    #pragma unroll
                    for (int lev = 0; lev < 6; ++lev) tmem_ld4(tmem + lane_base + (uint32_t)lev * 64u + (uint32_t)(part * 16), r[0][lev]);
                    tmem_ld_wait_regs(r[0]);
    #pragma unroll
                    for (int ch = 0; ch < 4; ++ch) {
                        const uint32_t n0 = (uint32_t)(part * 16 + ch * 4);
                        if (ch < 3) {
    #pragma unroll
                            for (int lev = 0; lev < 6; ++lev)
                                tmem_ld4(tmem + lane_base + (uint32_t)lev * 64u + n0 + 4u, r[ch + 1][lev]);
                        }
    #pragma unroll
                        for (int a = 0; a < 2; ++a) {
                            const uint32_t L = gbase | offt[(n0 >> 1) + a];
                            if (!write) {  // the pre-run was stored with the digits
                                if (post)
                                    buf[L] = ArithDFRaw::elem_store(
                                        ArithDF::mul(tab_post[run_index(lut_post, L)], ArithDFRaw::elem_load(buf[L])));
                                continue;
                            }
                            float h[2], l[2];
    #pragma unroll
                            for (int p = 0; p < 2; ++p) {
                                const int c = a * 2 + p;
                                const float S[6] = {__uint_as_float(r[ch][0][c]), __uint_as_float(r[ch][1][c]),
                                                    __uint_as_float(r[ch][2][c]), __uint_as_float(r[ch][3][c]),
                                                    __uint_as_float(r[ch][4][c]), __uint_as_float(r[ch][5][c])};
                                level_sum_to_df(S, h[p], l[p]);
                            }
                            if (post) {
                                const float4 v = ArithDF::mul(tab_post[run_index(lut_post, L)], make_float4(h[0], h[1], l[0], l[1]));
                                h[0] = v.x;
                                h[1] = v.y;
                                l[0] = v.z;
                                l[1] = v.w;
                            }
                            // a zero group (Eb = 0): the offset puts every output below
                            // the double range, so it is 0 (no branch)
                            const int c0 = a * 2, ez = Eb == 0 ? -4096 : 0;
                            buf[L] = make_double2(df_to_double_scaled(h[0], l[0], Eb + ez + ecol[n0 + c0] - 2059),
                                                  df_to_double_scaled(h[1], l[1], Eb + ez + ecol[n0 + c0 + 1] - 2059));
                        }
                        if (ch < 3) tmem_ld_wait_regs(r[ch + 1]);
                    }
                } else if (post) {
                    run_apply(buf, tab_post, lut_post);
                }
            }
            fence_proxy_async();
            fence_before_sync();
            bar_sync(1, kCompute);
            if (threadIdx.x == 0) mbar_arrive(&tdone[s]);
        }
    } else {
        // ---- compute warps (complex64): three digits per state real (exact
        // levels 0-3), runs in FP32 complex, outputs rounded to float
        const int q4 = warp & 3, part = warp >> 2, g = q4 * 32 + lane;
        const OpDesc& tc = d.ops[u.tc_op];
        const uint32_t lane_base = (uint32_t)(q4 * 32) << 16;
        const bool pre = u.tc_op > 0, post = u.tc_op + 1 < d.nops;
        const int npre = pre ? 1 << __popc(u.run_mask[0]) : 0, npost = post ? 1 << __popc(u.run_mask[1]) : 0;
        float2* tab_pre = reinterpret_cast<float2*>(sm + S::kTab);
        float2* tab_post = tab_pre + (1 << kUmmaRunBits);
        const float2* ewp = reinterpret_cast<const float2*>(sm + S::kEw);
        const uint8_t* lut_pre = lut;
        const uint8_t* lut_post = lut + 128;
        auto build_pre = [&](uint64_t b) {
            for (int i = threadIdx.x; i < npre; i += kCompute)
                tab_pre[i] = run_entry64(ewp, d, 0, u.tc_op, u.run_mask[0], (uint32_t)i, b);
        };
        auto build_post = [&](uint64_t b) {
            for (int i = threadIdx.x; i < npost; i += kCompute)
                tab_post[i] = run_entry64(ewp, d, u.tc_op + 1, d.nops, u.run_mask[1], (uint32_t)i, b);
        };
        const Walk walk(d, blockIdx.x, gridDim.x);
        uint64_t base = walk.base;
        if (my_n > 0) build_pre(base);
        for (uint64_t it = 0; it < my_n; ++it, base = walk.after(base)) {
            const int s = (int)(it & 1);
            float2* buf = reinterpret_cast<float2*>(sm + (s ? S::kTile1 : S::kTile0));
            mbar_wait(&full[s], (uint32_t)((it >> 1) & 1), abort);
            bar_sync(1, kCompute);
            if (*abort) break;
            const bool act = (base & tc.ctrl_outer) == tc.ctrl_outer;
            const uint32_t gbase = gb[g];
            const bool write = (gbase & tc.ctrl_local) == tc.ctrl_local;
            if (act) {
                // group g, inputs 8 part .. 8 part + 7 (the pre-run applied)
                float2 xv[8];
                float mx = 0.f;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const uint32_t L = gbase | offt[part * 8 + i];
                    float2 v = buf[L];
                    if (pre) {
                        v = ArithF32::mul(tab_pre[run_index(lut_pre, L)], v);
                        if (!write) buf[L] = v;
                    }
                    xv[i] = v;
                    mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
                }
                reinterpret_cast<float*>(mxs)[threadIdx.x] = mx;
                bar_sync(1, kCompute);
                const float* mxf = reinterpret_cast<const float*>(mxs);
                const int Ef = (int)(__float_as_uint(fmaxf(fmaxf(mxf[g], mxf[128 + g]), fmaxf(mxf[256 + g], mxf[384 + g]))) >> 23);
                // X' = x 2^k; the group's output scale is 2^-k (0: all zero)
                const int k = min(134 - Ef, 126);
                if (part == 0) erow[g] = Ef == 0 ? 0 : 127 - k;
                const float sk = __uint_as_float((uint32_t)(k + 127) << 23);
#pragma unroll
                for (int bt = 0; bt < 2; ++bt) {
                    uint32_t pl[3][4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        float dr[3], di[3];
                        digits3(xv[bt * 4 + i].x, sk, dr);
                        digits3(xv[bt * 4 + i].y, sk, di);
#pragma unroll
                        for (int q = 0; q < 3; ++q) pl[q][i] = pack_h2(dr[q], di[q]);
                    }
                    const uint32_t e0 = (uint32_t)(part * 8 + bt * 4);
#pragma unroll
                    for (int q = 0; q < 3; ++q)
                        tmem_st4(tmem + lane_base + S::kTmPlanes + (uint32_t)q * 32u + e0, pl[q][0], pl[q][1], pl[q][2], pl[q][3]);
                }
                tmem_st_wait();
            } else if (pre) {
                run_apply64(buf, tab_pre, lut_pre);
            }
            fence_before_sync();
            bar_sync(1, kCompute);
            if (threadIdx.x == 0) mbar_arrive(pbar);
            // while the MMAs run: this tile's post-run table, the next tile's pre-run table
            if (post) build_post(base);
            if (pre && it + 1 < my_n) build_pre(walk.after(base));
            mbar_wait(mbar, (uint32_t)(it & 1), abort);
            bar_sync(1, kCompute);
            if (*abort) break;
            fence_after_sync();
            if (act) {
                // outputs: group g, output reals 16 part .. 16 part + 15; the
                // tensor-memory loads are warp-collective (every thread takes part)
                const int gexp = erow[g];
                const float gs = __uint_as_float((uint32_t)gexp << 23);  // 0 for a zero group
                const float* cs = reinterpret_cast<const float*>(sm + S::kEcol);
                uint32_t r[4][4][4];
#pragma unroll
                for (int lev = 0; lev < 4; ++lev) tmem_ld4(tmem + lane_base + (uint32_t)lev * 64u + (uint32_t)(part * 16), r[0][lev]);
                tmem_ld_wait_regs(r[0]);
#pragma unroll
                for (int ch = 0; ch < 4; ++ch) {
                    const uint32_t n0 = (uint32_t)(part * 16 + ch * 4);
                    if (ch < 3) {
#pragma unroll
                        for (int lev = 0; lev < 4; ++lev)
                            tmem_ld4(tmem + lane_base + (uint32_t)lev * 64u + n0 + 4u, r[ch + 1][lev]);
                    }
#pragma unroll
                    for (int a = 0; a < 2; ++a) {
                        const uint32_t L = gbase | offt[(n0 >> 1) + a];
                        if (!write) {  // the pre-run was stored with the digits
                            if (post) buf[L] = ArithF32::mul(tab_post[run_index(lut_post, L)], buf[L]);
                            continue;
                        }
                        float y[2];
#pragma unroll
                        for (int p = 0; p < 2; ++p) {
                            const int c = a * 2 + p;
                            const float Sl[4] = {__uint_as_float(r[ch][0][c]), __uint_as_float(r[ch][1][c]),
                                                 __uint_as_float(r[ch][2][c]), __uint_as_float(r[ch][3][c])};
                            y[p] = __fmul_rn(__fmul_rn(level_sum4(Sl), cs[n0 + c]), gs);
                        }
                        float2 v = make_float2(y[0], y[1]);
                        if (post) v = ArithF32::mul(tab_post[run_index(lut_post, L)], v);
                        buf[L] = v;
                    }
                    if (ch < 3) tmem_ld_wait_regs(r[ch + 1]);
                }
                        } else if (post) {
                run_apply64(buf, tab_post, lut_post);
            }
            fence_proxy_async();
            fence_before_sync();
            bar_sync(1, kCompute);
            if (threadIdx.x == 0) mbar_arrive(&tdone[s]);
        }
    }

    // ---- tear-down
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == kMmaWarp) tmem_dealloc(tmem, kTmemCols);
    if (threadIdx.x == 0 && *abort) atomicOr(err, 1);
}

// ------------------------------------------------------------------ host
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

constexpr int kMaxDev = 64;
std::mutex g_umma_mu;
int* g_err_word[kMaxDev] = {nullptr};
bool g_attr_set[kMaxDev][2] = {};

int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return -1;
    return dev;
}

}  // namespace

size_t umma_smem_bytes() { return Sm<false>::kBytes; }

cudaError_t launch_umma_pass(void* state, const void* mats, const UmmaDesc& u, cudaStream_t s) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return cudaErrorNotSupported;
    const bool c64 = u.c64 != 0;
    // the state viewed as reals (doubles, or floats for complex64): each
    // dimension spans dim_bits state positions from dim_pos (dimension 0
    // also the re/im pair), its box the dim_box positions at its bottom
    const uint64_t amp = c64 ? 8 : 16;
    cuuint64_t gdim[5], gstr[4];
    cuuint32_t box[5], es[5];
    for (int i = 0; i < u.rank; ++i) {
        gdim[i] = (i == 0 ? 2ULL : 1ULL) << u.dim_bits[i];
        box[i] = (i == 0 ? 2u : 1u) << u.dim_box[i];
        es[i] = 1;
        if (i > 0) gstr[i - 1] = amp << u.dim_pos[i];
    }
    CUtensorMap tm;
    const CUresult r = enc(&tm, c64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                           (cuuint32_t)u.rank, state, gdim, u.rank > 1 ? gstr : nullptr, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    const int dev = current_device();
    if (dev < 0) return cudaErrorInvalidDevice;
    const uint32_t smem = c64 ? Sm<true>::kBytes : Sm<false>::kBytes;
    int* err = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_umma_mu);
        if (!g_err_word[dev]) {
            cudaError_t e = cudaMalloc(&g_err_word[dev], sizeof(int));
            if (e != cudaSuccess) return e;
            e = cudaMemset(g_err_word[dev], 0, sizeof(int));
            if (e != cudaSuccess) return e;
        }
        if (!g_attr_set[dev][c64 ? 1 : 0]) {
            cudaError_t e = c64 ? cudaFuncSetAttribute(umma_pass_kernel<true>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                                : cudaFuncSetAttribute(umma_pass_kernel<false>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            g_attr_set[dev][c64 ? 1 : 0] = true;
        }
        err = g_err_word[dev];
    }
    const uint64_t ntiles = 1ULL << (u.d.n - u.d.nins);
    const unsigned grid = (unsigned)std::min<uint64_t>(ntiles, (uint64_t)device_sm_count());
    if (c64)
        umma_pass_kernel<true><<<grid, kThreadsU, smem, s>>>(tm, u, static_cast<const unsigned char*>(mats), err);
    else
        umma_pass_kernel<false><<<grid, kThreadsU, smem, s>>>(tm, u, static_cast<const unsigned char*>(mats), err);
    return cudaGetLastError();
}

cudaError_t umma_check_error(bool* failed) {
    *failed = false;
    const int dev = current_device();
    if (dev < 0) return cudaSuccess;
    int* err = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_umma_mu);
        err = g_err_word[dev];
    }
    if (!err) return cudaSuccess;
    int h = 0;
    cudaError_t e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    if (h) {
        *failed = true;
        e = cudaMemset(err, 0, sizeof(int));
    }
    return e;
}

}  // namespace hqs
