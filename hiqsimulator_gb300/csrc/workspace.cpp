#include "workspace.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>

namespace hqs {

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

Workspace::Workspace() {
    cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaMalloc(&rs_.d_partials, sizeof(double) * kMaxPartials * 4), "cudaMalloc(partials)");
    cuda_check(cudaMalloc(&rs_.d_result, sizeof(double) * 4), "cudaMalloc(result)");
    cuda_check(cudaMallocHost(&rs_.h_result, sizeof(double) * 4), "cudaMallocHost(result)");
    cuda_check(cudaEventCreateWithFlags(&staging_free_, cudaEventDisableTiming), "cudaEventCreate");
}

Workspace::~Workspace() {
    if (stream_) cudaStreamSynchronize(stream_);
    cudaFree(rs_.d_partials);
    cudaFree(rs_.d_result);
    cudaFreeHost(rs_.h_result);
    cudaFree(pool_);
    cudaFreeHost(pinned_);
    cudaFree(scratch_);
    cudaFree(up_);
    if (staging_free_) cudaEventDestroy(staging_free_);
    for (auto& t : timed_) {
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    for (cudaEvent_t e : event_pool_) cudaEventDestroy(e);
    if (stream_) cudaStreamDestroy(stream_);
}

void Workspace::synchronize_checked() {
    cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    bool failed = false;
    cuda_check(umma_check_error(&failed), "umma_check_error");
    if (failed) throw CudaError("tensor-memory pass: a bounded device wait ran out (results of the pass are invalid)");
}

void* Workspace::scratch(size_t bytes) {
    if (bytes > scratch_bytes_) {
        cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        cudaFree(scratch_);
        scratch_ = nullptr;
        scratch_bytes_ = 0;
        cuda_check(cudaMalloc(&scratch_, bytes), "cudaMalloc(scratch)");
        scratch_bytes_ = bytes;
    }
    return scratch_;
}

void* Workspace::upload(const void* host, size_t bytes) {
    if (bytes > up_bytes_) {
        cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        cudaFree(up_);
        up_ = nullptr;
        up_bytes_ = 0;
        const size_t cap = std::max<size_t>(bytes, 4096);
        cuda_check(cudaMalloc(&up_, cap), "cudaMalloc(upload)");
        up_bytes_ = cap;
    }
    cuda_check(cudaMemcpyAsync(up_, host, bytes, cudaMemcpyHostToDevice, stream_), "cudaMemcpyAsync(upload)");
    // the host source may be reused by the caller right after return
    cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return up_;
}

void Workspace::ensure_pool(size_t bytes) {
    if (bytes <= pool_bytes_) return;
    cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    cudaFree(pool_);
    pool_ = nullptr;
    pool_bytes_ = 0;
    const size_t cap = std::max<size_t>(bytes * 2, 1 << 20);
    cuda_check(cudaMalloc(&pool_, cap), "cudaMalloc(matrix pool)");
    pool_bytes_ = cap;
}

void Workspace::ensure_pinned(size_t bytes) {
    if (staging_pending_) {
        cuda_check(cudaEventSynchronize(staging_free_), "cudaEventSynchronize");
        staging_pending_ = false;
    }
    if (bytes <= pinned_bytes_) return;
    cudaFreeHost(pinned_);
    pinned_ = nullptr;
    pinned_bytes_ = 0;
    const size_t cap = std::max<size_t>(bytes * 2, 1 << 20);
    cuda_check(cudaMallocHost(&pinned_, cap), "cudaMallocHost(staging)");
    pinned_bytes_ = cap;
}

static int popc64(uint64_t v) { return __builtin_popcountll(v); }

// Digits per state real (A) and per gate real (B) of the digit-plane
// tensor-core modes.
static int tc_digits(int arith) { return arith == kArithTC64 ? kTcDigits64 : kTcDigits; }
static int tc_digits_b(int arith) { return arith == kArithTC64 ? kTcDigits64B : kTcDigits; }

// Pool bytes of a tensor-core gate. Digit planes: int32 E_col[2D] + one
// plane per digit of 2D rows x (2D + 8) fp16. 3xTF32: (2D/8)^2 fragment
// blocks of 32 lanes x float4.
static size_t tc_pool_bytes(int arith, int k) {
    const size_t KK = (size_t)2 << k;
    if (arith == kArithTF32) return KK * KK * 8;
    return 4 * KK + (size_t)tc_digits_b(arith) * KK * (KK + 8) * 2;
}

// Shared-memory scratch of a digit-plane gate on a 2^q tile: the tile's
// digit planes (G = 2^(q-k) rows), the rows' exponents, and the tile
// offsets of the groups (G) and of the inputs (D).
static size_t tc_scratch_bytes(int arith, int q, int k) {
    if (arith == kArithTF32) return 0;
    const size_t G = (size_t)1 << (q - k), KK = (size_t)2 << k;
    return (size_t)tc_digits(arith) * G * (KK + 8) * 2 + 8 * G + 4 * (KK / 2);
}

// Dense gates that run on the tensor cores: k >= 3 for complex128 (the
// double-float alternative costs ~10 FP32 operations per real product);
// k = 5 only for complex64, whose FP32 gates are cheaper below that (measured
// in serving of <= 4-qubit fused gates: 174 circuits/s with 4-qubit gates on
// the tensor cores against 279 on FP32 cores)
bool tc_candidate(int arith, const GateOp& op) {
    if (!arith_has_tc(arith) || op.diag) return false;
    return op.k >= (arith == kArithTC ? 3 : 5);
}

// Pool elements (of mat_elem_bytes) an op occupies.
static size_t pool_elems(int arith, const GateOp& op, bool tc) {
    const size_t melem = Workspace::mat_elem_bytes(arith);
    if (tc) return (tc_pool_bytes(arith, op.k) + melem - 1) / melem;
    return op.m.size();
}

// Pass over ops [i, j): tile, op descriptors, prefetch mode, sweep bytes
// (pool_off is set by the caller).
static PassPlan build_pass(int n, int arith, const GateOp* ops, size_t i, size_t j, int max_tile_bits) {
    const size_t melem = Workspace::mat_elem_bytes(arith);
    const size_t store = arith_is_c64(arith) ? 8 : 16;
    uint64_t tset = 0;
    for (size_t o = i; o < j; ++o)
        if (!ops[o].diag)
            for (int t = 0; t < ops[o].k; ++t) tset |= 1ULL << ops[o].pos[t];
    PassPlan pl;
    PassDesc& d = pl.desc;
    std::memset(&d, 0, sizeof(d));
    // tile: the pass's targets plus at least 4 low positions, 2^10 amplitudes
    // at least (enough index groups for every thread), at most 2^max_tile_bits
    // complex128 digit-plane passes use 2^9-amplitude tiles (16 index
    // groups for a 5-qubit gate) so that three CTAs fit on an SM next to
    // the gate's digit planes; 3xTF32 passes 2^11 (64 groups: every warp
    // gets a task of four n-tiles)
    bool has_tc = false;
    for (size_t o = i; o < j; ++o) has_tc = has_tc || tc_candidate(arith, ops[o]);
    const int base_q = !has_tc ? 10 : arith == kArithTF32 ? 11 : arith == kArithTC ? 9 : 10;
    int q = std::min(n, std::max(popc64(tset), std::min(max_tile_bits, std::max(popc64(tset) + 4, base_q))));
    // keep the pass within one CTA's shared memory: shrink the tile (not
    // below the targets), then give up tensor-core gates if still too big
    bool allow_tc = true;
    auto smem_estimate = [&](int qq, bool tcok) {
        size_t mat = 0, tcb = 0;
        for (size_t o = i; o < j; ++o) {
            const bool tc = tcok && tc_candidate(arith, ops[o]) && qq >= ops[o].k + 4;
            mat += pool_elems(arith, ops[o], tc) * melem + (tc ? 8 : 0);
            if (tc) tcb = std::max(tcb, tc_scratch_bytes(arith, qq, ops[o].k));
        }
        return mat + 2 * (store << qq) + 8 * ((size_t)1 << qq) + 32 + tcb;
    };
    const size_t smem_budget = 200 * 1024;
    while (smem_estimate(q, allow_tc) > smem_budget && q > std::max(popc64(tset), std::min(n, 10))) --q;
    if (smem_estimate(q, allow_tc) > smem_budget) allow_tc = false;
    uint64_t tile = tset;
    for (int b = 0; b < n && popc64(tile) < q; ++b) tile |= 1ULL << b;
    int slot[64];
    int c = 0;
    for (int b = 0; b < n; ++b)
        if ((tile >> b) & 1ULL) {
            slot[b] = c;
            d.tile_pos[c++] = (uint8_t)b;
        }
    d.n = n;
    d.q = q;
    d.w = 0;
    while (d.w < q && d.tile_pos[d.w] == d.w) ++d.w;
    uint64_t fixed = ~0ULL;
    for (size_t o = i; o < j; ++o) fixed &= ops[o].ctrl_mask & ~tile;
    if (j == i) fixed = 0;
    d.fixed_mask = fixed;
    const uint64_t ins = tile | fixed;
    d.nins = 0;
    for (int b = 0; b < 64; ++b)
        if ((ins >> b) & 1ULL) d.ins_pos[d.nins++] = (uint8_t)b;
    d.nops = (int)(j - i);
    uint32_t moff = 0;
    size_t tcb = 0;
    for (size_t o = i; o < j; ++o) {
        const GateOp& op = ops[o];
        OpDesc& od = d.ops[o - i];
        od.k = op.k;
        od.diag = op.diag ? 1 : 0;
        // tensor-core gates need at least 16 index groups per tile
        od.tc = (allow_tc && tc_candidate(arith, op) && q >= op.k + 4) ? 1 : 0;
        // 3xTF32 fragments are read as float4: 16-byte aligned in the pool
        if (od.tc && arith == kArithTF32) moff = (moff + 1) & ~1u;
        if (od.tc) tcb = std::max(tcb, tc_scratch_bytes(arith, q, op.k));
        od.ctrl_outer = op.ctrl_mask & ~tile;
        uint32_t cl = 0;
        for (int b = 0; b < n; ++b)
            if (((op.ctrl_mask & tile) >> b) & 1ULL) cl |= 1u << slot[b];
        od.ctrl_local = cl;
        for (int t = 0; t < op.k; ++t)
            od.tslot[t] = ((tile >> op.pos[t]) & 1ULL) ? (uint8_t)slot[op.pos[t]]
                                                         : (uint8_t)(kOuterSlot | op.pos[t]);
        od.mat_off = moff;
        moff += (uint32_t)pool_elems(arith, op, od.tc != 0);
    }
    d.mat_elems = moff;
    d.tc_bytes = (uint32_t)((tcb + 15) & ~(size_t)15);
    // stream the next tile in while computing this one: into the second
    // tile buffer when every op works in place on raw state elements,
    // else into a staging buffer unless that costs a resident CTA per SM
    // (228 KB per SM, 1 KB reserved per CTA, at most 227 KB per CTA)
    bool inplace = true, has_tc_op = false;
    for (int o = 0; o < d.nops; ++o) {
        const OpDesc& od = d.ops[o];
        has_tc_op = has_tc_op || od.tc;
        inplace = inplace && (od.k == 0 || od.diag || (od.tc && arith != kArithTF32));
    }
    const bool raw = arith == kArithF64 || arith == kArithF32 || arith == kArithTF32 || arith == kArithTC64 ||
                     (arith == kArithTC && has_tc_op);
    if (raw && inplace && d.nops > 0) {
        d.prefetch = 2;
    } else {
        const int regc = pass_reg_ctas(arith, d);
        auto ctas = [&](size_t sm) { return std::min<size_t>((size_t)regc, 233472 / (sm + 1024)); };
        d.prefetch = 0;
        const size_t s0 = pass_smem_bytes(arith, d);
        d.prefetch = 1;
        const size_t s1 = pass_smem_bytes(arith, d);
        d.prefetch = (s1 <= 232448 && ctas(s1) >= ctas(s0)) ? 1 : 0;
    }
    pl.bytes = 2ULL * (1ULL << (n - popc64(fixed))) * store;
    return pl;
}

// Resident CTAs per SM of a pass: its kernel's register budget and its
// shared memory (228 KB per SM, 1 KB reserved per CTA).
static int pass_ctas(int arith, const PassDesc& d) {
    return std::min(pass_reg_ctas(arith, d), (int)(233472 / (pass_smem_bytes(arith, d) + 1024)));
}

std::vector<PassPlan> plan_passes(int n, int arith, const GateOp* ops, size_t nops, int max_tile_bits, int max_ops,
                                  std::vector<size_t>* op_first, size_t max_passes, int min_ctas) {
    const size_t melem = Workspace::mat_elem_bytes(arith);
    // staged matrices per pass; 3xTF32 passes take two 5-qubit gates
    const size_t mat_budget = (arith == kArithTF32 ? 72 : 64) * 1024;
    max_tile_bits = std::max(5, std::min(max_tile_bits, kMaxTileBits));
    max_ops = std::max(1, std::min(max_ops, kMaxOpsPerPass));
    std::vector<PassPlan> plans;
    size_t i = 0, pool_off = 0;
    while (i < nops && plans.size() < max_passes) {
        uint64_t tset = 0;
        size_t mbytes = 0, j = i;
        if (op_first) op_first->push_back(i);
        while (j < nops && (int)(j - i) < max_ops) {
            const GateOp& op = ops[j];
            // a diagonal gate needs none of its targets in the tile (the tile
            // base supplies the bits of those outside it)
            uint64_t tm = 0;
            if (!op.diag)
                for (int t = 0; t < op.k; ++t) tm |= 1ULL << op.pos[t];
            const uint64_t ns = tset | tm;
            const size_t ob = pool_elems(arith, op, tc_candidate(arith, op)) * melem;
            if (j > i && (popc64(ns) + 4 > max_tile_bits || mbytes + ob > mat_budget)) break;
            tset = ns;
            mbytes += ob;
            ++j;
        }
        PassPlan pl = build_pass(n, arith, ops, i, j, max_tile_bits);
        // leave out trailing ops whose matrices would cost a resident CTA per
        // SM: the pass then runs at the occupancy of its first op
        if (min_ctas != 0 && j - i > 1) {
            int best = pass_ctas(arith, build_pass(n, arith, ops, i, i + 1, max_tile_bits).desc);
            if (min_ctas > 0) best = std::min(best, min_ctas);
            while (j - i > 1 && pass_ctas(arith, pl.desc) < best) {
                --j;
                pl = build_pass(n, arith, ops, i, j, max_tile_bits);
            }
        }
        pl.pool_off = pool_off;
        pool_off += ((size_t)pl.desc.mat_elems * melem + 255) & ~(size_t)255;
        plans.push_back(pl);
        i = j;
    }
    return plans;
}

static uint16_t half_of_int(int d) {
    if (d == 0) return 0;
    const uint16_t sgn = d < 0 ? 0x8000 : 0;
    const int a = d < 0 ? -d : d;
    const int e = 31 - __builtin_clz((unsigned)a);
    return (uint16_t)(sgn | ((e + 15) << 10) | ((a << (10 - e)) & 0x3FF));
}

static int biased_exponent(double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    return (int)((u >> 52) & 0x7FF);
}

// The nd balanced base-2^10 digits of v relative to the biased exponent
// ebmax of its column (same rule as the device-side digits of the state):
// a = round(|v| 2^(10 nd - 1 - E)) (to nearest, ties to even) cut into 10-bit
// fields, balanced into [-512, 511] with carries upward, then given v's sign.
static void digits_host(double v, int ebmax, int nd, int* d) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    const int eb = (int)((u >> 52) & 0x7FF);
    uint64_t a = 0;
    const int sh = 4 + 10 * (kTcDigits - nd) + ebmax - eb;
    if (eb != 0 && sh < 62) {
        const uint64_t M = (u & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
        a = (M + (1ULL << (sh - 1)) - 1ULL + ((M >> sh) & 1ULL)) >> sh;
    }
    int r[kTcDigits];
    for (int i = 0; i < nd; ++i) r[nd - 1 - i] = (int)((a >> (10 * i)) & 1023u);
    r[0] = (int)(a >> (10 * (nd - 1)));
    for (int i = nd - 1; i >= 1; --i) {
        const int c = (r[i] + 512) >> 10;
        r[i] -= c << 10;
        r[i - 1] += c;
    }
    const bool neg = (u >> 63) != 0;
    for (int i = 0; i < nd; ++i) d[i] = neg ? -r[i] : r[i];
}

// Real form of a complex gate for the tensor-core path (B with Y = X B, X the
// interleaved real and imaginary parts of a group's inputs).
// complex128 (nd = 5): int32 E_col per column. complex64 (nd = 3): the column
// scale 2^(E_col - 19) as a float, 0 (and no digits) for a column whose
// largest entry is below 2^-107.
static void convert_tc(const GateOp& op, int nd, unsigned char* dst) {
    const int D = 1 << op.k, KK = 2 * D, RH = KK + 8;
    // interleaved real form: row 2c + p_in is part p_in of input c, column
    // 2r + p_out part p_out of output r
    auto bval = [&](int kk, int j) -> double {
        const cplx m = op.m[(size_t)(j >> 1) * D + (kk >> 1)];
        const int pin = kk & 1, pout = j & 1;
        if (pin == 0) return pout == 0 ? m.real() : m.imag();
        return pout == 0 ? -m.imag() : m.real();
    };
    int32_t* ecol = reinterpret_cast<int32_t*>(dst);
    uint16_t* planes = reinterpret_cast<uint16_t*>(dst + 4 * KK);
    std::memset(planes, 0, (size_t)nd * KK * RH * 2);
    for (int j = 0; j < KK; ++j) {
        int ebmax = 0;
        for (int kk = 0; kk < KK; ++kk) ebmax = std::max(ebmax, biased_exponent(bval(kk, j)));
        ecol[j] = ebmax - 1022;
        if (nd != kTcDigits) {
            float sc = 0.f;
            if (ebmax - 1022 - 19 >= -126) sc = std::ldexp(1.0f, ebmax - 1022 - 19);
            std::memcpy(&ecol[j], &sc, 4);
            if (sc == 0.f) continue;
        }
        for (int kk = 0; kk < KK; ++kk) {
            int d[kTcDigits];
            digits_host(bval(kk, j), ebmax, nd, d);
            for (int s2 = 0; s2 < nd; ++s2) planes[(size_t)s2 * KK * RH + (size_t)j * RH + kk] = half_of_int(d[s2]);
        }
    }
}

// FP32 value rounded to TF32 (10 fraction bits), nearest with ties away from
// zero, as a float; infinities and NaNs pass through.
static float tf32_round(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) != 0x7F800000u) u = (u + 0x1000u) & 0xFFFFE000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

// 3xTF32 form of a complex gate: the interleaved real B of convert_tc, each
// entry split into hi = tf32(b), lo = tf32(b - hi), stored in m16n8k8
// B-fragment order (k-step ks, n-tile nt, lane l: {hi b0, hi b1, lo b0,
// lo b1}, b0 = B[8ks + l%4][8nt + l/4], b1 = B[8ks + l%4 + 4][8nt + l/4]).
static void convert_tf32(const GateOp& op, unsigned char* dst) {
    const int D = 1 << op.k, KK = 2 * D, NT = KK / 8;
    auto bval = [&](int kk, int j) -> double {
        const cplx m = op.m[(size_t)(j >> 1) * D + (kk >> 1)];
        const int pin = kk & 1, pout = j & 1;
        if (pin == 0) return pout == 0 ? m.real() : m.imag();
        return pout == 0 ? -m.imag() : m.real();
    };
    float* out = reinterpret_cast<float*>(dst);
    for (int ks = 0; ks < NT; ++ks)
        for (int nt = 0; nt < NT; ++nt)
            for (int l = 0; l < 32; ++l) {
                const int n = nt * 8 + l / 4, k0 = ks * 8 + l % 4;
                const double b0 = bval(k0, n), b1 = bval(k0 + 4, n);
                const float h0 = tf32_round((float)b0), h1 = tf32_round((float)b1);
                float* f = out + ((size_t)(ks * NT + nt) * 32 + l) * 4;
                f[0] = h0;
                f[1] = h1;
                f[2] = tf32_round((float)(b0 - (double)h0));
                f[3] = tf32_round((float)(b1 - (double)h1));
            }
}

static void convert_tc_any(int arith, const GateOp& op, unsigned char* dst) {
    if (arith == kArithTF32) convert_tf32(op, dst);
    else convert_tc(op, tc_digits_b(arith), dst);
}

// Dense gates are stored transposed (element c * dim + r holds M[r][c]): the
// pass kernel's threads own output rows and read one column entry per input.
static void convert_matrix(int arith, const GateOp& op, unsigned char* dst) {
    std::vector<cplx> t;
    const std::vector<cplx>* src = &op.m;
    if (op.k > 0 && !op.diag) {
        const size_t dim = (size_t)1 << op.k;
        t.resize(op.m.size());
        for (size_t r = 0; r < dim; ++r)
            for (size_t c = 0; c < dim; ++c) t[c * dim + r] = op.m[r * dim + c];
        src = &t;
    }
    const std::vector<cplx>& m = *src;
    if (arith == kArithF64) {
        double* p = reinterpret_cast<double*>(dst);
        for (size_t e = 0; e < m.size(); ++e) {
            p[2 * e] = m[e].real();
            p[2 * e + 1] = m[e].imag();
        }
    } else if (arith == kArithDF || arith == kArithTC) {
        float* p = reinterpret_cast<float*>(dst);
        for (size_t e = 0; e < m.size(); ++e) {
            const double re = m[e].real(), im = m[e].imag();
            const float hr = (float)re, hi = (float)im;
            p[4 * e] = hr;
            p[4 * e + 1] = hi;
            p[4 * e + 2] = (float)(re - (double)hr);
            p[4 * e + 3] = (float)(im - (double)hi);
        }
    } else {
        float* p = reinterpret_cast<float*>(dst);
        for (size_t e = 0; e < m.size(); ++e) {
            p[2 * e] = (float)m[e].real();
            p[2 * e + 1] = (float)m[e].imag();
        }
    }
}

size_t pass_pool_bytes(int arith, const PassDesc& d) {
    return ((size_t)d.mat_elems * Workspace::mat_elem_bytes(arith) + 255) & ~(size_t)255;
}

std::shared_ptr<const std::vector<unsigned char>> make_tc_pool(int arith, const GateOp& op) {
    auto v = std::make_shared<std::vector<unsigned char>>(tc_pool_bytes(arith, op.k));
    convert_tc_any(arith, op, v->data());
    return v;
}

void write_pass_pool(int arith, const PassDesc& d, const GateOp* ops, unsigned char* dst) {
    const size_t melem = Workspace::mat_elem_bytes(arith);
    for (int o = 0; o < d.nops; ++o) {
        unsigned char* p = dst + (size_t)d.ops[o].mat_off * melem;
        const bool tc = d.ops[o].tc != 0;
        if (tc && ops[o].tc_pool) std::memcpy(p, ops[o].tc_pool->data(), ops[o].tc_pool->size());
        else if (tc) convert_tc_any(arith, ops[o], p);
        else convert_matrix(arith, ops[o], p);
    }
}

// ------------------------------------------------------- tensor-memory passes

bool umma_enabled() {
    static const bool on = [] {
        const char* v = std::getenv("HQS_UMMA");
        return !(v && v[0] == '0');
    }();
    return on;
}

bool umma_candidate(int arith, const GateOp& op) {
    return (arith == kArithTC || arith == kArithTC64) && !op.diag && op.k >= 3 && op.k <= 5;
}

static bool elementwise_op(const GateOp& op) { return op.k == 0 || op.diag; }

// matrix entries of an element-wise op in a tensor-memory pass: double-float
// complex (16 B) for complex128 states, FP32 complex (8 B) for complex64
static size_t ew_pool_bytes(const GateOp& op, int arith) { return op.m.size() * (arith == kArithTC64 ? 8 : 16); }

// The six balanced base-2^9 digits of a gate real v relative to its column's
// largest biased exponent ebmax, with the column scaled to |v'| < 2^7:
// a = rint(|v| 2^(1074 - ebmax)) (to nearest, ties to even; a < 2^52) cut
// into 9-bit fields, balanced into [-256, 255] with carries upward (the top
// digit ends at most 128), then given v's sign.
// With nd = 4 (complex64) the same column scale keeps the top four digits:
// a = rint(|v| 2^(1056 - ebmax)) < 2^34.
static void gate_digits9(double v, int ebmax, int nd, int (&d)[6]) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    const int eb = (int)((u >> 52) & 0x7FF);
    uint64_t a = 0;
    const int sh = ebmax - eb + 1 + 9 * (6 - nd);
    if (eb != 0 && sh < 62) {
        const uint64_t M = (u & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
        a = (M + (1ULL << (sh - 1)) - 1ULL + ((M >> sh) & 1ULL)) >> sh;
    }
    int r[6];
    for (int i = 1; i < nd; ++i) r[i] = (int)((a >> (9 * (nd - 1 - i))) & 511u);
    r[0] = (int)(a >> (9 * (nd - 1)));
    for (int i = nd - 1; i >= 1; --i) {
        const int c = (r[i] + 256) >> 9;
        r[i] -= c << 9;
        r[i - 1] += c;
    }
    const bool neg = (u >> 63) != 0;
    for (int i = 0; i < 6; ++i) d[i] = i >= nd ? 0 : neg ? -r[i] : r[i];
}

// Gate block of a tensor-memory pass: the gate widened to the five target
// positions pos5 (ascending; e bit j <-> pos5[j], identity on the positions
// that are not the gate's targets), in real form B[k][n] (k = 2c + part of
// input c, n = 2r + part of output r), as six digit planes (plane j: rows
// n = 0..63 of 64 fp16 over k, K-major with the 128-byte swizzle of the MMA
// operand), then the 64 column exponents as int32. complex64: four digit
// planes. halves (complex128 passes that hold only the dense gate): the rows
// ordered by output half, then plane (row 192 h + 32 j + n mod 32 for n in
// half h = n / 32), so that one MMA covers all digit planes of a half.
static void build_umma_gate(const GateOp& g, const int (&pos5)[5], bool c64, bool halves, unsigned char* dst) {
    int realbit[5];
    for (int j = 0; j < 5; ++j) {
        realbit[j] = -1;
        for (int t = 0; t < g.k; ++t)
            if (g.pos[t] == pos5[j]) realbit[j] = t;
    }
    const int D = 1 << g.k;
    auto u5 = [&](int r5, int c5) -> cplx {
        int r = 0, c = 0;
        for (int j = 0; j < 5; ++j) {
            const int rb = (r5 >> j) & 1, cb = (c5 >> j) & 1;
            if (realbit[j] < 0) {
                if (rb != cb) return cplx(0.0, 0.0);
            } else {
                r |= rb << realbit[j];
                c |= cb << realbit[j];
            }
        }
        return g.m[(size_t)r * D + c];
    };
    auto bval = [&](int kk, int nn) -> double {
        const cplx m = u5(nn >> 1, kk >> 1);
        const int pin = kk & 1, pout = nn & 1;
        if (pin == 0) return pout == 0 ? m.real() : m.imag();
        return pout == 0 ? -m.imag() : m.real();
    };
    const uint32_t plane_bytes = c64 ? kUmmaGatePlaneBytes64 : kUmmaGatePlaneBytes;
    const int nd = c64 ? 4 : 6;
    uint16_t* planes = reinterpret_cast<uint16_t*>(dst);
    std::memset(planes, 0, plane_bytes);
    int32_t* ecol = reinterpret_cast<int32_t*>(dst + plane_bytes);
    for (int nn = 0; nn < 64; ++nn) {
        int ebmax = 0;
        for (int kk = 0; kk < 64; ++kk) ebmax = std::max(ebmax, biased_exponent(bval(kk, nn)));
        ecol[nn] = ebmax;
        for (int kk = 0; kk < 64; ++kk) {
            int dg[6];
            gate_digits9(bval(kk, nn), ebmax, nd, dg);
            for (int j = 0; j < nd; ++j) {
                const int row = halves ? 192 * (nn >> 5) + 32 * j + (nn & 31) : 64 * j + nn;
                const size_t byte = (size_t)row * 128 + ((size_t)(((2 * kk) >> 4) ^ (row & 7)) << 4) + ((2 * kk) & 15);
                planes[byte / 2] = half_of_int(dg[j]);
            }
        }
    }
}

// Tensor-memory pass over ops [i0, i1) with the dense gate at tc. Tile: the
// gate's targets, then the lowest other positions up to 12; when the gate has
// fewer than five targets, the highest of those positions that are not its
// controls become extra targets with identity factors. Returns kUmmaOk, or
// why the pass cannot be formed: the run before / after the dense gate
// depends on too many tile slots, or another reason (state too small,
// element-wise matrices too large).
enum { kUmmaOk = 0, kUmmaPreWide = 1, kUmmaPostWide = 2, kUmmaNo = 3 };
static int build_umma(int n, int arith, const GateOp* ops, size_t i0, size_t tc, size_t i1, UmmaDesc& u,
                      uint64_t& bytes) {
    const GateOp& g = ops[tc];
    uint64_t tmask = 0;
    for (int t = 0; t < g.k; ++t) tmask |= 1ULL << g.pos[t];
    std::vector<int> picks;
    for (int b = 0; b < n && (int)picks.size() < kUmmaTileBits - g.k; ++b)
        if (!((tmask >> b) & 1ULL)) picks.push_back(b);
    if ((int)picks.size() < kUmmaTileBits - g.k) return kUmmaNo;
    uint64_t t5 = tmask;
    int extra_t = 5 - g.k;
    for (int i = (int)picks.size() - 1; i >= 0 && extra_t > 0; --i)
        if (!((g.ctrl_mask >> picks[i]) & 1ULL)) {
            t5 |= 1ULL << picks[i];
            --extra_t;
        }
    if (extra_t > 0) return kUmmaNo;
    uint64_t tile = tmask;
    for (int p : picks) tile |= 1ULL << p;
    size_t ewb = 0;
    for (size_t o = i0; o < i1; ++o)
        if (o != tc) ewb += ew_pool_bytes(ops[o], arith);
    if (ewb > kUmmaEwMaxBytes || i1 - i0 > (size_t)kMaxOpsPerPass) return kUmmaNo;

    std::memset(&u, 0, sizeof(u));
    u.c64 = arith == kArithTC64 ? 1 : 0;
    PassDesc& d = u.d;
    int slot[64];
    int c = 0;
    for (int b = 0; b < n; ++b)
        if ((tile >> b) & 1ULL) {
            slot[b] = c;
            d.tile_pos[c++] = (uint8_t)b;
        }
    d.n = n;
    d.q = kUmmaTileBits;
    d.w = 0;
    while (d.w < d.q && d.tile_pos[d.w] == d.w) ++d.w;
    uint64_t fixed = ~0ULL;
    for (size_t o = i0; o < i1; ++o) fixed &= ops[o].ctrl_mask & ~tile;
    d.fixed_mask = fixed;
    const uint64_t ins = tile | fixed;
    d.nins = 0;
    for (int b = 0; b < 64; ++b)
        if ((ins >> b) & 1ULL) d.ins_pos[d.nins++] = (uint8_t)b;
    d.nops = (int)(i1 - i0);
    int pos5[5], np = 0;
    for (int b = 0; b < n; ++b)
        if ((t5 >> b) & 1ULL) pos5[np++] = b;
    for (int j = 0; j < 5; ++j) u.tslot[j] = (uint8_t)slot[pos5[j]];
    uint32_t moff = 0;
    for (size_t o = i0; o < i1; ++o) {
        const GateOp& op = ops[o];
        OpDesc& od = d.ops[o - i0];
        od.ctrl_outer = op.ctrl_mask & ~tile;
        uint32_t cl = 0;
        for (int b = 0; b < n; ++b)
            if (((op.ctrl_mask & tile) >> b) & 1ULL) cl |= 1u << slot[b];
        od.ctrl_local = cl;
        if (o == tc) {
            od.k = 5;
            od.tc = 1;
            for (int j = 0; j < 5; ++j) od.tslot[j] = u.tslot[j];
            continue;
        }
        od.k = op.k;
        od.diag = op.diag ? 1 : 0;
        uint32_t rm = cl;
        for (int t = 0; t < op.k; ++t) {
            const bool in = ((tile >> op.pos[t]) & 1ULL) != 0;
            od.tslot[t] = in ? (uint8_t)slot[op.pos[t]] : (uint8_t)(kOuterSlot | op.pos[t]);
            if (in) rm |= 1u << slot[op.pos[t]];
        }
        u.run_mask[o < tc ? 0 : 1] |= rm;
        od.mat_off = moff;
        moff += (uint32_t)op.m.size();
    }
    if (__builtin_popcount(u.run_mask[0]) > kUmmaRunBits) return kUmmaPreWide;
    if (__builtin_popcount(u.run_mask[1]) > kUmmaRunBits) return kUmmaPostWide;
    u.tc_op = (int)(tc - i0);
    u.ew_bytes = (uint32_t)ewb;
    u.gate_off = (uint32_t)((ewb + 1023) & ~(size_t)1023);

    // TMA plan: the state as doubles; every dimension spans a run of tile
    // positions (inside the box, at most 256 elements: 7 positions for the
    // first dimension with its re/im pair, 8 for the others) and the gap of
    // non-tile positions above it (its coordinate comes from the tile base).
    // With more than five runs the fifth dimension spans everything from its
    // run up, and the tile positions above that run are fetched as separate
    // copies.
    struct Dim {
        int pos, box, bits;
    };
    std::vector<Dim> dims;
    for (int b = 0; b < n;) {
        int e = b;
        while (e < n && ((tile >> e) & 1ULL)) ++e;
        while (e - b > (b == 0 ? 7 : 8)) {  // a run longer than a box dimension takes two
            const int cap = b == 0 ? 7 : 8;
            dims.push_back({b, cap, cap});
            b += cap;
        }
        int g = e;
        while (g < n && !((tile >> g) & 1ULL)) ++g;
        dims.push_back({b, e - b, g - b});
        b = g;
    }
    int rank = 0, tbits = 0;
    for (size_t r = 0; r < dims.size() && rank < 5; ++r) {
        const bool rest = rank == 4 && r + 1 < dims.size();
        u.dim_kind[rank] = rest ? 2 : 1;
        u.dim_pos[rank] = (int8_t)dims[r].pos;
        u.dim_box[rank] = (int8_t)dims[r].box;
        u.dim_bits[rank] = (int8_t)(rest ? n - dims[r].pos : dims[r].bits);
        tbits += dims[r].box;
        ++rank;
        if (rest) {
            int ne = 0;
            for (int b = dims[r].pos + dims[r].box; b < n; ++b)
                if ((tile >> b) & 1ULL) u.extra_pos[ne++] = (int8_t)b;
            u.nextra = (uint8_t)ne;
        }
    }
    u.rank = (uint8_t)rank;
    if (tbits + u.nextra != kUmmaTileBits) return kUmmaNo;
    const uint32_t amp = u.c64 ? 8u : 16u;
    u.box_bytes = amp << tbits;
    bytes = 2ULL * (1ULL << (n - popc64(fixed))) * amp;
    return kUmmaOk;
}

void write_umma_pool(const UmmaDesc& u, const GateOp* ops, unsigned char* dst) {
    const PassDesc& d = u.d;
    for (int o = 0; o < d.nops; ++o) {
        if (o == u.tc_op) continue;
        // element-wise matrices, untransposed: double-float complex for a
        // complex128 state, FP32 complex for complex64
        const GateOp& op = ops[o];
        float* p = reinterpret_cast<float*>(dst + (size_t)d.ops[o].mat_off * (u.c64 ? 8 : 16));
        for (size_t e = 0; e < op.m.size(); ++e) {
            const double re = op.m[e].real(), im = op.m[e].imag();
            const float hr = (float)re, hi = (float)im;
            if (u.c64) {
                p[2 * e] = hr;
                p[2 * e + 1] = hi;
                continue;
            }
            p[4 * e] = hr;
            p[4 * e + 1] = hi;
            p[4 * e + 2] = (float)(re - (double)hr);
            p[4 * e + 3] = (float)(im - (double)hi);
        }
    }
    int pos5[5];
    for (int j = 0; j < 5; ++j) pos5[j] = d.tile_pos[u.tslot[j]];
    build_umma_gate(ops[u.tc_op], pos5, u.c64 != 0, !u.c64 && d.nops == 1, dst + u.gate_off);
}

std::vector<LaunchPlan> plan_launches(int n, int arith, const std::vector<GateOp>& ops, int max_tile_bits, int max_ops,
                                      bool allow_umma) {
    std::vector<LaunchPlan> out;
    const size_t nops = ops.size();
    auto classic = [&](size_t a, size_t b) {
        if (a >= b) return;
        std::vector<size_t> first;
        std::vector<PassPlan> pl = plan_passes(n, arith, ops.data() + a, b - a, max_tile_bits, max_ops, &first);
        for (size_t i = 0; i < pl.size(); ++i) {
            LaunchPlan L;
            L.pass = pl[i];
            L.first = a + first[i];
            L.pool_bytes = pass_pool_bytes(arith, pl[i].desc);
            L.bytes = pl[i].bytes;
            out.push_back(L);
        }
    };
    const bool umma = allow_umma && (arith == kArithTC || arith == kArithTC64) && n >= kUmmaTileBits;
    size_t i = 0;
    while (i < nops) {
        size_t j = i;
        if (umma)
            while (j < nops && !umma_candidate(arith, ops[j])) ++j;
        else
            j = nops;
        if (j == nops) {
            classic(i, nops);
            break;
        }
        // element-wise gates just before the dense gate join its pass
        size_t p = j;
        size_t ewb = 0;
        while (p > i && elementwise_op(ops[p - 1]) && ewb + ew_pool_bytes(ops[p - 1], arith) <= kUmmaEwMaxBytes &&
               j - p + 1 < (size_t)kMaxOpsPerPass) {
            ewb += ew_pool_bytes(ops[p - 1], arith);
            --p;
        }
        size_t e = j + 1;
        while (e < nops && elementwise_op(ops[e]) && ewb + ew_pool_bytes(ops[e], arith) <= kUmmaEwMaxBytes &&
               e - p < (size_t)kMaxOpsPerPass) {
            ewb += ew_pool_bytes(ops[e], arith);
            ++e;
        }
        LaunchPlan L;
        uint64_t by = 0;
        int st;
        // leave out gates of the runs until each run's factor depends on at
        // most kUmmaRunBits tile slots
        while ((st = build_umma(n, arith, ops.data(), p, j, e, L.udesc, by)) == kUmmaPreWide ||
               st == kUmmaPostWide) {
            if (st == kUmmaPreWide) ++p;
            else --e;
        }
        if (st != kUmmaOk) {
            classic(i, j + 1);
            i = j + 1;
            continue;
        }
        classic(i, p);
        L.umma = true;
        L.first = p;
        L.pool_bytes = L.udesc.gate_off + (L.udesc.c64 ? kUmmaGateBytes64 : kUmmaGateBytes);
        L.bytes = by;
        out.push_back(L);
        i = e;
    }
    return out;
}

uint64_t Workspace::apply_ops(void* state, int n, int arith, const std::vector<GateOp>& ops, int max_tile_bits,
                              int max_ops, uint64_t* passes_out) {
    if (ops.empty()) return 0;
    if ((arith == kArithTC || arith == kArithTC64) && umma_enabled() && n >= kUmmaTileBits) {
        std::vector<LaunchPlan> L = plan_launches(n, arith, ops, max_tile_bits, max_ops, true);
        size_t total = 0;
        for (auto& l : L) {
            total = (total + 1023) & ~(size_t)1023;
            l.pool_off = total;
            total += (l.pool_bytes + 255) & ~(size_t)255;
        }
        total = std::max<size_t>(total, 256);
        ensure_pinned(total);
        ensure_pool(total);
        unsigned char* host = static_cast<unsigned char*>(pinned_);
        for (const auto& l : L) {
            if (l.umma) write_umma_pool(l.udesc, ops.data() + l.first, host + l.pool_off);
            else write_pass_pool(arith, l.pass.desc, ops.data() + l.first, host + l.pool_off);
        }
        cuda_check(cudaMemcpyAsync(pool_, pinned_, total, cudaMemcpyHostToDevice, stream_), "cudaMemcpyAsync(matrices)");
        cuda_check(cudaEventRecord(staging_free_, stream_), "cudaEventRecord");
        staging_pending_ = true;
        uint64_t bytes = 0;
        for (size_t li = 0; li < L.size(); ++li) {
            const auto& l = L[li];
            const size_t lend = li + 1 < L.size() ? L[li + 1].first : ops.size();
            uint64_t tmask = 0;
            if (l.umma)
                for (int j = 0; j < 5; ++j) tmask |= 1ULL << l.udesc.d.tile_pos[l.udesc.tslot[j]];
            TimedLaunch tl{nullptr, nullptr, l.bytes, l.umma ? 1 : 0, (int)(lend - l.first),
                           l.umma ? 1 << l.udesc.nextra : 0, tmask};
            if (timing_) {
                tl.a = take_event();
                tl.b = take_event();
                cuda_check(cudaEventRecord(tl.a, stream_), "cudaEventRecord");
            }
            unsigned char* mats = static_cast<unsigned char*>(pool_) + l.pool_off;
            if (l.umma) cuda_check(launch_umma_pass(state, mats, l.udesc, stream_), "launch_umma_pass");
            else cuda_check(launch_pass(arith, state, mats, l.pass.desc, stream_), "launch_pass");
            if (timing_) {
                cuda_check(cudaEventRecord(tl.b, stream_), "cudaEventRecord");
                timed_.push_back(tl);
            }
            bytes += l.bytes;
        }
        if (passes_out) *passes_out = L.size();
        return bytes;
    }
    std::vector<size_t> first;
    std::vector<PassPlan> plans = plan_passes(n, arith, ops, max_tile_bits, max_ops, &first);
    size_t total = 0;
    for (const auto& p : plans) {
        const size_t end = p.pool_off + ((size_t)p.desc.mat_elems * mat_elem_bytes(arith) + 255) / 256 * 256;
        total = std::max(total, end);
    }
    total = std::max<size_t>(total, 256);
    ensure_pinned(total);
    ensure_pool(total);
    unsigned char* host = static_cast<unsigned char*>(pinned_);
    for (size_t pi = 0; pi < plans.size(); ++pi) {
        const PassPlan& p = plans[pi];
        write_pass_pool(arith, p.desc, ops.data() + first[pi], host + p.pool_off);
    }
    cuda_check(cudaMemcpyAsync(pool_, pinned_, total, cudaMemcpyHostToDevice, stream_), "cudaMemcpyAsync(matrices)");
    cuda_check(cudaEventRecord(staging_free_, stream_), "cudaEventRecord");
    staging_pending_ = true;
    uint64_t bytes = 0;
    for (size_t pi = 0; pi < plans.size(); ++pi) {
        const PassPlan& p = plans[pi];
        const size_t pend = pi + 1 < plans.size() ? first[pi + 1] : ops.size();
        TimedLaunch tl{nullptr, nullptr, p.bytes, 0, (int)(pend - first[pi]), 0, 0};
        if (timing_) {
            tl.a = take_event();
            tl.b = take_event();
            cuda_check(cudaEventRecord(tl.a, stream_), "cudaEventRecord");
        }
        cuda_check(launch_pass(arith, state, static_cast<unsigned char*>(pool_) + p.pool_off, p.desc, stream_),
                   "launch_pass");
        if (timing_) {
            cuda_check(cudaEventRecord(tl.b, stream_), "cudaEventRecord");
            timed_.push_back(tl);
        }
        bytes += p.bytes;
    }
    if (passes_out) *passes_out = plans.size();
    return bytes;
}

cudaEvent_t Workspace::take_event() {
    if (!event_pool_.empty()) {
        cudaEvent_t e = event_pool_.back();
        event_pool_.pop_back();
        return e;
    }
    cudaEvent_t e;
    cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    return e;
}

Workspace::PassTiming Workspace::collect_timing() {
    PassTiming t;
    for (auto& tl : timed_) {
        cuda_check(cudaEventSynchronize(tl.b), "cudaEventSynchronize");
        float ms = 0.f;
        cuda_check(cudaEventElapsedTime(&ms, tl.a, tl.b), "cudaEventElapsedTime");
        t.ms += ms;
        t.bytes += tl.bytes;
        ++t.launches;
        t.log.push_back({tl.kind, tl.nops, tl.copies, tl.target_mask, tl.bytes, (double)ms});
        event_pool_.push_back(tl.a);
        event_pool_.push_back(tl.b);
    }
    timed_.clear();
    return t;
}

}  // namespace hqs
