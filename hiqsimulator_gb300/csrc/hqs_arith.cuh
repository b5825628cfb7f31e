// Arithmetic policies for the state-vector kernels.
//
//   F64  complex128 storage, native FP64 arithmetic (the reference's own
//        arithmetic; limited by GB300's FP64 rate).
//   DF   complex128 storage, double-float arithmetic on the FP32 pipe. Each
//        double is split into hi + lo floats with integer bit operations
//        (no FP64 instruction and no F2F conversion, which also run on the
//        FP64 pipe), products are formed exactly with FMA, sums are kept in
//        (hi, lo) pairs, and results are re-assembled into a double with
//        integer operations. About 47-48 significant bits per operation.
//   F32  complex64 storage, FP32 arithmetic.
//   TC   complex128 storage; dense 3..5-qubit gates on the fp16 tensor cores
//        as exact products of five base-2^10 digits (kernels.cu, apply_tc),
//        every other op as DF on the raw doubles (ArithDFRaw).
//   TC64 complex64 storage; the same tensor-core scheme with two digits,
//        every other op as F32.
//   TF32 complex64 storage; dense 3..5-qubit gates as 3xTF32 tensor-core
//        products (apply_tf32), every other op as F32.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hqs {

// ---------------------------------------------------------------- double-float
struct DF {
    float h, l;
};

// Split a double into h + l (|l| < ulp(h)) with integer operations.
// |x| < 2^-126 is flushed to zero (absolute error below 1.2e-38); the low
// part is dropped when |x| < 2^-75.
__device__ __forceinline__ DF df_split(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned hi32 = (unsigned)(u >> 32), lo32 = (unsigned)u;
    const unsigned s = hi32 & 0x80000000u;
    const int E = (int)((hi32 >> 20) & 0x7FFu);
    const int ef = E - 896;
    DF r;
    if (ef <= 0) { r.h = 0.f; r.l = 0.f; return r; }
    if (ef >= 255) { r.h = __uint_as_float(s | 0x7f800000u); r.l = 0.f; return r; }
    const unsigned mhi = ((hi32 & 0xFFFFFu) << 3) | (lo32 >> 29);
    r.h = __uint_as_float(s | ((unsigned)ef << 23) | mhi);
    const unsigned mlo = lo32 & 0x1FFFFFFFu;
    const int es = E - 948;  // biased exponent of 2^(E - 1075)
    if (es >= 1 && mlo != 0u) {
        const float lf = __uint2float_rn(mlo) * __uint_as_float((unsigned)es << 23);
        r.l = __uint_as_float(__float_as_uint(lf) | s);
    } else {
        r.l = 0.f;
    }
    return r;
}

// Re-assemble h + l into the nearest double with integer operations.
// Requires |l| < 2 ulp(h) in float terms (true for df_split outputs and for
// pairs normalised by df_norm); h == 0 implies l == 0.
__device__ __forceinline__ double df_combine(float h, float l) {
    const unsigned hb = __float_as_uint(h);
    const unsigned s = hb & 0x80000000u;
    const int ef = (int)((hb >> 23) & 0xFFu);
    if (ef == 0) return __longlong_as_double((long long)((unsigned long long)s << 32));
    if (ef == 255) return (double)h;  // inf / nan: rare, FP64 conversion is fine
    const unsigned mf = hb & 0x7FFFFFu;
    const long long mag = ((long long)(ef + 896) << 52) | ((long long)mf << 29);
    const unsigned lb = __float_as_uint(l);
    const int el = (int)((lb >> 23) & 0xFFu);
    long long delta = 0;
    if (el != 0) {
        const bool neg = ((lb ^ hb) & 0x80000000u) != 0u;
        // |l| in units of ulp_double(h) = 2^(ef - 127 - 52); below a power of two
        // the units of the lower binade are half as large.
        int ne = el + 179 - ef + ((neg && mf == 0u) ? 1 : 0);
        if (ne >= 1) {
            const float ls = __uint_as_float((lb & 0x007FFFFFu) | ((unsigned)ne << 23));
            const long long li = (long long)__float2int_rn(ls);  // |ls| < 2^30
            delta = neg ? -li : li;
        }
    }
    return __longlong_as_double((mag + delta) | (long long)((unsigned long long)s << 32));
}

// (sh, sl) += (ah + al) * (bh + bl), dropping the al*bl term.
__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float bh, float bl) {
    const float p = ah * bh;
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
    const float s = sh + p;
    const float bb = s - sh;
    const float err = (sh - (s - bb)) + (p - bb);
    sh = s;
    sl += err + e;
}

__device__ __forceinline__ void df_norm(float& h, float& l) {
    const float s = h + l;
    l = l - (s - h);
    h = s;
}

// ------------------------------------------------------------------- policies
// store_t: element of the state in HBM. comp_t: element of a tile in shared
// memory (converted once when a tile is loaded and once when it is stored).
// mat_t: matrix element in the pass's matrix pool.
struct ArithF64 {
    using store_t = double2;
    using comp_t = double2;
    using mat_t = double2;
    struct acc_t { double re, im; };
    static constexpr int kId = 1;
    __device__ __forceinline__ static comp_t to_comp(const store_t v) { return v; }
    __device__ __forceinline__ static store_t from_comp(const comp_t v) { return v; }
    __device__ __forceinline__ static void zero(acc_t& a) { a.re = 0.0; a.im = 0.0; }
    __device__ __forceinline__ static void mac(acc_t& a, const mat_t m, const comp_t x) {
        a.re = fma(m.x, x.x, a.re);
        a.re = fma(-m.y, x.y, a.re);
        a.im = fma(m.x, x.y, a.im);
        a.im = fma(m.y, x.x, a.im);
    }
    __device__ __forceinline__ static comp_t finish(acc_t& a) { return make_double2(a.re, a.im); }
    __device__ __forceinline__ static comp_t mul(const mat_t m, const comp_t v) {
        return make_double2(fma(m.x, v.x, -m.y * v.y), fma(m.x, v.y, m.y * v.x));
    }
    // element-wise chains (runs of diagonal and scalar gates) work on comp_t itself
    using elem_t = comp_t;
    __device__ __forceinline__ static elem_t elem_load(const comp_t v) { return v; }
    __device__ __forceinline__ static comp_t elem_store(const elem_t v) { return v; }
    __device__ __forceinline__ static elem_t elem_mul(const mat_t m, const elem_t v) { return mul(m, v); }
};

struct ArithDF {
    using store_t = double2;
    using comp_t = float4;  // (hi.re, hi.im, lo.re, lo.im)
    using mat_t = float4;   // (hi.re, hi.im, lo.re, lo.im)
    struct acc_t { float rh, rl, ih, il; };
    static constexpr int kId = 2;
    __device__ __forceinline__ static comp_t to_comp(const store_t v) {
        const DF a = df_split(v.x), b = df_split(v.y);
        return make_float4(a.h, b.h, a.l, b.l);
    }
    __device__ __forceinline__ static store_t from_comp(const comp_t v) {
        return make_double2(df_combine(v.x, v.z), df_combine(v.y, v.w));
    }
    __device__ __forceinline__ static void zero(acc_t& a) { a.rh = a.rl = a.ih = a.il = 0.f; }
    __device__ __forceinline__ static void mac(acc_t& a, const mat_t m, const comp_t x) {
        df_mac(a.rh, a.rl, m.x, m.z, x.x, x.z);
        df_mac(a.rh, a.rl, -m.y, -m.w, x.y, x.w);
        df_mac(a.ih, a.il, m.x, m.z, x.y, x.w);
        df_mac(a.ih, a.il, m.y, m.w, x.x, x.z);
    }
    __device__ __forceinline__ static comp_t finish(acc_t& a) {
        df_norm(a.rh, a.rl);
        df_norm(a.ih, a.il);
        return make_float4(a.rh, a.ih, a.rl, a.il);
    }
    __device__ __forceinline__ static comp_t mul(const mat_t m, const comp_t v) {
        acc_t a;
        zero(a);
        mac(a, m, v);
        return finish(a);
    }
    // element-wise chains (runs of diagonal and scalar gates) work on comp_t itself
    using elem_t = comp_t;
    __device__ __forceinline__ static elem_t elem_load(const comp_t v) { return v; }
    __device__ __forceinline__ static comp_t elem_store(const elem_t v) { return v; }
    __device__ __forceinline__ static elem_t elem_mul(const mat_t m, const elem_t v) { return mul(m, v); }
};

struct ArithF32 {
    using store_t = float2;
    using comp_t = float2;
    using mat_t = float2;
    struct acc_t { float re, im; };
    static constexpr int kId = 3;
    __device__ __forceinline__ static comp_t to_comp(const store_t v) { return v; }
    __device__ __forceinline__ static store_t from_comp(const comp_t v) { return v; }
    __device__ __forceinline__ static void zero(acc_t& a) { a.re = 0.f; a.im = 0.f; }
    __device__ __forceinline__ static void mac(acc_t& a, const mat_t m, const comp_t x) {
        a.re = fmaf(m.x, x.x, a.re);
        a.re = fmaf(-m.y, x.y, a.re);
        a.im = fmaf(m.x, x.y, a.im);
        a.im = fmaf(m.y, x.x, a.im);
    }
    __device__ __forceinline__ static comp_t finish(acc_t& a) { return make_float2(a.re, a.im); }
    __device__ __forceinline__ static comp_t mul(const mat_t m, const comp_t v) {
        return make_float2(fmaf(m.x, v.x, -m.y * v.y), fmaf(m.x, v.y, m.y * v.x));
    }
    // element-wise chains (runs of diagonal and scalar gates) work on comp_t itself
    using elem_t = comp_t;
    __device__ __forceinline__ static elem_t elem_load(const comp_t v) { return v; }
    __device__ __forceinline__ static comp_t elem_store(const elem_t v) { return v; }
    __device__ __forceinline__ static elem_t elem_mul(const mat_t m, const elem_t v) { return mul(m, v); }
};

// complex64 passes that also run 3xTF32 tensor-core gates: the same FP32
// arithmetic for every other op, a separate kernel instance (register and
// occupancy budget of the tensor-core tasks).
struct ArithTF32 : ArithF32 {
    static constexpr int kId = 5;
};

// complex64 passes that also run two-digit fp16 tensor-core gates.
struct ArithTC64 : ArithF32 {
    static constexpr int kId = 6;
};

// complex128 tiles kept as raw doubles; each operation splits its inputs into
// double-float pairs on the fly and re-assembles its outputs. Used by passes
// that also run tensor-core gates, which read the raw doubles.
struct ArithDFRaw {
    using store_t = double2;
    using comp_t = double2;
    using mat_t = float4;
    using acc_t = ArithDF::acc_t;
    static constexpr int kId = 4;
    __device__ __forceinline__ static comp_t to_comp(const store_t v) { return v; }
    __device__ __forceinline__ static store_t from_comp(const comp_t v) { return v; }
    __device__ __forceinline__ static void zero(acc_t& a) { ArithDF::zero(a); }
    __device__ __forceinline__ static void mac(acc_t& a, const mat_t m, const comp_t x) {
        ArithDF::mac(a, m, ArithDF::to_comp(x));
    }
    __device__ __forceinline__ static comp_t finish(acc_t& a) { return ArithDF::from_comp(ArithDF::finish(a)); }
    __device__ __forceinline__ static comp_t mul(const mat_t m, const comp_t v) {
        return ArithDF::from_comp(ArithDF::mul(m, ArithDF::to_comp(v)));
    }
    // a run of diagonal and scalar gates splits each amplitude once, multiplies
    // in double-float, and re-assembles once
    using elem_t = float4;
    __device__ __forceinline__ static elem_t elem_load(const comp_t v) { return ArithDF::to_comp(v); }
    __device__ __forceinline__ static comp_t elem_store(const elem_t v) { return ArithDF::from_comp(v); }
    __device__ __forceinline__ static elem_t elem_mul(const mat_t m, const elem_t v) { return ArithDF::mul(m, v); }
};

// -------------------------------------------------- |a|^2 accumulation policies
// Probability-type sums are accumulated per thread to about 48 significant bits
// (double-float for complex128 / complex64 storage in DF / F32 mode, FP64 in
// F64 mode) and reduced across threads in FP64.
struct NormAccF64 {
    double s = 0.0;
    __device__ __forceinline__ void add(double2 a) { s = fma(a.x, a.x, fma(a.y, a.y, s)); }
    __device__ __forceinline__ void addv(double v) { s += v; }
    __device__ __forceinline__ double value() const { return s; }
};

struct NormAccDF {
    float h = 0.f, l = 0.f;
    __device__ __forceinline__ void add_real(float xh, float xl) {
        // (h, l) += (xh + xl)^2 ~ xh^2 + 2 xh xl
        const float p = xh * xh;
        float e = fmaf(xh, xh, -p);
        e = fmaf(2.f * xh, xl, e);
        const float s = h + p;
        const float bb = s - h;
        const float err = (h - (s - bb)) + (p - bb);
        h = s;
        l += err + e;
    }
    __device__ __forceinline__ void add(double2 a) {
        const DF r = df_split(a.x), i = df_split(a.y);
        add_real(r.h, r.l);
        add_real(i.h, i.l);
    }
    __device__ __forceinline__ void add(float2 a) {
        add_real(a.x, 0.f);
        add_real(a.y, 0.f);
    }
    __device__ __forceinline__ double value() const { return (double)h + (double)l; }
};

}  // namespace hqs
