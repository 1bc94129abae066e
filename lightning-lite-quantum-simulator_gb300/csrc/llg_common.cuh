// llg_common.cuh -- amplitude precisions, double-float arithmetic and index helpers shared by
// every kernel of the GB300 state-vector engine.
//
// Three ways of holding a complex amplitude in HBM (all kernels are templated on one of them):
//   PolF64  : double2 {re, im}, IEEE FP64 arithmetic.  GB300 issues ~1.6 DFMA/clk/SM, so FP64
//             gate sweeps are FP64-bound at 30-60% of HBM; kept as the plain reference-precision
//             path.
//   PolDF64 : float4 {re.hi, im.hi, re.lo, im.lo}, 16 bytes like complex128.  Each real part is
//             an unevaluated sum hi + lo of two fp32 values (|lo| <= ulp(hi)/2, ~48-bit
//             significand), updated with error-free FP32 transformations (TwoSum, FMA-based
//             TwoProd) on the FP32 pipe (~115 FFMA/clk/SM).  Absolute error per gate is a few
//             2^-48 of the amplitude scale.
//   PolF32  : float2 {re, im}, complex64, FP32 arithmetic.
// Reductions accumulate per thread in double-float (DF64/F32 states) or double (F64 states)
// and finish in FP64.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "llg_common_host.h"

namespace llg {

// ------------------------------------------------------------------------------------------
// double-float scalar
// ------------------------------------------------------------------------------------------
struct df {
    float hi, lo;
};

// Knuth TwoSum: s + e == a + b exactly.
__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// Dekker Fast2Sum (exact when |a| >= |b|; otherwise still within an ulp of s).
__device__ __forceinline__ df fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

__device__ __forceinline__ df df_neg(df x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ df df_add(df x, df y) {
    const df s = two_sum(x.hi, y.hi);
    const float e = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
    return fast_two_sum(s.hi, e);
}

__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

// The products below come in two forms.  The _raw form stops before the closing Fast2Sum: hi + lo
// is the same value, but |lo| may exceed half an ulp of hi.  Amplitudes stored that way stay exact
// sums hi + lo, and every later use takes lo in full (the cross terms of the products, TwoSum of
// the high parts, hi + lo in FP64, the Dot2 and norm accumulators), so an operation's error stays
// a few 2^-46 of its inputs' scale.  Code that splits hi and lo separately against a scale taken
// from hi renormalises first.

// a*x + b*y with one rounding of the high parts removed by TwoSum (16 FP32 instructions raw)
__device__ __forceinline__ df df_lin2_raw(df a, df x, df b, df y) {
    const float p1 = __fmul_rn(a.hi, x.hi);
    const float e1 = fmaf(a.hi, x.hi, -p1);
    const float p2 = __fmul_rn(b.hi, y.hi);
    const float e2 = fmaf(b.hi, y.hi, -p2);
    const df s = two_sum(p1, p2);
    float t = __fadd_rn(e1, e2);
    t = fmaf(a.hi, x.lo, t);
    t = fmaf(a.lo, x.hi, t);
    t = fmaf(b.hi, y.lo, t);
    t = fmaf(b.lo, y.hi, t);
    return {s.hi, __fadd_rn(t, s.lo)};
}
__device__ __forceinline__ df df_lin2(df a, df x, df b, df y) {
    const df r = df_lin2_raw(a, x, b, y);
    return fast_two_sum(r.hi, r.lo);
}

// x + a*y (12 FP32 instructions raw, 15 renormalised, against 19 for df_lin2)
__device__ __forceinline__ df df_fma_raw(df a, df y, df x) {
    const float p = __fmul_rn(a.hi, y.hi);
    const float e = fmaf(a.hi, y.hi, -p);
    const df s = two_sum(x.hi, p);
    float t = __fadd_rn(e, x.lo);
    t = fmaf(a.hi, y.lo, t);
    t = fmaf(a.lo, y.hi, t);
    return {s.hi, __fadd_rn(t, s.lo)};
}
__device__ __forceinline__ df df_fma(df a, df y, df x) {
    const df r = df_fma_raw(a, y, x);
    return fast_two_sum(r.hi, r.lo);
}

// a*x + b*y + c*z + d*w (40 FP32 instructions raw)
__device__ __forceinline__ df df_lin4_raw(df a, df x, df b, df y, df c, df z, df d, df w) {
    const float p1 = __fmul_rn(a.hi, x.hi);
    const float e1 = fmaf(a.hi, x.hi, -p1);
    const float p2 = __fmul_rn(b.hi, y.hi);
    const float e2 = fmaf(b.hi, y.hi, -p2);
    const float p3 = __fmul_rn(c.hi, z.hi);
    const float e3 = fmaf(c.hi, z.hi, -p3);
    const float p4 = __fmul_rn(d.hi, w.hi);
    const float e4 = fmaf(d.hi, w.hi, -p4);
    const df s12 = two_sum(p1, p2);
    const df s34 = two_sum(p3, p4);
    const df s = two_sum(s12.hi, s34.hi);
    float t = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(e3, e4));
    t = fmaf(a.hi, x.lo, t);
    t = fmaf(a.lo, x.hi, t);
    t = fmaf(b.hi, y.lo, t);
    t = fmaf(b.lo, y.hi, t);
    t = fmaf(c.hi, z.lo, t);
    t = fmaf(c.lo, z.hi, t);
    t = fmaf(d.hi, w.lo, t);
    t = fmaf(d.lo, w.hi, t);
    return {s.hi, __fadd_rn(t, __fadd_rn(s.lo, __fadd_rn(s12.lo, s34.lo)))};
}
__device__ __forceinline__ df df_lin4(df a, df x, df b, df y, df c, df z, df d, df w) {
    const df r = df_lin4_raw(a, x, b, y, c, z, d, w);
    return fast_two_sum(r.hi, r.lo);
}

// Dot2 accumulator (Ogita, Rump and Oishi, SIAM J. Sci. Comput. 2005): s + e carries a sum of
// double-float products, each high product split exactly by FMA and added by TwoSum
struct DotDF {
    float s = 0.0f, e = 0.0f;
    __device__ __forceinline__ void add(df a, df b) {
        const float p = __fmul_rn(a.hi, b.hi);
        const float pe = fmaf(a.hi, b.hi, -p);
        const df t = two_sum(s, p);
        s = t.hi;
        float c = fmaf(a.hi, b.lo, pe);
        c = fmaf(a.lo, b.hi, c);
        e = __fadd_rn(e, __fadd_rn(c, t.lo));
    }
    __device__ __forceinline__ df value() const { return fast_two_sum(s, e); }
};

// x*x + y*y (for |a|^2 accumulation)
__device__ __forceinline__ df df_sqsum(df x, df y) { return df_lin2(x, x, y, y); }

__device__ __forceinline__ double df_to_double(df x) { return (double)x.hi + (double)x.lo; }

__device__ __forceinline__ df double_to_df(double x) {
    const float h = __double2float_rn(x);
    const float l = __double2float_rn(x - (double)h);
    return {h, l};
}

// ------------------------------------------------------------------------------------------
// precision policies.  Each has: S (HBM element), R (real in registers), K (gate coefficient),
// C (complex in registers), Acc (reduction accumulator), and the scalar operations kernels use.
// ------------------------------------------------------------------------------------------
template <class R>
struct cplx {
    R re, im;
};

struct PolF64 {
    using S = double2;
    using R = double;
    using K = double;
    using Acc = double;
    using C = cplx<double>;
    static constexpr int kPrecision = 0;
    __device__ static C load(const S& s) { return {s.x, s.y}; }
    __device__ static S store(const C& c) { return make_double2(c.re, c.im); }
    __device__ static R lin2(K a, R x, K b, R y) { return fma(a, x, b * y); }
    __device__ static R lin2_raw(K a, R x, K b, R y) { return fma(a, x, b * y); }
    __device__ static R fma1(K a, R y, R x) { return fma(a, y, x); }
    __device__ static R fma1_raw(K a, R y, R x) { return fma(a, y, x); }
    __device__ static R lin4(K a, R x, K b, R y, K c, R z, K d, R w) {
        return fma(a, x, fma(b, y, fma(c, z, d * w)));
    }
    __device__ static R lin4_raw(K a, R x, K b, R y, K c, R z, K d, R w) { return lin4(a, x, b, y, c, z, d, w); }
    __device__ static R add(R x, R y) { return x + y; }
    __device__ static R sub(R x, R y) { return x - y; }
    // the sign bit flipped on the integer pipe (the same bits as IEEE negation); a plain -x that is
    // not folded into a multiply-add runs on the FP64 pipe, this GPU's scarcest
    __device__ static R neg(R x) { return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ULL); }
    __device__ static K kneg(K x) { return neg(x); }
    __device__ static R mulk(K a, R x) { return a * x; }
    __device__ static R zero() { return 0.0; }
    __device__ static Acc acc_zero() { return 0.0; }
    __device__ static Acc acc_add(Acc a, Acc b) { return a + b; }
    __device__ static Acc acc_norm(Acc a, const C& c) { return fma(c.re, c.re, fma(c.im, c.im, a)); }
    // acc + w * |c|^2 with a small integer weight w (exact in every format)
    __device__ static Acc acc_norm_w(Acc a, const C& c, float w) { return fma((double)w, c.re * c.re + c.im * c.im, a); }
    // acc + re(conj(x) * y) and acc + im(conj(x) * y)
    __device__ static Acc acc_dot_re(Acc a, const C& x, const C& y) { return fma(x.re, y.re, fma(x.im, y.im, a)); }
    __device__ static Acc acc_dot_im(Acc a, const C& x, const C& y) { return fma(x.re, y.im, fma(-x.im, y.re, a)); }
    // acc + d * |c|^2 for a real weight d given in double (a diagonal observable's eigenvalue)
    __device__ static Acc acc_norm_d(Acc a, const C& c, double d) { return fma(d, fma(c.re, c.re, c.im * c.im), a); }
    __device__ static double acc_to_double(Acc a) { return a; }
    __device__ static Acc acc_from_double(double a) { return a; }
    __device__ static C from_f64(double2 v) { return {v.x, v.y}; }
    __device__ static double2 to_f64(const C& c) { return make_double2(c.re, c.im); }
    __device__ static K k_from_bits(uint64_t b) { return __longlong_as_double((long long)b); }
    __device__ static K k_from_double(double d) { return d; }
    __device__ static R r_from_float(float f) { return (double)f; }
};

struct PolF32 {
    using S = float2;
    using R = float;
    using K = float;
    using Acc = df;
    using C = cplx<float>;
    static constexpr int kPrecision = 2;
    __device__ static C load(const S& s) { return {s.x, s.y}; }
    __device__ static S store(const C& c) { return make_float2(c.re, c.im); }
    __device__ static R lin2(K a, R x, K b, R y) { return fmaf(a, x, b * y); }
    __device__ static R lin2_raw(K a, R x, K b, R y) { return fmaf(a, x, b * y); }
    __device__ static R fma1(K a, R y, R x) { return fmaf(a, y, x); }
    __device__ static R fma1_raw(K a, R y, R x) { return fmaf(a, y, x); }
    __device__ static R lin4(K a, R x, K b, R y, K c, R z, K d, R w) {
        return fmaf(a, x, fmaf(b, y, fmaf(c, z, d * w)));
    }
    __device__ static R lin4_raw(K a, R x, K b, R y, K c, R z, K d, R w) { return lin4(a, x, b, y, c, z, d, w); }
    __device__ static R add(R x, R y) { return x + y; }
    __device__ static R sub(R x, R y) { return x - y; }
    __device__ static R neg(R x) { return -x; }
    __device__ static K kneg(K x) { return -x; }
    __device__ static R mulk(K a, R x) { return a * x; }
    __device__ static R zero() { return 0.0f; }
    __device__ static Acc acc_zero() { return {0.0f, 0.0f}; }
    __device__ static Acc acc_add(Acc a, Acc b) { return df_add(a, b); }
    __device__ static Acc acc_term(float v, Acc a) {
        const df s = two_sum(a.hi, v);
        return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
    }
    __device__ static Acc acc_norm(Acc a, const C& c) {
        // exact products of fp32 values, summed in double-float
        const float p = __fmul_rn(c.re, c.re), q = __fmul_rn(c.im, c.im);
        const float ep = fmaf(c.re, c.re, -p), eq = fmaf(c.im, c.im, -q);
        const df s = two_sum(p, q);
        const df v = fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(ep, eq)));
        return df_add(a, v);
    }
    __device__ static Acc acc_norm_w(Acc a, const C& c, float w) {
        const float p = __fmul_rn(c.re, c.re), q = __fmul_rn(c.im, c.im);
        const float ep = fmaf(c.re, c.re, -p), eq = fmaf(c.im, c.im, -q);
        const df s = two_sum(p, q);
        const df v = fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(ep, eq)));
        return df_add(a, df_mul(v, df{w, 0.0f}));
    }
    __device__ static Acc acc_dot_re(Acc a, const C& x, const C& y) {
        return df_add(a, df_lin2(df{x.re, 0.f}, df{y.re, 0.f}, df{x.im, 0.f}, df{y.im, 0.f}));
    }
    __device__ static Acc acc_dot_im(Acc a, const C& x, const C& y) {
        return df_add(a, df_lin2(df{x.re, 0.f}, df{y.im, 0.f}, df{-x.im, 0.f}, df{y.re, 0.f}));
    }
    __device__ static Acc acc_norm_d(Acc a, const C& c, double d) {
        const float p = __fmul_rn(c.re, c.re), q = __fmul_rn(c.im, c.im);
        const float ep = fmaf(c.re, c.re, -p), eq = fmaf(c.im, c.im, -q);
        const df s = two_sum(p, q);
        const df v = fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(ep, eq)));
        return df_add(a, df_mul(v, double_to_df(d)));
    }
    __device__ static double acc_to_double(Acc a) { return df_to_double(a); }
    __device__ static Acc acc_from_double(double a) { return double_to_df(a); }
    __device__ static C from_f64(double2 v) { return {__double2float_rn(v.x), __double2float_rn(v.y)}; }
    __device__ static double2 to_f64(const C& c) { return make_double2((double)c.re, (double)c.im); }
    __device__ static K k_from_bits(uint64_t b) { return __uint_as_float((uint32_t)b); }
    __device__ static K k_from_double(double d) { return __double2float_rn(d); }
    __device__ static R r_from_float(float f) { return f; }
};

struct PolDF64 {
    using S = float4;  // {re.hi, im.hi, re.lo, im.lo}
    using R = df;
    using K = df;
    using Acc = df;
    using C = cplx<df>;
    static constexpr int kPrecision = 1;
    __device__ static C load(const S& s) { return {df{s.x, s.z}, df{s.y, s.w}}; }
    __device__ static S store(const C& c) { return make_float4(c.re.hi, c.im.hi, c.re.lo, c.im.lo); }
    __device__ static R lin2(K a, R x, K b, R y) { return df_lin2(a, x, b, y); }
    __device__ static R lin2_raw(K a, R x, K b, R y) { return df_lin2_raw(a, x, b, y); }
    __device__ static R fma1(K a, R y, R x) { return df_fma(a, y, x); }  // x + a*y
    __device__ static R fma1_raw(K a, R y, R x) { return df_fma_raw(a, y, x); }
    __device__ static R lin4(K a, R x, K b, R y, K c, R z, K d, R w) { return df_lin4(a, x, b, y, c, z, d, w); }
    __device__ static R lin4_raw(K a, R x, K b, R y, K c, R z, K d, R w) {
        return df_lin4_raw(a, x, b, y, c, z, d, w);
    }
    __device__ static R add(R x, R y) { return df_add(x, y); }
    __device__ static R sub(R x, R y) { return df_sub(x, y); }
    __device__ static R neg(R x) { return df_neg(x); }
    __device__ static K kneg(K x) { return df_neg(x); }
    __device__ static R mulk(K a, R x) { return df_mul(a, x); }
    __device__ static R zero() { return {0.0f, 0.0f}; }
    __device__ static Acc acc_zero() { return {0.0f, 0.0f}; }
    __device__ static Acc acc_add(Acc a, Acc b) { return df_add(a, b); }
    __device__ static Acc acc_norm(Acc a, const C& c) { return df_add(a, df_sqsum(c.re, c.im)); }
    __device__ static Acc acc_norm_w(Acc a, const C& c, float w) {
        return df_add(a, df_mul(df_sqsum(c.re, c.im), df{w, 0.0f}));
    }
    __device__ static Acc acc_dot_re(Acc a, const C& x, const C& y) { return df_add(a, df_lin2(x.re, y.re, x.im, y.im)); }
    __device__ static Acc acc_dot_im(Acc a, const C& x, const C& y) {
        return df_add(a, df_lin2(x.re, y.im, df_neg(x.im), y.re));
    }
    __device__ static Acc acc_norm_d(Acc a, const C& c, double d) {
        return df_add(a, df_mul(df_sqsum(c.re, c.im), double_to_df(d)));
    }
    __device__ static double acc_to_double(Acc a) { return df_to_double(a); }
    __device__ static Acc acc_from_double(double a) { return double_to_df(a); }
    __device__ static C from_f64(double2 v) { return {double_to_df(v.x), double_to_df(v.y)}; }
    __device__ static double2 to_f64(const C& c) { return make_double2(df_to_double(c.re), df_to_double(c.im)); }
    __device__ static K k_from_bits(uint64_t b) {
        return df{__uint_as_float((uint32_t)b), __uint_as_float((uint32_t)(b >> 32))};
    }
    __device__ static K k_from_double(double d) { return double_to_df(d); }
    __device__ static R r_from_float(float f) { return df{f, 0.0f}; }
};

// ------------------------------------------------------------------------------------------
// reductions on the FP32 pipe: warp and block sums of double-float values.  GB300 issues FP64
// at ~1.6 ops/clk/SM, so a warp-wide DADD holds the FP64 pipe for ~20 cycles; partial sums of
// per-thread accumulators are therefore combined as double-float and converted once.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ df shfl_down_df(df v, int off) {
    return {__shfl_down_sync(0xffffffffu, v.hi, off), __shfl_down_sync(0xffffffffu, v.lo, off)};
}

__device__ __forceinline__ df warp_sum_df(df v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = df_add(v, shfl_down_df(v, off));
    return v;
}

__device__ __forceinline__ double warp_sum_dbl(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;
}

__device__ __forceinline__ df warp_sum_acc(df v) { return warp_sum_df(v); }
__device__ __forceinline__ double warp_sum_acc(double v) { return warp_sum_dbl(v); }

__device__ __forceinline__ df acc_plus(df a, df b) { return df_add(a, b); }
__device__ __forceinline__ double acc_plus(double a, double b) { return a + b; }
__device__ __forceinline__ df acc_minus(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ double acc_minus(double a, double b) { return a - b; }
__device__ __forceinline__ double acc_value(df a) { return df_to_double(a); }
__device__ __forceinline__ double acc_value(double a) { return a; }

// Sum over the block of one accumulator per thread; the result is valid in thread 0.  `sh` holds
// one entry per warp.  Starts with a barrier, so `sh` may be reused by consecutive calls.
template <class A>
__device__ __forceinline__ A block_sum_acc(A v, A* sh) {
    v = warp_sum_acc(v);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    A r = v;
    if (warp == 0) {  // the warp sums in a second shuffle tree (no serial loop in one thread)
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : A{};
        r = warp_sum_acc(r);
    }
    return r;
}

// ------------------------------------------------------------------------------------------
// index helpers
// ------------------------------------------------------------------------------------------
// Insert a 0 at bit `bit` (a power of two) of a 32-bit tile-local index: p + (p & ~(bit - 1))
// doubles the part above the bit and keeps the part below (two integer instructions).
__device__ __forceinline__ uint32_t ins0(uint32_t p, uint32_t bit) { return p + (p & (0u - bit)); }

__host__ __device__ __forceinline__ uint64_t insert0(uint64_t p, int q) {
    const uint64_t low = p & ((1ULL << q) - 1);
    return ((p >> q) << (q + 1)) | low;
}

// Insert zero bits at the positions of `mask` (ascending), i.e. the bit-deposit of p into ~mask.
__host__ __device__ __forceinline__ uint64_t insert0_mask(uint64_t p, uint64_t mask) {
    while (mask) {
#ifdef __CUDA_ARCH__
        const int b = __ffsll((long long)mask) - 1;
#else
        const int b = __builtin_ctzll(mask);
#endif
        p = insert0(p, b);
        mask &= mask - 1;
    }
    return p;
}

}  // namespace llg
