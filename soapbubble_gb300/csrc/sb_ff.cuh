// Float-float ("double-float") arithmetic for the accumulations of the
// implicit solve.  A value is the unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi) / 2, about 48 significant bits.  GB300 executes FP64 at a
// small fraction of its FP32 rate, so the solver's FP64-class dot products,
// iterate and refinement residual are carried on the FP32 pipes in this
// form; only per-phase scalars use hardware FP64.
//
// The building blocks are the error-free transformations TwoSum (Knuth,
// TAOCP vol. 2, 4.2.2), FastTwoSum (Dekker 1971) and TwoProd through a fused
// multiply-add; additions renormalise as in the "sloppy" double-double
// addition of Dekker's method.  Every operation is written with explicit
// round-to-nearest intrinsics, so the compiler can neither fuse nor
// reassociate them and results are reproducible bit for bit.
#pragma once
#include <cuda_runtime.h>

namespace sb {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_zero() { return {0.0f, 0.0f}; }

// a + b = s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// a + b = s + e exactly when |a| >= |b| (or a == 0).
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// a * b = p + e exactly (barring underflow).
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

__device__ __forceinline__ ff ff_add(ff x, ff y) {
    float s, e;
    two_sum(x.hi, y.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
    ff r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}

// x + a (a float).
__device__ __forceinline__ ff ff_add_f(ff x, float a) {
    float s, e;
    two_sum(x.hi, a, s, e);
    e = __fadd_rn(e, x.lo);
    ff r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}

// x + a * b with the product a * b (floats) taken exactly.
__device__ __forceinline__ ff ff_add_prod(ff x, float a, float b) {
    float p, pe, s, e;
    two_prod(a, b, p, pe);
    two_sum(x.hi, p, s, e);
    e = __fadd_rn(e, __fadd_rn(x.lo, pe));
    ff r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}

// x * a (a float).
__device__ __forceinline__ ff ff_mul_f(ff x, float a) {
    float p, e;
    two_prod(x.hi, a, p, e);
    e = __fmaf_rn(x.lo, a, e);
    ff r;
    fast_two_sum(p, e, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ ff ff_neg(ff x) { return {-x.hi, -x.lo}; }

// x / y: a float quotient corrected by one step on the float-float
// remainder x - q y (about 44 correct bits).
__device__ __forceinline__ ff ff_div(ff x, ff y) {
    const float q1 = __fdiv_rn(x.hi, y.hi);
    const ff r = ff_add(x, ff_neg(ff_mul_f(y, q1)));
    const float q2 = __fdiv_rn(r.hi, y.hi);
    ff q;
    fast_two_sum(q1, q2, q.hi, q.lo);
    return q;
}

// x <= y for normalised values.
__device__ __forceinline__ bool ff_le(ff x, ff y) {
    return x.hi < y.hi || (x.hi == y.hi && x.lo <= y.lo);
}

// Rounded to the nearest float (up to one rounding of hi + lo).
__device__ __forceinline__ float ff_to_f(ff x) { return __fadd_rn(x.hi, x.lo); }

// A double split into float-float (for scalars computed in FP64).
__device__ __forceinline__ ff ff_from_d(double v) {
    ff r;
    r.hi = __double2float_rn(v);
    r.lo = __double2float_rn(__dsub_rn(v, (double)r.hi));
    return r;
}

__device__ __forceinline__ double ff_to_d(ff x) { return __dadd_rn((double)x.hi, (double)x.lo); }

// Warp sum (butterfly; every lane gets the same value for equal inputs).
__device__ __forceinline__ ff ff_warp_sum(ff v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ff w;
        w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
        v = ff_add(v, w);
    }
    return v;
}

}  // namespace sb
