// Small-angle fast paths for the trigonometry of the step.
//
// The characteristic-map and trace geometry works with angles of a few grid
// cells (|x| well below 1 rad).  For those, truncated Taylor series in x^2
// (coefficients 1/(2k+1)!, 1/(2k)!, the binomial series of arcsin and the
// Gregory series of arctan) evaluated by Horner's rule are accurate to below
// float rounding; larger arguments fall back to the CUDA library functions.
// Truncation bounds on the fast intervals are given beside each function.
#pragma once
#include <math.h>

namespace sb {

// Cold paths: the library functions for arguments outside the fast
// intervals, kept out of line so that the hot loops stay small in the
// instruction cache.
__device__ __noinline__ void slow_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __noinline__ float slow_sinc(float x) { return sinf(x) / x; }
__device__ __noinline__ float slow_cos(float x) { return cosf(x); }
__device__ __noinline__ float slow_arc(float x) { return 2.0f * asinf(fminf(x, 1.0f)); }
__device__ __noinline__ float slow_atan2(float y, float x) { return atan2f(y, x); }

// sin and cos; Taylor to x^3 / x^4 on |x| <= 1/32 (the usual half-angle of
// a few cells; relative truncation < 1e-8), to x^7 / x^8 on |x| <= 0.2
// (< 2e-12), to x^11 / x^12 on |x| <= 0.8 (< 1e-11).
__device__ __forceinline__ void fsincos(float x, float* s, float* c) {
    if (fabsf(x) <= 0.03125f) {
        const float x2 = x * x;
        *s = fmaf(-1.6666666667e-1f * x2, x, x);                 // x - x^3/3!
        *c = fmaf(fmaf(x2, 4.1666666667e-2f, -0.5f), x2, 1.0f);  // 1 - x^2/2! + x^4/4!
        return;
    }
    if (fabsf(x) <= 0.2f) {
        const float x2 = x * x;
        float ps = -1.9841269841e-4f;          // -1/7!
        ps = fmaf(ps, x2, 8.3333333333e-3f);   //  1/5!
        ps = fmaf(ps, x2, -1.6666666667e-1f);  // -1/3!
        *s = fmaf(ps * x2, x, x);
        float pc = 2.4801587302e-5f;           //  1/8!
        pc = fmaf(pc, x2, -1.3888888889e-3f);  // -1/6!
        pc = fmaf(pc, x2, 4.1666666667e-2f);   //  1/4!
        pc = fmaf(pc, x2, -0.5f);
        *c = fmaf(pc, x2, 1.0f);
        return;
    }
    if (fabsf(x) <= 0.8f) {
        const float x2 = x * x;
        float ps = -2.5052108385e-8f;          // -1/11!
        ps = fmaf(ps, x2, 2.7557319224e-6f);   //  1/9!
        ps = fmaf(ps, x2, -1.9841269841e-4f);  // -1/7!
        ps = fmaf(ps, x2, 8.3333333333e-3f);   //  1/5!
        ps = fmaf(ps, x2, -1.6666666667e-1f);  // -1/3!
        *s = fmaf(ps * x2, x, x);
        float pc = 2.0876756988e-9f;           //  1/12!
        pc = fmaf(pc, x2, -2.7557319224e-7f);  // -1/10!
        pc = fmaf(pc, x2, 2.4801587302e-5f);   //  1/8!
        pc = fmaf(pc, x2, -1.3888888889e-3f);  // -1/6!
        pc = fmaf(pc, x2, 4.1666666667e-2f);   //  1/4!
        pc = fmaf(pc, x2, -0.5f);
        *c = fmaf(pc, x2, 1.0f);
        return;
    }
    slow_sincos(x, s, c);
}

// sin(x) / x; Taylor to x^8 on |x| <= 0.5 (truncation < 1e-11).
__device__ __forceinline__ float fsinc(float x) {
    const float x2 = x * x;
    if (x2 <= 0.25f) {
        float p = 2.7557319224e-6f;            //  1/9!
        p = fmaf(p, x2, -1.9841269841e-4f);    // -1/7!
        p = fmaf(p, x2, 8.3333333333e-3f);     //  1/5!
        p = fmaf(p, x2, -1.6666666667e-1f);    // -1/3!
        return fmaf(p, x2, 1.0f);
    }
    return slow_sinc(x);
}

// cos(x); Taylor to x^10 on |x| <= 0.5 (truncation < 1e-12).
__device__ __forceinline__ float fcos_small(float x) {
    const float x2 = x * x;
    if (x2 <= 0.25f) {
        float p = -2.7557319224e-7f;           // -1/10!
        p = fmaf(p, x2, 2.4801587302e-5f);     //  1/8!
        p = fmaf(p, x2, -1.3888888889e-3f);    // -1/6!
        p = fmaf(p, x2, 4.1666666667e-2f);     //  1/4!
        p = fmaf(p, x2, -0.5f);
        return fmaf(p, x2, 1.0f);
    }
    return slow_cos(x);
}

// 2 asin(c / 2) for a chord c in [0, 2]: the arc of a chord on the unit
// sphere.  Binomial series of arcsin to x^5 on x = c/2 <= 1/16 (truncation
// < 3e-9 relative), to x^11 on x <= 0.25 (< 3e-10).
__device__ __forceinline__ float farc_of_chord(float c) {
    const float x = 0.5f * c;
    if (x <= 0.0625f) {
        const float x2 = x * x;
        const float p = fmaf(x2, 7.5e-2f, 1.6666666667e-1f);  // 1/6 + 3/40 x^2
        return 2.0f * fmaf(p * x2, x, x);
    }
    if (x <= 0.25f) {
        const float x2 = x * x;
        float p = 2.2372159091e-2f;            // 63/2816
        p = fmaf(p, x2, 3.0381944444e-2f);     // 35/1152
        p = fmaf(p, x2, 4.4642857143e-2f);     // 5/112
        p = fmaf(p, x2, 7.5e-2f);              // 3/40
        p = fmaf(p, x2, 1.6666666667e-1f);     // 1/6
        return 2.0f * fmaf(p * x2, x, x);
    }
    return slow_arc(x);
}

// atan2(y, x); Gregory series of atan(y/x) to t^5 when x > 0 and
// |y| <= x/16 (truncation < 1e-8 relative), to t^15 when |y| <= x/4
// (< 1e-10), library atan2f otherwise.
__device__ __forceinline__ float fatan2(float y, float x) {
    if (x > 0.0f && fabsf(y) <= 0.25f * x) {
        const float t = y / x;
        const float t2 = t * t;
        if (t2 <= 0.00390625f) {
            const float p = fmaf(t2, 2.0e-1f, -3.3333333333e-1f);  // -1/3 + t^2/5
            return fmaf(p * t2, t, t);
        }
        float p = -6.6666666667e-2f;           // -1/15
        p = fmaf(p, t2, 7.6923076923e-2f);     //  1/13
        p = fmaf(p, t2, -9.0909090909e-2f);    // -1/11
        p = fmaf(p, t2, 1.1111111111e-1f);     //  1/9
        p = fmaf(p, t2, -1.4285714286e-1f);    // -1/7
        p = fmaf(p, t2, 2.0e-1f);              //  1/5
        p = fmaf(p, t2, -3.3333333333e-1f);    // -1/3
        return fmaf(p * t2, t, t);
    }
    return slow_atan2(y, x);
}

// fatan2 with the fast paths' quotient taken by __fdividef (reciprocal
// and product, at most 2 ulp from the rounded quotient): for positions that
// only select and weight samples (not stored in a characteristic map),
// where 2 ulp of an offset of a few cells is ~1e-6 of a cell.
__device__ __forceinline__ float fatan2_fast(float y, float x) {
    if (x > 0.0f && fabsf(y) <= 0.25f * x) {
        const float t = __fdividef(y, x);
        const float t2 = t * t;
        if (t2 <= 0.00390625f) {
            const float p = fmaf(t2, 2.0e-1f, -3.3333333333e-1f);  // -1/3 + t^2/5
            return fmaf(p * t2, t, t);
        }
        float p = -6.6666666667e-2f;           // -1/15
        p = fmaf(p, t2, 7.6923076923e-2f);     //  1/13
        p = fmaf(p, t2, -9.0909090909e-2f);    // -1/11
        p = fmaf(p, t2, 1.1111111111e-1f);     //  1/9
        p = fmaf(p, t2, -1.4285714286e-1f);    // -1/7
        p = fmaf(p, t2, 2.0e-1f);              //  1/5
        p = fmaf(p, t2, -3.3333333333e-1f);    // -1/3
        return fmaf(p * t2, t, t);
    }
    return slow_atan2(y, x);
}

}  // namespace sb
