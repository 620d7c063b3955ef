// Symmetric power-of-two scaling of the implicit surfactant system, shared
// by its assembly (sb_step.cu) and its solver (sb_solver.cu).
//
// FP32 range guard.  A cell's diagonal term t = sin(theta) / (dt gamma_adv)
// grows without bound as advection empties the cell of surfactant (1e-37
// leaves t near the FP32 maximum, a subnormal gamma puts it past it), and the
// preconditioner's factors take quotients by it and products of two of them.
// For t > 2^48 (tested as gamma < A 2^-48) the cell's unknown becomes y = dx / s with s = 2^-k,
// 2^45 < t s^2 <= 2^48, and its row and column of the matrix are multiplied
// by s: a symmetric scaling by powers of two, which FP32 applies exactly, so
// the solution is the unscaled system's.  t itself is never formed: k comes
// from the exponents of A = sin(theta) / dt and gamma, and t s^2 is
// A / (gamma 4^k), gamma 4^k being exact.  gamma_adv = 0 (where the
// reference's diagonal is infinite) is taken as the limit t -> infinity:
// t s^2 = 2^48 with s = 2^-64, so that the cell's increment is 0.
// Every kernel that needs a cell's k (the assembly for the cell and its
// neighbours, the solver's warm start and final pass) evaluates it from the
// same operands with the same operations, and so gets the same k.
#pragma once

namespace sb {

constexpr int kScaleLog2 = 48;
constexpr int kScaleZero = 64;  // k of gamma_adv = 0

// floor(log2 x) of a finite x > 0, subnormals included.
__device__ __forceinline__ int ilog2_pos(float x) {
    const unsigned u = __float_as_uint(x);
    const int ex = (int)((u >> 23) & 0xffu);
    if (ex != 0) return ex - 127;
    return (31 - __clz((int)(u & 0x7fffffu))) - 149;
}

__device__ __forceinline__ int diag_scale_k(float gamma, float sinT, float invDt) {
    const float A = sinT * invDt;
    if (gamma == 0.0f) return kScaleZero;
    if (!(gamma < A * 0x1p-48f)) return 0;  // t <= 2^48 (A 2^-48 is exact); also NaN
    const int e = ilog2_pos(A) - ilog2_pos(gamma);  // log2 t in (e - 1, e + 1), e >= 48
    return min(max((e - (kScaleLog2 - 2)) / 2, 1), 63);  // ceil((e - 47) / 2)
}

__device__ __forceinline__ float pow2_neg(int k) {  // 2^-k, 0 <= k <= 126
    return __int_as_float((127 - k) << 23);
}

__device__ __forceinline__ float pow2_pos(int k) {  // 2^k, 0 <= k <= 127
    return __int_as_float((127 + k) << 23);
}

// t s^2 for the cell's k (t itself when k = 0).
__device__ __forceinline__ float scaled_diag_term(float gamma, float sinT, float invDt, int k) {
    if (k == 0) return sinT * invDt / gamma;
    if (gamma == 0.0f) return 0x1p48f;
    return sinT * invDt / (gamma * pow2_pos(2 * k));
}

}  // namespace sb
