// Device-side geometry of the lat-long MAC grid: samplers with pole
// reflection, great-circle backtrace, and characteristic-map interpolation.
//
// Positions are kept relative to the thread's own grid point so that FP32
// keeps ~1e-7 cell precision at every grid size:
//   * a position is an integer base (bi, bj) plus float offsets (ox, oy) in
//     grid units, raw coordinates theta/h = bi + ox and phi/h = bj + oy;
//   * geometry is done in a local Cartesian frame rotated about z so that the
//     base point sits at azimuth 0: C = (sin t0, 0, cos t0), e_theta =
//     (cos t0, 0, -sin t0), e_phi = (0, 1, 0); nearby points are carried as
//     displacements d = P - C, converted to and from grid offsets with
//     half-angle formulas that never subtract two O(1) quantities;
//   * characteristic maps store, per cell, the mapped point's displacement
//     from the cell centre in the cell's own frame (a float4: x, y, z, 0).
//     A lookup from another cell's frame rotates it about z by the column
//     difference and adds the difference of the two centres, both from
//     tables computed in FP64 (rottab: sin and cos - 1 of dc h; rowtab: sin
//     and cos of the row angles as hi + lo pairs, so that the difference of
//     two rows' values keeps full precision); writing a map entry is a
//     store of the displacement the step computed in the cell's frame.
// The arithmetic is the reference's (kernel/bubble.cu:116-606): geometric
// pole reflection with vector sign flips, NaN-skipping bilinear lerp,
// great-circle RK2 trace with parallel transport, spherical lerp of map
// points.  Only the representation of positions differs.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <cuda_bf16.h>

#include "sb_fastmath.cuh"
#include "sb_internal.h"
#include "sb_types.h"

// Inlining of the geometry helpers: the slerp and the map lookup are inlined
// (measured faster); the position of a displacement (pos_from_disp) stays
// out of line, which keeps the map kernels small in the instruction cache.
#ifndef SB_GEOM_INLINE
#define SB_GEOM_INLINE __forceinline__
#endif
#ifndef SB_CONV_INLINE
#define SB_CONV_INLINE __noinline__
#endif

namespace sb {

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float len3(f3 a) { return sqrtf(dot3(a, a)); }

// Local frame at a base grid point: raw coordinates (bi + fi, bj + fj),
// fi, fj in {0, 0.5, -0.5}; s0/c0 = sin/cos of its polar angle.
struct Frame {
    int bi, bj;
    float fi, fj;
    float s0, c0;
    float s0lo, c0lo;  // cell frames: the low parts of s0, c0 (rowtab); else 0
};

// A sample position: raw theta/h = bi + ox, raw phi/h = bj + oy.
struct Pos {
    int bi, bj;
    float ox, oy;
};

// NaN-skipping lerp (kernel/bubble.cu:153-160).
__device__ __forceinline__ float blerp(float from, float to, float a) {
    if (isnan(from)) return to;
    if (isnan(to)) return from;
    return (1.0f - a) * from + a * to;
}

// The same lerp without the NaN tests.  A bilinear sample is formed with it
// first: a result that is not NaN means no sample was NaN, and then every
// lerp took blerp's last line, so the result is bit for bit blerp's; a NaN
// result is formed again with blerp (the reference's NaN skipping).
__device__ __forceinline__ float lerp_raw(float from, float to, float a) {
    return (1.0f - a) * from + a * to;
}

// Bilinear sample from four values (lerp_raw first, blerp for a NaN).
__device__ __forceinline__ float bilerp(float f00, float f01, float f10, float f11, float a,
                                        float b) {
    const float r = lerp_raw(lerp_raw(f00, f01, b), lerp_raw(f10, f11, b), a);
    if (!isnan(r)) return r;
    return blerp(blerp(f00, f01, b), blerp(f10, f11, b), a);
}

// Grid position of the point C + d.  Points past a pole come back with the
// base column shifted by nTheta (azimuth + pi) so the float offset stays small.
__device__ SB_CONV_INLINE Pos pos_from_disp(Frame F, f3 d, float invh, int nT) {
    const float Px = F.s0 + d.x, Py = d.y, Pz = F.c0 + d.z;
    const float rho = sqrtf(Px * Px + Py * Py);
    const float den = rho + F.s0;
    const float rms0 = den > 0.0f ? (2.0f * F.s0 * d.x + d.x * d.x + d.y * d.y) / den : 0.0f;
    const float sdt = rms0 * F.c0 - d.z * F.s0;   // sin(t1 - t0) scaled by |P|
    const float cdt = rho * F.s0 + Pz * F.c0;     // cos(t1 - t0) scaled by |P|
    Pos q;
    q.bi = F.bi;
    q.ox = F.fi + fatan2(sdt, cdt) * invh;
    if (Px >= 0.0f) {
        q.bj = F.bj;
        q.oy = F.fj + fatan2(Py, Px) * invh;
    } else {
        q.bj = F.bj + nT;
        q.oy = F.fj + fatan2(-Py, -Px) * invh;
    }
    return q;
}

// pos_from_disp for positions that only select and weight samples (the
// departure points of field samples and of map lookups whose result is not
// stored): the same formulas with the quotients taken by __fdividef, which
// places the point within ~1e-6 of a cell.
__device__ SB_CONV_INLINE Pos pos_from_disp_fast(Frame F, f3 d, float invh, int nT) {
    const float Px = F.s0 + d.x, Py = d.y, Pz = F.c0 + d.z;
    const float rho = sqrtf(Px * Px + Py * Py);
    const float den = rho + F.s0;
    const float rms0 =
        den > 0.0f ? __fdividef(2.0f * F.s0 * d.x + d.x * d.x + d.y * d.y, den) : 0.0f;
    const float sdt = rms0 * F.c0 - d.z * F.s0;
    const float cdt = rho * F.s0 + Pz * F.c0;
    Pos q;
    q.bi = F.bi;
    q.ox = F.fi + fatan2_fast(sdt, cdt) * invh;
    if (Px >= 0.0f) {
        q.bj = F.bj;
        q.oy = F.fj + fatan2_fast(Py, Px) * invh;
    } else {
        q.bj = F.bj + nT;
        q.oy = F.fj + fatan2_fast(-Py, -Px) * invh;
    }
    return q;
}

// Great-circle angle (grid units) between the frame's base and C + d.
__device__ __forceinline__ float dist_from_disp(f3 d, float invh) {
    return farc_of_chord(len3(d)) * invh;
}

// Spherical lerp between C + dA and C + dB, returned as a displacement.
// Same great-circle interpolation as lerpCoords (kernel/bubble.cu:512-536):
// slerp(A, B, a) = sin((1-a)W)/sin W A + sin(aW)/sin W B, written so that
// nearby points keep full precision: slerp - C = cA dA + cB dB + k C with
// k = cA + cB - 1 = 2 sin((1-a)W/2) sin(aW/2) / cos(W/2).
__device__ __noinline__ f3 slerp_disp_far(float s0, float c0, f3 dA, f3 dB, float a) {
    const f3 e = dB - dA;
    const float W = farc_of_chord(len3(e));
    const float b = 1.0f - a;
    const float isW = 1.0f / fsinc(W);
    const float cA = b * fsinc(b * W) * isW;
    const float cB = a * fsinc(a * W) * isW;
    const float k = 0.5f * a * b * W * W * fsinc(0.5f * b * W) * fsinc(0.5f * a * W) /
                    fcos_small(0.5f * W);
    const f3 C = {s0, 0.0f, c0};
    return cA * dA + cB * dB + k * C;
}

// For chords up to 1/4 (W < 0.253) the coefficients are power series in
// u = W^2 (from the squared chord c2: u = c2 + c2^2/12 + c2^3/90 + c2^4/560):
//   cB / a = 1 + (1-a^2) u/6 + (1-a^2)(7-3a^2) u^2/360
//              + (1-a^2)(3a^4-18a^2+31) u^3/15120,
//   cA as cB with a -> 1-a,
//   k / (p u / 2) = 1 + (1+p) u/12 + (p^2+3p+3) u^2/360
//                   + (p^3+6p^2+17p+17) u^3/20160,   p = a (1-a);
// the truncation is below 1e-9 relative.  For chords up to 1/16 (u < 0.004)
// the u^2 and u^3 terms change the coefficients by less than 1e-9 and are
// dropped, and for chords up to 2^-6.5 (u < 1.3e-4) the u^2 term of k and
// c2^2/12 in u too.  Farther points take the exact formula out of line.
__device__ __forceinline__ f3 slerp_disp_inl(float s0, float c0, f3 dA, f3 dB, float a) {
    const f3 e = dB - dA;
    const float c2 = dot3(e, e);
    if (c2 > 0.0625f) return slerp_disp_far(s0, c0, dA, dB, a);
    const float b = 1.0f - a;
    if (c2 <= 0x1p-13f) {
        // chords up to 2^-6.5 (a grid step of 512 rows and finer): u = c2 and
        // first order in u (the dropped terms are below 2e-10 absolute)
        const float cB = a * fmaf(c2 * fmaf(-a, a, 1.0f), 1.0f / 6.0f, 1.0f);
        const float cA = b * fmaf(c2 * fmaf(-b, b, 1.0f), 1.0f / 6.0f, 1.0f);
        const float k = 0.5f * a * b * c2;
        const f3 C = {s0, 0.0f, c0};
        return cA * dA + cB * dB + k * C;
    }
    if (c2 <= 0.00390625f) {
        const float u = c2 * fmaf(c2, 1.0f / 12.0f, 1.0f);
        const float a2 = a * a, b2 = b * b;
        const float cB = a * fmaf(u * (1.0f - a2), fmaf(u, fmaf(a2, -3.0f, 7.0f) * (1.0f / 360.0f), 1.0f / 6.0f), 1.0f);
        const float cA = b * fmaf(u * (1.0f - b2), fmaf(u, fmaf(b2, -3.0f, 7.0f) * (1.0f / 360.0f), 1.0f / 6.0f), 1.0f);
        const float p = a * b;
        const float k = 0.5f * p * u * fmaf(u, (1.0f + p) * (1.0f / 12.0f), 1.0f);
        const f3 C = {s0, 0.0f, c0};
        return cA * dA + cB * dB + k * C;
    }
    const float u = c2 * fmaf(c2, fmaf(c2, fmaf(c2, 1.0f / 560.0f, 1.0f / 90.0f), 1.0f / 12.0f), 1.0f);
    const float a2 = a * a, b2 = b * b;
    const float pa = fmaf(u, fmaf(u, fmaf(a2, fmaf(a2, 3.0f, -18.0f), 31.0f) * (1.0f / 15120.0f),
                                  fmaf(a2, -3.0f, 7.0f) * (1.0f / 360.0f)),
                          1.0f / 6.0f);
    const float pb = fmaf(u, fmaf(u, fmaf(b2, fmaf(b2, 3.0f, -18.0f), 31.0f) * (1.0f / 15120.0f),
                                  fmaf(b2, -3.0f, 7.0f) * (1.0f / 360.0f)),
                          1.0f / 6.0f);
    const float cB = a * fmaf(u * (1.0f - a2), pa, 1.0f);
    const float cA = b * fmaf(u * (1.0f - b2), pb, 1.0f);
    const float p = a * b;
    const float pk = fmaf(u, fmaf(u, fmaf(p, fmaf(p, fmaf(p, 1.0f, 6.0f), 17.0f), 17.0f) *
                                      (1.0f / 20160.0f),
                                  fmaf(p, fmaf(p, 1.0f, 3.0f), 3.0f) * (1.0f / 360.0f)),
                          (1.0f + p) * (1.0f / 12.0f));
    const float k = 0.5f * p * u * fmaf(u, pk, 1.0f);
    const f3 C = {s0, 0.0f, c0};
    return cA * dA + cB * dB + k * C;
}

__device__ SB_GEOM_INLINE f3 slerp_disp(float s0, float c0, f3 dA, f3 dB, float a) {
    return slerp_disp_inl(s0, c0, dA, dB, a);
}

// ---------------------------------------------------------------------------
// Stencils
// ---------------------------------------------------------------------------

// Geometric unfolding of a raw position across the poles (validateCoord,
// kernel/bubble.cu:116-137, in raw coordinates).  Returns true when flipped.
__device__ __forceinline__ bool unfold(int nT, int& bi, float& ox, int& bj) {
    if ((float)bi + ox < 0.0f) {
        bi = -bi;
        ox = -ox;
        bj += nT;
        return true;
    }
    if ((float)(bi - nT) + ox > 0.0f) {
        bi = 2 * nT - bi;
        ox = -ox;
        bj += nT;
        return true;
    }
    return false;
}

// Row and column stencil of a cell-centred grid (rows at raw theta i + 0.5,
// columns at raw phi j).  Rows -1 and nT are the across-pole reflections of
// rows 0 and nT-1 (azimuth + pi); `neg` marks them for vector fields.
struct CStencil {
    int r0, r1;        // physical rows
    int c00, c01;      // columns of the lower row
    int c10, c11;      // columns of the upper row
    bool v0, v1;       // lower / upper row is an across-pole reflection
    float a, b;        // theta / phi fractions
    bool flipped;
};

// Bound offsets to a finite range (NaN maps to the bound) so that the
// float-to-int conversions below never overflow.
__device__ __forceinline__ float bound_off(float v, float lim) {
    return fmaxf(fminf(v, lim), -lim);
}

__device__ __forceinline__ CStencil centred_stencil(const SbGrid& g, Pos q, float colOff) {
    CStencil s;
    int bi = q.bi, bj = q.bj;
    float ox = bound_off(q.ox, 4.0f * g.nT);
    q.oy = bound_off(q.oy, 4.0f * g.nP);
    s.flipped = unfold(g.nT, bi, ox, bj);
    const float t = ox - 0.5f;
    const float kf = floorf(t);
    int lo = bi + (int)kf;
    s.a = t - kf;
    // positions lie in [0, nT] after unfolding; the clamp keeps every access
    // in bounds even for non-finite input
    lo = max(-1, min(lo, g.nT - 1));
    const float ty = q.oy - colOff;
    const float kj = floorf(ty);
    const int j0 = (bj + (int)kj) & g.maskP;
    const int j1 = (j0 + 1) & g.maskP;
    s.b = ty - kj;
    const int nT = g.nT;
    // lower row
    if (lo < 0) {
        s.r0 = 0; s.v0 = true;
        s.c00 = (j0 + nT) & g.maskP; s.c01 = (j1 + nT) & g.maskP;
    } else {
        s.r0 = lo; s.v0 = false; s.c00 = j0; s.c01 = j1;
    }
    const int hi = lo + 1;
    if (hi > nT - 1) {
        s.r1 = nT - 1; s.v1 = true;
        s.c10 = (j0 + nT) & g.maskP; s.c11 = (j1 + nT) & g.maskP;
    } else {
        s.r1 = hi; s.v1 = false; s.c10 = j0; s.c11 = j1;
    }
    return s;
}

// Scalar or u_phi sample (sampleCentered kernel/bubble.cu:320-376, sampleVPhi
// 178-240).  VEC: across-pole rows and flipped positions change sign.
template <bool VEC>
__device__ __forceinline__ float sample_centred(const SbGrid& g, const float* __restrict__ f,
                                                Pos q, float colOff) {
    const CStencil s = centred_stencil(g, q, colOff);
    const int nP = g.nP;
    const float f00 = f[s.r0 * nP + s.c00], f01 = f[s.r0 * nP + s.c01];
    const float f10 = f[s.r1 * nP + s.c10], f11 = f[s.r1 * nP + s.c11];
    float l = lerp_raw(f00, f01, s.b);
    float u = lerp_raw(f10, f11, s.b);
    if (VEC) {
        if (s.v0) l = -l;
        if (s.v1) u = -u;
    }
    float r = lerp_raw(l, u, s.a);
    if (isnan(r)) {  // a NaN sample: the reference's NaN-skipping lerps
        l = blerp(f00, f01, s.b);
        u = blerp(f10, f11, s.b);
        if (VEC) {
            if (s.v0) l = -l;
            if (s.v1) u = -u;
        }
        r = blerp(l, u, s.a);
    }
    if (VEC && s.flipped) r = -r;
    return r;
}

__device__ __forceinline__ float sample_scalar(const SbGrid& g, const float* __restrict__ f, Pos q) {
    return sample_centred<false>(g, f, q, 0.0f);
}
__device__ __forceinline__ float sample_uphi(const SbGrid& g, const float* __restrict__ f, Pos q) {
    return sample_centred<true>(g, f, q, -0.5f);
}

// u_theta sample (sampleVTheta, kernel/bubble.cu:247-313).  Rows sit at raw
// theta i + 1, i = 0..nT-2; next to a pole the nearest samples are the row and
// its across-pole reflection two cells away.
__device__ __forceinline__ float sample_utheta(const SbGrid& g, const float* __restrict__ f, Pos q) {
    int bi = q.bi, bj = q.bj;
    float ox = bound_off(q.ox, 4.0f * g.nT);
    q.oy = bound_off(q.oy, 4.0f * g.nP);
    const bool flipped = unfold(g.nT, bi, ox, bj);
    const int nT = g.nT, nP = g.nP;
    const float kf = floorf(ox);
    int lo = bi - 1 + (int)kf;  // row coordinate s = raw - 1
    float a = ox - kf;
    lo = max(-1, min(lo, nT - 1));
    const float ty = q.oy;
    const float kj = floorf(ty);
    const int j0 = (bj + (int)kj) & g.maskP;
    const int j1 = (j0 + 1) & g.maskP;
    const float b = ty - kj;
    float r;
    if (lo < 0) {
        // between the reflection of row 0 (s = -2) and row 0 (s = 0)
        const float s = (float)lo + a;  // in [-1, 0)
        const float w = 0.5f * (s + 2.0f);
        const float l = -blerp(f[(j0 + nT) & g.maskP], f[(j1 + nT) & g.maskP], b);
        const float u = blerp(f[j0], f[j1], b);
        r = blerp(l, u, w);
    } else if (lo >= nT - 2) {
        // between row nT-2 (s = nT-2) and its reflection (s = nT)
        const float s = (float)(lo - (nT - 2)) + a;  // in [0, 1]
        const int row = (nT - 2) * nP;
        const float l = blerp(f[row + j0], f[row + j1], b);
        const float u = -blerp(f[row + ((j0 + nT) & g.maskP)], f[row + ((j1 + nT) & g.maskP)], b);
        r = blerp(l, u, 0.5f * s);
    } else {
        r = bilerp(f[lo * nP + j0], f[lo * nP + j1], f[(lo + 1) * nP + j0], f[(lo + 1) * nP + j1],
                   a, b);
    }
    return flipped ? -r : r;
}

// Displacement, in the cell frame F, of the map point stored for cell
// (r, c) (D: its displacement in its own frame).  With Delta = (c - F.bj) h
// the rotation from the entry's frame to F's and C_r, C_F the two centres:
// P - C_F = R(Delta) (C_r + D) - C_F, evaluated as sums of small terms
// (each product of two precise factors) so that the result keeps ~1e-7 of
// its own size next to the poles too.
__device__ __forceinline__ f3 map_point(const SbGrid& g, const Frame& F, float4 D, int r, int c) {
    const float4 R = __ldg(&g.rowtab[r]);
    const int dc = ((c - F.bj + g.nT) & g.maskP) - g.nT;
    const float2 t = __ldg(&g.rottab[dc + g.nT]);  // sin(Delta), cos(Delta) - 1
    const float ds = (R.x - F.s0) + (R.y - F.s0lo);  // s_r - s_F
    const float dz = (R.z - F.c0) + (R.w - F.c0lo);  // c_r - c_F
    f3 P;
    P.x = ds + D.x + t.y * R.x + t.y * D.x - t.x * D.y;
    P.y = t.x * R.x + t.x * D.x + D.y + t.y * D.y;
    P.z = dz + D.z;
    return P;
}

// Characteristic-map lookup (sampleMapping, kernel/bubble.cu:539-606): the
// four map points around q, slerped along phi on each row and then along
// theta.  The result is a displacement in the cell frame F.  The lookup for
// a stencil already computed at the query point (the same cell-centred
// stencil also serves scalar samples there).
__device__ SB_GEOM_INLINE f3 map_at_stencil(const SbGrid& g, const float4* __restrict__ map,
                                             const Frame& F, const CStencil& s) {
    const int nP = g.nP;
    if (!(s.v0 | s.v1)) {
        // Rows r0, r0 + 1 and columns c00, c00 + 1: the four points are
        // formed in the frame of entry (r0, c00), where that entry needs no
        // conversion, the next row adds the difference of the row centres and
        // the next column is a rotation by one grid step (a uniform table
        // entry); the interpolated point is converted to F once.
        const float4 Dll = map[s.r0 * nP + s.c00], Dlr = map[s.r0 * nP + s.c01];
        const float4 Dhl = map[s.r1 * nP + s.c10], Dhr = map[s.r1 * nP + s.c11];
        const float4 R0 = __ldg(&g.rowtab[s.r0]), R1 = __ldg(&g.rowtab[s.r1]);
        const float2 t = __ldg(&g.rottab[g.nT + 1]);  // sin h, cos h - 1
        const float ds = (R1.x - R0.x) + (R1.y - R0.y), dz = (R1.z - R0.z) + (R1.w - R0.w);
        const f3 ll = {Dll.x, Dll.y, Dll.z};
        const f3 lr = {Dlr.x + t.y * R0.x + t.y * Dlr.x - t.x * Dlr.y,
                       t.x * R0.x + t.x * Dlr.x + Dlr.y + t.y * Dlr.y, Dlr.z};
        const f3 hl = {ds + Dhl.x, Dhl.y, dz + Dhl.z};
        const f3 hr = {ds + Dhr.x + t.y * R1.x + t.y * Dhr.x - t.x * Dhr.y,
                       t.x * R1.x + t.x * Dhr.x + Dhr.y + t.y * Dhr.y, dz + Dhr.z};
        const f3 lo = slerp_disp(R0.x, R0.z, ll, lr, s.b);
        const f3 hi = slerp_disp(R0.x, R0.z, hl, hr, s.b);
        const f3 m = slerp_disp(R0.x, R0.z, lo, hi, s.a);
        return map_point(g, F, make_float4(m.x, m.y, m.z, 0.0f), s.r0, s.c00);
    }
    const f3 ll = map_point(g, F, map[s.r0 * nP + s.c00], s.r0, s.c00);
    const f3 lr = map_point(g, F, map[s.r0 * nP + s.c01], s.r0, s.c01);
    const f3 hl = map_point(g, F, map[s.r1 * nP + s.c10], s.r1, s.c10);
    const f3 hr = map_point(g, F, map[s.r1 * nP + s.c11], s.r1, s.c11);
    const f3 lo = slerp_disp(F.s0, F.c0, ll, lr, s.b);
    const f3 hi = slerp_disp(F.s0, F.c0, hl, hr, s.b);
    return slerp_disp(F.s0, F.c0, lo, hi, s.a);
}

__device__ __forceinline__ f3 sample_map(const SbGrid& g, const float4* __restrict__ map,
                                         const Frame& F, Pos q) {
    return map_at_stencil(g, map, F, centred_stencil(g, q, 0.0f));
}

// Velocity (u_theta, u_phi) at an arbitrary position.
__device__ __forceinline__ void velocity_at(const SbGrid& g, const float* __restrict__ uth,
                                            const float* __restrict__ uph, Pos q, float& vt,
                                            float& vp) {
    vt = sample_utheta(g, uth, q);
    vp = sample_uphi(g, uph, q);
}

// Local basis at the point P (unnormalised), as the reference derives it from
// (acos(Pz), atan2(Py, Px)) (kernel/bubble.cu:462-471).
// Reciprocal square roots in place of square roots and quotients (within
// 2 ulp: the basis weights velocity samples).
__device__ __forceinline__ void basis_at(f3 P, f3& eth, f3& eph) {
    const float rho2 = P.x * P.x + P.y * P.y;
    const float ir = rsqrtf(rho2 + P.z * P.z);
    float cph = 1.0f, sph = 0.0f, irho = 0.0f;
    if (rho2 > 0.0f) {
        irho = rsqrtf(rho2);
        cph = P.x * irho;
        sph = P.y * irho;
    }
    const float ct = P.z * ir, st = rho2 * irho * ir;
    eth = {ct * cph, ct * sph, -st};
    eph = {-sph, cph, 0.0f};
}

// Result of a great-circle backtrace from a frame base.
struct Trace {
    f3 d;        // displacement of the departure point
    f3 u_, v_;   // final great-circle direction and its normal
    float sd, cd;  // sin / cos of the final arc step
    float fail;    // the zero or NaN speed that stopped the trace
    bool moved;
};

// traceGreatCircle (kernel/bubble.cu:416-506) from the frame base with the
// base velocity (gt, gp) already known.  dt > 0 traces backward.  rk2: the
// direction is first corrected with the velocity at the half step (the
// scalar traces always; the velocity advection under RUNGE_KUTTA,
// bubble.cu:689-730).
// FAST: the half-step position that picks the mid-point velocity samples
// comes from pos_from_disp_fast (the velocity advection); the map update
// keeps the exact quotients.
template <bool FAST = false>
__device__ __forceinline__ Trace trace_gc(const SbGrid& g, const float* __restrict__ uth,
                                          const float* __restrict__ uph, const Frame& F,
                                          float gt, float gp, float dt, bool rk2 = true) {
    Trace T;
    T.moved = false;
    T.fail = 0.0f;
    T.d = {0.0f, 0.0f, 0.0f};
    const f3 w = {F.s0, 0.0f, F.c0};
    const f3 eth = {F.c0, 0.0f, -F.s0};
    const f3 eph = {0.0f, 1.0f, 0.0f};
    f3 u = gt * eth + gp * eph;
    float un2 = dot3(u, u);
    if (!(un2 > 0.0f)) { T.fail = sqrtf(un2); return T; }
    float iun = rsqrtf(un2);
    float un = un2 * iun;
    f3 u_ = iun * u;
    f3 v_ = cross3(w, u_);
    float dS, sd, sh, ch, cdm1;
    if (rk2) {
        dS = -0.5f * un * dt;
        fsincos(0.5f * dS, &sh, &ch);
        sd = 2.0f * sh * ch;
        cdm1 = -2.0f * sh * sh;
        const f3 dmid = sd * u_ + cdm1 * w;
        const f3 midx = w + dmid;
        const Pos qm = FAST ? pos_from_disp_fast(F, dmid, g.invh, g.nT)
                            : pos_from_disp(F, dmid, g.invh, g.nT);
        float mt, mp;
        velocity_at(g, uth, uph, qm, mt, mp);
        f3 beth, beph;
        basis_at(midx, beth, beph);
        const f3 mu = mt * beth + mp * beph;
        const f3 uCircleMid = (1.0f + cdm1) * u_ - sd * w;
        const f3 vCircleMid = cross3(midx, uCircleMid);
        const float mgt = dot3(mu, vCircleMid);
        const float mgp = dot3(mu, uCircleMid);
        u = mgp * u_ + mgt * v_;
        un2 = dot3(u, u);
        if (!(un2 > 0.0f)) { T.fail = sqrtf(un2); return T; }
        iun = rsqrtf(un2);
        un = un2 * iun;
        u_ = iun * u;
        v_ = cross3(w, u_);
    }
    dS = -un * dt;
    fsincos(0.5f * dS, &sh, &ch);
    sd = 2.0f * sh * ch;
    cdm1 = -2.0f * sh * sh;
    T.d = sd * u_ + cdm1 * w;
    T.u_ = u_;
    T.v_ = v_;
    T.sd = sd;
    T.cd = 1.0f + cdm1;
    T.moved = true;
    return T;
}

// Bilinear stencil of a cell-centred scalar at q (flat indices), so that
// several fields sampled at one position share the index work.
struct SStencil {
    int i00, i01, i10, i11;
    float a, b;
};

__device__ __forceinline__ SStencil sstencil_of(const SbGrid& g, const CStencil& c) {
    SStencil s;
    s.i00 = c.r0 * g.nP + c.c00;
    s.i01 = c.r0 * g.nP + c.c01;
    s.i10 = c.r1 * g.nP + c.c10;
    s.i11 = c.r1 * g.nP + c.c11;
    s.a = c.a;
    s.b = c.b;
    return s;
}

__device__ __forceinline__ SStencil scalar_stencil(const SbGrid& g, Pos q) {
    return sstencil_of(g, centred_stencil(g, q, 0.0f));
}

// A thickness or surfactant field in its storage type T.  FP32 fields hold
// the values.  BF16 fields hold the deviation from a per-field base value
// (the field's mean at upload, itself a BF16 number, so that 0 and the base
// are exact): loads return base + deviation in FP32, stores round
// value - base to nearest even.  Fields of order one with perturbations of
// a few percent keep about three significant digits of the perturbation
// instead of the 2^-8 absolute spacing of BF16 values near one.
template <class T>
__device__ __forceinline__ float ld_s(const SbScalar* p, int i, float base) {
    (void)base;
    return reinterpret_cast<const float*>(p)[i];
}
template <>
__device__ __forceinline__ float ld_s<__nv_bfloat16>(const SbScalar* p, int i, float base) {
    return base + __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(p)[i]);
}
template <class T>
__device__ __forceinline__ void st_s(SbScalar* p, int i, float v, float base) {
    (void)base;
    reinterpret_cast<float*>(p)[i] = v;
}
template <>
__device__ __forceinline__ void st_s<__nv_bfloat16>(SbScalar* p, int i, float v, float base) {
    reinterpret_cast<__nv_bfloat16*>(p)[i] = __float2bfloat16_rn(v - base);
}
// Element copy between two fields of the same base (exact).
template <class T>
__device__ __forceinline__ void cp_s(SbScalar* dst, const SbScalar* src, int i) {
    reinterpret_cast<T*>(dst)[i] = reinterpret_cast<const T*>(src)[i];
}

template <class T>
__device__ __forceinline__ float gather_s(const SbScalar* f, const SStencil& s, float base) {
    return bilerp(ld_s<T>(f, s.i00, base), ld_s<T>(f, s.i01, base), ld_s<T>(f, s.i10, base),
                  ld_s<T>(f, s.i11, base), s.a, s.b);
}

__device__ __forceinline__ float gather(const float* __restrict__ f, const SStencil& s) {
    return bilerp(f[s.i00], f[s.i01], f[s.i10], f[s.i11], s.a, s.b);
}

// Map lookups at the five MULTISAMPLE points of a cell, c + (-1/4, -1/4),
// (+1/4, -1/4), (-1/4, +1/4), (+1/4, +1/4), c (kernel/bubble.cu:981-993),
// in that order.  Their stencils all lie in the 3 x 3 neighbourhood of the
// cell, so its nine map points are converted once (rows -1 and nTheta are
// the across-pole reflections, as in the single lookup).  Results are
// displacements in the cell's frame F.
__device__ __forceinline__ void sample_map_multi5(const SbGrid& g, const float4* __restrict__ map,
                                                  const Frame& F, f3 out[5]) {
    const int nT = g.nT, nP = g.nP, i = F.bi, j = F.bj;
    f3 P[3][3];
#pragma unroll
    for (int dr = -1; dr <= 1; ++dr) {
        int row = i + dr, shift = 0;
        if (row < 0) { row = 0; shift = nT; }
        if (row > nT - 1) { row = nT - 1; shift = nT; }
#pragma unroll
        for (int dc = -1; dc <= 1; ++dc) {
            const int col = (j + dc + shift) & g.maskP;
            P[dr + 1][dc + 1] = map_point(g, F, map[row * nP + col], row, col);
        }
    }
    // (theta, phi) = (-1/4, -1/4): rows i-1, i; cols j-1, j; fractions 3/4
    out[0] = slerp_disp_inl(F.s0, F.c0, slerp_disp_inl(F.s0, F.c0, P[0][0], P[0][1], 0.75f),
                        slerp_disp_inl(F.s0, F.c0, P[1][0], P[1][1], 0.75f), 0.75f);
    out[1] = slerp_disp_inl(F.s0, F.c0, slerp_disp_inl(F.s0, F.c0, P[1][0], P[1][1], 0.75f),
                        slerp_disp_inl(F.s0, F.c0, P[2][0], P[2][1], 0.75f), 0.25f);
    out[2] = slerp_disp_inl(F.s0, F.c0, slerp_disp_inl(F.s0, F.c0, P[0][1], P[0][2], 0.25f),
                        slerp_disp_inl(F.s0, F.c0, P[1][1], P[1][2], 0.25f), 0.75f);
    out[3] = slerp_disp_inl(F.s0, F.c0, slerp_disp_inl(F.s0, F.c0, P[1][1], P[1][2], 0.25f),
                        slerp_disp_inl(F.s0, F.c0, P[2][1], P[2][2], 0.25f), 0.25f);
    out[4] = P[1][1];
}

__device__ __forceinline__ Frame cell_frame(const SbGrid& g, int i, int j) {
    Frame F;
    F.bi = i; F.bj = j; F.fi = 0.5f; F.fj = 0.0f;
    const float4 R = __ldg(&g.rowtab[i]);
    F.s0 = R.x; F.s0lo = R.y; F.c0 = R.z; F.c0lo = R.w;
    return F;
}

__device__ __forceinline__ Pos frame_pos(const Frame& F, float dth, float dph) {
    Pos q;
    q.bi = F.bi; q.bj = F.bj; q.ox = F.fi + dth; q.oy = F.fj + dph;
    return q;
}

}  // namespace sb
