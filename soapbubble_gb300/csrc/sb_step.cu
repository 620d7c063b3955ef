// Step kernels of the soap-bubble solver (everything except the implicit
// solve).  One thread per grid cell; a warp covers 32 consecutive phi cells
// of one theta row, so direct loads are coalesced and the sampler gathers of
// nearby departure points hit L1/L2.
//
// Stage map against the reference (kernel/solver.cu:260-292):
//   k_advect_maps  updateForward/updateBackward (bubble.cu:609-633, 1049-1116),
//                  advectionCentered for gamma (910-931), airFlowU/V (2301-2380)
//   k_velocity     advectionVSphereTheta/PhiKernel (639-904)
//   k_bimocq       advectionCenteredBimocq (967-1013)
//   k_assemble     concentrationLinearSystemKernel (1301-1473)
//   k_post         divergenceKernel_fromGamma, applyforcevel{theta,phi},
//                  applyforceThickness, substractPitched (1276-1295, 1819-1935,
//                  2041-2078); the VISCOUS forces (1218-1269, 1512-1816,
//                  1940-2038) in k_assemble and k_post
//   k_accum        accumulateChangesCentered x2 (2081-2114),
//                  estimateDistortionKernel + maxAbs (1131-1168, 1019-1043) and
//                  the error of correctCentered1 (2180-2216)
//   k_reinit       reInitializeMapping, correctCentered2 (2218-2280, 2509-2564)
// van der Waals is identically zero in the reference (W1 = W2 = 0,
// bubble.cu:2633-2638) and is folded out.

#include "sb_device.cuh"
#include "sb_internal.h"
#include "sb_scale.cuh"
#include "sb_sync.cuh"

namespace sb {

namespace {

constexpr int kBlock = 128;

__constant__ float kW5[5] = {0.125f, 0.125f, 0.125f, 0.125f, 0.5f};

__device__ __forceinline__ Frame face_frame_uphi(const SbGrid& g, int i, int j) {
    Frame F;
    F.bi = i; F.bj = j; F.fi = 0.5f; F.fj = -0.5f;
    F.s0 = g.sin_c[i]; F.c0 = g.cos_c[i];
    F.s0lo = 0.0f; F.c0lo = 0.0f;
    return F;
}

__device__ __forceinline__ Frame face_frame_utheta(const SbGrid& g, int i, int j) {
    Frame F;
    F.bi = i + 1; F.bj = j; F.fi = 0.0f; F.fj = 0.0f;
    F.s0 = g.sin_e[i + 1]; F.c0 = g.cos_e[i + 1];
    F.s0lo = 0.0f; F.c0lo = 0.0f;
    return F;
}

__device__ __forceinline__ Pos pos_of(const Frame& F, const Trace& T, const SbGrid& g) {
    return T.moved ? pos_from_disp(F, T.d, g.invh, g.nT) : frame_pos(F, 0.0f, 0.0f);
}

// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void advect_maps_cell(const SbGrid& g, const SbPhys& ph, const SbFields& f, int cur,
                                          int idx) {
    (void)cur;
    if (idx == 0) {
        f.stats->distortion_bits = 0u;
        f.stats->reinit = 0;
        f.stats->broken_cells = 0;
    }
    const int i = idx >> g.logP, j = idx & g.maskP;
    const float dt = f.step->dt;
    const Frame F = cell_frame(g, i, j);
    const Pos q0 = frame_pos(F, 0.0f, 0.0f);
    float gt, gp;
    velocity_at(g, f.uth, f.uph, q0, gt, gp);

    if (ph.plain_adv) {
        // advectionAllCentered (bubble.cu:937-961): thickness and gamma at the
        // backward trace; the maps are not used
        const Trace Tb = trace_gc(g, f.uth, f.uph, F, gt, gp, dt);
        const SStencil sb = sstencil_of(g, centred_stencil(g, pos_of(F, Tb, g), 0.0f));
        f.eta_adv[idx] = gather_s<T>(f.eta, sb, ph.base_eta);
        f.gam_adv[idx] = gather_s<T>(f.gam, sb, ph.base_gam);
    } else {
        // forward map: trace forward in time (negative step), sample the old map
        const Trace Tf = trace_gc(g, f.uth, f.uph, F, gt, gp, -dt);
        const f3 df = sample_map(g, f.fwd[cur], F, pos_of(F, Tf, g));
        f.fwd[cur ^ 1][idx] = make_float4(df.x, df.y, df.z, 0.0f);  // in the cell's own frame

        // backward map and gamma share the backward trace
        const Trace Tb = trace_gc(g, f.uth, f.uph, F, gt, gp, dt);
        const CStencil cb = centred_stencil(g, pos_of(F, Tb, g), 0.0f);
        const f3 db = map_at_stencil(g, f.bwd[cur], F, cb);
        f.bwd[cur ^ 1][idx] = make_float4(db.x, db.y, db.z, 0.0f);
        f.gam_adv[idx] = gather_s<T>(f.gam, sstencil_of(g, cb), ph.base_gam);
    }

    // air flow = initial wind + corridor(t); NaN -> 0
    const float wg = f.step->windg;
    float ua = f.uair_init[idx] + wg * f.corr_u[idx];
    f.uair[idx] = isnan(ua) ? 0.0f : ua;
    if (i < g.nT - 1) {
        float va = f.vair_init[idx] + wg * f.corr_v[idx];
        f.vair[idx] = isnan(va) ? 0.0f : va;
    }
}

// Velocity self-advection with parallel transport (RUNGE_KUTTA path).
__device__ __forceinline__ float advect_velocity(const SbGrid& g, const float* __restrict__ uth,
                                                 const float* __restrict__ uph, const Frame& F,
                                                 float gt, float gp, float dt, bool outPhi,
                                                 bool rk2) {
    const f3 w = {F.s0, 0.0f, F.c0};
    // a zero or NaN speed stops the trace; the reference then writes that
    // speed (bubble.cu:689-692, 727-730)
    const Trace T = trace_gc<true>(g, uth, uph, F, gt, gp, dt, rk2);
    if (!T.moved) return T.fail;
    const f3 P = w + T.d;
    const Pos qp = pos_from_disp_fast(F, T.d, g.invh, g.nT);
    float pt, pp;
    velocity_at(g, uth, uph, qp, pt, pp);
    f3 beth, beph;
    basis_at(P, beth, beph);
    const f3 pu = pt * beth + pp * beph;
    const f3 uCircleP = T.cd * T.u_ - T.sd * w;
    const f3 vCircleP = cross3(P, uCircleP);
    const float a = dot3(pu, vCircleP);
    const float b = dot3(pu, uCircleP);
    const f3 pu2 = b * T.u_ + a * T.v_;
    if (outPhi) return pu2.y;                       // e_phi = (0, 1, 0)
    return pu2.x * F.c0 - pu2.z * F.s0;             // e_theta = (c0, 0, -s0)
}

__device__ __forceinline__ void velocity_cell(const SbGrid& g, const SbPhys& ph, const SbFields& f, int cur,
                                          int idx) {
    (void)cur;
    const int i = idx >> g.logP, j = idx & g.maskP;
    const float dt = f.step->dt;
    {
        const Frame F = face_frame_uphi(g, i, j);
        const float gp = f.uph[idx];
        const float gt = sample_utheta(g, f.uth, frame_pos(F, 0.0f, 0.0f));
        f.uph_adv[idx] = advect_velocity(g, f.uth, f.uph, F, gt, gp, dt, true, !ph.single_step);
    }
    if (i < g.nT - 1) {
        const Frame F = face_frame_utheta(g, i, j);
        const float gt = f.uth[idx];
        const float gp = sample_uphi(g, f.uph, frame_pos(F, 0.0f, 0.0f));
        f.uth_adv[idx] = advect_velocity(g, f.uth, f.uph, F, gt, gp, dt, false, !ph.single_step);
    }
}

// BIMOCQ thickness: compose the new backward map with the previous one and
// blend the two reconstructions (MULTISAMPLE, 5 samples).
template <class T>
__device__ __forceinline__ void bimocq_cell(const SbGrid& g, const SbPhys& ph, const SbFields& f, int cur,
                                          int idx) {
    (void)cur;
    if (ph.plain_adv) return;  // thickness advected by k_advect_maps
    const int i = idx >> g.logP, j = idx & g.maskP;
    const float be = ph.base_eta;
    if (ld_s<T>(f.eta, idx, be) == 0.0f) {
        f.eta_adv[idx] = 0.0f;
        return;
    }
    const Frame F = cell_frame(g, i, j);
    const float blend = ph.blend;
    f3 d1s[5];
    sample_map_multi5(g, f.bwd[cur ^ 1], F, d1s);
    float attrib = 0.0f;
#pragma unroll 2
    for (int k = 0; k < 5; ++k) {
        const CStencil c1 = centred_stencil(g, pos_from_disp_fast(F, d1s[k], g.invh, g.nT), 0.0f);
        const f3 d2 = map_at_stencil(g, f.bwdprev, F, c1);
        const Pos q2 = pos_from_disp_fast(F, d2, g.invh, g.nT);
        const SStencil s1 = sstencil_of(g, c1);
        const SStencil s2 = scalar_stencil(g, q2);
        const float sDelta = gather(f.eta_delta, s1);
        attrib += (1.0f - blend) * kW5[k] *
                  (gather_s<T>(f.eta_initL, s2, be) + sDelta + gather(f.eta_deltaL, s2));
        attrib += blend * kW5[k] * (gather_s<T>(f.eta_init, s1, be) + sDelta);
    }
    f.eta_adv[idx] = fmaxf(0.0f, attrib);
}

// A cell at its maximum concentration or without film (kernel/bubble.cu:
// 1317; thr: SbPhys::gthr, the FP32 form of gmax - 1e-7).
__device__ __forceinline__ bool is_broken(float gamma, float eta, float thr) {
    return gamma > thr || eta == 0.0f;
}

// VISCOUS variant (include/header.cuh:98, off in the reference's build): the
// film's viscous stress forces fv on the u_theta faces (gravity included) and
// fu on the u_phi faces, from the advected velocities and thickness.  They
// enter the system's right-hand side in place of the gravity term and the
// velocity update.  k_assemble and k_post evaluate them where they need them
// instead of storing them: the same function on the same inputs gives both
// kernels the same values, and out-of-line calls keep the default path's
// register allocation free of them.

// div u at cell (i, j) (divergenceKernel, bubble.cu:1218-1269).
__device__ __forceinline__ float vel_div(const SbGrid& g, const SbFields& f, int i, int j) {
    const int nP = g.nP, c = i * nP + j;
    const float uW = f.uph_adv[c], uE = f.uph_adv[i * nP + ((j + 1) & g.maskP)];
    const float vN = i != 0 ? f.uth_adv[c - nP] : 0.0f;
    const float vS = i != g.nT - 1 ? f.uth_adv[c] : 0.0f;
    const float factor = (1.0f / g.sin_c[i]) * g.invh;
    return factor * (vS * g.sin_e[i + 1] - vN * g.sin_e[i]) + g.invh * (uE - uW);
}

// helper_math.h's clamp(f, a, b) = fmaxf(a, fminf(f, b)).
__device__ __forceinline__ float clamp_force(float v) { return fmaxf(-0.1f, fminf(v, 0.1f)); }

// fv at u_theta face (i, j), i < nT - 1 (computeforcevelthetaKernel,
// bubble.cu:1512-1643).
__device__ __noinline__ float viscous_fv(const SbGrid& g, const SbPhys& ph, const SbFields& f,
                                         int i, int j) {
    const int nP = g.nP, mP = g.maskP;
    const int jW = (j - 1) & mP, jE = (j + 1) & mP, jO = (j + nP / 2) & mP;
    const int rN = i * nP, rS = rN + nP;
    const float* __restrict__ u = f.uph_adv;
    const float* __restrict__ v = f.uth_adv;
    const float* __restrict__ e = f.eta_adv;
    const float ih = g.invh;
    const float etaN = e[rN + j], etaS = e[rS + j];
    const float invEta = 2.0f / (etaN + etaS);
    if (isinf(invEta)) return __int_as_float(0x7fffffff);
    const float u0 = u[rN + j], u1 = u[rN + jE], u2 = u[rS + j], u3 = u[rS + jE];
    const float divN = vel_div(g, f, i, j), divS = vel_div(g, f, i + 1, j);
    const float div = 0.5f * (divN + divS);
    const float uPhi = 0.25f * (u0 + u1 + u2 + u3);
    const float pDpx = 0.25f * ih * (e[rN + jE] + e[rS + jE] - e[rN + jW] - e[rS + jW]);
    const float pDpy = ih * (etaS - etaN);
    const float v1 = v[rN + j], v3 = v[rN + jW], v4 = v[rN + jE];
    const float vPole = 0.5f * (v1 - v[rN + jO]);  // across the pole
    const float v0 = i != 0 ? v[rN - nP + j] : vPole;
    const float v2 = i != g.nT - 2 ? v[rS + j] : vPole;
    const float pvpy = 0.5f * ih * (v2 - v0);
    const float pvpyN = ih * (v1 - v0), pvpyS = ih * (v2 - v1);
    const float pvpx = 0.5f * ih * (v4 - v3);
    const float pupy = 0.5f * ih * (u2 + u3 - u0 - u1);
    const float pupx = 0.5f * ih * (u1 + u3 - u0 - u2);
    const float pupxy = ih * ih * (u0 + u3 - u1 - u2);
    const float pvpxx = ih * ih * (v3 + v4 - 2.0f * v1);
    const float sinT = g.sin_e[i + 1], cosT = g.cos_e[i + 1];
    const float cscT = 1.0f / sinT, cotT = cosT * cscT;
    const float s11N = 2.0f * (pvpyN + divN), s11S = 2.0f * (pvpyS + divS);
    const float s22 = -2.0f * (pvpy - 2.0f * div);
    const float s12 = cscT * pvpx + pupy - uPhi * cotT;
    // d/dtheta (sin theta sigma11) across the face's half-cells
    const float psspy = ih * (s11S * g.sin_c[i + 1] - s11N * g.sin_c[i]);
    const float pspx = cscT * pvpxx + pupxy - cotT * pupx;
    const float re = ph.re;
    const float f2 = re * cscT * invEta * pDpx * s12;
    const float f4 = re * invEta * pDpy * 2.0f * (div + pvpy);
    const float f5 = re * cscT * (psspy + pspx - cosT * s22);
    const float f7 = ph.gs * sinT;
    if (sinT < 0.1f) return f7;
    return clamp_force(f2 + f5 + f4) + f7;
}

// fu at u_phi face (i, j) (computeforcevelphiKernel_viscous,
// bubble.cu:1647-1816).
__device__ __noinline__ float viscous_fu(const SbGrid& g, const SbPhys& ph, const SbFields& f,
                                         int i, int j) {
    const int nP = g.nP, mP = g.maskP, nT = g.nT;
    const int jW = (j - 1) & mP, jO = (j + nP / 2) & mP, jWO = (jW + nP / 2) & mP;
    const int r = i * nP;
    const float* __restrict__ u = f.uph_adv;
    const float* __restrict__ v = f.uth_adv;
    const float* __restrict__ e = f.eta_adv;
    const float ih = g.invh;
    const float etaW = e[r + jW], etaE = e[r + j];
    const float invEta = 2.0f / (etaW + etaE);
    if (isinf(invEta)) return __int_as_float(0x7fffffff);
    float v0, v1, v2, v3;
    if (i != 0) {
        v0 = v[r - nP + jW];
        v1 = v[r - nP + j];
    } else {
        v0 = 0.5f * (v[jW] - v[jWO]);
        v1 = 0.5f * (v[j] - v[jO]);
    }
    if (i != nT - 1) {
        v2 = v[r + jW];
        v3 = v[r + j];
    } else {
        v2 = 0.5f * (v[r - nP + jW] - v[r - nP + jWO]);
        v3 = 0.5f * (v[r - nP + j] - v[r - nP + jO]);
    }
    const float divW = vel_div(g, f, i, jW), divE = vel_div(g, f, i, j);
    const float div = 0.5f * (divW + divE);
    const float pvpx = 0.5f * ih * (v1 + v3 - v0 - v2);
    const float pvpyW = ih * (v2 - v0), pvpyE = ih * (v3 - v1);
    const float pvpy = 0.5f * ih * (v2 + v3 - v0 - v1);
    const float u1 = u[r + j];
    float u3, u4, pupyN = 0.0f, pupyS = 0.0f;
    if (i != 0) {
        u3 = u[r - nP + j];
        pupyN = ih * (u1 - u3);
    } else {
        u3 = -u[r + jO];
    }
    if (i != nT - 1) {
        u4 = u[r + nP + j];
        pupyS = ih * (u4 - u1);
    } else {
        u4 = -u[r + jO];
    }
    const float pupy = 0.5f * ih * (u4 - u3);
    const float sinT = g.sin_c[i], cosT = g.cos_c[i];
    const float cscT = 1.0f / sinT, cotT = cosT * cscT;
    const float s12 = cscT * pvpx + pupy - u1 * cotT;
    const float pDpx = ih * (etaE - etaW);
    const float d0 = i != 0 ? e[r - nP + jW] : e[r + jWO];
    const float d2 = i != 0 ? e[r - nP + j] : e[r + jO];
    const float d1 = i != nT - 1 ? e[r + nP + jW] : e[r + jWO];
    const float d3 = i != nT - 1 ? e[r + nP + j] : e[r + jO];
    const float pDpy = 0.25f * ih * (d1 + d3 - d0 - d2);
    float uN = 0.5f * (u3 + u1), uS = 0.5f * (u1 + u4);
    if (i == 0) uN = 0.5f * (u1 - u3);
    if (i == nT - 1) uS = 0.5f * (u1 - u4);
    const float psspy = ih * (ih * (v0 + v3 - v1 - v2) + g.sin_e[i + 1] * pupyS -
                              g.sin_e[i] * pupyN - g.cos_e[i + 1] * uS + g.cos_e[i] * uN);
    const float s22W = 2.0f * (2.0f * divW - pvpyW), s22E = 2.0f * (2.0f * divE - pvpyE);
    const float pspx = ih * (s22E - s22W);
    const float re = ph.re;
    const float f2 = re * invEta * pDpy * s12;
    const float f4 = re * invEta * cscT * pDpx * 2.0f * (2.0f * div - pvpy);
    const float f5 = re * cscT * (psspy + pspx + cosT * s12);
    if (sinT < 0.1f) return 0.0f;
    return clamp_force(f2 + f4 + f5);
}

// Implicit surfactant system (paper eq. 26), assembled for the increment
// dx = gamma_new - gamma_adv so that FP32 keeps its precision:
//   (A dx)_c = dmass_c dx_c + sum_n w_cn (dx_c - dx_n)
// with dmass = sin(theta) / (dt gamma) and the positive couplings w_cn (the
// reference's off-diagonals with the sign flipped; its diagonal is dmass +
// sum w).  The right-hand side r = b - A gamma_adv is formed analytically:
// dmass gamma = sin(theta) / dt cancels the leading term of b, leaving
// r = -sinThetaDiv - sum w (gamma_c - gamma_n).  The couplings across the
// poles carry sin(0) and sin(pi) and vanish.  A broken cell (gamma at its
// maximum or no film) keeps gamma = gmax: its row is dx = 0 and the weight
// of its couplings moves into the neighbours' dmass, which keeps A
// symmetric positive definite with the same solution as the reference's
// identity row.  A cell with almost no surfactant (t = sin(theta) / (dt
// gamma) > 2^48) enters with its row and column scaled by a power of two
// (sb_scale.cuh).
// 128-bit accesses to four consecutive cells (the arena's arrays are
// 256-byte aligned and four-cell groups never straddle a row).
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ void ld4(const float2* p, float2 (&v)[4]) {
    const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
    v[0] = make_float2(a.x, a.y); v[1] = make_float2(a.z, a.w);
    v[2] = make_float2(b.x, b.y); v[3] = make_float2(b.z, b.w);
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <class T>
__device__ __forceinline__ void st4_s(SbScalar* p, int i, const float (&v)[4], float base) {
    (void)base;
    st4(reinterpret_cast<float*>(p) + i, v);
}
template <>
__device__ __forceinline__ void st4_s<__nv_bfloat16>(SbScalar* p, int i, const float (&v)[4], float base) {
    const __nv_bfloat162 a = __floats2bfloat162_rn(v[0] - base, v[1] - base);
    const __nv_bfloat162 b = __floats2bfloat162_rn(v[2] - base, v[3] - base);
    *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(p) + i) =
        make_uint2(*reinterpret_cast<const unsigned*>(&a), *reinterpret_cast<const unsigned*>(&b));
}

// One cell's inputs to its row of the system, loaded: the advected gamma
// and thickness of the cell and its four neighbours (across a pole the
// mirrored cell's thickness), the advected face velocities, the wind at
// the faces and, with VISCOUS, the viscous forces at the faces.
struct AsmCell {
    float gamma, eta;
    float etaW, etaE, etaN, etaS;
    float gWr, gEr, gNr, gSr;          // neighbours' gamma as read (gNr / gSr: rows inside)
    float uW, uE, vN, vS;              // face velocities (NaN zeroed in assemble_compute)
    float uAirW, uAirE, vAirN, vAirS;  // wind at the faces
    float fuW, fuE, fvN, fvS;          // viscous forces (VISCOUS only)
};

// The row of an unbroken cell of row i (its values written to the outputs).
template <bool VISC>
__device__ __forceinline__ void assemble_compute(const SbGrid& g, const SbPhys& ph,
                                                 const SbFields& f, int i, AsmCell c,
                                                 float& o_dmass, float& o_cE, float& o_cS,
                                                 float& o_r0, float& o_rhs) {
    const int nT = g.nT;
    const float dt = f.step->dt, invDt = f.step->invDt;
    const float gmax = ph.gmax, Cr = ph.Cr;
    const float gamma = c.gamma, eta = c.eta;
    const float sinT = g.sin_c[i];
    const float sinN = g.sin_e[i];
    const float sinS = g.sin_e[i + 1];
    const float cscT = 1.0f / sinT;
    const float etaW = c.etaW, etaE = c.etaE, etaN = c.etaN, etaS = c.etaS;
    const float vAirN = c.vAirN, vAirS = c.vAirS, uAirW = c.uAirW, uAirE = c.uAirE;
    float vN = c.vN, vS = c.vS, uW = c.uW, uE = c.uE;
    if (isnan(vN)) vN = 0.0f;
    if (isnan(vS)) vS = 0.0f;
    if (isnan(uW)) uW = 0.0f;
    if (isnan(uE)) uE = 0.0f;

    const float CrDt = Cr * dt, MDt = ph.M * dt;
    const float s2 = g.invh * g.invh;
    const float etaUp = (etaN + eta) * 0.5f;
    const float etaLeft = (etaW + eta) * 0.5f;
    const float etaRight = (etaE + eta) * 0.5f;
    const float etaDown = (etaS + eta) * 0.5f;
    // Every face term of the reference's row divides by eta_face + Cr dt
    // (written there as eta/(eta + Cr dt), 1/(eta/(Cr dt) + 1) and
    // eta/(eta/dt + Cr)): one reciprocal per face serves all of them.
    const float rN = 1.0f / (etaUp + CrDt), rW = 1.0f / (etaLeft + CrDt);
    const float rE = 1.0f / (etaRight + CrDt), rS = 1.0f / (etaDown + CrDt);
    const float wN = (i == 0) ? 0.0f : s2 * sinN * MDt * rN;
    const float wW = s2 * cscT * MDt * rW;
    const float wE = s2 * cscT * MDt * rE;
    const float wS = (i == nT - 1) ? 0.0f : s2 * sinS * MDt * rS;

    float sinThetaDiv = g.invh * (uE * etaRight * rE - uW * etaLeft * rW +
                                  (vS * sinS * etaDown * rS - vN * sinN * etaUp * rN));
    sinThetaDiv += g.invh * CrDt *
                   (uAirE * rE - uAirW * rW + vAirS * sinS * rS - vAirN * sinN * rN);
    if (VISC) {
        // bubble.cu:1460-1466: the viscous forces, gravity inside fv
        sinThetaDiv += g.invh * dt *
                       (sinS * c.fvS * etaDown * rS - sinN * c.fvN * etaUp * rN +
                        c.fuE * etaRight * rE - c.fuW * etaLeft * rW);
    } else {
        sinThetaDiv += ph.gs * g.invh * dt *
                       (sinS * sinS * etaDown * rS - sinN * sinN * etaUp * rN);
    }

    // neighbour gamma (a broken neighbour holds gmax) and broken flags
    const float gEr = c.gEr, gWr = c.gWr;
    const bool bE = is_broken(gEr, etaE, ph.gthr), bW = is_broken(gWr, etaW, ph.gthr);
    const float gE = bE ? gmax : gEr, gW = bW ? gmax : gWr;
    bool bN = false, bS = false;
    float gN = gamma, gS = gamma, gNr = gamma, gSr = gamma;
    if (i != 0) {
        gNr = c.gNr;
        bN = is_broken(gNr, etaN, ph.gthr);
        gN = bN ? gmax : gNr;
    }
    if (i != nT - 1) {
        gSr = c.gSr;
        bS = is_broken(gSr, etaS, ph.gthr);
        gS = bS ? gmax : gSr;
    }
    const float lap = wE * (gamma - gE) + wW * (gamma - gW) + wN * (gamma - gN) + wS * (gamma - gS);
    float cE = bE ? 0.0f : wE, cS = bS ? 0.0f : wS;
    float r0 = -sinThetaDiv - lap;
    // rows and columns of cells with t > 2^48 are scaled by s = 2^-k
    // (sb_scale.cuh): this cell's row, and its couplings to such neighbours
    const int kc = diag_scale_k(gamma, sinT, invDt);
    const int kE = bE ? 0 : diag_scale_k(gEr, sinT, invDt);
    const int kW = bW ? 0 : diag_scale_k(gWr, sinT, invDt);
    const int kN = (i == 0 || bN) ? 0 : diag_scale_k(gNr, g.sin_c[i - 1], invDt);
    const int kS = (i == nT - 1 || bS) ? 0 : diag_scale_k(gSr, g.sin_c[i + 1], invDt);
    float dmass = scaled_diag_term(gamma, sinT, invDt, kc);
    if (!(kc | kE | kW | kN | kS)) {
        if (bE) dmass += wE;
        if (bW) dmass += wW;
        if (bN) dmass += wN;
        if (bS) dmass += wS;
    } else {
        // s_c A_cc s_c in excess form: t s_c^2 + s_c^2 (weights to broken
        // neighbours) + sum over the other couplings of w s_c (s_c - s_n)
        const float sc = pow2_neg(kc), sc2 = sc * sc;
        const float sE = pow2_neg(kE), sW = pow2_neg(kW), sN = pow2_neg(kN), sS = pow2_neg(kS);
        dmass += bE ? wE * sc2 : wE * sc * (sc - sE);
        dmass += bW ? wW * sc2 : wW * sc * (sc - sW);
        dmass += bN ? wN * sc2 : wN * sc * (sc - sN);
        dmass += bS ? wS * sc2 : wS * sc * (sc - sS);
        cE *= sc * sE;
        cS *= sc * sS;
        r0 *= sc;
    }
    o_dmass = dmass;
    o_cE = cE;
    o_cS = cS;
    o_r0 = r0;
    o_rhs = sinT * invDt - sinThetaDiv;
}

// A broken cell (gamma at its maximum or no film): the identity row
// dx = 0 with gamma_adv = gmax.
__device__ __forceinline__ void assemble_broken(const SbFields& f, float gmax, int idx) {
    f.dmass[idx] = 1.0f;
    f.cE[idx] = 0.0f;
    f.cS[idx] = 0.0f;
    f.r0[idx] = 0.0f;
    f.rhs[idx] = gmax;
    f.gam_adv[idx] = gmax;
}

template <bool VISC>
__device__ __forceinline__ void assemble_cell(const SbGrid& g, const SbPhys& ph, const SbFields& f, int cur,
                                          int idx) {
    (void)cur;
    const int i = idx >> g.logP, j = idx & g.maskP;
    const int nP = g.nP, nT = g.nT;
    const float mixA = f.step->mixA, mixB = f.step->mixB;
    const float gmax = ph.gmax;
    const float* eta_a = f.eta_adv;
    AsmCell c;
    c.gamma = f.gam_adv[idx];
    c.eta = eta_a[idx];
    if (is_broken(c.gamma, c.eta, ph.gthr)) {
        assemble_broken(f, gmax, idx);
        atomicAdd(&f.stats->broken_cells, 1);
        return;
    }
    const int jE = (j + 1) & g.maskP, jW = (j - 1) & g.maskP;
    const int iE = i * nP + jE, iW = i * nP + jW;
    c.etaW = eta_a[iW];
    c.etaE = eta_a[iE];
    c.vN = c.vS = c.vAirN = c.vAirS = 0.0f;
    c.gNr = c.gSr = c.gamma;
    const int opp = nP - j;            // flat mirrored index (reads next row at j = 0)
    const int oppE = nP - jE;
    if (i != 0) {
        const int n = (i - 1) * nP + j;
        c.vAirN = 0.5f * (f.vair[n] * mixA - f.vair[(i - 1) * nP + opp] * mixB);
        c.vN = f.uth_adv[n];
        c.etaN = eta_a[n];
        c.gNr = f.gam_adv[n];
    } else {
        c.etaN = eta_a[(j + nT) & g.maskP];
    }
    if (i != nT - 1) {
        c.vAirS = 0.5f * (f.vair[idx] * mixA - f.vair[i * nP + opp] * mixB);
        c.vS = f.uth_adv[idx];
        c.etaS = eta_a[idx + nP];
        c.gSr = f.gam_adv[idx + nP];
    } else {
        c.etaS = eta_a[i * nP + ((j + nT) & g.maskP)];
    }
    c.uW = f.uph_adv[idx];
    c.uE = f.uph_adv[iE];
    c.uAirW = 0.5f * (f.uair[idx] * mixA + f.uair[i * nP + opp] * mixB);
    c.uAirE = 0.5f * (f.uair[iE] * mixA + f.uair[i * nP + oppE] * mixB);
    c.gWr = f.gam_adv[iW];
    c.gEr = f.gam_adv[iE];
    c.fuW = c.fuE = c.fvN = c.fvS = 0.0f;
    if (VISC) {
        c.fuW = viscous_fu(g, ph, f, i, j);
        c.fuE = viscous_fu(g, ph, f, i, jE);
        c.fvN = i != 0 ? viscous_fv(g, ph, f, i - 1, j) : 0.0f;
        c.fvS = i != nT - 1 ? viscous_fv(g, ph, f, i, j) : 0.0f;
    }
    float dmass, cE, cS, r0, rhs;
    assemble_compute<VISC>(g, ph, f, i, c, dmass, cE, cS, r0, rhs);
    f.dmass[idx] = dmass;
    f.cE[idx] = cE;
    f.cS[idx] = cS;
    f.r0[idx] = r0;
    f.rhs[idx] = rhs;
}

// rowbase[nP - j - k], k = 0 .. 4, for a four-aligned j: the mirrored wind
// entries (nP - j reads the next row's first element at j = 0, as the
// reference's unpitched read does) as one 128-bit load and one scalar.
__device__ __forceinline__ void mirror5(const float* rowbase, int nP, int j, float (&m)[5]) {
    m[0] = rowbase[nP - j];
    const float4 q = *reinterpret_cast<const float4*>(rowbase + nP - j - 4);
    m[4] = q.x; m[3] = q.y; m[2] = q.z; m[1] = q.w;
}

// assemble_cell (without the viscous forces) on the four cells idx .. idx + 3
// of one row: the inputs of the row, the rows beside it and the wind arrive
// in 128-bit loads along phi (the cells beyond the group's ends in scalar
// ones), each cell does assemble_compute, and the outputs leave in 128-bit
// stores.
__device__ __forceinline__ void assemble_quad(const SbGrid& g, const SbPhys& ph, const SbFields& f,
                                              int idx) {
    const int i = idx >> g.logP, j = idx & g.maskP;
    const int nP = g.nP, nT = g.nT, row = i * nP;
    const float mixA = f.step->mixA, mixB = f.step->mixB;
    const float gmax = ph.gmax;
    const float* eta_a = f.eta_adv;
    const int jE4 = (j + 4) & g.maskP, jW = (j - 1) & g.maskP;
    float G[4], E[4], U[4], UA[4], EN[4], ES[4], GN[4], GS[4], VN[4], VS[4], VAN[4], VAS[4];
    float UAm[5], VANm[5], VASm[5];
    ld4(f.gam_adv + idx, G);
    ld4(eta_a + idx, E);
    ld4(f.uph_adv + idx, U);
    ld4(f.uair + idx, UA);
    mirror5(f.uair + row, nP, j, UAm);
    const float gW0 = f.gam_adv[row + jW], eW0 = eta_a[row + jW];
    const float gE3 = f.gam_adv[row + jE4], eE3 = eta_a[row + jE4];
    const float uE3 = f.uph_adv[row + jE4], uaE3 = f.uair[row + jE4];
    // k = 3 at the row's last group: jE = 0, mirrored index nP
    const float uaE3m = jE4 ? UAm[4] : f.uair[row + nP];
    if (i != 0) {
        const int n = idx - nP;
        ld4(eta_a + n, EN);
        ld4(f.gam_adv + n, GN);
        ld4(f.uth_adv + n, VN);
        ld4(f.vair + n, VAN);
        mirror5(f.vair + (i - 1) * nP, nP, j, VANm);
    } else {
        ld4(eta_a + ((j + nT) & g.maskP), EN);
    }
    if (i != nT - 1) {
        ld4(eta_a + idx + nP, ES);
        ld4(f.gam_adv + idx + nP, GS);
        ld4(f.uth_adv + idx, VS);
        ld4(f.vair + idx, VAS);
        mirror5(f.vair + row, nP, j, VASm);
    } else {
        ld4(eta_a + row + ((j + nT) & g.maskP), ES);
    }
    float oD[4], oE[4], oS[4], oR[4], oB[4];
    int broken = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        AsmCell c;
        c.gamma = G[k];
        c.eta = E[k];
        if (is_broken(c.gamma, c.eta, ph.gthr)) {
            oD[k] = 1.0f; oE[k] = 0.0f; oS[k] = 0.0f; oR[k] = 0.0f; oB[k] = gmax;
            f.gam_adv[idx + k] = gmax;
            ++broken;
            continue;
        }
        c.etaW = k ? E[k - 1] : eW0;
        c.etaE = k < 3 ? E[k + 1] : eE3;
        c.gWr = k ? G[k - 1] : gW0;
        c.gEr = k < 3 ? G[k + 1] : gE3;
        c.etaN = EN[k];
        c.etaS = ES[k];
        c.vN = c.vS = c.vAirN = c.vAirS = 0.0f;
        c.gNr = c.gSr = c.gamma;
        if (i != 0) {
            c.vAirN = 0.5f * (VAN[k] * mixA - VANm[k] * mixB);
            c.vN = VN[k];
            c.gNr = GN[k];
        }
        if (i != nT - 1) {
            c.vAirS = 0.5f * (VAS[k] * mixA - VASm[k] * mixB);
            c.vS = VS[k];
            c.gSr = GS[k];
        }
        c.uW = U[k];
        c.uE = k < 3 ? U[k + 1] : uE3;
        c.uAirW = 0.5f * (UA[k] * mixA + UAm[k] * mixB);
        c.uAirE = 0.5f * ((k < 3 ? UA[k + 1] : uaE3) * mixA + (k < 3 ? UAm[k + 1] : uaE3m) * mixB);
        c.fuW = c.fuE = c.fvN = c.fvS = 0.0f;
        assemble_compute<false>(g, ph, f, i, c, oD[k], oE[k], oS[k], oR[k], oB[k]);
    }
    st4(f.dmass + idx, oD);
    st4(f.cE + idx, oE);
    st4(f.cS + idx, oS);
    st4(f.r0 + idx, oR);
    st4(f.rhs + idx, oB);
    if (broken) atomicAdd(&f.stats->broken_cells, broken);
}

// After the solve: divergence from gamma, friction/Marangoni/gravity velocity
// update, thickness update with evaporation, and the per-step changes that
// BIMOCQ accumulates.  Increments are carried directly (dx from the solve,
// d_eta = -eta dt div + evap dt) instead of as differences of O(1) values.
// Neighbouring new gamma values are clamped on the fly exactly as
// divergenceKernel_fromGamma clamps them in place (kernel/bubble.cu:1287;
// thr as in is_broken).
__device__ __forceinline__ bool gamma_clamped(float gm, float thr) {
    return gm <= 0.0f || gm > thr;
}

// Difference gamma_new(a) - gamma_new(b) of two cells.  The increments
// are differenced as the solver's float-float pairs: next to the poles the
// new gamma varies along phi by parts in 1e5 of the increment, and the
// Marangoni force there (1/sin(theta) times that difference) would inherit
// the increment's FP32 rounding (2e-4 of u_phi at the config.txt grid).
__device__ __forceinline__ float gnew_diff(const SbFields& f, int a, int b, float gmax, float thr) {
    const float xa = f.x[a], xb = f.x[b];
    const bool ca = gamma_clamped(xa, thr), cb = gamma_clamped(xb, thr);
    if (!ca && !cb) {
        const float2 da = f.xff[a], db = f.xff[b];
        return (f.gam_adv[a] - f.gam_adv[b]) + ((da.x - db.x) + (da.y - db.y));
    }
    return (ca ? gmax : xa) - (cb ? gmax : xb);
}

template <class T, bool VISC>
__device__ __forceinline__ void post_cell(const SbGrid& g, const SbPhys& ph, const SbFields& f, int cur,
                                          int idx) {
    (void)cur;
    const int i = idx >> g.logP, j = idx & g.maskP;
    const int nP = g.nP;
    const float dt = f.step->dt, invDt = f.step->invDt;
    const float gmax = ph.gmax, M = ph.M, Cr = ph.Cr;
    const float gOld = f.gam_adv[idx];
    const float gNew = f.x[idx];
    float mdtdiv;  // -dt * div
    if (gamma_clamped(gNew, ph.gthr)) {
        st_s<T>(f.gam, idx, gmax, ph.base_gam);
        f.d_gam[idx] = gmax - gOld;
        mdtdiv = -1.0f;
    } else {
        const float dx = f.dx[idx];
        st_s<T>(f.gam, idx, gNew, ph.base_gam);
        f.d_gam[idx] = dx;
        // div = (1 - min(gNew, 2 gOld) / gOld) / dt
        mdtdiv = (gNew > 2.0f * gOld) ? 1.0f : dx / gOld;
    }

    const float e = f.eta_adv[idx];
    const float de = e * mdtdiv + f.step->evapDt;
    if (e + de >= 0.0f) {
        st_s<T>(f.eta, idx, e + de, ph.base_eta);
        f.d_eta[idx] = de;
    } else {
        st_s<T>(f.eta, idx, 0.0f, ph.base_eta);
        f.d_eta[idx] = -e;
    }

    // u_phi face between (i, j-1) and (i, j).  Under VISCOUS the reference
    // launches its u_phi update with the u_theta layout (nTheta - 1 rows,
    // kernel/bubble.cu:2463-2474), so u_phi's last theta row keeps its value
    // from before the step: the state buffer is left as it is.
    // The reference's update u = (u dt^-1 + f1 + f2 (+ f3)) / (dt^-1 + Cr / eta_f)
    // with f1 = -M grad(gamma) / eta_f, f2 = Cr uair / eta_f is evaluated
    // multiplied through by the face thickness eta_f = (eta_a + eta_b) / 2:
    // one quotient per face.  A face without film (eta_f = 0, the
    // reference's 1/eta_f infinite) gets a NaN velocity as there.
    if (!VISC || i < g.nT - 1) {
        const int w = i * nP + ((j - 1) & g.maskP);
        const float ef = 0.5f * (f.eta_adv[w] + e);
        const float u1 = f.uph_adv[idx];
        if (ef == 0.0f) {
            f.uph[idx] = __int_as_float(0x7fffffff);
        } else {
            const float cscT = 1.0f / g.sin_c[i];
            const float pGpx = g.invh * gnew_diff(f, idx, w, gmax, ph.gthr) * cscT;
            if (VISC) {
                // applyforcevelphiKernel_viscous (bubble.cu:1987-2038): the
                // mirrored wind mix and fu
                const float uAir = 0.5f * (f.uair[idx] * f.step->mixA +
                                           f.uair[i * nP + (nP - j)] * f.step->mixB);
                f.uph[idx] = ((u1 * invDt + viscous_fu(g, ph, f, i, j)) * ef - M * pGpx + Cr * uAir) /
                             (invDt * ef + Cr);
            } else {
                f.uph[idx] = (u1 * invDt * ef - M * pGpx + Cr * f.uair[idx]) / (invDt * ef + Cr);
            }
        }
    }
    // u_theta face between (i, j) and (i+1, j)
    if (i < g.nT - 1) {
        const int s = idx + nP;
        const float ef = 0.5f * (e + f.eta_adv[s]);
        const float v1 = f.uth_adv[idx];
        if (ef == 0.0f) {
            f.uth[idx] = __int_as_float(0x7fffffff);
        } else {
            const float pGpy = g.invh * gnew_diff(f, s, idx, gmax, ph.gthr);
            if (VISC) {
                // applyforcevelthetaKernel_viscous (bubble.cu:1940-1983)
                const float vAir = 0.5f * (f.vair[idx] * f.step->mixA -
                                           f.vair[i * nP + (nP - j)] * f.step->mixB);
                f.uth[idx] = ((v1 * invDt + viscous_fv(g, ph, f, i, j)) * ef - M * pGpy + Cr * vAir) /
                             (invDt * ef + Cr);
            } else {
                const float f3v = ph.gs * g.sin_e[i + 1];
                f.uth[idx] = ((v1 * invDt + f3v) * ef - M * pGpy + Cr * f.vair[idx]) /
                             (invDt * ef + Cr);
            }
        }
    }
}

// gnew_diff of two cells whose x, xff and gamma_adv are at hand.
__device__ __forceinline__ float gnew_diff_v(float xa, float2 da, float ga, float xb, float2 db,
                                             float gb, float gmax, float thr) {
    const bool ca = gamma_clamped(xa, thr), cb = gamma_clamped(xb, thr);
    if (!ca && !cb) return (ga - gb) + ((da.x - db.x) + (da.y - db.y));
    return (ca ? gmax : xa) - (cb ? gmax : xb);
}

// post_cell (without the viscous forces) on the four cells idx .. idx + 3
// of one row: every input and output moves in 128-bit accesses along phi
// (the west neighbour of the first cell in scalar ones), and each cell
// does post_cell's operations.
template <class T>
__device__ __forceinline__ void post_quad(const SbGrid& g, const SbPhys& ph, const SbFields& f,
                                          int idx) {
    const int i = idx >> g.logP, j = idx & g.maskP;
    const int nP = g.nP;
    const float invDt = f.step->invDt, evapDt = f.step->evapDt;
    const float gmax = ph.gmax, M = ph.M, Cr = ph.Cr;
    const bool hasS = i < g.nT - 1;
    float gO[4], X[4], DX[4], E[4], U1[4], UA[4];
    float2 XF[4];
    ld4(f.gam_adv + idx, gO);
    ld4(f.x + idx, X);
    ld4(f.dx + idx, DX);
    ld4(f.eta_adv + idx, E);
    ld4(f.uph_adv + idx, U1);
    ld4(f.uair + idx, UA);
    ld4(f.xff + idx, XF);
    const int w = i * nP + ((j - 1) & g.maskP);
    const float gW = f.gam_adv[w], xW = f.x[w], eW = f.eta_adv[w];
    const float2 xfW = f.xff[w];
    float gS[4], XS[4], ES[4], V1[4], VA[4];
    float2 XFS[4];
    if (hasS) {
        ld4(f.gam_adv + idx + nP, gS);
        ld4(f.x + idx + nP, XS);
        ld4(f.eta_adv + idx + nP, ES);
        ld4(f.xff + idx + nP, XFS);
        ld4(f.uth_adv + idx, V1);
        ld4(f.vair + idx, VA);
    }
    const float cscT = 1.0f / g.sin_c[i];
    const float f3v = hasS ? ph.gs * g.sin_e[i + 1] : 0.0f;
    const float nan = __int_as_float(0x7fffffff);
    float oG[4], oDG[4], oE[4], oDE[4], oU[4], oV[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float mdtdiv;  // -dt * div
        if (gamma_clamped(X[k], ph.gthr)) {
            oG[k] = gmax;
            oDG[k] = gmax - gO[k];
            mdtdiv = -1.0f;
        } else {
            oG[k] = X[k];
            oDG[k] = DX[k];
            mdtdiv = (X[k] > 2.0f * gO[k]) ? 1.0f : DX[k] / gO[k];
        }
        const float e = E[k];
        const float de = e * mdtdiv + evapDt;
        if (e + de >= 0.0f) {
            oE[k] = e + de;
            oDE[k] = de;
        } else {
            oE[k] = 0.0f;
            oDE[k] = -e;
        }
        // u_phi face between cells k - 1 and k (the face thickness form of
        // post_cell)
        const float ef = 0.5f * ((k ? E[k - 1] : eW) + e);
        if (ef == 0.0f) {
            oU[k] = nan;
        } else {
            const float dG = k ? gnew_diff_v(X[k], XF[k], gO[k], X[k - 1], XF[k - 1], gO[k - 1], gmax, ph.gthr)
                               : gnew_diff_v(X[k], XF[k], gO[k], xW, xfW, gW, gmax, ph.gthr);
            const float pGpx = g.invh * dG * cscT;
            oU[k] = (U1[k] * invDt * ef - M * pGpx + Cr * UA[k]) / (invDt * ef + Cr);
        }
        if (hasS) {
            const float es = 0.5f * (e + ES[k]);
            if (es == 0.0f) {
                oV[k] = nan;
            } else {
                const float pGpy =
                    g.invh * gnew_diff_v(XS[k], XFS[k], gS[k], X[k], XF[k], gO[k], gmax, ph.gthr);
                oV[k] = ((V1[k] * invDt + f3v) * es - M * pGpy + Cr * VA[k]) / (invDt * es + Cr);
            }
        }
    }
    st4_s<T>(f.gam, idx, oG, ph.base_gam);
    st4(f.d_gam + idx, oDG);
    st4_s<T>(f.eta, idx, oE, ph.base_eta);
    st4(f.d_eta + idx, oDE);
    st4(f.uph + idx, oU);
    if (hasS) st4(f.uth + idx, oV);
}

__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// BIMOCQ change accumulation through the forward map, fused with the
// forward/backward distortion estimate of the same maps and with the error
// estimate of a re-initialisation (correctCentered1, which samples the new
// fields at the same five points): the error is formed every step, and the
// re-initialisation, when the distortion calls for it, only corrects.
// returns the cell's distortion (0 outside the grid)
template <class T>
__device__ __forceinline__ float accum_cell(const SbGrid& g, const SbPhys& ph, const SbFields& f, int cur,
                                           int idx) {
    const int i = idx >> g.logP, j = idx & g.maskP;
    const Frame F = cell_frame(g, i, j);
    const float4* fwd = f.fwd[cur ^ 1];
    const float4* bwd = f.bwd[cur ^ 1];
    float ed = f.eta_delta[idx], gd = f.gam_delta[idx];
    float th = 0.0f, gm = 0.0f;
    f3 ds[5];
    sample_map_multi5(g, fwd, F, ds);
    CStencil c4;  // stencil of sample 4, the cell's own forward-map point
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const CStencil c = centred_stencil(g, pos_from_disp_fast(F, ds[k], g.invh, g.nT), 0.0f);
        if (k == 4) c4 = c;
        const SStencil s = sstencil_of(g, c);
        ed += kW5[k] * gather(f.d_eta, s);
        gd += kW5[k] * gather(f.d_gam, s);
        th += kW5[k] * gather_s<T>(f.eta, s, ph.base_eta);
        gm += kW5[k] * gather_s<T>(f.gam, s, ph.base_gam);
    }
    f.eta_delta[idx] = ed;
    f.gam_delta[idx] = gd;
    f.err_eta[idx] = (th - ed - ld_s<T>(f.eta_init, idx, ph.base_eta)) * 0.5f;
    f.err_gam[idx] = (gm - gd - ld_s<T>(f.gam_init, idx, ph.base_gam)) * 0.5f;
    // estimateDistortion: dist(x, bwd(fwd(x))) and dist(x, fwd(bwd(x))); fwd(x)
    // is sample 4 above (the cell's own map entry), whose stencil is reused
    const float d1 = dist_from_disp(map_at_stencil(g, bwd, F, c4), g.invh);
    const float4 m = bwd[idx];
    const float d2 = dist_from_disp(
        sample_map(g, fwd, F, pos_from_disp_fast(F, f3{m.x, m.y, m.z}, g.invh, g.nT)), g.invh);
    const float dist = fmaxf(fabsf(d1), fabsf(d2));
    return isnan(dist) ? 0.0f : dist;
}

// Block maximum of the distortion into the bubble's statistics (all
// threads of the block belong to one bubble).
__device__ __forceinline__ void block_max_distortion(float dist, SbDevStats* st) {
    __shared__ float smax[32];
    dist = warp_max(dist);
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = dist;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? smax[threadIdx.x] : 0.0f;
        v = warp_max(v);
        if (threadIdx.x == 0) atomicMax(&st->distortion_bits, __float_as_uint(v));
    }
}

// ---------------------------------------------------------------------------
// Kernels.  A launch covers a set of bubbles (one bubble, or every bubble of
// a batch): descs[k] points to bubble k's descriptor, and block b works on
// the cells tiles[b] = (bubble, first cell) .. + blockDim.x - 1 (a tile never
// straddles two bubbles).  One bubble stepped alone and inside a batch runs
// the same kernels on the same descriptor.
// The block's bubble descriptor is copied to shared memory first, so the
// cell code reads grid constants and array pointers from there.
__device__ __forceinline__ const SbBubbleDesc& stage_tile_desc(SbBubbleDesc* const* descs, int b,
                                                               SbBubbleDesc* s_d) {
    constexpr int kWords = (int)(sizeof(SbBubbleDesc) / 4);
    const int* src = reinterpret_cast<const int*>(descs[b]);
    int* dst = reinterpret_cast<int*>(s_d);
    for (int k = threadIdx.x; k < kWords; k += blockDim.x) dst[k] = src[k];
    __syncthreads();
    return *s_d;
}

// Kernels whose cells touch the stored thickness / surfactant fields are
// instantiated per storage type T (float or __nv_bfloat16); a plan launches
// the instantiation of its bubbles' storage.
#define SB_CELL_KERNEL_BODY(...)                                                       \
    __shared__ __align__(16) SbBubbleDesc s_d;                                         \
    const int2 t = tiles[blockIdx.x];                                                  \
    const SbBubbleDesc& d = stage_tile_desc(descs, t.x, &s_d);                         \
    if (d.halted) return;                                                              \
    const int idx = t.y + threadIdx.x;                                                 \
    if (idx < d.g.N) __VA_ARGS__(d.g, d.ph, d.f, d.cur, idx);

#define SB_CELL_KERNEL(name)                                                           \
    __global__ void __launch_bounds__(256) k_##name(SbBubbleDesc* const* __restrict__ descs, \
                                                    const int2* __restrict__ tiles) {  \
        SB_CELL_KERNEL_BODY(name##_cell)                                               \
    }

// k_advect_maps is held to 48 registers per thread (five 256-thread blocks
// per SM; a few spilled values): measured 61 -> 58 us on c1.
template <class T>
__global__ void __launch_bounds__(256, 5) k_advect_maps(SbBubbleDesc* const* __restrict__ descs,
                                                        const int2* __restrict__ tiles) {
    SB_CELL_KERNEL_BODY(advect_maps_cell<T>)
}
SB_CELL_KERNEL(velocity)
// k_bimocq is held to 64 registers per thread with its five samples taken two
// at a time (two independent map-lookup chains in flight per thread; a few
// spilled values): measured 79.7 -> 75.9 us on c1 (either change alone, or
// all five samples unrolled, is slower).
template <class T>
__global__ void __launch_bounds__(256, 4) k_bimocq(SbBubbleDesc* const* __restrict__ descs,
                                                   const int2* __restrict__ tiles) {
    SB_CELL_KERNEL_BODY(bimocq_cell<T>)
}
// k_assemble / k_post: the instantiations with VISC = true evaluate the
// viscous forces (every bubble of a plan has the same switch).
template <bool VISC>
__global__ void __launch_bounds__(256) k_assemble(SbBubbleDesc* const* __restrict__ descs,
                                                  const int2* __restrict__ tiles) {
    SB_CELL_KERNEL_BODY(assemble_cell<VISC>)
}

// The non-viscous assembly, four cells per thread (a tile of n cells runs
// in n / 4 threads), held to 64 registers: c1 16.4 us as one cell per
// thread, c2 49.2 us against 51.2 (uncapped, 114 registers: 18.4 and 49.0).
__global__ void __launch_bounds__(64, 16) k_assemble4(SbBubbleDesc* const* __restrict__ descs,
                                                  const int2* __restrict__ tiles) {
    __shared__ __align__(16) SbBubbleDesc s_d;
    const int2 t = tiles[blockIdx.x];
    const SbBubbleDesc& d = stage_tile_desc(descs, t.x, &s_d);
    if (d.halted) return;
    const int idx = t.y + 4 * threadIdx.x;
    if (idx < d.g.N) assemble_quad(d.g, d.ph, d.f, idx);
}

template <class T, bool VISC>
__global__ void __launch_bounds__(256) k_post(SbBubbleDesc* const* __restrict__ descs,
                                              const int2* __restrict__ tiles) {
    SB_CELL_KERNEL_BODY(post_cell<T, VISC>)
}

// The non-viscous post-solve update, four cells per thread (a tile of n
// cells runs in n / 4 threads).
template <class T>
__global__ void __launch_bounds__(64) k_post4(SbBubbleDesc* const* __restrict__ descs,
                                              const int2* __restrict__ tiles) {
    __shared__ __align__(16) SbBubbleDesc s_d;
    const int2 t = tiles[blockIdx.x];
    const SbBubbleDesc& d = stage_tile_desc(descs, t.x, &s_d);
    if (d.halted) return;
    const int idx = t.y + 4 * threadIdx.x;
    if (idx < d.g.N) post_quad<T>(d.g, d.ph, d.f, idx);
}

// k_accum is held to 64 registers per thread (a few spilled values): the
// occupancy it gains outweighs them (measured 87 -> 84 us on c1).
template <class T>
__global__ void __launch_bounds__(256, 4) k_accum(SbBubbleDesc* const* __restrict__ descs,
                                               const int2* __restrict__ tiles) {
    __shared__ __align__(16) SbBubbleDesc s_d;
    const int2 t = tiles[blockIdx.x];
    const SbBubbleDesc& d = stage_tile_desc(descs, t.x, &s_d);
    if (d.halted) return;  // the same in every thread of the block
    const int idx = t.y + threadIdx.x;
    const float dist = idx < d.g.N ? accum_cell<T>(d.g, d.ph, d.f, d.cur, idx) : 0.0f;
    block_max_distortion(dist, d.f.stats);
}

__device__ __forceinline__ bool reinit_now(const SbBubbleDesc& d) {
    if (d.halted) return false;
    const SbDevStats* st = d.f.stats;
    if (st->force_reinit >= 0) return st->force_reinit != 0;
    return __uint_as_float(st->distortion_bits) > 4.0f;
}

// 3x3 neighbour of (i, j) with the reference's across-pole rule (validateId).
__device__ __forceinline__ int nb_index(const SbGrid& g, int i, int j) {
    if (i < 0) { i = 0; j += g.nT; }
    else if (i >= g.nT) { i = g.nT - 1; j += g.nT; }
    return i * g.nP + (j & g.maskP);
}

// correctCentered2: subtract the error pulled back through the backward map,
// clamp to the 3x3 range of the uncorrected field, keep non-negative.  The
// result goes to the per-step increment buffers (read by k_accum, free from
// here on; the *_adv buffers keep the step's implicit system) and is
// committed in the next phase.
template <class T>
__device__ __forceinline__ void reinit_correct(const SbGrid& g, const SbPhys& ph, const SbFields& f, int cur,
                                               int idx) {
    const int i = idx >> g.logP, j = idx & g.maskP;
    const Frame F = cell_frame(g, i, j);
    const float4* bwd = f.bwd[cur ^ 1];
    const float be = ph.base_eta, bg = ph.base_gam;
    float th = ld_s<T>(f.eta, idx, be), gm = ld_s<T>(f.gam, idx, bg);
    f3 ds[5];
    sample_map_multi5(g, bwd, F, ds);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const SStencil s = scalar_stencil(g, pos_from_disp_fast(F, ds[k], g.invh, g.nT));
        th -= kW5[k] * gather(f.err_eta, s);
        gm -= kW5[k] * gather(f.err_gam, s);
    }
    float emin = ld_s<T>(f.eta, idx, be), emax = emin, gmin = ld_s<T>(f.gam, idx, bg), gmx = gmin;
    for (int t = -1; t <= 1; ++t)
        for (int p = -1; p <= 1; ++p) {
            const int n = nb_index(g, i + t, j + p);
            const float ev = ld_s<T>(f.eta, n, be), gv = ld_s<T>(f.gam, n, bg);
            emin = fminf(emin, ev); emax = fmaxf(emax, ev);
            gmin = fminf(gmin, gv); gmx = fmaxf(gmx, gv);
        }
    th = (th < emin) ? emin : (emax < th) ? emax : th;
    gm = (gm < gmin) ? gmin : (gmx < gm) ? gmx : gm;
    f.d_eta[idx] = fmaxf(0.0f, th);
    f.d_gam[idx] = fmaxf(0.0f, gm);
}

// Commit the correction, rotate the BIMOCQ buffers and reset the maps.
template <class T>
__device__ __forceinline__ void reinit_commit(const SbPhys& ph, const SbFields& f, int cur, int idx) {
    const float e = f.d_eta[idx], gm = f.d_gam[idx];
    st_s<T>(f.eta, idx, e, ph.base_eta);
    st_s<T>(f.gam, idx, gm, ph.base_gam);
    cp_s<T>(f.eta_initL, f.eta_init, idx);
    f.eta_deltaL[idx] = f.eta_delta[idx];
    cp_s<T>(f.gam_initL, f.gam_init, idx);
    f.gam_deltaL[idx] = f.gam_delta[idx];
    st_s<T>(f.eta_init, idx, e, ph.base_eta);
    f.eta_delta[idx] = 0.0f;
    st_s<T>(f.gam_init, idx, gm, ph.base_gam);
    f.gam_delta[idx] = 0.0f;
    f.bwdprev[idx] = f.bwd[cur ^ 1][idx];
    f.fwd[cur ^ 1][idx] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    f.bwd[cur ^ 1][idx] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// reInitializeMapping (kernel/bubble.cu:2509-2564) for every bubble of the
// set whose distortion exceeds 4 cells (or that forces it): one cooperative
// launch, two phases over the bubbles' tiles separated by a grid barrier
// (correct, then commit; the error estimate was formed by k_accum).
// The decisions are read from device memory, so no host synchronisation is
// needed; every block reads every bubble's decision, so all blocks agree on
// whether any phase runs, and without a re-initialisation they return at
// once.
template <class T>
__global__ void __launch_bounds__(kBlock)
k_reinit(SbBubbleDesc* const* __restrict__ descs, int nb, const int2* __restrict__ tiles,
         int ntiles, unsigned* gbar) {
    __shared__ int any;
    if (descs[0]->f.stats->wait_faults) return;  // the barrier word is not trusted any more
    if (threadIdx.x == 0) {
        int a = 0;
        for (int b = 0; b < nb; ++b) a |= reinit_now(*descs[b]) ? 1 : 0;
        any = a;
    }
    __syncthreads();
    if (!any) return;
    unsigned gen = grid_barrier_gen(gbar);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tl = tiles[t];
        const SbBubbleDesc& d = *descs[tl.x];
        if (!reinit_now(d)) continue;
        for (int idx = tl.y + threadIdx.x; idx < tl.y + kBlock && idx < d.g.N; idx += blockDim.x) {
            if (idx == 0) {
                d.f.stats->reinit = 1;
                d.f.stats->reinit_total += 1;
            }
            reinit_correct<T>(d.g, d.ph, d.f, d.cur, idx);
        }
    }
    if (!grid_barrier(gbar, gen, gridDim.x, &descs[0]->f.stats->wait_faults)) return;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tl = tiles[t];
        const SbBubbleDesc& d = *descs[tl.x];
        if (!reinit_now(d)) continue;
        for (int idx = tl.y + threadIdx.x; idx < tl.y + kBlock && idx < d.g.N; idx += blockDim.x)
            reinit_commit<T>(d.ph, d.f, d.cur, idx);
    }
}

// End of a step: every bubble's map parity flips and its step count
// advances.  A bubble whose frame loop stops at a failed solve
// (halt_on_fail, sb_run) halts here, after the step that failed: the
// kernels of later steps leave it untouched until the host clears the flag.
__global__ void k_flip(SbBubbleDesc* const* descs, int nb) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    SbBubbleDesc* d = descs[b];
    if (d->halted) return;
    d->cur ^= 1;
    SbDevStats* st = d->f.stats;
    st->steps_done += 1;
    if (d->halt_on_fail && !st->solver_converged) d->halted = 1;
    // a bounded wait of the set's cooperative kernels gave up (counted on
    // the set's first member): the barrier word is not trusted any more
    if (descs[0]->f.stats->wait_faults) d->halted = 1;
}

// Self-test of the bounded grid barrier: every block but `absent` waits at
// one barrier of the bubble's barrier word, with a poll limit; with a block
// absent the others give up and count a fault each in the bubble's
// statistics, and the kernel ends.  absent < 0: every block arrives.
__global__ void k_barrier_probe(SbBubbleDesc* d, int absent, unsigned limit) {
    if ((int)blockIdx.x == absent) return;
    unsigned gen = grid_barrier_gen(d->f.bar);
    grid_barrier(d->f.bar, gen, gridDim.x, &d->f.stats->wait_faults, limit);
}

__global__ void k_reset_maps(SbGrid g, SbFields f) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.N) return;
    const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    f.fwd[0][idx] = z; f.fwd[1][idx] = z;
    f.bwd[0][idx] = z; f.bwd[1][idx] = z;
    f.bwdprev[idx] = z;
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Mass integrals sum(eta sin theta), sum(gamma sin theta) for conservation checks.
template <class T>
__global__ void k_mass(SbGrid g, SbPhys ph, SbFields f) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    double me = 0.0, mg = 0.0;
    if (idx < g.N) {
        const double s = (double)g.sin_c[idx >> g.logP];
        me = (double)ld_s<T>(f.eta, idx, ph.base_eta) * s;
        mg = (double)ld_s<T>(f.gam, idx, ph.base_gam) * s;
    }
    me = warp_sum_d(me);
    mg = warp_sum_d(mg);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&f.stats->mass_eta, me);
        atomicAdd(&f.stats->mass_gamma, mg);
    }
}

// FP32 <-> stored type of a thickness or surfactant field (uploads and
// downloads of BF16-stored fields convert on the device).
template <class T>
__global__ void k_store(SbScalar* __restrict__ dst, const float* __restrict__ src, int n, float base) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) st_s<T>(dst, i, src[i], base);
}
template <class T>
__global__ void k_load(float* __restrict__ dst, const SbScalar* __restrict__ src, int n, float base) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = ld_s<T>(src, i, base);
}

// Co-resident grid of the cooperative re-initialisation kernel (both
// instantiations have the same resources; the smaller count is used).
int reinit_blocks() {
    static int cache[16] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    int& b = cache[dev & 15];
    if (b == 0) {
        int sms = 0, p32 = 0, p16 = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p32, k_reinit<float>, kBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p16, k_reinit<__nv_bfloat16>, kBlock, 0);
        const int per = p32 < p16 ? p32 : p16;
        b = sms * (per > 0 ? per : 1);
    }
    return b;
}

}  // namespace

const int kTileSizes[3] = {64, 128, 256};

cudaError_t prepare_plan(const SbStepPlan& P) {
    reinit_blocks();
    return prepare_solve(P.maxNP, P.solver, nullptr);
}

cudaError_t launch_plan_stage(const SbStepPlan& P, int stage, cudaStream_t s) {
    const int k = P.sel[stage];
    const int n = P.ntiles[k], block = kTileSizes[k];
    SbBubbleDesc* const* d = P.descs;
    const int2* t = P.tiles[k];
    const bool bf = P.storage == kStoreBF16;
    switch (stage) {
        case STAGE_MAPS:
            if (bf) k_advect_maps<__nv_bfloat16><<<n, block, 0, s>>>(d, t);
            else k_advect_maps<float><<<n, block, 0, s>>>(d, t);
            break;
        case STAGE_VELOCITY: k_velocity<<<n, block, 0, s>>>(d, t); break;
        case STAGE_BIMOCQ:
            if (bf) k_bimocq<__nv_bfloat16><<<n, block, 0, s>>>(d, t);
            else k_bimocq<float><<<n, block, 0, s>>>(d, t);
            break;
        case STAGE_ASSEMBLE:
            if (P.viscous) k_assemble<true><<<n, block, 0, s>>>(d, t);
            else k_assemble4<<<n, block / 4, 0, s>>>(d, t);
            break;
        case STAGE_SOLVE:
            return P.one ? launch_solve_one(P.one->g, P.one->f, P.set, P.solver, s)
                         : launch_solve(P.set, P.maxNP, P.solver, s);
        case STAGE_POST:
            if (P.viscous) {
                if (bf) k_post<__nv_bfloat16, true><<<n, block, 0, s>>>(d, t);
                else k_post<float, true><<<n, block, 0, s>>>(d, t);
            } else {
                if (bf) k_post4<__nv_bfloat16><<<n, block / 4, 0, s>>>(d, t);
                else k_post4<float><<<n, block / 4, 0, s>>>(d, t);
            }
            break;
        case STAGE_ACCUM:
            if (bf) k_accum<__nv_bfloat16><<<n, block, 0, s>>>(d, t);
            else k_accum<float><<<n, block, 0, s>>>(d, t);
            break;
        case STAGE_REINIT: {
            // the re-initialisation works on kBlock-cell tiles
            SbBubbleDesc* const* dd = P.descs;
            int nb = P.nb;
            const int2* tt = P.tiles[1];
            int nt = P.ntiles[1];
            unsigned* gb = P.set.bar;
            void* args[] = {&dd, &nb, &tt, &nt, &gb};
            const void* fn = bf ? (const void*)k_reinit<__nv_bfloat16> : (const void*)k_reinit<float>;
            return cudaLaunchCooperativeKernel(fn, dim3(reinit_blocks()), dim3(kBlock), args, 0, s);
        }
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_barrier_probe(SbBubbleDesc* d, int blocks, int absent, unsigned limit,
                                 cudaStream_t s) {
    void* args[] = {&d, &absent, &limit};
    return cudaLaunchCooperativeKernel((const void*)k_barrier_probe, dim3(blocks), dim3(kBlock), args,
                                       0, s);
}

cudaError_t launch_plan_flip(const SbStepPlan& P, cudaStream_t s) {
    k_flip<<<(P.nb + 127) / 128, 128, 0, s>>>(P.descs, P.nb);
    return cudaGetLastError();
}

cudaError_t launch_plan_step(const SbStepPlan& P, cudaStream_t s) {
    for (int st = 0; st < STAGE_COUNT; ++st) {
        cudaError_t e = launch_plan_stage(P, st, s);
        if (e != cudaSuccess) return e;
    }
    return launch_plan_flip(P, s);
}

cudaError_t launch_reset_maps(const SbGrid& g, const SbFields& f, cudaStream_t s) {
    k_reset_maps<<<(g.N + kBlock - 1) / kBlock, kBlock, 0, s>>>(g, f);
    return cudaGetLastError();
}

cudaError_t launch_mass(const SbGrid& g, const SbPhys& ph, const SbFields& f, int storage,
                        cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(&f.stats->mass_eta, 0, 2 * sizeof(double), s);
    if (e != cudaSuccess) return e;
    const int nb = (g.N + kBlock - 1) / kBlock;
    if (storage == kStoreBF16) k_mass<__nv_bfloat16><<<nb, kBlock, 0, s>>>(g, ph, f);
    else k_mass<float><<<nb, kBlock, 0, s>>>(g, ph, f);
    return cudaGetLastError();
}

cudaError_t launch_store(SbScalar* dst, const float* src, int n, float base, int storage,
                         cudaStream_t s) {
    const int nb = (n + kBlock - 1) / kBlock;
    if (storage == kStoreBF16) k_store<__nv_bfloat16><<<nb, kBlock, 0, s>>>(dst, src, n, base);
    else k_store<float><<<nb, kBlock, 0, s>>>(dst, src, n, base);
    return cudaGetLastError();
}

cudaError_t launch_load(float* dst, const SbScalar* src, int n, float base, int storage,
                        cudaStream_t s) {
    const int nb = (n + kBlock - 1) / kBlock;
    if (storage == kStoreBF16) k_load<__nv_bfloat16><<<nb, kBlock, 0, s>>>(dst, src, n, base);
    else k_load<float><<<nb, kBlock, 0, s>>>(dst, src, n, base);
    return cudaGetLastError();
}

}  // namespace sb
