// Plain-data structures shared by host and device code.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sb {

// Grid geometry and per-row trigonometric tables of one bubble.
struct SbGrid {
    int nT, nP, maskP, logP;  // nTheta, nPhi = 2 nTheta (power of two)
    int N, Nv;                // nT*nP cells, (nT-1)*nP u_theta faces
    float h, invh;            // pi / nT and its inverse
    const float* sin_c;       // sin((i + 0.5) h), i < nT
    const float* cos_c;
    const float* sin_e;       // sin(i h), i <= nT (row edges; u_theta faces at i + 1)
    const float* cos_e;
    // tables of the characteristic-map geometry (FP64 values rounded on the host):
    const float4* rowtab;     // per row i < nT: sin and cos of (i + 0.5) h as (hi, lo) pairs:
                              // (sin hi, sin lo, cos hi, cos lo)
    const float2* rottab;     // per column offset dc in [-nT, nT) at index dc + nT:
                              // (sin(dc h), cos(dc h) - 1)
};

// Scalars that change per step (kept in device memory so a captured graph
// can be replayed with new values).
struct SbStepParams {
    float dt;       // nondimensional step (timeStepGlobal)
    float invDt;
    float windg;    // air-flow corridor time factor 3 - |t - 3|
    float mixA;     // t / 12 (mirrored wind mix, kernel/bubble.cu:1360-1392)
    float mixB;     // 1 - t / 12
    float evapDt;   // evaporationRate * dt
    float pad[2];   // the struct stays 32 bytes
};

// Storage of the thickness and surfactant fields (the values of
// SB_STORE_FP32 / SB_STORE_BF16 in the public header).
enum { kStoreF32 = 0, kStoreBF16 = 1 };

// Constant physical coefficients of one bubble.
struct SbPhys {
    float M, Cr, gs, gmax, blend, evap;
    float gthr;       // gamma above gthr is at its maximum gmax (the cell is broken)
    float base_eta, base_gam;  // BF16 storage: offsets of the eta and gamma fields (else 0)
    int plain_adv;    // 1: thickness advected like gamma, no characteristic maps (BIMOCQ off)
    int single_step;  // 1: velocity traced in one step (RUNGE_KUTTA off)
    int viscous;      // 1: viscous stress forces in the system and the velocity update
    float re;         // nu / (U r), the film's inverse Reynolds number
};

// Per-step diagnostics written by the kernels.
struct SbDevStats {
    unsigned int distortion_bits;  // max distortion (float bits, non-negative)
    int reinit;                    // 1 when this step re-initialised the maps
    int solver_iters;
    int broken_cells;
    double solver_rel_resid;
    double solver_b_norm;
    int solver_converged;
    int force_reinit;              // -1 decide, 0 never, 1 always
    double mass_eta;               // sum eta * sin(theta)
    double mass_gamma;
    long long reinit_total;        // re-initialisations since creation
    int wait_faults;               // bounded waits that gave up (copy never landed)
    int solver_neumann;            // 1: the last solve used the Neumann term
    long long solves;              // implicit solves since creation
    long long solver_nonconverged; // solves that missed their tolerance since the last reset
    double solver_resid_max;       // largest relative residual since the last reset
    long long steps_done;          // steps completed (map parity flips) since creation
    int dx_valid;                  // 1: dx holds the last solve's increment of this state
                                   // (the next solve starts from it); uploads clear it
    int pad_;
};

}  // namespace sb
