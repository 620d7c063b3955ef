// Internal declarations shared by the CUDA translation units and the C ABI.
#pragma once
#include <cuda_runtime.h>

#include "sb_types.h"

namespace sb {

// Every device array of one bubble.  Fields are FP32, row-major [theta][phi]
// with row stride nPhi; u_theta has nTheta-1 rows.  "A" buffers hold the
// state between steps, "adv" buffers the advected intermediate state.
struct SbFields {
    float *eta, *gam, *uth, *uph;                  // state
    float *eta_adv, *gam_adv, *uth_adv, *uph_adv;  // after advection
    float *eta_init, *eta_delta, *eta_initL, *eta_deltaL;
    float *gam_init, *gam_delta, *gam_initL, *gam_deltaL;
    float2 *fwd[2], *bwd[2], *bwdprev;             // map offsets (ping-pong)
    float *uair_init, *vair_init, *corr_u, *corr_v;
    float *uair, *vair;                            // N+1, Nv+1 (last element 0)
    float *div, *d_eta, *d_gam, *err_eta, *err_gam;
    // implicit system for the increment dx = gamma_new - gamma_adv:
    // (A dx)_c = dmass_c dx_c + sum_n w_cn (dx_c - dx_n), weights w > 0 to
    // the east (cE) and south (cS) neighbours; r = b - A gamma_adv formed
    // analytically; rhs = b (for the norm only)
    float *dmass, *cE, *cS, *rhs, *r0;
    float *x, *dx, *r, *z, *p, *q;                 // solver vectors
    double *x64;                                   // mixed-precision iterate
    float2 *pcr;                                   // phi-line factors, (log2 nPhi) x N
    int *pcr_levels;                               // reduction levels per row
    double *partials;                              // per-block reduction slots
    SbStepParams* step;                            // device copy of step scalars
    SbDevStats* stats;
};

// One bubble of a batch, as the batched kernels see it (device memory).
struct SbBubbleDesc {
    SbGrid g;
    SbPhys ph;
    SbFields f;
    int cur;   // map parity, flipped on the device after every batch step
    int pad;
};

struct SolverConfig {
    int mode;       // 0: plain FP32, 1: mixed precision (FP64 dots + refinement)
    int max_iter;
    double tol;     // relative residual ||b - A x|| / ||b||
    int precond;    // 0: Jacobi, 1: exact phi-line (periodic tridiagonal per row)
};

// Step stages in launch order (sb_step.cu, sb_solver.cu).  `cur` selects the
// map ping-pong buffers.  Each stage is one kernel launch.
enum SbStage {
    STAGE_MAPS = 0,   // k_advect_maps: characteristic maps, gamma, air flow
    STAGE_VELOCITY,   // k_velocity: u_theta / u_phi self-advection
    STAGE_BIMOCQ,     // k_bimocq: thickness through the composed maps
    STAGE_ASSEMBLE,   // k_assemble: implicit surfactant system
    STAGE_SOLVE,      // k_pcg: cooperative PCG
    STAGE_POST,       // k_post: forces, thickness, increments
    STAGE_ACCUM,      // k_accum: BIMOCQ accumulation + distortion
    STAGE_REINIT,     // k_reinit: conditional map re-initialisation (cooperative)
    STAGE_COUNT
};

cudaError_t launch_stage(int stage, const SbGrid& g, const SbPhys& ph, const SbFields& f,
                         const struct SolverConfig& cfg, int cur, cudaStream_t s);
// Occupancy queries and function attributes of the cooperative kernels, done
// once before any stream capture.
cudaError_t prepare_launches(const SbGrid& g, const struct SolverConfig& cfg);
cudaError_t prepare_solve(const SbGrid& g, const struct SolverConfig& cfg);
cudaError_t launch_reset_maps(const SbGrid& g, const SbFields& f, cudaStream_t s);
cudaError_t launch_mass(const SbGrid& g, const SbFields& f, cudaStream_t s);

// Batched stages: one launch per stage over the tiles of every bubble.
// tiles[k] = (bubble, first cell) of block k; `block` threads per tile.
cudaError_t launch_stage_batch(int stage, const SbBubbleDesc* descs, const int2* tiles, int ntiles,
                               int block, cudaStream_t s);
cudaError_t launch_reinit_batch(const SbBubbleDesc* descs, int nb, const int2* tiles, int ntiles,
                                cudaStream_t s);
cudaError_t launch_flip_batch(SbBubbleDesc* descs, int nb, cudaStream_t s);
int reinit_batch_blocks();

// Batched implicit solve: every bubble's rows are owned by its own
// contiguous range of blocks.
struct SbBatchSolve {
    const SbBubbleDesc* descs;
    int nb;
    const int* blk_bubble;     // [G] bubble of each block
    const int* bub_first_blk;  // [nb]
    const int* bub_nblk;       // [nb]
    double* partials;          // [2 * 3 * G]
    int* nactive;              // [3] bubbles still iterating (rotating counters)
};
cudaError_t prepare_solve_batch(int maxNP, const SolverConfig& cfg, int* blocks);
cudaError_t launch_solve_batch(const SbBatchSolve& bs, int G, int maxNP, const SolverConfig& cfg,
                               cudaStream_t s);

// Implicit surfactant solve (sb_solver.cu).
cudaError_t launch_solve(const SbGrid& g, const SbPhys& ph, const SbFields& f,
                         const SolverConfig& cfg, cudaStream_t s);
int solver_partials_needed(const SbGrid& g);

}  // namespace sb
