// Internal declarations shared by the CUDA translation units and the C ABI.
#pragma once
#include <cuda_runtime.h>

#include "sb_types.h"

namespace sb {

struct SbBubbleDesc;
struct SbSolveRec;

// Byte layout of one row's phi-line preconditioner factors (sb_solver.cu)
// for rows of n = nPhi columns (a power of two, >= 16): q = n / 4 reduced
// equations and up to lp parallel-reduction levels.  Every offset is a
// multiple of 16 bytes.
struct SbFactorBlob {
    int n, q, lp;
    int cr1, cr2, pcr, fin, bs2, bs1, bytes;
};

__host__ __device__ inline SbFactorBlob factor_blob(int n) {
    SbFactorBlob b;
    b.n = n;
    b.q = n / 4;
    int lq = 0;
    while ((1 << lq) < b.q) ++lq;
    b.lp = lq > 1 ? lq - 1 : 0;
    b.cr1 = 0;                      // float2 [n/2]
    b.cr2 = 4 * n;                  // float2 [q]
    b.pcr = 6 * n;                  // float2 [lp][q]
    b.fin = b.pcr + 2 * n * b.lp;   // float2 [q]
    b.bs2 = b.fin + 2 * n;          // float [3][q]
    b.bs1 = b.bs2 + 3 * n;          // float [3][n/2]
    b.bytes = b.bs1 + 6 * n;
    return b;
}

// Every device array of one bubble.  Fields are FP32, row-major [theta][phi]
// with row stride nPhi; u_theta has nTheta-1 rows.  "A" buffers hold the
// state between steps, "adv" buffers the advected intermediate state.
// The thickness and surfactant fields that persist between steps (eta,
// gamma and the BIMOCQ reference fields eta/gamma_init and _initL) are
// stored as FP32 or, per bubble, as BF16 (SbScalar: an opaque element
// type; kernels read and write them through ld_s / st_s with the storage
// type as a template argument and do their arithmetic in FP32).  The BIMOCQ
// change accumulators (the _delta buffers) stay FP32 in both: they grow by
// small increments every step, which BF16 would round away.
struct SbScalar;

struct SbFields {
    SbScalar *eta, *gam;                           // state (stored type)
    float *uth, *uph;
    float *eta_adv, *gam_adv, *uth_adv, *uph_adv;  // after advection
    SbScalar *eta_init, *eta_initL, *gam_init, *gam_initL;
    float *eta_delta, *eta_deltaL, *gam_delta, *gam_deltaL;
    // characteristic maps (ping-pong): per cell the mapped point's
    // displacement from the cell centre in the cell's own frame (x, y, z, 0),
    // see sb_device.cuh
    float4 *fwd[2], *bwd[2], *bwdprev;
    float *uair_init, *vair_init, *corr_u, *corr_v;
    float *uair, *vair;                            // N+1, Nv+1 (last element 0)
    float *d_eta, *d_gam, *err_eta, *err_gam;  // per-step increments, re-initialisation errors
    // implicit system for the increment dx = gamma_new - gamma_adv:
    // (A dx)_c = dmass_c dx_c + sum_n w_cn (dx_c - dx_n), weights w > 0 to
    // the east (cE) and south (cS) neighbours; r = b - A gamma_adv formed
    // analytically; rhs = b (for the norm only)
    float *dmass, *cE, *cS, *rhs, *r0;
    float *x, *dx, *r, *z, *z1, *p, *q;            // solver vectors
    float2 *xff;                                   // mixed-precision iterate (float-float)
    float *pcr;                                    // phi-line factors, one blob per row
    int *pcr_levels;                               // reduction levels per row
    // the bubble's own solve set (one system): its device descriptor and
    // the solver's per-row and per-system scratch (see SbSolveSet)
    SbBubbleDesc* self;
    int *roff, *done_at, *cnt;
    SbSolveRec* rec;
    unsigned long long* acc;
    unsigned* bar;                                 // grid barrier words of its cooperative launches
    SbStepParams* step;                            // device copy of step scalars
    SbDevStats* stats;
};

// One bubble as the kernels see it (device memory, one per bubble, shared
// by every set that steps the bubble).
struct SbBubbleDesc {
    SbGrid g;
    SbPhys ph;
    SbFields f;
    int cur;           // map parity, flipped on the device at the end of every step
    int halted;        // 1: the kernels leave this bubble untouched (set by k_flip)
    int halt_on_fail;  // 1: a step whose solve missed its tolerance halts the bubble
                       // (the frame loop of sb_run stops at that step, as Bubble::run)
    int pad;
};

// Preconditioner of the implicit solve: the exact phi-line blocks B alone,
// with the Neumann term B^-1 C B^-1 added (C: the theta couplings), or
// chosen per solve from the previous solve's iteration count.
enum { kPrecLine = 1, kPrecNeumann = 2, kPrecAuto = 3 };

struct SolverConfig {
    int mode;       // 0: plain FP32, 1: mixed precision (FP64 dots + refinement)
    int max_iter;
    double tol;     // relative residual ||b - A x|| / ||b||
    int precond;    // kPrecLine, kPrecNeumann or kPrecAuto (sb_solver.cu)
    int warm;       // 1: start from the previous increment when it is valid (row_init)
    int blob;       // bytes of a block's shared-memory factor blob (set at launch)
    float tol2f;    // target r.r / |b|^2 of the iterate (set at launch)
};

// Step stages in launch order (sb_step.cu, sb_solver.cu).  `cur` selects the
// map ping-pong buffers.  Each stage is one kernel launch; a step ends with a
// flip of every bubble's map parity (one more launch).
enum SbStage {
    STAGE_MAPS = 0,   // k_advect_maps: characteristic maps, gamma, air flow
    STAGE_VELOCITY,   // k_velocity: u_theta / u_phi self-advection
    STAGE_BIMOCQ,     // k_bimocq: thickness through the composed maps
    STAGE_ASSEMBLE,   // k_assemble: implicit surfactant system
    STAGE_SOLVE,      // k_solve: cooperative PCG
    STAGE_POST,       // k_post: forces, thickness, increments
    STAGE_ACCUM,      // k_accum: BIMOCQ accumulation + distortion
    STAGE_REINIT,     // k_reinit: conditional map re-initialisation (cooperative)
    STAGE_COUNT
};

cudaError_t launch_reset_maps(const SbGrid& g, const SbFields& f, cudaStream_t s);
cudaError_t launch_mass(const SbGrid& g, const SbPhys& ph, const SbFields& f, int storage,
                        cudaStream_t s);
// FP32 <-> stored thickness / surfactant field (n elements, offset `base`).
cudaError_t launch_store(SbScalar* dst, const float* src, int n, float base, int storage,
                         cudaStream_t s);
cudaError_t launch_load(float* dst, const SbScalar* src, int n, float base, int storage,
                        cudaStream_t s);

// Scalars of one system of a solve, written by the block that completes the
// system's last row in a phase and read in the next phase (double buffered).
// Scalars of one system's conjugate-gradient iteration; float-float values
// are stored as (hi, lo) pairs.
struct SbSolveRec {
    float2 rz, rr, bb, tol2, alpha;  // r.z, r.r, |b|^2, target for r.r, step length
    float beta;
    int kind;   // the kind of the system's next phase (sb_solver.cu)
    int fresh;  // the next r.z starts a new search direction
    int it;
    int conv;
    int neu;    // 1: the preconditioner adds the Neumann term (chosen at set-up)
    int pad;
};

// Words of a system's exact dot-product accumulators: three buffers (used
// in rotation by phase) of three values of 10 fixed-point chunks and a flag.
constexpr int kSolveAccWords = 3 * 3 * 16;  // 3 buffers x 3 values x one 128-byte line
constexpr int kGridBarWords = 32;           // grid barrier word on its own 128-byte line (sb_sync.cuh)

// A set of implicit systems solved by one cooperative launch: the system of
// one bubble, or the systems of every bubble of a batch (at most 1024, with
// sum over systems of nT (2 nT + 256) below 2^32).  Device arrays.
struct SbSolveSet {
    SbBubbleDesc* const* descs;  // [nb] device pointers to each bubble's descriptor
    int nb;
    int R;                      // theta rows of all systems
    const int* roff;            // [nb + 1] first row of each system in the row list
    SbSolveRec* rec;            // [2 * nb]
    int* done_at;               // [nb] first phase in which the system is finished
    int* cnt;                   // [nb] rows completed in the current phase (0 between launches)
    unsigned long long* acc;    // [nb][kSolveAccWords] exact dot-product accumulators (0 between launches)
    unsigned* bar;              // [kGridBarWords] grid barrier of the cooperative launches
                                // (sb_sync.cuh; zeroed at creation)
};

// Implicit surfactant solve (sb_solver.cu).  prepare_solve sets the kernel
// attributes for rows of up to maxNP columns and returns the co-resident
// block count; call it before any stream capture.
cudaError_t prepare_solve(int maxNP, const SolverConfig& cfg, int* max_blocks);
cudaError_t launch_solve(const SbSolveSet& set, int maxNP, const SolverConfig& cfg,
                         cudaStream_t s);
// The same solve for a set of one system, with the descriptor passed as
// kernel parameters (bit-identical results).
cudaError_t launch_solve_one(const SbGrid& g, const SbFields& f, const SbSolveSet& set,
                             const SolverConfig& cfg, cudaStream_t s);

// Cells per block of the three tile sizes the stage kernels can use.
extern const int kTileSizes[3];

// Everything one step launches over a set of bubbles (one bubble, or every
// bubble of a batch; sb_step.cu).  Device arrays: descs[k] points to bubble
// k's own descriptor, so a bubble has one map parity whichever set steps it.
struct SbStepPlan {
    SbBubbleDesc* const* descs;  // [nb]
    int nb;
    const int2* tiles[3];        // (bubble, first cell) of every tile, per tile size
    int ntiles[3];
    int sel[STAGE_COUNT];        // tile size (index into kTileSizes) of every stage
    SbSolveSet set;              // every bubble's implicit system
    int maxNP;                   // widest grid of the set
    SolverConfig solver;
    int storage;                 // SB_STORE_FP32 or SB_STORE_BF16 (the same for every bubble)
    int viscous;                 // 1: viscous forces on (the same for every bubble)
    const SbBubbleDesc* one;     // host copy of the descriptor of a set of one bubble, else null
};

// Occupancy queries and kernel attributes; call before any stream capture.
cudaError_t prepare_plan(const SbStepPlan& P);
// One stage of a step, the map-parity flip that ends a step, or the whole step.
cudaError_t launch_plan_stage(const SbStepPlan& P, int stage, cudaStream_t s);
cudaError_t launch_plan_flip(const SbStepPlan& P, cudaStream_t s);
cudaError_t launch_plan_step(const SbStepPlan& P, cudaStream_t s);
// Self-test of the bounded grid barrier on a bubble's barrier word (`blocks`
// co-resident blocks, block `absent` never arrives; sb_step.cu).
cudaError_t launch_barrier_probe(SbBubbleDesc* d, int blocks, int absent, unsigned limit,
                                 cudaStream_t s);

}  // namespace sb
