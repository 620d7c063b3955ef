/*
 * soapbubble_gb300 -- C ABI of the GB300 soap-bubble time step.
 *
 * The reference (RiverIntheSky/SoapBubble) has no plugin or FFI layer: its
 * step is reached through the C++ classes Bubble (include/bubble.cuh:36-89,
 * constructor + run()), Solver (include/solver.cuh:15-150, stepForward() at
 * kernel/solver.cu:260-292) and Quantity (include/quantity.cuh:5-96, host
 * buffers indexed [theta][phi]).  These entry points replace that surface;
 * each declaration names the reference interface it stands in for.
 *
 * Conventions
 *   - Every function returns an sb_status (0 = success); sb_last_error()
 *     gives a message for the calling thread.  Nothing calls exit().
 *   - Host arrays are row-major [theta][phi] with row stride nPhi, exactly the
 *     reference's host buffers (kernel/quantity.cu:94-97): centred fields and
 *     u_phi have nTheta rows, u_theta has nTheta-1 rows.
 *   - Each handle owns its device memory and its CUDA stream.  Calls on
 *     different handles may run from different threads; calls on one handle
 *     must not overlap.
 */
#ifndef SOAPBUBBLE_GB300_H
#define SOAPBUBBLE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SB_OK = 0,
    SB_ERR_INVALID = 1,      /* bad argument or configuration */
    SB_ERR_CUDA = 2,         /* CUDA runtime error */
    SB_ERR_OOM = 3,          /* device allocation failed */
    SB_ERR_NOT_CONVERGED = 4,/* implicit solve missed its tolerance */
    SB_ERR_BROKEN = 5,       /* film broken (no thickness left) */
    SB_ERR_IO = 6            /* file output failed */
} sb_status;

/* The 17 keys of the reference's config.txt (kernel/main.cu:20-36) plus
 * solver and storage options.  Bubble::Bubble (kernel/bubble.cu:2568-2603)
 * derives the nondimensional coefficients from these. */
typedef struct {
    double radius;        /* m */
    double H;             /* mean half film thickness, m */
    double U;             /* characteristic velocity; the reference forces 1 */
    double c_m;           /* bulk concentration (unused by the step) */
    double Gamma_m;       /* surface mean concentration, mol m^-2 */
    double T;             /* temperature, K */
    double Ds;            /* soap diffusivity (unused by the step) */
    double rm;            /* Lennard-Jones distance (van der Waals is off) */
    int nTheta;           /* numberOfGridsInTheta; nPhi = 2 nTheta, a power of two */
    double dt;            /* timePerStep, s */
    double DT;            /* timePerFrame, s */
    int frames;           /* frameNumbers */
    double blendCoeff;    /* BIMOCQ blend */
    int device;           /* CUDA device ordinal */
    /* extensions (zero selects the default) */
    double gs_scale;      /* multiplies the nondimensional gravity (0 -> 1) */
    double M_scale;       /* multiplies the Marangoni coefficient M (0 -> 1) */
    int solver_mode;      /* 0: mixed precision (float-float iterate, exact dot-product sums,
                             true-residual refinement), 1: plain FP32 */
    double solver_tol;    /* relative residual target (0 -> 1e-6) */
    int solver_max_iter;  /* (0 -> 1000) */
    int force_reinit;     /* 0: decide by distortion > 4; 1: never; 2: every step */
    double nu_scale;      /* multiplies the air's kinematic viscosity in the drag
                             coefficient Cr (0 -> 1) */
    int storage;          /* SB_STORE_FP32 (0) or SB_STORE_BF16 (1): storage of the thickness
                             and surfactant fields between steps (eta, gamma and the BIMOCQ
                             reference fields *_init, *_init_last; the *_delta accumulators
                             stay FP32); arithmetic is FP32 either way */
    /* the reference's compile-time switches as runtime options (include/header.cuh:89-97) */
    int plain_advection;      /* 1: as without BIMOCQ: thickness advected like gamma
                                 (advectionAllCentered, kernel/bubble.cu:937-961), no
                                 characteristic maps updated, no re-initialisation */
    int single_step_velocity; /* 1: as without RUNGE_KUTTA: the velocity advection traces in
                                 one step (kernel/bubble.cu:689-730 skipped) */
    int viscous;              /* 1: as with VISCOUS: viscous stress forces of the film
                                 (kernel/bubble.cu:1218-1269, 1512-1816) enter the surfactant
                                 system in place of the gravity term (1460-1466) and the
                                 velocity update (1940-2038); gravity is part of the force */
    int write_velocity_frames;      /* sb_run also writes vel%04d.exr (WRITE_VELOCITY_DATA,
                                       kernel/bubble.cu:2646-2648, 2689-2691) */
    int write_concentration_frames; /* sb_run also writes con%04d.exr (WRITE_CONCENTRATION_DATA,
                                       kernel/bubble.cu:2649-2651, 2692-2694) */
    int solver_precond;       /* preconditioner of the implicit solve: 0 chooses per solve
                                 from the previous solve's iterations, 1 the exact phi-line
                                 blocks B alone, 2 B^-1 + B^-1 C B^-1 (C: the theta couplings) */
    int solver_cold_start;    /* 1: every solve starts from a zero increment (gamma_new =
                                 the advected gamma, as the reference's AmgX call starts from
                                 gamma); 0: from the previous step's increment after a
                                 converged solve of an unchanged state */
} sb_params;

enum { SB_STORE_FP32 = 0, SB_STORE_BF16 = 1 };

/* Diagnostics of the most recent step (the reference prints these:
 * kernel/solver.cu:282, kernel/bubble.cu:1495-1497, solver.cu:592). */
typedef struct {
    double distortion;        /* max BIMOCQ distortion, grid units */
    int reinit;               /* maps re-initialised in the last step */
    int solver_iters;
    double solver_rel_resid;  /* ||b - A x|| / ||b|| of the returned gamma (rows scaled by
                                 the range guard of sb_download_system enter scaled) */
    int solver_converged;
    int broken_cells;         /* identity rows of the implicit system */
    long long steps;          /* steps taken by this handle */
    long long reinits;        /* re-initialisations so far */
    double mass_eta;          /* sum eta sin(theta) (after sb_update_mass) */
    double mass_gamma;        /* sum gamma sin(theta) */
    long long launches;       /* CUDA kernels launched by this handle */
    int solver_precond_used;  /* preconditioner of the last solve: 1 phi-line blocks,
                                 2 with the Neumann term */
    long long solves;         /* implicit solves since creation */
    long long solver_nonconverged;  /* solves that missed their tolerance (iteration
                                       limit, breakdown or NaN) since sb_reset_stats */
    double solver_rel_resid_max;    /* largest relative residual of the solves since
                                       sb_reset_stats (NaN once a solve met NaN) */
} sb_stats;

typedef struct sb_bubble sb_bubble;

/* Field selectors for sb_upload_field / sb_download_field. */
typedef enum {
    SB_ETA = 0, SB_GAMMA, SB_UTHETA, SB_UPHI,
    SB_ETA_INIT, SB_ETA_DELTA, SB_ETA_INIT_LAST, SB_ETA_DELTA_LAST,
    SB_GAMMA_INIT, SB_GAMMA_DELTA, SB_GAMMA_INIT_LAST, SB_GAMMA_DELTA_LAST,
    SB_FWD_T, SB_FWD_P, SB_BWD_T, SB_BWD_P, SB_BWDPREV_T, SB_BWDPREV_P,
    SB_UAIR_INIT, SB_VAIR_INIT, SB_UAIR, SB_VAIR,
    SB_FIELD_COUNT
} sb_field;

/* Fill p with the reference's defaults (config.txt, include/bubble.cuh:78-84). */
void sb_default_params(sb_params* p);

/* Replaces Solver::Solver (kernel/solver.cu:63-160) and the constant upload of
 * Bubble::run (kernel/bubble.cu:2609-2638): allocates every device buffer of
 * one bubble, initialises eta = 0.5, gamma = 1, u = 0, identity maps
 * (kernel/initializer.cu:22-50, solver.cu:102-106, 145-160). */
int sb_create(const sb_params* p, sb_bubble** out);

/* Replaces Solver::~Solver (kernel/solver.cu:163-215). */
int sb_destroy(sb_bubble* b);

/* Replaces initThicknessfromPic / initAirflowfromPic / initWithConst
 * (kernel/initializer.cu:22-135): uploads the initial state from host FP64
 * arrays in the reference layout.  Any pointer may be NULL (field kept).
 * Resets the BIMOCQ buffers (init = initLast = field, delta = deltaLast = 0)
 * and the characteristic maps to identity. */
int sb_upload_fields(sb_bubble* b, const double* eta, const double* gamma,
                     const double* u_theta, const double* u_phi,
                     const double* uair_init, const double* vair_init);

/* Replaces Solver::initThicknessfromPic (kernel/initializer.cu:50-99):
 * thickness from the first channel (B) of an uncompressed scanline EXR,
 * resampled to nPhi x nTheta with half-pixel-centred bilinear weights
 * (cv::resize INTER_LINEAR), rescaled as eta = (C - 0.5) * 0.3 + 0.5; the
 * BIMOCQ buffers and the maps restart from it.  An empty path keeps
 * eta = 0.5 (SB_OK); an unreadable file keeps the current thickness and
 * returns SB_ERR_IO (the reference prints a message and continues). */
int sb_init_thickness_from_exr(sb_bubble* b, const char* path);

/* Replaces Solver::initAirflowfromPic (kernel/initializer.cu:101-135): the
 * initial wind from channels G (phi) and R (theta) of the resampled
 * texture, averaged onto the u_phi and u_theta faces and scaled by the
 * radius: uair = 0.5 (G(j,i) + G(j,i-1)) r, vair = -0.5 (R(j,i) + R(j+1,i)) r.
 * Empty path: zero wind (SB_OK); unreadable file: SB_ERR_IO, wind kept. */
int sb_init_airflow_from_exr(sb_bubble* b, const char* path);

/* Host utility (no device work): one channel of an uncompressed EXR
 * resampled to width x height as above, into out (width * height values). */
int sb_exr_load_resized(const char* path, const char* channel, int width, int height,
                        double* out);

/* Replaces Quantity::copyToGPU for any single buffer (kernel/quantity.cu:3-11),
 * including BIMOCQ buffers and maps (absolute grid coordinates theta/h,
 * phi/h as the reference's forward_t/forward_p).  n = element count. */
int sb_upload_field(sb_bubble* b, sb_field which, const double* src, size_t n);

/* Replaces Quantity::copyBackToCPU / Solver::copyToCPU (kernel/quantity.cu:14-18,
 * solver.cu:243-249) for any buffer; maps come back in absolute coordinates. */
int sb_download_field(sb_bubble* b, sb_field which, double* dst, size_t n);

/* Element count of a field. */
size_t sb_field_size(const sb_bubble* b, sb_field which);

/* The implicit surfactant system of the most recent step, for inspection
 * (the reference keeps its matrix inside AmgX: val/rhs of
 * Bubble::concentrationLinearSystem, kernel/bubble.cu:1301-1473).  The
 * library solves it for the increment dx = gamma_new - gamma_adv:
 *   (A dx)_c = dmass_c dx_c + sum_n w_cn (dx_c - dx_n),  A dx = r0,
 * whose dx is 0 in broken cells.  The reference's row c of an unbroken cell
 * is then: diagonal sin(theta)/(dt gamma_adv) + sum over all four
 * neighbours of w_cn, off-diagonal -w_cn; dmass_c holds the first term
 * plus the weights towards broken neighbours, and the stored east/south
 * weights are 0 across a broken cell.  A broken cell has dmass 1, no
 * weights, r0 0 and gamma_adv gmax (the reference's identity row).  A cell
 * left with almost no surfactant, whose term t = sin(theta) / (dt gamma_adv)
 * exceeds 2^48, has its row and column scaled by s = 2^-k (2^45 < t s^2 <=
 * 2^48; FP32 range guard, exact): its dmass, weights and r0 here are the
 * scaled ones, its dx is not.  Each array has nTheta * nPhi elements,
 * row-major. */
typedef enum {
    SB_SYS_ETA_ADV = 0,  /* advected thickness */
    SB_SYS_GAMMA_ADV,    /* advected concentration (gmax in broken cells) */
    SB_SYS_DMASS,        /* diagonal excess (sin(theta) / (dt gamma_adv) + broken couplings) */
    SB_SYS_WEAST,        /* coupling weight to the east neighbour (0 if either is broken) */
    SB_SYS_WSOUTH,       /* coupling weight to the south neighbour */
    SB_SYS_R0,           /* r0 = b - A gamma_adv */
    SB_SYS_RHS,          /* b */
    SB_SYS_DX,           /* the solved increment, FP32-rounded */
    SB_SYS_COUNT
} sb_system_array;
int sb_download_system(sb_bubble* b, sb_system_array which, double* dst, size_t n);

/* Replaces Solver::stepForward(dt) (kernel/solver.cu:252-292) called
 * n_steps times with currentTimeGlobal = t_frame (s) and the dimensional
 * step dt (s) -- Bubble::run keeps t at the frame start for every step of a
 * frame (kernel/bubble.cu:2661-2678).  Asynchronous on the handle's stream
 * unless an error must be reported. */
int sb_step(sb_bubble* b, int n_steps, double t_frame, double dt);

/* sb_step with CUDA events between the kernels of every step: adds each
 * stage's device time (ms) to stage_ms[0 .. sb_stage_count()-1] and
 * synchronises after each step.  Same results as sb_step.  The reference
 * times its phases with cudaEvent timers (kernel/solver.cu:261-279). */
int sb_step_timed(sb_bubble* b, int n_steps, double t_frame, double dt, double* stage_ms);

/* Picks, per stage, the tile size (64, 128 or 256 cells per block) with the
 * shortest device time, from one timed step at each size; tile_sizes
 * (optional, sb_stage_count() ints) receives the choice.  The three tuning
 * steps advance the bubble like sb_step_timed.  Results do not depend on
 * the tile sizes.  No counterpart in the reference. */
int sb_autotune(sb_bubble* b, double t_frame, double dt, int* tile_sizes);

/* Number of kernel stages of one step, and the kernel name of a stage.  A
 * step launches one kernel per stage plus one that flips the map parity. */
int sb_stage_count(void);
const char* sb_stage_name(int stage);

/* Asynchronous FP32 copies between a caller's host buffer (pinned for true
 * overlap) and one non-map field, ordered on the handle's stream; the
 * caller synchronises (sb_synchronize) before reading dst or reusing src.
 * The FP32 counterparts of Quantity::copyToGPU / copyBackToCPU
 * (kernel/quantity.cu:3-18). */
int sb_upload_field_f32(sb_bubble* b, sb_field which, const float* src, size_t n);
int sb_download_field_f32(sb_bubble* b, sb_field which, float* dst, size_t n);

/* Wait for the handle's queued work; returns SB_ERR_NOT_CONVERGED if the
 * last solve missed its tolerance (the reference's AmgX status check,
 * kernel/bubble.cu:1498-1507). */
int sb_synchronize(sb_bubble* b);

/* Self-test of the bounded wait of the grid barrier that the cooperative
 * kernels (implicit solve, map re-initialisation) synchronise with.  Four
 * co-resident blocks meet at one barrier on the bubble's barrier word; block
 * absent_block (0..3) never arrives, so the others give up after poll_limit
 * polls (1 .. 2^22; the kernels' own limit is 2^22, about a second) and each
 * counts a fault.  Afterwards sb_get_stats returns SB_ERR_CUDA, the bubble's
 * cooperative kernels return at once and the bubble halts at the end of its
 * next step, exactly as after a real give-up.  absent_block = -1: every
 * block arrives and nothing is counted.  Synchronises.  No counterpart in
 * the reference, whose kernels never wait on one another. */
int sb_selftest_grid_barrier(sb_bubble* b, int absent_block, unsigned poll_limit);

/* Restarts the running solver statistics of sb_stats (solver_nonconverged
 * and solver_rel_resid_max) from zero; synchronises.  No counterpart in the
 * reference, which prints each solve's outcome (kernel/bubble.cu:1495-1497). */
int sb_reset_stats(sb_bubble* b);

/* Staged I/O beside the steps (no counterpart in the reference, whose frame
 * loop copies synchronously).  Copies run on the handle's own copy stream
 * through per-field FP32 device buffers, so they overlap the kernels queued
 * on the compute stream:
 *   sb_stage_upload_f32 queues the host -> buffer copy of src (n =
 *     sb_field_size elements) now; the handle's next sb_step or
 *     sb_step_timed waits for it and moves it into the field (a device copy,
 *     or a conversion for BF16 storage) before its first kernel.  One staged
 *     upload per field until a step takes it (SB_ERR_INVALID otherwise);
 *   sb_stage_download_f32 copies the field, as it stands after the queued
 *     steps, into the buffer on the compute stream and then to dst on the
 *     copy stream;
 *   sb_wait_staged returns when every staged copy queued so far has landed.
 * Host buffers must be page-locked for the copies to overlap and stay valid
 * until sb_wait_staged (downloads) or the taking step (uploads) returns.
 * Fields: every field of sb_upload_field_f32 (the maps are not staged). */
int sb_stage_upload_f32(sb_bubble* b, sb_field which, const float* src, size_t n);
int sb_stage_download_f32(sb_bubble* b, sb_field which, float* dst, size_t n);
int sb_wait_staged(sb_bubble* b);

/* Statistics of the last step (synchronises).  Returns SB_ERR_CUDA (stats
 * still filled) once a bounded wait inside a kernel has given up (a grid
 * barrier of the implicit solve or the re-initialisation, or a
 * shared-memory copy): the step kernels never wait without a limit, and
 * after such a fault the bubble's cooperative kernels return at once and
 * the bubble halts at the end of that step (every kernel then leaves it
 * untouched), so its fields stop changing. */
int sb_get_stats(sb_bubble* b, sb_stats* out);

/* Computes the mass integrals into the stats (synchronises). */
int sb_update_mass(sb_bubble* b);

/* Replaces Solver::write_thickness_img (kernel/solver.cu:541-593): writes a
 * 3-channel (B, G, R equal) HALF EXR of eta * H * 2e5 to path and sets
 * *broken when no cell has eta > 0. */
int sb_write_thickness_exr(sb_bubble* b, const char* path, int* broken);

/* Replaces Solver::write_velocity_image (kernel/solver.cu:388-497): a HALF
 * EXR with R = u/2 + 0.5, G = v/2 + 0.5, B = 0.5, where u averages the u_phi
 * faces west and east of each cell and v the u_theta faces north and south
 * (next to a pole, 0.75 v - 0.25 v(phi + pi) of the nearest face row). */
int sb_write_velocity_exr(sb_bubble* b, const char* path);

/* Replaces Solver::write_concentration_image (kernel/solver.cu:500-538):
 * three equal HALF channels (gamma - 0.9) / 0.2. */
int sb_write_concentration_exr(sb_bubble* b, const char* path);

/* Host-only: writes img (height rows of width floats) as the reference's
 * grayscale frame format: 3 equal HALF channels B, G, R, no compression
 * (Solver::write_image, kernel/solver.cu:338-385).  Needs no GPU. */
int sb_write_exr_gray(const char* path, int width, int height, const float* img);

/* Replaces Bubble::run (kernel/bubble.cu:2607-2704): the frame loop with
 * full steps, a fractional last step per frame, and frame%04d.exr output
 * (plus vel%04d.exr / con%04d.exr when the params ask for them) into
 * out_dir (NULL: no output).  frames <= 0 uses p->frames.  The stop on a
 * broken film (SB_ERR_BROKEN: no cell of positive thickness) is decided
 * while a thickness frame is written, as in the reference, so a run
 * without output does not stop on it.  A solve that misses its tolerance
 * stops the run right after its step, as the reference's AmgX failure does
 * (kernel/bubble.cu:1500-1507, 2669): the later steps of the frame are
 * not taken (the device skips them, with no host synchronisation per
 * step), that frame is not written, and SB_ERR_NOT_CONVERGED is returned
 * with sb_stats.steps counting the steps actually taken. */
int sb_run(sb_bubble* b, const char* out_dir, int frames);

/* No counterpart in the reference.  The two mass integrals of
 * sb_update_mass (sum of eta sin(theta) and gamma sin(theta)) for callers
 * that may not allocate device memory: a framework that owns all device
 * memory through its own pool, a plug-in whose host application forbids
 * device allocations once it has started, or a real-time loop that cannot
 * afford cudaMalloc's implicit synchronisation.  eta and gamma are the
 * caller's device arrays ([theta][phi], nTheta x 2 nTheta FP32); mass_out
 * is the caller's device array of 2 doubles, written asynchronously on
 * `stream` (a cudaStream_t, NULL = legacy default stream).  It allocates
 * nothing: its scratch is a 20 KiB array compiled into the library (held on
 * every GPU that loads it), so nTheta is limited to powers of two in
 * [8, 1024] and larger grids are rejected with SB_ERR_INVALID.  The first
 * call in each device context (the first on a device, and the first after
 * a cudaDeviceReset) looks up the array's address and should come before
 * any stream capture.  All calls share the array: calls whose kernels
 * overlap on the GPU race and must be serialised by the caller.  A CUDA
 * error left pending by earlier work is not cleared: the call returns
 * SB_ERR_CUDA without doing any work. */
int sb_mass_integrals_noalloc(int nTheta, const float* eta, const float* gamma,
                              double* mass_out, void* stream);

/* Device bytes held by one bubble of this configuration (for admission). */
size_t sb_bytes_required(const sb_params* p);

/* CUDA stream of the handle (cudaStream_t), for callers that order their
 * own work after the step. */
void* sb_stream(sb_bubble* b);

/* Message for the last failing call on this thread. */
const char* sb_last_error(void);

/* ------------------------------------------------------------------------
 * Batches: an ensemble of bubbles (any mix of grid sizes on one device)
 * stepped together, one kernel launch per stage for all members.
 *
 * The reference has no counterpart; it steps one Solver per process
 * (Bubble::run, kernel/bubble.cu:2607-2704).  A batch step gives every
 * member exactly the result of sb_step on that member alone: the kernels
 * run the same per-cell code and the implicit solve keeps its own
 * reductions, iteration count and stopping test per member.
 *
 * Members stay owned by the caller and must outlive the batch; while a
 * batch exists, step its members only through it (sb_step on a member
 * would desynchronise the batch's view of its double-buffered maps).
 * Field I/O and statistics on members remain available after
 * sb_batch_synchronize.  All members share one solver configuration, one
 * field storage and one viscous switch (SB_ERR_INVALID otherwise); the step
 * time t and dt are common to all members.
 * ------------------------------------------------------------------------ */
typedef struct sb_batch sb_batch;

/* Builds the batch's tables (per-member descriptors, cell tiles of 64, 128
 * and 256 cells, solve-block ranges).  Synchronises the members' streams.
 * A bubble listed twice is rejected (SB_ERR_INVALID), and so is a batch
 * over its limits: at most 1024 members, and the sum over members of
 * nTheta (2 nTheta + 256) below 2^32 (the solver's 32-bit row tables). */
int sb_batch_create(sb_bubble* const* members, int n, sb_batch** out);
int sb_batch_destroy(sb_batch* batch);

/* n_steps steps of every member at time t_frame, step dt (seconds).
 * Replays one captured CUDA graph per step on the batch's stream. */
int sb_batch_step(sb_batch* batch, int n_steps, double t_frame, double dt);

/* As sb_batch_step with member k at frame time t_frames[k] (members at
 * different points of their runs, as in a serving loop). */
int sb_batch_step_each(sb_batch* batch, int n_steps, const double* t_frames, double dt);

/* As sb_batch_step but launching stage by stage and adding each stage's
 * device time (ms) to stage_ms[0 .. sb_stage_count()-1]; synchronises. */
int sb_batch_step_timed(sb_batch* batch, int n_steps, double t_frame, double dt,
                        double* stage_ms);

/* Times one step per tile size (64, 128, 256 cells per block) and keeps the
 * fastest for each stage; tile_sizes (optional, sb_stage_count() ints)
 * receives the choice.  The tuning steps advance the members (3 steps). */
int sb_batch_autotune(sb_batch* batch, double t_frame, double dt, int* tile_sizes);

/* Takes member `member` (its index in sb_batch_create's list) out of the
 * batch's work without rebuilding the batch: from the next step on every
 * kernel of the batch leaves it untouched (its state can still be read, and
 * the other members' results do not change).  The member must stay alive
 * until the batch is destroyed; it takes part again in a batch created
 * later.  Synchronises.  No counterpart in the reference; a serving loop
 * retires finished requests this way and rebuilds its batch only when
 * requests join. */
int sb_batch_retire(sb_batch* batch, int member);

int sb_batch_synchronize(sb_batch* batch);

/* CUDA stream of the batch (cudaStream_t). */
void* sb_batch_stream(sb_batch* batch);

#ifdef __cplusplus
}
#endif
#endif /* SOAPBUBBLE_GB300_H */
