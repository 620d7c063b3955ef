/*
 * FP64 host oracle for the soap-bubble time step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py load this library, and only
 * as the checker or as the timed CPU restatement of the reference.  The
 * product path (soapbubble_gb300) never links or calls it.
 *
 * This is a line-by-line CPU restatement of the reference's default step
 * (kernel/solver.cu:260-292 Solver::stepForward with the #defines of
 * include/header.cuh:37-98: greatCircle, RUNGE_KUTTA, BIMOCQ, MULTISAMPLE,
 * gravity, airflow, evaporation; VISCOUS off; fReal = double).  Each function
 * in oracle.cpp cites the reference file:line it follows.  The AmgX solve
 * (kernel/bubble.cu:1479-1508) is replaced by an FP64 conjugate-gradient solve
 * of the same assembled matrix to a tight relative residual.
 *
 * Parity status: UNPINNED against the reference binary.  The reference cannot
 * be built here (it needs AmgX, Boost.Filesystem and OpenCV libraries, none of
 * which are present) and it ships no golden vectors or tests.  The oracle is
 * pinned instead by analytic known-answer tests (tests/test_oracle_kat.py).
 *
 * Layout: every field is row-major [theta][phi] with row stride nPhi, as the
 * reference's host buffers (kernel/quantity.cu:94-97).  u_theta has nTheta-1
 * rows.  Map arrays hold absolute grid coordinates (theta/h, phi/h) exactly as
 * the reference's forward_t/forward_p/backward_* buffers.
 */
#ifndef SB_ORACLE_H
#define SB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nTheta;          /* rows of the centred grid; nPhi = 2 * nTheta */
    int nPhi;
    double radius;       /* r (m) */
    double dt;           /* nondimensional step, timeStepGlobal */
    double t;            /* currentTimeGlobal: frame start time (s) */
    double M, Cr, gs, gammaMax, evapRate, W1, W2, blend, U;
    int strict;          /* 1: mimic the reference's float intrinsics */
    int force_reinit;    /* -1: decide from distortion; 0: never; 1: always */
    double solver_tol;   /* relative residual target of the implicit solve */
    int solver_max_iter;
    int nthreads;        /* OpenMP threads (0 = default) */
    /* the reference's compile-time switches (include/header.cuh:89, 96) */
    int plain_advection;       /* 1: BIMOCQ undefined (advectionAllCentered, no maps) */
    int single_step_velocity;  /* 1: RUNGE_KUTTA undefined (velocity traced in one step) */
    int viscous;               /* 1: VISCOUS defined (include/header.cuh:98): viscous stress
                                  forces in the system and the velocity update */
    double re;                 /* reGlobal = nu / (U r), nu = 1.25e-4 (bubble.cu:2575) */
} sb_oracle_params;

typedef struct {
    double *eta, *gamma, *uth, *uph;                       /* N, N, Nv, N */
    double *eta_init, *eta_delta, *eta_initLast, *eta_deltaLast;
    double *gam_init, *gam_delta, *gam_initLast, *gam_deltaLast;
    double *fwd_t, *fwd_p, *bwd_t, *bwd_p, *bwdprev_t, *bwdprev_p;
    double *uair_init, *vair_init;                         /* N, Nv */
} sb_oracle_state;

typedef struct {
    double distortion;
    int reinit;
    int solver_iters;
    double solver_rel_resid;
    int broken_cells;
    int floor_oob;       /* strict mode: float floor hit a row past the grid */
} sb_oracle_stats;

/* Physical constants -> nondimensional coefficients, as Bubble::Bubble and
 * Bubble::run (kernel/bubble.cu:2568-2638). */
void sb_oracle_default_params(sb_oracle_params* p, int nTheta, double radius,
                              double H, double Gamma_m, double T, double dt_s,
                              double blend);

/* One full Solver::stepForward (kernel/solver.cu:260-292). */
int sb_oracle_step(const sb_oracle_params* p, sb_oracle_state* s, sb_oracle_stats* st);

/* Stages of the step, for per-kernel parity. */
void sb_oracle_update_maps(const sb_oracle_params* p, sb_oracle_state* s);
void sb_oracle_advection(const sb_oracle_params* p, sb_oracle_state* s);
int  sb_oracle_bodyforce(const sb_oracle_params* p, sb_oracle_state* s, sb_oracle_stats* st);
void sb_oracle_distortion(const sb_oracle_params* p, sb_oracle_state* s, sb_oracle_stats* st);
void sb_oracle_reinit(const sb_oracle_params* p, sb_oracle_state* s);

/* Assembly only (airflow + van der Waals + concentrationLinearSystemKernel).
 * val: 5N (up, left, centre, right, down), rhs: N, uair: N+1, vair: Nv+1.
 * gamma may be modified (broken cells are clamped to gammaMax). */
void sb_oracle_assemble(const sb_oracle_params* p, const sb_oracle_state* s,
                        double* gamma, double* val, double* rhs,
                        double* uair, double* vair);
/* Solve the assembled system, x holds x0 on entry. Returns iterations. */
int sb_oracle_solve(const sb_oracle_params* p, const double* val, const double* rhs,
                    double* x, double* rel_resid);

/* Point queries for unit tests (n points, coordinates in grid units). */
void sb_oracle_sample(const sb_oracle_params* p, int kind, const double* field,
                      int n, const double* coords, double* out);
void sb_oracle_trace(const sb_oracle_params* p, const double* uth, const double* uph,
                     double dt, int n, const double* coords, double* out);
void sb_oracle_sample_mapping(const sb_oracle_params* p, const double* map_t,
                              const double* map_p, int n, const double* coords,
                              double* out);
void sb_oracle_airflow(const sb_oracle_params* p, const double* uair_init,
                       const double* vair_init, double* uair, double* vair);
void sb_oracle_identity_map(int nTheta, int nPhi, double* map_t, double* map_p);
/* VISCOUS variant: div u (N), fv (Nv, gravity included) and fu (N) from the
 * velocities and thickness (kernel/bubble.cu:1218-1269, 1512-1816). */
void sb_oracle_viscous_forces(const sb_oracle_params* p, const double* uth, const double* uph,
                              const double* eta, double* div, double* fv, double* fu);

#ifdef __cplusplus
}
#endif
#endif
