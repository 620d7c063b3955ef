// Implicit surfactant solve: preconditioned conjugate gradients on the
// symmetric positive definite 5-point system assembled by k_assemble.  It
// replaces the reference's AmgX PCGF + AMG solve (kernel/bubble.cu:1479-1508,
// init/PCGF_F.json).  The reference starts from x0 = gamma; here the unknown
// is the increment dx = gamma_new - gamma_adv, starting from dx = 0, which is
// the same iteration with the large common part removed.
//
// One cooperative launch solves a set of systems: the one system of a
// bubble, or the systems of every bubble of a batch.  The theta rows of all
// systems form one list that is dealt to the blocks round robin; a phase
// (separated from the next by a grid barrier) visits the rows of the
// systems still iterating, so a system that needs more iterations than the
// others is spread over the whole GPU.  Every row adds its partial dot
// products into the system's exact fixed-point accumulator, so the sums,
// and the scalars advanced from them, do not depend on how rows are
// distributed or in which order blocks add: a bubble solved alone and
// inside a batch gives bit-identical results.
//
// Preconditioner: B^-1, the exact solve of each theta row's periodic
// tridiagonal block (phi couplings; the theta couplings stay on its
// diagonal), or the two-term Neumann series M^-1 = B^-1 + B^-1 C B^-1 of
// the splitting A = B - C, C the theta couplings, chosen per solve (see
// first_kind).  Near the poles the phi couplings carry 1/sin(theta) and
// dominate the diagonal by 1e4-1e5, which is what makes point Jacobi slow
// there; where the film has ruptured the theta couplings matter too, and
// the second term halves the iterations.  The row solve is
// cyclic / parallel cyclic reduction in shared memory, written in "excess"
// form: each equation keeps (excess e, |lower|, |upper|, rhs) with
// diagonal = e + |lower| + |upper|, and every update adds positive terms,
// so FP32 keeps full relative accuracy even when the diagonal exceeds the
// off-diagonal sum by a factor 1 + 1e-5 (the Grassmann-Taksar-Heyman idea
// applied to cyclic reduction).
//
// Phases of one CG iteration (each ends at a grid barrier, sb_sync.cuh):
// q = A p; the update of x and r with z = B^-1 r and r.z, r.r (B^-1 alone),
// or with z1 = B^-1 r followed by a phase forming z = z1 + B^-1 C z1 with
// r.z and r.r (Neumann term).  Rows of up to 1024 columns run in 256-thread
// blocks, rows of 2048 columns in 512-thread blocks (see kVThreads).
//
// Modes: plain FP32 (FP32 iterate, float products), or mixed precision
// (FP32 SpMV and preconditioner, float-float iterate, exact products in the
// dot products, and a float-float true-residual check that restarts CG from
// the refined iterate until the relative residual target holds).  Dot
// products are summed in float-float within a row and exactly across rows.
// (Rounding the products, as plain mode does, costs the mixed mode about a
// fifth more iterations on ruptured films.)

#include <algorithm>
#include <climits>

#include "sb_ff.cuh"
#include "sb_internal.h"
#include "sb_scale.cuh"
#include "sb_sync.cuh"

namespace sb {

namespace {

// Threads of a solve block: 256, or 512 for rows of 2048 columns (four
// columns per thread either way).  Dot products are formed in an order that
// does not depend on the block width: virtual thread v < 256 owns columns
// v + 256 k; its share is the float-float sum of its even k (in order) plus
// that of its odd k, and the row's value sums the 256 shares in a fixed
// order.  A block of 512 threads gives each virtual thread's even and odd k
// to threads v and v + 256, so a bubble gets the same sums whichever block
// width a solve set uses.
constexpr int kVThreads = 256;
constexpr int kWarps = kVThreads / 32;
constexpr int kMaxNP = 2048;
constexpr int kWaitPolls = 1 << 22;   // mbarrier polls before a copy counts as lost
constexpr int kMaxSystems = 1024;     // systems of one solve set
constexpr int kRowChunk = 16;         // rows a block counts at a time (sets)
// Phase kinds of the solve (what every row does in a phase):
//   K_SETUP    x = 0, r = r0, the preconditioner's factors, z1 = B^-1 r; |b|^2
//   K_NEUMANN  z = z1 + B^-1 (C z1) (C: the theta couplings); r.z, r.r
//   K_Q        p = z + beta p_old, q = A p; p.q
//   K_UPDATE   x += alpha p, r -= alpha q, z1 = B^-1 r
//   K_CHECK    r = r0 - A x of the float-float iterate (mixed mode); |r|^2
//   K_RESTART  z1 = B^-1 r from the refined iterate's residual
// and, with the line preconditioner alone (z = B^-1 r, no Neumann phase):
//   K_SETUP_L    as K_SETUP with z = B^-1 r; r.z, r.r, |b|^2
//   K_UPDATE_L   x += alpha p, r -= alpha q, z = B^-1 r; r.z, r.r
//   K_RESTART_L  z = B^-1 r from the refined iterate's residual; r.z, r.r
enum {
    K_SETUP = 0, K_NEUMANN = 1, K_Q = 2, K_UPDATE = 3, K_CHECK = 4, K_RESTART = 5,
    K_SETUP_L = 6, K_UPDATE_L = 7, K_RESTART_L = 8
};

// Dot-product values a phase kind produces (bit v: accumulator value v):
// r.z (0), r.r (1) and the set-up |b|^2 (2); q = A p and the refinement
// check one value each.
__host__ __device__ inline int kind_values(int kind) {
    switch (kind) {
        case K_SETUP: return 4;
        case K_SETUP_L: return 7;
        case K_NEUMANN: case K_UPDATE_L: case K_RESTART_L: return 3;
        case K_Q: case K_CHECK: return 1;
        default: return 0;
    }
}

// The line preconditioner alone costs two phases per CG iteration, with the
// Neumann term three (and one more at the start); the term pays where it
// removes more than about a third of the iterations, which happens where the
// theta couplings are strong (thin or ruptured films: c1 late in the run,
// 44 -> 24 iterations) and shows as many iterations, and not on smooth thick
// films (c1 early, c2: 2 iterations either way).  Auto mode turns the term
// on after a solve that needed kNeumannOn or more iterations with the line
// preconditioner alone (break-even near 6) and off after one that needed at
// most kNeumannOff with it.
constexpr int kNeumannOn = 7;
constexpr int kNeumannOff = 2;

__device__ __forceinline__ int first_kind(const SbDevStats* st, const SolverConfig& cfg) {
    bool neu;
    if (cfg.precond == kPrecNeumann) neu = true;
    else if (cfg.precond == kPrecLine) neu = false;
    else if (st->solver_neumann) neu = st->solver_iters > kNeumannOff;
    else neu = st->solver_iters >= kNeumannOn;
    return neu ? K_SETUP : K_SETUP_L;
}

// ---------------------------------------------------------------------------
// Shared-memory copy of one row's preconditioner factors.  A block keeps
// the factors of the row it last built or fetched; fetching another row's
// factors is one bulk asynchronous copy (cp.async.bulk, completion counted
// on an mbarrier), started before the row's update so that it lands while
// the update runs.  When a block owns a single row for the whole solve the
// factors never leave shared memory.
struct Stage {
    float* blob;           // factors of row `resident` (shared memory)
    float* work;           // reduction work arrays (shared memory)
    uint32_t bar;          // shared address of the mbarrier
    unsigned copies;       // bulk copies issued (and waited for) so far
    const float* resident; // global address of the factors in `blob`
    bool pending;          // a copy into `blob` is in flight
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void stage_init(Stage& S, uint64_t* bar, float* sm, int blob_bytes) {
    S.blob = sm;
    S.work = sm + blob_bytes / 4;
    S.bar = smem_u32(bar);
    S.copies = 0;
    S.resident = nullptr;
    S.pending = false;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(S.bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
}

// Start copying the factors at `src` (bytes, a multiple of 16) unless they
// are the block's resident ones.  Called by every thread with the same
// arguments; every earlier read of the blob must be complete.
__device__ __forceinline__ void stage_fetch(Stage& S, const float* src, int bytes) {
    if (src == S.resident) return;
    if (threadIdx.x == 0) {
        // the block's generic reads of the blob come before the copy's writes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(S.bar),
                     "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(S.blob)),
            "l"(src), "r"(bytes), "r"(S.bar)
            : "memory");
    }
    S.resident = src;
    S.pending = true;
}

// Every thread: wait (bounded) for the copy in flight.  A wait that gives
// up is counted in the stats, and the solve is then reported as failed
// instead of hanging.
__device__ __forceinline__ void stage_wait(Stage& S, SbDevStats* st) {
    if (!S.pending) return;
    const uint32_t parity = S.copies & 1u;
    for (int k = 0;; ++k) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(S.bar), "r"(parity) : "memory");
        if (ok) break;
        if (k >= kWaitPolls) {
            if (threadIdx.x == 0) atomicAdd(&st->wait_faults, 1);
            break;
        }
    }
    ++S.copies;
    S.pending = false;
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ ff ld_ff(const float2* v, int c) {
    const float2 t = v[c];
    return {t.x, t.y};
}

// (A x)_c in float-float for the float-float iterate x at cell c = (i, j).
__device__ __forceinline__ ff apply_A_ff(const SbGrid& g, const SbFields& f, const float2* x, int c,
                                         int i, int j) {
    const int nP = g.nP;
    const int e = i * nP + ((j + 1) & g.maskP);
    const int w = i * nP + ((j - 1) & g.maskP);
    const ff xc = ld_ff(x, c);
    ff s = ff_mul_f(xc, f.dmass[c]);
    s = ff_add(s, ff_mul_f(ff_add(xc, ff_neg(ld_ff(x, e))), f.cE[c]));
    s = ff_add(s, ff_mul_f(ff_add(xc, ff_neg(ld_ff(x, w))), f.cE[w]));
    if (i < g.nT - 1) s = ff_add(s, ff_mul_f(ff_add(xc, ff_neg(ld_ff(x, c + nP))), f.cS[c]));
    if (i > 0) s = ff_add(s, ff_mul_f(ff_add(xc, ff_neg(ld_ff(x, c - nP))), f.cS[c - nP]));
    return s;
}

// Dot-product terms: exact products in mixed mode, float products in plain
// mode, accumulated in float-float.
template <bool MIXED>
__device__ __forceinline__ ff acc(ff s, float a, float b) {
    return MIXED ? ff_add_prod(s, a, b) : ff_add_f(s, __fmul_rn(a, b));
}

// Column of element k of this thread in a row.
template <int TB>
__device__ __forceinline__ int col_of(int k) { return threadIdx.x + k * TB; }

// The two float-float accumulators of a thread's dot-product terms: element
// k of a 256-thread block goes to k's parity; a 512-thread block's thread
// holds one parity only (see kVThreads).
template <int TB>
__device__ __forceinline__ int half_of(int k) { return TB == kVThreads ? (k & 1) : 0; }

template <int TB>
__device__ __forceinline__ ff fold_halves(const ff (&h)[2]) {
    return TB == kVThreads ? ff_add(h[0], h[1]) : h[0];
}

// y = B_i^-1 v on theta row i: the exact solve of the row's periodic
// tridiagonal block B_i (phi couplings; the theta couplings stay on its
// diagonal).  rv[k] holds v at column col_of<TB>(k) (this thread's elements);
// the result is left in the block's work array D = S.work (D[j] for
// column j) for the caller.  PER = equations per thread
// (nP <= PER * TB).
//
// Row solve of n = nP equations (indices mod n) in excess form: equation j
//   (E_j + L_j + U_j) x_j - L_j x_{j-s} - U_j x_{j+s} = D_j,  E, L, U >= 0,
// at stride s = 1 to begin with:
//   1. cyclic reduction at stride 1: every even equation absorbs its odd
//      neighbours (D_j += a D_{j-1} + c D_{j+1}) and couples at stride 2;
//   2. the same at stride 2 for the equations j = 0 mod 4;
//   3. parallel cyclic reduction of the q = n/4 equations j = 0 mod 4 at
//      strides 4, 8, .., n/4 (stopping once every coupling is below 2^-26
//      of its excess, the row having decoupled to float precision), ending
//      with 2 x 2 solves of j and j + n/2;
//   4. back substitution of j = 2 mod 4 from their stride-2 equations, then
//      of the odd j from the original ones: x_j = g D_j + a' x_{j-s} +
//      b' x_{j+s} with g = 1 / diagonal and a' + b' < 1.
// Every update of an excess or a right-hand side adds non-negative terms
// (the Grassmann-Taksar-Heyman idea applied to cyclic reduction), so FP32
// keeps full relative accuracy even when the diagonal exceeds the
// off-diagonal sum by a factor 1 + 1e-5.  Steps 1, 2 and 4 are O(n) work and
// step 3 O(n/4 log n), against O(n log n) for parallel reduction of the
// whole row.
//
// The row matrix does not change during a solve: the first application
// (BUILD) computes the factors of every step into the block's shared-memory
// blob, copies the blob to the row's slot of f.pcr (layout factor_blob) and
// records the levels of step 3 in f.pcr_levels; later applications replay
// the right-hand-side updates with the factors (fetched by stage_fetch
// unless the block still holds them), with the same arithmetic.
template <int PER, int TB, bool BUILD>
__device__ __forceinline__ void precondition_row(const SbGrid& g, const SbFields& f, int i,
                                                 Stage& S, const float (&rv)[PER],
                                                 bool store = true) {
    const int nP = g.nP, nT = g.nT, mask = g.maskP;
    const int row = i * nP;
    constexpr int H = PER >= 2 ? PER / 2 : 1;  // items per thread of the n/2-item steps
    constexpr int Q = PER >= 4 ? PER / 4 : 1;  // and of the n/4-item steps
    const SbFactorBlob B = factor_blob(nP);
    const int n = nP, h = n / 2, q = B.q, qmask = q - 1;
    char* const bl = reinterpret_cast<char*>(S.blob);
    float2* const cr1 = reinterpret_cast<float2*>(bl + B.cr1);
    float2* const cr2 = reinterpret_cast<float2*>(bl + B.cr2);
    float2* const pcr = reinterpret_cast<float2*>(bl + B.pcr);
    float2* const fin = reinterpret_cast<float2*>(bl + B.fin);
    float* const g2 = reinterpret_cast<float*>(bl + B.bs2);  // [3][q]: g, a', b' of 4m + 2
    float* const g1 = reinterpret_cast<float*>(bl + B.bs1);  // [3][h]: g, a', b' of 2m + 1
    float* const D = S.work;                                  // right-hand side, then x
    if (BUILD) {
        float* const E = S.work + n;      // excess: diagonal minus the phi couplings
        float* const L = S.work + 2 * n;  // coupling to j - s
        float* const U = S.work + 3 * n;  // coupling to j + s
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int j = col_of<TB>(k);
            if (j < n) {
                const int c = row + j;
                float ex = f.dmass[c];
                if (i < nT - 1) ex += f.cS[c];
                if (i > 0) ex += f.cS[c - nP];
                E[j] = ex;
                U[j] = f.cE[c];
                L[j] = f.cE[row + ((j - 1) & mask)];
                D[j] = rv[k];
            }
        }
        __syncthreads();
        // step 1; an even entry is read only by its own thread: in place
#pragma unroll
        for (int t = 0; t < H; ++t) {
            const int m = threadIdx.x + t * TB;
            if (m < h) {
                const int j = 2 * m, jm = (j - 1) & mask, jp = j + 1;
                const float bm = E[jm] + L[jm] + U[jm];
                const float bp = E[jp] + L[jp] + U[jp];
                // fast division: the preconditioner stays a fixed operator
                const float am = __fdividef(L[j], bm), cp = __fdividef(U[j], bp);
                cr1[m] = make_float2(am, cp);
                const float gi = __fdividef(1.0f, bp);  // odd equation jp
                g1[m] = gi;
                g1[h + m] = L[jp] * gi;
                g1[2 * h + m] = U[jp] * gi;
                const float nE = E[j] + am * E[jm] + cp * E[jp];
                const float nL = am * L[jm], nU = cp * U[jp];
                D[j] = D[j] + am * D[jm] + cp * D[jp];
                E[j] = nE;
                L[j] = nL;
                U[j] = nU;
            }
        }
        __syncthreads();
        // step 2, into compact arrays (index m = j / 4) that reuse the space
        // of E, L, U once every thread has read them
        float sE[Q], sL[Q], sU[Q], sD[Q];
#pragma unroll
        for (int t = 0; t < Q; ++t) {
            const int m = threadIdx.x + t * TB;
            if (m < q) {
                const int j = 4 * m, jm = (j - 2) & mask, jp = j + 2;
                const float bm = E[jm] + L[jm] + U[jm];
                const float bp = E[jp] + L[jp] + U[jp];
                const float am = __fdividef(L[j], bm), cp = __fdividef(U[j], bp);
                cr2[m] = make_float2(am, cp);
                const float gi = __fdividef(1.0f, bp);  // equation jp = 4m + 2
                g2[m] = gi;
                g2[q + m] = L[jp] * gi;
                g2[2 * q + m] = U[jp] * gi;
                sE[t] = E[j] + am * E[jm] + cp * E[jp];
                sL[t] = am * L[jm];
                sU[t] = cp * U[jp];
                sD[t] = D[j] + am * D[jm] + cp * D[jp];
            }
        }
        __syncthreads();
        float* const P = S.work + n;  // two sets (E, L, U, D) of q entries
        bool need = false;
#pragma unroll
        for (int t = 0; t < Q; ++t) {
            const int m = threadIdx.x + t * TB;
            if (m < q) {
                P[m] = sE[t];
                P[q + m] = sL[t];
                P[2 * q + m] = sU[t];
                P[3 * q + m] = sD[t];
                need |= (sL[t] + sU[t]) > 1.4901161e-8f * sE[t];
            }
        }
        // step 3, ping-pong between the two sets
        bool decoupled = !__syncthreads_or(need);
        int levels = 0, cur = 0;
        for (int s = 1; !decoupled && s <= q / 4; s <<= 1) {
            const float* Ei = P + cur * 4 * q;
            const float *Li = Ei + q, *Ui = Ei + 2 * q, *Di = Ei + 3 * q;
            float* Eo = P + (cur ^ 1) * 4 * q;
            need = false;
#pragma unroll
            for (int t = 0; t < Q; ++t) {
                const int m = threadIdx.x + t * TB;
                if (m < q) {
                    const int mm = (m - s) & qmask, mp = (m + s) & qmask;
                    const float bm = Ei[mm] + Li[mm] + Ui[mm];
                    const float bp = Ei[mp] + Li[mp] + Ui[mp];
                    const float am = __fdividef(Li[m], bm), cp = __fdividef(Ui[m], bp);
                    pcr[levels * q + m] = make_float2(am, cp);
                    const float nE = Ei[m] + am * Ei[mm] + cp * Ei[mp];
                    const float nL = am * Li[mm], nU = cp * Ui[mp];
                    Eo[m] = nE;
                    Eo[q + m] = nL;
                    Eo[2 * q + m] = nU;
                    Eo[3 * q + m] = Di[m] + am * Di[mm] + cp * Di[mp];
                    need |= (nL + nU) > 1.4901161e-8f * nE;
                }
            }
            ++levels;
            cur ^= 1;
            decoupled = !__syncthreads_or(need);
        }
        if (threadIdx.x == 0) f.pcr_levels[i] = decoupled ? levels : -levels;
        // 2 x 2 solves of m and m + q/2 (or the decoupled diagonal): x at
        // j = 4m, whose D entry is free since step 2
        {
            const float* Ef = P + cur * 4 * q;
            const float *Lf = Ef + q, *Uf = Ef + 2 * q, *Df = Ef + 3 * q;
#pragma unroll
            for (int t = 0; t < Q; ++t) {
                const int m = threadIdx.x + t * TB;
                if (m < q) {
                    const int kk = (m + q / 2) & qmask;
                    float c1, c2;
                    if (decoupled) {
                        c1 = 1.0f / (Ef[m] + Lf[m] + Uf[m]);
                        c2 = 0.0f;
                    } else {
                        const float mj = Lf[m] + Uf[m], mk = Lf[kk] + Uf[kk];
                        const float ej = Ef[m], ek = Ef[kk];
                        const float idet = 1.0f / (ej * ek + ej * mk + mj * ek);
                        c1 = (ek + mk) * idet;
                        c2 = mj * idet;
                    }
                    fin[m] = make_float2(c1, c2);
                    D[4 * m] = c1 * Df[m] + c2 * Df[kk];
                }
            }
        }
        __syncthreads();
    } else {
        // replay: the factors are in the blob (or on their way)
        const int lv = f.pcr_levels[i];
        const int levels = lv < 0 ? -lv : lv;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int j = col_of<TB>(k);
            if (j < n) D[j] = rv[k];
        }
        stage_wait(S, f.stats);
        __syncthreads();
#pragma unroll
        for (int t = 0; t < H; ++t) {
            const int m = threadIdx.x + t * TB;
            if (m < h) {
                const int j = 2 * m;
                const float2 c = cr1[m];
                D[j] = D[j] + c.x * D[(j - 1) & mask] + c.y * D[j + 1];
            }
        }
        __syncthreads();
        float* Pi = S.work + n;
        float* Po = Pi + q;
#pragma unroll
        for (int t = 0; t < Q; ++t) {
            const int m = threadIdx.x + t * TB;
            if (m < q) {
                const int j = 4 * m;
                const float2 c = cr2[m];
                Pi[m] = D[j] + c.x * D[(j - 2) & mask] + c.y * D[j + 2];
            }
        }
        __syncthreads();
        for (int l = 0, s = 1; l < levels; ++l, s <<= 1) {
#pragma unroll
            for (int t = 0; t < Q; ++t) {
                const int m = threadIdx.x + t * TB;
                if (m < q) {
                    const float2 c = pcr[l * q + m];
                    Po[m] = Pi[m] + c.x * Pi[(m - s) & qmask] + c.y * Pi[(m + s) & qmask];
                }
            }
            __syncthreads();
            float* tmp = Pi;
            Pi = Po;
            Po = tmp;
        }
#pragma unroll
        for (int t = 0; t < Q; ++t) {
            const int m = threadIdx.x + t * TB;
            if (m < q) {
                const float2 c = fin[m];
                D[4 * m] = c.x * Pi[m] + c.y * Pi[(m + q / 2) & qmask];
            }
        }
        __syncthreads();
    }
    // step 4 (both paths)
#pragma unroll
    for (int t = 0; t < Q; ++t) {
        const int m = threadIdx.x + t * TB;
        if (m < q) {
            const int j = 4 * m + 2;
            D[j] = g2[m] * D[j] + g2[q + m] * D[j - 2] + g2[2 * q + m] * D[(j + 2) & mask];
        }
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < H; ++t) {
        const int m = threadIdx.x + t * TB;
        if (m < h) {
            const int j = 2 * m + 1;
            D[j] = g1[m] * D[j] + g1[h + m] * D[j - 1] + g1[2 * h + m] * D[(j + 1) & mask];
        }
    }
    __syncthreads();
    if (BUILD) {
        // the row's factors to its global slot, for fetches by any block in
        // later phases (not when every block keeps its one row for the whole
        // solve: no fetch happens then); the blob is the block's resident copy
        float* const dst = f.pcr + (size_t)i * (B.bytes / 4);
        const float4* src = reinterpret_cast<const float4*>(S.blob);
        if (store)
            for (int k = threadIdx.x; k < B.bytes / 16; k += TB)
                reinterpret_cast<float4*>(dst)[k] = src[k];
        S.resident = dst;
        // generic writes of both copies before later bulk copies from the
        // global slot and into the blob
        asm volatile("fence.proxy.async.global;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();  // the blob is free again; D holds the result
}

// Global slot of row i's factors.
__device__ __forceinline__ const float* row_blob(const SbGrid& g, const SbFields& f, int i) {
    return f.pcr + (size_t)i * (factor_blob(g.nP).bytes / 4);
}

// ---------------------------------------------------------------------------
// Row bodies.  Every thread handles the columns col_of<TB>(0 .. PER-1) of a theta
// row, one column after the other (measured faster than issuing all loads
// of a thread's columns first, which costs registers).  Dot-product terms
// are accumulated in column order.

// The initial iterate and residual, p_old = 0; rv = r; adds |rhs|^2 to bb.
// With warm starts on, the iterate starts from the previous step's
// increment dx when the previous solve converged and the state has not
// been replaced since (stats->dx_valid and solver_converged, the same in
// every block during a solve): the increment of gamma changes little from
// one step to the next, so r = r0 - A dx_prev is much smaller than r0 and
// the solve needs fewer iterations; it stops at the same relative residual
// of the same system.  A non-finite previous value starts from zero.
// Otherwise the iterate starts from dx = 0 (gamma_new = gamma_adv).
template <bool MIXED, int PER, int TB>
__device__ __forceinline__ void row_init(const SbGrid& g, const SbFields& f, int i,
                                         const SolverConfig& cfg, float (&rv)[PER], ff& bb) {
    const int nP = g.nP, nT = g.nT, row = i * nP;
    const bool warm = cfg.warm && f.stats->dx_valid != 0 && f.stats->solver_converged != 0;
    // The previous increment, bounded by |x0| <= min(gamma_adv, gmax - gamma_adv):
    // 0 in a broken cell (gamma_adv = gmax, its row is dx = 0), and where
    // advection brought a tiny concentration into the cell, its diagonal
    // sin(theta) / (dt gamma_adv) times x0 stays below sin(theta) / dt
    // (unbounded, 6e24 x 1e2 made a residual whose square overflows FP32).
    // The bound depends on the cell alone, so every row that reads x0 of a
    // neighbour sees the same value.
    // The iterate of a scaled cell (sb_scale.cuh) is dx / s.
    const float gmax = f.self->ph.gmax, invDt = f.step->invDt;
    // The previous increment is read where this phase does not write it:
    // f.dx in mixed mode (the iterate is xff), xff's leading part in plain
    // mode (whose iterate is dx; the last pass of every solve leaves
    // xff = (dx, 0)), so that a row reads its neighbours' values of the
    // previous solve whatever the order in which the rows are set up.
    auto prev = [&](int c, int ic) {
        const float v = MIXED ? f.dx[c] : f.xff[c].x, ga = f.gam_adv[c];
        const float lim = fminf(ga, gmax - ga);
        const float x0 = isfinite(v) ? fminf(fmaxf(v, -lim), lim) : 0.0f;
        const int k = diag_scale_k(ga, g.sin_c[ic], invDt);
        return k ? x0 * pow2_pos(k) : x0;
    };
    ff h[2] = {ff_zero(), ff_zero()};
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = col_of<TB>(k);
        rv[k] = 0.0f;
        if (j < nP) {
            const int c = row + j;
            float r = f.r0[c];
            const float rhs = f.rhs[c];
            if (warm) {
                const float x0 = prev(c, i);
                const int e = row + ((j + 1) & g.maskP), w = row + ((j - 1) & g.maskP);
                float ax = f.dmass[c] * x0 + f.cE[c] * (x0 - prev(e, i)) + f.cE[w] * (x0 - prev(w, i));
                if (i < nT - 1) ax += f.cS[c] * (x0 - prev(c + nP, i + 1));
                if (i > 0) ax += f.cS[c - nP] * (x0 - prev(c - nP, i - 1));
                r -= ax;
                if (MIXED) f.xff[c] = make_float2(x0, 0.0f);
                else f.dx[c] = x0;
            } else {
                if (MIXED) f.xff[c] = make_float2(0.0f, 0.0f);
                else f.dx[c] = 0.0f;
            }
            rv[k] = r;
            f.r[c] = r;
            f.q[c] = 0.0f;
            h[half_of<TB>(k)] = ff_add_prod(h[half_of<TB>(k)], rhs, rhs);
        }
    }
    bb = fold_halves<TB>(h);
}

// p_new = z + beta p_old on the row and, on the fly, on the neighbours it
// reads (so no barrier is needed between forming p and using it); q = A p_new
// is kept in f.x.  Returns the row's p.q.  Every load of a column is issued
// before its arithmetic, through restrict-qualified pointers so that the
// compiler may also start the next column's loads early.
template <bool MIXED, int PER, int TB>
__device__ __forceinline__ ff row_spmv(const SbGrid& g, const SbFields& f, int i, float beta,
                                       const float* __restrict__ pold, float* __restrict__ pnew) {
    const int nP = g.nP, nT = g.nT, row = i * nP;
    const float* __restrict__ z = f.z;
    const float* __restrict__ dmass = f.dmass;
    const float* __restrict__ cE = f.cE;
    const float* __restrict__ cS = f.cS;
    float* __restrict__ qout = f.x;
    const bool hasS = i < nT - 1, hasN = i > 0;
    ff pq[2] = {ff_zero(), ff_zero()};
    // columns in pairs: both columns' loads are issued before either's
    // arithmetic (two L2 round trips per row instead of four at PER = 4)
    constexpr int G2 = PER >= 2 ? 2 : 1;
#pragma unroll
    for (int k0 = 0; k0 < PER; k0 += G2) {
        float zc[G2], pc0[G2], ze[G2], pe[G2], zw[G2], pw[G2], zs[G2], ps[G2], zn[G2], pn[G2];
        float dm[G2], ce[G2], cw[G2], cs[G2], cn[G2];
        int cc[G2];
#pragma unroll
        for (int u = 0; u < G2; ++u) {
            const int j = col_of<TB>(k0 + u);
            const int jj = j < nP ? j : 0;  // rows shorter than the block: a valid dummy
            const int c = row + jj;
            const int e = row + ((jj + 1) & g.maskP);
            const int w = row + ((jj - 1) & g.maskP);
            const int sc = hasS ? c + nP : c, nc = hasN ? c - nP : c;
            cc[u] = c;
            zc[u] = z[c]; pc0[u] = pold[c];
            ze[u] = z[e]; pe[u] = pold[e]; zw[u] = z[w]; pw[u] = pold[w];
            zs[u] = z[sc]; ps[u] = pold[sc]; zn[u] = z[nc]; pn[u] = pold[nc];
            dm[u] = dmass[c]; ce[u] = cE[c]; cw[u] = cE[w];
            cs[u] = hasS ? cS[c] : 0.0f;
            cn[u] = hasN ? cS[nc] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < G2; ++u) {
            if (col_of<TB>(k0 + u) < nP) {
                const float pc = zc[u] + beta * pc0[u];
                const float dE = pc - (ze[u] + beta * pe[u]);
                const float dS = pc - (zs[u] + beta * ps[u]);
                float qf = dm[u] * pc + ce[u] * dE + cw[u] * (pc - (zw[u] + beta * pw[u]));
                if (hasS) qf += cs[u] * dS;
                if (hasN) qf += cn[u] * (pc - (zn[u] + beta * pn[u]));
                pnew[cc[u]] = pc;
                qout[cc[u]] = qf;
                // p.q = p^T A p in its energy form: dmass p^2 plus w (p_c -
                // p_n)^2 over each east and south face once, every term
                // non-negative.  The sum of the products p_c q_c of the FP32
                // q = A p cancels to almost nothing on ruptured films
                // (weights 1e5 times the mass terms) and could lose its
                // sign there, which broke the iteration down.
                ff& h = pq[half_of<TB>(k0 + u)];
                h = acc<MIXED>(h, dm[u] * pc, pc);
                h = acc<MIXED>(h, ce[u] * dE, dE);
                if (hasS) h = acc<MIXED>(h, cs[u] * dS, dS);
            }
        }
    }
    return fold_halves<TB>(pq);
}

// True residual r = r0 - A x of the float-float iterate (mixed mode),
// carried in float-float; stores it (rounded) in f.r and returns the row's
// |r|^2.
template <int PER, int TB>
__device__ __forceinline__ ff row_true_residual(const SbGrid& g, const SbFields& f, int i) {
    const int nP = g.nP, row = i * nP;
    ff a[2] = {ff_zero(), ff_zero()};
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = col_of<TB>(k);
        if (j < nP) {
            const int c = row + j;
            const ff r = ff_add_f(ff_neg(apply_A_ff(g, f, f.xff, c, i, j)), f.r0[c]);
            f.r[c] = ff_to_f(r);
            // r^2 = hi^2 + 2 hi lo (+ lo^2, below the float-float precision)
            ff& ah = a[half_of<TB>(k)];
            ah = ff_add_f(ff_add_prod(ah, r.hi, r.hi), __fmul_rn(2.0f, __fmul_rn(r.hi, r.lo)));
        }
    }
    return fold_halves<TB>(a);
}

// x += alpha p_new, r -= alpha q; rv = the new r.  Every load of the
// thread's columns is issued before any arithmetic.
template <bool MIXED, int PER, int TB>
__device__ __forceinline__ void row_update(const SbGrid& g, const SbFields& f, int i, ff alpha,
                                           const float* __restrict__ pnew, float (&rv)[PER]) {
    const int nP = g.nP, row = i * nP;
    const float af = ff_to_f(alpha);
    const ff a2 = alpha;
    float pc[PER], rc[PER], qc[PER];
    float2 xc[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = col_of<TB>(k);
        const int c = row + (j < nP ? j : 0);
        pc[k] = pnew[c];
        rc[k] = f.r[c];
        qc[k] = f.x[c];
        if (MIXED) xc[k] = f.xff[c];
        else xc[k].x = f.dx[c];
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = col_of<TB>(k);
        rv[k] = 0.0f;
        if (j < nP) {
            const int c = row + j;
            if (MIXED) {
                const ff x = ff_add({xc[k].x, xc[k].y}, ff_mul_f(a2, pc[k]));
                f.xff[c] = make_float2(x.hi, x.lo);
            } else {
                f.dx[c] = xc[k].x + af * pc[k];
            }
            rv[k] = rc[k] - af * qc[k];
            f.r[c] = rv[k];
        }
    }
}

// rv = r (restart from the refined iterate's residual).
template <int PER, int TB>
__device__ __forceinline__ void row_load_r(const SbGrid& g, const SbFields& f, int i,
                                           float (&rv)[PER]) {
    const int nP = g.nP, row = i * nP;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = col_of<TB>(k);
        rv[k] = j < nP ? f.r[row + j] : 0.0f;
    }
}

// The increment and the new gamma: dx, x = gamma_adv + dx; xff keeps the
// increment as a float-float pair in both modes (plain mode: (dx, 0)),
// which the post-solve stage differences between neighbours.
template <bool MIXED, int PER, int TB>
__device__ __forceinline__ void row_final(const SbGrid& g, const SbFields& f, int i) {
    const int nP = g.nP, row = i * nP;
    const float invDt = f.step->invDt;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = col_of<TB>(k);
        if (j < nP) {
            const int c = row + j;
            float dx = MIXED ? ff_to_f(ld_ff(f.xff, c)) : f.dx[c];
            const float ga = f.gam_adv[c];
            const int ks = diag_scale_k(ga, g.sin_c[i], invDt);
            if (ks) {  // a scaled cell's iterate is dx / s (sb_scale.cuh)
                const float sc = pow2_neg(ks);
                dx *= sc;
                if (MIXED) {
                    const float2 v = f.xff[c];
                    f.xff[c] = make_float2(v.x * sc, v.y * sc);
                }
            }
            f.dx[c] = dx;
            f.x[c] = ga + dx;
            if (!MIXED) f.xff[c] = make_float2(dx, 0.0f);
        }
    }
}

// ---------------------------------------------------------------------------
// Exact sums.  A row's dot-product partials (float-float) are added into a
// long fixed-point accumulator: every float is an integer multiple of
// 2^-149 below 2^128, so 9 chunks of 32 bits held in 64-bit integers (and a
// tenth for carries) cover it exactly, and integer additions do not depend
// on their order.  The
// total is therefore the same whichever block adds which row, and the same
// for a system solved alone or inside a set; a system's blocks add with
// fire-and-forget atomics and nobody sums row partials.  A word per value
// flags NaN or infinity.  Each system has three buffers of three values,
// used in rotation by phase (p % 3): added in phase p, read at the end of
// phase p (sets) or at the start of phase p + 1 (one system), and zeroed
// again before phase p + 3.
constexpr int kAccChunks = 10;             // chunks 0..8 take additions, chunk 9 carries
constexpr int kAccWords = kAccChunks + 1;  // per value
constexpr int kAccSlot = 16;               // words per value in memory: one 128-byte line
constexpr int kAccBuf = 3 * kAccSlot;      // per buffer (three values)
static_assert(3 * kAccBuf == kSolveAccWords, "accumulator words per system");
static_assert(kAccWords <= kAccSlot, "a value fits its line");

__device__ __forceinline__ unsigned long long* acc_buf(const SbSolveSet& S, int b, int p) {
    return S.acc + (size_t)b * kSolveAccWords + (size_t)(p % 3) * kAccBuf;
}

// a += v exactly.
__device__ __forceinline__ void acc_add(unsigned long long* a, float v) {
    const unsigned u = __float_as_uint(v);
    const int ex = (int)((u >> 23) & 0xffu);
    if (ex == 0xff) {
        atomicOr(a + kAccChunks, 1ull);
        return;
    }
    long long m = (long long)(u & 0x7fffffu);
    if (ex == 0 && m == 0) return;  // +-0
    int P = 0;                      // exponent of the mantissa's last bit, plus 149
    if (ex != 0) {
        m |= 0x800000;
        P = ex - 1;
    }
    if (u >> 31) m = -m;
    const long long w = m << (P & 31);  // |w| < 2^55: two chunks
    const int k = P >> 5;
    atomicAdd(a + k, (unsigned long long)(w & 0xffffffffll));
    atomicAdd(a + k + 1, (unsigned long long)(w >> 32));
}

// x.hi + x.lo into value v of buffer a.
__device__ __forceinline__ void acc_add_ff(unsigned long long* a, int v, ff x) {
    acc_add(a + v * kAccSlot, x.hi);
    acc_add(a + v * kAccSlot, x.lo);
}

// Carries: chunks 0..8 into [0, 2^32), the sign in chunk 9.
__device__ __forceinline__ void acc_normalize(long long (&c)[kAccChunks]) {
    long long carry = 0;
#pragma unroll
    for (int k = 0; k < kAccChunks - 1; ++k) {
        const long long v = c[k] + carry;
        c[k] = v & 0xffffffffll;
        carry = v >> 32;
    }
    c[kAccChunks - 1] += carry;
}

// The accumulated value (words a[0 .. kAccWords)) as a normalised
// float-float, formed with integer and FP32 operations only: GB300 issues
// FP64 at a small fraction of its FP32 rate, and this sits on every phase's
// critical path.  The leading 48 bits are kept (truncated below).
__device__ __forceinline__ ff acc_ff(const unsigned long long* a) {
    if (a[kAccChunks]) return {__int_as_float(0x7fffffff), 0.0f};
    long long c[kAccChunks];
#pragma unroll
    for (int k = 0; k < kAccChunks; ++k) c[k] = (long long)a[k];
    acc_normalize(c);
    const bool neg = c[kAccChunks - 1] < 0;
    if (neg) {
#pragma unroll
        for (int k = 0; k < kAccChunks; ++k) c[k] = -c[k];
        acc_normalize(c);
    }
    // the top non-zero chunk t and the two below it (unrolled: the chunks
    // stay in registers)
    int t = -1;
    unsigned long long c0 = 0, c1 = 0, c2 = 0;
#pragma unroll
    for (int k = 0; k < kAccChunks; ++k) {
        if (c[k] != 0) {
            t = k;
            c0 = (unsigned long long)c[k];
            c1 = k >= 1 ? (unsigned long long)c[k - 1] : 0ull;
            c2 = k >= 2 ? (unsigned long long)c[k - 2] : 0ull;
        }
    }
    if (t < 0) return ff_zero();
    // 64-bit window from the top chunk, leading bit at bit 63: the value is
    // M 2^e0 up to the bits below the window
    const unsigned long long H = (c0 << 32) | c1;
    const unsigned long long L = c2;
    const int lz = __clzll(H);  // 0..31: c[t] is in [1, 2^32)
    const unsigned long long M = lz ? (H << lz) | (L >> (32 - lz)) : H;
    const int e0 = 32 * (t - 1) - lz - 149;
    const float hi = scalbnf((float)(unsigned)(M >> 40), e0 + 40);  // 24 bits: exact
    const unsigned long long rem = M & ((1ull << 40) - 1);
    const float lo = scalbnf(__fmaf_rn((float)(unsigned)(rem >> 20), 1048576.0f,
                                       (float)(unsigned)(rem & 0xfffffull)),
                             e0);
    ff r;
    fast_two_sum(hi, lo, r.hi, r.lo);
    return neg ? ff_neg(r) : r;
}

__device__ __forceinline__ void acc_zero(unsigned long long* a, int n, int tid, int nthreads) {
    for (int k = tid; k < n; k += nthreads) a[k] = 0ull;
}

// A row of system b is done: every thread left its shares of the phase's
// values (bit v of vals: value v) in tpart[v][thread].  Warp v sums value v
// over the block in a fixed order (each lane 8 threads' shares, then the
// lanes by shuffle tree) and adds the row's partial into the phase's exact
// accumulator.
template <int TB>
__device__ __forceinline__ void reduce_row(const SbSolveSet& S, int b, int p, int vals,
                                           ff* tpart) {
    __syncthreads();
    if (TB != kVThreads) {
        // a 512-thread block: virtual thread v's share is its even half
        // (thread v) plus its odd half (thread v + 256)
        if (threadIdx.x < kVThreads) {
#pragma unroll
            for (int v = 0; v < 3; ++v)
                if ((vals >> v) & 1)
                    tpart[v * TB + threadIdx.x] =
                        ff_add(tpart[v * TB + threadIdx.x], tpart[v * TB + kVThreads + threadIdx.x]);
        }
        __syncthreads();
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp < 3 && ((vals >> warp) & 1)) {
        const ff* t = tpart + warp * TB;
        ff x = ff_zero();
#pragma unroll
        for (int k = 0; k < kWarps; ++k) x = ff_add(x, t[lane + 32 * k]);
        x = ff_warp_sum(x);
        if (lane == 0) acc_add_ff(acc_buf(S, b, p), warp, x);
    }
    __syncthreads();
}

// Counts n finished rows of system b; returns (in every thread) whether
// they were the system's last.  The accumulator updates of the block (lane
// 0 of the first warps) come first.
__device__ __forceinline__ bool count_rows(const SbSolveSet& S, int b, int nT, int n, int* s_last) {
    if ((threadIdx.x & 31) == 0 && threadIdx.x < 32 * 3) __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const int old = atomicAdd(&S.cnt[b], n);
        *s_last = (old + n == nT);
    }
    __syncthreads();
    return *s_last != 0;
}

// ---------------------------------------------------------------------------
// Per-system scalars, in float-float on the FP32 pipes (no FP64 on the
// phase's critical path).  Records are read with L2 loads (__ldcg): they
// are written by other blocks between phases.
__device__ __forceinline__ ff to_ff(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ float2 to_f2(ff v) { return make_float2(v.hi, v.lo); }

__device__ __forceinline__ SbSolveRec load_rec(const SbSolveRec* p) {
    SbSolveRec r;
    r.rz = __ldcg(&p->rz);
    r.rr = __ldcg(&p->rr);
    r.bb = __ldcg(&p->bb);
    r.tol2 = __ldcg(&p->tol2);
    r.alpha = __ldcg(&p->alpha);
    r.beta = __ldcg(&p->beta);
    r.kind = __ldcg(&p->kind);
    r.fresh = __ldcg(&p->fresh);
    r.it = __ldcg(&p->it);
    r.conv = __ldcg(&p->conv);
    r.neu = __ldcg(&p->neu);
    return r;
}

// Final statistics of a system that leaves the solve (FP64, once).
// Written by one thread per system and solve; the counters and the worst
// residual run until sb_reset_stats (a NaN residual sticks).
__device__ __forceinline__ void write_stats(SbDevStats* st, const SbSolveRec& rc) {
    const double bb = ff_to_d(to_ff(rc.bb));
    const double rel = sqrt(ff_to_d(to_ff(rc.rr)) / bb);
    st->solver_iters = rc.it;
    st->solver_rel_resid = rel;
    st->solver_b_norm = sqrt(bb);
    st->solver_converged = rc.conv;
    st->solver_neumann = rc.neu;
    st->solves += 1;
    if (!rc.conv) st->solver_nonconverged += 1;
    if (!(rel <= st->solver_resid_max)) st->solver_resid_max = rel;
}

// The loop head of CG after r.z and r.r are known: iteration limit, NaN,
// target reached (mixed mode then checks the true residual first), else the
// next q = A p.  Returns true when the system is finished.
template <bool MIXED>
__device__ __forceinline__ bool loop_head(SbSolveRec& rc, const SolverConfig& cfg) {
    if (rc.it >= cfg.max_iter || !(rc.rr.x == rc.rr.x)) return true;
    if (ff_le(to_ff(rc.rr), to_ff(rc.tol2))) {
        if (!MIXED) {
            rc.conv = 1;
            return true;
        }
        rc.kind = K_CHECK;
        return false;
    }
    rc.kind = K_Q;
    return false;
}

// After a phase that formed r.z (A) and r.r (B): the next search direction's
// beta (none after a start or restart), then the loop head.
template <bool MIXED>
__device__ __forceinline__ bool after_rz(SbSolveRec& rc, ff A, ff B, const SolverConfig& cfg) {
    if (rc.fresh) {
        rc.beta = 0.0f;  // a new search direction (start or restart)
        rc.fresh = 0;
    } else {
        rc.beta = ff_to_f(ff_div(A, to_ff(rc.rz)));
        ++rc.it;
    }
    rc.rz = to_f2(A);
    rc.rr = to_f2(B);
    return loop_head<MIXED>(rc, cfg);
}

// Advances a system's scalars past a phase of kind rc.kind with its exact
// sums (A, B, C: the values kind_values names) and sets the next kind;
// returns true when the system is finished.  Every path that advances a
// system (one block for a set, every block for a single system) runs this
// same function on the same sums.
template <bool MIXED>
__device__ __forceinline__ bool transition(SbSolveRec& rc, ff A, ff B, ff C,
                                           const SolverConfig& cfg) {
    switch (rc.kind) {
        case K_SETUP:
        case K_SETUP_L: {
            const ff bb = C.hi > 0.0f ? C : ff{1.0f, 0.0f};
            rc.bb = to_f2(bb);
            // tol2f = tol^2 (plain) or (0.8 tol)^2 (mixed: the float-float
            // iterate is driven below tol so that the returned FP32 gamma, whose
            // rounding adds up to a few percent, still meets tol)
            rc.tol2 = to_f2(ff_mul_f(bb, cfg.tol2f));
            rc.alpha = make_float2(0.0f, 0.0f);
            rc.beta = 0.0f;
            rc.it = 0;
            rc.conv = 0;
            rc.fresh = 1;
            rc.neu = rc.kind == K_SETUP ? 1 : 0;
            if (rc.neu) {
                rc.kind = K_NEUMANN;
                return false;
            }
            return after_rz<MIXED>(rc, A, B, cfg);  // the set-up formed z = B^-1 r
        }
        case K_RESTART_L:
            rc.fresh = 1;
            return after_rz<MIXED>(rc, A, B, cfg);
        case K_NEUMANN:
        case K_UPDATE_L:
            return after_rz<MIXED>(rc, A, B, cfg);
        case K_Q:
            if (!(A.hi > 0.0f)) return true;  // breakdown: keep the current iterate
            rc.alpha = to_f2(ff_div(to_ff(rc.rz), A));
            rc.kind = rc.neu ? K_UPDATE : K_UPDATE_L;
            return false;
        case K_UPDATE:
            rc.kind = K_NEUMANN;
            return false;
        case K_CHECK:
            rc.rr = to_f2(A);
            if (ff_le(A, to_ff(rc.tol2))) {
                rc.conv = 1;
                return true;
            }
            rc.kind = rc.neu ? K_RESTART : K_RESTART_L;
            return false;
        default:  // K_RESTART
            rc.fresh = 1;
            rc.kind = K_NEUMANN;
            return false;
    }
}

// The three sums of buffer ab, for a whole block: warp 0 copies the buffer
// with coalesced L2 loads (one request per line, where a load per word from
// every block of the grid would queue on the same few lines), threads 0..2
// convert one value each; the sums land in out[0..2] (shared memory) for
// every thread after the call.
// Only the values of bit mask vals are read (each value is one line, so a
// phase that produced one value costs every block one line request, where
// all blocks of the grid read the same lines at once).
// Warp 0 only (the sums are in out[] for warp 0 afterwards).
__device__ __forceinline__ void acc_sums_warp0(const unsigned long long* ab,
                                               unsigned long long* s_w, ff* out, int vals) {
    const int lane = threadIdx.x;
    for (int l = lane; l < 3 * kAccWords; l += 32) {  // 33 words: lane 0 takes two
        const int v = l / kAccWords, w = l - v * kAccWords;
        if ((vals >> v) & 1) s_w[l] = __ldcg(ab + v * kAccSlot + w);
    }
    __syncwarp();
    if (lane < 3 && ((vals >> lane) & 1)) out[lane] = acc_ff(s_w + lane * kAccWords);
    __syncwarp();
}

__device__ __forceinline__ void acc_sums(const unsigned long long* ab, unsigned long long* s_w,
                                         ff* out, int vals) {
    if (threadIdx.x < 32) acc_sums_warp0(ab, s_w, out, vals);
    __syncthreads();
}

// Thread 0 of the block that completed system b's last row in phase p
// (sets of several systems): advance the system with the phase's sums and
// publish its scalars for phase p + 1, or retire it (from phase p + 1 on no
// block visits its rows).
template <bool MIXED>
__device__ __forceinline__ void advance(const SbSolveSet& S, int b, int p, const ff* sums,
                                        const SolverConfig& cfg) {
    SbSolveRec rc = load_rec(S.rec + (p & 1) * S.nb + b);
    if (p == 0) rc.kind = first_kind(S.descs[b]->f.stats, cfg);
    if (transition<MIXED>(rc, sums[0], sums[1], sums[2], cfg)) {
        write_stats(S.descs[b]->f.stats, rc);
        S.done_at[b] = p + 1;
        // retired: this block was the only reader of the system's buffers
        acc_zero(S.acc + (size_t)b * kSolveAccWords, kSolveAccWords, 0, 1);
    } else {
        S.rec[((p + 1) & 1) * S.nb + b] = rc;
        if (p == 0) S.done_at[b] = INT_MAX;
        acc_zero(acc_buf(S, b, p + 1), kAccBuf, 0, 1);  // read in phase p - 2
    }
    S.cnt[b] = 0;
}

// Work weight of one theta row of a system with nT rows (nP = 2 nT columns
// plus a fixed per-row cost of about 256 columns).
__device__ __forceinline__ unsigned row_weight(int nT) { return 2u * (unsigned)nT + 256u; }

// s_pre[b] = total weight of the systems before b that are active in phase
// p (every system in phase 0 and in the final pass, p < 0); s_pre[nb] is the
// total.  Every block computes the same table: a system's done_at only
// moves during phase p from INT_MAX to p + 1, which reads as active in p.
template <int TB>
__device__ __forceinline__ unsigned active_prefix(const SbSolveSet& S, int p, unsigned* s_pre) {
    __shared__ unsigned wsum[TB / 32];
    __shared__ unsigned carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < S.nb; base += TB) {
        const int b = base + threadIdx.x;
        unsigned v = 0;
        if (b < S.nb) {
            // a member retired from its batch (halted) takes no part
            const bool act = (p <= 0 || __ldcg(&S.done_at[b]) > p) && !__ldcg(&S.descs[b]->halted);
            if (act) v = (unsigned)(S.roff[b + 1] - S.roff[b]) * row_weight(S.roff[b + 1] - S.roff[b]);
        }
        unsigned incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        unsigned before = carry;
        for (int k = 0; k < w; ++k) before += wsum[k];
        if (b < S.nb) s_pre[b] = before + incl - v;
        __syncthreads();
        if (threadIdx.x == TB - 1) carry = before + incl;
        __syncthreads();
    }
    const unsigned total = carry;
    if (threadIdx.x == 0) s_pre[S.nb] = total;
    __syncthreads();
    return total;
}

// First system whose weight range ends after `x` (s_pre is non-decreasing).
__device__ __forceinline__ int first_system_after(const unsigned* s_pre, int nb, unsigned x) {
    int lo = 0, hi = nb;  // answer in [0, nb)
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s_pre[mid + 1] > x) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// Stages system b's descriptor in shared memory.
__device__ __forceinline__ void stage_desc(const SbSolveSet& S, int b, SbBubbleDesc* s_d) {
    constexpr int kWords = (int)(sizeof(SbBubbleDesc) / 4);
    const int* src = reinterpret_cast<const int*>(S.descs[b]);
    int* dst = reinterpret_cast<int*>(s_d);
    for (int k = threadIdx.x; k < kWords; k += blockDim.x) dst[k] = src[k];
    __syncthreads();
}

// Stores the preconditioner's result D (in the block's work array) as this
// thread's columns of row i of z1.
template <int PER, int TB>
__device__ __forceinline__ void store_z1(const SbGrid& g, const SbFields& f, int i,
                                         const Stage& St) {
    const int row = i * g.nP;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = col_of<TB>(k);
        if (j < g.nP) f.z1[row + j] = St.work[j];
    }
}

// Stores the preconditioner's result D as this thread's columns of row i
// of z and adds the columns' r.z and r.r terms (column order).
template <bool MIXED, int PER, int TB>
__device__ __forceinline__ void store_z_dots(const SbGrid& g, const SbFields& f, int i,
                                             const Stage& St, const float (&rv)[PER], ff& a,
                                             ff& b2) {
    const int row = i * g.nP;
    ff ha[2] = {ff_zero(), ff_zero()}, hb[2] = {ff_zero(), ff_zero()};
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = col_of<TB>(k);
        if (j < g.nP) {
            const float z = St.work[j];
            f.z[row + j] = z;
            const int hk = half_of<TB>(k);
            ha[hk] = acc<MIXED>(ha[hk], rv[k], z);
            hb[hk] = acc<MIXED>(hb[hk], rv[k], rv[k]);
        }
    }
    a = fold_halves<TB>(ha);
    b2 = fold_halves<TB>(hb);
}

// w = C z1 on row i: the theta couplings (weights cS of the faces north and
// south of each cell) applied to the neighbouring rows of z1; z1 and r of
// the row itself are returned in zo and ro (loaded with the rest, before
// the row solve that w feeds).
template <int PER, int TB>
__device__ __forceinline__ void row_theta_coupling(const SbGrid& g, const SbFields& f, int i,
                                                   float (&w)[PER], float (&zo)[PER],
                                                   float (&ro)[PER]) {
    const int nP = g.nP, nT = g.nT, row = i * nP;
    const float* __restrict__ z1 = f.z1;
    const float* __restrict__ cS = f.cS;
    const float* __restrict__ r = f.r;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = col_of<TB>(k);
        w[k] = 0.0f;
        zo[k] = 0.0f;
        ro[k] = 0.0f;
        if (j < nP) {
            const int c = row + j;
            float v = 0.0f;
            if (i < nT - 1) v = cS[c] * z1[c + nP];
            if (i > 0) v += cS[c - nP] * z1[c - nP];
            w[k] = v;
            zo[k] = z1[c];
            ro[k] = r[c];
        }
    }
}

// The work of a phase of kind `kind` on theta row i of one system (see the
// kinds above).  The preconditioner is a two-term Neumann series of the
// phi-line splitting A = B - C (C: the theta couplings, non-negative):
// M^-1 = B^-1 + B^-1 C B^-1, symmetric and positive definite because the
// splitting of this M-matrix is regular (spectral radius of B^-1 C below
// one).  Against B^-1 alone it halves the iterations on ruptured films (an
// offline study on oracle states: 29 -> 15 at step 600 of c1) at the cost
// of one more phase per iteration.  Each thread's shares of the row's dot
// products go to the block's work arrays (after the preconditioner's D)
// for reduce_row.
template <bool MIXED, int PER, int TB>
__device__ __forceinline__ void row_phase(const SbGrid& g, const SbFields& f,
                                          const SolverConfig& cfg, int i, int kind,
                                          float beta, ff alpha, float* pA, const float* pB,
                                          Stage& St, bool own_row = false) {
    (void)cfg;
    ff a = ff_zero(), b2 = ff_zero(), c2 = ff_zero();
    float rv[PER];
    switch (kind) {
        case K_SETUP:
        case K_SETUP_L:
            row_init<MIXED, PER, TB>(g, f, i, cfg, rv, c2);
            precondition_row<PER, TB, true>(g, f, i, St, rv, !own_row);
            break;
        case K_NEUMANN: {
            stage_fetch(St, row_blob(g, f, i), factor_blob(g.nP).bytes);
            float z1v[PER], r0v[PER];
            row_theta_coupling<PER, TB>(g, f, i, rv, z1v, r0v);
            precondition_row<PER, TB, false>(g, f, i, St, rv);
            const int row = i * g.nP;
            ff ha[2] = {ff_zero(), ff_zero()}, hb[2] = {ff_zero(), ff_zero()};
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const int j = col_of<TB>(k);
                if (j < g.nP) {
                    const int c = row + j;
                    const float z = z1v[k] + St.work[j];
                    const float r = r0v[k];
                    f.z[c] = z;
                    const int hk = half_of<TB>(k);
                    ha[hk] = acc<MIXED>(ha[hk], r, z);
                    hb[hk] = acc<MIXED>(hb[hk], r, r);
                }
            }
            a = fold_halves<TB>(ha);
            b2 = fold_halves<TB>(hb);
            break;
        }
        case K_Q:
            a = row_spmv<MIXED, PER, TB>(g, f, i, beta, pB, pA);
            break;
        case K_UPDATE:
        case K_UPDATE_L:
            // the row's factors travel while the update runs
            stage_fetch(St, row_blob(g, f, i), factor_blob(g.nP).bytes);
            row_update<MIXED, PER, TB>(g, f, i, alpha, pA, rv);
            precondition_row<PER, TB, false>(g, f, i, St, rv);
            break;
        case K_CHECK:
            if (MIXED) a = row_true_residual<PER, TB>(g, f, i);
            break;
        default:  // K_RESTART, K_RESTART_L
            stage_fetch(St, row_blob(g, f, i), factor_blob(g.nP).bytes);
            row_load_r<PER, TB>(g, f, i, rv);
            precondition_row<PER, TB, false>(g, f, i, St, rv);
            break;
    }
    // the line-preconditioner kinds (_L, the last three) store z = B^-1 r and
    // its dot products where the Neumann kinds store z1 = B^-1 r
    if (kind >= K_SETUP_L) store_z_dots<MIXED, PER, TB>(g, f, i, St, rv, a, b2);
    else if (kind == K_SETUP || kind == K_UPDATE || kind == K_RESTART) store_z1<PER, TB>(g, f, i, St);
    // this thread's shares of the values the kind produces, for reduce_row
    // (after D: the other threads may still read their D entries)
    const int vals = kind_values(kind);
    ff* tpart = reinterpret_cast<ff*>(St.work + g.nP);
    if (vals & 1) tpart[threadIdx.x] = a;
    if (vals & 2) tpart[TB + threadIdx.x] = b2;
    if (vals & 4) tpart[2 * TB + threadIdx.x] = c2;
}

// The solve of a set of systems: each system runs the phase kinds of its
// record (set-up, then per iteration q = A p, update, Neumann term; in
// mixed mode the refinement check and restart).  In
// every phase the rows of the systems still iterating are split into G
// contiguous ranges of equal work weight, one per block, so a block meets
// one or two systems per phase and a system that iterates longer than the
// others still spreads over the whole GPU.  Each block adds its rows'
// partials into the system's exact accumulator and counts the rows; the
// block that completes a system reads the sums and advances it.  The loop
// ends when no system is left.
template <bool MIXED, int PER, int TB>
__global__ void __launch_bounds__(TB, 1024 / TB)
k_solve(SbSolveSet S, SolverConfig cfg) {
    extern __shared__ __align__(16) float sm[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ __align__(16) SbBubbleDesc s_d;
    __shared__ unsigned s_pre[kMaxSystems + 1];
    __shared__ int s_last;
    __shared__ unsigned long long s_w[3 * kAccWords];
    __shared__ ff s_sums[3];
    __shared__ SbSolveRec s_rc;
    int staged = -1;  // system whose descriptor is in s_d
    int* const faults = &S.descs[0]->f.stats->wait_faults;
    if (*faults) return;  // a wait gave up earlier: the barrier word is not trusted any more
    unsigned gen = grid_barrier_gen(S.bar);
    Stage St;
    stage_init(St, &bar, sm, cfg.blob);
    const unsigned G = gridDim.x;

    for (int p = 0;; ++p) {
        const unsigned W = active_prefix<TB>(S, p, s_pre);
        if (W == 0) break;  // same in every block
        const unsigned lo = (unsigned)(((unsigned long long)W * blockIdx.x) / G);
        const unsigned hi = (unsigned)(((unsigned long long)W * (blockIdx.x + 1)) / G);
        for (int b = first_system_after(s_pre, S.nb, lo); b < S.nb && s_pre[b] < hi; ++b) {
            const unsigned w0 = s_pre[b];
            if (s_pre[b + 1] == w0) continue;  // not active
            const int nT = S.roff[b + 1] - S.roff[b];
            const unsigned wr = row_weight(nT);
            // rows whose start weight w0 + i wr lies in [lo, hi)
            const int i0 = lo > w0 ? (int)((lo - w0 + wr - 1) / wr) : 0;
            const int i1 = min(nT, (int)((hi - w0 + wr - 1) / wr));
            if (i0 >= i1) continue;
            // the system's scalars (one thread loads them: every block of the
            // grid reads the same record), staged with the descriptor
            if (threadIdx.x == 0) {
                SbSolveRec rc;
                rc.kind = p == 0 ? first_kind(S.descs[b]->f.stats, cfg) : K_SETUP;
                rc.it = 0;
                rc.beta = 0.0f;
                rc.alpha = make_float2(0.0f, 0.0f);
                if (p > 0) {
                    const SbSolveRec* rp = S.rec + (p & 1) * S.nb + b;
                    rc.kind = __ldcg(&rp->kind);
                    rc.it = __ldcg(&rp->it);
                    rc.beta = __ldcg(&rp->beta);
                    rc.alpha = __ldcg(&rp->alpha);
                }
                s_rc = rc;
            }
            if (b != staged) {
                stage_desc(S, b, &s_d);  // constant during the solve
                staged = b;
            } else {
                __syncthreads();
            }
            const int kind = s_rc.kind, it = s_rc.it, vals = kind_values(kind);
            const float beta = s_rc.beta;
            const ff alpha = to_ff(s_rc.alpha);
            const SbGrid& g = s_d.g;
            const SbFields& f = s_d.f;
            float* pA = (it & 1) ? f.q : f.p;  // p_new of iteration it
            float* pB = (it & 1) ? f.p : f.q;  // p_old
            bool last = false;
            for (int i = i0; i < i1; ++i) {
                const int k = (i - i0) % kRowChunk;
                row_phase<MIXED, PER, TB>(g, f, cfg, i, kind, beta, alpha, pA, pB, St);
                if (vals) reduce_row<TB>(S, b, p, vals, reinterpret_cast<ff*>(St.work + g.nP));
                // count every kRowChunk rows and at the end; the block that
                // completes the system advances it
                if (k == kRowChunk - 1 || i == i1 - 1) last = count_rows(S, b, nT, k + 1, &s_last);
            }
            if (last) {
                __threadfence();
                if (vals) acc_sums(acc_buf(S, b, p), s_w, s_sums, vals);
                if (threadIdx.x == 0) advance<MIXED>(S, b, p, s_sums, cfg);
            }
            __syncthreads();  // s_d and s_last are reused
        }
        if (!grid_barrier(S.bar, gen, G, faults)) {
            stage_wait(St, S.descs[0]->f.stats);  // no copy may land after the block left
            return;
        }
    }
    // the increment and the new gamma of every system, same split with all
    // systems counted
    const unsigned W = active_prefix<TB>(S, -1, s_pre);
    const unsigned lo = (unsigned)(((unsigned long long)W * blockIdx.x) / G);
    const unsigned hi = (unsigned)(((unsigned long long)W * (blockIdx.x + 1)) / G);
    for (int b = first_system_after(s_pre, S.nb, lo); b < S.nb && s_pre[b] < hi; ++b) {
        const unsigned w0 = s_pre[b];
        const int nT = S.roff[b + 1] - S.roff[b];
        const unsigned wr = row_weight(nT);
        const int i0 = lo > w0 ? (int)((lo - w0 + wr - 1) / wr) : 0;
        const int i1 = min(nT, (int)((hi - w0 + wr - 1) / wr));
        if (i0 >= i1) continue;
        stage_desc(S, b, &s_d);
        for (int i = i0; i < i1; ++i) row_final<MIXED, PER, TB>(s_d.g, s_d.f, i);
        if (i0 == 0 && threadIdx.x == 0) s_d.f.stats->dx_valid = 1;
        __syncthreads();
    }
}

// The solve of one system (a bubble stepped alone): the same phases, row
// work and scalar transitions as k_solve, with the bubble's descriptor in
// kernel parameters.  Rows are dealt round robin.  After every barrier each
// block reads the previous phase's exact sums and advances the scalars
// itself, so no block waits for another.  The sums, and so every scalar and
// result, are bit-identical to solving the same system inside a set (this
// file is compiled without multiply-add contraction, so both kernels round
// the same operations the same way).
template <bool MIXED, int PER, int TB>
__global__ void __launch_bounds__(TB, 1024 / TB)
k_solve_one(SbGrid g, SbFields f, SbSolveSet S, SolverConfig cfg) {
    extern __shared__ __align__(16) float sm[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ SbSolveRec s_rc;  // the system's scalars (the same in every block)
    __shared__ int s_done;
    __shared__ unsigned long long s_w[3 * kAccWords];
    __shared__ ff s_sums[3];
    if (f.stats->wait_faults) return;  // a wait gave up earlier: the barrier word is not trusted
    if (f.self->halted) return;        // the bubble stopped at a failed solve (sb_run)
    unsigned gen = grid_barrier_gen(S.bar);
    if (threadIdx.x == 0) s_rc.kind = first_kind(f.stats, cfg);
    Stage St;
    stage_init(St, &bar, sm, cfg.blob);  // (its barrier publishes s_rc.kind)
    const int G = gridDim.x, nT = g.nT;
    for (int p = 0;; ++p) {
        if (p > 0) {
            // warp 0 reads the sums (if the phase produced any) and advances
            // the scalars; one barrier
            if (threadIdx.x < 32) {
                const int pv = kind_values(s_rc.kind);
                if (pv) acc_sums_warp0(acc_buf(S, 0, p - 1), s_w, s_sums, pv);
                if (threadIdx.x == 0) {
                    s_done = transition<MIXED>(s_rc, s_sums[0], s_sums[1], s_sums[2], cfg) ? 1 : 0;
                    if (s_done && blockIdx.x == 0) write_stats(f.stats, s_rc);
                }
            }
            __syncthreads();
            if (s_done) break;  // same decision in every block
        }
        // the buffer of phase p + 1 was last read at the start of phase p - 1
        if (blockIdx.x == 0) acc_zero(acc_buf(S, 0, p + 1), kAccBuf, threadIdx.x, blockDim.x);
        const int kind = s_rc.kind, it = s_rc.it, vals = kind_values(kind);
        const float beta = s_rc.beta;
        const ff alpha = to_ff(s_rc.alpha);
        float* pA = (it & 1) ? f.q : f.p;  // p_new of iteration it
        float* pB = (it & 1) ? f.p : f.q;  // p_old
        for (int i = blockIdx.x; i < nT; i += G) {
            row_phase<MIXED, PER, TB>(g, f, cfg, i, kind, beta, alpha, pA, pB, St, G >= nT);
            if (vals) reduce_row<TB>(S, 0, p, vals, reinterpret_cast<ff*>(St.work + g.nP));
        }
        if (!grid_barrier(S.bar, gen, G, &f.stats->wait_faults)) {
            stage_wait(St, f.stats);  // no copy may land after the block left
            return;
        }
    }
    // every block has read its last sums: clear the buffers for the next solve
    if (!grid_barrier(S.bar, gen, G, &f.stats->wait_faults)) return;
    if (blockIdx.x == 0) acc_zero(S.acc, kSolveAccWords, threadIdx.x, blockDim.x);
    for (int i = blockIdx.x; i < nT; i += G) row_final<MIXED, PER, TB>(g, f, i);
    if (blockIdx.x == 0 && threadIdx.x == 0) f.stats->dx_valid = 1;
}

template <bool MIXED>
const void* solve_one_kernel(int per) {
    switch (per) {
        case 1: return (const void*)k_solve_one<MIXED, 1, 256>;
        case 2: return (const void*)k_solve_one<MIXED, 2, 256>;
        case 4: return (const void*)k_solve_one<MIXED, 4, 256>;
        default: return (const void*)k_solve_one<MIXED, 4, 512>;  // rows of 2048 columns
    }
}

template <bool MIXED>
const void* solve_kernel(int per) {
    switch (per) {
        case 1: return (const void*)k_solve<MIXED, 1, 256>;
        case 2: return (const void*)k_solve<MIXED, 2, 256>;
        case 4: return (const void*)k_solve<MIXED, 4, 256>;
        default: return (const void*)k_solve<MIXED, 4, 512>;  // rows of 2048 columns
    }
}

// Target r.r / |b|^2 of the iterate.
float tol2_factor(const SolverConfig& cfg) {
    return (float)((cfg.mode == 1 ? 0.64 : 1.0) * cfg.tol * cfg.tol);
}

// Kernel variant of rows of up to nP columns: 1, 2, 4 columns per thread
// of 256-thread blocks, or 8 for 2048 columns (512-thread blocks, four
// columns per thread).
int per_of(int nP) {
    int per = (nP + kVThreads - 1) / kVThreads;
    return per <= 1 ? 1 : per <= 2 ? 2 : per <= 4 ? 4 : 8;
}

int threads_of(int per) { return per == 8 ? 512 : kVThreads; }

// Dynamic shared memory of one solve block for rows of up to nP columns:
// the factor blob of one row and the work arrays: the four nP-float arrays
// of the preconditioner build (the replay needs 1.5 nP floats), which also
// hold the result D (nP floats) followed by the threads' dot-product shares
// (3 x threads float-float).  For
// nP = 1024 that is 47 KB, so four 256-thread blocks share an SM next to
// their static shared memory.
size_t solve_smem(int nP) {
    const size_t tb = (size_t)threads_of(per_of(nP));
    const size_t work = std::max<size_t>(16 * (size_t)nP, 4 * (size_t)nP + 3 * tb * sizeof(ff));
    return (size_t)factor_blob(nP).bytes + work;
}

const void* kernel_for(int per, int mode, bool one) {
    if (one) return mode == 1 ? solve_one_kernel<true>(per) : solve_one_kernel<false>(per);
    return mode == 1 ? solve_kernel<true>(per) : solve_kernel<false>(per);
}

// Largest dynamic shared memory of a kernel variant (PER columns per thread
// serve rows of up to PER * 256 columns; smaller rows need less).
size_t variant_smem(int per) {
    size_t m = 0;
    for (int nP = 16; nP <= per * kVThreads; nP *= 2)
        if (per_of(nP) == per) m = std::max(m, solve_smem(nP));
    return m;
}

// Co-resident blocks of a kernel variant (cached per device).  The first
// query also declares the variant's largest dynamic shared memory (the 48 KB
// default limit counts static shared memory too, and a launch above the
// declared size is refused).
int max_blocks(int per, int mode, bool one) {
    static int cache[16][4][2][2];
    int dev = 0;
    cudaGetDevice(&dev);
    const int pi = per == 1 ? 0 : per == 2 ? 1 : per == 4 ? 2 : 3;
    int& c = cache[dev & 15][pi][mode & 1][one ? 1 : 0];
    if (c > 0) return c;
    const void* fn = kernel_for(per, mode, one);
    const size_t smem = variant_smem(per);
    int sms = 0, occ = 0;
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads_of(per), smem);
    c = sms * (occ > 0 ? occ : 1);
    return c;
}

}  // namespace

cudaError_t prepare_solve(int maxNP, const SolverConfig& cfg, int* blocks) {
    if (maxNP > kMaxNP) return cudaErrorInvalidValue;
    const int b = max_blocks(per_of(maxNP), cfg.mode, false);
    max_blocks(per_of(maxNP), cfg.mode, true);
    if (blocks) *blocks = b;
    return cudaGetLastError();
}

cudaError_t launch_solve_one(const SbGrid& g, const SbFields& f, const SbSolveSet& set,
                             const SolverConfig& cfg, cudaStream_t s) {
    if (g.nP > kMaxNP || set.nb != 1) return cudaErrorInvalidValue;
    const int per = per_of(g.nP);
    const int G = std::min(g.nT, max_blocks(per, cfg.mode, true));
    SbGrid gg = g;
    SbFields ff = f;
    SbSolveSet ss = set;
    SolverConfig cc = cfg;
    cc.blob = factor_blob(g.nP).bytes;
    cc.tol2f = tol2_factor(cfg);
    void* args[] = {&gg, &ff, &ss, &cc};
    return cudaLaunchCooperativeKernel(kernel_for(per, cfg.mode, true), dim3(G), dim3(threads_of(per)),
                                       args, solve_smem(g.nP), s);
}

cudaError_t launch_solve(const SbSolveSet& set, int maxNP, const SolverConfig& cfg,
                         cudaStream_t s) {
    if (maxNP > kMaxNP || set.R <= 0) return cudaErrorInvalidValue;
    const int per = per_of(maxNP);
    const int G = std::min(set.R, max_blocks(per, cfg.mode, false));
    SbSolveSet ss = set;
    SolverConfig cc = cfg;
    cc.blob = factor_blob(maxNP).bytes;
    cc.tol2f = tol2_factor(cfg);
    void* args[] = {&ss, &cc};
    return cudaLaunchCooperativeKernel(kernel_for(per, cfg.mode, false), dim3(G), dim3(threads_of(per)),
                                       args, solve_smem(maxNP), s);
}

}  // namespace sb
