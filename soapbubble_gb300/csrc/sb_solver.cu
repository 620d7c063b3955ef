// Implicit surfactant solve: preconditioned conjugate gradients on the
// symmetric positive definite 5-point system assembled by k_assemble.  It
// replaces the reference's AmgX PCGF + AMG solve (kernel/bubble.cu:1479-1508,
// init/PCGF_F.json).  The reference starts from x0 = gamma; here the unknown
// is the increment dx = gamma_new - gamma_adv, starting from dx = 0, which is
// the same iteration with the large common part removed.
//
// One cooperative launch runs the whole solve.  Each block owns whole theta
// rows; phases are separated by grid-wide barriers; dot products are summed
// per block and then by every block in the same block order, so every block
// sees bit-identical scalars and takes the same loop decisions (the
// iteration count is bounded by max_iter).
//
// Preconditioner: exact solve of each theta row's periodic tridiagonal block
// (phi couplings; the theta couplings stay on its diagonal).  Near the poles
// the phi couplings carry 1/sin(theta) and dominate the diagonal by 1e4-1e5,
// which is what makes point Jacobi slow there.  The row solve is parallel
// cyclic reduction in shared memory, written in "excess" form: each equation
// keeps (excess e, |lower|, |upper|, rhs) with diagonal = e + |lower| + |upper|,
// and every update adds positive terms, so FP32 keeps full relative accuracy
// even when the diagonal exceeds the off-diagonal sum by a factor 1 + 1e-5
// (the Grassmann-Taksar-Heyman idea applied to cyclic reduction).
//
// Modes: plain FP32 (FP32 vectors and sums), or mixed precision (FP32 SpMV
// and preconditioner, FP64 iterate and dot products, and a true FP64
// residual check that restarts CG from the refined iterate until the
// relative residual target holds).
#include <cooperative_groups.h>

#include "sb_internal.h"

namespace cg = cooperative_groups;

namespace sb {

namespace {

constexpr int kSolveBlock = 256;

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block partial sums of three values into part[3 * blockIdx.x + k].
__device__ __forceinline__ void block_partial3(double a, double b, double c, double* part) {
    __shared__ double sm[3][kSolveBlock / 32];
    a = warp_sum(a);
    b = warp_sum(b);
    c = warp_sum(c);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { sm[0][w] = a; sm[1][w] = b; sm[2][w] = c; }
    __syncthreads();
    if (w == 0) {
        double x = l < kSolveBlock / 32 ? sm[0][l] : 0.0;
        double y = l < kSolveBlock / 32 ? sm[1][l] : 0.0;
        double z = l < kSolveBlock / 32 ? sm[2][l] : 0.0;
        x = warp_sum(x); y = warp_sum(y); z = warp_sum(z);
        if (l == 0) {
            part[3 * blockIdx.x + 0] = x;
            part[3 * blockIdx.x + 1] = y;
            part[3 * blockIdx.x + 2] = z;
        }
    }
    __syncthreads();
}

// Sum of all blocks' partials, same order in every block.
__device__ __forceinline__ void all_sum3(const double* part, int G, double& A, double& B,
                                         double& C) {
    __shared__ double res[3];
    if (threadIdx.x < 32) {
        double x = 0.0, y = 0.0, z = 0.0;
        for (int k = threadIdx.x; k < G; k += 32) {
            x += part[3 * k + 0];
            y += part[3 * k + 1];
            z += part[3 * k + 2];
        }
        x = warp_sum(x); y = warp_sum(y); z = warp_sum(z);
        if (threadIdx.x == 0) { res[0] = x; res[1] = y; res[2] = z; }
    }
    __syncthreads();
    A = res[0]; B = res[1]; C = res[2];
    __syncthreads();
}

// (A v)_c for a cell c = (i, j); T is float or double.
template <typename T, typename A>
__device__ __forceinline__ A apply_A(const SbGrid& g, const SbFields& f, const T* __restrict__ v,
                                     int c, int i, int j) {
    const int nP = g.nP;
    const int e = i * nP + ((j + 1) & g.maskP);
    const int w = i * nP + ((j - 1) & g.maskP);
    const A vc = (A)v[c];
    A s = (A)f.dmass[c] * vc + (A)f.cE[c] * (vc - (A)v[e]) + (A)f.cE[w] * (vc - (A)v[w]);
    if (i < g.nT - 1) s += (A)f.cS[c] * (vc - (A)v[c + nP]);
    if (i > 0) s += (A)f.cS[c - nP] * (vc - (A)v[c - nP]);
    return s;
}

// z = M^-1 r on theta row i: Jacobi, or the exact periodic tridiagonal solve.
// sm holds 4 * nP floats.  Adds this row's r.z and r.r to rz, rr.
// PER = equations per thread (nP <= PER * kSolveBlock).
//
// The row matrix does not change during a solve, so the first application
// (BUILD) runs the full cyclic reduction and stores, per level, the two
// elimination factors of every equation (f.pcr) and the number of levels the
// row needed (f.pcr_levels); later applications only replay
// D' = D + a D[j - s] + c D[j + s] with the stored factors.
template <bool MIXED, int PER, bool BUILD>
__device__ __forceinline__ void precondition_row(const SbGrid& g, const SbFields& f,
                                                 const SolverConfig& cfg, int i, float* sm,
                                                 double& rz, double& rr) {
    const int nP = g.nP, nT = g.nT, mask = g.maskP;
    const int row = i * nP;
    if (cfg.precond == 0) {
        for (int j = threadIdx.x; j < nP; j += blockDim.x) {
            const int c = row + j;
            float dg = f.dmass[c] + f.cE[c] + f.cE[row + ((j - 1) & mask)];
            if (i < nT - 1) dg += f.cS[c];
            if (i > 0) dg += f.cS[c - nP];
            const float rc = f.r[c];
            const float zc = rc / dg;
            f.z[c] = zc;
            rz += MIXED ? (double)rc * (double)zc : (double)(rc * zc);
            rr += MIXED ? (double)rc * (double)rc : (double)(rc * rc);
        }
        return;
    }
    // factor storage of this row: level l at f.pcr[(l * nT + i) * nP + j]
    const size_t lvl_stride = (size_t)nT * nP;
    float2* fac = f.pcr + (size_t)row;
    if (BUILD) {
        float* E = sm;            // excess: diagonal minus the phi couplings
        float* L = sm + nP;       // |coupling to j - s|
        float* U = sm + 2 * nP;   // |coupling to j + s|
        float* D = sm + 3 * nP;   // right-hand side
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int j = threadIdx.x + k * kSolveBlock;
            if (j < nP) {
                const int c = row + j;
                float ex = f.dmass[c];
                if (i < nT - 1) ex += f.cS[c];
                if (i > 0) ex += f.cS[c - nP];
                E[j] = ex;
                U[j] = f.cE[c];
                L[j] = f.cE[row + ((j - 1) & mask)];
                D[j] = f.r[c];
            }
        }
        __syncthreads();
        // Parallel cyclic reduction: after the step with stride s every
        // equation couples j to j -/+ 2s (indices mod nP).  It stops early
        // once every coupling is below 2^-26 of its excess (the row has
        // decoupled to float precision); otherwise it ends with 2 x 2
        // solves of j and j + nP/2.
        bool decoupled = false;
        int levels = 0;
        for (int s = 1; s <= nP / 4; s <<= 1) {
            float nE[PER], nL[PER], nU[PER], nD[PER];
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const int j = threadIdx.x + k * kSolveBlock;
                if (j < nP) {
                    const int jm = (j - s) & mask, jp = (j + s) & mask;
                    const float bm = E[jm] + L[jm] + U[jm];
                    const float bp = E[jp] + L[jp] + U[jp];
                    // fast division: the preconditioner stays a fixed operator
                    const float am = __fdividef(L[j], bm);
                    const float cp = __fdividef(U[j], bp);
                    fac[levels * lvl_stride + j] = make_float2(am, cp);
                    nE[k] = E[j] + am * E[jm] + cp * E[jp];
                    nL[k] = am * L[jm];
                    nU[k] = cp * U[jp];
                    nD[k] = D[j] + am * D[jm] + cp * D[jp];
                }
            }
            __syncthreads();
            bool need = false;
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const int j = threadIdx.x + k * kSolveBlock;
                if (j < nP) {
                    E[j] = nE[k]; L[j] = nL[k]; U[j] = nU[k]; D[j] = nD[k];
                    need |= (nL[k] + nU[k]) > 1.4901161e-8f * nE[k];
                }
            }
            ++levels;
            if (!__syncthreads_or(need)) {
                decoupled = true;
                break;
            }
        }
        if (threadIdx.x == 0) f.pcr_levels[i] = decoupled ? levels : -levels;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int j = threadIdx.x + k * kSolveBlock;
            if (j < nP) {
                float c1, c2;
                if (decoupled) {
                    c1 = 1.0f / (E[j] + L[j] + U[j]);
                    c2 = 0.0f;
                } else {
                    const int kk = (j + nP / 2) & mask;
                    const float mj = L[j] + U[j], mk = L[kk] + U[kk];
                    const float ej = E[j], ek = E[kk];
                    const float idet = 1.0f / (ej * ek + ej * mk + mj * ek);
                    c1 = (ek + mk) * idet;
                    c2 = mj * idet;
                }
                fac[levels * lvl_stride + j] = make_float2(c1, c2);
                const int kk = (j + nP / 2) & mask;
                const float zj = c1 * D[j] + c2 * D[kk];
                const int c = row + j;
                const float rc = f.r[c];
                f.z[c] = zj;
                rz += MIXED ? (double)rc * (double)zj : (double)(rc * zj);
                rr += MIXED ? (double)rc * (double)rc : (double)(rc * rc);
            }
        }
        __syncthreads();
        return;
    }
    // replay with the stored factors; D ping-pongs between two buffers
    float* D0 = sm;
    float* D1 = sm + nP;
    const int lv = f.pcr_levels[i];
    const int levels = lv < 0 ? -lv : lv;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = threadIdx.x + k * kSolveBlock;
        if (j < nP) D0[j] = f.r[row + j];
    }
    __syncthreads();
    // the factors of level l + 1 are loaded while level l is reduced
    float2 acn[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = threadIdx.x + k * kSolveBlock;
        acn[k] = j < nP ? fac[j] : make_float2(0.0f, 0.0f);
    }
    int s = 1;
    for (int l = 0; l < levels; ++l, s <<= 1) {
        float* Din = (l & 1) ? D1 : D0;
        float* Dout = (l & 1) ? D0 : D1;
        float2 ac[PER];
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            ac[k] = acn[k];
            const int j = threadIdx.x + k * kSolveBlock;
            if (j < nP) acn[k] = fac[(l + 1) * lvl_stride + j];
        }
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int j = threadIdx.x + k * kSolveBlock;
            if (j < nP)
                Dout[j] = Din[j] + ac[k].x * Din[(j - s) & mask] + ac[k].y * Din[(j + s) & mask];
        }
        __syncthreads();
    }
    const float* Dn = (levels & 1) ? D1 : D0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int j = threadIdx.x + k * kSolveBlock;
        if (j < nP) {
            const float2 cc = acn[k];  // the final factors
            const float zj = cc.x * Dn[j] + cc.y * Dn[(j + nP / 2) & mask];
            const int c = row + j;
            const float rc = f.r[c];
            f.z[c] = zj;
            rz += MIXED ? (double)rc * (double)zj : (double)(rc * zj);
            rr += MIXED ? (double)rc * (double)rc : (double)(rc * rc);
        }
    }
    __syncthreads();
}

// One cooperative launch per solve.  The search direction is double
// buffered: the SpMV phase forms p_new = z + beta p_old for its own rows and,
// on the fly, for the neighbouring rows it reads, so one grid barrier per
// iteration is saved.
template <bool MIXED, int PER>
__global__ void __launch_bounds__(kSolveBlock, 4)
k_pcg(SbGrid g, SbFields f, SolverConfig cfg) {
    extern __shared__ float sm[];
    cg::grid_group grid = cg::this_grid();
    const int G = gridDim.x;
    const int nP = g.nP, nT = g.nT;
    double* partA = f.partials;
    double* partB = f.partials + 3 * G;

    // dx = 0, r = r0, z = M^-1 r (p_old = 0, beta = 0)
    double rz = 0, rr = 0, bb = 0;
    {
        double a = 0, b2 = 0, c2 = 0;
        for (int i = blockIdx.x; i < nT; i += G) {
            for (int j = threadIdx.x; j < nP; j += blockDim.x) {
                const int c = i * nP + j;
                if (MIXED) f.x64[c] = 0.0;
                else f.dx[c] = 0.0f;
                f.r[c] = f.r0[c];
                f.q[c] = 0.0f;  // p_old
                const double b = (double)f.rhs[c];
                c2 += b * b;
            }
            __syncthreads();
            precondition_row<MIXED, PER, true>(g, f, cfg, i, sm, a, b2);
        }
        block_partial3(a, b2, c2, partA);
    }
    grid.sync();
    all_sum3(partA, G, rz, rr, bb);
    const double bnorm = bb > 0.0 ? sqrt(bb) : 1.0;
    // the FP64 iterate is driven to 0.8 tol so that the returned FP32 gamma
    // (whose rounding adds up to a few percent) still meets tol
    const double tol2 = (MIXED ? 0.64 : 1.0) * cfg.tol * cfg.tol * bnorm * bnorm;
    float* pold = f.q;
    float* pnew = f.p;
    float beta = 0.0f;
    int it = 0;
    bool conv = false;
    while (it < cfg.max_iter) {
        if (!(rr == rr)) break;  // NaN: give up (same decision in every block)
        if (rr <= tol2) {
            if (!MIXED) { conv = true; break; }
            // true FP64 residual of the refined iterate
            double a = 0;
            for (int i = blockIdx.x; i < nT; i += G)
                for (int j = threadIdx.x; j < nP; j += blockDim.x) {
                    const int c = i * nP + j;
                    const double r = (double)f.r0[c] - apply_A<double, double>(g, f, f.x64, c, i, j);
                    f.r[c] = (float)r;
                    a += r * r;
                }
            block_partial3(a, 0.0, 0.0, partB);
            grid.sync();
            double d1, d2;
            all_sum3(partB, G, rr, d1, d2);
            if (rr <= tol2) { conv = true; break; }
            // restart CG from the refined iterate
            double a2 = 0, b2 = 0;
            for (int i = blockIdx.x; i < nT; i += G) {
                precondition_row<MIXED, PER, false>(g, f, cfg, i, sm, a2, b2);
            }
            block_partial3(a2, b2, 0.0, partA);
            grid.sync();
            all_sum3(partA, G, rz, rr, d1);
            beta = 0.0f;
        }
        // p_new = z + beta p_old; q = A p_new; <p_new, q>
        {
            double pq = 0;
            for (int i = blockIdx.x; i < nT; i += G)
                for (int j = threadIdx.x; j < nP; j += blockDim.x) {
                    const int c = i * nP + j;
                    const int e = i * nP + ((j + 1) & g.maskP);
                    const int w = i * nP + ((j - 1) & g.maskP);
                    const float pc = f.z[c] + beta * pold[c];
                    pnew[c] = pc;
                    float qf = f.dmass[c] * pc + f.cE[c] * (pc - (f.z[e] + beta * pold[e])) +
                               f.cE[w] * (pc - (f.z[w] + beta * pold[w]));
                    if (i < nT - 1) {
                        const int sc = c + nP;
                        qf += f.cS[c] * (pc - (f.z[sc] + beta * pold[sc]));
                    }
                    if (i > 0) {
                        const int nc = c - nP;
                        qf += f.cS[nc] * (pc - (f.z[nc] + beta * pold[nc]));
                    }
                    f.x[c] = qf;  // q lives in x until the final phase
                    pq += MIXED ? (double)pc * (double)qf : (double)(pc * qf);
                }
            block_partial3(pq, 0.0, 0.0, partA);
        }
        grid.sync();
        double pq, d1, d2;
        all_sum3(partA, G, pq, d1, d2);
        if (!(pq > 0.0)) break;
        const double alpha = rz / pq;
        const float af = (float)alpha;
        double rz2 = 0, rr2 = 0;
        for (int i = blockIdx.x; i < nT; i += G) {
            for (int j = threadIdx.x; j < nP; j += blockDim.x) {
                const int c = i * nP + j;
                const float pc = pnew[c];
                if (MIXED) f.x64[c] += alpha * (double)pc;
                else f.dx[c] += af * pc;
                f.r[c] = f.r[c] - af * f.x[c];
            }
            __syncthreads();
            precondition_row<MIXED, PER, false>(g, f, cfg, i, sm, rz2, rr2);
        }
        block_partial3(rz2, rr2, 0.0, partB);
        grid.sync();
        all_sum3(partB, G, rz2, rr2, d1);
        beta = (float)(rz2 / rz);
        rz = rz2;
        rr = rr2;
        float* t = pold;
        pold = pnew;
        pnew = t;
        ++it;
    }
    // final increment and new gamma.  The reported residual is the FP64
    // residual of the refined iterate checked above (mixed mode; it is held
    // to 0.8 tol so that the FP32-rounded gamma also meets tol) or the
    // recursive residual (plain mode).
    for (int i = blockIdx.x; i < nT; i += G)
        for (int j = threadIdx.x; j < nP; j += blockDim.x) {
            const int c = i * nP + j;
            const float dx = MIXED ? (float)f.x64[c] : f.dx[c];
            const float g0 = f.gam_adv[c];
            f.dx[c] = dx;
            f.x[c] = g0 + dx;
        }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        f.stats->solver_iters = it;
        f.stats->solver_rel_resid = sqrt(rr) / bnorm;
        f.stats->solver_b_norm = bnorm;
        f.stats->solver_converged = conv ? 1 : 0;
    }
}

// Sum of the partials of blocks [first, first + nblk), same order in every
// block of that range.
__device__ __forceinline__ void range_sum3(const double* part, int first, int nblk, double& A,
                                           double& B, double& C) {
    __shared__ double res[3];
    if (threadIdx.x < 32) {
        double x = 0.0, y = 0.0, z = 0.0;
        for (int k = threadIdx.x; k < nblk; k += 32) {
            x += part[3 * (first + k) + 0];
            y += part[3 * (first + k) + 1];
            z += part[3 * (first + k) + 2];
        }
        x = warp_sum(x); y = warp_sum(y); z = warp_sum(z);
        if (threadIdx.x == 0) { res[0] = x; res[1] = y; res[2] = z; }
    }
    __syncthreads();
    A = res[0]; B = res[1]; C = res[2];
    __syncthreads();
}

// Batched PCG: k_pcg for every bubble of a batch in one cooperative launch.
// Block k works on bubble blk_bubble[k]; a bubble's blocks are a contiguous
// range and reduce only their own partials, in the same order as k_pcg, so
// a bubble that gets as many blocks as its own k_pcg launch would have
// produces bit-identical results.  The loop runs in slots of two grid
// barriers; in each slot a bubble either does one CG iteration (ITER), or
// the mixed-precision true-residual check followed by the restart (CHECK),
// or nothing (DONE).  These are the branches of k_pcg's loop in the same
// order.  The number of bubbles not yet done is counted on rotating
// counters one barrier ahead of its use, so every block agrees on when to
// stop without an extra barrier.
template <bool MIXED, int PER>
__global__ void __launch_bounds__(kSolveBlock, 4)
k_pcg_batch(SbBatchSolve bs, SolverConfig cfg) {
    enum { ITER = 0, CHECK = 1, DONE = 2 };
    extern __shared__ float sm[];
    cg::grid_group grid = cg::this_grid();
    const int G = gridDim.x;
    const int bub = bs.blk_bubble[blockIdx.x];
    const int first = bs.bub_first_blk[bub], nblk = bs.bub_nblk[bub];
    const int lb = blockIdx.x - first;
    const SbBubbleDesc& d = bs.descs[bub];
    const SbGrid& g = d.g;
    const SbFields& f = d.f;
    const int nP = g.nP, nT = g.nT;
    double* partA = bs.partials;
    double* partB = bs.partials + 3 * G;
    const bool lead = (lb == 0 && threadIdx.x == 0);
    if (blockIdx.x == 0 && threadIdx.x < 3) bs.nactive[threadIdx.x] = 0;

    // dx = 0, r = r0, z = M^-1 r (p_old = 0, beta = 0)
    double rz = 0, rr = 0, bb = 0;
    {
        double a = 0, b2 = 0, c2 = 0;
        for (int i = lb; i < nT; i += nblk) {
            for (int j = threadIdx.x; j < nP; j += blockDim.x) {
                const int c = i * nP + j;
                if (MIXED) f.x64[c] = 0.0;
                else f.dx[c] = 0.0f;
                f.r[c] = f.r0[c];
                f.q[c] = 0.0f;  // p_old
                const double bv = (double)f.rhs[c];
                c2 += bv * bv;
            }
            __syncthreads();
            precondition_row<MIXED, PER, true>(g, f, cfg, i, sm, a, b2);
        }
        block_partial3(a, b2, c2, partA);
    }
    grid.sync();
    range_sum3(partA, first, nblk, rz, rr, bb);
    const double bnorm = bb > 0.0 ? sqrt(bb) : 1.0;
    const double tol2 = (MIXED ? 0.64 : 1.0) * cfg.tol * cfg.tol * bnorm * bnorm;
    float* pold = f.q;
    float* pnew = f.p;
    float beta = 0.0f;
    int it = 0;
    bool conv = false;
    // the loop head of k_pcg: iteration limit, NaN, target reached
    auto next_state = [&]() -> int {
        if (it >= cfg.max_iter || !(rr == rr)) return DONE;
        if (rr <= tol2) {
            if (!MIXED) { conv = true; return DONE; }
            return CHECK;
        }
        return ITER;
    };
    int state = next_state();
    if (state != DONE && lead) atomicAdd(&bs.nactive[0], 1);
    for (int k = 0;; ++k) {
        if (blockIdx.x == 0 && threadIdx.x == 0) bs.nactive[(k + 2) % 3] = 0;
        // first half: q = A p_new (ITER) or the true residual (CHECK)
        double s1 = 0;
        if (state == ITER) {
            for (int i = lb; i < nT; i += nblk)
                for (int j = threadIdx.x; j < nP; j += blockDim.x) {
                    const int c = i * nP + j;
                    const int e = i * nP + ((j + 1) & g.maskP);
                    const int w = i * nP + ((j - 1) & g.maskP);
                    const float pc = f.z[c] + beta * pold[c];
                    pnew[c] = pc;
                    float qf = f.dmass[c] * pc + f.cE[c] * (pc - (f.z[e] + beta * pold[e])) +
                               f.cE[w] * (pc - (f.z[w] + beta * pold[w]));
                    if (i < nT - 1) {
                        const int sc = c + nP;
                        qf += f.cS[c] * (pc - (f.z[sc] + beta * pold[sc]));
                    }
                    if (i > 0) {
                        const int nc = c - nP;
                        qf += f.cS[nc] * (pc - (f.z[nc] + beta * pold[nc]));
                    }
                    f.x[c] = qf;  // q lives in x until the final phase
                    s1 += MIXED ? (double)pc * (double)qf : (double)(pc * qf);
                }
        } else if (MIXED && state == CHECK) {
            for (int i = lb; i < nT; i += nblk)
                for (int j = threadIdx.x; j < nP; j += blockDim.x) {
                    const int c = i * nP + j;
                    const double r = (double)f.r0[c] - apply_A<double, double>(g, f, f.x64, c, i, j);
                    f.r[c] = (float)r;
                    s1 += r * r;
                }
        }
        block_partial3(s1, 0.0, 0.0, partA);
        grid.sync();
        if (bs.nactive[k % 3] == 0) break;  // same value in every block
        double r1, d1, d2;
        range_sum3(partA, first, nblk, r1, d1, d2);
        // second half: update and precondition (ITER) or restart (CHECK)
        double rz2 = 0, rr2 = 0;
        if (state == ITER) {
            if (!(r1 > 0.0)) {
                state = DONE;  // breakdown: keep the current iterate
            } else {
                const double alpha = rz / r1;
                const float af = (float)alpha;
                for (int i = lb; i < nT; i += nblk) {
                    for (int j = threadIdx.x; j < nP; j += blockDim.x) {
                        const int c = i * nP + j;
                        const float pc = pnew[c];
                        if (MIXED) f.x64[c] += alpha * (double)pc;
                        else f.dx[c] += af * pc;
                        f.r[c] = f.r[c] - af * f.x[c];
                    }
                    __syncthreads();
                    precondition_row<MIXED, PER, false>(g, f, cfg, i, sm, rz2, rr2);
                }
            }
        } else if (state == CHECK) {
            rr = r1;
            if (rr <= tol2) {
                conv = true;
                state = DONE;
            } else {
                for (int i = lb; i < nT; i += nblk)
                    precondition_row<MIXED, PER, false>(g, f, cfg, i, sm, rz2, rr2);
            }
        }
        block_partial3(rz2, rr2, 0.0, partB);
        grid.sync();
        double d3;
        range_sum3(partB, first, nblk, rz2, rr2, d3);
        if (state == ITER) {
            beta = (float)(rz2 / rz);
            rz = rz2;
            rr = rr2;
            float* t = pold;
            pold = pnew;
            pnew = t;
            ++it;
            state = next_state();
        } else if (state == CHECK) {
            // restarted from the refined iterate: the next slot iterates
            rz = rz2;
            rr = rr2;
            beta = 0.0f;
            state = ITER;
        }
        if (state != DONE && lead) atomicAdd(&bs.nactive[(k + 1) % 3], 1);
    }
    // final increment and new gamma, as k_pcg
    for (int i = lb; i < nT; i += nblk)
        for (int j = threadIdx.x; j < nP; j += blockDim.x) {
            const int c = i * nP + j;
            const float dx = MIXED ? (float)f.x64[c] : f.dx[c];
            const float g0 = f.gam_adv[c];
            f.dx[c] = dx;
            f.x[c] = g0 + dx;
        }
    if (lead) {
        f.stats->solver_iters = it;
        f.stats->solver_rel_resid = sqrt(rr) / bnorm;
        f.stats->solver_b_norm = bnorm;
        f.stats->solver_converged = conv ? 1 : 0;
    }
}

template <bool MIXED>
const void* pcg_batch_kernel(int per) {
    switch (per) {
        case 1: return (const void*)k_pcg_batch<MIXED, 1>;
        case 2: return (const void*)k_pcg_batch<MIXED, 2>;
        case 4: return (const void*)k_pcg_batch<MIXED, 4>;
        default: return (const void*)k_pcg_batch<MIXED, 8>;
    }
}

template <bool MIXED>
const void* pcg_kernel(int per) {
    switch (per) {
        case 1: return (const void*)k_pcg<MIXED, 1>;
        case 2: return (const void*)k_pcg<MIXED, 2>;
        case 4: return (const void*)k_pcg<MIXED, 4>;
        default: return (const void*)k_pcg<MIXED, 8>;
    }
}

int per_of(int nP) {
    int per = (nP + kSolveBlock - 1) / kSolveBlock;
    return per <= 1 ? 1 : per <= 2 ? 2 : per <= 4 ? 4 : 8;
}

struct Occ {
    int sms = 0;
    int blocks = 0;
    int nP = -1;
};

int solve_blocks(const SbGrid& g) {
    static Occ cache[16];
    int dev = 0;
    cudaGetDevice(&dev);
    Occ& o = cache[dev & 15];
    if (o.nP != g.nP) {
        cudaDeviceGetAttribute(&o.sms, cudaDevAttrMultiProcessorCount, dev);
        const size_t smem = 4 * sizeof(float) * (size_t)g.nP;
        const int per = per_of(g.nP);
        int a = 0, b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, pcg_kernel<false>(per), kSolveBlock, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pcg_kernel<true>(per), kSolveBlock, smem);
        o.blocks = o.sms * (a < b ? a : b);
        o.nP = g.nP;
    }
    const int b = o.blocks > 0 ? o.blocks : 1;
    return g.nT < b ? g.nT : b;
}

}  // namespace

int solver_partials_needed(const SbGrid& g) { return 6 * solve_blocks(g); }

cudaError_t prepare_solve_batch(int maxNP, const SolverConfig& cfg, int* blocks) {
    if (maxNP > 8 * kSolveBlock) return cudaErrorInvalidValue;
    const size_t smem = 4 * sizeof(float) * (size_t)maxNP;
    const int per = per_of(maxNP);
    const void* fn = cfg.mode == 1 ? pcg_batch_kernel<true>(per) : pcg_batch_kernel<false>(per);
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kSolveBlock, smem);
    *blocks = sms * (occ > 0 ? occ : 1);
    return e;
}

cudaError_t launch_solve_batch(const SbBatchSolve& bs, int G, int maxNP, const SolverConfig& cfg,
                               cudaStream_t s) {
    const size_t smem = 4 * sizeof(float) * (size_t)maxNP;
    SbBatchSolve bb = bs;
    SolverConfig cc = cfg;
    void* args[] = {&bb, &cc};
    const int per = per_of(maxNP);
    const void* fn = cfg.mode == 1 ? pcg_batch_kernel<true>(per) : pcg_batch_kernel<false>(per);
    return cudaLaunchCooperativeKernel(fn, dim3(G), dim3(kSolveBlock), args, smem, s);
}

cudaError_t prepare_solve(const SbGrid& g, const SolverConfig& cfg) {
    if (g.nP > 8 * kSolveBlock) return cudaErrorInvalidValue;
    solve_blocks(g);
    const size_t smem = 4 * sizeof(float) * (size_t)g.nP;
    const int per = per_of(g.nP);
    const void* fn = cfg.mode == 1 ? pcg_kernel<true>(per) : pcg_kernel<false>(per);
    if (smem > 48 * 1024)
        return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaSuccess;
}

cudaError_t launch_solve(const SbGrid& g, const SbPhys& ph, const SbFields& f,
                         const SolverConfig& cfg, cudaStream_t s) {
    (void)ph;
    if (g.nP > 8 * kSolveBlock) return cudaErrorInvalidValue;
    const int G = solve_blocks(g);
    const size_t smem = 4 * sizeof(float) * (size_t)g.nP;
    SbGrid gg = g;
    SbFields ff = f;
    SolverConfig cc = cfg;
    void* args[] = {&gg, &ff, &cc};
    const int per = per_of(g.nP);
    const void* fn = cfg.mode == 1 ? pcg_kernel<true>(per) : pcg_kernel<false>(per);
    return cudaLaunchCooperativeKernel(fn, dim3(G), dim3(kSolveBlock), args, smem, s);
}

}  // namespace sb
