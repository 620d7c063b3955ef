// Implicit surfactant solve: preconditioned conjugate gradients on the
// symmetric 5-point system assembled by k_assemble.  It replaces the
// reference's AmgX PCGF + AMG solve (kernel/bubble.cu:1479-1508,
// init/PCGF_F.json); x0 is the current gamma, as in the reference.
//
// One cooperative launch runs the whole solve: every thread owns a strided
// set of cells, phases are separated by grid-wide barriers, and the dot
// products are reduced per block and then summed by every block in the same
// block order, so all blocks see bit-identical scalars and take identical
// loop decisions (the iteration count is bounded by max_iter).
//
// Modes: plain FP32 (FP32 vectors and per-thread sums), or mixed precision
// (FP32 SpMV and preconditioner, FP64 iterate and dot products, and a true
// FP64 residual check that restarts CG from the refined iterate until the
// relative residual target holds).
#include <cooperative_groups.h>

#include "sb_internal.h"

namespace cg = cooperative_groups;

namespace sb {

namespace {

constexpr int kSolveBlock = 256;

struct SolveCtx {
    int G;  // blocks
};

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

template <typename T>
__device__ __forceinline__ double spmv_at(const SbGrid& g, const SbFields& f, const T* __restrict__ v,
                                          int c) {
    const int i = c >> g.logP, j = c & g.maskP;
    const int nP = g.nP;
    const int e = i * nP + ((j + 1) & g.maskP);
    const int w = i * nP + ((j - 1) & g.maskP);
    double s = (double)f.diag[c] * (double)v[c] + (double)f.cE[c] * (double)v[e] +
               (double)f.cE[w] * (double)v[w];
    if (i < g.nT - 1) s += (double)f.cS[c] * (double)v[c + nP];
    if (i > 0) s += (double)f.cS[c - nP] * (double)v[c - nP];
    return s;
}

__device__ __forceinline__ float spmv_f(const SbGrid& g, const SbFields& f, const float* __restrict__ v,
                                        int c) {
    const int i = c >> g.logP, j = c & g.maskP;
    const int nP = g.nP;
    const int e = i * nP + ((j + 1) & g.maskP);
    const int w = i * nP + ((j - 1) & g.maskP);
    float s = f.diag[c] * v[c] + f.cE[c] * v[e] + f.cE[w] * v[w];
    if (i < g.nT - 1) s += f.cS[c] * v[c + nP];
    if (i > 0) s += f.cS[c - nP] * v[c - nP];
    return s;
}

template <bool MIXED>
__global__ void __launch_bounds__(kSolveBlock)
k_pcg(SbGrid g, SbFields f, SolverConfig cfg) {
    cg::grid_group grid = cg::this_grid();
    const int G = gridDim.x;
    const int stride = G * kSolveBlock;
    const int t0 = blockIdx.x * kSolveBlock + threadIdx.x;
    double* partA = f.partials;
    double* partB = f.partials + 3 * G;
    const int N = g.N;

    // r = b - A x0, z = M^-1 r, p = z
    double rz = 0, rr = 0, bb = 0;
    {
        double a = 0, b2 = 0, c2 = 0;
        for (int c = t0; c < N; c += stride) {
            const float x0 = f.gam_adv[c];
            if (MIXED) f.x64[c] = (double)x0;
            f.x[c] = x0;
            const double b = (double)f.rhs[c];
            const double r = b - spmv_at(g, f, f.gam_adv, c);
            const float rf = (float)r;
            const float zf = rf / f.diag[c];
            f.r[c] = rf;
            f.z[c] = zf;
            f.p[c] = zf;
            a += (double)rf * (double)zf;
            b2 += r * r;
            c2 += b * b;
        }
        block_partial3(a, b2, c2, partA);
    }
    grid.sync();
    all_sum3(partA, G, rz, rr, bb);
    const double bnorm = bb > 0.0 ? sqrt(bb) : 1.0;
    const double tol2 = cfg.tol * cfg.tol * bnorm * bnorm;
    int it = 0;
    bool conv = false;
    while (it < cfg.max_iter) {
        if (!(rr == rr)) break;  // NaN: give up (same decision in every block)
        if (rr <= tol2) {
            if (!MIXED) { conv = true; break; }
            // true FP64 residual of the refined iterate; restart CG from it
            double a = 0, b2 = 0;
            for (int c = t0; c < N; c += stride) {
                const double r = (double)f.rhs[c] - spmv_at(g, f, f.x64, c);
                const float rf = (float)r;
                const float zf = rf / f.diag[c];
                f.r[c] = rf;
                f.z[c] = zf;
                f.p[c] = zf;
                a += (double)rf * (double)zf;
                b2 += r * r;
            }
            block_partial3(a, b2, 0.0, partB);
            grid.sync();
            double dummy;
            all_sum3(partB, G, rz, rr, dummy);
            if (rr <= tol2) { conv = true; break; }
        }
        // q = A p, <p, q>
        {
            double pq = 0;
            for (int c = t0; c < N; c += stride) {
                const float qf = spmv_f(g, f, f.p, c);
                f.q[c] = qf;
                pq += MIXED ? (double)f.p[c] * (double)qf : (double)(f.p[c] * qf);
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
        for (int c = t0; c < N; c += stride) {
            const float pc = f.p[c];
            if (MIXED) f.x64[c] += alpha * (double)pc;
            else f.x[c] += af * pc;
            const float rf = f.r[c] - af * f.q[c];
            const float zf = rf / f.diag[c];
            f.r[c] = rf;
            f.z[c] = zf;
            rz2 += MIXED ? (double)rf * (double)zf : (double)(rf * zf);
            rr2 += MIXED ? (double)rf * (double)rf : (double)(rf * rf);
        }
        block_partial3(rz2, rr2, 0.0, partB);
        grid.sync();
        double dummy;
        all_sum3(partB, G, rz2, rr2, dummy);
        const float bf = (float)(rz2 / rz);
        rz = rz2;
        rr = rr2;
        for (int c = t0; c < N; c += stride) f.p[c] = f.z[c] + bf * f.p[c];
        grid.sync();
        ++it;
    }
    // final iterate and its true relative residual
    if (MIXED)
        for (int c = t0; c < N; c += stride) f.x[c] = (float)f.x64[c];
    grid.sync();
    {
        double a = 0;
        for (int c = t0; c < N; c += stride) {
            const double r = (double)f.rhs[c] - spmv_at(g, f, f.x, c);
            a += r * r;
        }
        block_partial3(a, 0.0, 0.0, partA);
    }
    grid.sync();
    double res2, d1, d2;
    all_sum3(partA, G, res2, d1, d2);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        f.stats->solver_iters = it;
        f.stats->solver_rel_resid = sqrt(res2) / bnorm;
        f.stats->solver_b_norm = bnorm;
        f.stats->solver_converged = conv ? 1 : 0;
    }
}

int g_blocks_cache_n = -1;
int g_blocks_cache_val = 0;

int solve_blocks(const SbGrid& g) {
    static int sms = 0, occ[2] = {0, 0};
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[0], k_pcg<false>, kSolveBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[1], k_pcg<true>, kSolveBlock, 0);
    }
    const int per = occ[0] < occ[1] ? occ[0] : occ[1];
    int maxb = sms * (per > 0 ? per : 1);
    int need = (g.N + kSolveBlock - 1) / kSolveBlock;
    return need < maxb ? need : maxb;
}

}  // namespace

int solver_partials_needed(const SbGrid& g) { return 6 * solve_blocks(g); }

cudaError_t launch_solve(const SbGrid& g, const SbPhys& ph, const SbFields& f,
                         const SolverConfig& cfg, cudaStream_t s) {
    (void)ph;
    const int G = solve_blocks(g);
    SbGrid gg = g;
    SbFields ff = f;
    SolverConfig cc = cfg;
    void* args[] = {&gg, &ff, &cc};
    if (cfg.mode == 1)
        return cudaLaunchCooperativeKernel((const void*)k_pcg<true>, dim3(G), dim3(kSolveBlock),
                                           args, 0, s);
    return cudaLaunchCooperativeKernel((const void*)k_pcg<false>, dim3(G), dim3(kSolveBlock), args,
                                       0, s);
}

}  // namespace sb
