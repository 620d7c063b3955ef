// Stand-in for the AmgX calls of the reference (test infrastructure).
//
// The reference uploads its CSR system (5 entries per row, built by
// initLinearSystem and concentrationLinearSystemKernel) and the current
// gamma as the initial guess, and lets AmgX's PCGF + AMG (init/PCGF_F.json)
// solve it to an absolute residual of 1e-7 (kernel/bubble.cu:1479-1508).
// AmgX is not available, so the same system is solved here on the host with
// restarted GMRES, right-preconditioned by the exact solve of each theta
// row's periodic tridiagonal part (the phi couplings, which dominate next
// to the poles), to a relative residual of 1e-13: the solution the matrix
// defines, more tightly than AmgX's tolerance.  A solve that does not get
// there reports AMGX_SOLVE_FAILED, which makes the reference flag the film
// as broken, as it does on an AmgX failure.
#include <cmath>
#include <cstring>
#include <vector>

#include "shim/amgx_c.h"

struct sbref_amgx_config { int unused; };
struct sbref_amgx_resources { int unused; };
struct sbref_amgx_matrix {
    int n = 0;
    std::vector<int> rp, ci;
    std::vector<double> v;
};
struct sbref_amgx_vector {
    std::vector<double> d;
};
struct sbref_amgx_solver {
    const sbref_amgx_matrix* A = nullptr;
    AMGX_SOLVE_STATUS status = AMGX_SOLVE_SUCCESS;
    int iters = 0;
};

namespace {

double sbref_last_rel_resid = 0.0;
int sbref_last_iters = 0;

void spmv(const sbref_amgx_matrix& A, const double* x, double* y) {
#pragma omp parallel for
    for (int i = 0; i < A.n; ++i) {
        double s = 0.0;
        for (int k = A.rp[i]; k < A.rp[i + 1]; ++k) s += A.v[k] * x[A.ci[k]];
        y[i] = s;
    }
}

// Exact solve of each theta row's periodic tridiagonal block (entries whose
// column is the west or east neighbour in the same row; every other entry,
// including the same-row pole couplings of the first and last rows, is left
// to GMRES).  Thomas algorithm with the Sherman-Morrison correction for the
// periodic corners.
struct LinePrecond {
    int nT = 0, nP = 0;
    std::vector<double> lo, di, up;  // per cell: coupling to west, diagonal, to east

    void build(const sbref_amgx_matrix& A) {
        nP = (int)std::lround(std::sqrt(2.0 * A.n));  // N = nT nP with nP = 2 nT
        nT = A.n / nP;
        lo.assign(A.n, 0.0);
        di.assign(A.n, 0.0);
        up.assign(A.n, 0.0);
        for (int i = 0; i < A.n; ++i) {
            const int row = i / nP, j = i % nP;
            const int w = row * nP + (j + nP - 1) % nP, e = row * nP + (j + 1) % nP;
            for (int k = A.rp[i]; k < A.rp[i + 1]; ++k) {
                const int c = A.ci[k];
                if (c == i) di[i] += A.v[k];
                else if (c == w) lo[i] += A.v[k];
                else if (c == e) up[i] += A.v[k];
            }
        }
    }

    // y = M^-1 x
    void apply(const double* x, double* y) const {
#pragma omp parallel for
        for (int r = 0; r < nT; ++r) {
            const int o = r * nP, n = nP;
            std::vector<double> a(n), b(n), c(n), d(n), u(n), z(n), cp(n);
            for (int j = 0; j < n; ++j) {
                a[j] = lo[o + j];
                b[j] = di[o + j];
                c[j] = up[o + j];
                d[j] = x[o + j];
            }
            // periodic: corner entries a[0] (to n-1) and c[n-1] (to 0)
            const double gamma = -b[0];
            std::vector<double> bb(b);
            bb[0] -= gamma;
            bb[n - 1] -= a[0] * c[n - 1] / gamma;
            for (int j = 0; j < n; ++j) u[j] = 0.0;
            u[0] = gamma;
            u[n - 1] = c[n - 1];
            auto thomas = [&](const std::vector<double>& rhs, std::vector<double>& out) {
                std::vector<double> dp(n);
                cp[0] = c[0] / bb[0];
                dp[0] = rhs[0] / bb[0];
                for (int j = 1; j < n; ++j) {
                    const double m = bb[j] - a[j] * cp[j - 1];
                    cp[j] = j < n - 1 ? c[j] / m : 0.0;
                    dp[j] = (rhs[j] - a[j] * dp[j - 1]) / m;
                }
                out[n - 1] = dp[n - 1];
                for (int j = n - 2; j >= 0; --j) out[j] = dp[j] - cp[j] * out[j + 1];
            };
            std::vector<double> yv(n), q(n);
            thomas(d, yv);
            thomas(u, q);
            const double vy = yv[0] + a[0] / gamma * yv[n - 1];
            const double vq = q[0] + a[0] / gamma * q[n - 1];
            const double f = vy / (1.0 + vq);
            for (int j = 0; j < n; ++j) y[o + j] = yv[j] - f * q[j];
        }
    }
};

double norm2(const std::vector<double>& v) {
    double s = 0.0;
    for (double x : v) s += x * x;
    return std::sqrt(s);
}

// Right-preconditioned restarted GMRES(m) from the initial guess in x.
bool gmres(const sbref_amgx_matrix& A, const std::vector<double>& b, std::vector<double>& x,
           double tol, int* iters_out, double* rel_out) {
    const int n = A.n, m = 60, max_restarts = 400;
    LinePrecond M;
    M.build(A);
    const double bn = norm2(b) > 0 ? norm2(b) : 1.0;
    std::vector<double> r(n), w(n), z(n);
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
    std::vector<std::vector<double>> H(m + 1, std::vector<double>(m, 0.0));
    std::vector<double> cs(m), sn(m), g(m + 1);
    int iters = 0;
    double rel = 0.0;
    for (int rs = 0; rs < max_restarts; ++rs) {
        spmv(A, x.data(), r.data());
        for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
        double beta = norm2(r);
        rel = beta / bn;
        if (rel <= tol) break;
        for (int i = 0; i < n; ++i) V[0][i] = r[i] / beta;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        for (; k < m; ++k) {
            M.apply(V[k].data(), z.data());
            spmv(A, z.data(), w.data());
            for (int j = 0; j <= k; ++j) {  // modified Gram-Schmidt
                double h = 0.0;
                for (int i = 0; i < n; ++i) h += w[i] * V[j][i];
                H[j][k] = h;
                for (int i = 0; i < n; ++i) w[i] -= h * V[j][i];
            }
            const double hn = norm2(w);
            H[k + 1][k] = hn;
            if (hn > 0) for (int i = 0; i < n; ++i) V[k + 1][i] = w[i] / hn;
            for (int j = 0; j < k; ++j) {  // earlier rotations
                const double t = cs[j] * H[j][k] + sn[j] * H[j + 1][k];
                H[j + 1][k] = -sn[j] * H[j][k] + cs[j] * H[j + 1][k];
                H[j][k] = t;
            }
            const double den = std::hypot(H[k][k], H[k + 1][k]);
            cs[k] = den > 0 ? H[k][k] / den : 1.0;
            sn[k] = den > 0 ? H[k + 1][k] / den : 0.0;
            H[k][k] = den;
            H[k + 1][k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            ++iters;
            if (std::fabs(g[k + 1]) / bn <= 0.1 * tol || hn == 0.0) {
                ++k;
                break;
            }
        }
        // y = H^-1 g, x += M^-1 V y
        std::vector<double> y(k, 0.0);
        for (int j = k - 1; j >= 0; --j) {
            double s = g[j];
            for (int l = j + 1; l < k; ++l) s -= H[j][l] * y[l];
            y[j] = s / H[j][j];
        }
        std::fill(w.begin(), w.end(), 0.0);
        for (int j = 0; j < k; ++j)
            for (int i = 0; i < n; ++i) w[i] += y[j] * V[j][i];
        M.apply(w.data(), z.data());
        for (int i = 0; i < n; ++i) x[i] += z[i];
    }
    spmv(A, x.data(), r.data());
    for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
    rel = norm2(r) / bn;
    *iters_out = iters;
    *rel_out = rel;
    return rel <= tol * 10;
}

}  // namespace

extern "C" double sbref_amgx_last_rel_resid() { return sbref_last_rel_resid; }
extern "C" int sbref_amgx_last_iters() { return sbref_last_iters; }

AMGX_RC AMGX_initialize() { return AMGX_RC_OK; }
AMGX_RC AMGX_initialize_plugins() { return AMGX_RC_OK; }
AMGX_RC AMGX_finalize() { return AMGX_RC_OK; }
AMGX_RC AMGX_finalize_plugins() { return AMGX_RC_OK; }
AMGX_RC AMGX_config_create_from_file(AMGX_config_handle* cfg, const char*) {
    *cfg = new sbref_amgx_config();
    return AMGX_RC_OK;
}
AMGX_RC AMGX_config_destroy(AMGX_config_handle cfg) {
    delete cfg;
    return AMGX_RC_OK;
}
AMGX_RC AMGX_resources_create(AMGX_resources_handle* r, AMGX_config_handle, void*, int, const int*) {
    *r = new sbref_amgx_resources();
    return AMGX_RC_OK;
}
AMGX_RC AMGX_resources_destroy(AMGX_resources_handle r) {
    delete r;
    return AMGX_RC_OK;
}
AMGX_RC AMGX_matrix_create(AMGX_matrix_handle* m, AMGX_resources_handle, AMGX_Mode) {
    *m = new sbref_amgx_matrix();
    return AMGX_RC_OK;
}
AMGX_RC AMGX_matrix_destroy(AMGX_matrix_handle m) {
    delete m;
    return AMGX_RC_OK;
}
AMGX_RC AMGX_vector_create(AMGX_vector_handle* v, AMGX_resources_handle, AMGX_Mode) {
    *v = new sbref_amgx_vector();
    return AMGX_RC_OK;
}
AMGX_RC AMGX_vector_destroy(AMGX_vector_handle v) {
    delete v;
    return AMGX_RC_OK;
}
AMGX_RC AMGX_solver_create(AMGX_solver_handle* s, AMGX_resources_handle, AMGX_Mode, AMGX_config_handle) {
    *s = new sbref_amgx_solver();
    return AMGX_RC_OK;
}
AMGX_RC AMGX_solver_destroy(AMGX_solver_handle s) {
    delete s;
    return AMGX_RC_OK;
}
AMGX_RC AMGX_vector_upload(AMGX_vector_handle v, int n, int, const void* data) {
    v->d.assign((const double*)data, (const double*)data + n);
    return AMGX_RC_OK;
}
AMGX_RC AMGX_vector_download(AMGX_vector_handle v, void* data) {
    std::memcpy(data, v->d.data(), v->d.size() * sizeof(double));
    return AMGX_RC_OK;
}
AMGX_RC AMGX_matrix_upload_all(AMGX_matrix_handle m, int n, int nnz, int, int, const int* rp,
                               const int* ci, const void* data, const void*) {
    m->n = n;
    m->rp.assign(rp, rp + n + 1);
    m->ci.assign(ci, ci + nnz);
    m->v.assign((const double*)data, (const double*)data + nnz);
    return AMGX_RC_OK;
}
AMGX_RC AMGX_solver_setup(AMGX_solver_handle s, AMGX_matrix_handle m) {
    s->A = m;
    return AMGX_RC_OK;
}
AMGX_RC AMGX_solver_solve(AMGX_solver_handle s, AMGX_vector_handle b, AMGX_vector_handle x) {
    int it = 0;
    double rel = 0.0;
    const bool ok = gmres(*s->A, b->d, x->d, 1e-13, &it, &rel);
    s->status = ok ? AMGX_SOLVE_SUCCESS : AMGX_SOLVE_FAILED;
    s->iters = it;
    sbref_last_rel_resid = rel;
    sbref_last_iters = it;
    return AMGX_RC_OK;
}
AMGX_RC AMGX_solver_get_status(AMGX_solver_handle s, AMGX_SOLVE_STATUS* st) {
    *st = s->status;
    return AMGX_RC_OK;
}
AMGX_RC AMGX_solver_get_iterations_number(AMGX_solver_handle s, int* n) {
    *n = s->iters;
    return AMGX_RC_OK;
}
