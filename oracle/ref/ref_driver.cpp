// Driver of the reference's own step code on the host (test
// infrastructure).  This translation unit includes the reference's
// kernel/bubble.cu (rewritten only in its launch syntax by build_ref.py) so
// that it can set the file-static __constant__ parameters exactly as
// Bubble::run does (kernel/bubble.cu:2607-2656), and exposes a C API that
// creates the reference's Solver, initialises it through its own
// initialisers, steps it with Solver::stepForward, and reads or writes any
// of its buffers.  Nothing here computes physics: every number comes from
// the reference's code.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "shim/cuda_runtime.h"
#include "shim/opencv2/opencv.hpp"

// private members of Bubble / Solver / Quantity are read by the driver
#define private public
#define protected public
#include SBREF_BUBBLE_CU
#undef private
#undef protected

// ---------------------------------------------------------------------------
// cv::imread / cv::resize of the shim: images registered by the driver.
namespace {
std::map<std::string, cv::Mat> g_images;
}

namespace cv {
Mat imread(const std::string& path, int) {
    auto it = g_images.find(path);
    if (it == g_images.end()) return Mat();
    Mat m = it->second;
    m.attach();
    return m;
}
void resize(const Mat& in, Mat& out, Size size) {
    if (in.cols != size.width || in.rows != size.height) {
        std::cerr << "host execution: images must be registered at the grid's size\n";
        abort();
    }
    out = in;
    out.attach();
}
}  // namespace cv

namespace {

struct RefSim {
    Bubble* bubble = nullptr;
    Solver* solver = nullptr;
};

std::ostringstream g_quiet;  // the reference's progress output goes here

struct Quiet {
    std::streambuf *old, *old_err;
    Quiet() : old(std::cout.rdbuf(g_quiet.rdbuf())), old_err(std::cerr.rdbuf(g_quiet.rdbuf())) {}
    ~Quiet() {
        std::cout.rdbuf(old);
        std::cerr.rdbuf(old_err);
        g_quiet.str("");
    }
};

// the reference's constant uploads of Bubble::run (kernel/bubble.cu:2611-2638)
void upload_constants(Bubble& B) {
    checkCudaErrors(cudaMemcpyToSymbol(nPhiGlobal, &(B.nPhi), sizeof(size_t)));
    checkCudaErrors(cudaMemcpyToSymbol(nThetaGlobal, &(B.nTheta), sizeof(size_t)));
    checkCudaErrors(cudaMemcpyToSymbol(radiusGlobal, &(B.radius), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(invRadiusGlobal, &(B.invRadius), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(timeStepGlobal, &(B.dt), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(gridLenGlobal, &(B.gridLen), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(invGridLenGlobal, &(B.invGridLen), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(SGlobal, &(B.S), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(MGlobal, &(B.M), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(reGlobal, &(B.re), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(gGlobal, &(B.gs), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(DsGlobal, &(B.Ds), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(CrGlobal, &(B.Cr), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(UGlobal, &(B.U), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(blend_coeff, &(B.blendCoeff), sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(gammaMaxGlobal, &(B.gammaMax), sizeof(fReal)));
    fReal eva = evaporation * B.radius / (B.H * B.U);
    checkCudaErrors(cudaMemcpyToSymbol(evaporationRate, &eva, sizeof(fReal)));
    fReal epsilon_ = .0;
    fReal W2_ = B.radius / (B.U * B.U) * pow(B.rm / B.H, 2) * epsilon_;
    fReal W1_ = 0.5 * W2_ * pow(B.rm / B.H, 2);
    checkCudaErrors(cudaMemcpyToSymbol(W1, &W1_, sizeof(fReal)));
    checkCudaErrors(cudaMemcpyToSymbol(W2, &W2_, sizeof(fReal)));
}

cv::Mat image_of(int rows, int cols, const float* bgr) {
    cv::Mat m;
    m.rows = rows;
    m.cols = cols;
    m.pix.assign(bgr, bgr + (size_t)rows * cols * 3);
    return m;
}

// A buffer of the solver by name, with its row count and row pitch
// (elements); the pitched quantities report their pitch.
struct Buf {
    fReal* p = nullptr;
    size_t rows = 0, cols = 0, pitch = 0;
};

Buf buffer_of(Solver& S, const std::string& n) {
    const size_t nT = S.nTheta, nP = S.nPhi, pitch = S.pitch;
    auto q = [&](BimocqQuantity* Q, fReal* p) {
        return Buf{p, Q->getNTheta(), nP, Q->getThisStepPitchInElements()};
    };
    if (n == "eta") return q(S.thickness, S.thickness->getGPUThisStep());
    if (n == "gamma") return q(S.concentration, S.concentration->getGPUThisStep());
    if (n == "u_theta") return q(S.velTheta, S.velTheta->getGPUThisStep());
    if (n == "u_phi") return q(S.velPhi, S.velPhi->getGPUThisStep());
    if (n == "eta_init") return q(S.thickness, S.thickness->getGPUInit());
    if (n == "eta_delta") return q(S.thickness, S.thickness->getGPUDelta());
    if (n == "eta_init_last") return q(S.thickness, S.thickness->getGPUInitLast());
    if (n == "eta_delta_last") return q(S.thickness, S.thickness->getGPUDeltaLast());
    if (n == "gamma_init") return q(S.concentration, S.concentration->getGPUInit());
    if (n == "gamma_delta") return q(S.concentration, S.concentration->getGPUDelta());
    if (n == "gamma_init_last") return q(S.concentration, S.concentration->getGPUInitLast());
    if (n == "gamma_delta_last") return q(S.concentration, S.concentration->getGPUDeltaLast());
    if (n == "fwd_t") return Buf{S.forward_t, nT, nP, nP};
    if (n == "fwd_p") return Buf{S.forward_p, nT, nP, nP};
    if (n == "bwd_t") return Buf{S.backward_t, nT, nP, nP};
    if (n == "bwd_p") return Buf{S.backward_p, nT, nP, nP};
    if (n == "bwdprev_t") return Buf{S.backward_tprev, nT, nP, nP};
    if (n == "bwdprev_p") return Buf{S.backward_pprev, nT, nP, nP};
    if (n == "uair_init") return Buf{S.uair_init, nT, nP, nP};
    if (n == "vair_init") return Buf{S.vair_init, nT - 1, nP, nP};
    if (n == "uair") return Buf{S.uair, nT, nP, nP};
    if (n == "vair") return Buf{S.vair, nT - 1, nP, nP};
    if (n == "rhs") return Buf{S.rhs, nT, nP, nP};
    // the other buffer of each pair: after a step, the advected state the
    // body forces started from
    if (n == "eta_next") return q(S.thickness, S.thickness->getGPUNextStep());
    if (n == "gamma_next") return q(S.concentration, S.concentration->getGPUNextStep());
    if (n == "u_theta_next") return q(S.velTheta, S.velTheta->getGPUNextStep());
    if (n == "u_phi_next") return q(S.velPhi, S.velPhi->getGPUNextStep());
    if (n == "div") return Buf{S.div, nT, nP, nP};
    if (n == "fu") return Buf{S.fu, nT, nP, nP};
    if (n == "fv") return Buf{S.fv, nT - 1, nP, nP};
    if (n == "val") return Buf{S.val, nT * nP, 5, 5};
    (void)pitch;
    return Buf{};
}

}  // namespace

extern "C" {

// Bubble(radius, H, U, c_m, Gamma_m, T, Ds, rm, nTheta, dt, DT, frames,
// outputDir, thicknessImage, device, AMGconfig, blendCoeff) and the Solver
// that Bubble::run makes, with its constants uploaded.
void* sbref_create(double radius, double H, double U, double c_m, double Gamma_m, double T,
                   double Ds, double rm, int nTheta, double dt, double DT, int frames,
                   double blendCoeff) {
    Quiet q;
    RefSim* s = new RefSim();
    s->bubble = new Bubble(radius, H, U, c_m, Gamma_m, T, Ds, rm, (size_t)nTheta, dt, DT, frames,
                           "host-execution", "thickness", 0, "", blendCoeff);
    Bubble& B = *s->bubble;
    s->solver = new Solver(B.nPhi, B.nTheta, B.radius, B.dt * B.radius / B.U, B.H, B.device,
                           B.AMGconfig);
    upload_constants(B);
    return s;
}

void sbref_destroy(void* h) {
    RefSim* s = (RefSim*)h;
    if (!s) return;
    Quiet q;
    delete s->solver;
    delete s->bubble;
    delete s;
}

// The reference's initialisers (kernel/initializer.cu:50-135) on images of
// nTheta rows x nPhi columns x (B, G, R) floats (NULL: the initialiser's
// no-image path).
void sbref_init_from_images(void* h, const float* thickness_bgr, const float* airflow_bgr) {
    RefSim* s = (RefSim*)h;
    Quiet q;
    const int rows = (int)s->solver->nTheta, cols = (int)s->solver->nPhi;
    g_images.clear();
    if (thickness_bgr) g_images["thickness"] = image_of(rows, cols, thickness_bgr);
    if (airflow_bgr) g_images["airflow"] = image_of(rows, cols, airflow_bgr);
    s->solver->initThicknessfromPic(thickness_bgr ? "thickness" : "");
    s->solver->initAirflowfromPic(airflow_bgr ? "airflow" : "");
}

// One Solver::stepForward at frame time t (s): currentTimeGlobal = t as the
// frame loop sets it (kernel/bubble.cu:2662-2678); a step of dt_s other than
// the configured one is the frame's fractional last step.  Returns 1 when the
// solver flagged the film as broken.
int sbref_step(void* h, double t, double dt_s) {
    RefSim* s = (RefSim*)h;
    Bubble& B = *s->bubble;
    Quiet q;
    fReal T = t;
    checkCudaErrors(cudaMemcpyToSymbol(currentTimeGlobal, &T, sizeof(fReal)));
    const fReal full = B.dt * B.radius / B.U;
    if (dt_s == full) {
        checkCudaErrors(cudaMemcpyToSymbol(timeStepGlobal, &(B.dt), sizeof(fReal)));
        s->solver->stepForward();
    } else {
        fReal tmp_dt = dt_s * B.U / B.radius;
        checkCudaErrors(cudaMemcpyToSymbol(timeStepGlobal, &tmp_dt, sizeof(fReal)));
        s->solver->stepForward(dt_s);
    }
    return s->solver->isBroken() ? 1 : 0;
}

// Copies a buffer (row-major, its rows x nPhi, unpitched) out or in;
// returns the element count, 0 for an unknown name.  "val" is the CSR
// values (5 per row).
long long sbref_get(void* h, const char* name, double* out) {
    const Buf b = buffer_of(*((RefSim*)h)->solver, name);
    if (!b.p) return 0;
    if (out)
        for (size_t r = 0; r < b.rows; ++r)
            std::memcpy(out + r * b.cols, b.p + r * b.pitch, b.cols * sizeof(double));
    return (long long)(b.rows * b.cols);
}

long long sbref_set(void* h, const char* name, const double* in) {
    const Buf b = buffer_of(*((RefSim*)h)->solver, name);
    if (!b.p) return 0;
    for (size_t r = 0; r < b.rows; ++r)
        std::memcpy(b.p + r * b.pitch, in + r * b.cols, b.cols * sizeof(double));
    return (long long)(b.rows * b.cols);
}

// Nondimensional coefficients as Bubble::Bubble derived them: dt, M, Cr, gs,
// gammaMax, evaporation rate, blend (kernel/bubble.cu:2568-2581).
void sbref_coefficients(void* h, double* out7) {
    Bubble& B = *((RefSim*)h)->bubble;
    out7[0] = B.dt;
    out7[1] = B.M;
    out7[2] = B.Cr;
    out7[3] = B.gs;
    out7[4] = B.gammaMax;
    out7[5] = evaporation * B.radius / (B.H * B.U);
    out7[6] = B.blendCoeff;
}

int sbref_broken(void* h) { return ((RefSim*)h)->solver->isBroken() ? 1 : 0; }

}  // extern "C"
