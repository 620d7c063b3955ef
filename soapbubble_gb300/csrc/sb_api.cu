// C ABI of the GB300 soap-bubble step: bubble lifetime, device memory,
// host<->device field conversion, step orchestration, frame output.
//
// Device memory of one bubble is a single arena (cudaMalloc once, carved
// into 256-byte aligned arrays), so admission control can budget a bubble
// exactly (sb_bytes_required) and creation is one allocation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/soapbubble.h"
#include "sb_exr.h"
#include "sb_internal.h"

using namespace sb;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA;
}

#define SB_CHECK(call)                                      \
    do {                                                    \
        cudaError_t _e = (call);                            \
        if (_e != cudaSuccess) return cuda_fail(_e, #call); \
    } while (0)

constexpr double kPi = 3.14159265358979323846;
constexpr double kHalfPi = 1.57079632679489661923;
// include/header.cuh:76-83, 93
constexpr double kGasR = 8.3144598, kSigmaA = 0.07275, kRho = 1e3, kG = 9.8;
constexpr double kRhoA = 1.184, kNuA = 1.562e-5, kEvaporation = -0.00000003;
constexpr double kNu = 1.25e-4;  // soap solution kinematic viscosity (VISCOUS variant)

struct Layout {
    size_t bytes = 0;
    size_t take(size_t n) {
        size_t off = bytes;
        bytes += (n + 255) & ~size_t(255);
        return off;
    }
};

bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

}  // namespace

namespace sb {
// Records an error for sb_last_error() from other translation units.
int api_fail(int code, const char* msg) { return fail(code, msg); }
}  // namespace sb

struct sb_bubble {
    sb_params params;
    SbGrid g;
    SbPhys ph;
    SbFields f;
    SolverConfig solver;
    int force_reinit;  // -1 decide, 0 never, 1 always
    int storage;       // kStoreF32 / kStoreBF16 (thickness and surfactant fields)
    int device;
    cudaStream_t stream = nullptr;
    char* arena = nullptr;
    size_t arena_bytes = 0;
    float* tables = nullptr;
    int cur = 0;  // map ping-pong
    long long steps = 0;
    double last_dt = -1, last_t = -1e300;
    SbStepParams* h_step = nullptr;  // pinned
    long long launches = 0;          // kernels launched by this handle
    cudaEvent_t ev[STAGE_COUNT + 1] = {};
    SbStepPlan plan{};                 // this bubble as a set of one
    SbBubbleDesc desc{};               // host copy of the bubble's descriptor
    cudaGraphExec_t graph = nullptr;   // one captured step
    // staged I/O (sb_stage_upload_f32 / sb_stage_download_f32): a copy
    // stream, per field and direction an FP32 device buffer (made on first
    // use), and the events that order the buffers between the two streams
    cudaStream_t copy_stream = nullptr;
    float* stage_buf[2][SB_FIELD_COUNT] = {};      // [0] uploads, [1] downloads
    cudaEvent_t stage_ev[4][SB_FIELD_COUNT] = {};  // kUpLanded, kUpTaken, kDnReady, kDnDone
    bool up_pending[SB_FIELD_COUNT] = {};
};

static_assert(SB_STORE_FP32 == kStoreF32 && SB_STORE_BF16 == kStoreBF16, "storage codes");

namespace {

// Nondimensional coefficients as Bubble::Bubble (kernel/bubble.cu:2568-2603)
// and the constant upload of Bubble::run (2609-2638).
void derive_phys(const sb_params& p, SbPhys& ph) {
    const double U = 1.0;  // Bubble::Bubble forces U = 1
    const double sigma_r = kGasR * p.T;
    double M = p.Gamma_m * sigma_r / (3 * kRho * p.H * U * U);
    double gs = kG * p.radius / (U * U);
    if (p.M_scale > 0) M *= p.M_scale;
    if (p.gs_scale > 0) gs *= p.gs_scale;
    ph.M = (float)M;
    const double nuA = kNuA * (p.nu_scale > 0 ? p.nu_scale : 1.0);
    ph.Cr = (float)(kRhoA * std::sqrt(nuA * p.radius / U) / (kRho * p.H));
    ph.gs = (float)gs;
    ph.re = (float)(kNu / (U * p.radius));
    ph.viscous = p.viscous ? 1 : 0;
    const double gmax = kSigmaA / sigma_r / p.Gamma_m;
    ph.gmax = (float)gmax;
    // The reference marks gamma > gmax - 1e-7 as at its maximum
    // (kernel/bubble.cu:28, FP64).  Near gmax ~ 29 that band is below FP32's
    // resolution (1.9e-6) and gmax - 1e-7 rounds to gmax itself, so a cell
    // holding gmax would not count.  The threshold is the lower of
    // gmax - 1e-7 and the float two steps below gmax: gmax and the float
    // just below it (an interpolation of gmax values, rounded) are at the
    // maximum, and a broken cell whose gamma is set to gmax stays broken
    // for every reader.
    ph.gthr = std::min((float)(gmax - 1e-7), std::nextafter(std::nextafter(ph.gmax, 0.0f), 0.0f));
    ph.blend = (float)p.blendCoeff;
    ph.evap = (float)(kEvaporation * p.radius / (p.H * U));
}

// Spatial factor of the air-flow corridor (airFlowU/V, kernel/bubble.cu:
// 2301-2380) at one face; the time factor 3 - |t - 3| is applied per step.
double corridor(double radius, double gTheta, double gPhi, bool phiComponent) {
    const double sT = std::sin(gTheta), cT = std::cos(gTheta);
    const double sP = std::sin(gPhi), cP = std::cos(gPhi);
    const double angle = kPi / 2.;
    double wind[3] = {0., std::cos(angle), std::sin(angle)};
    double wl = 1.0 / std::sqrt(wind[0] * wind[0] + wind[1] * wind[1] + wind[2] * wind[2]);
    for (double& v : wind) v *= wl;
    const double pos[3] = {1., 0., 0.};
    double nrm[3] = {pos[1] * wind[2] - pos[2] * wind[1], pos[2] * wind[0] - pos[0] * wind[2],
                     pos[0] * wind[1] - pos[1] * wind[0]};
    double nl = 1.0 / std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    for (double& v : nrm) v *= nl;
    const double cur[3] = {sT * cP, sT * sP, cT};
    const double dn = nrm[0] * cur[0] + nrm[1] * cur[1] + nrm[2] * cur[2];
    const double beta = std::acos(std::fmax(-1.0, std::fmin(1.0, dn)));
    double prj[3] = {cur[0] - dn * nrm[0], cur[1] - dn * nrm[1], cur[2] - dn * nrm[2]};
    double pl = 1.0 / std::sqrt(prj[0] * prj[0] + prj[1] * prj[1] + prj[2] * prj[2]);
    for (double& v : prj) v *= pl;
    const double pw[3] = {nrm[1] * prj[2] - nrm[2] * prj[1], nrm[2] * prj[0] - nrm[0] * prj[2],
                          nrm[0] * prj[1] - nrm[1] * prj[0]};
    double x = (std::fabs(beta - kHalfPi) - 0.2) / (0.4 - 0.2);
    x = std::fmax(0.0, std::fmin(1.0, x));
    const double ss = x * x * (3.0 - 2.0 * x);
    const double s = 0.5 * std::sin(beta) / 1.0 * radius * (1. - ss);
    if (phiComponent) return s * (pw[0] * -sP + pw[1] * cP);
    return s * (pw[0] * cT * cP + pw[1] * cT * sP - pw[2] * sT);
}

// The corridor factors of every face of a grid (u_phi faces, then u_theta
// faces).  They depend on the grid and the radius only, and computing them
// in FP64 costs about 0.2 s at 512 x 1024, so they are made once per
// (nTheta, radius) and shared by later bubbles (a serving loop creates many
// bubbles of few sizes); at most 16 grids are kept.
struct Corridor {
    std::vector<float> u, v;
};

std::shared_ptr<const Corridor> corridor_factors(int nT, double radius) {
    static std::mutex mu;
    static std::map<std::pair<int, double>, std::shared_ptr<const Corridor>> cache;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(nT, radius);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    const int nP = 2 * nT;
    const double h = kPi / nT;
    auto c = std::make_shared<Corridor>();
    c->u.resize((size_t)nT * nP);
    c->v.resize((size_t)(nT - 1) * nP);
    for (int i = 0; i < nT; ++i)
        for (int j = 0; j < nP; ++j) {
            c->u[(size_t)i * nP + j] = (float)corridor(radius, (i + 0.5) * h, (j - 0.5) * h, true);
            if (i < nT - 1)
                c->v[(size_t)i * nP + j] = (float)corridor(radius, (i + 1.0) * h, j * h, false);
        }
    if (cache.size() >= 16) cache.clear();
    cache.emplace(key, c);
    return c;
}

struct ArenaPlan {
    Layout L;
    size_t tables, rowtab, rottab, eta, gam, uth, uph, eta_adv, gam_adv, uth_adv, uph_adv;
    size_t bim[8];
    size_t fwd[2], bwd[2], bwdprev;
    size_t uair_init, vair_init, corr_u, corr_v, uair, vair;
    size_t d_eta, d_gam, err_eta, err_gam;
    size_t dmass, cE, cS, rhs, r0, x, dx, r, z, z1, p, q, xff, pcr, pcr_levels, step, stats;
    size_t self, self_list, roff, done_at, cnt, rec, acc, bar;  // the bubble's solve set
    size_t tiles[3];                                           // its cell tiles
};

// Bytes of one stored thickness / surfactant element.
size_t scalar_bytes(int storage) { return storage == kStoreBF16 ? 2 : 4; }

ArenaPlan plan_arena(const SbGrid& g, int storage) {
    ArenaPlan a;
    const size_t N = (size_t)g.N, Nv = (size_t)g.Nv, F = sizeof(float);
    a.tables = a.L.take((size_t)(4 * g.nT + 2) * F);
    a.rowtab = a.L.take((size_t)g.nT * sizeof(float4));
    a.rottab = a.L.take((size_t)g.nP * sizeof(float2));
    const size_t S = scalar_bytes(storage);
    a.eta = a.L.take(N * S); a.gam = a.L.take(N * S);
    a.uth = a.L.take(Nv * F); a.uph = a.L.take(N * F);
    a.eta_adv = a.L.take(N * F); a.gam_adv = a.L.take(N * F);
    a.uth_adv = a.L.take(Nv * F); a.uph_adv = a.L.take(N * F);
    // init, delta, initL, deltaL of eta, then of gamma: the reference fields
    // in the stored type, the accumulators in FP32
    for (int k = 0; k < 8; ++k) a.bim[k] = a.L.take(N * ((k & 1) ? F : S));
    for (int k = 0; k < 2; ++k) {
        a.fwd[k] = a.L.take(N * sizeof(float4));
        a.bwd[k] = a.L.take(N * sizeof(float4));
    }
    a.bwdprev = a.L.take(N * sizeof(float4));
    a.uair_init = a.L.take(N * F); a.vair_init = a.L.take(Nv * F);
    a.corr_u = a.L.take(N * F); a.corr_v = a.L.take(Nv * F);
    a.uair = a.L.take((N + 1) * F); a.vair = a.L.take((Nv + 1) * F);
    a.d_eta = a.L.take(N * F); a.d_gam = a.L.take(N * F);
    a.err_eta = a.L.take(N * F); a.err_gam = a.L.take(N * F);
    a.dmass = a.L.take(N * F); a.cE = a.L.take(N * F); a.cS = a.L.take(N * F);
    a.rhs = a.L.take(N * F); a.r0 = a.L.take(N * F); a.x = a.L.take(N * F); a.dx = a.L.take(N * F);
    a.r = a.L.take(N * F);
    a.z = a.L.take(N * F); a.z1 = a.L.take(N * F); a.p = a.L.take(N * F); a.q = a.L.take(N * F);
    a.xff = a.L.take(N * 8);
    a.pcr = a.L.take((size_t)g.nT * factor_blob(g.nP).bytes);
    a.pcr_levels = a.L.take((size_t)g.nT * 4);
    a.self = a.L.take(sizeof(SbBubbleDesc));
    a.self_list = a.L.take(sizeof(SbBubbleDesc*));
    for (int k = 0; k < 3; ++k)
        a.tiles[k] = a.L.take(sizeof(int2) * (size_t)((g.N + kTileSizes[k] - 1) / kTileSizes[k]));
    a.roff = a.L.take(8);
    a.done_at = a.L.take(4);
    a.cnt = a.L.take(4);
    a.rec = a.L.take(2 * sizeof(SbSolveRec));
    a.acc = a.L.take(sizeof(unsigned long long) * kSolveAccWords);
    a.bar = a.L.take(sizeof(unsigned) * kGridBarWords);
    a.step = a.L.take(sizeof(SbStepParams));
    a.stats = a.L.take(sizeof(SbDevStats) + 64);
    return a;
}

int validate(const sb_params* p) {
    if (!p) return fail(SB_ERR_INVALID, "null params");
    if (!is_pow2(p->nTheta) || p->nTheta < 8 || p->nTheta > 1024)
        return fail(SB_ERR_INVALID, "nTheta must be a power of two in [8, 1024]");
    if (!(p->radius > 0) || !(p->H > 0) || !(p->Gamma_m > 0) || !(p->T > 0))
        return fail(SB_ERR_INVALID, "radius, H, Gamma_m and T must be positive");
    if (!(p->dt > 0)) return fail(SB_ERR_INVALID, "timePerStep must be positive");
    if (p->storage != SB_STORE_FP32 && p->storage != SB_STORE_BF16)
        return fail(SB_ERR_INVALID, "storage must be SB_STORE_FP32 or SB_STORE_BF16");
    if (p->solver_precond < 0 || p->solver_precond > 2)
        return fail(SB_ERR_INVALID, "solver_precond must be 0 (auto), 1 or 2");
    return SB_OK;
}

// The stored thickness / surfactant fields (FP32 or BF16 per bubble).
SbScalar* sptr(sb_bubble* b, sb_field w) {
    SbFields& f = b->f;
    switch (w) {
        case SB_ETA: return f.eta;
        case SB_GAMMA: return f.gam;
        case SB_ETA_INIT: return f.eta_init;
        case SB_ETA_INIT_LAST: return f.eta_initL;
        case SB_GAMMA_INIT: return f.gam_init;
        case SB_GAMMA_INIT_LAST: return f.gam_initL;
        default: return nullptr;
    }
}

// The FP32 fields.
float* fptr(sb_bubble* b, sb_field w) {
    SbFields& f = b->f;
    switch (w) {
        case SB_UTHETA: return f.uth;
        case SB_UPHI: return f.uph;
        case SB_ETA_DELTA: return f.eta_delta;
        case SB_ETA_DELTA_LAST: return f.eta_deltaL;
        case SB_GAMMA_DELTA: return f.gam_delta;
        case SB_GAMMA_DELTA_LAST: return f.gam_deltaL;
        case SB_UAIR_INIT: return f.uair_init;
        case SB_VAIR_INIT: return f.vair_init;
        case SB_UAIR: return f.uair;
        case SB_VAIR: return f.vair;
        default: return nullptr;
    }
}

float4* map_ptr(sb_bubble* b, sb_field w, int& comp) {
    comp = (w == SB_FWD_P || w == SB_BWD_P || w == SB_BWDPREV_P) ? 1 : 0;
    switch (w) {
        case SB_FWD_T: case SB_FWD_P: return b->f.fwd[b->cur];
        case SB_BWD_T: case SB_BWD_P: return b->f.bwd[b->cur];
        case SB_BWDPREV_T: case SB_BWDPREV_P: return b->f.bwdprev;
        default: return nullptr;
    }
}

// A map entry of cell (i, j) (the mapped point's displacement from the cell
// centre in the cell's frame, whose x axis lies at azimuth j h) and the
// mapped point's absolute grid coordinates (theta / h, phi / h in [0, nPhi)),
// in FP64 both ways.
void map_entry_to_abs(int i, int j, int nT, float4 D, double* th, double* ph) {
    const double h = kPi / nT, t0 = (i + 0.5) * h;
    const double X = std::sin(t0) + D.x, Y = D.y, Z = std::cos(t0) + D.z;
    *th = std::atan2(std::hypot(X, Y), Z) / h;
    double p = j + std::atan2(Y, X) / h;
    p = std::fmod(p, 2.0 * nT);
    if (p < 0) p += 2.0 * nT;
    *ph = p;
}

float4 map_entry_from_abs(int i, int j, int nT, double th, double ph) {
    const double h = kPi / nT, t0 = (i + 0.5) * h;
    const double t = th * h, dp = (ph - j) * h;
    const double X = std::sin(t) * std::cos(dp), Y = std::sin(t) * std::sin(dp), Z = std::cos(t);
    return make_float4((float)(X - std::sin(t0)), (float)Y, (float)(Z - std::cos(t0)), 0.0f);
}

// Writes the per-step scalars into the pinned slot and copies them to the
// device on `stream`; the caller makes sure no earlier copy of the slot is
// still in flight.
int write_step_params(sb_bubble* b, double t, double dt_s, cudaStream_t stream) {
    const double dtn = dt_s * 1.0 / b->params.radius;  // dt U / r with U = 1
    SbStepParams* s = b->h_step;
    s->dt = (float)dtn;
    s->invDt = (float)(1.0 / dtn);
    s->windg = (float)(3.0 - std::fabs(t - 3.0));
    s->mixA = (float)(t / 12.0);
    s->mixB = (float)(1.0 - t / 12.0);
    s->evapDt = (float)((double)b->ph.evap * dtn);
    s->pad[0] = s->pad[1] = 0.f;
    SB_CHECK(cudaMemcpyAsync(b->f.step, s, sizeof(SbStepParams), cudaMemcpyHostToDevice, stream));
    b->last_dt = dt_s;
    b->last_t = t;
    return SB_OK;
}

int set_step_params(sb_bubble* b, double t, double dt_s) {
    if (dt_s == b->last_dt && t == b->last_t) return SB_OK;
    SB_CHECK(cudaStreamSynchronize(b->stream));  // the pinned slot may be in flight
    return write_step_params(b, t, dt_s, b->stream);
}

// The next solve starts from dx = 0: the state it would warm-start from has
// been replaced (a field upload or initialiser).
int invalidate_warm_start(sb_bubble* b, cudaStream_t s) {
    SB_CHECK(cudaMemsetAsync(&b->f.stats->dx_valid, 0, sizeof(int), s));
    return SB_OK;
}

// Fields that define the state a solve warm-starts from (not the wind).
bool state_field(sb_field w) {
    return !(w == SB_UAIR_INIT || w == SB_VAIR_INIT || w == SB_UAIR || w == SB_VAIR);
}

int reset_bimocq(sb_bubble* b) {
    const size_t N = (size_t)b->g.N * scalar_bytes(b->storage), N4 = (size_t)b->g.N * 4;
    SbFields& f = b->f;
    SB_CHECK(cudaMemcpyAsync(f.eta_init, f.eta, N, cudaMemcpyDeviceToDevice, b->stream));
    SB_CHECK(cudaMemcpyAsync(f.eta_initL, f.eta, N, cudaMemcpyDeviceToDevice, b->stream));
    SB_CHECK(cudaMemcpyAsync(f.gam_init, f.gam, N, cudaMemcpyDeviceToDevice, b->stream));
    SB_CHECK(cudaMemcpyAsync(f.gam_initL, f.gam, N, cudaMemcpyDeviceToDevice, b->stream));
    SB_CHECK(cudaMemsetAsync(f.eta_delta, 0, N4, b->stream));
    SB_CHECK(cudaMemsetAsync(f.eta_deltaL, 0, N4, b->stream));
    SB_CHECK(cudaMemsetAsync(f.gam_delta, 0, N4, b->stream));
    SB_CHECK(cudaMemsetAsync(f.gam_deltaL, 0, N4, b->stream));
    SB_CHECK(launch_reset_maps(b->g, b->f, b->stream));
    return invalidate_warm_start(b, b->stream);
}

int upload_f32(sb_bubble* b, float* dst, const double* src, size_t n) {
    std::vector<float> tmp(n);
    for (size_t i = 0; i < n; ++i) tmp[i] = (float)src[i];
    SB_CHECK(cudaMemcpyAsync(dst, tmp.data(), n * sizeof(float), cudaMemcpyHostToDevice, b->stream));
    SB_CHECK(cudaStreamSynchronize(b->stream));
    return SB_OK;
}

// Device FP32 staging for stored fields: the re-initialisation error
// array, which only lives inside a step (k_accum -> k_reinit), while
// uploads and downloads run between steps on the bubble's stream.
float* staging(sb_bubble* b) { return b->f.err_eta; }

// Offset of a stored field (its family's base: eta or gamma).
float base_of(const sb_bubble* b, const SbScalar* p) {
    const SbFields& f = b->f;
    const bool gam = p == f.gam || p == f.gam_init || p == f.gam_initL;
    return gam ? b->ph.base_gam : b->ph.base_eta;
}

// FP32 data already on the device (staging) into a stored field.
int store_from_staging(sb_bubble* b, SbScalar* dst, size_t n) {
    SB_CHECK(launch_store(dst, staging(b), (int)n, base_of(b, dst), b->storage, b->stream));
    b->launches += 1;
    return SB_OK;
}

// A stored field as FP32 into the staging array.
int load_to_staging(sb_bubble* b, const SbScalar* src, size_t n) {
    SB_CHECK(launch_load(staging(b), src, (int)n, base_of(b, src), b->storage, b->stream));
    b->launches += 1;
    return SB_OK;
}

// v rounded to the nearest BF16 number (ties to even), as a float.
float bf16_round(float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
    std::memcpy(&v, &u, 4);
    return v;
}

// BF16 storage: the base of a field family becomes the mean of the values
// about to be stored (a BF16 number, so that 0 and the base stay exact);
// the kernels read it from the device descriptor.
int set_base(sb_bubble* b, bool gamma, const double* v, size_t n) {
    if (b->storage != kStoreBF16) return SB_OK;
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s += v[i];
    const float base = bf16_round(n ? (float)(s / (double)n) : 0.0f);
    (gamma ? b->ph.base_gam : b->ph.base_eta) = base;
    b->desc.ph = b->ph;
    SB_CHECK(cudaMemcpyAsync(&b->f.self->ph, &b->ph, sizeof(SbPhys), cudaMemcpyHostToDevice,
                             b->stream));
    SB_CHECK(cudaStreamSynchronize(b->stream));
    return SB_OK;
}

int upload_scalar(sb_bubble* b, SbScalar* dst, const double* src, size_t n) {
    std::vector<float> tmp(n);
    for (size_t i = 0; i < n; ++i) tmp[i] = (float)src[i];
    SB_CHECK(cudaMemcpyAsync(staging(b), tmp.data(), n * sizeof(float), cudaMemcpyHostToDevice,
                             b->stream));
    int rc = store_from_staging(b, dst, n);
    if (rc != SB_OK) return rc;
    SB_CHECK(cudaStreamSynchronize(b->stream));
    return SB_OK;
}

int fill_const(sb_bubble* b, SbScalar* dst, size_t n, float v) {
    std::vector<double> tmp(n, (double)v);
    return upload_scalar(b, dst, tmp.data(), n);
}

}  // namespace

extern "C" {

void sb_default_params(sb_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->radius = 0.05;
    p->H = 0.000001;
    p->U = 1.0;
    p->c_m = 0.5;
    p->Gamma_m = 0.000001;
    p->T = 298.15;
    p->Ds = 0.0;
    p->rm = 0.000000005;
    p->nTheta = 256;
    p->dt = 0.005;
    p->DT = 0.02;
    p->frames = 500;
    p->blendCoeff = 0.5;
    p->device = 0;
}

size_t sb_bytes_required(const sb_params* p) {
    if (validate(p) != SB_OK) return 0;
    SbGrid g{};
    g.nT = p->nTheta;
    g.nP = 2 * p->nTheta;
    g.N = g.nT * g.nP;
    g.Nv = (g.nT - 1) * g.nP;
    return plan_arena(g, p->storage).L.bytes;
}

int sb_create(const sb_params* p, sb_bubble** out) {
    if (!out) return fail(SB_ERR_INVALID, "null output handle");
    *out = nullptr;
    int rc = validate(p);
    if (rc != SB_OK) return rc;
    SB_CHECK(cudaSetDevice(p->device));
    sb_bubble* b = new sb_bubble();
    b->params = *p;
    b->device = p->device;
    SbGrid& g = b->g;
    g.nT = p->nTheta;
    g.nP = 2 * p->nTheta;
    g.maskP = g.nP - 1;
    g.logP = 0;
    while ((1 << g.logP) < g.nP) ++g.logP;
    g.N = g.nT * g.nP;
    g.Nv = (g.nT - 1) * g.nP;
    g.h = (float)(kPi / g.nT);
    g.invh = (float)(g.nT / kPi);
    derive_phys(*p, b->ph);
    b->solver.mode = p->solver_mode == 1 ? 0 : 1;
    b->solver.tol = p->solver_tol > 0 ? p->solver_tol : 1e-6;
    b->solver.max_iter = p->solver_max_iter > 0 ? p->solver_max_iter : 1000;
    b->solver.warm = p->solver_cold_start ? 0 : 1;
    b->solver.precond = p->solver_precond == 1 ? kPrecLine
                        : p->solver_precond == 2 ? kPrecNeumann : kPrecAuto;
    b->force_reinit = p->force_reinit == 1 ? 0 : (p->force_reinit == 2 ? 1 : -1);
    b->storage = p->storage;
    b->ph.plain_adv = p->plain_advection ? 1 : 0;
    b->ph.single_step = p->single_step_velocity ? 1 : 0;
    if (b->ph.plain_adv) b->force_reinit = 0;  // no maps: nothing to re-initialise
    // BF16 storage: offsets of the initial fields (eta = 0.5, gamma = 1)
    b->ph.base_eta = b->storage == kStoreBF16 ? 0.5f : 0.0f;
    b->ph.base_gam = b->storage == kStoreBF16 ? 1.0f : 0.0f;

    ArenaPlan a = plan_arena(g, p->storage);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->arena, a.L.bytes);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->h_step, sizeof(SbStepParams));
    if (e != cudaSuccess) {
        int r = cuda_fail(e, "sb_create allocation");
        sb_destroy(b);
        return r;
    }
    b->arena_bytes = a.L.bytes;
    e = cudaMemset(b->arena, 0, a.L.bytes);
    if (e != cudaSuccess) { int r = cuda_fail(e, "memset"); sb_destroy(b); return r; }
    char* A = b->arena;
    auto F32 = [&](size_t off) { return (float*)(A + off); };
    SbFields& f = b->f;
    b->tables = F32(a.tables);
    auto SCL = [&](size_t off) { return (SbScalar*)(A + off); };
    f.eta = SCL(a.eta); f.gam = SCL(a.gam); f.uth = F32(a.uth); f.uph = F32(a.uph);
    f.eta_adv = F32(a.eta_adv); f.gam_adv = F32(a.gam_adv);
    f.uth_adv = F32(a.uth_adv); f.uph_adv = F32(a.uph_adv);
    f.eta_init = SCL(a.bim[0]); f.eta_delta = F32(a.bim[1]);
    f.eta_initL = SCL(a.bim[2]); f.eta_deltaL = F32(a.bim[3]);
    f.gam_init = SCL(a.bim[4]); f.gam_delta = F32(a.bim[5]);
    f.gam_initL = SCL(a.bim[6]); f.gam_deltaL = F32(a.bim[7]);
    for (int k = 0; k < 2; ++k) {
        f.fwd[k] = (float4*)(A + a.fwd[k]);
        f.bwd[k] = (float4*)(A + a.bwd[k]);
    }
    f.bwdprev = (float4*)(A + a.bwdprev);
    f.uair_init = F32(a.uair_init); f.vair_init = F32(a.vair_init);
    f.corr_u = F32(a.corr_u); f.corr_v = F32(a.corr_v);
    f.uair = F32(a.uair); f.vair = F32(a.vair);
    f.d_eta = F32(a.d_eta); f.d_gam = F32(a.d_gam);
    f.err_eta = F32(a.err_eta); f.err_gam = F32(a.err_gam);
    f.dmass = F32(a.dmass); f.cE = F32(a.cE); f.cS = F32(a.cS); f.rhs = F32(a.rhs); f.r0 = F32(a.r0);
    f.x = F32(a.x); f.dx = F32(a.dx); f.r = F32(a.r); f.z = F32(a.z); f.z1 = F32(a.z1);
    f.p = F32(a.p); f.q = F32(a.q);
    f.xff = (float2*)(A + a.xff);
    f.pcr = (float*)(A + a.pcr);
    f.pcr_levels = (int*)(A + a.pcr_levels);
    f.step = (SbStepParams*)(A + a.step);
    f.stats = (SbDevStats*)(A + a.stats);
    // the solve set of this bubble alone (rows 0 .. nT-1; the memset above
    // leaves the row counter at zero)
    f.self = (SbBubbleDesc*)(A + a.self);
    f.roff = (int*)(A + a.roff);
    f.done_at = (int*)(A + a.done_at);
    f.cnt = (int*)(A + a.cnt);
    f.rec = (SbSolveRec*)(A + a.rec);
    f.acc = (unsigned long long*)(A + a.acc);
    f.bar = (unsigned*)(A + a.bar);

    // trigonometric tables in FP64, stored FP32
    std::vector<float> tab(4 * g.nT + 2);
    float* sin_c = tab.data();
    float* cos_c = sin_c + g.nT;
    float* sin_e = cos_c + g.nT;
    float* cos_e = sin_e + g.nT + 1;
    const double h = kPi / g.nT;
    for (int i = 0; i < g.nT; ++i) {
        sin_c[i] = (float)std::sin((i + 0.5) * h);
        cos_c[i] = (float)std::cos((i + 0.5) * h);
    }
    for (int i = 0; i <= g.nT; ++i) {
        sin_e[i] = (float)std::sin(i * h);
        cos_e[i] = (float)std::cos(i * h);
    }
    sin_e[0] = 0.0f;
    sin_e[g.nT] = 0.0f;  // sin(0) and sin(pi): the pole couplings vanish
    cos_e[0] = 1.0f;
    cos_e[g.nT] = -1.0f;
    g.sin_c = b->tables;
    g.cos_c = b->tables + g.nT;
    g.sin_e = b->tables + 2 * g.nT;
    g.cos_e = b->tables + 3 * g.nT + 1;
    e = cudaMemcpy(b->tables, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { int r = cuda_fail(e, "tables"); sb_destroy(b); return r; }
    // characteristic-map geometry: row angles as (hi, lo) float pairs and
    // the rotation by every column offset
    {
        std::vector<float4> row((size_t)g.nT);
        for (int i = 0; i < g.nT; ++i) {
            const double sv = std::sin((i + 0.5) * h), cv = std::cos((i + 0.5) * h);
            const float sh = (float)sv, ch = (float)cv;
            row[i] = make_float4(sh, (float)(sv - sh), ch, (float)(cv - ch));
        }
        std::vector<float2> rot((size_t)g.nP);
        for (int k = 0; k < g.nP; ++k) {
            const double d = (k - g.nT) * h, sh = std::sin(0.5 * d);
            rot[k] = make_float2((float)std::sin(d), (float)(-2.0 * sh * sh));
        }
        g.rowtab = (const float4*)(A + a.rowtab);
        g.rottab = (const float2*)(A + a.rottab);
        e = cudaMemcpy((void*)g.rowtab, row.data(), row.size() * sizeof(float4), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy((void*)g.rottab, rot.data(), rot.size() * sizeof(float2),
                           cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { int r = cuda_fail(e, "map tables"); sb_destroy(b); return r; }
    }

    // static corridor factors
    {
        const std::shared_ptr<const Corridor> c = corridor_factors(g.nT, p->radius);
        e = cudaMemcpy(f.corr_u, c->u.data(), c->u.size() * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(f.corr_v, c->v.data(), c->v.size() * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { int r = cuda_fail(e, "corridor"); sb_destroy(b); return r; }
    }
    // Solver::Solver initial state: eta = 0.5, gamma = 1, u = 0, no wind
    rc = fill_const(b, f.eta, (size_t)g.N, 0.5f);
    if (rc == SB_OK) rc = fill_const(b, f.gam, (size_t)g.N, 1.0f);
    if (rc == SB_OK) rc = reset_bimocq(b);
    if (rc == SB_OK) {
        SbDevStats st{};
        st.force_reinit = b->force_reinit;
        e = cudaMemcpy(f.stats, &st, sizeof(st), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_fail(e, "stats");
    }
    if (rc == SB_OK) {
        // the bubble's own descriptor, and the launch plan of the bubble
        // as a set of one
        SbBubbleDesc d{};
        d.g = g;
        d.ph = b->ph;
        d.f = f;
        d.cur = 0;
        const int roff[2] = {0, g.nT};
        SbBubbleDesc** self_list = (SbBubbleDesc**)(A + a.self_list);
        e = cudaMemcpy(f.self, &d, sizeof(d), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(f.roff, roff, sizeof(roff), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(self_list, &f.self, sizeof(f.self), cudaMemcpyHostToDevice);
        SbStepPlan& P = b->plan;
        P.descs = self_list;
        P.nb = 1;
        for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
            std::vector<int2> tl;
            for (int c = 0; c < g.N; c += kTileSizes[k]) tl.push_back(make_int2(0, c));
            P.tiles[k] = (const int2*)(A + a.tiles[k]);
            P.ntiles[k] = (int)tl.size();
            e = cudaMemcpy((void*)P.tiles[k], tl.data(), sizeof(int2) * tl.size(), cudaMemcpyHostToDevice);
        }
        for (int st = 0; st < STAGE_COUNT; ++st) P.sel[st] = 1;
        SbSolveSet& S = P.set;
        S.descs = self_list;
        S.nb = 1;
        S.R = g.nT;
        S.roff = f.roff;
        S.rec = f.rec;
        S.done_at = f.done_at;
        S.cnt = f.cnt;
        S.acc = f.acc;
        S.bar = f.bar;
        P.maxNP = g.nP;
        P.solver = b->solver;
        P.storage = b->storage;
        P.viscous = b->ph.viscous;
        b->desc = d;
        P.one = &b->desc;
        if (e != cudaSuccess) rc = cuda_fail(e, "step plan");
    }
    if (rc == SB_OK) {
        e = prepare_plan(b->plan);
        if (e != cudaSuccess) rc = cuda_fail(e, "prepare_plan");
    }
    if (rc == SB_OK) rc = set_step_params(b, 0.0, p->dt);
    if (rc == SB_OK) {
        e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "sb_create sync");
    }
    if (rc != SB_OK) {
        sb_destroy(b);
        return rc;
    }
    *out = b;
    return SB_OK;
}

int sb_destroy(sb_bubble* b) {
    if (!b) return SB_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->copy_stream) {
        cudaStreamSynchronize(b->copy_stream);
        cudaStreamDestroy(b->copy_stream);
    }
    for (auto& row : b->stage_buf)
        for (float* p : row)
            if (p) cudaFree(p);
    for (auto& row : b->stage_ev)
        for (cudaEvent_t e : row)
            if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : b->ev)
        if (e) cudaEventDestroy(e);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->arena) cudaFree(b->arena);
    if (b->h_step) cudaFreeHost(b->h_step);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return SB_OK;
}

size_t sb_field_size(const sb_bubble* b, sb_field which) {
    if (!b) return 0;
    if (which == SB_UTHETA || which == SB_VAIR_INIT) return (size_t)b->g.Nv;
    if (which == SB_UAIR) return (size_t)b->g.N + 1;
    if (which == SB_VAIR) return (size_t)b->g.Nv + 1;
    if (which < 0 || which >= SB_FIELD_COUNT) return 0;
    return (size_t)b->g.N;
}

int sb_upload_field(sb_bubble* b, sb_field which, const double* src, size_t n) {
    if (!b || !src) return fail(SB_ERR_INVALID, "null argument");
    if (n != sb_field_size(b, which)) return fail(SB_ERR_INVALID, "element count mismatch");
    SB_CHECK(cudaSetDevice(b->device));
    if (state_field(which)) {
        int r = invalidate_warm_start(b, b->stream);
        if (r != SB_OK) return r;
    }
    int comp = 0;
    float4* m = map_ptr(b, which, comp);
    if (m) {
        // absolute grid coordinates of one component -> displacements (the
        // other component is kept: read, converted, replaced, written back)
        const int nT = b->g.nT, nP = b->g.nP;
        std::vector<float4> tmp((size_t)b->g.N);
        SB_CHECK(cudaMemcpyAsync(tmp.data(), m, tmp.size() * sizeof(float4), cudaMemcpyDeviceToHost,
                                 b->stream));
        SB_CHECK(cudaStreamSynchronize(b->stream));
        for (int i = 0; i < nT; ++i)
            for (int j = 0; j < nP; ++j) {
                const size_t c = (size_t)i * nP + j;
                double th, ph;
                map_entry_to_abs(i, j, nT, tmp[c], &th, &ph);
                if (comp == 0) th = src[c];
                else ph = src[c];
                tmp[c] = map_entry_from_abs(i, j, nT, th, ph);
            }
        SB_CHECK(cudaMemcpyAsync(m, tmp.data(), tmp.size() * sizeof(float4), cudaMemcpyHostToDevice,
                                 b->stream));
        SB_CHECK(cudaStreamSynchronize(b->stream));
        return SB_OK;
    }
    if (SbScalar* s = sptr(b, which)) return upload_scalar(b, s, src, n);
    float* d = fptr(b, which);
    if (!d) return fail(SB_ERR_INVALID, "unknown field");
    return upload_f32(b, d, src, n);
}

int sb_download_field(sb_bubble* b, sb_field which, double* dst, size_t n) {
    if (!b || !dst) return fail(SB_ERR_INVALID, "null argument");
    if (n != sb_field_size(b, which)) return fail(SB_ERR_INVALID, "element count mismatch");
    SB_CHECK(cudaSetDevice(b->device));
    int comp = 0;
    float4* m = map_ptr(b, which, comp);
    if (m) {
        const int nT = b->g.nT, nP = b->g.nP;
        std::vector<float4> tmp((size_t)b->g.N);
        SB_CHECK(cudaMemcpyAsync(tmp.data(), m, tmp.size() * sizeof(float4), cudaMemcpyDeviceToHost,
                                 b->stream));
        SB_CHECK(cudaStreamSynchronize(b->stream));
        for (int i = 0; i < nT; ++i)
            for (int j = 0; j < nP; ++j) {
                const size_t c = (size_t)i * nP + j;
                double th, ph;
                map_entry_to_abs(i, j, nT, tmp[c], &th, &ph);
                dst[c] = comp == 0 ? th : ph;
            }
        return SB_OK;
    }
    const float* d = fptr(b, which);
    if (SbScalar* s = sptr(b, which)) {
        int rc = load_to_staging(b, s, n);
        if (rc != SB_OK) return rc;
        d = staging(b);
    }
    if (!d) return fail(SB_ERR_INVALID, "unknown field");
    std::vector<float> tmp(n);
    SB_CHECK(cudaMemcpyAsync(tmp.data(), d, n * sizeof(float), cudaMemcpyDeviceToHost, b->stream));
    SB_CHECK(cudaStreamSynchronize(b->stream));
    for (size_t i = 0; i < n; ++i) dst[i] = (double)tmp[i];
    return SB_OK;
}

int sb_download_system(sb_bubble* b, sb_system_array which, double* dst, size_t n) {
    if (!b || !dst) return fail(SB_ERR_INVALID, "null argument");
    if (n != (size_t)b->g.N) return fail(SB_ERR_INVALID, "element count mismatch");
    const SbFields& f = b->f;
    const float* d = nullptr;
    switch (which) {
        case SB_SYS_ETA_ADV: d = f.eta_adv; break;
        case SB_SYS_GAMMA_ADV: d = f.gam_adv; break;
        case SB_SYS_DMASS: d = f.dmass; break;
        case SB_SYS_WEAST: d = f.cE; break;
        case SB_SYS_WSOUTH: d = f.cS; break;
        case SB_SYS_R0: d = f.r0; break;
        case SB_SYS_RHS: d = f.rhs; break;
        case SB_SYS_DX: d = f.dx; break;
        default: return fail(SB_ERR_INVALID, "unknown system array");
    }
    SB_CHECK(cudaSetDevice(b->device));
    std::vector<float> tmp(n);
    SB_CHECK(cudaMemcpyAsync(tmp.data(), d, n * sizeof(float), cudaMemcpyDeviceToHost, b->stream));
    SB_CHECK(cudaStreamSynchronize(b->stream));
    for (size_t i = 0; i < n; ++i) dst[i] = (double)tmp[i];
    return SB_OK;
}

int sb_exr_load_resized(const char* path, const char* channel, int width, int height,
                        double* out) {
    if (!path || !channel || !out || width <= 0 || height <= 0)
        return fail(SB_ERR_INVALID, "bad argument");
    int w = 0, h = 0;
    std::vector<float> img;
    std::string err;
    if (!read_exr_channel(path, channel, &w, &h, img, err)) return fail(SB_ERR_IO, err);
    std::vector<float> r((size_t)width * height);
    resize_linear(img.data(), w, h, r.data(), width, height);
    for (size_t i = 0; i < r.size(); ++i) out[i] = (double)r[i];
    return SB_OK;
}

int sb_init_thickness_from_exr(sb_bubble* b, const char* path) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    if (!path || !*path) return SB_OK;  // eta = 0.5 from sb_create
    const int nT = b->g.nT, nP = b->g.nP;
    std::vector<double> c((size_t)nT * nP);
    int rc = sb_exr_load_resized(path, "B", nP, nT, c.data());
    if (rc != SB_OK) return rc;
    for (double& v : c) v = (v - 0.5) * 0.3 + 0.5;  // initializer.cu:74-75
    SB_CHECK(cudaSetDevice(b->device));
    rc = set_base(b, false, c.data(), c.size());
    if (rc == SB_OK) rc = upload_scalar(b, b->f.eta, c.data(), c.size());
    if (rc == SB_OK) rc = reset_bimocq(b);
    if (rc == SB_OK) {
        cudaError_t e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "thickness init");
    }
    return rc;
}

int sb_init_airflow_from_exr(sb_bubble* b, const char* path) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    const int nT = b->g.nT, nP = b->g.nP;
    const size_t N = (size_t)nT * nP, Nv = (size_t)(nT - 1) * nP;
    std::vector<double> u(N, 0.0), v(Nv, 0.0);
    if (path && *path) {
        std::vector<double> G(N), R(N);
        int rc = sb_exr_load_resized(path, "G", nP, nT, G.data());
        if (rc == SB_OK) rc = sb_exr_load_resized(path, "R", nP, nT, R.data());
        if (rc != SB_OK) return rc;
        const double r = b->params.radius;
        for (int j = 0; j < nT; ++j)
            for (int i = 0; i < nP; ++i) {
                const size_t c = (size_t)j * nP + i;
                u[c] = 0.5 * (G[c] + G[(size_t)j * nP + (i + nP - 1) % nP]) * r;
                if (j < nT - 1) v[c] = -0.5 * (R[c] + R[c + nP]) * r;
            }
    }
    SB_CHECK(cudaSetDevice(b->device));
    int rc = upload_f32(b, b->f.uair_init, u.data(), N);
    if (rc == SB_OK) rc = upload_f32(b, b->f.vair_init, v.data(), Nv);
    return rc;
}

int sb_upload_fields(sb_bubble* b, const double* eta, const double* gamma, const double* u_theta,
                     const double* u_phi, const double* uair_init, const double* vair_init) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    SB_CHECK(cudaSetDevice(b->device));
    const size_t N = (size_t)b->g.N, Nv = (size_t)b->g.Nv;
    int rc = SB_OK;
    if (eta && rc == SB_OK) rc = set_base(b, false, eta, N);
    if (eta && rc == SB_OK) rc = upload_scalar(b, b->f.eta, eta, N);
    if (gamma && rc == SB_OK) rc = set_base(b, true, gamma, N);
    if (gamma && rc == SB_OK) rc = upload_scalar(b, b->f.gam, gamma, N);
    if (u_theta && rc == SB_OK) rc = upload_f32(b, b->f.uth, u_theta, Nv);
    if (u_phi && rc == SB_OK) rc = upload_f32(b, b->f.uph, u_phi, N);
    if (uair_init && rc == SB_OK) rc = upload_f32(b, b->f.uair_init, uair_init, N);
    if (vair_init && rc == SB_OK) rc = upload_f32(b, b->f.vair_init, vair_init, Nv);
    if (rc == SB_OK) rc = reset_bimocq(b);
    if (rc == SB_OK) {
        cudaError_t e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "upload sync");
    }
    return rc;
}

}  // extern "C"

namespace {

// One step of a plan captured as a CUDA graph.  The per-step scalars and
// every bubble's map parity live in device memory, so the graph is replayed
// unchanged step after step.
int capture_plan(const SbStepPlan& P, cudaStream_t s, cudaGraphExec_t* out) {
    cudaGraph_t graph = nullptr;
    SB_CHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_plan_step(P, s);
    cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "step graph capture");
    return SB_OK;
}

// One step launched stage by stage with events between the stages; adds
// every stage's device time (ms) to stage_ms.  Synchronises.
int timed_plan_step(const SbStepPlan& P, cudaStream_t s, cudaEvent_t* ev, double* stage_ms) {
    if (!ev[0])
        for (int k = 0; k <= STAGE_COUNT; ++k) SB_CHECK(cudaEventCreate(&ev[k]));
    SB_CHECK(cudaEventRecord(ev[0], s));
    for (int st = 0; st < STAGE_COUNT; ++st) {
        SB_CHECK(launch_plan_stage(P, st, s));
        SB_CHECK(cudaEventRecord(ev[st + 1], s));
    }
    SB_CHECK(launch_plan_flip(P, s));
    SB_CHECK(cudaEventSynchronize(ev[STAGE_COUNT]));
    for (int st = 0; st < STAGE_COUNT; ++st) {
        float ms = 0.f;
        SB_CHECK(cudaEventElapsedTime(&ms, ev[st], ev[st + 1]));
        stage_ms[st] += ms;
    }
    return SB_OK;
}

// Tile-size autotuner: one timed step with every tile size, then the
// fastest size of each stage.  The kernels compute the same values at every
// tile size.  `step` runs one timed step (and keeps the handle's
// bookkeeping).
template <typename StepFn>
int autotune_plan(SbStepPlan& P, StepFn step, int* tile_sizes) {
    double ms[3][STAGE_COUNT + 1] = {};
    for (int k = 0; k < 3; ++k) {
        for (int st = 0; st < STAGE_COUNT; ++st) P.sel[st] = k;
        int rc = step(ms[k]);
        if (rc != SB_OK) return rc;
    }
    for (int st = 0; st < STAGE_COUNT; ++st) {
        int best = 1;
        for (int k = 0; k < 3; ++k)
            if (ms[k][st] < ms[best][st]) best = k;
        P.sel[st] = best;
        if (tile_sizes) tile_sizes[st] = kTileSizes[best];
    }
    return SB_OK;
}

void bubble_advance(sb_bubble* b, int n) {
    b->launches += (long long)n * (STAGE_COUNT + 1);
    b->steps += n;
    b->cur ^= (n & 1);
}

}  // namespace

extern "C" {

namespace {

enum { kUpLanded = 0, kUpTaken = 1, kDnReady = 2, kDnDone = 3 };

// The copy stream, the buffer of `which` for direction dir (0 up, 1 down)
// and the field's events, made on first use.
int stage_prepare(sb_bubble* b, sb_field which, int dir) {
    if (!b->copy_stream) SB_CHECK(cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking));
    if (!b->stage_ev[0][which])
        for (int k = 0; k < 4; ++k)
            SB_CHECK(cudaEventCreateWithFlags(&b->stage_ev[k][which], cudaEventDisableTiming));
    if (!b->stage_buf[dir][which]) {
        const size_t n = sb_field_size(b, which);
        if (cudaMalloc(&b->stage_buf[dir][which], n * sizeof(float)) != cudaSuccess)
            return fail(SB_ERR_OOM, "staging buffer allocation failed");
    }
    return SB_OK;
}

// Moves the staged uploads that have not been taken yet into their fields,
// on stream s, after their host copies have landed.
int take_staged_uploads(sb_bubble* b, cudaStream_t s) {
    for (int w = 0; w < SB_FIELD_COUNT; ++w) {
        if (!b->up_pending[w]) continue;
        const sb_field which = (sb_field)w;
        const size_t n = sb_field_size(b, which);
        const float* src = b->stage_buf[0][w];
        SB_CHECK(cudaStreamWaitEvent(s, b->stage_ev[kUpLanded][w], 0));
        SbScalar* sp = sptr(b, which);
        if (sp && b->storage != kStoreF32) {
            SB_CHECK(launch_store(sp, src, (int)n, base_of(b, sp), b->storage, s));
            b->launches += 1;
        } else {
            float* dst = sp ? reinterpret_cast<float*>(sp) : fptr(b, which);
            SB_CHECK(cudaMemcpyAsync(dst, src, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        }
        SB_CHECK(cudaEventRecord(b->stage_ev[kUpTaken][w], s));
        b->up_pending[w] = false;
        if (state_field(which)) {
            int r = invalidate_warm_start(b, s);
            if (r != SB_OK) return r;
        }
    }
    return SB_OK;
}

bool stageable(sb_bubble* b, sb_field which) {
    return which >= 0 && which < SB_FIELD_COUNT && (sptr(b, which) || fptr(b, which));
}

}  // namespace

int sb_stage_upload_f32(sb_bubble* b, sb_field which, const float* src, size_t n) {
    if (!b || !src) return fail(SB_ERR_INVALID, "null argument");
    if (!stageable(b, which)) return fail(SB_ERR_INVALID, "maps cannot be staged");
    if (n != sb_field_size(b, which)) return fail(SB_ERR_INVALID, "element count mismatch");
    if (b->up_pending[which])
        return fail(SB_ERR_INVALID, "the field's previous staged upload has not been taken by a step");
    SB_CHECK(cudaSetDevice(b->device));
    int rc = stage_prepare(b, which, 0);
    if (rc != SB_OK) return rc;
    // the buffer is free once the step that took the previous upload has copied it
    SB_CHECK(cudaStreamWaitEvent(b->copy_stream, b->stage_ev[kUpTaken][which], 0));
    SB_CHECK(cudaMemcpyAsync(b->stage_buf[0][which], src, n * sizeof(float),
                             cudaMemcpyHostToDevice, b->copy_stream));
    SB_CHECK(cudaEventRecord(b->stage_ev[kUpLanded][which], b->copy_stream));
    b->up_pending[which] = true;
    return SB_OK;
}

int sb_stage_download_f32(sb_bubble* b, sb_field which, float* dst, size_t n) {
    if (!b || !dst) return fail(SB_ERR_INVALID, "null argument");
    if (!stageable(b, which)) return fail(SB_ERR_INVALID, "maps cannot be staged");
    if (n != sb_field_size(b, which)) return fail(SB_ERR_INVALID, "element count mismatch");
    SB_CHECK(cudaSetDevice(b->device));
    int rc = stage_prepare(b, which, 1);
    if (rc != SB_OK) return rc;
    float* buf = b->stage_buf[1][which];
    // snapshot of the field after the queued steps (the buffer is free once
    // the previous staged download of the field has left it)
    SB_CHECK(cudaStreamWaitEvent(b->stream, b->stage_ev[kDnDone][which], 0));
    SbScalar* sp = sptr(b, which);
    if (sp && b->storage != kStoreF32) {
        SB_CHECK(launch_load(buf, sp, (int)n, base_of(b, sp), b->storage, b->stream));
        b->launches += 1;
    } else {
        const float* src = sp ? reinterpret_cast<const float*>(sp) : fptr(b, which);
        SB_CHECK(cudaMemcpyAsync(buf, src, n * sizeof(float), cudaMemcpyDeviceToDevice, b->stream));
    }
    SB_CHECK(cudaEventRecord(b->stage_ev[kDnReady][which], b->stream));
    SB_CHECK(cudaStreamWaitEvent(b->copy_stream, b->stage_ev[kDnReady][which], 0));
    SB_CHECK(cudaMemcpyAsync(dst, buf, n * sizeof(float), cudaMemcpyDeviceToHost, b->copy_stream));
    SB_CHECK(cudaEventRecord(b->stage_ev[kDnDone][which], b->copy_stream));
    return SB_OK;
}

int sb_wait_staged(sb_bubble* b) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    if (!b->copy_stream) return SB_OK;
    SB_CHECK(cudaSetDevice(b->device));
    SB_CHECK(cudaStreamSynchronize(b->copy_stream));
    return SB_OK;
}

int sb_step(sb_bubble* b, int n_steps, double t_frame, double dt) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    if (n_steps < 0 || !(dt > 0)) return fail(SB_ERR_INVALID, "bad step count or dt");
    SB_CHECK(cudaSetDevice(b->device));
    int rc = set_step_params(b, t_frame, dt);
    if (rc != SB_OK) return rc;
    if ((rc = take_staged_uploads(b, b->stream)) != SB_OK) return rc;
    if (n_steps > 0 && !b->graph && (rc = capture_plan(b->plan, b->stream, &b->graph)) != SB_OK)
        return rc;
    for (int s = 0; s < n_steps; ++s) SB_CHECK(cudaGraphLaunch(b->graph, b->stream));
    bubble_advance(b, n_steps);
    return SB_OK;
}

int sb_step_timed(sb_bubble* b, int n_steps, double t_frame, double dt, double* stage_ms) {
    if (!b || !stage_ms) return fail(SB_ERR_INVALID, "null argument");
    if (n_steps < 0 || !(dt > 0)) return fail(SB_ERR_INVALID, "bad step count or dt");
    SB_CHECK(cudaSetDevice(b->device));
    int rc = set_step_params(b, t_frame, dt);
    if (rc != SB_OK) return rc;
    if ((rc = take_staged_uploads(b, b->stream)) != SB_OK) return rc;
    for (int s = 0; s < n_steps; ++s) {
        if ((rc = timed_plan_step(b->plan, b->stream, b->ev, stage_ms)) != SB_OK) return rc;
        bubble_advance(b, 1);
    }
    return SB_OK;
}

int sb_autotune(sb_bubble* b, double t_frame, double dt, int* tile_sizes) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    if (!(dt > 0)) return fail(SB_ERR_INVALID, "bad dt");
    SB_CHECK(cudaSetDevice(b->device));
    int rc = set_step_params(b, t_frame, dt);
    if (rc != SB_OK) return rc;
    rc = autotune_plan(b->plan, [&](double* ms) {
        int r = timed_plan_step(b->plan, b->stream, b->ev, ms);
        if (r == SB_OK) bubble_advance(b, 1);
        return r;
    }, tile_sizes);
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return rc;
}

int sb_stage_count(void) { return STAGE_COUNT; }

const char* sb_stage_name(int stage) {
    static const char* names[STAGE_COUNT] = {"k_advect_maps", "k_velocity", "k_bimocq",
                                             "k_assemble", "k_solve", "k_post", "k_accum",
                                             "k_reinit"};
    return (stage >= 0 && stage < STAGE_COUNT) ? names[stage] : "";
}

int sb_upload_field_f32(sb_bubble* b, sb_field which, const float* src, size_t n) {
    if (!b || !src) return fail(SB_ERR_INVALID, "null argument");
    if (n != sb_field_size(b, which)) return fail(SB_ERR_INVALID, "element count mismatch");
    SbScalar* s = sptr(b, which);
    float* d = s ? (b->storage == kStoreF32 ? reinterpret_cast<float*>(s) : staging(b))
                 : fptr(b, which);
    if (!d) return fail(SB_ERR_INVALID, "maps move through sb_upload_field");
    SB_CHECK(cudaSetDevice(b->device));
    if (state_field(which)) {
        int r = invalidate_warm_start(b, b->stream);
        if (r != SB_OK) return r;
    }
    SB_CHECK(cudaMemcpyAsync(d, src, n * sizeof(float), cudaMemcpyHostToDevice, b->stream));
    if (s && b->storage != kStoreF32) return store_from_staging(b, s, n);
    return SB_OK;
}

int sb_download_field_f32(sb_bubble* b, sb_field which, float* dst, size_t n) {
    if (!b || !dst) return fail(SB_ERR_INVALID, "null argument");
    if (n != sb_field_size(b, which)) return fail(SB_ERR_INVALID, "element count mismatch");
    SbScalar* s = sptr(b, which);
    const float* d = s ? (b->storage == kStoreF32 ? reinterpret_cast<const float*>(s) : staging(b))
                       : fptr(b, which);
    if (!d) return fail(SB_ERR_INVALID, "maps move through sb_download_field");
    SB_CHECK(cudaSetDevice(b->device));
    if (s && b->storage != kStoreF32) {
        int rc = load_to_staging(b, s, n);
        if (rc != SB_OK) return rc;
    }
    SB_CHECK(cudaMemcpyAsync(dst, d, n * sizeof(float), cudaMemcpyDeviceToHost, b->stream));
    return SB_OK;
}

int sb_synchronize(sb_bubble* b) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    SB_CHECK(cudaSetDevice(b->device));
    SB_CHECK(cudaStreamSynchronize(b->stream));
    // the outcome of the most recent solve (none before the first step)
    SbDevStats st;
    SB_CHECK(cudaMemcpy(&st, b->f.stats, sizeof(st), cudaMemcpyDeviceToHost));
    if (st.solves > 0 && !st.solver_converged)
        return fail(SB_ERR_NOT_CONVERGED, "the last implicit solve missed its tolerance");
    return SB_OK;
}

int sb_selftest_grid_barrier(sb_bubble* b, int absent_block, unsigned poll_limit) {
    constexpr int kProbeBlocks = 4;
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    if (absent_block < -1 || absent_block >= kProbeBlocks)
        return fail(SB_ERR_INVALID, "absent_block must be -1 or a block index below 4");
    if (poll_limit < 1 || poll_limit > (1u << 22))
        return fail(SB_ERR_INVALID, "poll_limit must be in [1, 2^22]");
    SB_CHECK(cudaSetDevice(b->device));
    SB_CHECK(launch_barrier_probe(b->f.self, kProbeBlocks, absent_block, poll_limit, b->stream));
    b->launches += 1;
    SB_CHECK(cudaStreamSynchronize(b->stream));
    return SB_OK;
}

int sb_reset_stats(sb_bubble* b) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    SB_CHECK(cudaSetDevice(b->device));
    // solver_nonconverged and solver_resid_max are adjacent: one memset
    static_assert(offsetof(SbDevStats, solver_resid_max) ==
                      offsetof(SbDevStats, solver_nonconverged) + sizeof(long long),
                  "reset range");
    SB_CHECK(cudaMemsetAsync(&b->f.stats->solver_nonconverged, 0,
                             sizeof(long long) + sizeof(double), b->stream));
    SB_CHECK(cudaStreamSynchronize(b->stream));
    return SB_OK;
}

int sb_get_stats(sb_bubble* b, sb_stats* out) {
    if (!b || !out) return fail(SB_ERR_INVALID, "null argument");
    SB_CHECK(cudaSetDevice(b->device));
    SbDevStats st;
    SB_CHECK(cudaMemcpyAsync(&st, b->f.stats, sizeof(st), cudaMemcpyDeviceToHost, b->stream));
    SB_CHECK(cudaStreamSynchronize(b->stream));
    std::memset(out, 0, sizeof(*out));
    float d;
    std::memcpy(&d, &st.distortion_bits, 4);
    out->distortion = d;
    out->reinit = st.reinit;
    out->solver_iters = st.solver_iters;
    out->solver_rel_resid = st.solver_rel_resid;
    out->solver_converged = st.solver_converged;
    out->broken_cells = st.broken_cells;
    out->steps = st.steps_done;
    out->reinits = st.reinit_total;
    out->solves = st.solves;
    out->solver_nonconverged = st.solver_nonconverged;
    out->solver_rel_resid_max = st.solver_resid_max;
    out->launches = b->launches;
    out->mass_eta = st.mass_eta;
    out->mass_gamma = st.mass_gamma;
    out->solver_precond_used = st.solver_neumann ? 2 : 1;
    if (st.wait_faults)
        return fail(SB_ERR_CUDA, "a bounded wait inside a kernel (grid barrier or shared-memory copy) gave up; the bubble halts");
    return SB_OK;
}

int sb_update_mass(sb_bubble* b) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    SB_CHECK(cudaSetDevice(b->device));
    SB_CHECK(launch_mass(b->g, b->ph, b->f, b->storage, b->stream));
    b->launches += 1;
    SB_CHECK(cudaStreamSynchronize(b->stream));
    return SB_OK;
}

int sb_write_thickness_exr(sb_bubble* b, const char* path, int* broken) {
    if (!b || !path) return fail(SB_ERR_INVALID, "null argument");
    SB_CHECK(cudaSetDevice(b->device));
    const size_t N = (size_t)b->g.N;
    std::vector<float> eta(N);
    const float* src = reinterpret_cast<const float*>(b->f.eta);
    if (b->storage != kStoreF32) {
        int rc = load_to_staging(b, b->f.eta, N);
        if (rc != SB_OK) return rc;
        src = staging(b);
    }
    SB_CHECK(cudaMemcpyAsync(eta.data(), src, N * 4, cudaMemcpyDeviceToHost, b->stream));
    SB_CHECK(cudaStreamSynchronize(b->stream));
    // Solver::write_thickness_img (kernel/solver.cu:541-593)
    const double ratio = 2e5;
    bool br = true;
    std::vector<float> img(N);
    for (size_t c = 0; c < N; ++c) {
        const double D = eta[c];
        if (D > 0) br = false;
        img[c] = (float)(D * b->params.H * ratio);
    }
    if (broken) *broken = br ? 1 : 0;
    if (!write_exr_gray3(path, b->g.nP, b->g.nT, img.data()))
        return fail(SB_ERR_IO, std::string("cannot write ") + path);
    return SB_OK;
}

int sb_write_velocity_exr(sb_bubble* b, const char* path) {
    if (!b || !path) return fail(SB_ERR_INVALID, "null argument");
    const int nT = b->g.nT, nP = b->g.nP;
    std::vector<float> uph((size_t)nT * nP), uth((size_t)(nT - 1) * nP);
    int rc = sb_download_field_f32(b, SB_UPHI, uph.data(), uph.size());
    if (rc == SB_OK) rc = sb_download_field_f32(b, SB_UTHETA, uth.data(), uth.size());
    if (rc != SB_OK) return rc;
    SB_CHECK(cudaStreamSynchronize(b->stream));
    // Solver::write_velocity_image (kernel/solver.cu:388-497): face velocities
    // averaged to the cell centres; at the poles the missing face is
    // extrapolated from the nearest face row and its opposite meridian
    const size_t N = (size_t)nT * nP;
    std::vector<float> R(N), G(N), B(N, 0.5f);
    auto vt = [&](int t, int p) { return (double)uth[(size_t)t * nP + p]; };
    for (int j = 0; j < nT; ++j)
        for (int i = 0; i < nP; ++i) {
            const int opp = (i + nP / 2) % nP;
            const double uW = uph[(size_t)j * nP + i];
            const double uE = uph[(size_t)j * nP + (i + 1) % nP];
            const double vN = j != 0 ? vt(j - 1, i) : 0.75 * vt(j, i) - 0.25 * vt(j, opp);
            const double vS = j != nT - 1 ? vt(j, i) : 0.75 * vt(j - 1, i) - 0.25 * vt(j - 1, opp);
            const double u = 0.5 * (uW + uE), v = 0.5 * (vN + vS);
            R[(size_t)j * nP + i] = (float)(u / 2 + 0.5);
            G[(size_t)j * nP + i] = (float)(v / 2 + 0.5);
        }
    if (!write_exr_bgr(path, nP, nT, B.data(), G.data(), R.data()))
        return fail(SB_ERR_IO, std::string("cannot write ") + path);
    return SB_OK;
}

int sb_write_concentration_exr(sb_bubble* b, const char* path) {
    if (!b || !path) return fail(SB_ERR_INVALID, "null argument");
    const size_t N = (size_t)b->g.N;
    std::vector<float> gam(N);
    int rc = sb_download_field_f32(b, SB_GAMMA, gam.data(), N);
    if (rc != SB_OK) return rc;
    SB_CHECK(cudaStreamSynchronize(b->stream));
    // Solver::write_concentration_image (kernel/solver.cu:500-538)
    std::vector<float> img(N);
    for (size_t c = 0; c < N; ++c) img[c] = (float)(((double)gam[c] - 0.9) / 0.2);
    if (!write_exr_gray3(path, b->g.nP, b->g.nT, img.data()))
        return fail(SB_ERR_IO, std::string("cannot write ") + path);
    return SB_OK;
}

namespace {

// The frame loop's halt switch (SbBubbleDesc::halt_on_fail / halted) on the
// bubble's device descriptor, in stream order.
int set_halt_on_fail(sb_bubble* b, int on) {
    static const int zero_on[2][2] = {{0, 0}, {0, 1}};  // (halted, halt_on_fail)
    SB_CHECK(cudaMemcpyAsync(&b->f.self->halted, zero_on[on ? 1 : 0], 2 * sizeof(int),
                             cudaMemcpyHostToDevice, b->stream));
    SB_CHECK(cudaStreamSynchronize(b->stream));
    return SB_OK;
}

// After a halted run: the host mirrors of the map parity and the step count
// follow the device, whose kernels skipped the steps after the failed one.
int resync_after_halt(sb_bubble* b) {
    int cur = 0;
    SbDevStats st;
    SB_CHECK(cudaMemcpy(&cur, &b->f.self->cur, sizeof(int), cudaMemcpyDeviceToHost));
    SB_CHECK(cudaMemcpy(&st, b->f.stats, sizeof(st), cudaMemcpyDeviceToHost));
    b->cur = cur;
    b->steps = st.steps_done;
    return SB_OK;
}

}  // namespace

int sb_run(sb_bubble* b, const char* out_dir, int frames) {
    if (!b) return fail(SB_ERR_INVALID, "null handle");
    const sb_params& p = b->params;
    if (frames <= 0) frames = p.frames;
    std::string dir = out_dir ? out_dir : "";
    if (!dir.empty() && dir.back() != '/') dir.push_back('/');
    auto frame_path = [&](const char* kind, int i) {
        char name[32];
        std::snprintf(name, sizeof(name), "%s%04d.exr", kind, i);
        return dir + name;
    };
    // frame i: thickness (WRITE_THICKNESS_DATA), and velocity and surfactant
    // when asked (WRITE_VELOCITY_DATA / WRITE_CONCENTRATION_DATA,
    // kernel/bubble.cu:2643-2651, 2686-2694)
    int broken = 0;
    auto write_frame = [&](int i) {
        int r = sb_write_thickness_exr(b, frame_path("frame", i).c_str(), &broken);
        if (r == SB_OK && p.write_velocity_frames)
            r = sb_write_velocity_exr(b, frame_path("vel", i).c_str());
        if (r == SB_OK && p.write_concentration_frames)
            r = sb_write_concentration_exr(b, frame_path("con", i).c_str());
        return r;
    };
    SB_CHECK(cudaSetDevice(b->device));
    int rc = SB_OK;
    if (out_dir && (rc = write_frame(0)) != SB_OK) return rc;
    // A solve that misses its tolerance ends the run after that step, as the
    // reference's AmgX failure sets `broken`, which the step loop tests
    // before every step (kernel/bubble.cu:1500-1507, 2669-2682): the step's
    // k_flip halts the bubble on the device, the kernels of the frame's
    // remaining steps leave it untouched, and the frame's end reports it.
    if ((rc = set_halt_on_fail(b, 1)) != SB_OK) return rc;
    auto finish = [&](int r) {
        const int r2 = set_halt_on_fail(b, 0);
        return r != SB_OK ? r : r2;
    };
    // Bubble::run frame loop (kernel/bubble.cu:2656-2696); U = 1
    const double dt_ = p.dt, DT = p.DT;
    double T = 0.0;
    for (int i = 1; i < frames && !broken; ++i) {
        const double tf = T;
        int n = 0;
        while ((T + dt_) <= i * DT) {
            ++n;
            T += dt_;
        }
        if (n > 0 && (rc = sb_step(b, n, tf, dt_)) != SB_OK) return finish(rc);
        if ((T + 1e-7) < i * DT) {
            if ((rc = sb_step(b, 1, tf, i * DT - T)) != SB_OK) return finish(rc);
        }
        sb_stats st;
        if ((rc = sb_get_stats(b, &st)) != SB_OK) return finish(rc);
        if (!st.solver_converged) {
            if ((rc = resync_after_halt(b)) != SB_OK) return finish(rc);
            return finish(fail(SB_ERR_NOT_CONVERGED, "implicit solve did not converge; the run "
                                                     "stopped after that step"));
        }
        T = i * DT;
        if (out_dir && (rc = write_frame(i)) != SB_OK) return finish(rc);
    }
    if ((rc = finish(SB_OK)) != SB_OK) return rc;
    if (broken) return fail(SB_ERR_BROKEN, "film is broken");
    return SB_OK;
}

int sb_write_exr_gray(const char* path, int width, int height, const float* img) {
    if (!path || !img || width <= 0 || height <= 0) return fail(SB_ERR_INVALID, "bad image");
    if (!write_exr_gray3(path, width, height, img))
        return fail(SB_ERR_IO, std::string("cannot write ") + path);
    return SB_OK;
}

void* sb_stream(sb_bubble* b) { return b ? (void*)b->stream : nullptr; }

const char* sb_last_error(void) { return g_err.c_str(); }

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: many bubbles stepped together, one launch per stage.
// ---------------------------------------------------------------------------

struct sb_batch {
    std::vector<sb_bubble*> m;
    std::vector<char> retired;  // members taken out by sb_batch_retire
    int device = 0;
    cudaStream_t stream = nullptr;
    char* arena = nullptr;
    SbStepPlan plan{};  // the members as one set: their own descriptors, tiles, solve set
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev[STAGE_COUNT + 1] = {};
    long long steps = 0;
};

namespace {

// Step scalars of every member for frame time t[k] (members may be at
// different points of their runs); rewritten only when a member's (t, dt)
// changes.  Each member's last (t, dt) mirrors its device copy.
int batch_set_params_each(sb_batch* B, const double* t, double dt) {
    bool same = true;
    for (size_t k = 0; k < B->m.size() && same; ++k)
        same = B->m[k]->last_t == t[k] && B->m[k]->last_dt == dt;
    if (same) return SB_OK;
    SB_CHECK(cudaStreamSynchronize(B->stream));  // pinned slots may be in flight
    for (size_t k = 0; k < B->m.size(); ++k) {
        int rc = write_step_params(B->m[k], t[k], dt, B->stream);
        if (rc != SB_OK) return rc;
    }
    return SB_OK;
}

int batch_set_params(sb_batch* B, double t, double dt) {
    std::vector<double> ts(B->m.size(), t);
    return batch_set_params_each(B, ts.data(), dt);
}

// The host mirrors (map parity, step and launch counts) of the members the
// steps moved; a retired member's device state stays as it was.
void batch_advance(sb_batch* B, int n) {
    B->steps += n;
    for (size_t k = 0; k < B->m.size(); ++k)
        if (!B->retired[k]) bubble_advance(B->m[k], n);
}

}  // namespace

extern "C" {

int sb_batch_create(sb_bubble* const* bubbles, int n, sb_batch** out) {
    if (!out || !bubbles || n <= 0) return fail(SB_ERR_INVALID, "bad batch arguments");
    *out = nullptr;
    for (int k = 0; k < n; ++k)
        if (!bubbles[k]) return fail(SB_ERR_INVALID, "batch members must be valid bubbles on one device");
    {
        // a member listed twice would be stepped twice per launch (two sets of
        // blocks on the same fields, its map parity flipped twice)
        std::vector<sb_bubble*> sorted(bubbles, bubbles + n);
        std::sort(sorted.begin(), sorted.end());
        if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
            return fail(SB_ERR_INVALID, "a bubble appears twice in the batch");
    }
    sb_batch* B = new sb_batch();
    B->device = bubbles[0]->device;
    SbStepPlan& P = B->plan;
    P.solver = bubbles[0]->solver;
    P.storage = bubbles[0]->storage;
    P.viscous = bubbles[0]->ph.viscous;
    for (int k = 0; k < n; ++k) {
        sb_bubble* b = bubbles[k];
        if (b->device != B->device) {
            delete B;
            return fail(SB_ERR_INVALID, "batch members must be valid bubbles on one device");
        }
        const SolverConfig& c = b->solver;
        if (c.mode != P.solver.mode || c.max_iter != P.solver.max_iter ||
            c.tol != P.solver.tol || c.precond != P.solver.precond || c.warm != P.solver.warm) {
            delete B;
            return fail(SB_ERR_INVALID, "batch members must share one solver configuration");
        }
        if (b->storage != P.storage) {
            delete B;
            return fail(SB_ERR_INVALID, "batch members must share one field storage");
        }
        if (b->ph.viscous != P.viscous) {
            delete B;
            return fail(SB_ERR_INVALID, "batch members must share the viscous switch");
        }
        B->m.push_back(b);
        B->retired.push_back(0);
        if (b->g.nP > P.maxNP) P.maxNP = b->g.nP;
    }
    // the row list of the solve: every member's theta rows, member by member
    std::vector<int> roff(n + 1, 0);
    unsigned long long weight = 0;
    for (int k = 0; k < n; ++k) {
        const int nT = B->m[k]->g.nT;
        roff[k + 1] = roff[k] + nT;
        weight += (unsigned long long)nT * (2ull * nT + 256ull);
    }
    const int R = roff[n];
    if (n > 1024 || weight >= (1ull << 32)) {
        delete B;
        return fail(SB_ERR_INVALID, "a batch holds at most 1024 members of bounded total size");
    }
    cudaError_t e = cudaSetDevice(B->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = prepare_plan(P);
    if (e != cudaSuccess) {
        int r = cuda_fail(e, "sb_batch_create");
        sb_batch_destroy(B);
        return r;
    }
    // tiles for the three tile sizes
    std::vector<int2> tiles[3];
    for (int s = 0; s < 3; ++s)
        for (int k = 0; k < n; ++k)
            for (int c = 0; c < B->m[k]->g.N; c += kTileSizes[s]) tiles[s].push_back(make_int2(k, c));
    Layout L;
    const size_t o_desc = L.take(sizeof(SbBubbleDesc*) * n);
    size_t o_tiles[3];
    for (int s = 0; s < 3; ++s) o_tiles[s] = L.take(sizeof(int2) * tiles[s].size());
    const size_t o_roff = L.take(sizeof(int) * (n + 1)),
                 o_rec = L.take(sizeof(SbSolveRec) * 2 * n), o_done = L.take(sizeof(int) * n),
                 o_cnt = L.take(sizeof(int) * n),
                 o_acc = L.take(sizeof(unsigned long long) * kSolveAccWords * n),
                 o_bar = L.take(sizeof(unsigned) * kGridBarWords);
    e = cudaMalloc((void**)&B->arena, L.bytes);
    if (e == cudaSuccess) e = cudaMemset(B->arena, 0, L.bytes);
    if (e != cudaSuccess) {
        int r = cuda_fail(e, "sb_batch_create allocation");
        sb_batch_destroy(B);
        return r;
    }
    char* A = B->arena;
    // the members' own descriptors: a member keeps one map parity whether it
    // is stepped alone or here
    std::vector<SbBubbleDesc*> descs(n);
    for (int k = 0; k < n; ++k) descs[k] = B->m[k]->f.self;
    P.descs = (SbBubbleDesc* const*)(A + o_desc);
    P.nb = n;
    for (int s = 0; s < 3; ++s) {
        P.tiles[s] = (const int2*)(A + o_tiles[s]);
        P.ntiles[s] = (int)tiles[s].size();
    }
    for (int st = 0; st < STAGE_COUNT; ++st) P.sel[st] = 1;
    P.one = nullptr;
    SbSolveSet& S = P.set;
    S.descs = P.descs;
    S.nb = n;
    S.R = R;
    S.roff = (const int*)(A + o_roff);
    S.rec = (SbSolveRec*)(A + o_rec);
    S.done_at = (int*)(A + o_done);
    S.cnt = (int*)(A + o_cnt);
    S.acc = (unsigned long long*)(A + o_acc);
    S.bar = (unsigned*)(A + o_bar);
    // members may have work queued on their own streams; a member retired
    // from an earlier batch takes part again
    for (sb_bubble* b : B->m) e = e == cudaSuccess ? cudaStreamSynchronize(b->stream) : e;
    for (sb_bubble* b : B->m)
        if (e == cudaSuccess) e = cudaMemset(&b->f.self->halted, 0, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemcpy((void*)P.descs, descs.data(), sizeof(SbBubbleDesc*) * n, cudaMemcpyHostToDevice);
    for (int s = 0; s < 3 && e == cudaSuccess; ++s)
        e = cudaMemcpy((void*)P.tiles[s], tiles[s].data(), sizeof(int2) * tiles[s].size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy((void*)S.roff, roff.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        int r = cuda_fail(e, "sb_batch_create upload");
        sb_batch_destroy(B);
        return r;
    }
    *out = B;
    return SB_OK;
}

int sb_batch_destroy(sb_batch* B) {
    if (!B) return SB_OK;
    cudaSetDevice(B->device);
    if (B->stream) cudaStreamSynchronize(B->stream);
    if (B->graph) cudaGraphExecDestroy(B->graph);
    for (cudaEvent_t e : B->ev)
        if (e) cudaEventDestroy(e);
    if (B->arena) cudaFree(B->arena);
    if (B->stream) cudaStreamDestroy(B->stream);
    delete B;
    return SB_OK;
}

int sb_batch_step(sb_batch* B, int n_steps, double t_frame, double dt) {
    if (!B) return fail(SB_ERR_INVALID, "null batch");
    if (n_steps < 0 || !(dt > 0)) return fail(SB_ERR_INVALID, "bad step count or dt");
    SB_CHECK(cudaSetDevice(B->device));
    int rc = batch_set_params(B, t_frame, dt);
    if (rc != SB_OK) return rc;
    if (n_steps > 0 && !B->graph && (rc = capture_plan(B->plan, B->stream, &B->graph)) != SB_OK)
        return rc;
    for (int s = 0; s < n_steps; ++s) SB_CHECK(cudaGraphLaunch(B->graph, B->stream));
    batch_advance(B, n_steps);
    return SB_OK;
}

int sb_batch_step_each(sb_batch* B, int n_steps, const double* t_frames, double dt) {
    if (!B || !t_frames) return fail(SB_ERR_INVALID, "null argument");
    if (n_steps < 0 || !(dt > 0)) return fail(SB_ERR_INVALID, "bad step count or dt");
    SB_CHECK(cudaSetDevice(B->device));
    int rc = batch_set_params_each(B, t_frames, dt);
    if (rc != SB_OK) return rc;
    if (n_steps > 0 && !B->graph && (rc = capture_plan(B->plan, B->stream, &B->graph)) != SB_OK)
        return rc;
    for (int s = 0; s < n_steps; ++s) SB_CHECK(cudaGraphLaunch(B->graph, B->stream));
    batch_advance(B, n_steps);
    return SB_OK;
}

int sb_batch_step_timed(sb_batch* B, int n_steps, double t_frame, double dt, double* stage_ms) {
    if (!B || !stage_ms) return fail(SB_ERR_INVALID, "null argument");
    if (n_steps < 0 || !(dt > 0)) return fail(SB_ERR_INVALID, "bad step count or dt");
    SB_CHECK(cudaSetDevice(B->device));
    int rc = batch_set_params(B, t_frame, dt);
    if (rc != SB_OK) return rc;
    for (int s = 0; s < n_steps; ++s) {
        if ((rc = timed_plan_step(B->plan, B->stream, B->ev, stage_ms)) != SB_OK) return rc;
        batch_advance(B, 1);
    }
    return SB_OK;
}

int sb_batch_autotune(sb_batch* B, double t_frame, double dt, int* tile_sizes) {
    if (!B) return fail(SB_ERR_INVALID, "null batch");
    if (!(dt > 0)) return fail(SB_ERR_INVALID, "bad dt");
    SB_CHECK(cudaSetDevice(B->device));
    int rc = batch_set_params(B, t_frame, dt);
    if (rc != SB_OK) return rc;
    rc = autotune_plan(B->plan, [&](double* ms) {
        int r = timed_plan_step(B->plan, B->stream, B->ev, ms);
        if (r == SB_OK) batch_advance(B, 1);
        return r;
    }, tile_sizes);
    if (B->graph) {
        cudaGraphExecDestroy(B->graph);
        B->graph = nullptr;
    }
    return rc;
}

int sb_batch_retire(sb_batch* B, int member) {
    if (!B) return fail(SB_ERR_INVALID, "null batch");
    if (member < 0 || member >= (int)B->m.size()) return fail(SB_ERR_INVALID, "no such member");
    SB_CHECK(cudaSetDevice(B->device));
    static const int one = 1;
    SB_CHECK(cudaMemcpyAsync(&B->m[member]->f.self->halted, &one, sizeof(int),
                             cudaMemcpyHostToDevice, B->stream));
    SB_CHECK(cudaStreamSynchronize(B->stream));
    B->retired[member] = 1;
    return SB_OK;
}

int sb_batch_synchronize(sb_batch* B) {
    if (!B) return fail(SB_ERR_INVALID, "null batch");
    SB_CHECK(cudaSetDevice(B->device));
    SB_CHECK(cudaStreamSynchronize(B->stream));
    return SB_OK;
}

void* sb_batch_stream(sb_batch* B) { return B ? (void*)B->stream : nullptr; }

}  // extern "C"
