// FP64 host oracle for the soap-bubble time step -- TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement, function by function, of the reference's default step
// (RiverIntheSky/SoapBubble).  Each function names the reference file:line it
// follows.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use
// it, as the checker and as the timed CPU baseline; the product never does.
//
// Parity UNPINNED against the reference binary: the reference needs AmgX,
// Boost.Filesystem and OpenCV libraries (unbuildable here) and ships no golden
// vectors.  Analytic known-answer tests pin this restatement instead.
//
// strict = 1 mimics the float intrinsics the reference applies to double data
// (floorf on coordinates, sinf/cosf in the assembly, fminf/fmaxf in the
// extremum clamp, powf in van der Waals, float smoothstep in the air flow, the
// float max reduction of the distortion).  strict = 0 is the same algorithm in
// plain FP64.  The reference's -use_fast_math intrinsics (__sinf etc.) cannot be
// reproduced bit for bit on a CPU; strict mode uses the C library's float
// functions on the float-rounded arguments.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Constants (include/header.cuh:20-22, 76-83, 93)
// ---------------------------------------------------------------------------
constexpr double kPi = 3.14159265358979323846;
constexpr double kHalfPi = 1.57079632679489661923;
constexpr double kGasR = 8.3144598;
constexpr double kSigmaA = 0.07275;
constexpr double kRho = 1e3;
constexpr double kG = 9.8;
constexpr double kRhoA = 1.184;
constexpr double kNuA = 1.562e-5;
constexpr double kNu = 1.25e-4;   // soap solution kinematic viscosity
constexpr double kEvaporation = -0.00000003;
constexpr double kThresh = 0.0;   // bubble.cu:27
constexpr double kEps = 1e-7;     // bubble.cu:28

struct d2 { double x, y; };       // (theta, phi) in grid units
struct d3 { double x, y, z; };

inline d2 operator+(d2 a, d2 b) { return {a.x + b.x, a.y + b.y}; }
inline d2 operator-(d2 a, d2 b) { return {a.x - b.x, a.y - b.y}; }
inline d2 operator*(d2 a, double s) { return {a.x * s, a.y * s}; }
inline d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline d3 operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline d3 operator*(double s, d3 a) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double length(d3 v) { return std::sqrt(dot(v, v)); }
inline d3 cross(d3 a, d3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// include/utils.h:83-86: v * rsqrt(dot(v,v)); a zero vector gives NaN.
inline d3 normalize(d3 v) { double inv = 1.0 / std::sqrt(dot(v, v)); return v * inv; }
// include/utils.h:102-104 (CUDA min/max on doubles ignore a NaN operand).
inline double safe_acos(double x) { return std::acos(std::fmax(-1.0, std::fmin(1.0, x))); }
// include/utils.h:106-110
inline double clampd(double v, double lo, double hi) { return (v < lo) ? lo : (hi < v) ? hi : v; }

struct Ctx {
    size_t nTheta, nPhi;
    double gridLen, invGridLen;
    int strict;
    std::atomic<long>* oob;
};

Ctx make_ctx(const sb_oracle_params* p, std::atomic<long>* oob) {
    Ctx c;
    c.nTheta = (size_t)p->nTheta;
    c.nPhi = (size_t)p->nPhi;
    // Bubble uploads gridLen = M_PI / nTheta (kernel/bubble.cu:2579, 2615).
    c.gridLen = kPi / (double)p->nTheta;
    c.invGridLen = (double)p->nTheta / kPi;
    c.strict = p->strict;
    c.oob = oob;
    return c;
}

inline size_t umod(long long a, size_t n) { return (size_t)a % n; }  // int % size_t

// floorf() applied to a double coordinate (bubble.cu:183-184 and the three
// other samplers).  In strict mode the float rounding can move an index one
// row past the last one the branch logic expects; the reference then reads
// past its buffer, so the exact floor is used there and the event counted.
inline int index_floor(const Ctx& c, double v, int maxIdx) {
    int e = (int)std::floor(v);
    if (!c.strict) return e;
    int s = (int)std::floor((float)v);
    if (s > maxIdx) { if (c.oob) (*c.oob)++; return e; }
    return s;
}

// bubble.cu:116-137
bool validateCoord(const Ctx& c, d2& Id) {
    bool ret = false;
    if (Id.x >= (double)c.nTheta) {
        Id.x = (double)c.nPhi - Id.x;
        Id.y += (double)c.nTheta;
        ret = !ret;
    }
    if (Id.x < 0) {
        Id.x = -Id.x;
        Id.y += (double)c.nTheta;
        ret = !ret;
    }
    Id.y = std::fmod(Id.y + (double)c.nPhi, (double)c.nPhi);
    return ret;
}

// bubble.cu:140-147 (int % size_t: unsigned wrap, exact for power-of-two nPhi)
void validateId(const Ctx& c, int& ix, int& iy) {
    ix = (int)((size_t)(long long)ix % c.nPhi);
    if ((size_t)ix >= c.nTheta) {
        ix = (int)(c.nPhi - 1 - (size_t)ix);
        iy = (int)((size_t)(long long)iy + c.nTheta);
    }
    iy = (int)((size_t)(long long)iy % c.nPhi);
}

// bubble.cu:153-160
inline double bubbleLerp(double from, double to, double alpha) {
    if (std::isnan(from)) return to;
    if (std::isnan(to)) return from;
    return (1.0 - alpha) * from + alpha * to;
}

// bubble.cu:178-240
double sampleVPhi(const Ctx& c, const double* input, d2 rawId, size_t pitch) {
    d2 Id = rawId - d2{0.5, -0.5};
    bool isFlippedPole = validateCoord(c, Id);
    int phiIndex = index_floor(c, Id.y, 1 << 30);
    int thetaIndex = index_floor(c, Id.x, isFlippedPole ? (int)c.nTheta : (int)c.nTheta - 1);
    double alphaPhi = Id.y - (double)phiIndex;
    double alphaTheta = Id.x - (double)thetaIndex;
    const size_t nP = c.nPhi;

    if (thetaIndex == 0 && isFlippedPole) {
        size_t phiLower = umod(phiIndex, nP);
        size_t phiHigher = (phiLower + 1) % nP;
        double higherBelt = -bubbleLerp(input[phiLower + pitch * thetaIndex],
                                        input[phiHigher + pitch * thetaIndex], alphaPhi);
        phiLower = umod((long long)phiIndex + (long long)(nP / 2), nP);
        phiHigher = (phiLower + 1) % nP;
        double lowerBelt = bubbleLerp(input[phiLower + pitch * thetaIndex],
                                      input[phiHigher + pitch * thetaIndex], alphaPhi);
        return bubbleLerp(lowerBelt, higherBelt, alphaTheta);
    }
    if (isFlippedPole) thetaIndex -= 1;
    if ((size_t)(long long)thetaIndex == c.nTheta - 1) {
        size_t phiLower = umod(phiIndex, nP);
        size_t phiHigher = (phiLower + 1) % nP;
        double lowerBelt = bubbleLerp(input[phiLower + pitch * thetaIndex],
                                      input[phiHigher + pitch * thetaIndex], alphaPhi);
        phiLower = umod((long long)phiIndex + (long long)(nP / 2), nP);
        phiHigher = (phiLower + 1) % nP;
        double higherBelt = -bubbleLerp(input[phiLower + pitch * thetaIndex],
                                        input[phiHigher + pitch * thetaIndex], alphaPhi);
        double lerped = bubbleLerp(lowerBelt, higherBelt, alphaTheta);
        if (isFlippedPole) lerped = -lerped;
        return lerped;
    }
    size_t phiLower = umod(phiIndex, nP);
    size_t phiHigher = (phiLower + 1) % nP;
    size_t thetaLower = (size_t)thetaIndex;
    size_t thetaHigher = thetaLower + 1;
    double lowerBelt = bubbleLerp(input[phiLower + pitch * thetaLower],
                                  input[phiHigher + pitch * thetaLower], alphaPhi);
    double higherBelt = bubbleLerp(input[phiLower + pitch * thetaHigher],
                                   input[phiHigher + pitch * thetaHigher], alphaPhi);
    double lerped = bubbleLerp(lowerBelt, higherBelt, alphaTheta);
    if (isFlippedPole) lerped = -lerped;
    return lerped;
}

// bubble.cu:247-313
double sampleVTheta(const Ctx& c, const double* input, d2 rawId, size_t pitch) {
    d2 Id = rawId - d2{1.0, 0.0};
    bool isFlippedPole = validateCoord(c, Id);
    int phiIndex = index_floor(c, Id.y, 1 << 30);
    int thetaIndex = index_floor(c, Id.x, isFlippedPole ? (int)c.nTheta : (int)c.nTheta - 2);
    double alphaPhi = Id.y - (double)phiIndex;
    double alphaTheta = Id.x - (double)thetaIndex;
    const double nT = (double)c.nTheta;
    const size_t nP = c.nPhi;

    if ((rawId.x < 0 && rawId.x > -1) || (rawId.x > nT && rawId.x < nT + 1)) {
        thetaIndex -= 1;
        alphaTheta += 1;
    } else if (rawId.x >= nT + 1 || rawId.x <= -1) {
        thetaIndex -= 2;
    }
    // rawId.x == nTheta exactly makes the reference read row nTheta-1 of a
    // (nTheta-1)-row buffer; the pole branch is the geometric value there.
    if (!isFlippedPole && thetaIndex > (int)c.nTheta - 2) {
        if (c.oob) (*c.oob)++;
        thetaIndex = (int)c.nTheta - 2;
    }

    if (thetaIndex == 0 && isFlippedPole && rawId.x > -1) {
        size_t phiLower = umod(phiIndex, nP);
        size_t phiHigher = (phiLower + 1) % nP;
        double higherBelt = -bubbleLerp(input[phiLower + pitch * thetaIndex],
                                        input[phiHigher + pitch * thetaIndex], alphaPhi);
        phiLower = (phiLower + nP / 2) % nP;
        phiHigher = (phiHigher + nP / 2) % nP;
        double lowerBelt = bubbleLerp(input[phiLower + pitch * thetaIndex],
                                      input[phiHigher + pitch * thetaIndex], alphaPhi);
        alphaTheta = 0.5 * alphaTheta;
        return bubbleLerp(lowerBelt, higherBelt, alphaTheta);
    }
    if ((size_t)(long long)thetaIndex == c.nTheta - 2) {
        size_t phiLower = umod(phiIndex, nP);
        size_t phiHigher = (phiLower + 1) % nP;
        double lowerBelt = bubbleLerp(input[phiLower + pitch * thetaIndex],
                                      input[phiHigher + pitch * thetaIndex], alphaPhi);
        phiLower = (phiLower + nP / 2) % nP;
        phiHigher = (phiHigher + nP / 2) % nP;
        double higherBelt = -bubbleLerp(input[phiLower + pitch * thetaIndex],
                                        input[phiHigher + pitch * thetaIndex], alphaPhi);
        alphaTheta = 0.5 * alphaTheta;
        double lerped = bubbleLerp(lowerBelt, higherBelt, alphaTheta);
        if (isFlippedPole) lerped = -lerped;
        return lerped;
    }
    size_t phiLower = umod(phiIndex, nP);
    size_t phiHigher = (phiLower + 1) % nP;
    size_t thetaLower = (size_t)thetaIndex;
    size_t thetaHigher = thetaLower + 1;
    double lowerBelt = bubbleLerp(input[phiLower + pitch * thetaLower],
                                  input[phiHigher + pitch * thetaLower], alphaPhi);
    double higherBelt = bubbleLerp(input[phiLower + pitch * thetaHigher],
                                   input[phiHigher + pitch * thetaHigher], alphaPhi);
    double lerped = bubbleLerp(lowerBelt, higherBelt, alphaTheta);
    if (isFlippedPole) lerped = -lerped;
    return lerped;
}

// bubble.cu:320-376
double sampleCentered(const Ctx& c, const double* input, d2 rawId, size_t pitch) {
    d2 Id = rawId - d2{0.5, 0.0};
    bool isFlippedPole = validateCoord(c, Id);
    int phiIndex = index_floor(c, Id.y, 1 << 30);
    int thetaIndex = index_floor(c, Id.x, isFlippedPole ? (int)c.nTheta : (int)c.nTheta - 1);
    double alphaPhi = Id.y - (double)phiIndex;
    double alphaTheta = Id.x - (double)thetaIndex;
    const size_t nP = c.nPhi;

    if (thetaIndex == 0 && isFlippedPole) {
        size_t phiLower = umod(phiIndex, nP);
        size_t phiHigher = (phiLower + 1) % nP;
        double higherBelt = bubbleLerp(input[phiLower + pitch * thetaIndex],
                                       input[phiHigher + pitch * thetaIndex], alphaPhi);
        phiLower = (phiLower + nP / 2) % nP;
        phiHigher = (phiHigher + nP / 2) % nP;
        double lowerBelt = bubbleLerp(input[phiLower + pitch * thetaIndex],
                                      input[phiHigher + pitch * thetaIndex], alphaPhi);
        return bubbleLerp(lowerBelt, higherBelt, alphaTheta);
    }
    if (isFlippedPole) thetaIndex -= 1;
    if ((size_t)(long long)thetaIndex == c.nTheta - 1) {
        size_t phiLower = umod(phiIndex, nP);
        size_t phiHigher = (phiLower + 1) % nP;
        double lowerBelt = bubbleLerp(input[phiLower + pitch * thetaIndex],
                                      input[phiHigher + pitch * thetaIndex], alphaPhi);
        phiLower = (phiLower + nP / 2) % nP;
        phiHigher = (phiHigher + nP / 2) % nP;
        double higherBelt = bubbleLerp(input[phiLower + pitch * thetaIndex],
                                       input[phiHigher + pitch * thetaIndex], alphaPhi);
        return bubbleLerp(lowerBelt, higherBelt, alphaTheta);
    }
    size_t phiLower = umod(phiIndex, nP);
    size_t phiHigher = (phiLower + 1) % nP;
    size_t thetaLower = (size_t)thetaIndex;
    size_t thetaHigher = thetaLower + 1;
    double lowerBelt = bubbleLerp(input[phiLower + pitch * thetaLower],
                                  input[phiHigher + pitch * thetaLower], alphaPhi);
    double higherBelt = bubbleLerp(input[phiLower + pitch * thetaHigher],
                                   input[phiHigher + pitch * thetaHigher], alphaPhi);
    return bubbleLerp(lowerBelt, higherBelt, alphaTheta);
}

// bubble.cu:416-506 (greatCircle, fReal = double)
d2 traceGreatCircle(const Ctx& c, const double* velTheta, const double* velPhi, double dt,
                    d2 gId, size_t pitch) {
    d2 gCoord = gId * c.gridLen;
    double sinTheta = std::sin(gCoord.x), cosTheta = std::cos(gCoord.x);
    double sinPhi = std::sin(gCoord.y), cosPhi = std::cos(gCoord.y);
    d3 eTheta = {cosTheta * cosPhi, cosTheta * sinPhi, -sinTheta};
    d3 ePhi = {-sinPhi, cosPhi, 0.0};
    double guTheta = sampleVTheta(c, velTheta, gId, pitch);
    double guPhi = sampleVPhi(c, velPhi, gId, pitch);
    d3 u, u_, v_;
    double u_norm, deltaS;
    d3 w_ = {cosPhi * sinTheta, sinPhi * sinTheta, cosTheta};
    u = guTheta * eTheta + guPhi * ePhi;
    u_norm = length(u);
    if (u_norm > 0) { u_ = normalize(u); v_ = cross(w_, u_); } else { return gId; }
    deltaS = -0.5 * u_norm * dt;
    d3 midx = u_ * std::sin(deltaS) + w_ * std::cos(deltaS);
    d2 midCoord = {safe_acos(midx.z), std::atan2(midx.y, midx.x)};
    d2 midId = midCoord * c.invGridLen;
    double muTheta = sampleVTheta(c, velTheta, midId, pitch);
    double muPhi = sampleVPhi(c, velPhi, midId, pitch);
    d3 mu = {muTheta * std::cos(midCoord.x) * std::cos(midCoord.y) - muPhi * std::sin(midCoord.y),
             muTheta * std::cos(midCoord.x) * std::sin(midCoord.y) + muPhi * std::cos(midCoord.y),
             -muTheta * std::sin(midCoord.x)};
    d3 uCircleMid_ = u_ * std::cos(deltaS) - w_ * std::sin(deltaS);
    d3 vCircleMid_ = cross(midx, uCircleMid_);
    double mguTheta = dot(mu, vCircleMid_);
    double mguPhi = dot(mu, uCircleMid_);
    u = mguPhi * u_ + mguTheta * v_;
    u_norm = length(u);
    if (u_norm > 0) { u_ = normalize(u); v_ = cross(w_, u_); } else { return gId; }
    deltaS = -u_norm * dt;
    d3 px = u_ * std::sin(deltaS) + w_ * std::cos(deltaS);
    return d2{safe_acos(px.z), std::atan2(px.y, px.x)} * c.invGridLen;
}

// bubble.cu:512-536
d2 lerpCoords(const Ctx& c, d2 from, d2 to, double alpha) {
    double gridLenD = kPi / (double)c.nTheta;
    double from_theta = from.x * gridLenD, from_phi = from.y * gridLenD;
    double to_theta = to.x * gridLenD, to_phi = to.y * gridLenD;
    d3 from3 = normalize(d3{std::cos(from_phi) * std::sin(from_theta),
                            std::sin(from_phi) * std::sin(from_theta), std::cos(from_theta)});
    d3 to3 = normalize(d3{std::cos(to_phi) * std::sin(to_theta),
                          std::sin(to_phi) * std::sin(to_theta), std::cos(to_theta)});
    d3 k = normalize(cross(from3, to3));
    if (std::isnan(k.x)) return from;
    double span = safe_acos(dot(from3, to3));
    span *= alpha;
    d3 interpolated3 = from3 * std::cos(span) + cross(k, from3) * std::sin(span) +
                       k * dot(k, from3) * (1 - std::cos(span));
    return d2{safe_acos(interpolated3.z), std::atan2(interpolated3.y, interpolated3.x)} *
           (1.0 / gridLenD);
}

// bubble.cu:539-606
d2 sampleMapping(const Ctx& c, const double* map_t, const double* map_p, d2 rawId) {
    d2 Id = rawId - d2{0.5, 0.0};
    bool isFlippedPole = validateCoord(c, Id);
    int phiIndex = index_floor(c, Id.y, 1 << 30);
    int thetaIndex = index_floor(c, Id.x, isFlippedPole ? (int)c.nTheta : (int)c.nTheta - 1);
    double alphaPhi = Id.y - (double)phiIndex;
    double alphaTheta = Id.x - (double)thetaIndex;
    const size_t nP = c.nPhi;
    d2 ll{0, 0}, lr{0, 0}, hl{0, 0}, hr{0, 0};
    if (isFlippedPole) {
        if (thetaIndex == 0) {
            size_t phiLower = umod(phiIndex, nP);
            size_t phiHigher = (phiLower + 1) % nP;
            hl = {map_t[phiLower], map_p[phiLower]};
            hr = {map_t[phiHigher], map_p[phiHigher]};
            phiLower = (phiLower + nP / 2) % nP;
            phiHigher = (phiHigher + nP / 2) % nP;
            ll = {map_t[phiLower], map_p[phiLower]};
            lr = {map_t[phiHigher], map_p[phiHigher]};
        } else {
            thetaIndex -= 1;
        }
    }
    if ((size_t)(long long)thetaIndex == c.nTheta - 1) {
        size_t phiLower = umod(phiIndex, nP);
        size_t phiHigher = (phiLower + 1) % nP;
        size_t r = nP * (size_t)thetaIndex;
        ll = {map_t[phiLower + r], map_p[phiLower + r]};
        lr = {map_t[phiHigher + r], map_p[phiHigher + r]};
        phiLower = (phiLower + nP / 2) % nP;
        phiHigher = (phiHigher + nP / 2) % nP;
        hl = {map_t[phiLower + r], map_p[phiLower + r]};
        hr = {map_t[phiHigher + r], map_p[phiHigher + r]};
    } else if (thetaIndex != 0 || (thetaIndex == 0 && !isFlippedPole)) {
        size_t phiLower = umod(phiIndex, nP);
        size_t phiHigher = (phiLower + 1) % nP;
        size_t rl = nP * (size_t)thetaIndex, rh = rl + nP;
        ll = {map_t[phiLower + rl], map_p[phiLower + rl]};
        lr = {map_t[phiHigher + rl], map_p[phiHigher + rl]};
        hl = {map_t[phiLower + rh], map_p[phiLower + rh]};
        hr = {map_t[phiHigher + rh], map_p[phiHigher + rh]};
    }
    return lerpCoords(c, lerpCoords(c, ll, lr, alphaPhi), lerpCoords(c, hl, hr, alphaPhi),
                      alphaTheta);
}

// bubble.cu:60-79
double dist(const Ctx& c, d2 Id1, d2 Id2) {
    Id1 = Id1 * c.gridLen;
    Id2 = Id2 * c.gridLen;
    d3 a = normalize(d3{std::cos(Id1.y) * std::sin(Id1.x), std::sin(Id1.y) * std::sin(Id1.x),
                        std::cos(Id1.x)});
    d3 b = normalize(d3{std::cos(Id2.y) * std::sin(Id2.x), std::sin(Id2.y) * std::sin(Id2.x),
                        std::cos(Id2.x)});
    return c.invGridLen * safe_acos(dot(a, b));
}

// helper_math.h:1152-1155, 1432-1436 (float), or the same formula in double.
double smoothstep(int strict, double a, double b, double x) {
    if (strict) {
        float fa = (float)a, fb = (float)b, fx = (float)x;
        float y = std::fmax(0.0f, std::fmin((fx - fa) / (fb - fa), 1.0f));
        return (double)(y * y * (3.0f - (2.0f * y)));
    }
    double y = std::fmax(0.0, std::fmin((x - a) / (b - a), 1.0));
    return y * y * (3.0 - 2.0 * y);
}

const double kW[5] = {0.125, 0.125, 0.125, 0.125, 0.5};
const d2 kDir[5] = {{-0.25, -0.25}, {0.25, -0.25}, {-0.25, 0.25}, {0.25, 0.25}, {0.0, 0.0}};

int nthreads_of(const sb_oracle_params* p) {
#ifdef _OPENMP
    return p->nthreads > 0 ? p->nthreads : omp_get_max_threads();
#else
    (void)p;
    return 1;
#endif
}

#define CELL_LOOP(NT_ROWS, ...)                                             \
    _Pragma("omp parallel for schedule(static) num_threads(nth)")            \
    for (long long cell = 0; cell < (long long)(NT_ROWS) * (long long)nP; ++cell) { \
        const int thetaId = (int)(cell / (long long)nP);                     \
        const int phiId = (int)(cell % (long long)nP);                       \
        (void)thetaId; (void)phiId;                                          \
        __VA_ARGS__                                                          \
    }

// kernel/solver.cu:12-22
void initMapping(int nTheta, int nPhi, double* map_t, double* map_p) {
    for (int t = 0; t < nTheta; ++t)
        for (int f = 0; f < nPhi; ++f) {
            map_t[(size_t)t * nPhi + f] = (double)t + 0.5;
            map_p[(size_t)t * nPhi + f] = (double)f + 0.0;
        }
}

// bubble.cu:609-633
void updateMappingKernel(const sb_oracle_params* p, const Ctx& c, const double* velTheta,
                         const double* velPhi, double dt, const double* map_t,
                         const double* map_p, double* tmp_t, double* tmp_p) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    CELL_LOOP(p->nTheta, {
        d2 pos = d2{(double)thetaId, (double)phiId} + d2{0.5, 0.0};
        d2 back_pos = traceGreatCircle(c, velTheta, velPhi, dt, pos, (size_t)nP);
        d2 sampledId = sampleMapping(c, map_t, map_p, back_pos);
        validateCoord(c, sampledId);
        tmp_p[cell] = sampledId.y;
        tmp_t[cell] = sampledId.x;
    })
}

// Shared body of advectionVSpherePhiKernel (bubble.cu:639-768) and
// advectionVSphereThetaKernel (bubble.cu:775-904): great-circle backtrace
// with parallel transport of the sampled velocity; with RUNGE_KUTTA (rk2) the
// direction is corrected at the half step first (bubble.cu:689-730).
double advectVelocity(const Ctx& c, const double* velPhiInput, const double* velThetaInput,
                      double dt, d2 gId, double guTheta, double guPhi, bool outPhi,
                      bool rk2) {
    d2 gCoord = gId * c.gridLen;
    double sinTheta = std::sin(gCoord.x), cosTheta = std::cos(gCoord.x);
    double sinPhi = std::sin(gCoord.y), cosPhi = std::cos(gCoord.y);
    const size_t pitch = c.nPhi;
    d3 eTheta = {cosTheta * cosPhi, cosTheta * sinPhi, -sinTheta};
    d3 ePhi = {-sinPhi, cosPhi, 0.0};
    d3 u, u_, v_;
    double u_norm, deltaS;
    d3 w_ = {cosPhi * sinTheta, sinPhi * sinTheta, cosTheta};
    u = guTheta * eTheta + guPhi * ePhi;
    u_norm = length(u);
    if (u_norm > 0) { u_ = normalize(u); v_ = cross(w_, u_); } else { return u_norm; }
    if (rk2) {
        deltaS = -0.5 * u_norm * dt;
        d3 midx = u_ * std::sin(deltaS) + w_ * std::cos(deltaS);
        d2 midCoord = {safe_acos(midx.z), std::atan2(midx.y, midx.x)};
        d2 midId = midCoord * c.invGridLen;
        double muTheta = sampleVTheta(c, velThetaInput, midId, pitch);
        double muPhi = sampleVPhi(c, velPhiInput, midId, pitch);
        d3 mu = {muTheta * std::cos(midCoord.x) * std::cos(midCoord.y) - muPhi * std::sin(midCoord.y),
                 muTheta * std::cos(midCoord.x) * std::sin(midCoord.y) + muPhi * std::cos(midCoord.y),
                 -muTheta * std::sin(midCoord.x)};
        d3 uCircleMid_ = u_ * std::cos(deltaS) - w_ * std::sin(deltaS);
        d3 vCircleMid_ = cross(midx, uCircleMid_);
        double mguTheta = dot(mu, vCircleMid_);
        double mguPhi = dot(mu, uCircleMid_);
        u = mguPhi * u_ + mguTheta * v_;
        u_norm = length(u);
        if (u_norm > 0) { u_ = normalize(u); v_ = cross(w_, u_); } else { return u_norm; }
    }
    deltaS = -u_norm * dt;
    d3 px = u_ * std::sin(deltaS) + w_ * std::cos(deltaS);
    d2 pCoord = {safe_acos(px.z), std::atan2(px.y, px.x)};
    d2 pId = pCoord * c.invGridLen;
    double puTheta = sampleVTheta(c, velThetaInput, pId, pitch);
    double puPhi = sampleVPhi(c, velPhiInput, pId, pitch);
    d3 pu = {puTheta * std::cos(pCoord.x) * std::cos(pCoord.y) - puPhi * std::sin(pCoord.y),
             puTheta * std::cos(pCoord.x) * std::sin(pCoord.y) + puPhi * std::cos(pCoord.y),
             -puTheta * std::sin(pCoord.x)};
    d3 uCircleP_ = u_ * std::cos(deltaS) - w_ * std::sin(deltaS);
    d3 vCircleP_ = cross(px, uCircleP_);
    puTheta = dot(pu, vCircleP_);
    puPhi = dot(pu, uCircleP_);
    pu = puPhi * u_ + puTheta * v_;
    return outPhi ? dot(pu, ePhi) : dot(pu, eTheta);
}

// bubble.cu:967-1013
void advectionCenteredBimocq(const sb_oracle_params* p, const Ctx& c, double* out,
                             const double* in, const double* init, const double* delta,
                             const double* initLast, const double* deltaLast,
                             const double* bwd_t, const double* bwd_p,
                             const double* bwd_tprev, const double* bwd_pprev) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    const double blend = p->blend;
    const size_t pitch = (size_t)nP;
    CELL_LOOP(p->nTheta, {
        d2 gId = d2{(double)thetaId, (double)phiId} + d2{0.5, 0.0};
        if (in[cell] == kThresh) {
            out[cell] = kThresh;
        } else {
            double attrib = 0.0;
            for (int i = 0; i < 5; i++) {
                d2 posId = gId + kDir[i];
                d2 initPosId = sampleMapping(c, bwd_t, bwd_p, posId);
                d2 lastPosId = sampleMapping(c, bwd_tprev, bwd_pprev, initPosId);
                attrib += (1.0 - blend) * kW[i] *
                          (sampleCentered(c, initLast, lastPosId, pitch) +
                           sampleCentered(c, delta, initPosId, pitch) +
                           sampleCentered(c, deltaLast, lastPosId, pitch));
                attrib += blend * kW[i] *
                          (sampleCentered(c, init, initPosId, pitch) +
                           sampleCentered(c, delta, initPosId, pitch));
            }
            out[cell] = std::fmax(kThresh, attrib);
        }
    })
}

// bubble.cu:2301-2339 (airFlowU) and 2342-2380 (airFlowV).  The corridor term
// depends on the face position and on t = currentTimeGlobal.
double airCorridor(const sb_oracle_params* p, double gTheta, double gPhi, bool phiComponent) {
    double sinTheta = std::sin(gTheta), cosTheta = std::cos(gTheta);
    double sinPhi = std::sin(gPhi), cosPhi = std::cos(gPhi);
    double angle = kPi / 2.;
    d3 wind = normalize(d3{0., std::cos(angle), std::sin(angle)});
    d3 position = {1., 0, 0};
    d3 normal = normalize(cross(position, wind));
    d3 currentPosition = {sinTheta * cosPhi, sinTheta * sinPhi, cosTheta};
    double beta = safe_acos(dot(normal, currentPosition));
    d3 projected = normalize(currentPosition - dot(normal, currentPosition) * normal);
    d3 projectedWind = cross(normal, projected);
    double s = 0.5 * std::sin(beta) / p->U * p->radius;
    d3 Air = (s * projectedWind) * (1. - smoothstep(p->strict, 0.2, 0.4, std::fabs(beta - kHalfPi))) *
             (3. - std::fabs(p->t - 3.));
    if (phiComponent) {
        d3 ePhi = {-sinPhi, cosPhi, 0.};
        return dot(Air, ePhi);
    }
    d3 eTheta = {cosTheta * cosPhi, cosTheta * sinPhi, -sinTheta};
    return dot(Air, eTheta);
}

void airFlow(const sb_oracle_params* p, const Ctx& c, const double* uair_init,
             const double* vair_init, double* uair, double* vair) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    CELL_LOOP(p->nTheta, {
        double gPhi = ((double)phiId - 0.5) * c.gridLen;
        double gTheta = ((double)thetaId + 0.5) * c.gridLen;
        uair[cell] = uair_init[cell] + airCorridor(p, gTheta, gPhi, true);
        if (std::isnan(uair[cell])) uair[cell] = 0.0;
    })
    CELL_LOOP(p->nTheta - 1, {
        double gTheta = ((double)thetaId + 1.0) * c.gridLen;
        double gPhi = ((double)phiId + 0.0) * c.gridLen;
        vair[cell] = vair_init[cell] + airCorridor(p, gTheta, gPhi, false);
        if (std::isnan(vair[cell])) vair[cell] = 0.0;
    })
    // The assembly's mirrored wind read runs one element past both buffers
    // (bubble.cu:1364-1392); that element is defined here as zero.
    uair[(size_t)p->nTheta * nP] = 0.0;
    vair[(size_t)(p->nTheta - 1) * nP] = 0.0;
}

// bubble.cu:2283-2298
void vanDerWaals(const sb_oracle_params* p, double* W, const double* eta) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    CELL_LOOP(p->nTheta, {
        double Eta = eta[cell];
        double invEta = 1.0 / Eta;
        if (Eta > kThresh) {
            if (p->strict)
                W[cell] = p->W1 * (double)powf((float)invEta, 4.0f) -
                          p->W2 * (double)powf((float)invEta, 2.0f);
            else
                W[cell] = p->W1 * std::pow(invEta, 4.0) - p->W2 * std::pow(invEta, 2.0);
        } else {
            W[cell] = 0.0;
        }
    })
}

inline double ssin(int strict, double x) { return strict ? (double)sinf((float)x) : std::sin(x); }
inline double scos(int strict, double x) { return strict ? (double)cosf((float)x) : std::cos(x); }

// bubble.cu:1301-1473 (airflow, gravity; VISCOUS off)
void concentrationLinearSystem(const sb_oracle_params* p, const Ctx& c, const double* velPhi_a,
                               const double* velTheta_a, double* gamma_a, const double* eta_a,
                               const double* W, const double* uair, const double* vair,
                               const double* fu, const double* fv, double* val, double* rhs) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    const size_t pitch = (size_t)nP;
    const double dt = p->dt, t = p->t;
    CELL_LOOP(p->nTheta, {
        const long long idx = cell, idx5 = 5 * cell;
        double gamma = gamma_a[cell];
        double eta = eta_a[cell];
        if (gamma > (p->gammaMax - kEps) || eta == kThresh) {
            val[idx5] = 0.0; val[idx5 + 1] = 0.0; val[idx5 + 3] = 0.0; val[idx5 + 4] = 0.0;
            val[idx5 + 2] = 1.0;
            rhs[idx] = p->gammaMax;
            gamma_a[cell] = p->gammaMax;
        } else {
            double invDt = 1.0 / dt;
            double gTheta = ((double)thetaId + 0.5) * c.gridLen;
            double halfStep = 0.5 * c.gridLen;
            double sinThetaSouth = ssin(p->strict, gTheta + halfStep);
            double sinThetaNorth = ssin(p->strict, gTheta - halfStep);
            double sinTheta = ssin(p->strict, gTheta);
            double cscTheta = 1. / sinTheta;
            int phiIdEast = (phiId + 1) % (int)nP;
            int phiIdWest = (phiId - 1 + (int)nP) % (int)nP;
            double etaWest = eta_a[(size_t)thetaId * pitch + phiIdWest];
            double etaEast = eta_a[(size_t)thetaId * pitch + phiIdEast];
            double etaNorth = 0.0, etaSouth = 0.0;
            double WMid = W[cell];
            double WWest = W[(size_t)thetaId * pitch + phiIdWest];
            double WEast = W[(size_t)thetaId * pitch + phiIdEast];
            double WNorth = 0.0, WSouth = 0.0;
            double uWest = velPhi_a[(size_t)thetaId * pitch + phiId];
            double uEast = velPhi_a[(size_t)thetaId * pitch + phiIdEast];
            double vNorth = 0.0, vSouth = 0.0;
            // unpitched at(): array[phi + theta * nPhi]; nPhi - 0 reads the next row
            long long oppositePhiId = nP - phiId;
            double uAirWest = 0.5 * (uair[thetaId * nP + phiId] * t / 12.0 +
                                     uair[thetaId * nP + oppositePhiId] * (1 - t / 12.0));
            long long oppositePhiIdEast = nP - phiIdEast;
            double uAirEast = 0.5 * (uair[thetaId * nP + phiIdEast] * t / 12.0 +
                                     uair[thetaId * nP + oppositePhiIdEast] * (1 - t / 12.0));
            double vAirNorth = 0.0, vAirSouth = 0.0;
            if (thetaId != 0) {
                long long thetaNorthIdx = thetaId - 1;
                vAirNorth = 0.5 * (vair[thetaNorthIdx * nP + phiId] * t / 12.0 -
                                   vair[thetaNorthIdx * nP + oppositePhiId] * (1 - t / 12.0));
                vNorth = velTheta_a[thetaNorthIdx * nP + phiId];
                etaNorth = eta_a[thetaNorthIdx * nP + phiId];
                WNorth = W[thetaNorthIdx * nP + phiId];
            } else {
                int opp = (int)(((size_t)phiId + c.nTheta) % c.nPhi);
                etaNorth = eta_a[opp];
                WNorth = W[opp];
            }
            if ((size_t)thetaId != c.nTheta - 1) {
                vAirSouth = 0.5 * (vair[thetaId * nP + phiId] * t / 12.0 -
                                   vair[thetaId * nP + oppositePhiId] * (1 - t / 12.0));
                vSouth = velTheta_a[thetaId * nP + phiId];
                etaSouth = eta_a[(thetaId + 1) * nP + phiId];
                WSouth = W[(thetaId + 1) * nP + phiId];
            } else {
                int opp = (int)(((size_t)phiId + c.nTheta) % c.nPhi);
                etaSouth = eta_a[thetaId * nP + opp];
                WSouth = W[thetaId * nP + opp];
            }
            if (std::isnan(vNorth)) vNorth = 0.0;
            if (std::isnan(vSouth)) vSouth = 0.0;
            if (std::isnan(uWest)) uWest = 0.0;
            if (std::isnan(uEast)) uEast = 0.0;
            double CrDt = p->Cr * dt;
            double MDt = p->M * dt;
            double s2 = c.invGridLen * c.invGridLen;
            double etaUp = (etaNorth + eta) / 2.0;
            val[idx5] = -s2 * sinThetaNorth * MDt / (etaUp + CrDt);
            double etaLeft = (etaWest + eta) / 2.0;
            val[idx5 + 1] = -s2 * cscTheta * MDt / (etaLeft + CrDt);
            double etaRight = (etaEast + eta) / 2.0;
            val[idx5 + 3] = -s2 * cscTheta * MDt / (etaRight + CrDt);
            double etaDown = (etaSouth + eta) / 2.0;
            val[idx5 + 4] = -s2 * sinThetaSouth * MDt / (etaDown + CrDt);
            val[idx5 + 2] = sinTheta * invDt / gamma -
                            (val[idx5] + val[idx5 + 1] + val[idx5 + 3] + val[idx5 + 4]);
            const double Cr = p->Cr;
            double sinThetaDiv = c.invGridLen *
                (uEast * etaRight / (etaRight + Cr * dt) - uWest * etaLeft / (etaLeft + Cr * dt) +
                 (vSouth * sinThetaSouth * etaDown / (etaDown + Cr * dt) -
                  vNorth * sinThetaNorth * etaUp / (etaUp + Cr * dt)));
            sinThetaDiv -= c.invGridLen * c.invGridLen *
                (cscTheta * ((WEast - WMid) * etaRight / (invDt * etaRight + Cr) -
                             (WMid - WWest) * etaLeft / (invDt * etaLeft + Cr)) +
                 sinThetaSouth * (WSouth - WMid) * etaDown / (invDt * etaDown + Cr) -
                 sinThetaNorth * (WMid - WNorth) * etaUp / (invDt * etaUp + Cr));
            sinThetaDiv += c.invGridLen *
                (uAirEast / (etaRight / Cr * invDt + 1.0) - uAirWest / (etaLeft / Cr * invDt + 1.0) +
                 vAirSouth * sinThetaSouth / (etaDown / Cr * invDt + 1.0) -
                 vAirNorth * sinThetaNorth / (etaUp / Cr * invDt + 1.0));
            if (p->viscous) {
                // bubble.cu:1460-1466: the viscous forces (gravity inside fv)
                double fuWest = fu[cell], fuEast = fu[(long long)thetaId * nP + phiIdEast];
                double fvNorth = 0.0, fvSouth = 0.0;
                if (thetaId != 0) fvNorth = fv[(long long)(thetaId - 1) * nP + phiId];
                if ((size_t)thetaId != c.nTheta - 1) fvSouth = fv[cell];
                sinThetaDiv += c.invGridLen *
                    (sinThetaSouth * fvSouth * etaDown / (invDt * etaDown + Cr) -
                     sinThetaNorth * fvNorth * etaUp / (invDt * etaUp + Cr) +
                     fuEast * etaRight / (invDt * etaRight + Cr) -
                     fuWest * etaLeft / (invDt * etaLeft + Cr));
            } else {
                sinThetaDiv += p->gs * c.invGridLen *
                    (sinThetaSouth * sinThetaSouth * etaDown / (invDt * etaDown + Cr) -
                     sinThetaNorth * sinThetaNorth * etaUp / (invDt * etaUp + Cr));
            }
            rhs[idx] = sinTheta * invDt - sinThetaDiv;
        }
    })
    (void)scos;
}

// Column of the k-th entry of row idx (kernel/solver.cu:25-60).
inline long long colOf(long long idx, int k, long long nT, long long nP) {
    switch (k) {
        case 0: return idx < nP ? (idx + nT) % nP : idx - nP;
        case 1: return (idx % nP) == 0 ? idx + nP - 1 : idx - 1;
        case 2: return idx;
        case 3: return (idx % nP) == nP - 1 ? idx - nP + 1 : idx + 1;
        default:
            if (idx >= (nT - 1) * nP + nT) return idx - nT;
            if (idx >= (nT - 1) * nP) return idx + nT;
            return idx + nP;
    }
}

// Replaces AmgX (bubble.cu:1479-1508, init/PCGF_F.json): FP64 Jacobi-PCG on
// the same matrix.  Identity rows (broken cells) are known values; they are
// moved to the right-hand side of their neighbours so that CG runs on the
// remaining symmetric positive definite block.  The solution is that of the
// assembled system.
int solveSystem(const sb_oracle_params* p, const double* val, const double* rhs, double* x,
                double* rel_resid_out) {
    const long long nT = p->nTheta, nP = p->nPhi, N = nT * nP;
    const int nth = nthreads_of(p);
    std::vector<char> fixedRow(N);
    for (long long i = 0; i < N; ++i) {
        fixedRow[i] = (val[5 * i + 1] == 0.0 && val[5 * i + 3] == 0.0 && val[5 * i + 2] == 1.0);
        if (fixedRow[i]) x[i] = rhs[i];
    }
    std::vector<double> b(N), r(N), z(N), pv(N), q(N), dinv(N);
    double bnorm2 = 0.0;
#pragma omp parallel for reduction(+ : bnorm2) num_threads(nth)
    for (long long i = 0; i < N; ++i) bnorm2 += rhs[i] * rhs[i];
    // reduced right-hand side
#pragma omp parallel for num_threads(nth)
    for (long long i = 0; i < N; ++i) {
        if (fixedRow[i]) { b[i] = 0; dinv[i] = 0; continue; }
        double bi = rhs[i];
        for (int k = 0; k < 5; ++k) {
            if (k == 2) continue;
            long long j = colOf(i, k, nT, nP);
            if (fixedRow[j]) bi -= val[5 * i + k] * x[j];
        }
        b[i] = bi;
        dinv[i] = 1.0 / val[5 * i + 2];
    }
    auto spmv = [&](const double* in, double* out) {
#pragma omp parallel for num_threads(nth)
        for (long long i = 0; i < N; ++i) {
            if (fixedRow[i]) { out[i] = 0; continue; }
            double s = val[5 * i + 2] * in[i];
            for (int k = 0; k < 5; ++k) {
                if (k == 2) continue;
                long long j = colOf(i, k, nT, nP);
                if (!fixedRow[j]) s += val[5 * i + k] * in[j];
            }
            out[i] = s;
        }
    };
    // full-system residual norm (identity rows contribute zero)
    auto fullResid = [&]() {
        double s = 0.0;
#pragma omp parallel for reduction(+ : s) num_threads(nth)
        for (long long i = 0; i < N; ++i) {
            double ax = 0.0;
            for (int k = 0; k < 5; ++k) ax += val[5 * i + k] * x[colOf(i, k, nT, nP)];
            double d = rhs[i] - ax;
            s += d * d;
        }
        return std::sqrt(s);
    };
    const double bnorm = std::sqrt(bnorm2) > 0 ? std::sqrt(bnorm2) : 1.0;
    std::vector<double> xr(N);
    for (long long i = 0; i < N; ++i) xr[i] = fixedRow[i] ? 0.0 : x[i];
    spmv(xr.data(), q.data());
    double rz = 0.0;
#pragma omp parallel for reduction(+ : rz) num_threads(nth)
    for (long long i = 0; i < N; ++i) {
        r[i] = b[i] - q[i];
        z[i] = dinv[i] * r[i];
        pv[i] = z[i];
        rz += r[i] * z[i];
    }
    int it = 0;
    double rel = fullResid() / bnorm;
    while (rel > p->solver_tol && it < p->solver_max_iter) {
        spmv(pv.data(), q.data());
        double pq = 0.0;
#pragma omp parallel for reduction(+ : pq) num_threads(nth)
        for (long long i = 0; i < N; ++i) pq += pv[i] * q[i];
        if (!(pq > 0)) break;
        double alpha = rz / pq;
        double rz2 = 0.0, rr = 0.0;
#pragma omp parallel for reduction(+ : rz2, rr) num_threads(nth)
        for (long long i = 0; i < N; ++i) {
            xr[i] += alpha * pv[i];
            r[i] -= alpha * q[i];
            z[i] = dinv[i] * r[i];
            rz2 += r[i] * z[i];
            rr += r[i] * r[i];
        }
        double beta = rz2 / rz;
        rz = rz2;
#pragma omp parallel for num_threads(nth)
        for (long long i = 0; i < N; ++i) pv[i] = z[i] + beta * pv[i];
        ++it;
        if (std::sqrt(rr) / bnorm <= p->solver_tol || (it % 20) == 0) {
            for (long long i = 0; i < N; ++i) if (!fixedRow[i]) x[i] = xr[i];
            rel = fullResid() / bnorm;
        }
    }
    for (long long i = 0; i < N; ++i) if (!fixedRow[i]) x[i] = xr[i];
    rel = fullResid() / bnorm;
    if (rel_resid_out) *rel_resid_out = rel;
    return it;
}

// bubble.cu:1276-1295
void divergenceFromGamma(const sb_oracle_params* p, double* div, double* gammaNext,
                         const double* gammaThis) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    CELL_LOOP(p->nTheta, {
        double gamma_a = gammaThis[cell];
        double gamma = gammaNext[cell];
        if (gamma <= 0.0 || gamma > p->gammaMax - kEps) {
            gammaNext[cell] = p->gammaMax;
            div[cell] = 1.0 / p->dt;
        } else {
            gamma = std::fmin(gamma, 2 * gamma_a);
            div[cell] = (1.0 - gamma / gamma_a) / p->dt;
        }
    })
}

// bubble.cu:1819-1876
void applyForceVelTheta(const sb_oracle_params* p, const Ctx& c, double* out, const double* in,
                        double* delta, const double* thickness, const double* W,
                        const double* conc, const double* vair) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    const double dt = p->dt;
    CELL_LOOP(p->nTheta - 1, {
        double gTheta = ((double)thetaId + 1.0) * c.gridLen;
        long long s = cell + nP;
        double v1 = in[cell];
        double GammaNorth = conc[cell], GammaSouth = conc[s];
        double EtaNorth = thickness[cell], EtaSouth = thickness[s];
        double WNorth = W[cell], WSouth = W[s];
        double invEta = 2. / (EtaNorth + EtaSouth);
        if (std::isinf(invEta)) {
            out[cell] = NAN; delta[cell] = NAN;
        } else {
            double pGpy = c.invGridLen * (GammaSouth - GammaNorth);
            double f1 = -p->M * invEta * pGpy;
            double f2 = p->Cr * invEta * vair[cell];
            double f3 = p->gs * std::sin(gTheta);
            double f4 = c.invGridLen * (WNorth - WSouth);
            out[cell] = (v1 / dt + f1 + f2 + f3 + f4) / (1. / dt + p->Cr * invEta);
            delta[cell] = out[cell] - v1;
        }
    })
}

// bubble.cu:1879-1935
void applyForceVelPhi(const sb_oracle_params* p, const Ctx& c, double* out, const double* in,
                      double* delta, const double* thickness, const double* W,
                      const double* conc, const double* uair) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    const double dt = p->dt;
    CELL_LOOP(p->nTheta, {
        double gTheta = ((double)thetaId + 0.5) * c.gridLen;
        double sinTheta = std::sin(gTheta);
        double cscTheta = 1.0 / sinTheta;
        long long w = (long long)thetaId * nP + (phiId - 1 + nP) % nP;
        double EtaWest = thickness[w], EtaEast = thickness[cell];
        double GammaWest = conc[w], GammaEast = conc[cell];
        double WWest = W[w], WEast = W[cell];
        double u1 = in[cell];
        double invEta = 2. / (EtaWest + EtaEast);
        if (std::isinf(invEta)) {
            out[cell] = NAN; delta[cell] = NAN;
        } else {
            double pGpx = c.invGridLen * (GammaEast - GammaWest) * cscTheta;
            double f1 = -p->M * invEta * pGpx;
            double f2 = p->Cr * invEta * uair[cell];
            double f3 = 0.0;
            double f4 = c.invGridLen * (WWest - WEast) * cscTheta;
            out[cell] = (u1 / dt + (f1 + f2 + f3 + f4)) / (1. / dt + p->Cr * invEta);
            delta[cell] = out[cell] - u1;
        }
    })
}

// ---------------------------------------------------------------------------
// VISCOUS variant (include/header.cuh:98, off in the reference's build):
// viscous stress forces fv (u_theta faces) and fu (u_phi faces) from the
// advected velocities and thickness, fed to the surfactant system's
// right-hand side in place of the gravity term and to the velocity update
// (Solver::bodyforce, bubble.cu:2406-2420, 2454-2476).
// ---------------------------------------------------------------------------

// helper_math.h's clamp is fmaxf(a, fminf(f, b)) with float, int and uint
// overloads only, so the reference's clamp(double, -0.1, 0.1) runs in float
// (strict mode mimics the rounding); a NaN force comes out as 0.1 either way.
inline double clamp_force(int strict, double v) {
    if (strict) return (double)std::fmax(-0.1f, std::fmin((float)v, 0.1f));
    return std::fmax(-0.1, std::fmin(v, 0.1));
}

// bubble.cu:1218-1269 (divergenceKernel): div u at the cell centres.
void divergenceFromVelocity(const sb_oracle_params* p, const Ctx& c, double* div,
                            const double* velPhi, const double* velTheta) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    const long long nT = p->nTheta;
    CELL_LOOP(p->nTheta, {
        double thetaCoord = ((double)thetaId + 0.5) * c.gridLen;
        double halfStep = 0.5 * c.gridLen;
        double uWest = velPhi[cell];
        double uEast = velPhi[(long long)thetaId * nP + (phiId + 1) % nP];
        double vNorth = 0.0, vSouth = 0.0;
        if (thetaId != 0) vNorth = velTheta[(long long)(thetaId - 1) * nP + phiId];
        if (thetaId != nT - 1) vSouth = velTheta[cell];
        double invGridSine = 1.0 / ssin(c.strict, thetaCoord);
        double sinNorth = ssin(c.strict, thetaCoord - halfStep);
        double sinSouth = ssin(c.strict, thetaCoord + halfStep);
        double factor = invGridSine * c.invGridLen;
        double termTheta = factor * (vSouth * sinSouth - vNorth * sinNorth);
        double termPhi = c.invGridLen * (uEast - uWest);
        div[cell] = termTheta + termPhi;
    })
}

// bubble.cu:1512-1643 (computeforcevelthetaKernel): fv on the u_theta faces,
// gravity included.
void computeForceVelTheta(const sb_oracle_params* p, const Ctx& c, double* fv,
                          const double* velTheta, const double* velPhi, const double* thickness,
                          const double* divCentered) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    const long long nT = p->nTheta;
    const double ih = c.invGridLen;
    CELL_LOOP(p->nTheta - 1, {
        double gTheta = ((double)thetaId + 1.0) * c.gridLen;
        long long tN = thetaId, tS = thetaId + 1;
        long long pW = (phiId - 1 + nP) % nP, pE = (phiId + 1) % nP;
        double u0 = velPhi[tN * nP + phiId], u1 = velPhi[tN * nP + pE];
        double u2 = velPhi[tS * nP + phiId], u3 = velPhi[tS * nP + pE];
        double divNorth = divCentered[tN * nP + phiId], divSouth = divCentered[tS * nP + phiId];
        double EtaNorth = thickness[tN * nP + phiId], EtaSouth = thickness[tS * nP + phiId];
        double invEta = 2. / (EtaNorth + EtaSouth);
        if (std::isinf(invEta)) {
            fv[cell] = NAN;
        } else {
            double div = 0.5 * (divNorth + divSouth);
            double uPhi = 0.25 * (u0 + u1 + u2 + u3);
            double d0 = thickness[tN * nP + pW], d1 = thickness[tN * nP + pE];
            double d2 = thickness[tS * nP + pW], d3 = thickness[tS * nP + pE];
            double pDpx = 0.25 * ih * (d1 + d3 - d0 - d2);
            double pDpy = ih * (EtaSouth - EtaNorth);
            double v1 = velTheta[cell];
            double v3 = velTheta[tN * nP + pW], v4 = velTheta[tN * nP + pE];
            long long opp = (phiId + nP / 2) % nP;
            double v0, v2;
            if (thetaId != 0) v0 = velTheta[(tN - 1) * nP + phiId];
            else v0 = 0.5 * (velTheta[cell] - velTheta[tN * nP + opp]);
            if (thetaId != nT - 2) v2 = velTheta[tS * nP + phiId];
            else v2 = 0.5 * (velTheta[cell] - velTheta[tN * nP + opp]);
            double pvpy = 0.5 * ih * (v2 - v0);
            double pvpyNorth = ih * (v1 - v0);
            double pvpySouth = ih * (v2 - v1);
            double pvpx = 0.5 * ih * (v4 - v3);
            double pupy = 0.5 * ih * (u2 + u3 - u0 - u1);
            double pupx = 0.5 * ih * (u1 + u3 - u0 - u2);
            double pupxy = ih * ih * (u0 + u3 - u1 - u2);
            double pvpxx = ih * ih * (v3 + v4 - 2 * v1);
            double sinTheta = std::sin(gTheta);
            double cscTheta = 1. / sinTheta;
            double cosTheta = std::cos(gTheta);
            double cotTheta = cosTheta * cscTheta;
            double sigma11North = 0. + 2. * (pvpyNorth + divNorth);
            double sigma11South = 0. + 2. * (pvpySouth + divSouth);
            double sigma22 = -2. * (pvpy - 2. * div);
            double sigma12 = cscTheta * pvpx + pupy - uPhi * cotTheta;
            double halfStep = 0.5 * c.gridLen;
            double sinNorth = std::sin(gTheta - halfStep);
            double sinSouth = std::sin(gTheta + halfStep);
            double psspy = ih * (sigma11South * sinSouth - sigma11North * sinNorth);
            double pspx = cscTheta * pvpxx + pupxy - cotTheta * pupx;
            double f2 = p->re * cscTheta * invEta * pDpx * sigma12;
            double f4 = p->re * invEta * pDpy * 2 * (div + pvpy);
            double f5 = p->re * cscTheta * (psspy + pspx - cosTheta * sigma22);
            double f7 = p->gs * sinTheta;
            fv[cell] = clamp_force(c.strict, f2 + f5 + f4) + f7;
            if (sinTheta < 0.1) fv[cell] = f7;
        }
    })
}

// bubble.cu:1647-1816 (computeforcevelphiKernel_viscous): fu on the u_phi
// faces.
void computeForceVelPhi(const sb_oracle_params* p, const Ctx& c, double* fu,
                        const double* velPhi, const double* velTheta, const double* thickness,
                        const double* divCentered) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    const long long nT = p->nTheta;
    const double ih = c.invGridLen;
    CELL_LOOP(p->nTheta, {
        double gTheta = ((double)thetaId + 0.5) * c.gridLen;
        long long t0 = thetaId;
        long long pW = (phiId - 1 + nP) % nP;
        long long oppW = (pW + nP / 2) % nP, opp = (phiId + nP / 2) % nP;
        double divWest = divCentered[t0 * nP + pW], divEast = divCentered[cell];
        double EtaWest = thickness[t0 * nP + pW], EtaEast = thickness[cell];
        double v0, v1, v2, v3;
        if (thetaId != 0) {
            v0 = velTheta[(t0 - 1) * nP + pW];
            v1 = velTheta[(t0 - 1) * nP + phiId];
        } else {
            v0 = 0.5 * (velTheta[t0 * nP + pW] - velTheta[t0 * nP + oppW]);
            v1 = 0.5 * (velTheta[t0 * nP + phiId] - velTheta[t0 * nP + opp]);
        }
        if (thetaId != nT - 1) {
            v2 = velTheta[t0 * nP + pW];
            v3 = velTheta[t0 * nP + phiId];
        } else {
            v2 = 0.5 * (velTheta[(t0 - 1) * nP + pW] - velTheta[(t0 - 1) * nP + oppW]);
            v3 = 0.5 * (velTheta[(t0 - 1) * nP + phiId] - velTheta[(t0 - 1) * nP + opp]);
        }
        double invEta = 2. / (EtaWest + EtaEast);
        if (std::isinf(invEta)) {
            fu[cell] = NAN;
        } else {
            double div = 0.5 * (divWest + divEast);
            double pvpx = 0.5 * ih * (v1 + v3 - v0 - v2);
            double pvpyWest = ih * (v2 - v0);
            double pvpyEast = ih * (v3 - v1);
            double pvpy = 0.5 * ih * (v2 + v3 - v0 - v1);
            double pupyNorth = 0.0, pupySouth = 0.0;
            double u1 = velPhi[cell], u3, u4;
            if (thetaId != 0) {
                u3 = velPhi[(t0 - 1) * nP + phiId];
                pupyNorth = ih * (u1 - u3);
            } else {
                u3 = -velPhi[t0 * nP + opp];
            }
            if (thetaId != nT - 1) {
                u4 = velPhi[(t0 + 1) * nP + phiId];
                pupySouth = ih * (u4 - u1);
            } else {
                u4 = -velPhi[t0 * nP + opp];
            }
            double pupy = 0.5 * ih * (u4 - u3);
            double sinTheta = std::sin(gTheta);
            double cscTheta = 1. / sinTheta;
            double cosTheta = std::cos(gTheta);
            double cotTheta = cosTheta * cscTheta;
            double sigma12 = cscTheta * pvpx + pupy - u1 * cotTheta;
            double pDpx = ih * (EtaEast - EtaWest);
            double d0, d1, d2, d3;
            if (thetaId != 0) {
                d0 = thickness[(t0 - 1) * nP + pW];
                d2 = thickness[(t0 - 1) * nP + phiId];
            } else {
                d0 = thickness[t0 * nP + oppW];
                d2 = thickness[t0 * nP + opp];
            }
            if (thetaId != nT - 1) {
                d1 = thickness[(t0 + 1) * nP + pW];
                d3 = thickness[(t0 + 1) * nP + phiId];
            } else {
                d1 = thickness[t0 * nP + oppW];
                d3 = thickness[t0 * nP + opp];
            }
            double pDpy = 0.25 * ih * (d1 + d3 - d0 - d2);
            double halfStep = 0.5 * c.gridLen;
            double sinNorth = ssin(c.strict, gTheta - halfStep);
            double sinSouth = ssin(c.strict, gTheta + halfStep);
            double cosNorth = scos(c.strict, gTheta - halfStep);
            double cosSouth = scos(c.strict, gTheta + halfStep);
            double uNorth = 0.5 * (u3 + u1);
            double uSouth = 0.5 * (u1 + u4);
            if (thetaId == 0) uNorth = 0.5 * (u1 - u3);
            if (thetaId == nT - 1) uSouth = 0.5 * (u1 - u4);
            double psspy = ih * (ih * (v0 + v3 - v1 - v2) + sinSouth * pupySouth -
                                 sinNorth * pupyNorth - cosSouth * uSouth + cosNorth * uNorth);
            double sigma22West = 2 * (2 * divWest - pvpyWest);
            double sigma22East = 2 * (2 * divEast - pvpyEast);
            double pspx = ih * (sigma22East - sigma22West);
            double f2 = p->re * invEta * pDpy * sigma12;
            double f4 = p->re * invEta * cscTheta * pDpx * 2 * (2 * div - pvpy);
            double f5 = p->re * cscTheta * (psspy + pspx + cosTheta * sigma12);
            fu[cell] = clamp_force(c.strict, f2 + f4 + f5);
            if (sinTheta < 0.1) fu[cell] = 0.;
        }
    })
}

// bubble.cu:1940-1983 (applyforcevelthetaKernel_viscous): backward Euler
// with Marangoni, mirrored wind (flat index nPhi - phi) and fv.
void applyForceVelThetaViscous(const sb_oracle_params* p, const Ctx& c, double* out,
                               const double* in, const double* thickness, const double* conc,
                               const double* vair, const double* fv) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    const double dt = p->dt, t = p->t;
    CELL_LOOP(p->nTheta - 1, {
        long long s = cell + nP;
        double GammaNorth = conc[cell], GammaSouth = conc[s];
        double EtaNorth = thickness[cell], EtaSouth = thickness[s];
        double invEta = 2. / (EtaNorth + EtaSouth);
        if (std::isinf(invEta)) {
            out[cell] = NAN;
        } else {
            double v1 = in[cell];
            double pGpy = c.invGridLen * (GammaSouth - GammaNorth);
            double f3 = -p->M * invEta * pGpy;
            long long opp = nP - phiId;
            double vAir = 0.5 * (vair[(long long)thetaId * nP + phiId] * t / 12.0 -
                                 vair[(long long)thetaId * nP + opp] * (1 - t / 12.0));
            double f6 = p->Cr * invEta * vAir;
            out[cell] = (v1 / dt + f3 + f6 + fv[cell]) / (1. / dt + p->Cr * invEta);
        }
    })
}

// bubble.cu:1987-2038 (applyforcevelphiKernel_viscous).
void applyForceVelPhiViscous(const sb_oracle_params* p, const Ctx& c, double* out,
                             const double* in, const double* thickness, const double* conc,
                             const double* uair, const double* fu) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    const double dt = p->dt, t = p->t;
    CELL_LOOP(p->nTheta, {
        double gTheta = ((double)thetaId + 0.5) * c.gridLen;
        long long w = (long long)thetaId * nP + (phiId - 1 + nP) % nP;
        double EtaWest = thickness[w], EtaEast = thickness[cell];
        double GammaWest = conc[w], GammaEast = conc[cell];
        double invEta = 2. / (EtaWest + EtaEast);
        if (std::isinf(invEta)) {
            out[cell] = NAN;
        } else {
            double u1 = in[cell];
            double cscTheta = 1. / std::sin(gTheta);
            double pGpx = c.invGridLen * (GammaEast - GammaWest);
            double f3 = -p->M * invEta * cscTheta * pGpx;
            long long opp = nP - phiId;
            double uAir = 0.5 * (uair[(long long)thetaId * nP + phiId] * t / 12.0 +
                                 uair[(long long)thetaId * nP + opp] * (1 - t / 12.0));
            double f6 = p->Cr * invEta * uAir;
            out[cell] = (u1 / dt + f3 + f6 + fu[cell]) / (1. / dt + p->Cr * invEta);
        }
    })
}

// Solver::bodyforce under VISCOUS (bubble.cu:2406-2420): div u, then fv and
// fu; empty vectors when the variant is off.
void viscousForces(const sb_oracle_params* p, const Ctx& c, const sb_oracle_state* s,
                   std::vector<double>& fu, std::vector<double>& fv) {
    if (!p->viscous) return;
    const size_t N = (size_t)p->nTheta * p->nPhi, Nv = N - (size_t)p->nPhi;
    std::vector<double> div(N);
    fu.assign(N, 0.0);
    fv.assign(Nv, 0.0);
    divergenceFromVelocity(p, c, div.data(), s->uph, s->uth);
    computeForceVelTheta(p, c, fv.data(), s->uth, s->uph, s->eta, div.data());
    computeForceVelPhi(p, c, fu.data(), s->uph, s->uth, s->eta, div.data());
}

// bubble.cu:2041-2063
void applyForceThickness(const sb_oracle_params* p, double* out, const double* in, double* delta,
                         const double* div) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    CELL_LOOP(p->nTheta, {
        double eta = in[cell];
        double f = div[cell];
        double o = eta * (1 - p->dt * f);
        o += p->evapRate * p->dt;
        o = std::fmax(kThresh, o);
        out[cell] = o;
        delta[cell] = o - eta;
    })
}

// bubble.cu:2081-2114
void accumulateChangesCentered(const sb_oracle_params* p, const Ctx& c, double* attribDelta,
                               const double* attribDeltaTemp, const double* fwd_t,
                               const double* fwd_p) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    CELL_LOOP(p->nTheta, {
        d2 gId = d2{(double)thetaId, (double)phiId} + d2{0.5, 0.0};
        for (int i = 0; i < 5; i++) {
            d2 posId = gId + kDir[i];
            d2 initPosId = sampleMapping(c, fwd_t, fwd_p, posId);
            attribDelta[cell] += kW[i] * sampleCentered(c, attribDeltaTemp, initPosId, (size_t)nP);
        }
    })
}

// bubble.cu:1131-1150 + maxAbs (bubble.cu:1019-1043, maxValKernel 85-105)
double estimateDistortion(const sb_oracle_params* p, const Ctx& c, const double* map1_t,
                          const double* map1_p, const double* map2_t, const double* map2_p) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    double best = 0.0;
#pragma omp parallel for reduction(max : best) num_threads(nth)
    for (long long cell = 0; cell < (long long)p->nTheta * nP; ++cell) {
        const int thetaId = (int)(cell / nP), phiId = (int)(cell % nP);
        d2 gId = d2{(double)thetaId, (double)phiId} + d2{0.5, 0.0};
        d2 pos1 = {map1_t[cell], map1_p[cell]};
        d2 pos2 = sampleMapping(c, map2_t, map2_p, pos1);
        double d = dist(c, gId, pos2);
        double a = c.strict ? (double)std::fabs((float)d) : std::fabs(d);
        if (a > best) best = a;
    }
    return best;
}

// bubble.cu:2180-2215
void correctCentered1(const sb_oracle_params* p, const Ctx& c, const double* thicknessCurr,
                      double* thicknessError, const double* thicknessDelta,
                      const double* thicknessInit, const double* gammaCurr, double* gammaError,
                      const double* gammaDelta, const double* gammaInit, const double* fwd_t,
                      const double* fwd_p) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    CELL_LOOP(p->nTheta, {
        double thickness = 0.0, gamma = 0.0;
        d2 gId = d2{(double)thetaId, (double)phiId} + d2{0.5, 0.0};
        for (int i = 0; i < 5; i++) {
            d2 posId = gId + kDir[i];
            d2 initPosId = sampleMapping(c, fwd_t, fwd_p, posId);
            thickness += kW[i] * sampleCentered(c, thicknessCurr, initPosId, (size_t)nP);
            gamma += kW[i] * sampleCentered(c, gammaCurr, initPosId, (size_t)nP);
        }
        thicknessError[cell] = (thickness - thicknessDelta[cell] - thicknessInit[cell]) * 0.5;
        gammaError[cell] = (gamma - gammaDelta[cell] - gammaInit[cell]) * 0.5;
    })
}

// bubble.cu:2218-2280
void correctCentered2(const sb_oracle_params* p, const Ctx& c, double* thicknessOutput,
                      const double* thicknessInput, const double* thicknessError,
                      double* gammaOutput, const double* gammaInput, const double* gammaError,
                      const double* bwd_t, const double* bwd_p) {
    const long long nP = p->nPhi; const int nth = nthreads_of(p);
    auto mn = [&](double a, double b) {
        return c.strict ? (double)std::fmin((float)a, (float)b) : std::fmin(a, b);
    };
    auto mx = [&](double a, double b) {
        return c.strict ? (double)std::fmax((float)a, (float)b) : std::fmax(a, b);
    };
    CELL_LOOP(p->nTheta, {
        d2 gId = d2{(double)thetaId, (double)phiId} + d2{0.5, 0.0};
        for (int i = 0; i < 5; i++) {
            d2 posId = gId + kDir[i];
            d2 sampleId = sampleMapping(c, bwd_t, bwd_p, posId);
            thicknessOutput[cell] -= kW[i] * sampleCentered(c, thicknessError, sampleId, (size_t)nP);
            gammaOutput[cell] -= kW[i] * sampleCentered(c, gammaError, sampleId, (size_t)nP);
        }
        const int range[3] = {-1, 0, 1};
        double minVal = thicknessInput[cell], maxVal = minVal;
        for (int tt : range)
            for (int pp : range) {
                int ix = thetaId + tt, iy = phiId + pp;
                validateId(c, ix, iy);
                double cur = thicknessInput[(size_t)iy + (size_t)ix * (size_t)nP];
                minVal = mn(minVal, cur);
                maxVal = mx(maxVal, cur);
            }
        thicknessOutput[cell] = clampd(thicknessOutput[cell], minVal, maxVal);
        thicknessOutput[cell] = std::fmax(kThresh, thicknessOutput[cell]);
        minVal = gammaInput[cell]; maxVal = minVal;
        for (int tt : range)
            for (int pp : range) {
                int ix = thetaId + tt, iy = phiId + pp;
                validateId(c, ix, iy);
                double cur = gammaInput[(size_t)iy + (size_t)ix * (size_t)nP];
                minVal = mn(minVal, cur);
                maxVal = mx(maxVal, cur);
            }
        gammaOutput[cell] = clampd(gammaOutput[cell], minVal, maxVal);
        gammaOutput[cell] = std::fmax(kThresh, gammaOutput[cell]);
    })
}

}  // namespace

extern "C" {

void sb_oracle_default_params(sb_oracle_params* p, int nTheta, double radius, double H,
                              double Gamma_m, double T, double dt_s, double blend) {
    std::memset(p, 0, sizeof(*p));
    const double U = 1.0;  // Bubble::Bubble forces U = 1 (bubble.cu:2573)
    p->nTheta = nTheta;
    p->nPhi = 2 * nTheta;
    p->radius = radius;
    p->U = U;
    double sigma_r = kGasR * T;
    p->M = Gamma_m * sigma_r / (3 * kRho * H * U * U);
    p->Cr = kRhoA * std::sqrt(kNuA * radius / U) / (kRho * H);
    p->gs = kG * radius / (U * U);
    p->re = kNu / (U * radius);
    p->gammaMax = kSigmaA / sigma_r / Gamma_m;
    p->dt = dt_s * U / radius;
    p->evapRate = kEvaporation * radius / (H * U);
    p->W1 = 0.0;  // epsilon_ = 0 (bubble.cu:2633-2638)
    p->W2 = 0.0;
    p->blend = blend;
    p->t = 0.0;
    p->strict = 0;
    p->force_reinit = -1;
    p->solver_tol = 1e-13;
    p->solver_max_iter = 20000;
    p->nthreads = 0;
}

void sb_oracle_identity_map(int nTheta, int nPhi, double* map_t, double* map_p) {
    initMapping(nTheta, nPhi, map_t, map_p);
}

void sb_oracle_viscous_forces(const sb_oracle_params* p, const double* uth, const double* uph,
                              const double* eta, double* div, double* fv, double* fu) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    divergenceFromVelocity(p, c, div, uph, uth);
    computeForceVelTheta(p, c, fv, uth, uph, eta, div);
    computeForceVelPhi(p, c, fu, uph, uth, eta, div);
}

// Solver::updateForward / updateBackward (bubble.cu:1049-1116); the new map
// replaces the old one (the reference swaps with tmp).
void sb_oracle_update_maps(const sb_oracle_params* p, sb_oracle_state* s) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    const size_t N = (size_t)p->nTheta * p->nPhi;
    std::vector<double> tt(N), tp(N);
    updateMappingKernel(p, c, s->uth, s->uph, -p->dt, s->fwd_t, s->fwd_p, tt.data(), tp.data());
    std::memcpy(s->fwd_t, tt.data(), N * 8);
    std::memcpy(s->fwd_p, tp.data(), N * 8);
    updateMappingKernel(p, c, s->uth, s->uph, p->dt, s->bwd_t, s->bwd_p, tt.data(), tp.data());
    std::memcpy(s->bwd_t, tt.data(), N * 8);
    std::memcpy(s->bwd_p, tp.data(), N * 8);
}

// Solver::advection (bubble.cu:1171-1214)
void sb_oracle_advection(const sb_oracle_params* p, sb_oracle_state* s) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    const long long nP = p->nPhi;
    const size_t N = (size_t)p->nTheta * nP, Nv = N - nP;
    std::vector<double> uthN(Nv), uphN(N), etaN(N), gamN(N);
    const int nth = nthreads_of(p);
    const double dt = p->dt;
    const double* uth = s->uth;
    const double* uph = s->uph;
    const bool rk2 = !p->single_step_velocity;
    CELL_LOOP(p->nTheta - 1, {
        d2 gId = d2{(double)thetaId, (double)phiId} + d2{1.0, 0.0};
        double guTheta = uth[cell];
        double guPhi = sampleVPhi(c, uph, gId, (size_t)nP);
        uthN[cell] = advectVelocity(c, uph, uth, dt, gId, guTheta, guPhi, false, rk2);
    })
    CELL_LOOP(p->nTheta, {
        d2 gId = d2{(double)thetaId, (double)phiId} + d2{0.5, -0.5};
        double guTheta = sampleVTheta(c, uth, gId, (size_t)nP);
        double guPhi = uph[cell];
        uphN[cell] = advectVelocity(c, uph, uth, dt, gId, guTheta, guPhi, true, rk2);
    })
    const double* gam = s->gamma;
    if (p->plain_advection) {
        // advectionAllCentered (bubble.cu:937-961): both scalars at the trace
        const double* eta = s->eta;
        CELL_LOOP(p->nTheta, {
            d2 gId = d2{(double)thetaId, (double)phiId} + d2{0.5, 0.0};
            d2 traceId = traceGreatCircle(c, uth, uph, dt, gId, (size_t)nP);
            etaN[cell] = sampleCentered(c, eta, traceId, (size_t)nP);
            gamN[cell] = sampleCentered(c, gam, traceId, (size_t)nP);
        })
    } else {
        advectionCenteredBimocq(p, c, etaN.data(), s->eta, s->eta_init, s->eta_delta,
                                s->eta_initLast, s->eta_deltaLast, s->bwd_t, s->bwd_p,
                                s->bwdprev_t, s->bwdprev_p);
        // bubble.cu:910-931: concentration without BIMOCQ
        CELL_LOOP(p->nTheta, {
            d2 gId = d2{(double)thetaId, (double)phiId} + d2{0.5, 0.0};
            d2 traceId = traceGreatCircle(c, uth, uph, dt, gId, (size_t)nP);
            gamN[cell] = sampleCentered(c, gam, traceId, (size_t)nP);
        })
    }
    std::memcpy(s->uth, uthN.data(), Nv * 8);
    std::memcpy(s->uph, uphN.data(), N * 8);
    std::memcpy(s->eta, etaN.data(), N * 8);
    std::memcpy(s->gamma, gamN.data(), N * 8);
}

void sb_oracle_airflow(const sb_oracle_params* p, const double* uair_init,
                       const double* vair_init, double* uair, double* vair) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    airFlow(p, c, uair_init, vair_init, uair, vair);
}

void sb_oracle_assemble(const sb_oracle_params* p, const sb_oracle_state* s, double* gamma,
                        double* val, double* rhs, double* uair, double* vair) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    const size_t N = (size_t)p->nTheta * p->nPhi;
    airFlow(p, c, s->uair_init, s->vair_init, uair, vair);
    std::vector<double> W(N), fu, fv;
    vanDerWaals(p, W.data(), s->eta);
    viscousForces(p, c, s, fu, fv);
    concentrationLinearSystem(p, c, s->uph, s->uth, gamma, s->eta, W.data(), uair, vair,
                              fu.data(), fv.data(), val, rhs);
}

int sb_oracle_solve(const sb_oracle_params* p, const double* val, const double* rhs, double* x,
                    double* rel_resid) {
    return solveSystem(p, val, rhs, x, rel_resid);
}

// Solver::bodyforce (bubble.cu:2383-2506)
int sb_oracle_bodyforce(const sb_oracle_params* p, sb_oracle_state* s, sb_oracle_stats* st) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    const long long nP = p->nPhi;
    const size_t N = (size_t)p->nTheta * nP, Nv = N - nP;
    std::vector<double> uair(N + 1), vair(Nv + 1), W(N), val(5 * N), rhs(N);
    airFlow(p, c, s->uair_init, s->vair_init, uair.data(), vair.data());
    vanDerWaals(p, W.data(), s->eta);  // stored in thickness->NextStep by the reference
    std::vector<double> fu, fv;
    viscousForces(p, c, s, fu, fv);
    concentrationLinearSystem(p, c, s->uph, s->uth, s->gamma, s->eta, W.data(), uair.data(),
                              vair.data(), fu.data(), fv.data(), val.data(), rhs.data());
    std::vector<double> gamNext(s->gamma, s->gamma + N);
    double rel = 0.0;
    int iters = solveSystem(p, val.data(), rhs.data(), gamNext.data(), &rel);
    std::vector<double> div(N), uthN(Nv), uphN(N), tmp_t(N), tmp_p(N), etaN(N);
    divergenceFromGamma(p, div.data(), gamNext.data(), s->gamma);
    if (p->viscous) {
        applyForceVelThetaViscous(p, c, uthN.data(), s->uth, s->eta, gamNext.data(), vair.data(),
                                  fv.data());
        applyForceVelPhiViscous(p, c, uphN.data(), s->uph, s->eta, gamNext.data(), uair.data(),
                                fu.data());
    } else {
        applyForceVelTheta(p, c, uthN.data(), s->uth, tmp_t.data(), s->eta, W.data(),
                           gamNext.data(), vair.data());
        applyForceVelPhi(p, c, uphN.data(), s->uph, tmp_p.data(), s->eta, W.data(),
                         gamNext.data(), uair.data());
    }
    applyForceThickness(p, etaN.data(), s->eta, tmp_t.data(), div.data());
    accumulateChangesCentered(p, c, s->eta_delta, tmp_t.data(), s->fwd_t, s->fwd_p);
    for (size_t i = 0; i < N; ++i) tmp_p[i] = gamNext[i] - s->gamma[i];
    accumulateChangesCentered(p, c, s->gam_delta, tmp_p.data(), s->fwd_t, s->fwd_p);
    int broken = 0;
    for (size_t i = 0; i < N; ++i) broken += (val[5 * i + 2] == 1.0 && val[5 * i + 1] == 0.0);
    std::memcpy(s->eta, etaN.data(), N * 8);
    std::memcpy(s->gamma, gamNext.data(), N * 8);
    std::memcpy(s->uth, uthN.data(), Nv * 8);
    std::memcpy(s->uph, uphN.data(), N * 8);
    if (st) {
        st->solver_iters = iters;
        st->solver_rel_resid = rel;
        st->broken_cells = broken;
        st->floor_oob += (int)oob.load();
    }
    return (rel <= p->solver_tol * 10 || rel < 1e-10) ? 0 : 1;
}

void sb_oracle_distortion(const sb_oracle_params* p, sb_oracle_state* s, sb_oracle_stats* st) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    double a = estimateDistortion(p, c, s->fwd_t, s->fwd_p, s->bwd_t, s->bwd_p);
    double b = estimateDistortion(p, c, s->bwd_t, s->bwd_p, s->fwd_t, s->fwd_p);
    if (st) {
        st->distortion = std::max(a, b);
        st->floor_oob += (int)oob.load();
    }
}

// Solver::reInitializeMapping (bubble.cu:2509-2564)
void sb_oracle_reinit(const sb_oracle_params* p, sb_oracle_state* s) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    const size_t N = (size_t)p->nTheta * p->nPhi;
    std::vector<double> etaNext(s->eta, s->eta + N), gamNext(s->gamma, s->gamma + N);
    std::vector<double> tmp_t(N), tmp_p(N);
    correctCentered1(p, c, s->eta, tmp_t.data(), s->eta_delta, s->eta_init, s->gamma, tmp_p.data(),
                     s->gam_delta, s->gam_init, s->fwd_t, s->fwd_p);
    correctCentered2(p, c, s->eta, etaNext.data(), tmp_t.data(), s->gamma, gamNext.data(),
                     tmp_p.data(), s->bwd_t, s->bwd_p);
    // swap(initLast, init), swap(deltaLast, delta), swap(bwdprev, bwd); then
    // init <- current, delta <- 0, fwd = bwd = identity.
    std::memcpy(s->eta_initLast, s->eta_init, N * 8);
    std::memcpy(s->eta_deltaLast, s->eta_delta, N * 8);
    std::memcpy(s->gam_initLast, s->gam_init, N * 8);
    std::memcpy(s->gam_deltaLast, s->gam_delta, N * 8);
    std::memcpy(s->bwdprev_t, s->bwd_t, N * 8);
    std::memcpy(s->bwdprev_p, s->bwd_p, N * 8);
    std::memcpy(s->eta_init, s->eta, N * 8);
    std::memset(s->eta_delta, 0, N * 8);
    std::memcpy(s->gam_init, s->gamma, N * 8);
    std::memset(s->gam_delta, 0, N * 8);
    initMapping(p->nTheta, p->nPhi, s->fwd_t, s->fwd_p);
    initMapping(p->nTheta, p->nPhi, s->bwd_t, s->bwd_p);
}

// Solver::stepForward (kernel/solver.cu:260-292); without BIMOCQ the maps
// are neither updated nor checked for distortion (solver.cu:265-288), while
// bodyforce still accumulates the changes through the (identity) maps
int sb_oracle_step(const sb_oracle_params* p, sb_oracle_state* s, sb_oracle_stats* st) {
    sb_oracle_stats local{};
    // Under VISCOUS the reference launches applyforcevelphiKernel_viscous
    // with the u_theta launch layout (nTheta - 1 rows: the VISCOUS branch of
    // bubble.cu:2463-2474 has no determineLayout for velPhi), so the last
    // theta row of the output buffer is never written; after the buffer
    // swap it holds u_phi from before the step's advection.
    const size_t N = (size_t)p->nTheta * p->nPhi, nP = (size_t)p->nPhi;
    std::vector<double> uph_last;
    if (p->viscous) uph_last.assign(s->uph + (N - nP), s->uph + N);
    if (!p->plain_advection) sb_oracle_update_maps(p, s);
    sb_oracle_advection(p, s);
    int rc = sb_oracle_bodyforce(p, s, &local);
    if (p->viscous) std::copy(uph_last.begin(), uph_last.end(), s->uph + (N - nP));
    bool re = false;
    if (!p->plain_advection) {
        sb_oracle_distortion(p, s, &local);
        re = p->force_reinit < 0 ? (local.distortion > 4.f) : (p->force_reinit != 0);
    }
    if (re) sb_oracle_reinit(p, s);
    local.reinit = re ? 1 : 0;
    if (st) *st = local;
    return rc;
}

void sb_oracle_sample(const sb_oracle_params* p, int kind, const double* field, int n,
                      const double* coords, double* out) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    for (int i = 0; i < n; ++i) {
        d2 q = {coords[2 * i], coords[2 * i + 1]};
        if (kind == 0) out[i] = sampleCentered(c, field, q, c.nPhi);
        else if (kind == 1) out[i] = sampleVPhi(c, field, q, c.nPhi);
        else out[i] = sampleVTheta(c, field, q, c.nPhi);
    }
}

void sb_oracle_trace(const sb_oracle_params* p, const double* uth, const double* uph, double dt,
                     int n, const double* coords, double* out) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    for (int i = 0; i < n; ++i) {
        d2 r = traceGreatCircle(c, uth, uph, dt, d2{coords[2 * i], coords[2 * i + 1]}, c.nPhi);
        out[2 * i] = r.x;
        out[2 * i + 1] = r.y;
    }
}

void sb_oracle_sample_mapping(const sb_oracle_params* p, const double* map_t,
                              const double* map_p, int n, const double* coords, double* out) {
    std::atomic<long> oob{0};
    Ctx c = make_ctx(p, &oob);
    for (int i = 0; i < n; ++i) {
        d2 r = sampleMapping(c, map_t, map_p, d2{coords[2 * i], coords[2 * i + 1]});
        out[2 * i] = r.x;
        out[2 * i + 1] = r.y;
    }
}

}  // extern "C"
