// Shared host-side definitions: TDEP's unit system and tolerances, error reporting,
// small 3x3 linear algebra. Constant values are those of src/libolle/konstanter.f90.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdint>
#include <string>
#include <functional>
#include <thread>
#include <vector>

namespace tdg {

using cplx = std::complex<double>;

// ---- physical constants and conversions (src/libolle/konstanter.f90:26-109) ----
constexpr double kPi = 3.141592653589793;
constexpr double kTwoPi = 6.283185307179586;
constexpr double kEvToJoule = 1.6021766208E-19;
constexpr double kHartreeToEv = 27.21138602;
constexpr double kEvToHartree = 1.0 / kHartreeToEv;
constexpr double kHartreeToJoule = kHartreeToEv * kEvToJoule;
constexpr double kBohrToM = 0.52917721067E-10;
constexpr double kBohrToA = 0.52917721067;
constexpr double kAToBohr = 1.0 / kBohrToA;
constexpr double kHbarEv = 6.582119514E-16;
constexpr double kHbarJoule = kHbarEv * kEvToJoule;
constexpr double kHbarHartree = kHbarEv * kEvToHartree;
constexpr double kKbEv = 8.6173303E-5;
constexpr double kKbHartree = kKbEv * kEvToHartree;
constexpr double kAmuToKg = 1.660539040E-27;
constexpr double kEmuToKg = 9.10938356E-31;
constexpr double kAmuToEmu = kAmuToKg / kEmuToKg;
constexpr double kTimeAuToS = kHbarJoule / kHartreeToJoule;
constexpr double kFc2EvAToHaBohr = kEvToHartree / (kAToBohr * kAToBohr);
constexpr double kFc3EvAToHaBohr = kEvToHartree / (kAToBohr * kAToBohr * kAToBohr);
constexpr double kFc4EvAToHaBohr = kEvToHartree / (kAToBohr * kAToBohr * kAToBohr * kAToBohr);
constexpr double kFreqHartreeToTHz = 1E-12 / kTwoPi / kHbarHartree;
constexpr double kFreqTHzToHartree = 1.0 / kFreqHartreeToTHz;
constexpr double kKappaAuToSI = kHartreeToJoule / kTimeAuToS / kBohrToM;
constexpr double kGroupVelAuToMs = kBohrToM / kTimeAuToS;  // lo_groupvel_Hartreebohr_to_ms
constexpr double kMToBohr = 1.0 / kBohrToM;

// ---- tolerances (konstanter.f90:113-140) ----
constexpr double kTol = 1E-5;
constexpr double kSqTol = kTol * kTol;
constexpr double kFreqTol = kTol * 1E-4;
constexpr double kGroupVelTol = kTol * 1E-5;
constexpr double kTemperatureTol = 1E-3;
constexpr int32_t kHugeInt = 2147483647;
constexpr double kDegenVector[3] = {1.0E-8, 1.33E-8, 1.45624623E-8};

// ---- status codes (konstanter.f90:160-172) + device ----
enum Status : int {
    kOk = 0,
    kErrBadDim = 1,
    kErrLinalg = 2,
    kErrPhysical = 3,
    kErrSymmetry = 4,
    kErrParam = 5,
    kErrIo = 6,
    kErrDevice = 8,
};

// Records the message for tdg_last_error() and returns the code.
int set_error(int code, const std::string &msg);

// Host-phase timing for diagnostics: when the environment variable TDG_TRACE is set, the
// time between successive mark() calls is summed per label and printed to stderr when the
// timer goes out of scope. Costs one clock read per mark otherwise.
class PhaseTimer {
  public:
    explicit PhaseTimer(const char *scope);
    ~PhaseTimer();
    void mark(const char *label);

  private:
    const char *scope_;
    bool on_;
    double t_;
    std::vector<std::pair<const char *, double>> sums_;
};

// f(i) for i in [0, n) on all hardware threads (dynamic assignment, one index at a time);
// f must be safe to run concurrently for different i. Runs on a fixed pool of worker threads
// created on first use (one job at a time; a call made while another runs, or in a child
// process after fork, runs serially in the caller).
bool pool_run(int64_t n, const std::function<void(int64_t)> &f);

template <typename F>
void parallel_for(int64_t n, F f) {
    if (n <= 1) {
        for (int64_t i = 0; i < n; ++i) f(i);
        return;
    }
    const std::function<void(int64_t)> fn = f;
    if (!pool_run(n, fn))
        for (int64_t i = 0; i < n; ++i) f(i);
}
const char *last_error();

// ---- 3x3 helpers, column-major like the Fortran arrays: m[i + 3*j] ----
struct M3 {
    double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double &operator()(int i, int j) { return a[i + 3 * j]; }
    double operator()(int i, int j) const { return a[i + 3 * j]; }
};
struct V3 {
    double x[3] = {0, 0, 0};
    double &operator[](int i) { return x[i]; }
    double operator[](int i) const { return x[i]; }
};
inline V3 mul(const M3 &m, const V3 &v) {
    V3 r;
    for (int i = 0; i < 3; ++i) r[i] = m(i, 0) * v[0] + m(i, 1) * v[1] + m(i, 2) * v[2];
    return r;
}
inline M3 mul(const M3 &a, const M3 &b) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += a(i, k) * b(k, j);
            r(i, j) = s;
        }
    return r;
}
inline M3 transpose(const M3 &a) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r(i, j) = a(j, i);
    return r;
}
inline double det(const M3 &m) {
    return m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) -
           m(0, 1) * (m(1, 0) * m(2, 2) - m(1, 2) * m(2, 0)) +
           m(0, 2) * (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0));
}
inline M3 inverse(const M3 &m) {
    M3 r;
    const double d = det(m);
    r(0, 0) = (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) / d;
    r(0, 1) = (m(0, 2) * m(2, 1) - m(0, 1) * m(2, 2)) / d;
    r(0, 2) = (m(0, 1) * m(1, 2) - m(0, 2) * m(1, 1)) / d;
    r(1, 0) = (m(1, 2) * m(2, 0) - m(1, 0) * m(2, 2)) / d;
    r(1, 1) = (m(0, 0) * m(2, 2) - m(0, 2) * m(2, 0)) / d;
    r(1, 2) = (m(0, 2) * m(1, 0) - m(0, 0) * m(1, 2)) / d;
    r(2, 0) = (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0)) / d;
    r(2, 1) = (m(0, 1) * m(2, 0) - m(0, 0) * m(2, 1)) / d;
    r(2, 2) = (m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0)) / d;
    return r;
}
inline double sqnorm(const V3 &v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }

// Fortran anint: round half away from zero.
inline double anint(double x) { return std::round(x); }

// Physics helpers (gottochblandat_physics.f90:160-186, 331-366).
double planck(double temperature, double omega);
double harmonic_oscillator_cv(double temperature, double omega);

}  // namespace tdg
