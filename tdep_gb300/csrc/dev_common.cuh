// Device helpers shared by the three- and four-phonon kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tdg {

namespace {

constexpr double kSqrt2PiInv = 0.398942280401433;
constexpr double kFreqTolD = 1E-9;
constexpr double kTwoPiD = 6.283185307179586;
constexpr int kMaxRed = 192;

template <typename R>
struct CT;
template <>
struct CT<double> {
    using C = double2;
};
template <>
struct CT<float> {
    using C = float2;
};

template <typename C>
__device__ __forceinline__ C czero();
template <>
__device__ __forceinline__ double2 czero<double2>() {
    return make_double2(0.0, 0.0);
}
template <>
__device__ __forceinline__ float2 czero<float2>() {
    return make_float2(0.f, 0.f);
}

template <typename C>
__device__ __forceinline__ void cfma(C &acc, const C &a, const C &b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}

__device__ __forceinline__ bool nonzero(double x) { return (__double_as_longlong(x) << 1) != 0; }

// om1 - (m2 + m3) from the FP32 pairs omega = h + l (h = the FP32 omega, l the FP32 rest):
// the sums of the h parts with their exact rounding errors (Knuth's TwoSum, FP32 additions
// only) plus the l parts. Accurate to about 2^-24 of the difference plus 2^-46 of omega, as
// the FP64 difference rounded to FP32; no FP64 operation (GB300 issues FP64 at 1/64 of the
// FP32 rate).
__device__ __forceinline__ float centre_diff_f32(float h1, float l1, float h2, float l2, float h3, float l3) {
    const float s = h2 + h3;
    const float bs = s - h2;
    const float es = (h2 - (s - bs)) + (h3 - bs);  // h2 + h3 = s + es exactly
    const float d = h1 - s;
    const float bd = d - h1;
    const float ed = (h1 - (d - bd)) + (-s - bd);  // h1 - s = d + ed exactly
    return d + (ed + ((l1 - l2 - l3) - es));
}

// |x - y| < lo_freqtol (1e-9) for x = h1 + l1 and y = h2 + l2 given as FP32 (hi, rest)
// pairs: where the test can hold, h1 - h2 is exact (Sterbenz) and the result is the FP64
// difference to ~1e-17.
__device__ __forceinline__ bool close_f32(float h1, float l1, float h2, float l2) {
    return fabsf((h1 - h2) + (l1 - l2)) < 1e-9f;
}

// Double-float accumulation on the FP32 pipe: s += p (TwoSum of the high parts), and the
// sum of two double-float values.
__device__ __forceinline__ void df_acc(float2 &s, float p) {
    const float t = s.x + p;
    const float bb = t - s.x;
    s.y += (s.x - (t - bb)) + (p - bb);
    s.x = t;
}
__device__ __forceinline__ float2 df_merge(float2 a, float2 b) {
    const float t = a.x + b.x;
    const float bb = t - a.x;
    const float e = (a.x - (t - bb)) + (b.x - bb);
    return make_float2(t, a.y + b.y + e);
}

// Square root by the hardware approximation (sqrt.approx.f32, a few ulp): for the FP32
// screens, whose windows carry a relative margin of 1e-3.
__device__ __forceinline__ float sqrt_screen(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Exclusive scan of one int per thread over the block (blockDim a multiple of 32).
__device__ __forceinline__ int block_exclusive_scan(int v, int *wsum, int &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < nw ? wsum[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) wsum[lane] = s;
    }
    __syncthreads();
    total = wsum[nw - 1];
    const int res = (w > 0 ? wsum[w - 1] : 0) + x - v;
    __syncthreads();
    return res;
}

}  // namespace

// exp(-t) for 0 <= t <= 40 in FP64, written from the mathematics: t = (64 m + j) ln2/64 + r
// (Cody-Waite reduction with a two-part ln2/64, |r| <= ln2/128), exp(-t) =
// 2^-m * 2^(-j/64) * exp(-r), exp(-r) by its Taylor series to degree 6 (truncation below
// 3e-20 relative), 2^(-j/64) from a 64-entry table built on the host. 13 FP64 operations
// against about twice that for the general exp(); tested against exp() on the device.
__device__ __forceinline__ double exp_neg(double t, const double *tab64) {
    constexpr double kInvLn2x64 = 92.33248261689366;            // 64 / ln 2
    constexpr double kLn2o64Hi = 0.010830424696244734;          // ln2/64 to 41 bits: k*Hi exact
    constexpr double kLn2o64Lo = 4.411764150473684e-15;         // ln2/64 - Hi
    constexpr double kShift = 6755399441055744.0;               // 1.5 * 2^52
    const double ys = fma(t, kInvLn2x64, kShift);
    const int k = __double2loint(ys);                            // rint(t * 64/ln2)
    const double kf = ys - kShift;
    double r = fma(-kf, kLn2o64Hi, t);
    r = fma(-kf, kLn2o64Lo, r);
    const double s = -r;
    double p = fma(s, 1.0 / 720.0, 1.0 / 120.0);
    p = fma(s, p, 1.0 / 24.0);
    p = fma(s, p, 1.0 / 6.0);
    p = fma(s, p, 0.5);
    p = fma(s, p, 1.0);
    p = fma(s, p, 1.0);
    const int mm = k >> 6, j = k & 63;
    const double scale = __hiloint2double((1023 - mm) << 20, 0);  // 2^-mm
    return (tab64[j] * p) * scale;
}

namespace {

// lo_gauss (gottochblandat_calculus.f90:268-288) for x - mu = dx, with 8 sigma, the
// exponent factor 0.5/sigma^2 and 1/(sigma sqrt(2 pi)) supplied.
__device__ __forceinline__ double gauss(double dx, double win8, double h, double c, const double *tab64) {
    if (fabs(dx) > win8) return 0.0;
    return exp_neg(dx * dx * h, tab64) * c;
}

// d0 = g(om1; -om2+om3) - g(om1; om2-om3), d1 = g(om1; om2+om3) - g(om1; -om2-om3)
// (get_dirac, scattering_threephonon.f90:262-267), evaluating only the Gaussians whose bit
// (0..3 in that order) is set in live; the others are 0 (outside their window). One
// Gaussian per loop trip, so a warp runs as many trips as its lane with the most live bits
// instead of every branch some lane needs. The centre is (+-om2) + (+-om3) with the signs
// applied to the bit patterns: the same rounding as the reference's expressions.
__device__ __forceinline__ void dirac3(uint32_t live, double o1, double o2, double o3, double win8, double h,
                                       double c, const double *tab, double &d0, double &d1) {
    double g0 = 0.0, g1 = 0.0, g2 = 0.0, g3 = 0.0;
    const long long b2 = __double_as_longlong(o2), b3 = __double_as_longlong(o3);
    constexpr long long kSign = (long long)0x8000000000000000ULL;
    while (live) {
        const int j = __ffs(live) - 1;
        live &= live - 1;
        const double m2 = __longlong_as_double((j == 1 || j == 2) ? b2 : (b2 ^ kSign));
        const double m3 = __longlong_as_double((j == 0 || j == 2) ? b3 : (b3 ^ kSign));
        const double g = gauss(o1 - (m2 + m3), win8, h, c, tab);
        g0 = j == 0 ? g : g0;
        g1 = j == 1 ? g : g1;
        g2 = j == 2 ? g : g2;
        g3 = j == 3 ? g : g3;
    }
    d0 = g0 - g1;
    d1 = g2 - g3;
}

__device__ __forceinline__ double adaptive_pair(const double *va, const double *vb, const double *rl) {
    // sqrt(maxval(matmul(va - vb, reclat)**2) * 0.5)
    double m = 0;
    for (int j = 0; j < 3; ++j) {
        double s = 0;
        for (int i = 0; i < 3; ++i) s += (va[i] - vb[i]) * rl[i + 3 * j];
        m = fmax(m, s * s);
    }
    return sqrt(m * 0.5);
}


}  // namespace

}  // namespace tdg
