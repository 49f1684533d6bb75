// K2+K3+K4: fused three-phonon scattering for one accepted irreducible q-triplet per
// CTA iteration (persistent grid-stride loop over the triplet list).
//
// Reference (src/thermal_conductivity/scattering_threephonon.f90):
//   pretransform_phi3 (:275-317)   ptf(a,b,c) = sum_t mwm_t(i,j,k) exp(-2 pi i (q2.lv2 + q3.lv3))
//   zgeru x2 + dot_product (:93-113)  c0 = sum_abc e1(a) e2(b) e3(c) ptf(a,b,c), e = egv/sqrt(omega)
//   get_dirac (:219-271) and accumulation (:115-135) for Gamma and the Xi row terms.
// The reference recomputes ptf and evp for every b1 of q1 and contracts per (b2,b3)
// (2 n^5 complex MACs per row); here one CTA builds ptf once per q-triplet and contracts
// it with all three eigenvector matrices for all (b1,b2,b3) at once:
//   T1[b1][b][c] = sum_a E1[a][b1] P[a][b][c]
//   T2[b1][b2][c] = sum_b E2[b][b2] T1[b1][b][c]
//   Psi[b1][b2][b3] = sum_c E3[c][b3] T2[b1][b2][c]          (3 n^4 complex MACs)
// The phase factors are exact roots of unity: q = g/N on the mesh and lv are integer
// lattice vectors, so q.lv = sum_d g_d lv_d / N_d and exp(-2 pi i q.lv) is one entry of a
// table of exp(-2 pi i K / L), L = lcm of the mesh dimensions.
//
// The delta weights stay FP64 as in the reference, but GB300's FP64 pipe is narrow, so
// every mode triplet is first screened in FP32 against the 8-sigma window of lo_gauss
// with a safety margin; only triplets that may fall inside it take the exact FP64 path,
// which reproduces the reference's arithmetic (same window test, same formulas).
//
// Everything for one triplet lives in shared memory: P and T (two n^3 complex buffers),
// the three scaled eigenvector matrices, the phase chunk and per-mode scalars. Precision R
// is double (FP64 path) or float (mixed path: FP32 pretransform and contraction, FP64
// delta weights, occupations and accumulation).
#include <cuda_runtime.h>

#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr double kThreePhononPrefactor = 3.141592653589793 / 16.0;
constexpr double kSqrt2PiInv = 0.398942280401433;
constexpr double kFreqTolD = 1E-9;
constexpr int kMaxRed = 192;
constexpr int kPhaseChunk = 1024;

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

// lo_gauss (gottochblandat_calculus.f90:268-288) with 1/sigma supplied.
__device__ __forceinline__ double gauss(double x, double mu, double sigma, double invsig) {
    if (fabs(x - mu) > 8.0 * sigma) return 0.0;
    return exp(-(x - mu) * (x - mu) * 0.5 * invsig * invsig) * kSqrt2PiInv * invsig;
}

template <typename T>
__device__ __forceinline__ T adaptive_pair(const T *va, const T *vb, const double *rl) {
    // sqrt(maxval(matmul(va - vb, reclat)**2) * 0.5)
    T m = 0;
    for (int j = 0; j < 3; ++j) {
        T s = 0;
        for (int i = 0; i < 3; ++i) s += (va[i] - vb[i]) * (T)rl[i + 3 * j];
        m = max(m, s * s);
    }
    return sqrt(m * (T)0.5);
}

template <typename R>
__device__ __forceinline__ const R *mwm_ptr(const Fc3Dev &fc);
template <>
__device__ __forceinline__ const double *mwm_ptr<double>(const Fc3Dev &fc) {
    return fc.mwm;
}
template <>
__device__ __forceinline__ const float *mwm_ptr<float>(const Fc3Dev &fc) {
    return fc.mwm32;
}

template <typename C>
__device__ __forceinline__ C twiddle_at(const Fc3Dev &fc, int k);
template <>
__device__ __forceinline__ double2 twiddle_at<double2>(const Fc3Dev &fc, int k) {
    return fc.twiddle[k];
}
template <>
__device__ __forceinline__ float2 twiddle_at<float2>(const Fc3Dev &fc, int k) {
    return fc.twiddle32[k];
}

template <typename C>
__device__ __forceinline__ const C *egvs_ptr(const PhononDev &ph);
template <>
__device__ __forceinline__ const double2 *egvs_ptr<double2>(const PhononDev &ph) {
    return ph.egvs;
}
template <>
__device__ __forceinline__ const float2 *egvs_ptr<float2>(const PhononDev &ph) {
    return ph.egvs32;
}

// Shared-memory layout (bytes) for mode count n and complex size cs.
struct Layout {
    size_t om1, om2, om3, inv1, be2, be3, s1, s2, s3, v1, v2, v3, wrow, r2, f32, E1, E2, E3, A, B, ph, rowid, red,
        total;
};
__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ inline Layout make_layout(int n, int cs) {
    Layout L;
    size_t o = 0;
    const size_t dn = align16(sizeof(double) * n);
    const size_t n2 = (size_t)n * n, n3 = n2 * n;
    L.om1 = o; o += dn;
    L.om2 = o; o += dn;
    L.om3 = o; o += dn;
    L.inv1 = o; o += dn;
    L.be2 = o; o += dn;
    L.be3 = o; o += dn;
    L.s1 = o; o += dn;
    L.s2 = o; o += dn;
    L.s3 = o; o += dn;
    L.v1 = o; o += 3 * dn;
    L.v2 = o; o += 3 * dn;
    L.v3 = o; o += 3 * dn;
    L.wrow = o; o += dn;
    L.r2 = o; o += align16(sizeof(double) * n2);
    L.f32 = o; o += align16(sizeof(float) * n * 6);  // float copies: om1..3, s1..3
    L.E1 = o; o += align16(cs * n2);
    L.E2 = o; o += align16(cs * n2);
    L.E3 = o; o += align16(cs * n2);
    // A and B must each hold n^3 complex values and at least n^3 doubles.
    const size_t csz = (size_t)cs > sizeof(double) ? (size_t)cs : sizeof(double);
    const size_t buf = align16(csz * n3);
    L.A = o; o += buf;
    L.B = o; o += buf;
    L.ph = o; o += align16((size_t)cs * kPhaseChunk);
    L.rowid = o; o += align16(sizeof(int) * n);
    L.red = o; o += align16(sizeof(int2) * kMaxRed);
    L.total = o;
    return L;
}

template <int N, typename R>
__global__ void __launch_bounds__(((N * N + 31) / 32) * 32)
    k_threephonon(ThreePhArgs a) {
    using C = typename CT<R>::C;
    constexpr int N2 = N * N, N3 = N2 * N;
    constexpr int NA = N / 3;
    extern __shared__ __align__(16) unsigned char smem[];
    const Layout L = make_layout(N, sizeof(C));
    double *om1 = (double *)(smem + L.om1);
    double *om2 = (double *)(smem + L.om2);
    double *om3 = (double *)(smem + L.om3);
    double *inv1 = (double *)(smem + L.inv1);
    double *be2 = (double *)(smem + L.be2);
    double *be3 = (double *)(smem + L.be3);
    double *s1 = (double *)(smem + L.s1);
    double *s2 = (double *)(smem + L.s2);
    double *s3 = (double *)(smem + L.s3);
    double *v1 = (double *)(smem + L.v1);
    double *v2 = (double *)(smem + L.v2);
    double *v3 = (double *)(smem + L.v3);
    double *wrow = (double *)(smem + L.wrow);
    double *R2 = (double *)(smem + L.r2);
    float *fo1 = (float *)(smem + L.f32);
    float *fo2 = fo1 + N, *fo3 = fo2 + N, *fs1 = fo3 + N, *fs2 = fs1 + N, *fs3 = fs2 + N;
    C *E1 = (C *)(smem + L.E1);
    C *E2 = (C *)(smem + L.E2);
    C *E3 = (C *)(smem + L.E3);
    C *A = (C *)(smem + L.A);
    C *B = (C *)(smem + L.B);
    C *ph = (C *)(smem + L.ph);
    int *rowid = (int *)(smem + L.rowid);
    int2 *red = (int2 *)(smem + L.red);
    const int tid = threadIdx.x, bd = blockDim.x;
    const MeshDev &m = a.mesh;
    const PhononDev &P = a.ph;
    const Fc3Dev &fc = a.fc;
    const R *mwm = mwm_ptr<R>(fc);
    const C *egvs = egvs_ptr<C>(P);
    const int64_t ld = (int64_t)m.n_full * N;
    const int it = P.integrationtype;
    const float sigfix32 = (float)P.sigma_fixed;

    for (int t = blockIdx.x; t < a.n_trip; t += gridDim.x) {
        const TripletRec rec = a.trip[t];
        const int f1 = m.irr_full[rec.q1];
        const int q2 = rec.q2, q3 = rec.q3;
        const int i2 = m.full_irr[q2], i3 = m.full_irr[q3];
        const uint32_t *mask = a.cand_mask + (size_t)rec.cand * 4;
        const int nred = rec.red_cnt;
        // ---- per-mode scalars and scaled eigenvectors ----
        for (int b = tid; b < N; b += bd) {
            om1[b] = P.omega[(size_t)f1 * N + b];
            om2[b] = P.omega[(size_t)q2 * N + b];
            om3[b] = P.omega[(size_t)q3 * N + b];
            inv1[b] = om1[b] > 0.0 ? 1.0 / om1[b] : 0.0;
            be2[b] = P.be[(size_t)i2 * N + b];
            be3[b] = P.be[(size_t)i3 * N + b];
            s1[b] = P.sigsq[(size_t)rec.q1 * N + b];
            s2[b] = P.sigsq[(size_t)i2 * N + b];
            s3[b] = P.sigsq[(size_t)i3 * N + b];
            fo1[b] = (float)om1[b];
            fo2[b] = (float)om2[b];
            fo3[b] = (float)om3[b];
            fs1[b] = (float)s1[b];
            fs2[b] = (float)s2[b];
            fs3[b] = (float)s3[b];
            for (int d = 0; d < 3; ++d) {
                v1[b * 3 + d] = P.vel[((size_t)f1 * N + b) * 3 + d];
                v2[b * 3 + d] = P.vel[((size_t)q2 * N + b) * 3 + d];
                v3[b * 3 + d] = P.vel[((size_t)q3 * N + b) * 3 + d];
            }
            const int r = a.rows.rowidx[(size_t)rec.q1 * N + b];
            const bool on = (mask[b >> 5] >> (b & 31)) & 1u;
            rowid[b] = on ? r : -1;
            wrow[b] = r >= 0 ? a.rows.weight3[r] : 0.0;
        }
        for (int i = tid; i < nred && i < kMaxRed; i += bd) red[i] = a.red[rec.red_off + i];
        for (int i = tid; i < 3 * N2; i += bd) {
            const int which = i / N2, e = i % N2;
            const int r = e / N, b = e % N;  // element (r) of mode b
            const int q = which == 0 ? f1 : (which == 1 ? q2 : q3);
            C *E = which == 0 ? E1 : (which == 1 ? E2 : E3);
            E[r * N + b] = egvs[((size_t)q * N + b) * N + r];
        }
        // ---- K2: pretransform into A ----
        for (int i = tid; i < N3; i += bd) A[i] = czero<C>();
        int gi2[3], gi3[3];
        {
            const int n12 = m.grid[1] * m.grid[2];
            gi2[0] = q2 / n12; gi2[1] = (q2 / m.grid[2]) % m.grid[1]; gi2[2] = q2 % m.grid[2];
            gi3[0] = q3 / n12; gi3[1] = (q3 / m.grid[2]) % m.grid[1]; gi3[2] = q3 % m.grid[2];
        }
        for (int c0 = 0; c0 < fc.n; c0 += kPhaseChunk) {
            const int cn = min(kPhaseChunk, fc.n - c0);
            __syncthreads();
            for (int i = tid; i < cn; i += bd) {
                const int32_t *lv = fc.lv + (size_t)(c0 + i) * 6;
                int K = 0;
                for (int d = 0; d < 3; ++d) {
                    int kd = (gi2[d] * lv[d] + gi3[d] * lv[3 + d]) % m.grid[d];
                    if (kd < 0) kd += m.grid[d];
                    K += kd * m.lmul[d];
                }
                ph[i] = twiddle_at<C>(fc, K % m.L);
            }
            __syncthreads();
            for (int idx = tid; idx < N3; idx += bd) {
                const int blk = idx / 27, ijk = idx % 27;
                const int lo = max(fc.blk_ptr[blk], c0), hi = min(fc.blk_ptr[blk + 1], c0 + cn);
                if (lo >= hi) continue;
                const int a1 = blk / (NA * NA), a2 = (blk / NA) % NA, a3 = blk % NA;
                const int ii = ijk % 3, jj = (ijk / 3) % 3, kk = ijk / 9;
                const int pa = 3 * a1 + ii, pb = 3 * a2 + jj, pc = 3 * a3 + kk;
                C acc = A[(pa * N + pb) * N + pc];
                for (int tt = lo; tt < hi; ++tt) {
                    const R mv = __ldg(mwm + (size_t)tt * 27 + ijk);
                    const C p = ph[tt - c0];
                    acc.x = fma(mv, p.x, acc.x);
                    acc.y = fma(mv, p.y, acc.y);
                }
                A[(pa * N + pb) * N + pc] = acc;
            }
        }
        __syncthreads();
        // ---- K3: T1 into B, T2 into A ----
        if (tid < N2) {
            const int bc = tid;
            C acc[N];
#pragma unroll
            for (int b1 = 0; b1 < N; ++b1) acc[b1] = czero<C>();
#pragma unroll 3
            for (int aa = 0; aa < N; ++aa) {
                const C p = A[aa * N2 + bc];
#pragma unroll
                for (int b1 = 0; b1 < N; ++b1) cfma(acc[b1], E1[aa * N + b1], p);
            }
#pragma unroll
            for (int b1 = 0; b1 < N; ++b1) B[b1 * N2 + bc] = acc[b1];
        }
        __syncthreads();
        if (tid < N2) {
            const int b1 = tid / N, c = tid % N;
            C acc[N];
#pragma unroll
            for (int b2 = 0; b2 < N; ++b2) acc[b2] = czero<C>();
#pragma unroll 3
            for (int b = 0; b < N; ++b) {
                const C tv = B[(b1 * N + b) * N + c];
#pragma unroll
                for (int b2 = 0; b2 < N; ++b2) cfma(acc[b2], E2[b * N + b2], tv);
            }
#pragma unroll
            for (int b2 = 0; b2 < N; ++b2) A[(b1 * N + b2) * N + c] = acc[b2];
        }
        __syncthreads();
        // ---- Psi and K4 epilogue: F[b1][b2][b3] into B (as doubles), R2 = sum over b3 ----
        double *F = (double *)B;
        if (tid < N2) {
            const int b1 = tid / N, b2 = tid % N;
            C acc[N];
#pragma unroll
            for (int b3 = 0; b3 < N; ++b3) acc[b3] = czero<C>();
#pragma unroll 3
            for (int c = 0; c < N; ++c) {
                const C tv = A[(b1 * N + b2) * N + c];
#pragma unroll
                for (int b3 = 0; b3 < N; ++b3) cfma(acc[b3], E3[c * N + b3], tv);
            }
            const int row = rowid[b1];
            const double o1 = om1[b1], o2 = om2[b2];
            const float f_o1 = fo1[b1], f_o2 = fo2[b2];
            const double perm = (q2 == q3) ? 1.0 : 2.0;
            const bool skip12 = row < 0 || o2 < kFreqTolD || fabs(o1 - o2) < kFreqTolD;
            double r2 = 0.0;
#pragma unroll
            for (int b3 = 0; b3 < N; ++b3) {
                double f = 0.0;
                const double o3 = om3[b3];
                if (!skip12 && !(o3 < kFreqTolD) && !(fabs(o1 - o3) < kFreqTolD || fabs(o2 - o3) < kFreqTolD)) {
                    // FP32 screen: the nearest of the four Gaussian centres against 8 sigma,
                    // with a relative margin and an absolute margin of the FP32 rounding.
                    const float f_o3 = fo3[b3];
                    float sg = 0.f;
                    if (it == 1) {
                        sg = sigfix32;
                    } else if (it == 2) {
                        sg = sqrtf(fs1[b1] + fs2[b2] + fs3[b3]);
                    }
                    // One bit per Gaussian of get_dirac that may lie inside its window; the
                    // velocity-difference width of -it 6 can cancel in FP32, so it is not screened.
                    const float win = 8.0f * sg * 1.001f + 1e-6f * (f_o1 + f_o2 + f_o3);
                    unsigned live = 15u;
                    if (it != 6) {
                        live = (fabsf(f_o1 + f_o2 - f_o3) <= win ? 1u : 0u) | (fabsf(f_o1 - f_o2 + f_o3) <= win ? 2u : 0u) |
                               (fabsf(f_o1 - f_o2 - f_o3) <= win ? 4u : 0u) | (f_o1 + f_o2 + f_o3 <= win ? 8u : 0u);
                    }
                    if (live) {
                        double sigma, invsig;
                        if (it == 1) {
                            sigma = P.sigma_fixed;
                            invsig = 1.0 / sigma;
                        } else if (it == 2) {
                            const double s = s1[b1] + s2[b2] + s3[b3];
                            invsig = rsqrt(s);
                            sigma = s * invsig;
                        } else {
                            sigma = adaptive_pair<double>(v1 + 3 * b1, v2 + 3 * b2, P.reclat_g) / 3.0;
                            sigma += adaptive_pair<double>(v1 + 3 * b1, v3 + 3 * b3, P.reclat_g) / 3.0;
                            sigma += adaptive_pair<double>(v2 + 3 * b2, v3 + 3 * b3, P.reclat_g) / 3.0;
                            sigma += P.thresh_sigma;
                            invsig = 1.0 / sigma;
                        }
                        const double ga = (live & 1u) ? gauss(o1, -o2 + o3, sigma, invsig) : 0.0;
                        const double gb = (live & 2u) ? gauss(o1, o2 - o3, sigma, invsig) : 0.0;
                        const double gc = (live & 4u) ? gauss(o1, o2 + o3, sigma, invsig) : 0.0;
                        const double gd = (live & 8u) ? gauss(o1, -o2 - o3, sigma, invsig) : 0.0;
                        const double d0 = ga - gb;
                        const double d1 = gc - gd;
                        if (nonzero(d0) || nonzero(d1)) {
                            const double cr = (double)acc[b3].x, ci = (double)acc[b3].y;
                            const double psisq = kThreePhononPrefactor * (cr * cr + ci * ci) * wrow[b1];
                            const double n2 = be2[b2], n3 = be3[b3];
                            const double plf0 = n2 - n3;
                            const double plf1 = n2 + n3 + 1.0;
                            const double f0 = perm * psisq * plf0 * d0;
                            const double f1 = perm * psisq * plf1 * d1;
                            f = f0 + f1;
                            r2 += f;
                        }
                    }
                }
                F[(b1 * N + b2) * N + b3] = f;
            }
            R2[tid] = r2;
        }
        __syncthreads();
        // ---- R3 = sum over b2, into A (as doubles); Gamma per b1 ----
        double *R3 = (double *)A;
        for (int e = tid; e < N2; e += bd) {
            const int b1 = e / N, b3 = e % N;
            double s = 0.0;
            for (int b2 = 0; b2 < N; ++b2) {
                const double f = F[(b1 * N + b2) * N + b3];
                if (nonzero(f)) s += f;
            }
            R3[e] = s;
        }
        __syncthreads();
        if (tid < N) {
            const int row = rowid[tid];
            if (row >= 0) {
                double g = 0.0;
                for (int b2 = 0; b2 < N; ++b2) g += R2[tid * N + b2];
                if (nonzero(g)) atomicAdd(a.gamma + row, (double)nred * g);
            }
        }
        for (int i = tid; i < 2 * N2 * nred; i += bd) {
            const int r = i / (2 * N2), e = i % (2 * N2);
            const int2 pr = red[r];
            if (e < N2) {
                const int b1 = e / N, b2 = e % N;
                const int row = rowid[b1];
                const double v = R2[e];
                if (row >= 0 && nonzero(v))
                    atomicAdd(a.od + row * ld + (int64_t)pr.x * N + b2, 2.0 * v * om2[b2] * inv1[b1]);
            } else {
                const int e3 = e - N2, b1 = e3 / N, b3 = e3 % N;
                const int row = rowid[b1];
                const double v = R3[e3];
                if (row >= 0 && nonzero(v))
                    atomicAdd(a.od + row * ld + (int64_t)pr.y * N + b3, 2.0 * v * om3[b3] * inv1[b1]);
            }
        }
        __syncthreads();
    }
}

template <int N, typename R>
cudaError_t launch_n(const ThreePhArgs &a, int n_sm, cudaStream_t s) {
    const Layout L = make_layout(N, sizeof(typename CT<R>::C));
    const int threads = ((N * N + 31) / 32) * 32;
    cudaError_t e = cudaFuncSetAttribute(k_threephonon<N, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)L.total);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_threephonon<N, R>, threads, L.total);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int grid = n_sm * per_sm;
    if (grid > a.n_trip) grid = a.n_trip;
    if (grid < 1) return cudaSuccess;
    k_threephonon<N, R><<<grid, threads, L.total, s>>>(a);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_prec(const ThreePhArgs &a, int n_sm, cudaStream_t s) {
    switch (a.mesh.n_mode) {
        case 3: return launch_n<3, R>(a, n_sm, s);
        case 6: return launch_n<6, R>(a, n_sm, s);
        case 9: return launch_n<9, R>(a, n_sm, s);
        case 12: return launch_n<12, R>(a, n_sm, s);
        case 15: return launch_n<15, R>(a, n_sm, s);
        case 18: return launch_n<18, R>(a, n_sm, s);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace

size_t threephonon_smem_bytes(int n, int precision, int) {
    return make_layout(n, precision == 0 ? sizeof(double2) : sizeof(float2)).total;
}

cudaError_t launch_threephonon(const ThreePhArgs &a, int precision, int n_sm, cudaStream_t s) {
    if (a.n_trip <= 0) return cudaSuccess;
    if (precision == 0) return launch_prec<double>(a, n_sm, s);
    return launch_prec<float>(a, n_sm, s);
}

}  // namespace tdg
