// Isotope scattering, the two scattering-matrix symmetrisations and the BTE product.
#include <cuda_runtime.h>

#include <algorithm>

#include "dev_common.cuh"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr double kIsotopePrefactor = 3.141592653589793 / 4.0;

__device__ __forceinline__ double lo_gauss(double x, double mu, double sigma) {
    if (fabs(x - mu) > 8.0 * sigma) return 0.0;
    const double invsig = 1.0 / sigma;
    return exp(-(x - mu) * (x - mu) * 0.5 * invsig * invsig) * kSqrt2PiInv * invsig;
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)((blockDim.x + 31) / 32); ++i) s += sh[i];
    __syncthreads();
    return s;
}

// compute_isotope_scattering (scattering_isotope.f90:1-91): one thread per (q2, b2) of a row.
__global__ void k_isotope(MeshDev m, PhononDev ph, RowsDev rows, const int32_t *row_q1, const int32_t *row_b1,
                          const double *disorder, int32_t n_atom, double *gamma, double *xi) {
    __shared__ double sh[32];
    const int n = m.n_mode;
    const int r = blockIdx.y;
    const int q1 = row_q1[r], b1 = row_b1[r];
    const int f1 = m.irr_full[q1];
    const int64_t ld = (int64_t)m.n_full * n;
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double f0 = 0.0;
    if (j < ld) {
        const int q2 = (int)(j / n), b2 = (int)(j % n);
        const double om1 = ph.omega[(size_t)f1 * n + b1];
        const double om2 = ph.omega[(size_t)q2 * n + b2];
        if (!(om2 < kFreqTolD)) {
            double sigma;
            if (ph.integrationtype == 1) {
                sigma = ph.sigma_fixed;
            } else if (ph.integrationtype == 2) {
                sigma = sqrt(ph.sigsq[(size_t)q1 * n + b1] + ph.sigsq[(size_t)m.full_irr[q2] * n + b2]);
            } else {
                const double *v = ph.vel + ((size_t)q2 * n + b2) * 3;
                double mx = 0.0;
                for (int jj = 0; jj < 3; ++jj) {
                    double s = 0.0;
                    for (int i = 0; i < 3; ++i) s += v[i] * ph.reclat_g[i + 3 * jj];
                    mx = fmax(mx, s * s);
                }
                sigma = sqrt(mx * 0.5) + ph.thresh_sigma;
            }
            const double2 *e1 = ph.egv + ((size_t)f1 * n + b1) * n;
            const double2 *e2 = ph.egv + ((size_t)q2 * n + b2) * n;
            double f1s = 0.0;
            for (int a = 0; a < n_atom; ++a) {
                double fa = 0.0;
                for (int x = 0; x < 3; ++x) {
                    const double2 u = e1[a * 3 + x], v = e2[a * 3 + x];
                    // |conjg(u) * v|
                    const double re = u.x * v.x + u.y * v.y, im = u.x * v.y - u.y * v.x;
                    fa += sqrt(re * re + im * im);
                }
                fa = fa * fa;
                f1s += fa * disorder[a];
            }
            const double prefactor = kIsotopePrefactor * (1.0 / (double)m.n_full);
            const double psisq = f1s * prefactor;
            f0 = psisq * om1 * om2 * lo_gauss(om1, om2, sigma);
            if (f0 != 0.0) xi[(int64_t)r * ld + j] += f0 * om2 / om1;
        }
    }
    const double s = block_sum(f0, sh);
    if (threadIdx.x == 0 && s != 0.0) atomicAdd(gamma + r, s);
}

// symmetrize_and_distribute (scattering_threephonon.f90:143-205, scattering_fourphonon.f90:195-250).
// Orbit tables of the little group of every irreducible q1, built once per mesh: q2 is a
// representative when no on-grid image is smaller (the reference's "cycle allq2" rule);
// its images are kept in operation order, -1 for operations that leave the grid.
__global__ void k_orbit_flag(MeshDev m, int32_t *flag) {
    const int q2 = blockIdx.x * blockDim.x + threadIdx.x;
    const int q1 = blockIdx.y;
    if (q2 >= m.n_full) return;
    const int nop = m.irr_nop[q1];
    const int32_t *ops = m.irr_ops + (size_t)q1 * m.n_op;
    int rep = 1;
    for (int j = 0; j < nop; ++j) {
        const int q2p = m.rot[(size_t)ops[j] * m.n_full + q2];
        if (q2p >= 0 && q2p < q2) {
            rep = 0;
            break;
        }
    }
    flag[(size_t)q1 * m.n_full + q2] = rep;
}

// Images are stored once each, in order of first appearance over the operations, with
// their multiplicity (operations that map q2 to the same point); cnt counts every
// on-grid operation, as the reference's averages do.
__global__ void k_orbit_fill(MeshDev m, const int32_t *flag, const int32_t *scan, OrbitDev o) {
    const int q2 = blockIdx.x * blockDim.x + threadIdx.x;
    const int q1 = blockIdx.y;
    if (q2 >= m.n_full) return;
    const size_t i = (size_t)q1 * m.n_full + q2;
    int32_t *orb_of = const_cast<int32_t *>(o.orb_of);
    if (!flag[i]) {
        orb_of[i] = -1;
        return;
    }
    const int k = scan[i];
    orb_of[i] = k;
    const_cast<int32_t *>(o.rep)[k] = q2;
    const int nop = m.irr_nop[q1];
    const int32_t *ops = m.irr_ops + (size_t)q1 * m.n_op;
    int32_t *img = const_cast<int32_t *>(o.img) + (size_t)k * m.n_op;
    int32_t *mult = const_cast<int32_t *>(o.mult) + (size_t)k * m.n_op;
    int c = 0, nu = 0;
    for (int j = 0; j < nop; ++j) {
        const int q2p = m.rot[(size_t)ops[j] * m.n_full + q2];
        if (q2p < 0) continue;
        ++c;
        int u = 0;
        while (u < nu && img[u] != q2p) ++u;
        if (u == nu) {
            img[nu] = q2p;
            mult[nu] = 0;
            ++nu;
        }
        ++mult[u];
    }
    const_cast<int32_t *>(o.cnt)[k] = c;
    const_cast<int32_t *>(o.nuniq)[k] = nu;
}

__device__ __forceinline__ bool positive(double v) { return __double_as_longlong(v) > 0; }  // v > 0, v not NaN

// symmetrize_and_distribute (scattering_threephonon.f90:143-205, scattering_fourphonon.f90:195-250)
// in place on one row per CTA: for every sampled q2 that represents its orbit, each mode's
// entries with od > 0 are averaged over the on-grid operations (images counted with their
// multiplicity) and the average is written to every image. Orbits are disjoint, so
// threads never touch the same entries; a bitmap ignores repeated entries of a sample
// (the reference would process them again to the same result).
// When xi != nullptr the symmetrised row is then added to xi.
__global__ void k_sym_distribute(MeshDev m, OrbitDev o, const int32_t *row_q1, const int64_t *rbeg,
                                 const int32_t *rlen, const int32_t *list, double *od, double *xi) {
    extern __shared__ uint32_t seen[];
    const int n = m.n_mode;
    const int r = blockIdx.x;
    const int q1 = row_q1[r];
    const int64_t ld = (int64_t)m.n_full * n;
    double *odr = od + (int64_t)r * ld;
    const int nw = (m.n_full + 31) / 32;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) seen[i] = 0u;
    __syncthreads();
    for (int64_t qi = rbeg[r] + threadIdx.x; qi < rbeg[r] + rlen[r]; qi += blockDim.x) {
        const int q2 = list[qi] - 1;
        const int k = o.orb_of[(size_t)q1 * m.n_full + q2];
        if (k < 0) continue;
        const uint32_t bit = 1u << (q2 & 31);
        if (atomicOr(&seen[q2 >> 5], bit) & bit) continue;
        const int32_t *im = o.img + (size_t)k * m.n_op;
        const int32_t *mu = o.mult + (size_t)k * m.n_op;
        const int nu = o.nuniq[k];
        for (int b2 = 0; b2 < n; ++b2) {
            double buf = 0.0;
            int nn = 0;
            for (int u = 0; u < nu; ++u) {
                const double v = odr[(int64_t)im[u] * n + b2];
                if (positive(v)) {
                    nn += mu[u];
                    for (int rep = 0; rep < mu[u]; ++rep) buf += v;
                }
            }
            if (nn == 0) continue;
            const double avg = buf * o.rcp[nn];
            for (int u = 0; u < nu; ++u) odr[(int64_t)im[u] * n + b2] = avg;
        }
    }
    if (xi == nullptr) return;
    __syncthreads();
    double *xr = xi + (int64_t)r * ld;
    for (int64_t j = threadIdx.x; j < ld; j += blockDim.x) xr[j] += odr[j];
}

// Both row symmetrisations on tiles of whole orbits: symmetrize_and_distribute of the
// three-phonon terms (scattering_threephonon.f90:143-205; only orbits whose representative
// the row sampled, entries > 0 averaged) and symmetrize_scatmat (scattering.f90:296-357;
// every orbit, all entries). A CTA takes K = min(256, T / |G_q1|) consecutive orbits of its
// row's q1 (at most T points), gathers their images' n modes into shared memory with
// independent loads, averages there (each image weighted by its mult with one FMA, in
// first-appearance order: the reference adds it mult times, which differs in the last bit)
// and writes the images back. With both passes in one kernel Xi crosses HBM once instead of
// twice. q1 whose little group is the identity
// alone are skipped: every orbit is one point with count 1, and both averages return it.
__global__ void __launch_bounds__(256) k_sym_tile(MeshDev m, OrbitDev o, const int32_t *row_q1, double *xi,
                                                  const uint32_t *sbits, int do_dist, int do_scat) {
    extern __shared__ double sym_sm[];
    __shared__ int wsum[8];
    const int n = m.n_mode, T = o.tile_pts;
    const int r = blockIdx.y, q1 = row_q1[r];
    const int nop = m.irr_nop[q1];
    if (nop <= 1) return;
    const int K = min(256, T / nop);
    const int kb = o.rep_ptr[q1], ke = o.rep_ptr[q1 + 1];
    const int k0 = kb + blockIdx.x * K;
    if (k0 >= ke) return;
    const int nk = min(K, ke - k0);
    double *vals = sym_sm;                                 // [T][n]
    double *pmud = vals + (size_t)T * n;                   // [T] multiplicity as a double
    int *pts = (int *)(pmud + T);                          // [T] image of each position
    int *pmu = pts + T;                                    // [T] its multiplicity
    int *off = pmu + T;                                    // [257] first position of each orbit
    const int tid = threadIdx.x;
    const int nu_t = tid < nk ? o.nuniq[k0 + tid] : 0;
    int P = 0;
    const int my = block_exclusive_scan(nu_t, wsum, P);
    if (tid < nk) {
        off[tid] = my;
        const int32_t *im = o.img + (size_t)(k0 + tid) * m.n_op;
        const int32_t *mu = o.mult + (size_t)(k0 + tid) * m.n_op;
        for (int u = 0; u < nu_t; ++u) {
            pts[my + u] = im[u];
            pmu[my + u] = mu[u];
            pmud[my + u] = (double)mu[u];  // converted once per image, not once per mode
        }
    }
    if (tid == 0) off[nk] = P;
    __syncthreads();
    double *xr = xi + (int64_t)r * m.n_full * n;
    // gather: eight independent loads in flight per thread before their stores (one load
    // per loop trip left each thread waiting on one gather at a time); p = e / n through
    // the float reciprocal, exact here (e < 2^13, and (e + 0.5) / n is at least 0.5 / n
    // from an integer)
    const int tot = P * n;
    const float inv_n = 1.0f / (float)n;
    constexpr int kGather = 8;
    for (int e0 = tid; e0 < tot; e0 += kGather * blockDim.x) {
        double v[kGather];
#pragma unroll
        for (int u = 0; u < kGather; ++u) {
            const int e = e0 + u * blockDim.x;
            const int p = (int)(((float)e + 0.5f) * inv_n), b2 = e - p * n;
            v[u] = e < tot ? xr[(int64_t)pts[p < P ? p : 0] * n + b2] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kGather; ++u) {
            const int e = e0 + u * blockDim.x;
            if (e < tot) vals[e] = v[u];
        }
    }
    __syncthreads();
    const uint32_t *bits = sbits ? sbits + (size_t)r * ((m.n_full + 31) / 32) : nullptr;
    for (int it = tid; it < nk * n; it += blockDim.x) {
        const int t = it / n, b2 = it - t * n, k = k0 + t;
        const int p0 = off[t], p1 = off[t + 1];
        // Each image enters a sum once per operation that gives it: one FMA with its mult,
        // converted to double once per image (conversions run on the FP64 pipe too: the sums
        // are FP64 on a pipe of 2 operations per clock per SM, the bound of this kernel).
        bool averaged = false;
        if (do_dist) {
            const int q2 = o.rep[k];
            if ((bits[q2 >> 5] >> (q2 & 31)) & 1u) {
                double buf = 0.0;
                int nn = 0;
                for (int p = p0; p < p1; ++p) {
                    const double v = vals[p * n + b2];
                    if (__double_as_longlong(v) > 0) {  // v > 0, v not NaN
                        nn += pmu[p];
                        buf = fma(v, pmud[p], buf);
                    }
                }
                if (nn) {
                    const double avg = buf * o.rcp[nn];
                    for (int p = p0; p < p1; ++p) vals[p * n + b2] = avg;
                    averaged = true;
                }
            }
        }
        // symmetrize_scatmat: the mean over the operations, cnt = sum of mult; on an orbit the
        // distribution just set to one value that mean is the value itself
        if (do_scat && !averaged) {
            const int cnt = o.cnt[k];
            if (cnt) {
                double buf = 0.0;
                for (int p = p0; p < p1; ++p) buf = fma(vals[p * n + b2], pmud[p], buf);
                buf *= o.rcp[cnt];
                for (int p = p0; p < p1; ++p) vals[p * n + b2] = buf;
            }
        }
    }
    __syncthreads();
    for (int e = tid; e < tot; e += blockDim.x) {
        const int p = (int)(((float)e + 0.5f) * inv_n), b2 = e - p * n;
        xr[(int64_t)pts[p] * n + b2] = vals[e];
    }
}

// Bitmap of the q-points each row sampled, [n_row][ceil(n_full/32)] words, built in shared
// memory (dynamic, nw words) and written out once.
__global__ void k_sample_bits(int32_t n_full, const int64_t *rbeg, const int32_t *rlen, const int32_t *list,
                              uint32_t *bits) {
    extern __shared__ uint32_t sb[];
    const int r = blockIdx.x, nw = (n_full + 31) / 32;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) sb[i] = 0u;
    __syncthreads();
    for (int64_t i = rbeg[r] + threadIdx.x; i < rbeg[r] + rlen[r]; i += blockDim.x) {
        const int q2 = list[i] - 1;
        atomicOr(sb + (q2 >> 5), 1u << (q2 & 31));
    }
    __syncthreads();
    uint32_t *br = bits + (size_t)r * nw;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) br[i] = sb[i];
}

// K8: three dot products per row of Xi (kappa.f90:411-413, the lo_gemv calls).
// Xi streams from HBM once per BTE iteration; F (3 x n_col) stays in L2. GB300's FP64 pipe
// (2 FMA per SM and clock) would make an FP64 product with three right-hand sides
// compute-bound at ~1.2 TB/s of Xi, so the product runs on the FP32 pipe: Xi and F as
// (hi, lo) float pairs with hi + lo = x to ~2^-48 (converted once per kappa call, k_split_xi,
// and per iteration for F, k_foldout), each term accumulated in double-float (exact leading
// product by FMA, cross terms, TwoSum of the high parts); ~1e-14 relative, the bytes of FP64.
// The rows go in pairs: pair p and column j are one float4 (hi of rows 2p and 2p + 1, lo of
// both), so that the double-float arithmetic of the two rows runs in the packed FP32x2
// instructions (__ffma2_rn, __fadd2_rn, __fmul2_rn: per component the scalar IEEE operation),
// half the instructions of the scalar form, which left the product issue-bound at 0.58 of
// the copy peak.
// Floats for Xi (half the bytes) were the mixed-precision format until they failed the
// convergence test: the modes whose F is zero by symmetry (v = 0 at a high-symmetry point)
// carry 1e-7 of the typical |F| from the rounding of Xi, above the test's lo_sqtol floor,
// and their relative change kept the sum of the last three checks above 1e-6 (rocksalt took
// 200 iterations, the limit, instead of 31-33, with kappa already converged).
// A CTA takes PAIRS row pairs (2 or 4, autotuned) and one of the column ranges (gridDim.y):
// each F value read from L2 serves 2 PAIRS rows. Partial sums go to part[row][range][3]
// (FP64) and are added in range order by k_xi_reduce, so the result does not depend on
// scheduling. The in-CTA reduction stays in double-float too: FP64 shuffles and adds in
// every CTA's epilogue cost more than the product itself once there are more than a few
// ranges.
constexpr int kGemvRows = 4;
constexpr int kGemvMaxSplit = 32;

// Ranges of at most 32768 columns, and enough CTAs for about two waves of 4 per SM.
int gemv_split(int32_t n_row, int64_t n_col, int n_sm) {
    const int64_t groups = (n_row + kGemvRows - 1) / kGemvRows;
    int64_t k = (n_col + 32767) / 32768;
    const int64_t w = (8 * (int64_t)n_sm + groups - 1) / groups;
    if (w > k) k = w;
    if (k > n_col / 256) k = n_col / 256;
    return (int)(k < 1 ? 1 : (k > kGemvMaxSplit ? kGemvMaxSplit : k));
}

// x = hi + lo by integer operations on the bits (double <-> float conversions run on the
// FP64 pipe): hi keeps the leading 24 significant bits of x, lo the remaining 29 rounded to
// 24, so hi + lo = x to 2^-48 relative. Zero and subnormal doubles give 0; magnitudes
// outside [2^-74, 2^127) take the FP64 conversions.
__device__ __forceinline__ float2 split_df(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e == 0) return make_float2(0.f, 0.f);
    if (e < 949 || e > 1150) {
        const float h = (float)x;
        return make_float2(h, (float)(x - (double)h));
    }
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    const float hi = __uint_as_float(sign | ((unsigned int)(e - 896) << 23) | (unsigned int)((b >> 29) & 0x7FFFFFu));
    // remainder r * 2^(e - 1075), r < 2^29; the power of two is a normal float for e >= 949
    const float lo = __uint2float_rn((unsigned int)(b & 0x1FFFFFFFu)) * __uint_as_float((unsigned int)(e - 948) << 23);
    return make_float2(hi, sign ? -lo : lo);
}

// (a.x + a.y) + (b.x + b.y) in double-float (TwoSum of the high parts)
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float t = a.x + b.x;
    const float bb = t - a.x;
    const float e = (a.x - (t - bb)) + (b.x - bb);
    return make_float2(t, a.y + b.y + e);
}

// Two double-float accumulators (s, sl: high and low parts of rows 2p and 2p + 1) += x * f
// for the two rows' elements (x, xl) and one F value (f, fl, the same in both components);
// nx = -x. The scalar form per component: p = x f, pe = fma(x, f, -p), cross = fma(x, fl,
// xl f), TwoSum of s and p, sl += (e + pe) + cross. A subtraction a - b is fma(b, -1, a),
// rounded once as a - b is.
__device__ __forceinline__ void df2_fma(float2 &s, float2 &sl, float2 x, float2 nx, float2 xl, float2 f, float2 fl) {
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 p = __fmul2_rn(x, f);
    const float2 npe = __ffma2_rn(nx, f, p);  // p - x f = -pe exactly
    const float2 cross = __ffma2_rn(x, fl, __fmul2_rn(xl, f));
    const float2 t = __fadd2_rn(s, p);
    const float2 bb = __ffma2_rn(s, m1, t);                        // t - s
    const float2 e1 = __ffma2_rn(__ffma2_rn(bb, m1, t), m1, s);    // s - (t - bb)
    const float2 e = __fadd2_rn(e1, __ffma2_rn(bb, m1, p));       // + (p - bb)
    s = t;
    sl = __fadd2_rn(sl, __fadd2_rn(__ffma2_rn(npe, m1, e), cross));  // sl + ((e + pe) + cross)
}

// Xi as double-float row pairs: pair p, column j at p * n_col + j as (hi of row 2p, hi of
// row 2p + 1, lo of row 2p, lo of row 2p + 1); an odd last row pairs with a zero row.
__global__ void k_split_xi(const double *xi, int32_t n_row, int64_t n_col, float4 *out) {
    const int n_pair = (n_row + 1) / 2;
    for (int p = blockIdx.y; p < n_pair; p += gridDim.y) {
        const double *r0 = xi + (int64_t)(2 * p) * n_col;
        const bool two = 2 * p + 1 < n_row;
        for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_col; j += (int64_t)gridDim.x * blockDim.x) {
            const float2 a = split_df(__ldcs(r0 + j));
            const float2 b = two ? split_df(__ldcs(r0 + n_col + j)) : make_float2(0.f, 0.f);
            out[(int64_t)p * n_col + j] = make_float4(a.x, b.x, a.y, b.y);
        }
    }
}

template <int PAIRS>
__global__ void __launch_bounds__(256) k_xi_gemv(const float4 *__restrict__ xi, int32_t n_row, int64_t n_col,
                                                 const float2 *__restrict__ fbb, double *part, const int32_t *skip) {
    __shared__ float2 sh[2 * PAIRS * 3][8];
    if (skip && *skip) return;
    const int p0 = blockIdx.x * PAIRS;
    const int np = min(PAIRS, (n_row + 1) / 2 - p0);
    const int r0 = 2 * p0, nr = min(2 * PAIRS, n_row - r0);
    const int64_t per = ((n_col + gridDim.y - 1) / gridDim.y + 7) / 8 * 8;
    const int64_t c0 = min(n_col, per * blockIdx.y), c1 = min(n_col, c0 + per);
    float2 ah[PAIRS][3], al[PAIRS][3];
#pragma unroll
    for (int k = 0; k < PAIRS; ++k)
#pragma unroll
        for (int d = 0; d < 3; ++d) ah[k][d] = al[k][d] = make_float2(0.f, 0.f);
    const float4 *xr[PAIRS];
#pragma unroll
    for (int k = 0; k < PAIRS; ++k) xr[k] = xi + (int64_t)(p0 + min(k, np - 1)) * n_col;
    const int64_t step = blockDim.x;
    int64_t j = c0 + threadIdx.x;
    auto column = [&](const float4 (&x)[PAIRS], int64_t jj) {
        float2 fh[3], fl[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float2 t = __ldg(fbb + jj * 3 + d);
            fh[d] = make_float2(t.x, t.x);
            fl[d] = make_float2(t.y, t.y);
        }
#pragma unroll
        for (int k = 0; k < PAIRS; ++k) {
            const float2 xh = make_float2(x[k].x, x[k].y), xl = make_float2(x[k].z, x[k].w);
            const float2 nx = make_float2(-x[k].x, -x[k].y);
#pragma unroll
            for (int d = 0; d < 3; ++d) df2_fma(ah[k][d], al[k][d], xh, nx, xl, fh[d], fl[d]);
        }
    };
    // four columns per thread and trip: 4 PAIRS 16-byte loads in flight
    for (; j + 3 * step < c1; j += 4 * step) {
        float4 x[4][PAIRS];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int k = 0; k < PAIRS; ++k)
                x[u][k] = k < np ? __ldcs(xr[k] + j + u * step) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < 4; ++u) column(x[u], j + u * step);
    }
    for (; j < c1; j += step) {
        float4 x[PAIRS];
#pragma unroll
        for (int k = 0; k < PAIRS; ++k) x[k] = k < np ? __ldcs(xr[k] + j) : make_float4(0.f, 0.f, 0.f, 0.f);
        column(x, j);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 2 * PAIRS; ++k)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float2 hp = ah[k / 2][d], lp = al[k / 2][d];
            float2 v = (k & 1) ? make_float2(hp.y, lp.y) : make_float2(hp.x, lp.x);
            for (int o = 16; o > 0; o >>= 1) {
                float2 u;
                u.x = __shfl_down_sync(0xffffffffu, v.x, o);
                u.y = __shfl_down_sync(0xffffffffu, v.y, o);
                v = df_add(v, u);
            }
            if (lane == 0) sh[k * 3 + d][w] = v;
        }
    __syncthreads();
    if (threadIdx.x < nr * 3) {
        float2 v = sh[threadIdx.x][0];
        for (int i = 1; i < 8; ++i) v = df_add(v, sh[threadIdx.x][i]);
        const int k = threadIdx.x / 3, d = threadIdx.x % 3;
        part[((int64_t)(r0 + k) * gridDim.y + blockIdx.y) * 3 + d] = (double)v.x + (double)v.y;
    }
}

__global__ void k_xi_reduce(const double *part, int32_t n_row, int split, double *buf, const int32_t *skip) {
    if (skip && *skip) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_row * 3) return;
    const int r = i / 3, d = i % 3;
    double v = 0.0;
    for (int c = 0; c < split; ++c) v += part[((int64_t)r * split + c) * 3 + d];
    buf[i] = v;
}

}  // namespace

cudaError_t launch_isotope(const MeshDev &m, const PhononDev &ph, const RowsDev &rows, const int32_t *row_q1,
                           const int32_t *row_b1, const double *disorder, int32_t n_atom, double *gamma,
                           double *xi, cudaStream_t s) {
    if (rows.n_row <= 0) return cudaSuccess;
    const int64_t ld = (int64_t)m.n_full * m.n_mode;
    dim3 grid((unsigned)((ld + 255) / 256), (unsigned)rows.n_row);
    k_isotope<<<grid, 256, 0, s>>>(m, ph, rows, row_q1, row_b1, disorder, n_atom, gamma, xi);
    return cudaGetLastError();
}

namespace {
__global__ void k_rep_ptr(const int32_t *scan, int32_t n_irr, int32_t n_full, int32_t *rep_ptr) {
    const int q1 = blockIdx.x * blockDim.x + threadIdx.x;
    if (q1 <= n_irr) rep_ptr[q1] = scan[(size_t)q1 * n_full];
}
}  // namespace

cudaError_t launch_orbit_flag(const MeshDev &m, int32_t *flag, cudaStream_t s) {
    dim3 grid((unsigned)((m.n_full + 127) / 128), (unsigned)m.n_irr);
    k_orbit_flag<<<grid, 128, 0, s>>>(m, flag);
    return cudaGetLastError();
}

cudaError_t launch_orbit_fill(const MeshDev &m, const int32_t *flag, const int32_t *scan, OrbitDev &o,
                              cudaStream_t s) {
    dim3 grid((unsigned)((m.n_full + 127) / 128), (unsigned)m.n_irr);
    k_orbit_fill<<<grid, 128, 0, s>>>(m, flag, scan, o);
    k_rep_ptr<<<(m.n_irr + 1 + 127) / 128, 128, 0, s>>>(scan, m.n_irr, m.n_full, const_cast<int32_t *>(o.rep_ptr));
    return cudaGetLastError();
}

cudaError_t launch_sym_distribute(const MeshDev &m, const OrbitDev &o, int32_t n_row, const int32_t *row_q1,
                                  const int64_t *rbeg, const int32_t *rlen, const int32_t *list, double *od, double *xi,
                                  cudaStream_t s) {
    if (n_row <= 0) return cudaSuccess;
    const size_t sm = sizeof(uint32_t) * (size_t)((m.n_full + 31) / 32);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_sym_distribute, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    k_sym_distribute<<<n_row, 256, sm, s>>>(m, o, row_q1, rbeg, rlen, list, od, xi);
    return cudaGetLastError();
}

int sym_tile_points(int n_mode) {
    const int t = 4096 / (n_mode > 0 ? n_mode : 1);
    return t < 64 ? 64 : (t > 1024 ? 1024 : t);
}

size_t sym_tile_smem(int n_mode) {
    const int T = sym_tile_points(n_mode);
    return sizeof(double) * (size_t)T * (n_mode + 1) + sizeof(int) * (2 * (size_t)T + 257);
}

int sym_tile_count(int n_rep, int n_ops, int n_mode) {
    if (n_ops <= 1 || n_rep <= 0) return 0;
    int K = sym_tile_points(n_mode) / n_ops;
    K = K > 256 ? 256 : K;
    return (n_rep + K - 1) / K;
}

cudaError_t launch_sample_bits(int32_t n_full, int32_t n_row, const int64_t *rbeg, const int32_t *rlen,
                               const int32_t *list, uint32_t *bits, cudaStream_t s) {
    if (n_row <= 0) return cudaSuccess;
    const size_t sm = sizeof(uint32_t) * (size_t)((n_full + 31) / 32);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_sample_bits, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    k_sample_bits<<<n_row, 256, sm, s>>>(n_full, rbeg, rlen, list, bits);
    return cudaGetLastError();
}

cudaError_t launch_sym_tile(const MeshDev &m, const OrbitDev &o, int32_t n_row, const int32_t *row_q1, double *xi,
                            const uint32_t *sbits, bool dist, bool scat, cudaStream_t s) {
    if (n_row <= 0 || o.max_tiles <= 0 || (!dist && !scat)) return cudaSuccess;
    const size_t sm = sym_tile_smem(m.n_mode);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_sym_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    dim3 grid((unsigned)o.max_tiles, (unsigned)n_row);
    k_sym_tile<<<grid, 256, sm, s>>>(m, o, row_q1, xi, sbits, dist ? 1 : 0, scat ? 1 : 0);
    return cudaGetLastError();
}

// foldout (kappa.f90:382-404): F of every full-mesh point from its irreducible point,
// Fbb(q, b) = sign(op) * R_|op| Fn(irr(q), b) as double-float pairs, one thread per (q, b).
__global__ void k_foldout(int32_t n_full, int32_t n_mode, const int32_t *full_op, const int32_t *full_irr,
                          const double *op_cart, const double *fn, float2 *fbb, const int32_t *skip) {
    if (skip && *skip) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n_full * n_mode) return;
    const int iq = (int)(i / n_mode), b = (int)(i % n_mode);
    const int iop = full_op[iq];
    const double *m = op_cart + 9 * (abs(iop) - 1);
    const double *v = fn + ((int64_t)full_irr[iq] * n_mode + b) * 3;
    const double sg = iop > 0 ? 1.0 : -1.0;
    for (int d = 0; d < 3; ++d) fbb[i * 3 + d] = split_df(sg * (m[d] * v[0] + m[d + 3] * v[1] + m[d + 6] * v[2]));
}

cudaError_t launch_foldout(int32_t n_full, int32_t n_mode, const int32_t *full_op, const int32_t *full_irr,
                           const double *op_cart, const double *fn, float2 *fbb, cudaStream_t s, const int32_t *skip) {
    const int64_t n = (int64_t)n_full * n_mode;
    if (n <= 0) return cudaSuccess;
    k_foldout<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n_full, n_mode, full_op, full_irr, op_cart, fn, fbb, skip);
    return cudaGetLastError();
}

size_t xi_gemv_part_elems(int32_t n_row) { return (size_t)n_row * kGemvMaxSplit * 3; }

size_t xi_pairs_elems(int32_t n_row, int64_t n_col) { return (size_t)((n_row + 1) / 2) * (size_t)n_col; }

cudaError_t launch_split_xi(const double *xi, int32_t n_row, int64_t n_col, float4 *out, cudaStream_t s) {
    if (n_row <= 0 || n_col <= 0) return cudaSuccess;
    const int n_pair = (n_row + 1) / 2;
    const int64_t bx = (n_col + 255) / 256;
    dim3 grid((unsigned)(bx < 64 ? bx : 64), (unsigned)(n_pair < 65535 ? n_pair : 65535));
    k_split_xi<<<grid, 256, 0, s>>>(xi, n_row, n_col, out);
    return cudaGetLastError();
}

int xi_gemv_default_split(int32_t n_row, int64_t n_col, int n_sm) { return gemv_split(n_row, n_col, n_sm); }

int xi_gemv_max_split(int64_t n_col) {
    const int64_t k = n_col / 256;
    return (int)(k < 1 ? 1 : (k > kGemvMaxSplit ? kGemvMaxSplit : k));
}

cudaError_t launch_xi_gemv(const float4 *xi, int32_t n_row, int64_t n_col, const float2 *fbb, double *part,
                           double *buf, int n_sm, cudaStream_t s, const int32_t *skip, int shape) {
    if (n_row <= 0) return cudaSuccess;
    // shape = rows per CTA * 100 + column ranges; 0: 4 rows and the default split
    int rows = shape / 100, split = shape % 100;
    if (rows != 8) rows = 4;
    if (split <= 0) split = gemv_split(n_row, n_col, n_sm);
    split = std::min(split, xi_gemv_max_split(n_col));
    dim3 grid((unsigned)((n_row + rows - 1) / rows), (unsigned)split);
    if (rows == 8)
        k_xi_gemv<4><<<grid, 256, 0, s>>>(xi, n_row, n_col, fbb, part, skip);
    else
        k_xi_gemv<2><<<grid, 256, 0, s>>>(xi, n_row, n_col, fbb, part, skip);
    k_xi_reduce<<<(n_row * 3 + 255) / 256, 256, 0, s>>>(part, n_row, split, buf, skip);
    return cudaGetLastError();
}

namespace {
// One BTE iteration's scalar part (kappa.f90:407-490) after the products buf = Xi . Fbb, in
// three kernels spread over the SMs (GB300's FP64 rate on a single SM, 2 operations per
// clock, made a one-CTA version take 80 us for the divisions alone):
//   k_bte_apply  applyXi: Fnb = -buf / qs for every (q1, b1) with a row, else 0;
//   k_bte_mix    per q1 (8 per CTA): distributeF (degeneracy average in the reference's in-place order,
//                then + F0) and addandcheck (relative change, mixing into Fn), partial sums
//                of the change per CTA;
//   k_bte_check  the change summed in a fixed order into scf, the convergence test on the
//                last three values, the mixing schedule, the done flag.
// Every kernel of an iteration returns at once when done is set.
// q1 per CTA of k_bte_mix (one warp, the other lanes idle): few per CTA spreads the FP64
// divisions over many SMs.
constexpr int kBteMixQ = 8;

__global__ void k_bte_apply(BteDev d, const double *buf) {
    if (d.ctl->done) return;
    const int n = d.n_mode;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n_irr * n) return;
    const int r = d.rowidx[i];
    const double q = d.qs[i];
    for (int x = 0; x < 3; ++x)
        d.fnb[(size_t)i * 3 + x] = (r < 0 || q < kFreqTolD) ? 0.0 : -buf[(size_t)r * 3 + x] / q;
}

__global__ void k_bte_mix(BteDev d) {
    __shared__ double red[32];
    extern __shared__ double sm_mix[];  // Fnb, F0 and Fn of the CTA's kBteMixQ points
    if (d.ctl->done) return;
    const int n = d.n_mode, tid = threadIdx.x, bd = blockDim.x;
    const int q0 = blockIdx.x * kBteMixQ, nq = min(kBteMixQ, d.n_irr - q0);
    const int m = nq * n * 3;
    double *fbs = sm_mix, *f0s = sm_mix + kBteMixQ * n * 3, *fns = f0s + kBteMixQ * n * 3;
    const size_t base = (size_t)q0 * n * 3;
    for (int i = tid; i < m; i += bd) {
        fbs[i] = d.fnb[base + i];
        f0s[i] = d.F0[base + i];
        fns[i] = d.fn[base + i];
    }
    __syncthreads();
    const double mixing = d.ctl->mixing;
    double g0 = 0.0;
    if (tid < nq) {
        const int q1 = q0 + tid;
        double *fb = fbs + tid * n * 3;
        const double *f0 = f0s + tid * n * 3;
        for (int b1 = 0; b1 < n; ++b1) {
            const int dg = d.degen[q1 * n + b1];
            const int32_t *dm = d.degen_mode + ((size_t)q1 * n + b1) * n;
            double v0[3] = {0.0, 0.0, 0.0};
            for (int j = 0; j < dg; ++j)
                for (int x = 0; x < 3; ++x) v0[x] += fb[(dm[j] - 1) * 3 + x];
            if (dg != 1)
                for (int x = 0; x < 3; ++x) v0[x] /= (double)dg;
            for (int j = 0; j < dg; ++j)
                for (int x = 0; x < 3; ++x) fb[(dm[j] - 1) * 3 + x] = v0[x];
            for (int x = 0; x < 3; ++x) fb[b1 * 3 + x] = f0[b1 * 3 + x] + fb[b1 * 3 + x];
        }
        double *fn = fns + tid * n * 3;
        for (int b1 = 0; b1 < n; ++b1) {
            double *v = fn + b1 * 3;
            const double *f = fb + b1 * 3;
            double g1 = 0.0, g2 = 0.0;
            for (int x = 0; x < 3; ++x) {
                g1 += (v[x] - f[x]) * (v[x] - f[x]);
                g2 += v[x] * v[x];
            }
            if (g2 > d.sqtol) g0 += g1 / g2;
            for (int x = 0; x < 3; ++x) v[x] = v[x] * (1.0 - mixing) + mixing * f[x];
        }
    }
    __syncthreads();
    for (int i = tid; i < m; i += bd) d.fn[base + i] = fns[i];
    for (int o = 16; o > 0; o >>= 1) g0 += __shfl_xor_sync(0xffffffffu, g0, o);
    if ((tid & 31) == 0) red[tid >> 5] = g0;
    __syncthreads();
    if (tid == 0) {
        double g = 0.0;
        for (int w = 0; w < (bd >> 5); ++w) g += red[w];
        d.part[blockIdx.x] = g;
    }
}

__global__ void k_bte_check(BteDev d, int n_part) {
    BteCtl *c = d.ctl;
    if (c->done) return;
    double g = 0.0;
    for (int i = threadIdx.x; i < n_part; i += 32) g += d.part[i];
    for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
    if (threadIdx.x != 0) return;
    const int iter = c->iter + 1;
    const double mixing = c->mixing;
    d.scf[iter - 1] = g / d.n_irr / d.n_mode;
    bool stop = false;
    if (iter >= 3) stop = d.scf[iter - 3] + d.scf[iter - 2] + d.scf[iter - 1] < d.tol;
    if (!stop && iter > 15 && mixing > 0.50) c->mixing = mixing * 0.98;
    c->iter = iter;
    if (stop || iter >= d.maxiter) c->done = 1;
}
}  // namespace

int bte_part_elems(int32_t n_irr) { return (n_irr + kBteMixQ - 1) / kBteMixQ; }

cudaError_t launch_bte_update(const BteDev &d, const double *buf, cudaStream_t s) {
    const int ne = d.n_irr * d.n_mode;
    k_bte_apply<<<(ne + 127) / 128, 128, 0, s>>>(d, buf);
    const int nb = bte_part_elems(d.n_irr);
    const size_t mix_smem = sizeof(double) * 3 * kBteMixQ * 3 * (size_t)d.n_mode;
    cudaError_t e = cudaFuncSetAttribute(k_bte_mix, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mix_smem);
    if (e != cudaSuccess) return e;
    k_bte_mix<<<nb, 64, mix_smem, s>>>(d);
    k_bte_check<<<1, 32, 0, s>>>(d, nb);
    return cudaGetLastError();
}

namespace {
// rot[o][q] = full-mesh index of R_o q, -1 when R_o q is off the mesh: (R q)_i = num / L with
// num = sum_j R_ij g_j (L / N_j) in 32-bit integers (|num| < 3 L max N), on the mesh when
// num is a multiple of L / N_i.
__global__ void k_rot_table(int g0, int g1, int g2, int L, int n_full, const int32_t *op_recfrac, int32_t *rot) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int o = blockIdx.y;
    if (q >= n_full) return;
    const int32_t *R = op_recfrac + 9 * o;
    const int g[3] = {g0, g1, g2};
    const int gi[3] = {q / (g1 * g2), (q / g2) % g1, q % g2};
    int out[3];
    for (int i = 0; i < 3; ++i) {
        const int num = R[i] * gi[0] * (L / g0) + R[i + 3] * gi[1] * (L / g1) + R[i + 6] * gi[2] * (L / g2);
        const int step = L / g[i];
        if (num % step != 0) {
            rot[(size_t)o * n_full + q] = -1;
            return;
        }
        int v = (num / step) % g[i];
        if (v < 0) v += g[i];
        out[i] = v;
    }
    rot[(size_t)o * n_full + q] = (out[0] * g1 + out[1]) * g2 + out[2];
}

// Eigenvectors scaled by 1/sqrt(omega) (scattering_threephonon.f90:67,93,102), FP64 and FP32,
// zero for omega < lo_freqtol; IEEE sqrt and division as on the host.
__global__ void k_egv_scaled(int64_t nm, int n, const double2 *egv, const double *omega, double2 *egvs,
                             float2 *egvs32) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nm * n) return;
    const double om = omega[i / n];
    double2 v = make_double2(0.0, 0.0);
    if (!(om < kFreqTolD)) {
        const double sq = sqrt(om);
        const double2 e = egv[i];
        v = make_double2(e.x / sq, e.y / sq);
    }
    egvs[i] = v;
    egvs32[i] = make_float2((float)v.x, (float)v.y);
}
}  // namespace

cudaError_t launch_rot_table(const int32_t grid[3], int L, int n_full, int n_op, const int32_t *op_recfrac,
                             int32_t *rot, cudaStream_t s) {
    if (n_full <= 0 || n_op <= 0) return cudaSuccess;
    dim3 g((unsigned)((n_full + 255) / 256), (unsigned)n_op);
    k_rot_table<<<g, 256, 0, s>>>(grid[0], grid[1], grid[2], L, n_full, op_recfrac, rot);
    return cudaGetLastError();
}

cudaError_t launch_egv_scaled(int64_t nm, int n, const double2 *egv, const double *omega, double2 *egvs,
                              float2 *egvs32, cudaStream_t s) {
    const int64_t total = nm * n;
    if (total <= 0) return cudaSuccess;
    k_egv_scaled<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(nm, n, egv, omega, egvs, egvs32);
    return cudaGetLastError();
}

}  // namespace tdg
