// Per-q-triplet stages shared by the two fused three-phonon kernels (the SIMT kernel of
// k_threephonon.cu and the tensor-core kernel of k_threephonon_tc.cu): loading the mode
// scalars, the skip rules as bit masks, the FP32 screen of the Gaussians, the delta weights
// of the survivors (FP64, or FP32 for the tensor-core kernel), and the row/column sums with
// the Gamma and Xi scatter.
//
// Reference (src/thermal_conductivity/scattering_threephonon.f90):
//   skip rules (:90-101), get_dirac (:219-271), accumulation into Gamma and the Xi row
//   terms for every equivalent triplet (:115-135).
#pragma once

#include "dev_common.cuh"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr double kThreePhononPrefactor = 3.141592653589793 / 16.0;

// Shared-memory arrays of one q-triplet (all length n unless noted).
struct K3Smem {
    double *om1, *om2, *om3, *inv1, *be2, *be3, *s1, *s2, *s3;
    double *v1, *v2, *v3;  // [3n]
    double *wrow;
    double *R2;            // [n^2] row sums, then Xi row terms
    double *R3;            // [n^2] column sums
    double *R2s, *R3s;     // [n^2] each: the Xi row terms of the sums
    double *F;             // [n^3] dense F (zero where no survivor)
    float *Ff;             // or F in FP32 (the tensor-core forward pass: k3_survivors_f32 and
                           // k3_sums_scatter with FLOAT_F)
    float *fo1, *fo2, *fo3, *fs1, *fs2, *fs3;
    float *fl1, *fl2, *fl3;  // omega - (double)fo in FP32: omega = fo + fl to about 2^-48
    float *fb2, *fb3, *fw1;  // be2, be3 and wrow in FP32 (the FP32 weights)
    uint32_t *m12, *m13, *m23;
    uint32_t *zmask;       // [2]: omega2 < tol, omega3 < tol
    uint32_t *rowbits;     // [n^2] b3 with a non-zero F for each (b1, b2)
    uint32_t *colbits;     // [n^2] b2 with a non-zero F for each (b1, b3)
    uint32_t *Q;           // survivor queue: (b1 b2 b3 index) | live bits << 16
    int *rowid;            // row of (q1, b1), -1 when the row does not sample q2
    int2 *red;             // [kMaxRed] equivalent triplets
    int *wsum;             // [33] block scan
};

// Per-mode scalars of the q-triplet, row ids of the rows that sample it, cleared masks and
// the equivalent triplets. Caller: a barrier before the next stage.
template <int N>
__device__ __forceinline__ void k3_load_modes(const K3Smem &S, const ThreePhArgs &a, const TripletRec &rec,
                                              int f1, int q2, int q3, int i2, int i3) {
    constexpr int N2 = N * N;
    const PhononDev &P = a.ph;
    const int tid = threadIdx.x, bd = blockDim.x;
    const uint32_t *mask = a.cand_mask + (size_t)rec.cand * 4;
    for (int b = tid; b < N; b += bd) {
        S.om1[b] = P.omega[(size_t)f1 * N + b];
        S.om2[b] = P.omega[(size_t)q2 * N + b];
        S.om3[b] = P.omega[(size_t)q3 * N + b];
        S.inv1[b] = P.inv_omega[(size_t)f1 * N + b];
        S.be2[b] = P.be[(size_t)i2 * N + b];
        S.be3[b] = P.be[(size_t)i3 * N + b];
        S.s1[b] = P.sigsq[(size_t)rec.q1 * N + b];
        S.s2[b] = P.sigsq[(size_t)i2 * N + b];
        S.s3[b] = P.sigsq[(size_t)i3 * N + b];
        const float h1 = P.omega32[(size_t)f1 * N + b], h2 = P.omega32[(size_t)q2 * N + b],
                    h3 = P.omega32[(size_t)q3 * N + b];
        S.fo1[b] = h1;
        S.fo2[b] = h2;
        S.fo3[b] = h3;
        S.fl1[b] = (float)(S.om1[b] - (double)h1);
        S.fl2[b] = (float)(S.om2[b] - (double)h2);
        S.fl3[b] = (float)(S.om3[b] - (double)h3);
        S.fb2[b] = (float)S.be2[b];
        S.fb3[b] = (float)S.be3[b];
        S.fs1[b] = P.sigsq32[(size_t)rec.q1 * N + b];
        S.fs2[b] = P.sigsq32[(size_t)i2 * N + b];
        S.fs3[b] = P.sigsq32[(size_t)i3 * N + b];
        for (int d = 0; d < 3; ++d) {
            S.v1[b * 3 + d] = P.vel[((size_t)f1 * N + b) * 3 + d];
            S.v2[b * 3 + d] = P.vel[((size_t)q2 * N + b) * 3 + d];
            S.v3[b * 3 + d] = P.vel[((size_t)q3 * N + b) * 3 + d];
        }
        const int r = a.rows.rowidx[(size_t)rec.q1 * N + b];
        const bool on = (mask[b >> 5] >> (b & 31)) & 1u;
        S.rowid[b] = on ? r : -1;
        S.wrow[b] = a.rows.w3q[(size_t)rec.q1 * N + b];
        S.fw1[b] = (float)S.wrow[b];
        S.m12[b] = 0u;
        S.m13[b] = 0u;
        S.m23[b] = 0u;
    }
    if (tid == 0) {
        S.zmask[0] = 0u;
        S.zmask[1] = 0u;
    }
    for (int i = tid; i < 2 * N2; i += bd) S.rowbits[i] = 0u;
    for (int i = tid; i < rec.red_cnt && i < kMaxRed; i += bd) S.red[i] = a.red[rec.red_off + i];
}

// Skip rules of scattering_threephonon.f90:90-101 as bit masks (after a barrier that made
// the mode scalars visible).
template <int N>
__device__ __forceinline__ void k3_skip_masks(const K3Smem &S) {
    constexpr int N2 = N * N;
    const int tid = threadIdx.x, bd = blockDim.x;
    for (int i = tid; i < 3 * N2 + 2 * N; i += bd) {
        if (i < 3 * N2) {
            const int which = i / N2, x = (i % N2) / N, y = i % N;
            const float *fa = which == 2 ? S.fo2 : S.fo1, *la = which == 2 ? S.fl2 : S.fl1;
            const float *fb = which == 0 ? S.fo2 : S.fo3, *lb = which == 0 ? S.fl2 : S.fl3;
            uint32_t *mk = which == 0 ? S.m12 : (which == 1 ? S.m13 : S.m23);
            // |x - y| < 1e-9 from the FP32 (hi, rest) frequency pairs (close_f32)
            if (close_f32(fa[x], la[x], fb[y], lb[y])) atomicOr(mk + x, 1u << y);
        } else {
            const int j = i - 3 * N2, which = j / N, b = j % N;
            const double w = which == 0 ? S.om2[b] : S.om3[b];
            if (w < kFreqTolD) atomicOr(S.zmask + which, 1u << b);
        }
    }
}

// Live bits of the four Gaussians of every b3 of one (b1, b2): the FP32 screen against
// the 8-sigma window of lo_gauss with a relative margin of 1e-3 and an absolute margin far
// above FP32 rounding (a Gaussian the screen drops is exactly 0 in the reference). Returns
// the number of surviving mode triplets; the live bits of b3 are packed 4 per b3 into
// lo (b3 < 8), hi (b3 < 16) and x (b3 < 18).
template <int N>
__device__ __forceinline__ int k3_screen(const K3Smem &S, int it, float sigfix32, int b1, int b2, uint32_t &live_lo,
                                         uint32_t &live_hi, uint32_t &live_x) {
    constexpr uint32_t kAll = (N >= 32) ? 0xffffffffu : ((1u << N) - 1u);
    live_lo = live_hi = live_x = 0u;
    int nsurv = 0;
    const bool skip12 = S.rowid[b1] < 0 || ((S.zmask[0] | S.m12[b1]) >> b2) & 1u;
    const uint32_t allowed = skip12 ? 0u : (kAll & ~(S.zmask[1] | S.m13[b1] | S.m23[b2]));
    const float f_o1 = S.fo1[b1], f_o2 = S.fo2[b2];
#pragma unroll
    for (int b3 = 0; b3 < N; ++b3) {
        if (!((allowed >> b3) & 1u)) continue;
        const float f_o3 = S.fo3[b3];
        float sg = 0.f;
        if (it == 1) sg = sigfix32;
        else if (it == 2) sg = sqrt_screen(S.fs1[b1] + S.fs2[b2] + S.fs3[b3]);
        const float win = 8.0f * sg * 1.001f + 1e-6f * (f_o1 + f_o2 + f_o3);
        uint32_t live = 15u;  // the -it 6 width can cancel in FP32: not screened
        if (it != 6) {
            live = (fabsf(f_o1 + f_o2 - f_o3) <= win ? 1u : 0u) | (fabsf(f_o1 - f_o2 + f_o3) <= win ? 2u : 0u) |
                   (fabsf(f_o1 - f_o2 - f_o3) <= win ? 4u : 0u) | (f_o1 + f_o2 + f_o3 <= win ? 8u : 0u);
        }
        if (live) {
            ++nsurv;
            if (b3 < 8) live_lo |= live << (4 * b3);
            else if (b3 < 16) live_hi |= live << (4 * (b3 - 8));
            else live_x |= live << (4 * (b3 - 16));
        }
    }
    return nsurv;
}

// Queue entries of one (b1, b2) from its live bits, starting at position k.
template <int N>
__device__ __forceinline__ void k3_enqueue(const K3Smem &S, int b1b2, int k, uint32_t live_lo, uint32_t live_hi,
                                           uint32_t live_x) {
#pragma unroll
    for (int b3 = 0; b3 < N; ++b3) {
        const uint32_t live = b3 < 8 ? (live_lo >> (4 * b3)) & 15u
                                     : (b3 < 16 ? (live_hi >> (4 * (b3 - 8))) & 15u : (live_x >> (4 * (b3 - 16))) & 15u);
        if (live) S.Q[k++] = (uint32_t)(b1b2 * N + b3) | (live << 16);
    }
}

// FP64 delta weights and occupations of the nq queued survivors, by full warps: F[idx] =
// perm |Psi|^2 ((n2 - n3) d0 + (n2 + n3 + 1) d1) (the adjoint keeps dF/d|Psi|^2: psisq(idx)
// returns 1) and the row/column bits of the non-zero entries. F must be zero beforehand.
template <int N, typename PsiSq>
__device__ __forceinline__ void k3_survivors(const K3Smem &S, const PhononDev &P, int nq, double perm,
                                             PsiSq psisq) {
    constexpr int N2 = N * N;
    const int it = P.integrationtype;
    for (int s = threadIdx.x; s < nq; s += blockDim.x) {
        const uint32_t qv = S.Q[s];
        const int idx = (int)(qv & 0xffffu);
        const uint32_t live = qv >> 16;
        const int b1 = idx / N2, b2 = (idx / N) % N, b3 = idx % N;
        const double o1 = S.om1[b1], o2 = S.om2[b2], o3 = S.om3[b3];
        double sigma, invsig;
        if (it == 1) {
            sigma = P.sigma_fixed;
            invsig = 1.0 / sigma;
        } else if (it == 2) {
            const double sq = S.s1[b1] + S.s2[b2] + S.s3[b3];
            invsig = rsqrt(sq);
            sigma = sq * invsig;
        } else {
            sigma = adaptive_pair(S.v1 + 3 * b1, S.v2 + 3 * b2, P.reclat_g) / 3.0;
            sigma += adaptive_pair(S.v1 + 3 * b1, S.v3 + 3 * b3, P.reclat_g) / 3.0;
            sigma += adaptive_pair(S.v2 + 3 * b2, S.v3 + 3 * b3, P.reclat_g) / 3.0;
            sigma += P.thresh_sigma;
            invsig = 1.0 / sigma;
        }
        const double win8 = 8.0 * sigma, h = 0.5 * invsig * invsig, cg = kSqrt2PiInv * invsig;
        double d0, d1;
        dirac3(live, o1, o2, o3, win8, h, cg, P.exp2tab, d0, d1);
        if (nonzero(d0) || nonzero(d1)) {
            const double pq = kThreePhononPrefactor * psisq(idx) * S.wrow[b1];
            const double n2 = S.be2[b2], n3 = S.be3[b3];
            const double f0 = perm * pq * (n2 - n3) * d0;
            const double f1 = perm * pq * (n2 + n3 + 1.0) * d1;
            const double fsum = f0 + f1;
            S.F[idx] = fsum;
            if (nonzero(fsum)) {
                atomicOr(S.rowbits + b1 * N + b2, 1u << b3);
                atomicOr(S.colbits + b1 * N + b3, 1u << b2);
            }
        }
    }
}

// The same in FP32 for the mixed-precision kernels: the centre differences om1 - (+-om2 +-
// om3) from FP32 pairs (centre_diff_f32, as accurate as the FP64 difference rounded to
// FP32), the width, the exponent and the Gaussian in FP32 (expf), the occupation factors
// and row weight from FP32 copies made once per mode, F in FP32 stored as a double for the
// FP64 sums. Relative error of a weight about 1e-6, against the 1e-5 of the BF16x3
// contraction.
template <int N, bool FLOAT_F = false, typename PsiSq>
__device__ __forceinline__ void k3_survivors_f32(const K3Smem &S, const PhononDev &P, int nq, float perm,
                                                 PsiSq psisq) {
    constexpr int N2 = N * N;
    constexpr float kSqrt2PiInvF = 0.3989422804014327f;
    const int it = P.integrationtype;
    const float sfix = (float)P.sigma_fixed;
    const float pref = (float)kThreePhononPrefactor;
    for (int s = threadIdx.x; s < nq; s += blockDim.x) {
        const uint32_t qv = S.Q[s];
        const int idx = (int)(qv & 0xffffu);
        uint32_t live = qv >> 16;
        const int b1 = idx / N2, b2 = (idx / N) % N, b3 = idx % N;
        float sigma;
        if (it == 1) {
            sigma = sfix;
        } else if (it == 2) {
            sigma = sqrtf(S.fs1[b1] + S.fs2[b2] + S.fs3[b3]);
        } else {
            sigma = (float)(adaptive_pair(S.v1 + 3 * b1, S.v2 + 3 * b2, P.reclat_g) / 3.0 +
                            adaptive_pair(S.v1 + 3 * b1, S.v3 + 3 * b3, P.reclat_g) / 3.0 +
                            adaptive_pair(S.v2 + 3 * b2, S.v3 + 3 * b3, P.reclat_g) / 3.0 + P.thresh_sigma);
        }
        const float invsig = 1.0f / sigma;
        const float win8 = 8.0f * sigma, h = 0.5f * invsig * invsig, cg = kSqrt2PiInvF * invsig;
        const float h1 = S.fo1[b1], l1 = S.fl1[b1], h2 = S.fo2[b2], l2 = S.fl2[b2], h3 = S.fo3[b3], l3 = S.fl3[b3];
        float g[4] = {0.f, 0.f, 0.f, 0.f};
        while (live) {
            const int j = __ffs(live) - 1;
            live &= live - 1;
            // Gaussian j centred at (-om2+om3, om2-om3, om2+om3, -om2-om3), get_dirac's order
            const float sg2 = (j == 1 || j == 2) ? 1.f : -1.f;
            const float sg3 = (j == 0 || j == 2) ? 1.f : -1.f;
            const float dx = centre_diff_f32(h1, l1, sg2 * h2, sg2 * l2, sg3 * h3, sg3 * l3);
            const float gj = fabsf(dx) > win8 ? 0.f : expf(-dx * dx * h) * cg;
            g[0] = j == 0 ? gj : g[0];
            g[1] = j == 1 ? gj : g[1];
            g[2] = j == 2 ? gj : g[2];
            g[3] = j == 3 ? gj : g[3];
        }
        const float d0 = g[0] - g[1], d1 = g[2] - g[3];
        if (d0 != 0.f || d1 != 0.f) {
            const float pq = pref * psisq(idx) * S.fw1[b1];
            const float n2 = S.fb2[b2], n3 = S.fb3[b3];
            const float fsum = perm * pq * ((n2 - n3) * d0 + (n2 + n3 + 1.0f) * d1);
            if constexpr (FLOAT_F)
                S.Ff[idx] = fsum;
            else
                S.F[idx] = (double)fsum;
            if (fsum != 0.f) {
                atomicOr(S.rowbits + b1 * N + b2, 1u << b3);
                atomicOr(S.colbits + b1 * N + b3, 1u << b2);
            }
        }
    }
}

// Row sums over b3 (R2) and column sums over b2 (R3) of the non-zero F, Gamma of every
// sampling row times the nred equivalent triplets, then the Xi row terms 2 F om/om1 added
// for each equivalent triplet (scattering_threephonon.f90:115-135). Starts and ends with
// barriers of its own.
template <int N, bool FLOAT_F = false>
__device__ __forceinline__ void k3_sums_scatter(const K3Smem &S, const ThreePhArgs &a, int nred) {
    constexpr int N2 = N * N;
    const int tid = threadIdx.x, bd = blockDim.x;
    const int64_t ld = (int64_t)a.mesh.n_full * N;
    __syncthreads();
    // FP32 F: the sums in double-float on the FP32 pipe (TwoSum; exact to ~2^-44 for these
    // at most n terms), one conversion to FP64 per sum, instead of a conversion and an FP64
    // add per term on GB300's 2-lane-per-clock FP64 pipe
    for (int e = tid; e < 2 * N2; e += bd) {
        double sum = 0.0;
        float2 dsum = make_float2(0.f, 0.f);
        if (e < N2) {
            for (uint32_t bits = S.rowbits[e]; bits; bits &= bits - 1) {
                const int i = e * N + __ffs(bits) - 1;
                if constexpr (FLOAT_F)
                    df_acc(dsum, S.Ff[i]);
                else
                    sum += S.F[i];
            }
            S.R2[e] = FLOAT_F ? (double)dsum.x + (double)dsum.y : sum;
        } else {
            const int e3 = e - N2, b1 = e3 / N, b3 = e3 % N;
            for (uint32_t bits = S.colbits[e3]; bits; bits &= bits - 1) {
                const int i = (b1 * N + __ffs(bits) - 1) * N + b3;
                if constexpr (FLOAT_F)
                    df_acc(dsum, S.Ff[i]);
                else
                    sum += S.F[i];
            }
            S.R3[e3] = FLOAT_F ? (double)dsum.x + (double)dsum.y : sum;
        }
    }
    __syncthreads();
    // Gamma from the row sums (threads < N) and the Xi row terms 2 F om/om1 of each entry,
    // computed once for all equivalent triplets into R2s / R3s
    if (tid < N) {
        const int row = S.rowid[tid];
        if (row >= 0) {
            double g = 0.0;
            for (int b2 = 0; b2 < N; ++b2) g += S.R2[tid * N + b2];
            if (nonzero(g)) atomicAdd(a.gamma + row, (double)nred * g);
        }
    }
    for (int e = tid; e < 2 * N2; e += bd) {
        if (e < N2) {
            const double v = S.R2[e];
            S.R2s[e] = nonzero(v) ? 2.0 * v * S.om2[e % N] * S.inv1[e / N] : 0.0;
        } else {
            const int e3 = e - N2;
            const double v = S.R3[e3];
            S.R3s[e3] = nonzero(v) ? 2.0 * v * S.om3[e3 % N] * S.inv1[e3 / N] : 0.0;
        }
    }
    __syncthreads();
    for (int i = tid; i < 2 * N2 * nred; i += bd) {
        const int r = i / (2 * N2), e = i % (2 * N2);
        const int2 pr = S.red[r];
        if (e < N2) {
            const int b1 = e / N, b2 = e % N;
            const int row = S.rowid[b1];
            const double v = S.R2s[e];
            if (row >= 0 && nonzero(v)) atomicAdd(a.od + row * ld + (int64_t)pr.x * N + b2, v);
        } else {
            const int e3 = e - N2, b1 = e3 / N, b3 = e3 % N;
            const int row = S.rowid[b1];
            const double v = S.R3s[e3];
            if (row >= 0 && nonzero(v)) atomicAdd(a.od + row * ld + (int64_t)pr.y * N + b3, v);
        }
    }
    __syncthreads();
}

}  // namespace

}  // namespace tdg
