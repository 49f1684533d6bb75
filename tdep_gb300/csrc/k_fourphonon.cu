// Fused four-phonon scattering for one accepted irreducible q-quartet per CTA iteration
// (persistent grid-stride loop over the quartet list).
//
// Reference (src/thermal_conductivity/scattering_fourphonon.f90):
//   pretransform_phi4 (:459-506)  ptf(a,b,c,d) = sum_t mwm_t(i,j,k,l) exp(-2 pi i (q2.lv2 + q3.lv3 + q4.lv4))
//   zgeru x3 + dot_product (:131-159)  c0 = sum_abcd e1(a) e2(b) e3(c) e4(d) ptf(a,b,c,d)
//   get_dirac (:267-327), multiplicities (:104-122), accumulation (:161-186).
// The reference rebuilds the n^4 ptf per row and contracts it per (b2,b3,b4) (2 n^4
// complex MACs per mode quadruplet, n^8 per row). Here, per q-quartet:
//   T1[b1][b][c][d] = sum_a E1[a][b1] ptf[a][b][c][d], ptf = sum_t mwm_t(i,j,k,l) phase_t
// is built once for every row mode b1 into a per-CTA slice of device scratch: first the
// pretransform ptf (n_fc4 * 81 real x complex MACs), then its contraction with E1 in place
// (n^5 complex MACs); for each row b1 the n^3 slice of T1 is contracted with E2, E3, E4 in
// shared memory (3 n^4 complex MACs per b1): 4 n^5 complex MACs per q-quartet in all.
// Phases are exact roots of unity from integer lattice vectors, as in the three-phonon
// kernel. An FP32 pre-screen with a safety margin skips Gaussians that are exactly zero in
// the reference. Precision R: double (FP64 path: delta weights, occupations and
// accumulation in FP64 with the reference's window test) or float (mixed path: FP32
// pretransform and contraction, FP32 delta weights and occupations from FP64 centre
// differences, FP64 accumulation).
#include <cuda_runtime.h>

#include "dev_common.cuh"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr double kFourPhononPrefactor = 3.141592653589793 / 96.0;
constexpr int kPhaseChunk4 = 512;

template <typename R>
__device__ __forceinline__ const R *mwm4_ptr(const Fc4Dev &fc);
template <>
__device__ __forceinline__ const double *mwm4_ptr<double>(const Fc4Dev &fc) {
    return fc.mwm;
}
template <>
__device__ __forceinline__ const float *mwm4_ptr<float>(const Fc4Dev &fc) {
    return fc.mwm32;
}

template <typename C>
__device__ __forceinline__ C twiddle4(const FourPhArgs &a, int k);
template <>
__device__ __forceinline__ double2 twiddle4<double2>(const FourPhArgs &a, int k) {
    return a.twiddle[k];
}
template <>
__device__ __forceinline__ float2 twiddle4<float2>(const FourPhArgs &a, int k) {
    return a.twiddle32[k];
}

template <typename C>
__device__ __forceinline__ const C *egvs4_ptr(const PhononDev &ph);
template <>
__device__ __forceinline__ const double2 *egvs4_ptr<double2>(const PhononDev &ph) {
    return ph.egvs;
}
template <>
__device__ __forceinline__ const float2 *egvs4_ptr<float2>(const PhononDev &ph) {
    return ph.egvs32;
}

struct Layout4 {
    size_t om, be, sg, vel, fo, inv1, wrow, rowid, red, R, occ, E, ph, A, B, total;
};
__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ inline Layout4 make_layout4(int n, int cs) {
    Layout4 L;
    size_t o = 0;
    const size_t n2 = (size_t)n * n, n3 = n2 * n;
    L.om = o; o += al16(sizeof(double) * 4 * n);     // omega of q1..q4
    L.be = o; o += al16(sizeof(double) * 4 * n);     // Bose factors of q2..q4 (slot 0 unused)
    L.sg = o; o += al16(sizeof(double) * 4 * n);     // sigsq of q1..q4
    L.vel = o; o += al16(sizeof(double) * 12 * n);   // velocities of q1..q4
    L.fo = o; o += al16(sizeof(float) * 8 * n);      // omega and sigsq in FP32
    L.inv1 = o; o += al16(sizeof(double) * n);
    L.wrow = o; o += al16(sizeof(double) * n);
    L.rowid = o; o += al16(sizeof(int) * n);
    L.red = o; o += al16(sizeof(int4) * kMaxRed);
    L.R = o; o += al16(sizeof(double) * 3 * n);
    L.occ = o; o += al16(sizeof(double) * (2 * n * n + 4 * n));  // occupation products (see below)
    L.E = o; o += al16((size_t)cs * 4 * n2);
    L.ph = o; o += al16((size_t)cs * kPhaseChunk4);
    const size_t csz = (size_t)cs > sizeof(double) ? (size_t)cs : sizeof(double);
    L.A = o; o += al16(csz * n3);
    L.B = o; o += al16(csz * n3);
    L.total = o;
    return L;
}

__host__ __device__ constexpr int threads4_for(int n) {
    return n * n * n >= 256 ? 256 : ((n * n * n + 31) / 32) * 32;
}

// Resident CTAs the register budget is sized for: at n = 15 in FP32 shared memory admits
// three per SM, which the in-place E1 contraction's registers would otherwise reduce to two.
__host__ __device__ constexpr int min_blocks4(int n, bool dbl) { return (n == 15 && !dbl) ? 3 : 1; }

template <int N, typename R>
__global__ void __launch_bounds__(threads4_for(N), min_blocks4(N, sizeof(R) == 8)) k_fourphonon(FourPhArgs a) {
    using C = typename CT<R>::C;
    constexpr int N2 = N * N, N3 = N2 * N;
    constexpr int NA = N / 3;
    extern __shared__ __align__(16) unsigned char smem[];
    const Layout4 L = make_layout4(N, sizeof(C));
    double *om = (double *)(smem + L.om);   // om[k*N + b], k = 0..3 for q1..q4
    double *be = (double *)(smem + L.be);
    double *sg = (double *)(smem + L.sg);
    double *vel = (double *)(smem + L.vel); // vel[(k*N + b)*3 + d]
    float *fo = (float *)(smem + L.fo);     // fo[k*N + b] omega, fo[(4+k)*N + b] sigsq
    double *inv1 = (double *)(smem + L.inv1);
    double *wrow = (double *)(smem + L.wrow);
    int *rowid = (int *)(smem + L.rowid);
    int4 *red = (int4 *)(smem + L.red);
    double *Rs = (double *)(smem + L.R);    // R2, R3, R4 of the current b1
    // Occupation products of the quartet, so that the four polynomials of the weights
    // (scattering_fourphonon.f90:161-186) cost 10 FP64 operations per mode quadruplet
    // instead of 26: per (b3, b4) P00 = n3 n4 and P11 = (n3+1)(n4+1), with n3 (n4+1) =
    // P00 + n3 and (n3+1) n4 = P00 + n4; per b2 n2, n2+1, 3 n2, 3 (n2+1). Two tables of n^2
    // keep three CTAs per SM at n = 15.
    double *P00 = (double *)(smem + L.occ), *P11 = P00 + N * N;
    double *N2v = P11 + N * N, *N2p = N2v + N, *N2x3 = N2p + N, *N2px3 = N2x3 + N;
    C *E = (C *)(smem + L.E);               // E[k*N2 + r*N + b], k = 0..3
    C *ph = (C *)(smem + L.ph);
    C *A = (C *)(smem + L.A);
    C *B = (C *)(smem + L.B);
    const int tid = threadIdx.x, bd = blockDim.x;
    const MeshDev &m = a.mesh;
    const PhononDev &P = a.ph;
    const Fc4Dev &fc = a.fc;
    const R *mwm = mwm4_ptr<R>(fc);
    const C *egvs = egvs4_ptr<C>(P);
    const int64_t ld = (int64_t)m.n_full * N;
    const int it = P.integrationtype;
    const float sigfix32 = (float)P.sigma_fixed;
    C *T1 = reinterpret_cast<C *>(a.scratch) + (size_t)blockIdx.x * N3 * N;

    for (int t = blockIdx.x; t < a.n_quart; t += gridDim.x) {
        __syncthreads();  // the previous quartet's shared data is no longer read
        const QuartetRec rec = a.quart[t];
        const int qf[4] = {m.irr_full[rec.q1], rec.q2, rec.q3, rec.q4};
        const int qi[4] = {rec.q1, m.full_irr[rec.q2], m.full_irr[rec.q3], m.full_irr[rec.q4]};
        const uint32_t *mask = a.cand_mask + (size_t)rec.cand * 4;
        const int nred = rec.red_cnt;
        const int q2 = rec.q2, q3 = rec.q3, q4 = rec.q4;
        // permutation multiplicities (scattering_fourphonon.f90:104-122)
        double mult0, mult1;
        if (q2 == q3 && q3 == q4) {
            mult0 = 1.0;
            mult1 = 1.0;
        } else if ((q2 != q3 && q3 == q4) || (q3 != q2 && q2 == q4) || (q4 != q2 && q2 == q3)) {
            mult0 = 3.0;
            mult1 = 1.0;
        } else {
            mult0 = 6.0;
            mult1 = 2.0;
        }
        // ---- per-mode scalars, eigenvectors, equivalent quartets ----
        for (int i = tid; i < 4 * N; i += bd) {
            const int k = i / N, b = i % N;
            const double w = P.omega[(size_t)qf[k] * N + b];
            om[i] = w;
            sg[i] = P.sigsq[(size_t)qi[k] * N + b];
            be[i] = k > 0 ? P.be[(size_t)qi[k] * N + b] : 0.0;
            // NaN marks omega < 1e-9 Ha: the skip test then runs in FP32 (double compares and
            // conversions per mode quadruplet would occupy GB300's narrow FP64 pipe)
            fo[i] = w < kFreqTolD ? __int_as_float(0x7fc00000) : (float)w;
            fo[4 * N + i] = (float)sg[i];
            for (int d = 0; d < 3; ++d) vel[i * 3 + d] = P.vel[((size_t)qf[k] * N + b) * 3 + d];
            if (k == 0) {
                inv1[b] = w > 0.0 ? 1.0 / w : 0.0;
                const int r = a.rows.rowidx[(size_t)rec.q1 * N + b];
                const bool on = (mask[b >> 5] >> (b & 31)) & 1u;
                rowid[b] = on ? r : -1;
                wrow[b] = r >= 0 ? a.rows.weight4[r] : 0.0;
            }
        }
        for (int i = tid; i < nred && i < kMaxRed; i += bd) red[i] = a.red[rec.red_off + i];
        for (int i = tid; i < 4 * N2; i += bd) {
            const int k = i / N2, e = i % N2;
            const int r = e / N, b = e % N;
            E[i] = egvs[((size_t)qf[k] * N + b) * N + r];
        }
        __syncthreads();  // be[] of q2..q4 is in shared memory
        for (int i = tid; i < N * N; i += bd) {
            const double n3 = be[2 * N + i / N], n4 = be[3 * N + i % N];
            P00[i] = n3 * n4;
            P11[i] = (n3 + 1.0) * (n4 + 1.0);
        }
        for (int b = tid; b < N; b += bd) {
            const double n2 = be[N + b];
            N2v[b] = n2;
            N2p[b] = n2 + 1.0;
            N2x3[b] = 3.0 * n2;
            N2px3[b] = 3.0 * (n2 + 1.0);
        }
        int g[3][3];
        {
            const int n12 = m.grid[1] * m.grid[2];
            for (int k = 0; k < 3; ++k) {
                const int q = qf[k + 1];
                g[k][0] = (q / n12) * m.lmul[0];  // g_d L/N_d
                g[k][1] = ((q / m.grid[2]) % m.grid[1]) * m.lmul[1];
                g[k][2] = (q % m.grid[2]) * m.lmul[2];
            }
        }
        // ---- ptf[a][bcd] (pretransform_phi4) into the T1 slice, one atom a1 at a time: the
        // force-constant quartets are sorted by atom block with a1 leading, so the phase
        // chunks of one a1 serve exactly its 3 n^3 outputs a = 3 a1 + i (n_fc4 * 81 real x
        // complex multiply-adds per q-quartet) ----
        constexpr int NA3 = NA * NA * NA;
        for (int a1 = 0; a1 < NA; ++a1) {
            C *P = T1 + (size_t)(3 * a1) * N3;
            const int t0 = fc.blk_ptr[a1 * NA3], t1 = fc.blk_ptr[(a1 + 1) * NA3];
            if (t0 >= t1) {
                for (int o = tid; o < 3 * N3; o += bd) P[o] = czero<C>();
                continue;
            }
            for (int c0 = t0; c0 < t1; c0 += kPhaseChunk4) {
                const int cn = min(kPhaseChunk4, t1 - c0);
                __syncthreads();
                // K = sum_d ((g2 lv2 + g3 lv3 + g4 lv4)_d mod N_d) L/N_d mod L, evaluated as
                // (sum_d (g2 L/N_d) lv2 + ...) mod L: the same integer with one division
                for (int i = tid; i < cn; i += bd) {
                    const int32_t *lv = fc.lv + (size_t)(c0 + i) * 9;
                    int S = 0;
#pragma unroll
                    for (int d = 0; d < 3; ++d) S += g[0][d] * lv[d] + g[1][d] * lv[3 + d] + g[2][d] * lv[6 + d];
                    int K = S % m.L;
                    if (K < 0) K += m.L;
                    ph[i] = twiddle4<C>(a, K);
                }
                __syncthreads();
                for (int o = tid; o < 3 * N3; o += bd) {
                    const int i = o / N3, bcd = o % N3;
                    const int b = bcd / N2, c = (bcd / N) % N, d = bcd % N;
                    const int blk = ((a1 * NA + b / 3) * NA + c / 3) * NA + d / 3;
                    const int ijkl = i + (b % 3) * 3 + (c % 3) * 9 + (d % 3) * 27;
                    C acc = c0 == t0 ? czero<C>() : P[o];
                    const int lo = max(fc.blk_ptr[blk], c0), hi = min(fc.blk_ptr[blk + 1], c0 + cn);
                    for (int tt = lo; tt < hi; ++tt) {
                        const R mv = __ldg(mwm + (size_t)tt * 81 + ijkl);
                        const C p = ph[tt - c0];
                        acc.x = fma(mv, p.x, acc.x);
                        acc.y = fma(mv, p.y, acc.y);
                    }
                    P[o] = acc;
                }
            }
        }
        __syncthreads();
        // ---- T1[b1][bcd] = sum_a E1[a][b1] ptf[a][bcd], column by column in place (n^5
        // complex multiply-adds, against n_fc4 * 81 * n when E1 is folded into every
        // force-constant term) ----
        for (int col = tid; col < N3; col += bd) {
            C v[N];
#pragma unroll
            for (int x = 0; x < N; ++x) v[x] = T1[(size_t)x * N3 + col];
            for (int b1 = 0; b1 < N; ++b1) {
                if (rowid[b1] < 0) continue;
                C acc = czero<C>();
#pragma unroll
                for (int x = 0; x < N; ++x) cfma(acc, E[x * N + b1], v[x]);
                T1[(size_t)b1 * N3 + col] = acc;
            }
        }
        __syncthreads();
        const C *E2 = E + N2, *E3 = E + 2 * N2, *E4 = E + 3 * N2;
        const double *om1 = om, *om2 = om + N, *om3 = om + 2 * N, *om4 = om + 3 * N;
        const float *fo1 = fo, *fo2 = fo + N, *fo3 = fo + 2 * N, *fo4 = fo + 3 * N;
        const float *fs1 = fo + 4 * N, *fs2 = fo + 5 * N, *fs3 = fo + 6 * N, *fs4 = fo + 7 * N;
        for (int b1 = 0; b1 < N; ++b1) {
            const int row = rowid[b1];
            if (row < 0) continue;
            for (int i = tid; i < N3; i += bd) A[i] = T1[(size_t)b1 * N3 + i];
            __syncthreads();
            // B[b2][c][d] = sum_b E2[b][b2] A[b][c][d]
            for (int o = tid; o < N3; o += bd) {
                const int b2 = o / N2, cd = o % N2;
                C acc = czero<C>();
#pragma unroll
                for (int b = 0; b < N; ++b) cfma(acc, E2[b * N + b2], A[b * N2 + cd]);
                B[o] = acc;
            }
            __syncthreads();
            // A[b2][b3][d] = sum_c E3[c][b3] B[b2][c][d]
            for (int o = tid; o < N3; o += bd) {
                const int b2 = o / N2, b3 = (o / N) % N, d = o % N;
                C acc = czero<C>();
#pragma unroll
                for (int c = 0; c < N; ++c) cfma(acc, E3[c * N + b3], B[(b2 * N + c) * N + d]);
                A[o] = acc;
            }
            __syncthreads();
            // B[b2][b3][b4] = sum_d E4[d][b4] A[b2][b3][d] = Psi
            for (int o = tid; o < N3; o += bd) {
                const int b4 = o % N, b23 = o / N;
                C acc = czero<C>();
#pragma unroll
                for (int d = 0; d < N; ++d) cfma(acc, E4[d * N + b4], A[b23 * N + d]);
                B[o] = acc;
            }
            __syncthreads();
            // ---- delta weights, occupations (FP64, or FP32 on the mixed path); F in A as doubles ----
            double *F = (double *)A;
            const double o1 = om1[b1], w1 = wrow[b1];
            const double pw4 = kFourPhononPrefactor * w1 * w1;
            const float f_o1 = fo1[b1];
            // FP32 F of one live mode quadruplet (mixed precision), the FP64 branch's algebra
            auto weights_f32 = [&](uint32_t live, int b1x, int b2, int b3, int b4) -> float {
                float sigma;
                if (it == 1) {
                    sigma = sigfix32;
                } else if (it == 2) {
                    sigma = sqrtf(fs1[b1x] + fs2[b2] + fs3[b3] + fs4[b4]);
                } else {
                    const double *v1 = vel + 3 * b1x, *v2 = vel + 3 * (N + b2), *v3 = vel + 3 * (2 * N + b3),
                                 *v4 = vel + 3 * (3 * N + b4);
                    sigma = (float)(adaptive_pair(v1, v2, P.reclat_g) / 6.0 + adaptive_pair(v1, v3, P.reclat_g) / 6.0 +
                                    adaptive_pair(v1, v4, P.reclat_g) / 6.0 + adaptive_pair(v2, v3, P.reclat_g) / 6.0 +
                                    adaptive_pair(v2, v4, P.reclat_g) / 6.0 + adaptive_pair(v3, v4, P.reclat_g) / 6.0 +
                                    P.thresh_sigma);
                }
                const float invsig = 1.0f / sigma;
                const float win8 = 8.0f * sigma, h = 0.5f * invsig * invsig, cg = 0.3989422804014327f * invsig;
                const double o2 = om2[b2], o3 = om3[b3], o4 = om4[b4];
                auto gf = [&](double centre) -> float {
                    const float dx = (float)(o1 - centre);
                    return fabsf(dx) > win8 ? 0.f : expf(-dx * dx * h) * cg;
                };
                const float d0 = ((live & 1u) ? gf(o2 + o3 + o4) : 0.f) - ((live & 2u) ? gf(-o2 - o3 - o4) : 0.f);
                const float d1 = ((live & 4u) ? gf(-o2 + o3 + o4) : 0.f) - ((live & 8u) ? gf(o2 - o3 - o4) : 0.f);
                const float d2 = ((live & 16u) ? gf(o2 - o3 + o4) : 0.f) - ((live & 32u) ? gf(-o2 + o3 - o4) : 0.f);
                const float d3 = ((live & 64u) ? gf(o2 + o3 - o4) : 0.f) - ((live & 128u) ? gf(-o2 - o3 + o4) : 0.f);
                if (d0 == 0.f && d1 == 0.f && d2 == 0.f && d3 == 0.f) return 0.f;
                const C psi = B[b2 * N2 + b3 * N + b4];
                const float ps = fmaf((float)psi.x, (float)psi.x, (float)psi.y * (float)psi.y);
                const int k34 = b3 * N + b4;
                const float n2 = (float)N2v[b2], n2p = (float)N2p[b2], p00 = (float)P00[k34], p11 = (float)P11[k34];
                float acc = 0.f, a1 = 0.f;
                if (d0 != 0.f) acc = (float)mult0 * fmaf(n2p, p11, -n2 * p00) * d0;
                if (d1 != 0.f) a1 = fmaf((float)N2x3[b2], p11, -n2p * p00) * d1;
                if (d2 != 0.f || d3 != 0.f) {
                    const float q1 = p00 + (float)be[2 * N + b3], q2 = p00 + (float)be[3 * N + b4];
                    const float n2px3 = (float)N2px3[b2];
                    if (d2 != 0.f) a1 = fmaf(n2px3, q1, -n2 * q2) * d2 + a1;
                    if (d3 != 0.f) a1 = fmaf(n2px3, q2, -n2 * q1) * d3 + a1;
                }
                return (float)pw4 * ps * fmaf((float)mult1, a1, acc);
            };
            for (int o = tid; o < N3; o += bd) {
                const int b2 = o / N2, b3 = (o / N) % N, b4 = o % N;
                double fall = 0.0;
                const float f2 = fo2[b2], f3 = fo3[b3], f4 = fo4[b4];
                if (f2 == f2 && f3 == f3 && f4 == f4) {  // no omega below 1e-9 Ha
                    const double o2 = om2[b2], o3 = om3[b3], o4 = om4[b4];
                    uint32_t live = 0xffu;  // the -it 6 width can cancel in FP32: not screened
                    if (it != 6) {
                        float sgf = sigfix32;
                        if (it == 2) sgf = sqrtf(fs1[b1] + fs2[b2] + fs3[b3] + fs4[b4]);
                        const float win = 8.0f * sgf * 1.001f + 1e-6f * (f_o1 + f2 + f3 + f4);
                        const float s234 = f2 + f3 + f4;
                        live = (fabsf(f_o1 - s234) <= win ? 1u : 0u) | (f_o1 + s234 <= win ? 2u : 0u) |
                               (fabsf(f_o1 - (-f2 + f3 + f4)) <= win ? 4u : 0u) |
                               (fabsf(f_o1 - (f2 - f3 - f4)) <= win ? 8u : 0u) |
                               (fabsf(f_o1 - (f2 - f3 + f4)) <= win ? 16u : 0u) |
                               (fabsf(f_o1 - (-f2 + f3 - f4)) <= win ? 32u : 0u) |
                               (fabsf(f_o1 - (f2 + f3 - f4)) <= win ? 64u : 0u) |
                               (fabsf(f_o1 - (-f2 - f3 + f4)) <= win ? 128u : 0u);
                    }
                    if constexpr (sizeof(R) == 4) {
                        // mixed precision: the weights in FP32 from FP64 centre differences
                        // rounded to FP32 (as the three-phonon kernels), F in FP32; GB300 issues
                        // FP64 at 1/64 of the FP32 rate and the FP64 weights held this kernel's
                        // FP64 pipe at 76 %
                        if (live) fall = (double)weights_f32(live, b1, b2, b3, b4);
                        live = 0u;
                    }
                    if (live) {
                        double sigma, invsig;
                        if (it == 1) {
                            sigma = P.sigma_fixed;
                            invsig = 1.0 / sigma;
                        } else if (it == 2) {
                            const double sq = sg[b1] + sg[N + b2] + sg[2 * N + b3] + sg[3 * N + b4];
                            invsig = rsqrt(sq);
                            sigma = sq * invsig;
                        } else {
                            const double *v1 = vel + 3 * b1, *v2 = vel + 3 * (N + b2), *v3 = vel + 3 * (2 * N + b3),
                                         *v4 = vel + 3 * (3 * N + b4);
                            sigma = 0.0;
                            sigma += adaptive_pair(v1, v2, P.reclat_g) / 6.0;
                            sigma += adaptive_pair(v1, v3, P.reclat_g) / 6.0;
                            sigma += adaptive_pair(v1, v4, P.reclat_g) / 6.0;
                            sigma += adaptive_pair(v2, v3, P.reclat_g) / 6.0;
                            sigma += adaptive_pair(v2, v4, P.reclat_g) / 6.0;
                            sigma += adaptive_pair(v3, v4, P.reclat_g) / 6.0;
                            sigma += P.thresh_sigma;
                            invsig = 1.0 / sigma;
                        }
                        const double win8 = 8.0 * sigma, h = 0.5 * invsig * invsig, cg = kSqrt2PiInv * invsig;
                        const double *tab = P.exp2tab;
                        // a centre is formed only for a Gaussian that the screen left live
                        const double d0 = ((live & 1u) ? gauss(o1 - (o2 + o3 + o4), win8, h, cg, tab) : 0.0) -
                                          ((live & 2u) ? gauss(o1 - (-o2 - o3 - o4), win8, h, cg, tab) : 0.0);
                        const double d1 = ((live & 4u) ? gauss(o1 - (-o2 + o3 + o4), win8, h, cg, tab) : 0.0) -
                                          ((live & 8u) ? gauss(o1 - (o2 - o3 - o4), win8, h, cg, tab) : 0.0);
                        const double d2 = ((live & 16u) ? gauss(o1 - (o2 - o3 + o4), win8, h, cg, tab) : 0.0) -
                                          ((live & 32u) ? gauss(o1 - (-o2 + o3 - o4), win8, h, cg, tab) : 0.0);
                        const double d3 = ((live & 64u) ? gauss(o1 - (o2 + o3 - o4), win8, h, cg, tab) : 0.0) -
                                          ((live & 128u) ? gauss(o1 - (-o2 - o3 + o4), win8, h, cg, tab) : 0.0);
                        if (nonzero(d0) || nonzero(d1) || nonzero(d2) || nonzero(d3)) {
                            const C psi = B[o];
                            double ps;
                            if constexpr (sizeof(R) == 4) {
                                ps = (double)fmaf(psi.x, psi.x, psi.y * psi.y);  // |Psi|^2 of an FP32 Psi
                            } else {
                                ps = psi.x * psi.x + psi.y * psi.y;
                            }
                            // plf0 = (n2+1)(n3+1)(n4+1) - n2 n3 n4, plf1 = 3 n2 (n3+1)(n4+1) - (n2+1) n3 n4,
                            // plf2 = 3 n3 (n2+1)(n4+1) - (n3+1) n2 n4, plf3 = 3 n4 (n2+1)(n3+1) - (n4+1) n2 n3
                            const int k34 = b3 * N + b4;
                            const double n2 = N2v[b2], n2p = N2p[b2], p00 = P00[k34], p11 = P11[k34];
                            double acc = 0.0;
                            if (nonzero(d0)) acc = mult0 * fma(n2p, p11, -n2 * p00) * d0;
                            double a1 = 0.0;
                            if (nonzero(d1)) a1 = fma(N2x3[b2], p11, -n2p * p00) * d1;
                            if (nonzero(d2) || nonzero(d3)) {
                                const double q1 = p00 + be[2 * N + b3], q2 = p00 + be[3 * N + b4];
                                if (nonzero(d2)) a1 = fma(N2px3[b2], q1, -n2 * q2) * d2 + a1;
                                if (nonzero(d3)) a1 = fma(N2px3[b2], q2, -n2 * q1) * d3 + a1;
                            }
                            fall = pw4 * ps * fma(mult1, a1, acc);
                        }
                    }
                }
                F[o] = fall;
            }
            __syncthreads();
            // R2[b2] = sum_{b3,b4} F, R3[b3] = sum_{b2,b4} F, R4[b4] = sum_{b2,b3} F
            for (int e = tid; e < 3 * N; e += bd) {
                const int which = e / N, b = e % N;
                double sum = 0.0;
                for (int x = 0; x < N; ++x)
                    for (int y = 0; y < N; ++y) {
                        const int idx = which == 0 ? (b * N + x) * N + y : (which == 1 ? (x * N + b) * N + y : (x * N + y) * N + b);
                        const double f = F[idx];
                        if (nonzero(f)) sum += f;
                    }
                Rs[e] = sum;
            }
            __syncthreads();
            if (tid == 0) {
                double gsum = 0.0;
                for (int b2 = 0; b2 < N; ++b2) gsum += Rs[b2];
                if (nonzero(gsum)) atomicAdd(a.gamma + row, (double)nred * gsum);
            }
            // the row terms 2 R om / om1, formed once for all equivalent quartets (after Gamma
            // has read R2)
            __syncthreads();
            for (int e = tid; e < 3 * N; e += bd) {
                const double v = Rs[e];
                Rs[e] = nonzero(v) ? 2.0 * v * om[(e / N + 1) * N + e % N] * inv1[b1] : 0.0;
            }
            __syncthreads();
            for (int i = tid; i < 3 * N * nred; i += bd) {
                const int r = i / (3 * N), e = i % (3 * N);
                const int which = e / N, b = e % N;
                const double v = Rs[e];
                if (!nonzero(v)) continue;
                const int4 pr = red[r];
                const int qp = which == 0 ? pr.x : (which == 1 ? pr.y : pr.z);
                atomicAdd(a.od + row * ld + (int64_t)qp * N + b, v);
            }
            __syncthreads();
        }
    }
}

template <int N, typename R>
int grid_n(int n_sm, int n_quart) {
    const Layout4 L = make_layout4(N, sizeof(typename CT<R>::C));
    const int per_sm = resident_ctas((const void *)k_fourphonon<N, R>, threads4_for(N), L.total, nullptr, nullptr);
    if (per_sm < 1) return 0;
    int grid = n_sm * per_sm;
    if (grid > n_quart) grid = n_quart;
    return grid < 1 ? 1 : grid;
}

template <int N, typename R>
cudaError_t launch_n4(const FourPhArgs &a, int grid, cudaStream_t s) {
    const Layout4 L = make_layout4(N, sizeof(typename CT<R>::C));
    k_fourphonon<N, R><<<grid, threads4_for(N), L.total, s>>>(a);
    return cudaGetLastError();
}

template <typename R>
int grid_prec(int n, int n_sm, int n_quart) {
    switch (n) {
        case 3: return grid_n<3, R>(n_sm, n_quart);
        case 6: return grid_n<6, R>(n_sm, n_quart);
        case 9: return grid_n<9, R>(n_sm, n_quart);
        case 12: return grid_n<12, R>(n_sm, n_quart);
        case 15: return grid_n<15, R>(n_sm, n_quart);
        default: return 0;
    }
}

template <typename R>
cudaError_t launch_prec4(const FourPhArgs &a, int grid, cudaStream_t s) {
    switch (a.mesh.n_mode) {
        case 3: return launch_n4<3, R>(a, grid, s);
        case 6: return launch_n4<6, R>(a, grid, s);
        case 9: return launch_n4<9, R>(a, grid, s);
        case 12: return launch_n4<12, R>(a, grid, s);
        case 15: return launch_n4<15, R>(a, grid, s);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace

int fourphonon_grid(int n, int precision, int n_sm, int n_quart) {
    if (n_quart <= 0) return 0;
    return precision == 0 ? grid_prec<double>(n, n_sm, n_quart) : grid_prec<float>(n, n_sm, n_quart);
}

size_t fourphonon_scratch_bytes(int n, int precision, int grid) {
    const size_t cs = precision == 0 ? sizeof(double2) : sizeof(float2);
    return (size_t)grid * n * n * n * n * cs;
}

cudaError_t launch_fourphonon(const FourPhArgs &a, int precision, int grid, cudaStream_t s) {
    if (a.n_quart <= 0 || grid <= 0) return cudaSuccess;
    if (precision == 0) return launch_prec4<double>(a, grid, s);
    return launch_prec4<float>(a, grid, s);
}

}  // namespace tdg
