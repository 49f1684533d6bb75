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
// Delta weights stay FP64 as in the reference. GB300's FP64 pipe is narrow and the mode
// triplets whose Gaussians fall inside the 8-sigma window of lo_gauss are sparse, so:
//   1. the reference's skip rules become per-triplet bit masks (3 n^2 FP64 compares);
//   2. every mode triplet and each of the four Gaussians of get_dirac is screened in FP32
//      against the window, with a relative margin of 1e-3 and an absolute margin far
//      above FP32 rounding (a Gaussian the screen drops is exactly 0 in the reference);
//   3. the survivors are compacted into a shared-memory queue (block scan) and evaluated
//      in FP64 by full warps, with the reference's own window test and formulas.
//
// Everything for one triplet lives in shared memory. Precision R is double (FP64 path)
// or float (mixed path: FP32 pretransform and contraction, FP64 delta weights,
// occupations and accumulation).
#include <cuda_runtime.h>

#include "dev_common.cuh"
#include "k3_parts.cuh"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr int kPhaseChunk = 512;
// Phase factors held in shared memory at a time: at least kPhaseChunk, more when the survivor
// queue, which later reuses the eigenvector and phase region, is larger anyway (n = 15 in
// FP32: 1008, so that 1115 force-constant triplets take two passes instead of three at no
// cost in shared memory).
__host__ __device__ constexpr int phase_chunk(int n, int cs) {
    const int ez = (cs * n * n + 15) / 16 * 16;
    const int qsz = (4 * n * n * n + 15) / 16 * 16;
    const int room = (qsz - 3 * ez) / cs / 16 * 16;
    return room > kPhaseChunk ? room : kPhaseChunk;
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

// The adjoint accumulates d L / d mwm per CTA: FP64 runs in FP64 (in shared memory when the
// n_fc3 * 27 entries fit, else straight into the CTA's FP64 slice in global memory); mixed
// runs in FP32 (flushed every kAdjFlush q-triplets from shared memory) into a slice of
// floats, summed over the slices in FP64 afterwards. GB300's FP64 pipe runs at 1/64 of the
// FP32 rate and every q-triplet adds into all n_fc3 * 27 entries: FP64 additions and
// conversions there were half of the mixed adjoint's FP64 pipe, and 4-byte slices keep the
// per-CTA slices of a large force-constant set (456 x 120 KB at n_fc3 = 1115) in L2 where
// (hi, lo) pairs spilled to DRAM. A slice takes a few hundred q-triplets' terms.
constexpr int kAdjFlush = 64;

// exp(-2 pi i (q2.lv2 + q3.lv3)) of force-constant triplet t as an exact root of unity:
// q = g/N on the mesh and lv integer, so the phase is twiddle[K] with
// K = sum_d ((g2_d lv2_d + g3_d lv3_d) mod N_d) L/N_d mod L, L = lcm(N). Since N_d (L/N_d) = L
// the inner reductions can be dropped: K = (sum_d (g2_d L/N_d) lv2_d + (g3_d L/N_d) lv3_d)
// mod L, the same integer with one division instead of four; u2, u3 hold g_d L/N_d of the
// q-triplet.
template <typename C>
__device__ __forceinline__ C phase3(const Fc3Dev &fc, const MeshDev &m, const int *u2, const int *u3, int t) {
    const int32_t *lv = fc.lv + (size_t)t * 6;
    int S = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) S += u2[d] * lv[d] + u3[d] * lv[3 + d];
    int K = S % m.L;
    if (K < 0) K += m.L;
    return twiddle_at<C>(fc, K);
}


// Shared-memory layout (bytes) for mode count n and complex size cs.
struct Layout {
    size_t om1, om2, om3, inv1, be2, be3, s1, s2, s3, v1, v2, v3, wrow, r2, f32, masks, E1, E2, E3, ph, Q, A, B,
        rowid, red, wsum, xb, total;
};
__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
// adj: the adjoint's extra n^2 doubles (column sums of the scattering-matrix cotangent).
__host__ __device__ inline Layout make_layout(int n, int cs, bool adj = false) {
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
    L.f32 = o; o += align16(sizeof(float) * n * 12);           // om1..3, s1..3, om lo parts, be2, be3, wrow in FP32
    L.masks = o; o += align16(sizeof(uint32_t) * (3 * n + 2 + 2 * n2));  // m12, m13, m23, z2, z3, row/col bits
    // E1..E3 and the phase chunk are dead once Psi is formed: the survivor queue reuses them.
    const size_t ez = align16(cs * n2);
    L.E1 = o;
    L.E2 = o + ez;
    L.E3 = o + 2 * ez;
    L.ph = o + 3 * ez;
    const size_t eph = 3 * ez + align16((size_t)cs * phase_chunk(n, cs));
    const size_t qsz = align16(sizeof(uint32_t) * n3);
    L.Q = o;
    o += eph > qsz ? eph : qsz;
    // A and B each hold n^3 complex values and at least n^3 doubles.
    const size_t csz = (size_t)cs > sizeof(double) ? (size_t)cs : sizeof(double);
    const size_t buf = align16(csz * n3);
    L.A = o; o += buf;
    L.B = o; o += buf;
    L.rowid = o; o += align16(sizeof(int) * n);
    L.red = o; o += align16(sizeof(int2) * kMaxRed);
    L.wsum = o; o += align16(sizeof(int) * 33);
    // The adjoint's xi_bar sums over b2 (n^2 doubles) live in the survivor-queue region: they
    // are written after the survivors are done and read before the eigenvectors are loaded
    // there again (4 n^3 >= 8 n^2 bytes). Keeping them separate cost 1.8 KB at n = 15 and
    // the third CTA per SM.
    L.xb = L.Q;
    (void)adj;
    L.total = o;
    return L;
}

__host__ __device__ constexpr int threads_for(int n) { return ((n * n + 31) / 32) * 32; }
// Resident CTAs per SM the register budget is sized for; FP64 buffers at n >= 12 already
// limit residency through shared memory. At n = 6 the FP32 forward pass runs faster with 16
// CTAs of 64 threads at 64 registers (a few spills) than with 12; the FP64 pass and the
// adjoint, with their larger live state, keep 12.
__host__ __device__ constexpr int min_blocks_for(int n, bool dbl, bool adj) {
    return n <= 3 ? 16
                  : (n <= 6 ? (adj || dbl ? 12 : 16)
                            : (n <= 9 ? 6 : (dbl ? (n <= 12 ? 2 : 1) : (n <= 15 ? 3 : 2))));
}

// ADJ = false: Gamma and the Xi row terms. ADJ = true: the adjoint pass, which recomputes
// the same Psi and delta weights and accumulates d L / d mwm for the row cotangents a.lam.
template <int N, typename R, bool ADJ>
__global__ void __launch_bounds__(threads_for(N), min_blocks_for(N, sizeof(R) == 8, ADJ)) k_threephonon(ThreePhArgs a) {
    using C = typename CT<R>::C;
    constexpr int N2 = N * N, N3 = N2 * N;
    constexpr int NA = N / 3;
    constexpr uint32_t kAll = (N >= 32) ? 0xffffffffu : ((1u << N) - 1u);
    extern __shared__ __align__(16) unsigned char smem[];
    const Layout L = make_layout(N, sizeof(C), ADJ);
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
    uint32_t *m12 = (uint32_t *)(smem + L.masks);
    uint32_t *m13 = m12 + N, *m23 = m13 + N, *zmask = m23 + N;  // zmask[0]: omega2 < tol, zmask[1]: omega3 < tol
    // b3 with a non-zero F for each (b1, b2), and b2 for each (b1, b3): the row and column sums
    // then add only those terms (adding an exact zero changes nothing)
    uint32_t *rowbits = zmask + 2, *colbits = rowbits + N2;
    C *E1 = (C *)(smem + L.E1);
    C *E2 = (C *)(smem + L.E2);
    C *E3 = (C *)(smem + L.E3);
    C *ph = (C *)(smem + L.ph);
    uint32_t *Q = (uint32_t *)(smem + L.Q);
    C *A = (C *)(smem + L.A);
    C *B = (C *)(smem + L.B);
    int *rowid = (int *)(smem + L.rowid);
    int2 *red = (int2 *)(smem + L.red);
    int *wsum = (int *)(smem + L.wsum);
    K3Smem S;
    S.om1 = om1; S.om2 = om2; S.om3 = om3; S.inv1 = inv1; S.be2 = be2; S.be3 = be3;
    S.s1 = s1; S.s2 = s2; S.s3 = s3; S.v1 = v1; S.v2 = v2; S.v3 = v3; S.wrow = wrow;
    S.R2 = R2; S.R3 = (double *)B; S.F = (double *)A; S.Ff = nullptr;
    S.R2s = S.R3 + N2; S.R3s = S.R2s + N2;  // B (8 n^3 or more bytes) is free when the sums start
    S.fo1 = fo1; S.fo2 = fo2; S.fo3 = fo3; S.fs1 = fs1; S.fs2 = fs2; S.fs3 = fs3;
    S.fl1 = fs3 + N; S.fl2 = fs3 + 2 * N; S.fl3 = fs3 + 3 * N; S.fb2 = fs3 + 4 * N; S.fb3 = fs3 + 5 * N;
    S.fw1 = fs3 + 6 * N;
    S.m12 = m12; S.m13 = m13; S.m23 = m23; S.zmask = zmask; S.rowbits = rowbits; S.colbits = colbits;
    S.Q = Q; S.rowid = rowid; S.red = red; S.wsum = wsum;
    const int tid = threadIdx.x, bd = blockDim.x;
    const MeshDev &m = a.mesh;
    const PhononDev &P = a.ph;
    const Fc3Dev &fc = a.fc;
    const R *mwm = mwm_ptr<R>(fc);
    const C *egvs = egvs_ptr<C>(P);
    const int64_t ld = (int64_t)m.n_full * N;
    const int it = P.integrationtype;
    const float sigfix32 = (float)P.sigma_fixed;
    R *acc = (R *)(smem + L.total);  // ADJ with acc_in_smem: [fc.n * 27]
    int since_flush = 0;
    if constexpr (ADJ) {
        if (a.acc_in_smem)
            for (int i = tid; i < fc.n * 27; i += bd) acc[i] = (R)0;
    }

    // the next q-triplet's record is loaded one iteration ahead, so that the per-mode loads
    // of an iteration wait for one round trip to memory instead of two
    TripletRec rec_next = blockIdx.x < a.n_trip ? a.trip[blockIdx.x] : TripletRec{};
    for (int t = blockIdx.x; t < a.n_trip; t += gridDim.x) {
        const TripletRec rec = rec_next;
        if (t + (int)gridDim.x < a.n_trip) rec_next = a.trip[t + gridDim.x];
        const int f1 = m.irr_full[rec.q1];
        const int q2 = rec.q2, q3 = rec.q3;
        const int i2 = m.full_irr[q2], i3 = m.full_irr[q3];
        const int nred = rec.red_cnt;
        const double perm = (q2 == q3) ? 1.0 : 2.0;
        k3_load_modes<N>(S, a, rec, f1, q2, q3, i2, i3);
        for (int i = tid; i < 3 * N2; i += bd) {
            const int which = i / N2, e = i % N2;
            const int r = e / N, b = e % N;  // element (r) of mode b
            const int q = which == 0 ? f1 : (which == 1 ? q2 : q3);
            C *E = which == 0 ? E1 : (which == 1 ? E2 : E3);
            E[r * N + b] = egvs[((size_t)q * N + b) * N + r];
        }
        for (int i = tid; i < N3; i += bd) A[i] = czero<C>();
        __syncthreads();
        // ---- skip rules of scattering_threephonon.f90:90-101 as bit masks ----
        k3_skip_masks<N>(S);
        // ---- K2: pretransform into A ----
        int gi2[3], gi3[3];
        {
            const int n12 = m.grid[1] * m.grid[2];
            gi2[0] = q2 / n12; gi2[1] = (q2 / m.grid[2]) % m.grid[1]; gi2[2] = q2 % m.grid[2];
            gi3[0] = q3 / n12; gi3[1] = (q3 / m.grid[2]) % m.grid[1]; gi3[2] = q3 % m.grid[2];
            for (int d = 0; d < 3; ++d) {  // g_d L/N_d (phase3)
                gi2[d] *= m.lmul[d];
                gi3[d] *= m.lmul[d];
            }
        }
        constexpr int PC = phase_chunk(N, sizeof(C));
        bool planned = false;
        if constexpr (sizeof(R) == 4) {
            // FP32 with a pretransform plan (all phase factors at once; k_threephonon_tc.cu
            // explains the plan): each thread's slots, 8 values and 8 words in flight, the
            // sums in the triplets' order as below
            if (a.plan_slots > 0) {
                planned = true;
                __syncthreads();
                // four triplets per thread in flight: their lattice vectors, then their table entries
                for (int i0 = tid; i0 < fc.n + 4; i0 += 4 * bd) {
                    int kk[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int i = i0 + u * bd;
                        kk[u] = -1;
                        if (i < fc.n) {
                            const int32_t *lv = fc.lv + (size_t)i * 6;
                            int S2 = 0;
#pragma unroll
                            for (int d = 0; d < 3; ++d) S2 += gi2[d] * __ldg(lv + d) + gi3[d] * __ldg(lv + 3 + d);
                            int K = S2 % m.L;
                            kk[u] = K < 0 ? K + m.L : K;
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int i = i0 + u * bd;
                        if (i < fc.n + 4) ph[i] = kk[u] >= 0 ? twiddle_at<C>(fc, kk[u]) : czero<C>();
                    }
                }
                __syncthreads();
                const float4 *pm = a.plan_pm + tid;
                const uint32_t *pw = a.plan_word + tid;
                float ar = 0.f, ai = 0.f;
#pragma unroll 1
                for (int s0 = 0; s0 < a.plan_slots; s0 += 8) {
                    float4 mv[8];
                    uint32_t wd[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        mv[u] = __ldg(pm + (size_t)(s0 + u) * bd);
                        wd[u] = __ldg(pw + (size_t)(s0 + u) * bd);
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const C *pp = ph + (wd[u] & 0xffffu);
                        const C p0 = pp[0], p1 = pp[1], p2 = pp[2], p3 = pp[3];
                        ar = fmaf(mv[u].x, p0.x, ar); ai = fmaf(mv[u].x, p0.y, ai);
                        ar = fmaf(mv[u].y, p1.x, ar); ai = fmaf(mv[u].y, p1.y, ai);
                        ar = fmaf(mv[u].z, p2.x, ar); ai = fmaf(mv[u].z, p2.y, ai);
                        ar = fmaf(mv[u].w, p3.x, ar); ai = fmaf(mv[u].w, p3.y, ai);
                        const uint32_t oc = wd[u] >> 16;  // on an element's last slot: its index + 1
                        if (oc) {
                            A[oc - 1u].x = ar;
                            A[oc - 1u].y = ai;
                            ar = 0.f;
                            ai = 0.f;
                        }
                    }
                }
            }
        }
        for (int c0 = 0; !planned && c0 < fc.n; c0 += PC) {
            const int cn = min(PC, fc.n - c0);
            __syncthreads();
            for (int i = tid; i < cn; i += bd) ph[i] = phase3<C>(fc, m, gi2, gi3, c0 + i);
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
        // ---- Psi into B; FP32 screen of the Gaussians, survivors counted per thread ----
        uint32_t live_lo = 0u, live_hi = 0u;  // 4-bit live masks of b3 = 0..7 and 8..15
        uint32_t live_x = 0u;                 // b3 = 16, 17
        int nsurv = 0;
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
#pragma unroll
            for (int b3 = 0; b3 < N; ++b3) B[(b1 * N + b2) * N + b3] = acc[b3];
            nsurv = k3_screen<N>(S, it, sigfix32, b1, b2, live_lo, live_hi, live_x);
        }
        int nq = 0;
        const int off = block_exclusive_scan(nsurv, wsum, nq);  // contains __syncthreads
        // E1..E3 and the phases are dead: the queue overwrites them.
        if (tid < N2 && nsurv) k3_enqueue<N>(S, tid, off, live_lo, live_hi, live_x);
        // dense F (doubles) in A; the forward pass reads it only where the row/column bits
        // are set (entries its survivors wrote), the adjoint all of it (zero where no survivor)
        double *F = (double *)A;
        if constexpr (ADJ)
            for (int i = tid; i < N3; i += bd) F[i] = 0.0;
        __syncthreads();
        // ---- delta weights and occupations for the survivors, full warps: FP64 for FP64
        // runs, FP32 (from FP64 centre differences) in mixed precision, as the tensor-core
        // kernel; the adjoint keeps d F / d|Psi|^2, i.e. F without |Psi|^2 ----
        if constexpr (sizeof(R) == 8) {
            k3_survivors<N>(S, P, nq, perm, [&](int idx) -> double {
                if constexpr (ADJ) {
                    return 1.0;
                } else {
                    const C psi = B[idx];
                    return (double)psi.x * (double)psi.x + (double)psi.y * (double)psi.y;
                }
            });
        } else {
            k3_survivors_f32<N>(S, P, nq, (float)perm, [&](int idx) -> float {
                if constexpr (ADJ) {
                    return 1.0f;
                } else {
                    const C psi = B[idx];
                    return (float)psi.x * (float)psi.x + (float)psi.y * (float)psi.y;
                }
            });
        }
        __syncthreads();
        if constexpr (ADJ) {
            // d L / d|Psi_b|^2 = lam[row(b1)] * nred * dF_b/d|Psi_b|^2 (Gamma += nred * sum F);
            // d|Psi|^2 / d P[abc] = 2 Re(conj(Psi) E1[a][b1] E2[b][b2] E3[c][b3]), so with
            // W = G conj(Psi):  Q[abc] = sum_b W_b E1[a][b1] E2[b][b2] E3[c][b3] and
            // d L / d mwm_t(i,j,k) = 2 Re(phase_t Q[3a1+i][3a2+j][3a3+k]).
            // with a scattering-matrix cotangent xi_bar (the BTE adjoint): the Xi row terms
            // 2 F om2/om1 at (q2', b2) and 2 F om3/om1 at (q3', b3) of every equivalent
            // triplet add xi_bar(row, .) times those factors to the cotangent of F;
            // R2[b1][b2] and XB[b1][b3] hold xi_bar summed over the equivalent triplets
            double *XB = (double *)(smem + L.xb);
            if (a.xi_bar) {
                for (int e = tid; e < 2 * N2; e += bd) {
                    const int x = e % N2, b1 = x / N, bb = x % N, row = rowid[b1];
                    double sum = 0.0;
                    if (row >= 0) {
                        const double *wr = a.xi_bar + (int64_t)row * ld;
                        for (int k = 0; k < nred; ++k) {
                            const int2 pr = red[k];
                            sum += wr[(int64_t)(e < N2 ? pr.x : pr.y) * N + bb];
                        }
                    }
                    if (e < N2) R2[x] = sum;
                    else XB[x] = sum;
                }
                __syncthreads();
            }
            for (int i = tid; i < N3; i += bd) {
                const int row = rowid[i / N2];
                double cot = row >= 0 ? a.lam[row] * (double)nred : 0.0;
                if (a.xi_bar && row >= 0) {
                    const int b1 = i / N2, b2 = (i / N) % N, b3 = i % N;
                    cot += 2.0 * (om2[b2] * R2[b1 * N + b2] + om3[b3] * XB[b1 * N + b3]) * inv1[b1];
                }
                const double g = cot * F[i];
                const C psi = B[i];
                C w;
                w.x = (R)(g * (double)psi.x);
                w.y = (R)(-g * (double)psi.y);
                B[i] = w;
            }
            __syncthreads();  // XB shares the eigenvectors' region
            // the survivor queue overwrote the eigenvectors: load them again
            for (int i = tid; i < 3 * N2; i += bd) {
                const int which = i / N2, e = i % N2;
                const int r = e / N, b = e % N;
                const int q = which == 0 ? f1 : (which == 1 ? q2 : q3);
                C *E = which == 0 ? E1 : (which == 1 ? E2 : E3);
                E[r * N + b] = egvs[((size_t)q * N + b) * N + r];
            }
            __syncthreads();
            if (tid < N2) {  // A[a][b2b3] = sum_b1 E1[a][b1] W[b1][b2b3]
                const int bc = tid;
                C acc[N];
#pragma unroll
                for (int x = 0; x < N; ++x) acc[x] = czero<C>();
#pragma unroll 3
                for (int b1 = 0; b1 < N; ++b1) {
                    const C w = B[b1 * N2 + bc];
#pragma unroll
                    for (int x = 0; x < N; ++x) cfma(acc[x], E1[x * N + b1], w);
                }
#pragma unroll
                for (int x = 0; x < N; ++x) A[x * N2 + bc] = acc[x];
            }
            __syncthreads();
            if (tid < N2) {  // B[a][b][b3] = sum_b2 E2[b][b2] A[a][b2][b3]
                const int aa = tid / N, b3 = tid % N;
                C acc[N];
#pragma unroll
                for (int x = 0; x < N; ++x) acc[x] = czero<C>();
#pragma unroll 3
                for (int b2 = 0; b2 < N; ++b2) {
                    const C tv = A[(aa * N + b2) * N + b3];
#pragma unroll
                    for (int x = 0; x < N; ++x) cfma(acc[x], E2[x * N + b2], tv);
                }
#pragma unroll
                for (int x = 0; x < N; ++x) B[(aa * N + x) * N + b3] = acc[x];
            }
            __syncthreads();
            if (tid < N2) {  // A[a][b][c] = sum_b3 E3[c][b3] B[a][b][b3]
                const int ab = tid;
                C acc[N];
#pragma unroll
                for (int x = 0; x < N; ++x) acc[x] = czero<C>();
#pragma unroll 3
                for (int b3 = 0; b3 < N; ++b3) {
                    const C tv = B[ab * N + b3];
#pragma unroll
                    for (int x = 0; x < N; ++x) cfma(acc[x], E3[x * N + b3], tv);
                }
#pragma unroll
                for (int x = 0; x < N; ++x) A[ab * N + x] = acc[x];
            }
            // the CTA's slice: doubles on the FP64 path, floats on the mixed path (contiguous
            // slices of n_fc3 * 27 entries of either type)
            double *slice = a.mwm_bar + (size_t)blockIdx.x * fc.n * 27;
            float *slicef = reinterpret_cast<float *>(a.mwm_bar) + (size_t)blockIdx.x * fc.n * 27;
            // thread -> one (i,j,k) of the 27 and every groups-th force-constant triplet; within a
            // q-triplet exactly one thread touches each entry, and q-triplets are separated by
            // barriers
            const int groups = bd / 27, grp = tid / 27, ijk = tid % 27;
            const int off = (ijk % 3) * N2 + ((ijk / 3) % 3) * N + ijk / 9;
            constexpr int PCA = phase_chunk(N, sizeof(C));
            for (int c0 = 0; c0 < fc.n; c0 += PCA) {
                const int cn = min(PCA, fc.n - c0);
                __syncthreads();
                for (int i = tid; i < cn; i += bd) ph[i] = phase3<C>(fc, m, gi2, gi3, c0 + i);
                __syncthreads();
                if (grp < groups) {
                    for (int tl = grp; tl < cn; tl += groups) {
                        const int tt = c0 + tl;
                        const C q = A[fc.abase[tt] + off];
                        const C p = ph[tl];
                        const R v = (R)2 * (p.x * q.x - p.y * q.y);
                        if (a.acc_in_smem) {
                            acc[(size_t)tt * 27 + ijk] += v;
                        } else if constexpr (sizeof(R) == 8) {
                            slice[(size_t)tt * 27 + ijk] += (double)v;
                        } else {
                            slicef[(size_t)tt * 27 + ijk] += (float)v;
                        }
                    }
                }
            }
            __syncthreads();
            if (a.acc_in_smem && ++since_flush == kAdjFlush) {
                for (int i = tid; i < fc.n * 27; i += bd) {
                    if constexpr (sizeof(R) == 8)
                        slice[i] += (double)acc[i];
                    else
                        slicef[i] += (float)acc[i];
                    acc[i] = (R)0;
                }
                since_flush = 0;
                __syncthreads();
            }
            continue;
        }
        // ---- R2 = sum over b3, R3 = sum over b2 (into B as doubles), Gamma and Xi ----
        k3_sums_scatter<N>(S, a, nred);
    }
    if constexpr (ADJ) {
        if (a.acc_in_smem) {
            __syncthreads();
            double *slice = a.mwm_bar + (size_t)blockIdx.x * fc.n * 27;
            float *slicef = reinterpret_cast<float *>(a.mwm_bar) + (size_t)blockIdx.x * fc.n * 27;
            for (int i = tid; i < fc.n * 27; i += bd) {
                if constexpr (sizeof(R) == 8)
                    slice[i] += (double)acc[i];
                else
                    slicef[i] += (float)acc[i];
            }
        }
    }
}

// Persistent grid: resident CTAs per SM times the SM count, at most one CTA per item.
// `extra` bytes of dynamic shared memory follow the kernel's layout (adjoint accumulator).
template <int N, typename R, bool ADJ>
int grid_n(int n_sm, int n_trip, size_t extra, int ctas_per_sm = 0, int *api = nullptr, int *count = nullptr) {
    const Layout L = make_layout(N, sizeof(typename CT<R>::C), ADJ);
    const size_t bytes = L.total + extra;
    int per_sm = resident_ctas((const void *)k_threephonon<N, R, ADJ>, threads_for(N), bytes, api, count);
    if (per_sm < 1) return 0;
    if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
    const int grid = n_sm * per_sm;
    return grid > n_trip ? (n_trip > 0 ? n_trip : 1) : grid;
}

template <int N, typename R, bool ADJ>
cudaError_t launch_grid(const ThreePhArgs &a, int grid, size_t extra, cudaStream_t s) {
    const Layout L = make_layout(N, sizeof(typename CT<R>::C), ADJ);
    k_threephonon<N, R, ADJ><<<grid, threads_for(N), L.total + extra, s>>>(a);
    return cudaGetLastError();
}

template <int N, typename R>
cudaError_t launch_n(const ThreePhArgs &a, int n_sm, int ctas_per_sm, cudaStream_t s) {
    const int grid = grid_n<N, R, false>(n_sm, a.n_trip, 0, ctas_per_sm);
    if (grid < 1) return cudaErrorInvalidConfiguration;
    return launch_grid<N, R, false>(a, grid, 0, s);
}

template <typename R, bool ADJ>
int grid_prec(int n, int n_sm, int n_trip, size_t extra, int *api = nullptr, int *count = nullptr) {
    switch (n) {
        case 3: return grid_n<3, R, ADJ>(n_sm, n_trip, extra, 0, api, count);
        case 6: return grid_n<6, R, ADJ>(n_sm, n_trip, extra, 0, api, count);
        case 9: return grid_n<9, R, ADJ>(n_sm, n_trip, extra, 0, api, count);
        case 12: return grid_n<12, R, ADJ>(n_sm, n_trip, extra, 0, api, count);
        case 15: return grid_n<15, R, ADJ>(n_sm, n_trip, extra, 0, api, count);
        case 18: return grid_n<18, R, ADJ>(n_sm, n_trip, extra, 0, api, count);
        default: return 0;
    }
}

template <typename R>
cudaError_t launch_adj_prec(const ThreePhArgs &a, int grid, size_t extra, cudaStream_t s) {
    switch (a.mesh.n_mode) {
        case 3: return launch_grid<3, R, true>(a, grid, extra, s);
        case 6: return launch_grid<6, R, true>(a, grid, extra, s);
        case 9: return launch_grid<9, R, true>(a, grid, extra, s);
        case 12: return launch_grid<12, R, true>(a, grid, extra, s);
        case 15: return launch_grid<15, R, true>(a, grid, extra, s);
        case 18: return launch_grid<18, R, true>(a, grid, extra, s);
        default: return cudaErrorNotSupported;
    }
}

__global__ void k_sum_slices(const double *slices, int32_t n_slice, int64_t n, double *out) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int g = 0; g < n_slice; ++g) acc += slices[(int64_t)g * n + e];
        out[e] = acc;
    }
}

// The same over float slices (mixed-precision adjoint).
__global__ void k_sum_slices_f(const float *slices, int32_t n_slice, int64_t n, double *out) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int g = 0; g < n_slice; ++g) acc += (double)slices[(int64_t)g * n + e];
        out[e] = acc;
    }
}

template <typename R>
cudaError_t launch_prec(const ThreePhArgs &a, int n_sm, int ctas_per_sm, cudaStream_t s) {
    switch (a.mesh.n_mode) {
        case 3: return launch_n<3, R>(a, n_sm, ctas_per_sm, s);
        case 6: return launch_n<6, R>(a, n_sm, ctas_per_sm, s);
        case 9: return launch_n<9, R>(a, n_sm, ctas_per_sm, s);
        case 12: return launch_n<12, R>(a, n_sm, ctas_per_sm, s);
        case 15: return launch_n<15, R>(a, n_sm, ctas_per_sm, s);
        case 18: return launch_n<18, R>(a, n_sm, ctas_per_sm, s);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace

namespace {
__global__ void k_exp_neg_check(const double *t, int32_t n, double *out, const double *tab) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = exp_neg(t[i], tab);
}
}  // namespace

cudaError_t launch_exp_neg_check(const double *t, int32_t n, double *out, const double *tab, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_exp_neg_check<<<(n + 255) / 256, 256, 0, s>>>(t, n, out, tab);
    return cudaGetLastError();
}

int threephonon_threads(int n) { return threads_for(n); }

bool threephonon_plan_fits(int n, int n_fc) {
    // the plan path holds all phase factors (and 4 zero ones after them) in the phase region
    return n >= 3 && n <= 16 && n_fc + 4 <= phase_chunk(n, (int)sizeof(float2));
}

size_t threephonon_smem_bytes(int n, int precision, int) {
    return make_layout(n, precision == 0 ? sizeof(double2) : sizeof(float2)).total;
}

cudaError_t launch_threephonon(const ThreePhArgs &a, int precision, int n_sm, int ctas_per_sm, cudaStream_t s) {
    if (a.n_trip <= 0) return cudaSuccess;
    if (precision == 0) return launch_prec<double>(a, n_sm, ctas_per_sm, s);
    return launch_prec<float>(a, n_sm, ctas_per_sm, s);
}

int threephonon_max_per_sm(int n, int precision, int *api, int *count) {
    // grid_n with one SM and an unbounded item count gives the CTAs that fit on one SM
    return precision == 0 ? grid_prec<double, false>(n, 1, 1 << 30, 0, api, count)
                          : grid_prec<float, false>(n, 1, 1 << 30, 0, api, count);
}

int threephonon_adjoint_grid(int n, int precision, int n_sm, int n_trip, int n_fc, bool acc_in_smem) {
    const size_t extra = acc_in_smem ? (size_t)n_fc * 27 * (precision == 0 ? sizeof(double) : sizeof(float)) : 0;
    return precision == 0 ? grid_prec<double, true>(n, n_sm, n_trip, extra)
                          : grid_prec<float, true>(n, n_sm, n_trip, extra);
}

cudaError_t launch_threephonon_adjoint(const ThreePhArgs &a, int precision, int grid, cudaStream_t s) {
    if (a.n_trip <= 0 || grid <= 0) return cudaSuccess;
    const size_t extra =
        a.acc_in_smem ? (size_t)a.fc.n * 27 * (precision == 0 ? sizeof(double) : sizeof(float)) : 0;
    if (precision == 0) return launch_adj_prec<double>(a, grid, extra, s);
    return launch_adj_prec<float>(a, grid, extra, s);
}

cudaError_t launch_sum_slices(const double *slices, int32_t n_slice, int64_t n, int precision, double *out,
                              cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int64_t blocks = (n + 255) / 256;
    const unsigned g = (unsigned)(blocks < 4096 ? blocks : 4096);
    if (precision == 0)
        k_sum_slices<<<g, 256, 0, s>>>(slices, n_slice, n, out);
    else
        k_sum_slices_f<<<g, 256, 0, s>>>(reinterpret_cast<const float *>(slices), n_slice, n, out);
    return cudaGetLastError();
}

}  // namespace tdg
