// Large-cell three-phonon path (n_mode beyond the shared-memory kernel, e.g. a 40-atom cell
// with 120 modes): the same arithmetic as k_threephonon, restructured for n^3 tensors that
// do not fit on chip, with the Psi contraction on the tcgen05 tensor cores.
//
// Per batch of q-triplets (one slot each):
//   phases  exp(-2 pi i (q2.lv2 + q3.lv3)) of every force-constant triplet (exact roots of unity)
//   P       pretransform_phi3 (scattering_threephonon.f90:275-317) into the stage-1 operand
//   3 GEMM  stages, each contracting the leading component index of the tensor with one
//           eigenvector matrix: X[(ri,a)][(b,c)] -> Y[(b,c)][(ri',b1)] with the complex product
//           written as a real one, [Yr | Yi] = [Xr | Xi] [[Er, Ei], [-Ei, Er]]; the epilogue
//           writes the next stage's operand with the new index last, so that after
//           contracting a (E1), b (E2) and c (E3) the result is Psi[b1][b2][b3]
//   delta   get_dirac and the accumulation of Gamma and the Xi row terms
//           (scattering_threephonon.f90:115-135, 219-271), FP64 weights and sums.
// GEMM operands are BF16 hi/lo splits of FP32 values (hi*hi + hi*lo + lo*hi into an FP32
// tensor-memory accumulator, about 16 significant bits per operand) in shared memory as
// 8 x 16-byte core matrices without swizzle, both operands MN-major; the layout and the
// descriptor reading (leading byte offset = K-direction core stride, stride byte offset =
// MN-direction core stride) are the ones the one-tile self-check verifies.
#include <cuda_bf16.h>

#include "dev_common.cuh"
#include "tc_common.cuh"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr double kLnPrefactor = 3.141592653589793 / 16.0;
constexpr long long kLnWaitCycles = 4000000000LL;  // about 2 s at 2 GHz

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void store_split(__nv_bfloat16 *hi, __nv_bfloat16 *lo, int64_t i, float v) {
    unsigned short h, l;
    tc::split_bf16(v, h, l);
    hi[i] = __ushort_as_bfloat16(h);
    lo[i] = __ushort_as_bfloat16(l);
}

// ---- real-split eigenvector matrices of every mesh point ----
// bmat[((q*2 + h)*kp + k)*kp + c], h = 0 hi / 1 lo; k = ri*n + a, c = rj*n + b:
// [[Er, Ei], [-Ei, Er]] with E[a][b] = component a of mode b of egv/sqrt(omega).
// With transpose, E is replaced by its transpose (E^T[a][b] = E[b][a]): the matrices of the
// adjoint's back-contraction, which turns a mode index back into a component index.
__global__ void k_build_bmat(int n, int kp, int n_q, const float2 *egvs32, __nv_bfloat16 *bmat, int transpose) {
    const int64_t per = (int64_t)kp * kp;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n_q * per) return;
    const int q = (int)(i / per);
    const int64_t e = i % per;
    const int k = (int)(e / kp), c = (int)(e % kp);
    float v = 0.f;
    if (k < 2 * n && c < 2 * n) {
        const int ri = k / n, a = k % n, rj = c / n, b = c % n;
        const float2 E = transpose ? egvs32[((size_t)q * n + a) * n + b] : egvs32[((size_t)q * n + b) * n + a];
        v = ri == 0 ? (rj == 0 ? E.x : E.y) : (rj == 0 ? -E.y : E.x);
    }
    store_split(bmat + ((int64_t)q * 2) * per, bmat + ((int64_t)q * 2 + 1) * per, e, v);
}

// ---- phases of the force-constant triplets, per slot ----
__global__ void k_ln_phases(Fc3Dev fc, MeshDev m, const TripletRec *trip, int nb, float2 *ph) {
    const int s = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nb || t >= fc.n) return;
    const TripletRec rec = trip[s];
    const int n12 = m.grid[1] * m.grid[2];
    const int g2[3] = {rec.q2 / n12, (rec.q2 / m.grid[2]) % m.grid[1], rec.q2 % m.grid[2]};
    const int g3[3] = {rec.q3 / n12, (rec.q3 / m.grid[2]) % m.grid[1], rec.q3 % m.grid[2]};
    const int32_t *lv = fc.lv + (size_t)t * 6;
    int K = 0;
    for (int d = 0; d < 3; ++d) {
        int kd = (g2[d] * lv[d] + g3[d] * lv[3 + d]) % m.grid[d];
        if (kd < 0) kd += m.grid[d];
        K += kd * m.lmul[d];
    }
    ph[(size_t)s * fc.n + t] = fc.twiddle32[K % m.L];
}

// ---- pretransform into the stage-1 operand: X[k][m], k = ri*n + a, m = b*n + c ----
__global__ void k_ln_pretransform(int n, int na, Fc3Dev fc, const float2 *ph, int nb, int64_t plane, int mp,
                                  __nv_bfloat16 *xhi, __nv_bfloat16 *xlo) {
    const int s = blockIdx.y;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n3 = (int64_t)n * n * n;
    if (s >= nb || e >= n3) return;
    const int nn = n * n;
    const int a = (int)(e / nn), bc = (int)(e % nn), b = bc / n, c = bc % n;
    const int blk = ((a / 3) * na + b / 3) * na + c / 3;
    const int ijk = (a % 3) + 3 * (b % 3) + 9 * (c % 3);
    float2 acc = make_float2(0.f, 0.f);
    const float2 *phs = ph + (size_t)s * fc.n;
    for (int tt = fc.blk_ptr[blk]; tt < fc.blk_ptr[blk + 1]; ++tt) {
        const float mv = __ldg(fc.mwm32 + (size_t)tt * 27 + ijk);
        const float2 p = phs[tt];
        acc.x = fmaf(mv, p.x, acc.x);
        acc.y = fmaf(mv, p.y, acc.y);
    }
    __nv_bfloat16 *hi = xhi + (int64_t)s * plane, *lo = xlo + (int64_t)s * plane;
    store_split(hi, lo, (int64_t)a * mp + bc, acc.x);
    store_split(hi, lo, (int64_t)(n + a) * mp + bc, acc.y);
}

// ---- one contraction stage on the tensor cores ----
struct LnGemmArgs {
    const __nv_bfloat16 *xhi, *xlo;  // operand planes, slot s at + s * plane: X[k][m], M stride mp
    int64_t plane;
    int mp;
    const __nv_bfloat16 *bmat;       // k_build_bmat
    const TripletRec *trip;          // the batch's q-triplets (slot order)
    const int32_t *irr_full;         // 0-based full index of irreducible q1
    int stage;                       // 1, 2, 3: contract with E(q1), E(q2), E(q3)
    int n, kp;                       // modes, padded 2n (multiple of 16)
    __nv_bfloat16 *ohi, *olo;        // stages 1-2: next operand planes
    float2 *psi;                     // stage 3: [slot][n^3]
    int32_t *status;
};

// Tile = 128 rows of M = n^2 for one slot, all kp columns. kLnStages shared-memory stages
// hold K chunks of 16 of both operands (hi and lo); cp.async keeps kLnStages - 1 chunks in
// flight ahead of the MMAs, and a stage is refilled only after the MMAs that read it have
// arrived on its mbarrier. The epilogue reads tensor memory straight into registers: warps
// w and w + 4 share TMEM lane group w and split the columns.
constexpr int kLnStages = 4;
constexpr int kLnThreads = 256;

__device__ __forceinline__ uint4 pack8(const unsigned short (&h)[8]) {
    uint4 r;
    r.x = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
    r.y = (uint32_t)h[2] | ((uint32_t)h[3] << 16);
    r.z = (uint32_t)h[4] | ((uint32_t)h[5] << 16);
    r.w = (uint32_t)h[6] | ((uint32_t)h[7] << 16);
    return r;
}

__global__ void __launch_bounds__(kLnThreads, 1) k_ln_gemm(LnGemmArgs g) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t mbar[kLnStages];
    __shared__ uint32_t tbase;
    constexpr int S = kLnStages;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int s = blockIdx.y, m0 = blockIdx.x * 128;
    const int n = g.n, kp = g.kp, M = n * n;
    const int nch = kp / 16;
    const uint32_t a_bytes = 128u * 16u * 2u, b_bytes = 16u * (uint32_t)kp * 2u;
    const uint32_t stage_bytes = 2u * (a_bytes + b_bytes);
    const uint32_t a_ck = 16u * 128u, b_ck = 16u * (uint32_t)kp;  // K-direction core strides
    const uint32_t ncols = kp <= 32 ? 32u : (kp <= 64 ? 64u : (kp <= 128 ? 128u : 256u));
    const TripletRec rec = g.trip[s];
    const int q = g.stage == 1 ? g.irr_full[rec.q1] : (g.stage == 2 ? rec.q2 : rec.q3);
    const int64_t bper = (int64_t)kp * kp;
    const __nv_bfloat16 *bsrc[2] = {g.bmat + ((int64_t)q * 2) * bper, g.bmat + ((int64_t)q * 2 + 1) * bper};
    const __nv_bfloat16 *xsrc[2] = {g.xhi + (int64_t)s * g.plane, g.xlo + (int64_t)s * g.plane};

    if (warp == 0) tc::tmem_alloc(&tbase, ncols);
    if (tid == 0) {
        for (int i = 0; i < S; ++i) tc::mbar_init(&mbar[i], 1);
        tc::fence_mbar_init();
    }
    // one cp.async group per chunk (an empty group past the end keeps the count uniform)
    auto load_chunk = [&](int c) {
        if (c < nch) {
            unsigned char *base = sm + (c % S) * stage_bytes;
            const int k0 = c * 16;
            for (int i = tid; i < 2 * 16 * 16; i += kLnThreads) {  // A: 2 planes x 16 k x 16 m-blocks
                const int h = i >> 8, k = (i >> 4) & 15, mb = i & 15;
                const uint32_t dst = tc::smem_u32(base + h * a_bytes + mb * 128 + (k >> 3) * a_ck + (k & 7) * 16);
                cp_async16(dst, xsrc[h] + (int64_t)(k0 + k) * g.mp + m0 + 8 * mb);
            }
            const int nbs = kp / 8;
            for (int i = tid; i < 2 * 16 * nbs; i += kLnThreads) {  // B: 2 planes x 16 k x kp/8 blocks
                const int h = i / (16 * nbs), r = i % (16 * nbs), k = r / nbs, nb = r % nbs;
                const uint32_t dst =
                    tc::smem_u32(base + 2 * a_bytes + h * b_bytes + nb * 128 + (k >> 3) * b_ck + (k & 7) * 16);
                cp_async16(dst, bsrc[h] + (int64_t)(k0 + k) * kp + 8 * nb);
            }
        }
        cp_async_commit();
    };
    for (int c = 0; c < S - 1; ++c) load_chunk(c);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;
    const uint32_t idesc = tc::idesc_bf16_f32(128, kp, true, true);
    // every wait ends within kLnWaitCycles; its outcome is made uniform across the CTA
    // before any thread acts on it, so that no barrier is skipped by part of the block
    bool ok = true;
    for (int c = 0; c < nch; ++c) {
        const int pf = c + S - 1;  // refills the stage chunk c - 1 used
        if (pf < nch && c >= 1) {
            const bool w = tc::mbar_wait(&mbar[(c - 1) % S], ((c - 1) / S) & 1, kLnWaitCycles);
            ok = __syncthreads_and(w ? 1 : 0) != 0;
            if (!ok) break;
        }
        load_chunk(pf);
        cp_async_wait<S - 1>();  // chunk c has landed
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            unsigned char *base = sm + (c % S) * stage_bytes;
            const uint32_t ah = tc::smem_u32(base), al = tc::smem_u32(base + a_bytes);
            const uint32_t bh = tc::smem_u32(base + 2 * a_bytes), bl = tc::smem_u32(base + 2 * a_bytes + b_bytes);
            const uint64_t dah = tc::smem_desc(ah, a_ck, 128), dal = tc::smem_desc(al, a_ck, 128);
            const uint64_t dbh = tc::smem_desc(bh, b_ck, 128), dbl = tc::smem_desc(bl, b_ck, 128);
            tc::mma_bf16(taddr, dah, dbh, idesc, c > 0 ? 1u : 0u);
            tc::mma_bf16(taddr, dah, dbl, idesc, 1u);
            tc::mma_bf16(taddr, dal, dbh, idesc, 1u);
            tc::mma_commit(&mbar[c % S]);
        }
    }
    if (ok) {
        const bool w = tc::mbar_wait(&mbar[(nch - 1) % S], ((nch - 1) / S) & 1, kLnWaitCycles);
        ok = __syncthreads_and(w ? 1 : 0) != 0;
    }
    cp_async_wait<0>();
    if (!ok) {
        if (tid == 0) atomicExch(g.status, kDevOverflow);
        // let whatever was issued drain before the tensor memory goes back
        tc::mbar_wait(&mbar[(nch - 1) % S], ((nch - 1) / S) & 1, kLnWaitCycles);
    }
    __syncthreads();
    tc::fence_after_sync();
    // ---- epilogue ----
    const int lg = warp & 3, half = warp >> 2;
    const int ml = 32 * lg + lane, m = m0 + ml;
    const uint32_t trow = taddr + ((uint32_t)(32 * lg) << 16);
    if (ok && g.stage < 3) {
        // D[m = u*n + v][ri*n + w] -> X'[(ri*n + u)*mp + v*n + w]
        __nv_bfloat16 *hi = g.ohi + (int64_t)s * g.plane, *lo = g.olo + (int64_t)s * g.plane;
        const int u = m / n, v = m % n;
        const int c_lo = half * (kp / 2), c_hi = c_lo + kp / 2;
        for (int c0 = c_lo; c0 < c_hi; c0 += 8) {
            float x[8];
            tc::tmem_ld8(trow + (uint32_t)c0, x);
            if (m >= M) continue;
            if (n % 8 == 0 && c0 + 8 <= 2 * n) {
                const int ri = c0 / n, w0 = c0 % n;
                unsigned short h[8], l[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) tc::split_bf16(x[i], h[i], l[i]);
                const int64_t o = (int64_t)(ri * n + u) * g.mp + v * n + w0;
                *reinterpret_cast<uint4 *>(hi + o) = pack8(h);
                *reinterpret_cast<uint4 *>(lo + o) = pack8(l);
            } else {
                for (int i = 0; i < 8; ++i) {
                    const int c = c0 + i;
                    if (c >= 2 * n) break;
                    store_split(hi, lo, (int64_t)((c / n) * n + u) * g.mp + v * n + c % n, x[i]);
                }
            }
        }
    } else if (ok) {
        // Psi[m][w] = (D[m][w], D[m][n + w]); the two halves take the w ranges
        float2 *out = g.psi + (int64_t)s * M * n;
        const int wh = ((n + 15) / 16) * 8;  // w range of half 0, a multiple of 8
        const int w_lo = half * wh, w_hi = min(n, w_lo + wh);
        for (int w0 = w_lo; w0 < w_hi; w0 += 8) {
            float re[8], im[8];
            tc::tmem_ld8(trow + (uint32_t)w0, re);
            tc::tmem_ld8(trow + (uint32_t)(n + w0), im);
            if (m >= M) continue;
            for (int i = 0; i < 8 && w0 + i < w_hi; ++i) out[(int64_t)m * n + w0 + i] = make_float2(re[i], im[i]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, ncols);
}

// ---- delta weights and accumulation: one CTA per (slot, b1) ----
// GB300's FP64 pipe is 1/64 of FP32, and only a fraction of the n^2 mode pairs (b2, b3) has a
// Gaussian inside its 8-sigma window. In blocks of kLnBB rows b2: (A) every pair is screened
// in FP32 (window with a margin far above FP32 rounding, degeneracy skips pre-checked in
// FP32), the survivors are compacted into a queue with a block scan; (B) full warps evaluate
// the queue with the reference's FP64 window test, weights and occupations into a dense F;
// (C) R2[b2] = sum_b3 F and R3[b3] += sum_b2 F.
constexpr int kLnBB = 32;

struct LnDeltaArgs {
    MeshDev mesh;
    PhononDev ph;
    RowsDev rows;
    const TripletRec *trip;
    const int2 *red;
    const uint32_t *cand_mask;
    const float2 *psi;
    int n;
    double *gamma, *od;
    // adjoint: cotangents of the rows; W = G conj(Psi) is written over psi
    const double *lam;
    float2 *w;
};

__host__ __device__ inline size_t ln_delta_smem(int n) {
    return sizeof(double) * ((size_t)14 * n + (size_t)kLnBB * n) + sizeof(uint32_t) * (size_t)kLnBB * n +
           sizeof(int) * 33 + 16;
}

// ADJ: the adjoint's weights. F holds G_b = lam(row) * nred * dF_b/d|Psi_b|^2 of the
// survivors (F without |Psi|^2), and W_b = G_b conj(Psi_b) replaces Psi_b for every (b2, b3)
// of the row mode b1, zero where nothing survives or the row is not sampled.
template <bool ADJ>
__global__ void __launch_bounds__(256) k_ln_delta(LnDeltaArgs a) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int n = a.n;
    const int s = blockIdx.y, b1 = blockIdx.x;
    const int tid = threadIdx.x, bd = blockDim.x;
    const TripletRec rec = a.trip[s];
    const MeshDev &m = a.mesh;
    const PhononDev &P = a.ph;
    const uint32_t *mask = a.cand_mask + (size_t)rec.cand * 4;
    const int row = a.rows.rowidx[(size_t)rec.q1 * n + b1];
    if (!((mask[b1 >> 5] >> (b1 & 31)) & 1u) || row < 0) {
        if (ADJ) {
            float2 *wr = a.w + ((int64_t)s * n + b1) * n * n;
            for (int e = tid; e < n * n; e += bd) wr[e] = make_float2(0.f, 0.f);
        }
        return;
    }
    const int f1 = m.irr_full[rec.q1], q2 = rec.q2, q3 = rec.q3;
    const int i2 = m.full_irr[q2], i3 = m.full_irr[q3];
    double *om2 = (double *)sm, *om3 = om2 + n, *be2 = om3 + n, *be3 = be2 + n, *s2 = be3 + n, *s3 = s2 + n;
    double *v2 = s3 + n, *v3 = v2 + 3 * n, *R2 = v3 + 3 * n, *R3 = R2 + n, *F = R3 + n;
    uint32_t *Q = (uint32_t *)(F + (size_t)kLnBB * n);
    int *wsum = (int *)(Q + (size_t)kLnBB * n);
    for (int b = tid; b < n; b += bd) {
        om2[b] = P.omega[(size_t)q2 * n + b];
        om3[b] = P.omega[(size_t)q3 * n + b];
        be2[b] = P.be[(size_t)i2 * n + b];
        be3[b] = P.be[(size_t)i3 * n + b];
        s2[b] = P.sigsq[(size_t)i2 * n + b];
        s3[b] = P.sigsq[(size_t)i3 * n + b];
        for (int d = 0; d < 3; ++d) {
            v2[b * 3 + d] = P.vel[((size_t)q2 * n + b) * 3 + d];
            v3[b * 3 + d] = P.vel[((size_t)q3 * n + b) * 3 + d];
        }
        R3[b] = 0.0;
    }
    __syncthreads();
    const double o1 = P.omega[(size_t)f1 * n + b1];
    const double s1 = P.sigsq[(size_t)rec.q1 * n + b1];
    double v1[3];
    for (int d = 0; d < 3; ++d) v1[d] = P.vel[((size_t)f1 * n + b1) * 3 + d];
    const double w = a.rows.weight3[row];
    const double perm = q2 == q3 ? 1.0 : 2.0;
    const int it = P.integrationtype;
    const float fo1 = (float)o1, fs1 = (float)s1;
    const float2 *psi = a.psi + ((int64_t)s * n + b1) * n * n;
    // 4-bit live mask of the Gaussians of pair (b2, b3), 0 when a skip rule applies
    // (scattering_threephonon.f90:90-101) or no Gaussian can reach its window
    auto screen = [&](int b2, int b3) -> uint32_t {
        const double o2 = om2[b2], o3 = om3[b3];
        const float f2 = (float)o2, f3 = (float)o3;
        // |x - y| < 1e-9 in FP64 needs |fx - fy| below 1e-8 in FP32 at these magnitudes
        if (o2 < kFreqTolD || o3 < kFreqTolD) return 0u;
        if (fabsf(fo1 - f2) < 1e-8f && fabs(o1 - o2) < kFreqTolD) return 0u;
        if (fabsf(fo1 - f3) < 1e-8f && fabs(o1 - o3) < kFreqTolD) return 0u;
        if (fabsf(f2 - f3) < 1e-8f && fabs(o2 - o3) < kFreqTolD) return 0u;
        if (it == 6) return 15u;  // the velocity-difference width can cancel in FP32: not screened
        const float sg = it == 1 ? (float)P.sigma_fixed : sqrtf(fs1 + (float)s2[b2] + (float)s3[b3]);
        const float win = 8.0f * sg * 1.001f + 1e-6f * (fo1 + f2 + f3);
        return (fabsf(fo1 + f2 - f3) <= win ? 1u : 0u) | (fabsf(fo1 - f2 + f3) <= win ? 2u : 0u) |
               (fabsf(fo1 - f2 - f3) <= win ? 4u : 0u) | (fo1 + f2 + f3 <= win ? 8u : 0u);
    };
    for (int bb = 0; bb < n; bb += kLnBB) {
        const int nbb = min(kLnBB, n - bb), cnt = nbb * n;
        // (A) contiguous chunk per thread (at most 16 entries: kLnBB * 128 / 256)
        const int per = (cnt + bd - 1) / bd;
        const int e0 = min(cnt, tid * per), e1 = min(cnt, e0 + per);
        uint64_t lives = 0;
        int ns = 0;
        for (int e = e0; e < e1; ++e) {
            const uint32_t l = screen(bb + e / n, e % n);
            lives |= (uint64_t)l << (4 * (e - e0));
            ns += l != 0u;
        }
        for (int e = tid; e < cnt; e += bd) F[e] = 0.0;
        int total = 0;
        int k = block_exclusive_scan(ns, wsum, total);  // contains __syncthreads
        for (int e = e0; e < e1; ++e) {
            const uint32_t l = (uint32_t)(lives >> (4 * (e - e0))) & 15u;
            if (l) Q[k++] = (uint32_t)e | (l << 16);
        }
        __syncthreads();
        // (B) FP64 delta weights and occupations of the survivors, full warps
        for (int i = tid; i < total; i += bd) {
            const uint32_t qv = Q[i];
            const int e = (int)(qv & 0xffffu);
            const uint32_t live = qv >> 16;
            const int b2 = bb + e / n, b3 = e % n;
            const double o2 = om2[b2], o3 = om3[b3];
            double sigma, invsig;
            if (it == 1) {
                sigma = P.sigma_fixed;
                invsig = 1.0 / sigma;
            } else if (it == 2) {
                const double sq = s1 + s2[b2] + s3[b3];
                invsig = rsqrt(sq);
                sigma = sq * invsig;
            } else {
                sigma = adaptive_pair(v1, v2 + 3 * b2, P.reclat_g) / 3.0;
                sigma += adaptive_pair(v1, v3 + 3 * b3, P.reclat_g) / 3.0;
                sigma += adaptive_pair(v2 + 3 * b2, v3 + 3 * b3, P.reclat_g) / 3.0;
                sigma += P.thresh_sigma;
                invsig = 1.0 / sigma;
            }
            const double win8 = 8.0 * sigma, h = 0.5 * invsig * invsig, cg = kSqrt2PiInv * invsig;
            const double *tab = P.exp2tab;
            double d0, d1;
            dirac3(live, o1, o2, o3, win8, h, cg, tab, d0, d1);
            if (!nonzero(d0) && !nonzero(d1)) continue;
            const double n2 = be2[b2], n3 = be3[b3];
            if (ADJ) {
                F[e] = a.lam[row] * (double)rec.red_cnt * perm * kLnPrefactor * w *
                       ((n2 - n3) * d0 + (n2 + n3 + 1.0) * d1);
                continue;
            }
            const float2 ps = psi[b2 * n + b3];
            const double cr = ps.x, ci = ps.y;
            const double psisq = kLnPrefactor * (cr * cr + ci * ci) * w;
            F[e] = perm * psisq * (n2 - n3) * d0 + perm * psisq * (n2 + n3 + 1.0) * d1;
        }
        __syncthreads();
        if (ADJ) {
            float2 *wr = a.w + ((int64_t)s * n + b1) * n * n + (int64_t)bb * n;
            for (int e = tid; e < cnt; e += bd) {
                const float g = (float)F[e];
                const float2 ps = wr[e];
                wr[e] = make_float2(g * ps.x, -g * ps.y);
            }
            __syncthreads();
            continue;
        }
        // (C) row sums of the block and running column sums
        for (int r = tid; r < nbb; r += bd) {
            double sum = 0.0;
            for (int b3 = 0; b3 < n; ++b3) {
                const double f = F[r * n + b3];
                if (nonzero(f)) sum += f;
            }
            R2[bb + r] = sum;
        }
        for (int b3 = tid; b3 < n; b3 += bd) {
            double sum = R3[b3];
            for (int r = 0; r < nbb; ++r) {
                const double f = F[r * n + b3];
                if (nonzero(f)) sum += f;
            }
            R3[b3] = sum;
        }
        __syncthreads();
    }
    if (ADJ) return;
    const int nred = rec.red_cnt;
    if (tid == 0) {
        double gsum = 0.0;
        for (int b2 = 0; b2 < n; ++b2) gsum += R2[b2];
        if (nonzero(gsum)) atomicAdd(a.gamma + row, (double)nred * gsum);
    }
    const double inv1 = 1.0 / o1;
    const int64_t ldx = (int64_t)m.n_full * n;
    for (int i = tid; i < 2 * n * nred; i += bd) {
        const int r = i / (2 * n), e = i % (2 * n);
        const int2 pr = a.red[rec.red_off + r];
        if (e < n) {
            const double v = R2[e];
            if (nonzero(v)) atomicAdd(a.od + row * ldx + (int64_t)pr.x * n + e, 2.0 * v * om2[e] * inv1);
        } else {
            const int b3 = e - n;
            const double v = R3[b3];
            if (nonzero(v)) atomicAdd(a.od + row * ldx + (int64_t)pr.y * n + b3, 2.0 * v * om3[b3] * inv1);
        }
    }
}

// ---- adjoint: W[b1][b2][b3] into the stage-1 operand planes X[(ri, b1)][b2 n + b3] ----
__global__ void k_ln_pack(int n, const float2 *w, int nb, int64_t plane, int mp, __nv_bfloat16 *xhi,
                          __nv_bfloat16 *xlo) {
    const int s = blockIdx.y;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n3 = (int64_t)n * n * n;
    if (s >= nb || e >= n3) return;
    const int nn = n * n;
    const int b1 = (int)(e / nn), bc = (int)(e % nn);
    const float2 v = w[(int64_t)s * n3 + e];
    __nv_bfloat16 *hi = xhi + (int64_t)s * plane, *lo = xlo + (int64_t)s * plane;
    store_split(hi, lo, (int64_t)b1 * mp + bc, v.x);
    store_split(hi, lo, (int64_t)(n + b1) * mp + bc, v.y);
}

// ---- adjoint: d L / d mwm_t(i,j,k) += 2 Re(phase_t Q[3a1+i][3a2+j][3a3+k]) over the batch ----
// One thread per (force-constant triplet t, ijk), summing the batch's slots in FP32 and adding
// the sum into a double-float accumulator (hi, lo): GB300's FP64 pipe would make one FP64
// add per entry and batch the most expensive part of the pass.
__global__ void k_ln_grad(int n, Fc3Dev fc, const float2 *ph, const float2 *q, int nb, float *ghi, float *glo) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)fc.n * 27) return;
    const int t = (int)(i / 27), ijk = (int)(i % 27);
    const int64_t n3 = (int64_t)n * n * n;
    const int64_t off = fc.abase[t] + (int64_t)(ijk % 3) * n * n + ((ijk / 3) % 3) * n + ijk / 9;
    float acc = 0.f;
    for (int s = 0; s < nb; ++s) {
        const float2 p = ph[(size_t)s * fc.n + t];
        const float2 v = q[(int64_t)s * n3 + off];
        acc = fmaf(p.x, v.x, fmaf(-p.y, v.y, acc));
    }
    acc *= 2.f;
    const float h = ghi[i];
    const float tsum = h + acc, bb = tsum - h;
    glo[i] += (h - (tsum - bb)) + (acc - bb);
    ghi[i] = tsum;
}

}  // namespace

int ln_kp(int n) { return ((2 * n + 15) / 16) * 16; }

size_t ln_gemm_smem(int kp) { return (size_t)kLnStages * 2 * ((size_t)128 * 16 * 2 + (size_t)16 * kp * 2); }

cudaError_t launch_ln_bmat(int n, int n_q, const float2 *egvs32, __nv_bfloat16 *bmat, bool transpose,
                           cudaStream_t s) {
    const int kp = ln_kp(n);
    const int64_t total = (int64_t)n_q * kp * kp;
    if (total <= 0) return cudaSuccess;
    k_build_bmat<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n, kp, n_q, egvs32, bmat, transpose ? 1 : 0);
    return cudaGetLastError();
}

namespace {
// The three tcgen05 stages from the operand in the xa planes to b.psi, with the real-split
// matrices bmat (forward: E; adjoint: E^T).
cudaError_t ln_contract(const LnBatch &b, const __nv_bfloat16 *bmat, cudaStream_t s) {
    const int n = b.n, kp = ln_kp(n), M = n * n;
    cudaError_t e;
    const size_t smem = ln_gemm_smem(kp);
    if ((e = cudaFuncSetAttribute(k_ln_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
        return e;
    LnGemmArgs g;
    g.plane = b.plane;
    g.mp = b.mp;
    g.bmat = bmat;
    g.trip = b.trip;
    g.irr_full = b.mesh.irr_full;
    g.n = n;
    g.kp = kp;
    g.psi = b.psi;
    g.status = b.status;
    dim3 grid((unsigned)((M + 127) / 128), (unsigned)b.nb);
    for (int stage = 1; stage <= 3; ++stage) {
        const bool from_a = stage != 2;
        g.stage = stage;
        g.xhi = from_a ? b.xa_hi : b.xb_hi;
        g.xlo = from_a ? b.xa_lo : b.xb_lo;
        g.ohi = from_a ? b.xb_hi : b.xa_hi;
        g.olo = from_a ? b.xb_lo : b.xa_lo;
        k_ln_gemm<<<grid, kLnThreads, smem, s>>>(g);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

LnDeltaArgs delta_args(const LnBatch &b) {
    LnDeltaArgs d;
    d.mesh = b.mesh;
    d.ph = b.ph;
    d.rows = b.rows;
    d.trip = b.trip;
    d.red = b.red;
    d.cand_mask = b.cand_mask;
    d.psi = b.psi;
    d.n = b.n;
    d.gamma = b.gamma;
    d.od = b.od;
    d.lam = b.lam;
    d.w = b.psi;
    return d;
}
}  // namespace

cudaError_t launch_ln_adjoint_batch(const LnBatch &b, cudaStream_t s) {
    const int n = b.n, kp = ln_kp(n);
    if (b.nb <= 0) return cudaSuccess;
    if (kp > 256) return cudaErrorNotSupported;
    cudaError_t e;
    const int64_t n3 = (int64_t)n * n * n;
    {
        dim3 grid((unsigned)((b.fc.n + 255) / 256), (unsigned)b.nb);
        k_ln_phases<<<grid, 256, 0, s>>>(b.fc, b.mesh, b.trip, b.nb, b.phase);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        dim3 g2((unsigned)((n3 + 255) / 256), (unsigned)b.nb);
        k_ln_pretransform<<<g2, 256, 0, s>>>(n, n / 3, b.fc, b.phase, b.nb, b.plane, b.mp, b.xa_hi, b.xa_lo);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = ln_contract(b, b.bmat, s)) != cudaSuccess) return e;  // Psi
    const LnDeltaArgs d = delta_args(b);
    const size_t dsm = ln_delta_smem(n);
    if ((e = cudaFuncSetAttribute(k_ln_delta<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm)) !=
        cudaSuccess)
        return e;
    k_ln_delta<true><<<dim3((unsigned)n, (unsigned)b.nb), 256, dsm, s>>>(d);  // W over Psi
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    {
        dim3 grid((unsigned)((n3 + 255) / 256), (unsigned)b.nb);
        k_ln_pack<<<grid, 256, 0, s>>>(n, b.psi, b.nb, b.plane, b.mp, b.xa_hi, b.xa_lo);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = ln_contract(b, b.bmat_t, s)) != cudaSuccess) return e;  // Q over W
    const int64_t ne = (int64_t)b.fc.n * 27;
    k_ln_grad<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(n, b.fc, b.phase, b.psi, b.nb, b.grad_hi, b.grad_lo);
    return cudaGetLastError();
}

cudaError_t launch_ln_batch(const LnBatch &b, cudaStream_t s) {
    const int n = b.n, kp = ln_kp(n);
    if (b.nb <= 0) return cudaSuccess;
    if (kp > 256) return cudaErrorNotSupported;
    cudaError_t e;
    {
        dim3 grid((unsigned)((b.fc.n + 255) / 256), (unsigned)b.nb);
        k_ln_phases<<<grid, 256, 0, s>>>(b.fc, b.mesh, b.trip, b.nb, b.phase);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    {
        const int64_t n3 = (int64_t)n * n * n;
        dim3 grid((unsigned)((n3 + 255) / 256), (unsigned)b.nb);
        k_ln_pretransform<<<grid, 256, 0, s>>>(n, n / 3, b.fc, b.phase, b.nb, b.plane, b.mp, b.xa_hi, b.xa_lo);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = ln_contract(b, b.bmat, s)) != cudaSuccess) return e;
    const LnDeltaArgs d = delta_args(b);
    const size_t dsm = ln_delta_smem(n);
    if ((e = cudaFuncSetAttribute(k_ln_delta<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm)) !=
        cudaSuccess)
        return e;
    k_ln_delta<false><<<dim3((unsigned)n, (unsigned)b.nb), 256, dsm, s>>>(d);
    return cudaGetLastError();
}

}  // namespace tdg
