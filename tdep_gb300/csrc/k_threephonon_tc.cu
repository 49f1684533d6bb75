// Fused three-phonon kernel with the Psi contraction on the tcgen05 tensor cores, for
// small cells (9, 12 or 15 modes; mixed precision). One CTA of 256 threads takes one
// accepted irreducible q-triplet at a time (persistent grid-stride loop, several CTAs per
// SM so that one CTA's SIMT stages overlap another's tensor-core stages).
//
// Reference (src/thermal_conductivity/scattering_threephonon.f90):
//   pretransform_phi3 (:275-317)      P(a,b,c) = sum_t mwm_t(i,j,k) exp(-2 pi i (q2.lv2 + q3.lv3))
//   zgeru x2 + dot_product (:93-113)   Psi(b1,b2,b3) = sum_abc E1(a,b1) E2(b,b2) E3(c,b3) P(a,b,c)
//   get_dirac (:219-271) and accumulation (:115-135), shared with the SIMT kernel (k3_parts.cuh);
//   the delta weights of the survivors here in FP32 (k3_survivors_f32), the sums in FP64.
//
// Contraction. With the modes padded to 16, each of the three stages contracts one
// component index of a 16^3 complex tensor with one eigenvector matrix E (16 x 16 complex,
// e/sqrt(omega), not conjugated), as a real GEMM with M = 256 rows (the two uncontracted
// indices, two M = 128 tiles), K = 32 and N = 32:
//   [Yr | Yi] = [Xr | Xi] [[Er, Ei], [-Ei, Er]]
//   stage 1: rows (c, b), k = a   -> T1 columns b1
//   stage 2: rows (c, b1), k = b  -> T2 columns b2
//   stage 3: rows (b1, b2), k = c -> Psi columns b3
// Operands are BF16 hi/lo splits of FP32 values (x = hi + lo, about 16 significant bits);
// a product is hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory (2 accumulators
// of 32 columns). The B operands (the real-split E of every mesh point, 4 KB each) are
// built once per context and brought into shared memory by bulk copies on mbarriers (the
// forward pass: E1 and E2 at the start of a q-triplet, E3 once the pretransform is done);
// each stage's accumulator rows are read by the thread of that row (tcgen05.ld), split and
// stored as the next stage's A operand, in 8 x 16-byte core matrices without swizzle, all
// MN-major (a core-matrix row is 8 consecutive M indices at one k). The row orders of the
// table make every such row one thread's 8 consecutive accumulator columns, so a
// transition is 16-byte stores. Into the stage-2 operand the 8 lanes of a store phase
// hold 8 different k (= b) and hit 8 different bank groups; into the stage-3 operand they
// share k (= c) and conflict. The padding (modes and components 15, or 9-15 / 12-15) is
// zero in P and E and stays exactly zero through the stages.
//
// Pretransform. Output element (atom triple, ijk) sums its block's force-constant triplets
// times their phase factors; the blocks hold 0 to several dozen triplets. A static plan,
// built once per force-constant set, deals the elements out to the 256 threads (largest
// first, each to the least-loaded thread) and lays their values out slot-major: slot s of
// thread t is 4 consecutive triplets of one element (16 bytes at [s][t], zero-padded) and
// a word with the index of their first phase factor and, on an element's last slot, its
// operand offset. Every load of a thread is independent of the others (8 in flight per
// thread), the warp's loads are coalesced, and the threads' slot counts differ by at most
// one element. The sums run in the triplets' order, as before the plan. The phase factors
// are exact roots of unity from the mesh table, computed once per q-triplet into shared
// memory.
//
// Every wait is bounded: an MMA or copy that does not complete within about 1 s makes all
// threads leave together (the decision is a barrier reduction), after waiting for their
// copies and MMAs in flight (bounded as well); the tensor memory is freed and the status
// word reports the timeout.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <queue>
#include <utility>
#include <vector>

#include "dev_common.cuh"
#include "k3_parts.cuh"
#include "tc_common.cuh"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr int kTcThreads = 256;
constexpr int kEImgBytes = 4096;           // one real-split E: hi plane + lo plane, 32 x 32 BF16 each
constexpr int kAPlane = 16384;             // one A plane: 256 rows x 32 k x 2 bytes
constexpr long long kTcWait = 2000000000LL;  // about 1 s at 2 GHz

// Shared-memory layout (bytes) of the tensor-core kernel for mode count n and nt
// force-constant triplets. Region X holds the A operand (hi, lo), the E images and the
// phase factors while Psi is formed; afterwards it is reused.
//  forward: E1 and E2 at the start of each q-triplet, E3 into the phase factors' place once
//           the pretransform is done; after stage 3 the survivor queue, F in FP32 and
//           |Psi|^2 (then the row and column sums) all in X: 55.5 KB at 15 modes and 1115
//           force-constant triplets, 4 CTAs per SM;
//  adjoint: the three E images at once (the back-contraction reloads them as E^T), the
//           phase factors kept to the end for 2 Re(phase Q); queue and FP64 F in X, |Psi|^2
//           after it (74.4 KB, 3 CTAs per SM).
struct TcLayout {
    size_t A, E, E3, ph, Q, F, psq, om, f32, v, masks, rowid, red, wsum, mbar, tslot, total;
};
__host__ __device__ inline size_t tc_al(size_t x, size_t a = 16) { return (x + a - 1) / a * a; }
__host__ __device__ inline TcLayout tc_layout(int n, int nt, bool adj) {
    TcLayout L;
    const size_t n2 = (size_t)n * n, n3 = n2 * n;
    const size_t phb = tc_al(sizeof(float2) * ((size_t)nt + 4));
    L.A = 0;
    L.E = 2 * kAPlane;
    L.Q = 0;
    L.F = tc_al(sizeof(uint32_t) * n3);
    size_t o;
    if (!adj) {
        L.ph = L.E + 2 * kEImgBytes;
        L.E3 = L.ph;
        const size_t x_end = L.ph + (phb > (size_t)kEImgBytes ? phb : (size_t)kEImgBytes);
        L.psq = L.F + tc_al(sizeof(float) * n3);
        // |Psi|^2, then the row and column sums and their Xi row terms (4 n^2 doubles)
        const size_t y_end = L.psq + tc_al(sizeof(float) * n3 > 4 * n2 * sizeof(double) ? sizeof(float) * n3
                                                                                         : 4 * n2 * sizeof(double));
        o = tc_al(x_end > y_end ? x_end : y_end, 128);
    } else {
        L.ph = L.E + 3 * kEImgBytes;
        L.E3 = L.E + 2 * kEImgBytes;
        const size_t x_end = L.ph + phb;
        const size_t y_end = L.F + sizeof(double) * n3;
        o = tc_al(x_end > y_end ? x_end : y_end, 128);
        L.psq = o; o += tc_al(sizeof(float) * n3);  // |Psi|^2, then the row and column sums (2 n^2 doubles)
    }
    L.om = o; o += 9 * tc_al(sizeof(double) * n) + tc_al(sizeof(double) * n);  // om1..3 inv1 be2 be3 s1..3, wrow
    L.v = o; o += 3 * tc_al(sizeof(double) * 3 * n);
    L.f32 = o; o += tc_al(sizeof(float) * 12 * n);
    L.masks = o; o += tc_al(sizeof(uint32_t) * (3 * n + 2 + 2 * n2));
    L.rowid = o; o += tc_al(sizeof(int) * n);
    L.red = o; o += tc_al(sizeof(int2) * kMaxRed);
    L.wsum = o; o += tc_al(sizeof(int) * 33);
    L.mbar = o; o += 32;  // [0] E1, E2 (and E3 in the adjoint) copies, [1] MMA completion, [2] E3 copy
    L.tslot = o; o += 16;
    L.total = o;
    return L;
}

// Byte offset of element (m, k) in a 256 x 32 A plane: core matrices of 8 rows x 16 bytes,
// M groups 128 bytes apart, K groups 4096 bytes apart. MN-major: a core's 8 rows are 8 k,
// each 8 consecutive m; K-major: its rows are 8 m, each 8 consecutive k.
__host__ __device__ __forceinline__ uint32_t a_off_mn(int m, int k) {
    return (uint32_t)(((m >> 3) << 7) + ((k >> 3) << 12) + ((k & 7) << 4) + ((m & 7) << 1));
}
__device__ __forceinline__ uint32_t a_off_k(int m, int k) {
    return (uint32_t)(((m >> 3) << 7) + ((k >> 3) << 12) + ((m & 7) << 4) + ((k & 7) << 1));
}


__device__ __forceinline__ void st_split(unsigned char *plane_hi, uint32_t off, float x) {
    unsigned short h, l;
    tc::split_bf16(x, h, l);
    *(unsigned short *)(plane_hi + off) = h;
    *(unsigned short *)(plane_hi + kAPlane + off) = l;
}

// One core-matrix row of both planes: the hi and lo parts of x[0..7] as 16 bytes each at
// off (16-byte aligned) and kAPlane + off.
__device__ __forceinline__ void st_split8(unsigned char *plane_hi, uint32_t off, const float *x) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        unsigned short h0, l0, h1, l1;
        tc::split_bf16(x[2 * i], h0, l0);
        tc::split_bf16(x[2 * i + 1], h1, l1);
        h[i] = (uint32_t)h0 | ((uint32_t)h1 << 16);
        l[i] = (uint32_t)l0 | ((uint32_t)l1 << 16);
    }
    *(uint4 *)(plane_hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *(uint4 *)(plane_hi + kAPlane + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

// 32 lanes x 32 consecutive columns: thread i of the warp gets lane (base lane + i).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Index into the mesh's table of exp(-2 pi i k / L) of the phase factor
// exp(-2 pi i (q2.lv2 + q3.lv3)) of force-constant triplet t, an exact root of unity (see
// the SIMT kernel): u2, u3 hold g_d L/N_d of q2 and q3.
__device__ __forceinline__ int tc_phase_index(const Fc3Dev &fc, const MeshDev &m, const int *u2, const int *u3,
                                              int t) {
    const int32_t *lv = fc.lv + (size_t)t * 6;
    int S = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) S += u2[d] * __ldg(lv + d) + u3[d] * __ldg(lv + 3 + d);
    int K = S % m.L;
    if (K < 0) K += m.L;
    return K;
}


// One stage: 2 tiles x 2 K chunks x 3 split products of 128 x 32 x 16, issued by one thread.
__device__ __forceinline__ void issue_stage(uint32_t tbase, uint32_t a_base, uint32_t e_base, bool a_mn) {
    const uint32_t idesc = tc::idesc_bf16_f32(128, 32, a_mn, true);
#pragma unroll
    for (int t = 0; t < 2; ++t) {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                const uint32_t pa = p == 2 ? kAPlane : 0u, pb = p == 1 ? 2048u : 0u;
                const uint64_t ad = tc::smem_desc(a_base + pa + 2048u * t + 8192u * j, 4096u, 128u);
                const uint64_t bd = tc::smem_desc(e_base + pb + 1024u * j, 512u, 128u);
                tc::mma_bf16(tbase + 32u * t, ad, bd, idesc, (j | p) ? 1u : 0u);
            }
        }
    }
}

// ADJ: the adjoint of the linewidths (and, with a.xi_bar, of the Xi row terms) with respect
// to the force constants; see the comment at the adjoint tail below.
template <int N, bool ADJ>
__global__ void __launch_bounds__(kTcThreads, ADJ ? 3 : 4) k_threephonon_tc(ThreePhArgs a) {
    constexpr int N2 = N * N, N3 = N2 * N;
    extern __shared__ __align__(1024) unsigned char smem[];
    const Fc3Dev &fc = a.fc;
    const MeshDev &m = a.mesh;
    const PhononDev &P = a.ph;
    const TcLayout L = tc_layout(N, fc.n, ADJ);
    unsigned char *Aop = smem + L.A;
    unsigned char *Eimg = smem + L.E;
    float2 *ph = (float2 *)(smem + L.ph);
    float *psq = (float *)(smem + L.psq);
    uint64_t *mb = (uint64_t *)(smem + L.mbar);  // [0] E-image copies, [1] MMA completion, [2] E3 (forward)
    uint32_t *tslot = (uint32_t *)(smem + L.tslot);
    K3Smem S;
    {
        double *d = (double *)(smem + L.om);
        const size_t dn = tc_al(sizeof(double) * N) / sizeof(double);
        S.om1 = d; S.om2 = d + dn; S.om3 = d + 2 * dn; S.inv1 = d + 3 * dn; S.be2 = d + 4 * dn; S.be3 = d + 5 * dn;
        S.s1 = d + 6 * dn; S.s2 = d + 7 * dn; S.s3 = d + 8 * dn; S.wrow = d + 9 * dn;
        double *v = (double *)(smem + L.v);
        const size_t dv = tc_al(sizeof(double) * 3 * N) / sizeof(double);
        S.v1 = v; S.v2 = v + dv; S.v3 = v + 2 * dv;
        float *f = (float *)(smem + L.f32);
        S.fo1 = f; S.fo2 = f + N; S.fo3 = f + 2 * N; S.fs1 = f + 3 * N; S.fs2 = f + 4 * N; S.fs3 = f + 5 * N;
        S.fl1 = f + 6 * N; S.fl2 = f + 7 * N; S.fl3 = f + 8 * N; S.fb2 = f + 9 * N; S.fb3 = f + 10 * N;
        S.fw1 = f + 11 * N;
        uint32_t *mk = (uint32_t *)(smem + L.masks);
        S.m12 = mk; S.m13 = mk + N; S.m23 = mk + 2 * N; S.zmask = mk + 3 * N;
        S.rowbits = S.zmask + 2; S.colbits = S.rowbits + N2;
        S.R2 = (double *)(smem + L.psq);  // |Psi|^2 is dead when the sums start
        S.R3 = S.R2 + N2;
        S.R2s = S.R3 + N2;
        S.R3s = S.R2s + N2;
        S.F = ADJ ? (double *)(smem + L.F) : nullptr;
        S.Ff = ADJ ? nullptr : (float *)(smem + L.F);
        S.Q = (uint32_t *)(smem + L.Q);
        S.rowid = (int *)(smem + L.rowid);
        S.red = (int2 *)(smem + L.red);
        S.wsum = (int *)(smem + L.wsum);
    }
    const int tid = threadIdx.x, warp = tid >> 5;
    const int it = P.integrationtype;
    const float sigfix32 = (float)P.sigma_fixed;

    if (warp == 0) tc::tmem_alloc(tslot, 64);
    if (tid == 0) {
        tc::mbar_init(&mb[0], 1);
        tc::mbar_init(&mb[1], 1);
        tc::mbar_init(&mb[2], 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;
    // this thread's accumulator row: tile t = warp / 4, lane 32 (warp % 4) + lane
    const int tile = warp >> 2;
    const int row = tid & 127;
    const int mrow = 128 * tile + row;  // row of the 256-row operand (two uncontracted indices, 16 x 16)
    const uint32_t taddr = tbase + ((uint32_t)(32 * (warp & 3)) << 16) + 32u * (uint32_t)tile;
    const uint32_t a_u = tc::smem_u32(Aop), e_u = tc::smem_u32(Eimg), e3_u = tc::smem_u32(smem + L.E3);
    uint32_t e_ph = 0, m_ph = 0, e3_ph = 0;
    bool e3_pending = false;  // thread 0: an E3 copy was issued and not yet waited for
    bool ok = true;

    // the next q-triplet's record is loaded one iteration ahead
    TripletRec rec_next;
    if ((int)blockIdx.x < a.n_trip) rec_next = a.trip[blockIdx.x];
    for (int t = blockIdx.x; t < a.n_trip && ok; t += gridDim.x) {
        const TripletRec rec = rec_next;
        if (t + (int)gridDim.x < a.n_trip) rec_next = a.trip[t + gridDim.x];
        const int f1 = m.irr_full[rec.q1];
        const int q2 = rec.q2, q3 = rec.q3;
        const int i2 = m.full_irr[q2], i3 = m.full_irr[q3];
        const int nred = rec.red_cnt;
        const double perm = (q2 == q3) ? 1.0 : 2.0;
        // E images of q1 and q2 (the adjoint: and q3) into shared memory (the region was last
        // read by the previous q-triplet's MMAs and reused by its queue, F and |Psi|^2, all
        // finished before the last barrier); the forward pass brings E3 once the
        // pretransform has released the phase factors' place
        if (tid == 0) {
            tc::fence_async_smem();  // the generic accesses of the region (ordered by the last barrier) come first
            tc::mbar_arrive_expect_tx(&mb[0], (ADJ ? 3u : 2u) * kEImgBytes);
            tc::bulk_g2s(e_u, a.tc_eimg + (size_t)f1 * kEImgBytes, kEImgBytes, &mb[0]);
            tc::bulk_g2s(e_u + kEImgBytes, a.tc_eimg + (size_t)q2 * kEImgBytes, kEImgBytes, &mb[0]);
            if constexpr (ADJ)
                tc::bulk_g2s(e3_u, a.tc_eimg + (size_t)q3 * kEImgBytes, kEImgBytes, &mb[0]);
        }
        k3_load_modes<N>(S, a, rec, f1, q2, q3, i2, i3);
        // A operand zeroed (padding must be exact zeros), phase factors of all triplets
        for (int i = tid; i < 2 * kAPlane / 16; i += kTcThreads) ((uint4 *)Aop)[i] = make_uint4(0u, 0u, 0u, 0u);
        {
            int u2[3], u3[3];
            const int n12 = m.grid[1] * m.grid[2];
            u2[0] = q2 / n12; u2[1] = (q2 / m.grid[2]) % m.grid[1]; u2[2] = q2 % m.grid[2];
            u3[0] = q3 / n12; u3[1] = (q3 / m.grid[2]) % m.grid[1]; u3[2] = q3 % m.grid[2];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                u2[d] *= m.lmul[d];
                u3[d] *= m.lmul[d];
            }
            // four triplets per thread in flight: their lattice vectors, then their table entries
            for (int i0 = tid; i0 < fc.n + 4; i0 += 4 * kTcThreads) {
                int kk[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + u * kTcThreads;
                    kk[u] = i < fc.n ? tc_phase_index(fc, m, u2, u3, i) : -1;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + u * kTcThreads;
                    if (i < fc.n + 4) ph[i] = kk[u] >= 0 ? __ldg(fc.twiddle32 + kk[u]) : make_float2(0.f, 0.f);
                }
            }
        }
        __syncthreads();
        k3_skip_masks<N>(S);
        // ---- pretransform into the stage-1 operand: rows (c, b), k = a (re) and 16 + a (im) ----
        // (the plan's slots of this thread: 8 loads of values and 8 of words in flight)
        {
            const float4 *pm = a.plan_pm + tid;
            const uint32_t *pw = a.plan_word + tid;
            float ar = 0.f, ai = 0.f;
#pragma unroll 1
            for (int s0 = 0; s0 < a.plan_slots; s0 += 8) {
                float4 mv[8];
                uint32_t wd[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    mv[u] = __ldg(pm + (size_t)(s0 + u) * kTcThreads);
                    wd[u] = __ldg(pw + (size_t)(s0 + u) * kTcThreads);
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const float2 *pp = ph + (wd[u] & 0xffffu);
                    const float2 p0 = pp[0], p1 = pp[1], p2 = pp[2], p3 = pp[3];
                    ar = fmaf(mv[u].x, p0.x, ar); ai = fmaf(mv[u].x, p0.y, ai);
                    ar = fmaf(mv[u].y, p1.x, ar); ai = fmaf(mv[u].y, p1.y, ai);
                    ar = fmaf(mv[u].z, p2.x, ar); ai = fmaf(mv[u].z, p2.y, ai);
                    ar = fmaf(mv[u].w, p3.x, ar); ai = fmaf(mv[u].w, p3.y, ai);
                    const uint32_t oc = wd[u] >> 16;  // on an element's last slot: operand offset / 2 + 1
                    if (oc) {
                        const uint32_t off = 2u * (oc - 1u);
                        st_split(Aop, off, ar);
                        st_split(Aop, off + 8192u, ai);
                        ar = 0.f;
                        ai = 0.f;
                    }
                }
            }
        }
        // ---- three contraction stages ----
#pragma unroll 1
        for (int stage = 0; stage < 3; ++stage) {
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                bool go = true;
                if (stage == 0) {
                    go = tc::mbar_wait(&mb[0], e_ph, kTcWait);
                    if (go) e_ph ^= 1u;  // else the abort path waits on the same phase again
                    if (!ADJ && go) {
                        // the pretransform is done (the barrier above): E3 into the phase
                        // factors' place, for stage 3
                        tc::mbar_arrive_expect_tx(&mb[2], kEImgBytes);
                        tc::bulk_g2s(e3_u, a.tc_eimg + (size_t)q3 * kEImgBytes, kEImgBytes, &mb[2]);
                        e3_pending = true;
                    }
                }
                if (!ADJ && stage == 2 && go) {
                    go = tc::mbar_wait(&mb[2], e3_ph, kTcWait);
                    if (go) {
                        e3_ph ^= 1u;
                        e3_pending = false;
                    }
                }
                if (go) {
                    issue_stage(tbase, a_u, stage == 2 ? e3_u : e_u + (uint32_t)stage * kEImgBytes, true);
                    tc::mma_commit(&mb[1]);
                }
            }
            const bool done = tc::mbar_wait(&mb[1], m_ph, kTcWait);
            ok = __syncthreads_and(done) != 0;
            if (!ok) break;  // m_ph unchanged: the abort path waits on that phase again
            m_ph ^= 1u;
            tc::fence_after_sync();
            float v[32];
            tmem_ld32(taddr, v);
            if (stage < 2) {
                // stage 0: row (c, b) of T1 over b1 -> stage-2 operand rows (c, b1), k = b;
                // stage 1: row (c, b1) of T2 over b2 -> stage-3 operand rows (b1, b2), k = c.
                // Columns 8g..8g+7 of the row are one core-matrix row: M = 16 hi + 8g, k = lo
                // (and 16 + lo for the imaginary part, 8192 bytes on).
                const int hi = stage == 0 ? (mrow >> 4) : (mrow & 15), lo = stage == 0 ? (mrow & 15) : (mrow >> 4);
#pragma unroll
                for (int g = 0; g < 2; ++g) {
                    const uint32_t off = a_off_mn(16 * hi + 8 * g, lo);
                    st_split8(Aop, off, v + 8 * g);
                    st_split8(Aop, off + 8192u, v + 16 + 8 * g);
                }
            } else {
                // row (b1, b2) of Psi over b3 -> |Psi|^2 of the valid modes
                const int b1 = mrow >> 4, b2 = mrow & 15;
                if (b1 < N && b2 < N) {
#pragma unroll
                    for (int b3 = 0; b3 < N; ++b3) psq[(b1 * N + b2) * N + b3] = v[b3] * v[b3] + v[16 + b3] * v[16 + b3];
                }
            }
        }
        if (!ok) break;
        tc::fence_before_sync();
        // ---- FP32 screen of the Gaussians, survivors queued, FP32 weights, FP64 sums ----
        uint32_t live_lo = 0u, live_hi = 0u, live_x = 0u;
        int nsurv = 0;
        const int b1 = mrow >> 4, b2 = mrow & 15;
        const bool mine = b1 < N && b2 < N;
        if (mine) nsurv = k3_screen<N>(S, it, sigfix32, b1, b2, live_lo, live_hi, live_x);
        int nq = 0;
        const int off = block_exclusive_scan(nsurv, S.wsum, nq);  // contains barriers: the operands are dead
        if (mine && nsurv) k3_enqueue<N>(S, b1 * N + b2, off, live_lo, live_hi, live_x);
        // the forward pass reads F only where the row and column bits are set (entries written
        // by this q-triplet's survivors); the adjoint reads all of it
        if constexpr (ADJ)
            for (int i = tid; i < N3; i += kTcThreads) S.F[i] = 0.0;
        __syncthreads();
        if constexpr (!ADJ) {
            k3_survivors_f32<N, true>(S, P, nq, (float)perm, [&](int idx) -> float { return psq[idx]; });
            k3_sums_scatter<N, true>(S, a, nred);
        } else {
            // ---- adjoint tail (the SIMT adjoint's algebra, k_threephonon.cu): F without |Psi|^2
            // gives G_b = cot_b dF_b/d|Psi_b|^2 with cot = lam(row) nred (+ the Xi row terms'
            // cotangents 2 om2/om1 xi_bar(q2', b2) + 2 om3/om1 xi_bar(q3', b3) over the
            // equivalent triplets); W = G conj(Psi); Q[abc] = sum_b W_b E1[a,b1] E2[b,b2] E3[c,b3]
            // by three GEMMs against the real-split E^T images (W E3^T over b3, then E2^T over
            // b2, then E1^T over b1); d L / d mwm_t(i,j,k) = 2 Re(phase_t Q[3a1+i][3a2+j][3a3+k]).
            k3_survivors_f32<N>(S, P, nq, (float)perm, [](int) -> float { return 1.0f; });
            __syncthreads();
            double *R2 = S.R2, *XB = S.R3;  // in the |Psi|^2 region, which the adjoint does not use
            if (a.xi_bar) {
                const int64_t ld = (int64_t)m.n_full * N;
                for (int e = tid; e < 2 * N2; e += kTcThreads) {
                    const int x = e % N2, eb1 = x / N, bb = x % N, r = S.rowid[eb1];
                    double sum = 0.0;
                    if (r >= 0) {
                        const double *wr = a.xi_bar + (int64_t)r * ld;
                        for (int k = 0; k < nred; ++k) {
                            const int2 pr = S.red[k];
                            sum += wr[(int64_t)(e < N2 ? pr.x : pr.y) * N + bb];
                        }
                    }
                    if (e < N2)
                        R2[x] = sum;
                    else
                        XB[x] = sum;
                }
                __syncthreads();
            }
            float gw[16];
#pragma unroll
            for (int b3 = 0; b3 < 16; ++b3) gw[b3] = 0.f;
            {
                const int r = mine ? S.rowid[b1] : -1;
                if (r >= 0) {
                    const double lr = a.lam[r] * (double)nred;
#pragma unroll
                    for (int b3 = 0; b3 < N; ++b3) {
                        double cot = lr;
                        if (a.xi_bar) cot += 2.0 * (S.om2[b2] * R2[b1 * N + b2] + S.om3[b3] * XB[b1 * N + b3]) * S.inv1[b1];
                        gw[b3] = (float)(cot * S.F[(b1 * N + b2) * N + b3]);
                    }
                }
            }
            // F, the queue and the sums are read: the image region takes E3^T, E2^T, E1^T and
            // the operand region W (K-major: a core-matrix row is 8 consecutive b3 of one row)
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc::fence_async_smem();
                tc::mbar_arrive_expect_tx(&mb[0], 3u * kEImgBytes);
                tc::bulk_g2s(e_u, a.tc_eimg_t + (size_t)q3 * kEImgBytes, kEImgBytes, &mb[0]);
                tc::bulk_g2s(e_u + kEImgBytes, a.tc_eimg_t + (size_t)q2 * kEImgBytes, kEImgBytes, &mb[0]);
                tc::bulk_g2s(e_u + 2 * kEImgBytes, a.tc_eimg_t + (size_t)f1 * kEImgBytes, kEImgBytes, &mb[0]);
            }
            tc::fence_after_sync();
            {
                float v[32], w[32];
                tmem_ld32(taddr, v);  // Psi row (b1, b2): stage 3's accumulator is still in tensor memory
#pragma unroll
                for (int b3 = 0; b3 < 16; ++b3) {
                    w[b3] = gw[b3] * v[b3];
                    w[16 + b3] = -gw[b3] * v[16 + b3];
                }
#pragma unroll
                for (int g = 0; g < 2; ++g) {
                    const uint32_t off = a_off_k(mrow, 8 * g);
                    st_split8(Aop, off, w + 8 * g);
                    st_split8(Aop, off + 8192u, w + 16 + 8 * g);
                }
            }
            // back stages: rows (b1, b2) over c, rows (b1, c) over b, rows (c, b) over a
#pragma unroll 1
            for (int stage = 0; stage < 3; ++stage) {
                tc::fence_async_smem();
                tc::fence_before_sync();
                __syncthreads();
                if (tid == 0) {
                    tc::fence_after_sync();
                    bool go = true;
                    if (stage == 0) {
                        go = tc::mbar_wait(&mb[0], e_ph, kTcWait);
                        if (go) e_ph ^= 1u;
                    }
                    if (go) {
                        issue_stage(tbase, a_u, e_u + (uint32_t)stage * kEImgBytes, stage > 0);
                        tc::mma_commit(&mb[1]);
                    }
                }
                const bool done = tc::mbar_wait(&mb[1], m_ph, kTcWait);
                ok = __syncthreads_and(done) != 0;
                if (!ok) break;
                m_ph ^= 1u;
                tc::fence_after_sync();
                float v[32];
                tmem_ld32(taddr, v);
                if (stage < 2) {
                    // stage 0: row (b1, b2) over c -> rows (b1, c), k = b2;
                    // stage 1: row (b1, c) over b -> rows (c, b), k = b1 (MN-major, as forward)
                    const int hi = stage == 0 ? (mrow >> 4) : (mrow & 15), lo = stage == 0 ? (mrow & 15) : (mrow >> 4);
#pragma unroll
                    for (int g = 0; g < 2; ++g) {
                        const uint32_t off = a_off_mn(16 * hi + 8 * g, lo);
                        st_split8(Aop, off, v + 8 * g);
                        st_split8(Aop, off + 8192u, v + 16 + 8 * g);
                    }
                } else {
                    // row (c, b) of Q over a into the (finished) operand region as [a][b][c]
                    const int c = mrow >> 4, b = mrow & 15;
                    float2 *Qs = (float2 *)Aop;
                    if (b < N && c < N) {
#pragma unroll
                        for (int aa = 0; aa < N; ++aa) Qs[(aa * N + b) * N + c] = make_float2(v[aa], v[16 + aa]);
                    }
                }
            }
            if (!ok) break;
            __syncthreads();
            {
                const float2 *Qs = (const float2 *)Aop;
                float *slice = reinterpret_cast<float *>(a.mwm_bar) + (size_t)blockIdx.x * fc.n * 27;
                constexpr int kGroups = kTcThreads / 27;
                const int grp = tid / 27, ijk = tid % 27;
                const int qoff = (ijk % 3) * N2 + ((ijk / 3) % 3) * N + ijk / 9;
                if (grp < kGroups) {
                    for (int tt = grp; tt < fc.n; tt += kGroups) {
                        const float2 q = Qs[fc.abase[tt] + qoff];
                        const float2 p = ph[tt];
                        slice[(size_t)tt * 27 + ijk] += 2.f * (p.x * q.x - p.y * q.y);
                    }
                }
            }
            __syncthreads();  // the next q-triplet overwrites the operand region and the phases
        }
    }
    if (!ok) {
        // a wait ran out: record it, let the copies and MMAs in flight finish (bounded), free
        // the tensor memory
        if (tid == 0) {
            atomicExch(a.status, (int32_t)kDevTimeout);
            tc::mbar_wait(&mb[0], e_ph, kTcWait);
            tc::mbar_wait(&mb[1], m_ph, kTcWait);
            if (e3_pending) tc::mbar_wait(&mb[2], e3_ph, kTcWait);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tbase, 64);
}

// Values of the pretransform plan from the current FP32 force constants: slot word src =
// first triplet | ijk << 16 | valid triplets << 21 (0 to 4; the rest of the 16 bytes zero).
__global__ void k_fill_plan(const uint32_t *src, int64_t n_slot, const float *mwm32, float4 *pm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_slot) return;
    const uint32_t w = src[i];
    const int f = (int)(w & 0xffffu), ijk = (int)((w >> 16) & 31u), nv = (int)(w >> 21);
    float v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = u < nv ? mwm32[(size_t)(f + u) * 27 + ijk] : 0.f;
    pm[i] = make_float4(v[0], v[1], v[2], v[3]);
}

// Real-split eigenvector images of every mesh point: B = [[Er, Ei], [-Ei, Er]] (32 x 32,
// row k = component a (re) / 16 + a, column = mode b (re) / 16 + b), E = egvs32 padded with
// zeros, split into BF16 hi and lo planes, MN-major core matrices (N groups 128 bytes apart,
// K groups 512 bytes apart). transpose: the image of E^T (row k = mode, column = component),
// the right-multiplier of the adjoint's back-contraction.
__global__ void k_tc_eimg(int32_t n_full, int32_t n, const float2 *egvs32, unsigned char *out, int transpose) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n_full * 1024) return;
    const int q = (int)(i >> 10), e = (int)(i & 1023);
    const int k = e >> 5, c = e & 31;
    const int aa = transpose ? (c & 15) : (k & 15), b = transpose ? (k & 15) : (c & 15);  // component, mode
    const bool kim = k >= 16, cim = c >= 16;
    float2 z = make_float2(0.f, 0.f);
    if (aa < n && b < n) z = egvs32[((size_t)q * n + b) * n + aa];
    const float x = (kim == cim) ? z.x : (kim ? -z.y : z.y);
    unsigned short h, l;
    tc::split_bf16(x, h, l);
    const uint32_t off = (uint32_t)(((c >> 3) << 7) + ((k >> 3) << 9) + ((k & 7) << 4) + ((c & 7) << 1));
    unsigned char *img = out + (size_t)q * kEImgBytes;
    *(unsigned short *)(img + off) = h;
    *(unsigned short *)(img + 2048 + off) = l;
}

template <int N, bool ADJ>
int tc_per_sm(int n_fc, int *api, int *count) {
    const size_t bytes = tc_layout(N, n_fc, ADJ).total;
    const int per_sm = resident_ctas((const void *)k_threephonon_tc<N, ADJ>, kTcThreads, bytes, api, count);
    // tensor memory: 64 columns per CTA, 512 per SM
    return per_sm > 8 ? 8 : per_sm;
}

template <int N, bool ADJ>
int tc_grid(int n_fc, int n_trip, int n_sm, int ctas_per_sm) {
    int per_sm = tc_per_sm<N, ADJ>(n_fc, nullptr, nullptr);
    if (per_sm < 1) return 0;
    if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
    const int grid = n_sm * per_sm;
    return grid > n_trip ? (n_trip > 0 ? n_trip : 1) : grid;
}

template <int N, bool ADJ>
cudaError_t tc_launch_grid(const ThreePhArgs &a, int grid, cudaStream_t s) {
    if (grid < 1) return cudaErrorInvalidConfiguration;
    k_threephonon_tc<N, ADJ><<<grid, kTcThreads, tc_layout(N, a.fc.n, ADJ).total, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

bool threephonon_tc_supported(int n, int precision, int n_fc) {
    if (precision == 0 || (n != 9 && n != 12 && n != 15)) return false;
    // at least two CTAs per SM in both passes
    return tc_layout(n, n_fc, false).total <= 110 * 1024 && tc_layout(n, n_fc, true).total <= 110 * 1024;
}

int threephonon_tc_max_per_sm(int n, int n_fc, int *api, int *count) {
    switch (n) {
        case 9: return tc_per_sm<9, false>(n_fc, api, count);
        case 12: return tc_per_sm<12, false>(n_fc, api, count);
        case 15: return tc_per_sm<15, false>(n_fc, api, count);
        default: return 0;
    }
}

cudaError_t launch_threephonon_tc(const ThreePhArgs &a, int n_sm, int ctas_per_sm, cudaStream_t s) {
    if (a.n_trip <= 0) return cudaSuccess;
    if (!a.tc_eimg || !a.plan_pm || !a.plan_word || a.plan_slots < 8 || a.plan_slots % 8 != 0) return cudaErrorInvalidValue;
    switch (a.mesh.n_mode) {
        case 9: return tc_launch_grid<9, false>(a, tc_grid<9, false>(a.fc.n, a.n_trip, n_sm, ctas_per_sm), s);
        case 12: return tc_launch_grid<12, false>(a, tc_grid<12, false>(a.fc.n, a.n_trip, n_sm, ctas_per_sm), s);
        case 15: return tc_launch_grid<15, false>(a, tc_grid<15, false>(a.fc.n, a.n_trip, n_sm, ctas_per_sm), s);
        default: return cudaErrorNotSupported;
    }
}

int threephonon_tc_adjoint_grid(int n, int n_sm, int n_trip, int n_fc) {
    switch (n) {
        case 9: return tc_grid<9, true>(n_fc, n_trip, n_sm, 0);
        case 12: return tc_grid<12, true>(n_fc, n_trip, n_sm, 0);
        case 15: return tc_grid<15, true>(n_fc, n_trip, n_sm, 0);
        default: return 0;
    }
}

cudaError_t launch_threephonon_tc_adjoint(const ThreePhArgs &a, int grid, cudaStream_t s) {
    if (a.n_trip <= 0) return cudaSuccess;
    if (!a.tc_eimg || !a.tc_eimg_t || !a.plan_pm || !a.plan_word || a.plan_slots < 8 || a.plan_slots % 8 != 0 || !a.lam ||
        !a.mwm_bar)
        return cudaErrorInvalidValue;
    switch (a.mesh.n_mode) {
        case 9: return tc_launch_grid<9, true>(a, grid, s);
        case 12: return tc_launch_grid<12, true>(a, grid, s);
        case 15: return tc_launch_grid<15, true>(a, grid, s);
        default: return cudaErrorNotSupported;
    }
}

int pretransform_plan(int n, int n_blk, const int32_t *blk_ptr, int threads, bool tc_operand,
                      std::vector<uint32_t> &word, std::vector<uint32_t> &src) {
    const int na = n / 3;
    if (n % 3 != 0 || n > 16 || n_blk != na * na * na || blk_ptr[0] != 0 || threads < 32 || threads % 32 != 0)
        return 0;
    const int n_fc = blk_ptr[n_blk];
    if (n_fc < 0 || n_fc + 4 > 0xffff) return 0;
    // elements (block, ijk) with their slot counts, largest first (stable), each to the
    // least-loaded thread (lowest index on ties)
    std::vector<int> blocks(n_blk);
    for (int b = 0; b < n_blk; ++b) blocks[b] = b;
    auto slots_of = [&](int b) { return (blk_ptr[b + 1] - blk_ptr[b] + 3) / 4; };
    std::stable_sort(blocks.begin(), blocks.end(), [&](int x, int y) { return slots_of(x) > slots_of(y); });
    using Load = std::pair<int, int>;  // (slots, thread)
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
    for (int t = 0; t < threads; ++t) heap.push({0, t});
    std::vector<std::vector<int>> mine(threads);  // element = 27 block + ijk
    for (int b : blocks) {
        const int c = slots_of(b);
        if (c == 0) break;
        for (int ijk = 0; ijk < 27; ++ijk) {
            Load l = heap.top();
            heap.pop();
            mine[l.second].push_back(27 * b + ijk);
            heap.push({l.first + c, l.second});
        }
    }
    int most = 0;
    while (!heap.empty()) {
        most = std::max(most, heap.top().first);
        heap.pop();
    }
    const int slots = std::max(8, (most + 7) / 8 * 8);
    word.assign((size_t)slots * threads, 0u);
    src.assign((size_t)slots * threads, 0u);
    for (int t = 0; t < threads; ++t) {
        int sl = 0;
        for (int e : mine[t]) {
            const int b = e / 27, ijk = e % 27;
            const int lo = blk_ptr[b], c = blk_ptr[b + 1] - lo;
            const int a1 = b / (na * na), a2 = (b / na) % na, a3 = b % na;
            const int pa = 3 * a1 + ijk % 3, pb = 3 * a2 + (ijk / 3) % 3, pcc = 3 * a3 + ijk / 9;
            // tensor-core operand: byte offset / 2 (< 4096); fused SIMT kernel: index of
            // P(a, b, c) in its n^3 array (< 4096)
            const uint32_t code = tc_operand ? a_off_mn(16 * pcc + pb, pa) / 2u : (uint32_t)((pa * n + pb) * n + pcc);
            for (int j = 0; j < c; j += 4) {
                const size_t i = (size_t)sl * threads + t;
                const uint32_t f = (uint32_t)(lo + j), nv = (uint32_t)std::min(4, c - j);
                word[i] = f | (j + 4 >= c ? ((code + 1u) << 16) : 0u);
                src[i] = f | ((uint32_t)ijk << 16) | (nv << 21);
                ++sl;
            }
        }
    }
    return slots;
}

cudaError_t launch_fill_plan(const uint32_t *src, int slots, int threads, const float *mwm32, float4 *pm,
                             cudaStream_t s) {
    const int64_t n_slot = (int64_t)slots * threads;
    if (n_slot <= 0) return cudaErrorInvalidValue;
    k_fill_plan<<<(unsigned)((n_slot + 255) / 256), 256, 0, s>>>(src, n_slot, mwm32, pm);
    return cudaGetLastError();
}

cudaError_t launch_tc_eimg(int32_t n_full, int32_t n, const float2 *egvs32, unsigned char *out, cudaStream_t s,
                           bool transpose) {
    if (n > 16) return cudaErrorInvalidValue;
    const int64_t total = (int64_t)n_full * 1024;
    k_tc_eimg<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n_full, n, egvs32, out, transpose ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace tdg
