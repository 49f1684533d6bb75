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
//           (scattering_threephonon.f90:115-135, 219-271): FP32 screen, FP32 Gaussians
//           and occupation factors from FP32 frequency pairs, FP64 sums.
// GEMM operands are BF16 hi/lo splits of FP32 values (hi*hi + hi*lo + lo*hi into an FP32
// tensor-memory accumulator, about 16 significant bits per operand) in shared memory as
// 8 x 16-byte core matrices without swizzle, both operands MN-major; the layout and the
// descriptor reading (leading byte offset = K-direction core stride, stride byte offset =
// MN-direction core stride) are the ones the one-tile self-check verifies.
#include <cuda_bf16.h>

#include <algorithm>

#include "dev_common.cuh"
#include "tc_common.cuh"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr double kLnPrefactor = 3.141592653589793 / 16.0;
constexpr float kSqrt2PiInvF = 0.3989422804014327f;
constexpr long long kLnWaitCycles = 4000000000LL;  // about 2 s at 2 GHz

__device__ __forceinline__ void store_split(__nv_bfloat16 *hi, __nv_bfloat16 *lo, int64_t i, float v) {
    unsigned short h, l;
    tc::split_bf16(v, h, l);
    hi[i] = __ushort_as_bfloat16(h);
    lo[i] = __ushort_as_bfloat16(l);
}

// ---- tiled operand layout ----
// A stage contracts the component index of an operand X[k][p]: k = ri * np + a (real and
// imaginary parts, np = n rounded up to 8, rows a >= n zero) and p the position of the two
// other indices (x, y), x being the one the next stage contracts. Positions are grouped in
// tiles of 8 x by 16 y, the 128 rows of one MMA tile:
//   p = ((x / 8) * nyb + y / 16) * 128 + (y % 16) * 8 + x % 8,  nyb = ceil(n / 16),
// so that the outputs of one tile (8 x, 16 y, every new mode w) fill whole 2 KB runs of the
// next stage's operand (8 consecutive k' = ri' * np + x, every position of two tiles).
// Operand planes are stored in the exact byte image of one shared-memory pipeline stage, so
// that each stage is filled by contiguous bulk copies: the plane is cut into tiles of 16 k x
// 128 p, tile (p / 128, k / 16) at ((p / 128) * kp / 16 + k / 16) * 2048 elements; inside a
// tile, 8 x 8 core matrices (8 k rows of 8 consecutive p): core (k / 8, p / 8) at
// ((k / 8) % 2) * 1024 + ((p / 8) % 16) * 64 elements, row k % 8 at 8 elements.
__device__ __forceinline__ int64_t xt_off(int k, int p, int nchk) {
    return ((int64_t)(p >> 7) * nchk + (k >> 4)) * 2048 + ((k >> 3) & 1) * 1024 + ((p >> 3) & 15) * 64 + (k & 7) * 8 +
           (p & 7);
}
__host__ __device__ __forceinline__ int ln_np(int n) { return (n + 7) & ~7; }
// An eigenvector matrix B[k][c] (k, c < kp) in chunks of 16 k: chunk k / 16 at 16 kp
// elements; inside, core (k / 8, c / 8) at ((k / 8) % 2) * 8 kp + (c / 8) * 64, row k % 8.
__device__ __forceinline__ int64_t bt_off(int k, int c, int kp) {
    return (int64_t)(k >> 4) * 16 * kp + ((k >> 3) & 1) * 8 * kp + (c >> 3) * 64 + (k & 7) * 8 + (c & 7);
}

// ---- real-split eigenvector matrices of every mesh point ----
// bmat[(q*2 + h) * kp * kp + bt_off(k, c)], h = 0 hi / 1 lo; k = ri*np + a, c = rj*np + b:
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
    const int np = ln_np(n);
    float v = 0.f;
    if (k < 2 * np && c < 2 * np && k % np < n && c % np < n) {
        const int ri = k / np, a = k % np, rj = c / np, b = c % np;
        const float2 E = transpose ? egvs32[((size_t)q * n + a) * n + b] : egvs32[((size_t)q * n + b) * n + a];
        v = ri == 0 ? (rj == 0 ? E.x : E.y) : (rj == 0 ? -E.y : E.x);
    }
    store_split(bmat + ((int64_t)q * 2) * per, bmat + ((int64_t)q * 2 + 1) * per, bt_off(k, c, kp), v);
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

__device__ __forceinline__ uint4 pack8(const unsigned short (&h)[8]) {
    uint4 r;
    r.x = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
    r.y = (uint32_t)h[2] | ((uint32_t)h[3] << 16);
    r.z = (uint32_t)h[4] | ((uint32_t)h[5] << 16);
    r.w = (uint32_t)h[6] | ((uint32_t)h[7] << 16);
    return r;
}

// ---- pretransform into the stage-1 operand: X[k][p], k = ri*np + a, p = position of (b, c) ----
// One thread per (slot, position tile, group of 8 a, unit q): it sums the force constants of
// a = 8 ag + q % 8, c = 16 yb + q / 8 and the 8 b of the tile, and writes the 16-byte units
// of the real row (k = a) and the imaginary row (k = np + a); the 32 lanes of a warp write
// 512 contiguous bytes of each. Padding (a, b or c >= n) is written as zero.
__device__ __forceinline__ void store_unit(__nv_bfloat16 *hi, __nv_bfloat16 *lo, int64_t o, const float (&v)[8]) {
    unsigned short h[8], l[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) tc::split_bf16(v[i], h[i], l[i]);
    *reinterpret_cast<uint4 *>(hi + o) = pack8(h);
    *reinterpret_cast<uint4 *>(lo + o) = pack8(l);
}

__global__ void k_ln_pretransform(int n, int na, Fc3Dev fc, const float2 *ph, int nb, int64_t plane, int nchk, int nyb,
                                  __nv_bfloat16 *xhi, __nv_bfloat16 *xlo) {
    const int s = blockIdx.y;
    const int np = ln_np(n), nag = np / 8, n_mt = ((n + 7) / 8) * nyb;
    const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nb || u >= (int64_t)n_mt * nag * 128) return;
    const int q = (int)(u & 127);
    const int ag = (int)((u >> 7) % nag), mt = (int)((u >> 7) / nag);
    const int a = ag * 8 + (q & 7), c = (mt % nyb) * 16 + (q >> 3), b0 = (mt / nyb) * 8;
    float re[8], im[8];
    const float2 *phs = ph + (size_t)s * fc.n;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int b = b0 + i;
        float2 acc = make_float2(0.f, 0.f);
        if (a < n && b < n && c < n) {
            const int blk = ((a / 3) * na + b / 3) * na + c / 3;
            const int ijk = (a % 3) + 3 * (b % 3) + 9 * (c % 3);
            for (int tt = fc.blk_ptr[blk]; tt < fc.blk_ptr[blk + 1]; ++tt) {
                const float mv = __ldg(fc.mwm32 + (size_t)tt * 27 + ijk);
                const float2 p = phs[tt];
                acc.x = fmaf(mv, p.x, acc.x);
                acc.y = fmaf(mv, p.y, acc.y);
            }
        }
        re[i] = acc.x;
        im[i] = acc.y;
    }
    __nv_bfloat16 *hi = xhi + (int64_t)s * plane, *lo = xlo + (int64_t)s * plane;
    const int p = mt * 128 + (c & 15) * 8;
    store_unit(hi, lo, xt_off(a, p, nchk), re);
    store_unit(hi, lo, xt_off(np + a, p, nchk), im);
}

// ---- one contraction stage on the tensor cores ----
struct LnGemmArgs {
    const __nv_bfloat16 *xhi, *xlo;  // operand planes (tiled, xt_off), slot s at + s * plane
    int64_t plane;
    int n_mt;                        // position tiles of 128 per slot: ceil(n / 8) * nyb
    int nyb;                         // ceil(n / 16)
    int nb;                          // slots
    const __nv_bfloat16 *bmat;       // k_build_bmat
    const TripletRec *trip;          // the batch's q-triplets (slot order)
    const int32_t *irr_full;         // 0-based full index of irreducible q1
    int stage;                       // 1, 2, 3: contract with E(q1), E(q2), E(q3)
    int n, np, kp;                   // modes, n rounded up to 8, padded 2 np (multiple of 16)
    int n_stage;                     // shared-memory pipeline stages
    uint32_t acc_cols;               // tensor-memory columns of one accumulator (power of two >= kp)
    __nv_bfloat16 *ohi, *olo;        // stages 1-2: next operand planes (tiled)
    float2 *psi;                     // stage 3: [slot][n^3]
    int32_t *status;
};

// Persistent, warp-specialised: one CTA per SM walks the tiles (slot, 128 positions)
// t = blockIdx.x + i * gridDim.x, so that the CTAs working at one time share the slot's
// eigenvector matrix in L2.
//   warp 0 (one thread)  producer: per K chunk of 16, four bulk copies (A hi/lo 4 KB each,
//                        B hi/lo 16 kp * 2 bytes each) into a ring of n_stage stages, each
//                        stage with a `full` barrier (transaction bytes) and an `empty`
//                        barrier (the MMAs that read it have completed);
//   warp 1 (one thread)  MMA issuer: hi*hi + hi*lo + lo*hi per chunk (M = 128, N = kp,
//                        K = 16) into one of two tensor-memory accumulators, committed to
//                        the stage's `empty` barrier and, after the last chunk, to the
//                        accumulator's `afull` barrier;
//   warps 2-9            epilogue: wait on `afull`; copy the accumulator into a padded
//                        shared-memory staging tile (warp w reads the TMEM lanes of its lane
//                        group w % 4, warps w and w + 4 split the columns) and release it
//                        (`aempty`), so that the MMAs of tile i + 2 can start; then write the
//                        tile's outputs from the staging tile with coalesced stores: whole
//                        2 KB runs of the next operand (hi and lo), or whole rows of Psi.
// Every wait is bounded; a role that gives up sets a shared abort flag that makes the other
// roles leave their loops (the epilogue warps decide together, through a barrier reduction,
// so that none waits at a barrier the others have left), and the CTA drains its copies and
// MMAs before the tensor memory is freed.
constexpr int kLnMaxStages = 8;
constexpr int kLnGemmThreads = 320;
constexpr uint32_t kLnTileBytes = 128u * 16u * 2u;  // one plane of one A chunk
constexpr int kLnSmemLimit = 232448 - 1024;        // dynamic shared memory available to k_ln_gemm

__device__ __forceinline__ bool ln_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
    const long long t0 = clock64();
    while (!tc::mbar_try_wait(bar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > kLnWaitCycles) {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}

// Named barrier 1 over the 256 epilogue threads, with the AND of their predicates.
__device__ __forceinline__ bool epi_bar_and(bool p) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, 1, 256, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"(p ? 1u : 0u)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

__global__ void __launch_bounds__(kLnGemmThreads, 1) k_ln_gemm(LnGemmArgs g) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ uint64_t full[kLnMaxStages], empty[kLnMaxStages], afull[2], aempty[2], done;
    __shared__ uint32_t tbase;
    __shared__ volatile int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = g.n, np = g.np, kp = g.kp, S = g.n_stage, nyb = g.nyb;
    const int nch = kp / 16;
    const int n_tiles = g.nb * g.n_mt;
    const uint32_t b_bytes = 16u * (uint32_t)kp * 2u;
    const uint32_t stage_bytes = 2u * (kLnTileBytes + b_bytes);
    const uint32_t a_ck = 16u * 128u, b_ck = 16u * (uint32_t)kp;  // K-direction core strides (bytes)
    const int64_t bper = (int64_t)kp * kp;
    const int pitch = kp + 4;  // staging row pitch in floats: rows of consecutive lanes hit distinct banks
    float *stg = reinterpret_cast<float *>(sm + (size_t)S * stage_bytes);

    if (warp == 0) tc::tmem_alloc(&tbase, 2u * g.acc_cols);
    if (tid == 0) {
        for (int i = 0; i < S; ++i) {
            tc::mbar_init(&full[i], 1);
            tc::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&afull[i], 1);
            tc::mbar_init(&aempty[i], 8);
        }
        tc::mbar_init(&done, 1);
        abort_flag = 0;
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;

    if (warp == 0) {
        if (lane == 0) {  // ---- producer ----
            int it = 0;
            for (int t = blockIdx.x; t < n_tiles && !abort_flag; t += gridDim.x) {
                const int s = t / g.n_mt, mt = t % g.n_mt;
                const TripletRec rec = g.trip[s];
                const int q = g.stage == 1 ? g.irr_full[rec.q1] : (g.stage == 2 ? rec.q2 : rec.q3);
                const __nv_bfloat16 *bh = g.bmat + ((int64_t)q * 2) * bper, *bl = bh + bper;
                const __nv_bfloat16 *xh = g.xhi + (int64_t)s * g.plane + (int64_t)mt * nch * 2048;
                const __nv_bfloat16 *xl = g.xlo + (int64_t)s * g.plane + (int64_t)mt * nch * 2048;
                for (int c = 0; c < nch; ++c, ++it) {
                    const int st = it % S, use = it / S;
                    if (use > 0 && !ln_wait(&empty[st], (uint32_t)((use - 1) & 1), &abort_flag)) break;
                    unsigned char *base = sm + (size_t)st * stage_bytes;
                    tc::mbar_arrive_expect_tx(&full[st], stage_bytes);
                    tc::bulk_g2s(tc::smem_u32(base), xh + (int64_t)c * 2048, kLnTileBytes, &full[st]);
                    tc::bulk_g2s(tc::smem_u32(base + kLnTileBytes), xl + (int64_t)c * 2048, kLnTileBytes, &full[st]);
                    tc::bulk_g2s(tc::smem_u32(base + 2 * kLnTileBytes), bh + (int64_t)c * 16 * kp, b_bytes, &full[st]);
                    tc::bulk_g2s(tc::smem_u32(base + 2 * kLnTileBytes + b_bytes), bl + (int64_t)c * 16 * kp, b_bytes,
                                 &full[st]);
                }
            }
            // copies still in flight land before the CTA leaves: the last fill of every stage
            for (int j = it - 1; j >= 0 && j >= it - S; --j) {
                const long long t0 = clock64();
                while (!tc::mbar_try_wait(&full[j % S], (uint32_t)((j / S) & 1)) && clock64() - t0 < kLnWaitCycles) {
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {  // ---- MMA issuer ----
            const uint32_t idesc = tc::idesc_bf16_f32(128, kp, true, true);
            int it = 0, tl = 0;
            bool issued = false;
            for (int t = blockIdx.x; t < n_tiles && !abort_flag; t += gridDim.x, ++tl) {
                const int buf = tl & 1, use = tl >> 1;
                if (use > 0 && !ln_wait(&aempty[buf], (uint32_t)((use - 1) & 1), &abort_flag)) break;
                tc::fence_after_sync();
                const uint32_t d = taddr + (uint32_t)buf * g.acc_cols;
                bool ok = true;
                for (int c = 0; c < nch; ++c, ++it) {
                    const int st = it % S;
                    if (!ln_wait(&full[st], (uint32_t)((it / S) & 1), &abort_flag)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint32_t a0 = tc::smem_u32(sm + (size_t)st * stage_bytes);
                    const uint32_t ah = a0, al = a0 + kLnTileBytes, bh = a0 + 2 * kLnTileBytes, bl = bh + b_bytes;
                    const uint64_t dah = tc::smem_desc(ah, a_ck, 128), dal = tc::smem_desc(al, a_ck, 128);
                    const uint64_t dbh = tc::smem_desc(bh, b_ck, 128), dbl = tc::smem_desc(bl, b_ck, 128);
                    tc::mma_bf16(d, dah, dbh, idesc, c > 0 ? 1u : 0u);
                    tc::mma_bf16(d, dah, dbl, idesc, 1u);
                    tc::mma_bf16(d, dal, dbh, idesc, 1u);
                    tc::mma_commit(&empty[st]);
                    issued = true;
                }
                if (!ok) break;
                tc::mma_commit(&afull[buf]);
            }
            // every MMA issued by this thread has completed before the tensor memory goes back
            if (issued) {
                tc::mma_commit(&done);
                const long long t0 = clock64();
                while (!tc::mbar_try_wait(&done, 0u) && clock64() - t0 < kLnWaitCycles) {
                }
            }
        }
    } else {  // ---- epilogue (warps 2-9) ----
        const int lg = warp & 3, half = (warp - 2) >> 2, et = tid - 64;
        const int row = 32 * lg + lane;
        int tl = 0;
        for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++tl) {
            const int buf = tl & 1, use = tl >> 1;
            const bool w = ln_wait(&afull[buf], (uint32_t)(use & 1), &abort_flag);
            if (!epi_bar_and(w)) break;
            tc::fence_after_sync();
            // (1) accumulator row `row`, this warp's column half, into the staging tile
            const uint32_t trow = taddr + (uint32_t)buf * g.acc_cols + ((uint32_t)(32 * lg) << 16);
            float *srow = stg + (size_t)row * pitch;
            const int c_lo = half * (kp / 2), c_hi = c_lo + kp / 2;  // kp / 2 is a multiple of 8
            for (int c0 = c_lo; c0 < c_hi; c0 += 16) {
                float x[16];
                if (c0 + 16 <= c_hi) {
                    tc::tmem_ld16(trow + (uint32_t)c0, x);
#pragma unroll
                    for (int i = 0; i < 16; i += 4)
                        *reinterpret_cast<float4 *>(srow + c0 + i) = make_float4(x[i], x[i + 1], x[i + 2], x[i + 3]);
                } else {
                    float y[8];
                    tc::tmem_ld8(trow + (uint32_t)c0, y);
#pragma unroll
                    for (int i = 0; i < 8; i += 4)
                        *reinterpret_cast<float4 *>(srow + c0 + i) = make_float4(y[i], y[i + 1], y[i + 2], y[i + 3]);
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&aempty[buf]);
            epi_bar();
            // (2) coalesced stores from the staging tile; staging row r holds position
            // (x, y) = (8 xb + r % 8, 16 yb + r / 8) of this tile
            const int s = t / g.n_mt, mt = t % g.n_mt;
            const int x0 = (mt / nyb) * 8, y0 = (mt % nyb) * 16;
            if (g.stage < 3) {
                // D[(x, y)][ri np + w] -> X'[k' = ri np + x][position of (y, w)]: for every (ri, y half
                // jy, w block wb) one 2 KB run of 128 units of 16 bytes, unit q = (w % 16) * 8 +
                // x % 8 holding the 8 y of the half
                __nv_bfloat16 *hi = g.ohi + (int64_t)s * g.plane, *lo = g.olo + (int64_t)s * g.plane;
                const int nruns = 2 * 2 * nyb;
                for (int u = et; u < nruns * 128; u += 256) {
                    const int R = u >> 7, q = u & 127;
                    const int ri = R / (2 * nyb), jy = (R / nyb) & 1, wb = R % nyb;
                    const int xk = q & 7, w = wb * 16 + (q >> 3);
                    const int x = x0 + xk, ya = y0 + 8 * jy;
                    if (x >= n || w >= n || ya >= n) continue;
                    const int kq = ri * np + x;
                    const int64_t o = (((int64_t)((ya >> 3) * nyb + wb)) * nch + (kq >> 4)) * 2048 + ((kq >> 3) & 1) * 1024 +
                                      (int64_t)q * 8;
                    const float *col = stg + (size_t)(8 * 8 * jy + xk) * pitch + ri * np + w;
                    if (ya + 8 <= n) {
                        unsigned short h[8], l[8];
#pragma unroll
                        for (int i = 0; i < 8; ++i) tc::split_bf16(col[(size_t)8 * i * pitch], h[i], l[i]);
                        *reinterpret_cast<uint4 *>(hi + o) = pack8(h);
                        *reinterpret_cast<uint4 *>(lo + o) = pack8(l);
                    } else {
                        for (int i = 0; ya + i < n; ++i) store_split(hi, lo, o + i, col[(size_t)8 * i * pitch]);
                    }
                }
            } else {
                // Psi[(x n + y) n + b3] = (D[(x, y)][b3], D[(x, y)][np + b3]): for each x of the
                // tile the rows y0.. are one contiguous run
                float2 *out = g.psi + (int64_t)s * n * n * n;
                const int ny = min(16, n - y0);
                const int per_x = ny * n;
                for (int xk = 0; xk < 8; ++xk) {
                    const int x = x0 + xk;
                    if (x >= n) break;
                    float2 *dst = out + ((int64_t)x * n + y0) * n;
                    for (int e = et; e < per_x; e += 256) {
                        const int yy = e / n, b3 = e - yy * n;
                        const float *r = stg + (size_t)(yy * 8 + xk) * pitch;
                        dst[e] = make_float2(r[b3], r[np + b3]);
                    }
                }
            }
            epi_bar();  // the staging tile is free for the next tile
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (abort_flag && tid == 0) atomicExch(g.status, kDevOverflow);
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(taddr, 2u * g.acc_cols);
    }
}

// ---- delta weights and accumulation: one CTA per (slot, b1) ----
// GB300's FP64 pipe is 1/64 of FP32, and only a fraction of the n^2 mode pairs (b2, b3) has a
// Gaussian inside its 8-sigma window. In blocks of BB rows b2 (16 or 32, autotuned): (A) every pair is screened
// in FP32 (window with a margin far above FP32 rounding, degeneracy skips pre-checked in
// FP32), the survivors are compacted into a queue with a block scan; (B) full warps evaluate
// the queue's Gaussians (the reference's 8-sigma window) and occupations in FP32 into a
// dense FP64 F; (C) R2[b2] = sum_b3 F and R3[b3] += sum_b2 F in FP64.

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

__host__ __device__ inline size_t ln_delta_smem(int n, int bb) {
    return sizeof(double) * (size_t)14 * n + sizeof(float) * (size_t)bb * n + sizeof(uint32_t) * (size_t)bb * n +
           sizeof(int) * 33 + sizeof(float) * 8 * (size_t)n + 16;
}

// ADJ: the adjoint's weights. F holds G_b = lam(row) * nred * dF_b/d|Psi_b|^2 of the
// survivors (F without |Psi|^2), and W_b = G_b conj(Psi_b) replaces Psi_b for every (b2, b3)
// of the row mode b1, zero where nothing survives or the row is not sampled.
template <bool ADJ, int BB>
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
    double *v2 = s3 + n, *v3 = v2 + 3 * n, *R2 = v3 + 3 * n, *R3 = R2 + n;
    float *F = (float *)(R3 + n);  // the block's F in FP32 (its values are FP32 products)
    uint32_t *Q = (uint32_t *)(F + (size_t)BB * n);
    int *wsum = (int *)(Q + (size_t)BB * n);
    // FP32 copies for the screen (double -> float conversions run on the FP64 pipe, so they
    // are made once per mode here instead of once per pair); NaN marks omega < 1e-9 Ha.
    float *g2 = (float *)(wsum + 33), *g3 = g2 + n, *t2 = g3 + n, *t3 = t2 + n, *c2 = t3 + n, *c3 = c2 + n;
    float *l2 = c3 + n, *l3 = l2 + n;  // om - (double)g, the FP32 rest of each frequency
    for (int b = tid; b < n; b += bd) {
        om2[b] = P.omega[(size_t)q2 * n + b];
        om3[b] = P.omega[(size_t)q3 * n + b];
        be2[b] = P.be[(size_t)i2 * n + b];
        be3[b] = P.be[(size_t)i3 * n + b];
        s2[b] = P.sigsq[(size_t)i2 * n + b];
        s3[b] = P.sigsq[(size_t)i3 * n + b];
        g2[b] = om2[b] < kFreqTolD ? __int_as_float(0x7fc00000) : (float)om2[b];
        g3[b] = om3[b] < kFreqTolD ? __int_as_float(0x7fc00000) : (float)om3[b];
        t2[b] = (float)s2[b];
        t3[b] = (float)s3[b];
        c2[b] = (float)be2[b];
        c3[b] = (float)be3[b];
        l2[b] = om2[b] < kFreqTolD ? 0.f : (float)(om2[b] - (double)g2[b]);
        l3[b] = om3[b] < kFreqTolD ? 0.f : (float)(om3[b] - (double)g3[b]);
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
    // F = perm * (pi/16) |Psi|^2 w * ((n2 - n3) d0 + (n2 + n3 + 1) d1), constants folded;
    // the adjoint's G = lambda(row) * k * dF/d|Psi|^2
    const double pw = perm * kLnPrefactor * w;
    const double fadj = ADJ ? a.lam[row] * (double)rec.red_cnt * pw : 0.0;
    const float pwf = (float)pw, fadjf = (float)fadj;
    const int it = P.integrationtype;
    const float fo1 = (float)o1, fs1 = (float)s1, fsig = (float)P.sigma_fixed;
    const float fl1 = (float)(o1 - (double)fo1);
    const float2 *psi = a.psi + ((int64_t)s * n + b1) * n * n;
    // 4-bit live mask of the Gaussians of pair (b2, b3), 0 when a skip rule applies
    // (scattering_threephonon.f90:90-101) or no Gaussian can reach its window. FP64 work
    // only for the rare pairs whose FP32 frequencies nearly coincide.
    auto screen = [&](int b2, int b3) -> uint32_t {
        const float f2 = g2[b2], f3 = g3[b3];
        if (f2 != f2 || f3 != f3) return 0u;  // omega2 or omega3 below 1e-9 Ha
        // |x - y| < 1e-9 from the FP32 (hi, rest) pairs: the hi difference is exact where it
        // matters (Sterbenz), so the test is the FP64 one to ~1e-17; no FP64 instruction (a
        // short-circuit FP64 test is evaluated for every pair once the compiler if-converts it)
        if (close_f32(fo1, fl1, f2, l2[b2])) return 0u;
        if (close_f32(fo1, fl1, f3, l3[b3])) return 0u;
        if (close_f32(f2, l2[b2], f3, l3[b3])) return 0u;
        if (it == 6) return 15u;  // the velocity-difference width can cancel in FP32: not screened
        const float sg = it == 1 ? fsig : sqrt_screen(fs1 + t2[b2] + t3[b3]);
        const float win = 8.0f * sg * 1.001f + 1e-6f * (fo1 + f2 + f3);
        return (fabsf(fo1 + f2 - f3) <= win ? 1u : 0u) | (fabsf(fo1 - f2 + f3) <= win ? 2u : 0u) |
               (fabsf(fo1 - f2 - f3) <= win ? 4u : 0u) | (fo1 + f2 + f3 <= win ? 8u : 0u);
    };
    for (int bb = 0; bb < n; bb += BB) {
        const int nbb = min(BB, n - bb), cnt = nbb * n;
        // (A) contiguous chunk per thread (at most 16 entries: BB * 128 / 256)
        const int per = (cnt + bd - 1) / bd;
        const int e0 = min(cnt, tid * per), e1 = min(cnt, e0 + per);
        uint64_t lives = 0;
        int ns = 0;
        for (int e = e0; e < e1; ++e) {
            const uint32_t l = screen(bb + e / n, e % n);
            lives |= (uint64_t)l << (4 * (e - e0));
            ns += l != 0u;
        }
        for (int e = tid; e < cnt; e += bd) F[e] = 0.f;
        int total = 0;
        int k = block_exclusive_scan(ns, wsum, total);  // contains __syncthreads
        for (int e = e0; e < e1; ++e) {
            const uint32_t l = (uint32_t)(lives >> (4 * (e - e0))) & 15u;
            if (l) Q[k++] = (uint32_t)e | (l << 16);
        }
        __syncthreads();
        // (B) delta weights and occupations of the survivors, full warps: the Gaussians and
        // occupation factors in FP32, the centre differences from FP32 (hi, rest) frequency
        // pairs (the path is mixed precision; GB300 issues FP64 at 1/64 of the FP32 rate, and
        // an FP64 warp instruction holds its pipe for 16 cycles whatever its active lanes),
        // the sums in FP64
        for (int i = tid; i < total; i += bd) {
            const uint32_t qv = Q[i];
            const int e = (int)(qv & 0xffffu);
            uint32_t live = qv >> 16;
            const int b2 = bb + e / n, b3 = e % n;
            float sigma;
            if (it == 1) {
                sigma = fsig;
            } else if (it == 2) {
                sigma = sqrtf(fs1 + t2[b2] + t3[b3]);
            } else {
                sigma = (float)(adaptive_pair(v1, v2 + 3 * b2, P.reclat_g) / 3.0 +
                                adaptive_pair(v1, v3 + 3 * b3, P.reclat_g) / 3.0 +
                                adaptive_pair(v2 + 3 * b2, v3 + 3 * b3, P.reclat_g) / 3.0 + P.thresh_sigma);
            }
            const float invsig = 1.0f / sigma;
            const float win8 = 8.0f * sigma, h = 0.5f * invsig * invsig, cg = kSqrt2PiInvF * invsig;
            float gs[4] = {0.f, 0.f, 0.f, 0.f};
            const float h2 = g2[b2], r2 = l2[b2], h3 = g3[b3], r3 = l3[b3];
            while (live) {
                const int j = __ffs(live) - 1;
                live &= live - 1;
                // Gaussian j centred at (-om2+om3, om2-om3, om2+om3, -om2-om3), get_dirac's
                // order; the centre difference from the FP32 (hi, rest) pairs, no FP64
                const float sg2 = (j == 1 || j == 2) ? 1.f : -1.f;
                const float sg3 = (j == 0 || j == 2) ? 1.f : -1.f;
                const float dx = centre_diff_f32(fo1, fl1, sg2 * h2, sg2 * r2, sg3 * h3, sg3 * r3);
                const float gj = fabsf(dx) > win8 ? 0.f : expf(-dx * dx * h) * cg;
                gs[0] = j == 0 ? gj : gs[0];
                gs[1] = j == 1 ? gj : gs[1];
                gs[2] = j == 2 ? gj : gs[2];
                gs[3] = j == 3 ? gj : gs[3];
            }
            const float d0 = gs[0] - gs[1], d1 = gs[2] - gs[3];
            if (d0 == 0.f && d1 == 0.f) continue;
            const float n2 = c2[b2], n3 = c3[b3];
            const float occ = (n2 - n3) * d0 + (n2 + n3 + 1.0f) * d1;
            if (ADJ) {
                F[e] = fadjf * occ;
                continue;
            }
            const float2 ps = psi[b2 * n + b3];
            F[e] = pwf * fmaf(ps.x, ps.x, ps.y * ps.y) * occ;
        }
        __syncthreads();
        if (ADJ) {
            float2 *wr = a.w + ((int64_t)s * n + b1) * n * n + (int64_t)bb * n;
            for (int e = tid; e < cnt; e += bd) {
                const float g = F[e];
                const float2 ps = wr[e];
                wr[e] = make_float2(g * ps.x, -g * ps.y);
            }
            __syncthreads();
            continue;
        }
        // (C) row sums of the block and running column sums, spread over the whole block: a
        // warp per row with the columns split over its lanes, two threads per column; the
        // block sums in double-float on the FP32 pipe (TwoSum; exact to ~2^-44 for these
        // few hundred FP32 terms), turned into FP64 once per row and column: an FP64 warp
        // instruction holds GB300's FP64 pipe 16 cycles whatever its active lanes, and the
        // FP64 adds over the dense block had been about 40 % of the kernel
        {
            const int lane = tid & 31, wid = tid >> 5, nw = bd >> 5;
            for (int r = wid; r < nbb; r += nw) {
                float2 sum = make_float2(0.f, 0.f);
                for (int b3 = lane; b3 < n; b3 += 32) df_acc(sum, F[r * n + b3]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    sum = df_merge(sum, make_float2(__shfl_xor_sync(0xffffffffu, sum.x, o),
                                                    __shfl_xor_sync(0xffffffffu, sum.y, o)));
                if (lane == 0) R2[bb + r] = (double)sum.x + (double)sum.y;
            }
            const int n2c = ((2 * n + 31) / 32) * 32;
            for (int t = tid; t < n2c; t += bd) {  // warp-uniform trip count
                const int b3 = t >> 1, h = t & 1;
                float2 sum = make_float2(0.f, 0.f);
                if (b3 < n)
                    for (int r = h; r < nbb; r += 2) df_acc(sum, F[r * n + b3]);
                sum = df_merge(sum, make_float2(__shfl_xor_sync(0xffffffffu, sum.x, 1),
                                                __shfl_xor_sync(0xffffffffu, sum.y, 1)));
                if (h == 0 && b3 < n) R3[b3] += (double)sum.x + (double)sum.y;
            }
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

// ---- adjoint: W[b1][b2][b3] into the stage-1 operand planes X[(ri, b1)][the position of (b2, b3)] ----
// Same thread layout as k_ln_pretransform (b1 in place of a, b2 of b, b3 of c).
__global__ void k_ln_pack(int n, const float2 *w, int nb, int64_t plane, int nchk, int nyb, __nv_bfloat16 *xhi,
                          __nv_bfloat16 *xlo) {
    const int s = blockIdx.y;
    const int np = ln_np(n), nag = np / 8, n_mt = ((n + 7) / 8) * nyb;
    const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nb || u >= (int64_t)n_mt * nag * 128) return;
    const int q = (int)(u & 127);
    const int ag = (int)((u >> 7) % nag), mt = (int)((u >> 7) / nag);
    const int b1 = ag * 8 + (q & 7), b3 = (mt % nyb) * 16 + (q >> 3), b20 = (mt / nyb) * 8;
    const float2 *ws = w + (int64_t)s * n * n * n;
    float re[8], im[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int b2 = b20 + i;
        const float2 v = (b1 < n && b2 < n && b3 < n) ? ws[((int64_t)b1 * n + b2) * n + b3] : make_float2(0.f, 0.f);
        re[i] = v.x;
        im[i] = v.y;
    }
    __nv_bfloat16 *hi = xhi + (int64_t)s * plane, *lo = xlo + (int64_t)s * plane;
    const int p = mt * 128 + (b3 & 15) * 8;
    store_unit(hi, lo, xt_off(b1, p, nchk), re);
    store_unit(hi, lo, xt_off(np + b1, p, nchk), im);
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

int ln_kp(int n) { return ((2 * ln_np(n) + 15) / 16) * 16; }
int ln_mp(int n) { return ((n + 7) / 8) * ((n + 15) / 16) * 128; }

// Pipeline stages of k_ln_gemm for kp: up to 4 (deeper rings measured no faster), as many
// as fit beside the staging tile of 128 x (kp + 4) floats. The dynamic shared memory is at
// least 120 KB, so that one CTA holds an SM (and its 2 x 256 tensor-memory columns) alone.
size_t ln_staging_bytes(int kp) { return (size_t)128 * (kp + 4) * sizeof(float); }
int ln_gemm_stages(int kp) {
    const size_t stage = 2 * ((size_t)kLnTileBytes + (size_t)16 * kp * 2);
    const size_t room = (size_t)kLnSmemLimit - ln_staging_bytes(kp);
    return (int)std::min<size_t>(4, room / stage);
}
size_t ln_gemm_smem(int kp) {
    const size_t stage = 2 * ((size_t)kLnTileBytes + (size_t)16 * kp * 2);
    return std::max<size_t>((size_t)ln_gemm_stages(kp) * stage + ln_staging_bytes(kp), (size_t)120 << 10);
}

cudaError_t launch_ln_bmat(int n, int n_q, const float2 *egvs32, __nv_bfloat16 *bmat, bool transpose,
                           cudaStream_t s) {
    const int kp = ln_kp(n);
    const int64_t total = (int64_t)n_q * kp * kp;
    if (total <= 0) return cudaSuccess;
    k_build_bmat<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n, kp, n_q, egvs32, bmat, transpose ? 1 : 0);
    return cudaGetLastError();
}

namespace {
// Threads per slot of k_ln_pretransform and k_ln_pack: position tiles x groups of 8
// components x 128 units.
int64_t pack_threads(int n) { return (int64_t)((n + 7) / 8) * ((n + 15) / 16) * (ln_np(n) / 8) * 128; }

// The three tcgen05 stages from the operand in the xa planes to b.psi, with the real-split
// matrices bmat (forward: E; adjoint: E^T).
cudaError_t ln_contract(const LnBatch &b, const __nv_bfloat16 *bmat, cudaStream_t s) {
    const int n = b.n, kp = ln_kp(n);
    cudaError_t e;
    const size_t smem = ln_gemm_smem(kp);
    if ((e = cudaFuncSetAttribute(k_ln_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
        return e;
    LnGemmArgs g;
    g.plane = b.plane;
    g.n_mt = b.mp / 128;
    g.nyb = (n + 15) / 16;
    g.np = ln_np(n);
    g.nb = b.nb;
    g.bmat = bmat;
    g.trip = b.trip;
    g.irr_full = b.mesh.irr_full;
    g.n = n;
    g.kp = kp;
    g.n_stage = b.gemm_stages > 0 ? std::min(b.gemm_stages, ln_gemm_stages(kp)) : ln_gemm_stages(kp);
    g.acc_cols = kp <= 32 ? 32u : (kp <= 64 ? 64u : (kp <= 128 ? 128u : 256u));
    g.psi = b.psi;
    g.status = b.status;
    const int n_tiles = g.nb * g.n_mt;
    const int grid = std::max(1, std::min(n_tiles, b.n_sm > 0 ? b.n_sm : 148));
    for (int stage = 1; stage <= 3; ++stage) {
        const bool from_a = stage != 2;
        g.stage = stage;
        g.xhi = from_a ? b.xa_hi : b.xb_hi;
        g.xlo = from_a ? b.xa_lo : b.xb_lo;
        g.ohi = from_a ? b.xb_hi : b.xa_hi;
        g.olo = from_a ? b.xb_lo : b.xa_lo;
        k_ln_gemm<<<grid, kLnGemmThreads, smem, s>>>(g);
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

template <bool ADJ>
cudaError_t launch_ln_delta(const LnBatch &b, cudaStream_t s) {
    const LnDeltaArgs d = delta_args(b);
    const int bb = b.delta_bb == 16 ? 16 : 32;
    const size_t dsm = ln_delta_smem(b.n, bb);
    const dim3 grid((unsigned)b.n, (unsigned)b.nb);
    cudaError_t e;
    if (bb == 16) {
        if ((e = cudaFuncSetAttribute(k_ln_delta<ADJ, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm)) !=
            cudaSuccess)
            return e;
        k_ln_delta<ADJ, 16><<<grid, 256, dsm, s>>>(d);
    } else {
        if ((e = cudaFuncSetAttribute(k_ln_delta<ADJ, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm)) !=
            cudaSuccess)
            return e;
        k_ln_delta<ADJ, 32><<<grid, 256, dsm, s>>>(d);
    }
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_ln_adjoint_batch(const LnBatch &b, cudaStream_t s) {
    const int n = b.n, kp = ln_kp(n);
    if (b.nb <= 0) return cudaSuccess;
    if (kp > 256) return cudaErrorNotSupported;
    cudaError_t e;
    {
        dim3 grid((unsigned)((b.fc.n + 255) / 256), (unsigned)b.nb);
        k_ln_phases<<<grid, 256, 0, s>>>(b.fc, b.mesh, b.trip, b.nb, b.phase);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        dim3 g2((unsigned)((pack_threads(n) + 255) / 256), (unsigned)b.nb);
        k_ln_pretransform<<<g2, 256, 0, s>>>(n, n / 3, b.fc, b.phase, b.nb, b.plane, kp / 16, (n + 15) / 16, b.xa_hi,
                                             b.xa_lo);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = ln_contract(b, b.bmat, s)) != cudaSuccess) return e;  // Psi
    if ((e = launch_ln_delta<true>(b, s)) != cudaSuccess) return e;  // W over Psi
    {
        dim3 grid((unsigned)((pack_threads(n) + 255) / 256), (unsigned)b.nb);
        k_ln_pack<<<grid, 256, 0, s>>>(n, b.psi, b.nb, b.plane, kp / 16, (n + 15) / 16, b.xa_hi, b.xa_lo);
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
        dim3 grid((unsigned)((pack_threads(n) + 255) / 256), (unsigned)b.nb);
        k_ln_pretransform<<<grid, 256, 0, s>>>(n, n / 3, b.fc, b.phase, b.nb, b.plane, kp / 16, (n + 15) / 16,
                                               b.xa_hi, b.xa_lo);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = ln_contract(b, b.bmat, s)) != cudaSuccess) return e;
    return launch_ln_delta<false>(b, s);
}

}  // namespace tdg
