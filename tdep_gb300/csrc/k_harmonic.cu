// Harmonic stage on the device: the dynamical matrix and its q-gradient at the irreducible
// points, the Hermitian eigenproblem, the gauge of degenerate subspaces, group velocities and
// degeneracy tables, and the unfold onto the full mesh (tdg_problem_load_device).
//
// Reference (src/libolle):
//   D(q), dD/dq        type_forceconstant_secondorder_dynamicalmatrix.f90:484-788, polar
//                      correction type 3 (:654-714): reciprocal-space Ewald sum
//                      (lo_longrange_electrostatics_dynmat.f90:12-360, reconly) and the
//                      non-analytic term at Gamma (type_forceconstant_secondorder_loto.f90:130-163)
//   eigenproblem       :113-164 (zheev there; a cyclic complex Jacobi here)
//   velocities         :167-200, degenerate subspaces :313-360
//   degeneracy         type_phonon_dispersions.f90:1190-1212
//   unfold             type_phonon_dispersions_generation.f90:117-170 with
//                      lo_eigenvector_transformation_matrix (type_symmetryoperation.f90:243-290)
//
// Every step is the host stage's (host/phonons.cpp) operation for operation, in FP64, so the
// two agree to rounding (the device's sin, cos, exp and sqrt differ from the host library's
// by an ulp or so), except the order of the Jacobi rotations up to 24 modes (parallel
// ordering; the same rotations, the eigenpairs agree to rounding, degenerate subspaces up to
// their basis, which the velocity gauge then fixes). Kernels:
//   k_longrange  one CTA per irreducible point: the Ewald pair sums over the reciprocal
//                vectors (chunks of per-vector scalars in shared memory), then the Hermitian
//                completion, the Born charges on both sides and the on-site term;
//   k_dynmat     one CTA per irreducible point, one thread per matrix element: the pairs of
//                its atom pair in file order (the host's summation order), the long-range
//                blocks and the non-analytic term, with masses;
//   k_eigen      one warp per irreducible point (one per CTA), up to 24 modes the matrices in
//                shared memory and parallel-order Jacobi sweeps (one lane per rotation of a
//                step), beyond that global memory and cyclic sweeps with every lane deriving
//                the same rotation; sorting, the Gamma acoustic
//                modes, the velocity-operator gauge of degenerate subspaces, Hellmann-Feynman
//                velocities with the subspace mean, degeneracy tables;
//   k_unfold     one thread per (mesh point, mode, atom).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "dev_common.cuh"
#include "host/crystal.hpp"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr double kSqTolD = 1e-10;    // lo_sqtol
constexpr double kFreqTolH = 1e-9;   // lo_freqtol
constexpr double kPiD = 3.141592653589793;

struct HarmDev {
    int na, nb, nirr, nfull, nop;
    const int32_t *pair_ptr;  // [na*na + 1] pairs grouped by a1*na + a2, file order inside
    const double *lv;         // [np*3] Cartesian lattice vector, Bohr
    const double *m;          // [np*9] m(i,j) at i + 3j
    const double *ism;        // [na] 1/sqrt(mass)
    int polar, nG;
    const double *G;          // [nG*3] reciprocal vectors in the Ewald sphere, 1/Bohr, no 2 pi
    const double *eps;        // [9] dielectric tensor, column-major
    const double *Z;          // [na*9] Born charges Z(i,j,a) at a*9 + i + 3j
    const double *Zon;        // [na*9] on-site correction
    const double *rcart;      // [na*3]
    double lambda, volume;
    const double *qirr;       // [nirr*3] Cartesian, no 2 pi
    double2 *dl;              // [nirr][np2*36] Ewald pair sums (9 dl, 27 dq per pair a1 <= a2)
    double2 *P, *PG;          // [nirr][9 na^2], [nirr][27 na^2] long-range blocks
    double2 *D, *Gd;          // [nirr][nb^2], [nirr][3 nb^2] column-major
    double2 *V;               // [nirr][nb^2] eigenvectors, then the Hellmann-Feynman values
    double2 *S;               // [nirr][2 nb^2 + nb] scratch of the subspace gauge
    double *w;                // [nirr][nb]
    double *om;               // [nirr][nb] frequencies (output)
    double2 *egv;             // [nirr][nb][nb] eigenvector of mode b, component r (output)
    double *vel;              // [nirr][nb][3] (output)
    int32_t *degen, *degen_mode;  // [nirr][nb], [nirr][nb][nb] (output, 1-based modes)
    int32_t *status;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double cnorm(double2 a) { return a.x * a.x + a.y * a.y; }

__device__ __forceinline__ int pair_index(int a1, int a2, int na) {  // a1 <= a2, row-major upper triangle
    return a1 * na - a1 * (a1 - 1) / 2 + (a2 - a1);
}

// Ewald pair sums: dl[ip][i + 3j] = sum_K K_i K_j chi, dq[ip][d][i + 3j] = sum_K (K_i K_j v0_d +
// dK_iK_j/dK_d) chi with chi = exp(-|K|^2_eps / 4 lambda^2) / |K|^2_eps exp(-i K.tau) over
// K = 2 pi (G + q), |K|^2 above lo_sqtol^2; then the completed, Born-charge-weighted blocks.
__global__ void __launch_bounds__(256) k_longrange(HarmDev h) {
    __shared__ double sK[256][3], sP[256], sKe[256][3];
    __shared__ int sOk[256];
    const int iq = blockIdx.x, na = h.na, np2 = na * (na + 1) / 2;
    const double *q = h.qirr + 3 * iq;
    const double inv4l2 = 1.0 / (4.0 * h.lambda * h.lambda);
    const double *eps = h.eps;
    double2 *dl = h.dl + (size_t)iq * np2 * 36;
    const int items = np2 * 36;
    for (int i0 = 0; i0 < items; i0 += blockDim.x) {
        const int it = i0 + threadIdx.x;
        int ip = 0, comp = 0, a1 = 0, a2 = 0;
        double tau[3] = {0, 0, 0};
        if (it < items) {
            ip = it / 36;
            comp = it % 36;
            // pair (a1, a2) of index ip
            int r = ip;
            a1 = 0;
            while (r >= na - a1) {
                r -= na - a1;
                ++a1;
            }
            a2 = a1 + r;
            for (int d = 0; d < 3; ++d) {
                double t = h.rcart[3 * a2 + d] - h.rcart[3 * a1 + d];
                tau[d] = fabs(t) < kSqTolD ? 0.0 : t;
            }
        }
        double2 acc = make_double2(0.0, 0.0);
        for (int g0 = 0; g0 < h.nG; g0 += 256) {
            __syncthreads();
            const int g = g0 + threadIdx.x;
            if (threadIdx.x < 256) {
                int ok = 0;
                double K[3] = {0, 0, 0}, pchi = 0.0, keps[3] = {0, 0, 0};
                if (g < h.nG) {
                    for (int d = 0; d < 3; ++d) {
                        K[d] = (h.G[3 * g + d] + q[d]) * kTwoPiD;
                        if (fabs(K[d]) < kSqTolD) K[d] = 0.0;
                    }
                    if (K[0] * K[0] + K[1] * K[1] + K[2] * K[2] >= kSqTolD * kSqTolD) {
                        ok = 1;
                        double eK[3];
                        for (int i = 0; i < 3; ++i) eK[i] = eps[i] * K[0] + eps[i + 3] * K[1] + eps[i + 6] * K[2];
                        const double knorm = K[0] * eK[0] + K[1] * eK[1] + K[2] * eK[2];
                        const double inv = 1.0 / knorm;
                        pchi = exp(-knorm * inv4l2) * inv;
                        for (int i = 0; i < 3; ++i)
                            keps[i] = 2.0 * (K[0] * eps[3 * i] + K[1] * eps[3 * i + 1] + K[2] * eps[3 * i + 2]) *
                                      (inv + inv4l2);
                    }
                }
                sOk[threadIdx.x] = ok;
                sP[threadIdx.x] = pchi;
                for (int d = 0; d < 3; ++d) {
                    sK[threadIdx.x][d] = K[d];
                    sKe[threadIdx.x][d] = keps[d];
                }
            }
            __syncthreads();
            if (it < items) {
                const int ng = min(256, h.nG - g0);
                for (int k = 0; k < ng; ++k) {
                    if (!sOk[k]) continue;
                    const double *K = sK[k];
                    const double kr = -(K[0] * tau[0] + K[1] * tau[1] + K[2] * tau[2]);
                    double sn, cs;
                    sincos(kr, &sn, &cs);
                    const double2 chi = make_double2(sP[k] * cs, sP[k] * sn);
                    if (comp < 9) {
                        const int i = comp % 3, j = comp / 3;
                        const double kk = K[i] * K[j];
                        acc = cadd(acc, cscale(chi, kk));
                    } else {
                        const int c = comp - 9, d = c / 9, e = c % 9, i = e % 3, j = e / 3;
                        const double2 v0 = make_double2(-sKe[k][d], -tau[d]);  // i*(-tau_d) - keps_d
                        const double dkk = (i == d ? K[j] : 0.0) + (j == d ? K[i] : 0.0);
                        const double kk = K[i] * K[j];
                        const double2 t = make_double2(kk * v0.x + dkk, kk * v0.y);
                        acc = cadd(acc, cmul(t, chi));
                    }
                }
            }
        }
        if (it < items) dl[it] = acc;
    }
    __syncthreads();
    // completed blocks d0 (a1, a2) and the Born charges on both sides; on-site; chop of P
    const double f0 = 4.0 * kPiD / h.volume;
    const int nP = 9 * na * na, nPG = 27 * na * na;
    double2 *P = h.P + (size_t)iq * nP, *PG = h.PG + (size_t)iq * nPG;
    for (int o = threadIdx.x; o < nP + nPG; o += blockDim.x) {
        const bool grad = o >= nP;
        const int oo = grad ? o - nP : o;
        const int d = grad ? oo / (9 * na * na) : 0;
        const int rem = grad ? oo % (9 * na * na) : oo;
        const int blk = rem / 9, e = rem % 9, i = e % 3, j = e / 3;
        const int a1 = blk / na, a2 = blk % na;
        double2 acc = make_double2(0.0, 0.0);
        for (int jj = 0; jj < 3; ++jj)
            for (int ii = 0; ii < 3; ++ii) {
                double2 s;
                if (a1 <= a2) {
                    const int ip = pair_index(a1, a2, na);
                    s = dl[(size_t)ip * 36 + (grad ? 9 + 9 * d : 0) + ii + 3 * jj];
                } else {
                    const int ip = pair_index(a2, a1, na);
                    s = cconj(dl[(size_t)ip * 36 + (grad ? 9 + 9 * d : 0) + jj + 3 * ii]);
                }
                s = cscale(s, f0);
                acc = cadd(acc, cscale(s, h.Z[a1 * 9 + i + 3 * ii] * h.Z[a2 * 9 + j + 3 * jj]));
            }
        if (!grad) {
            if (a1 == a2) acc.x += h.Zon[a1 * 9 + e];
            if (fabs(acc.x) < kSqTolD) acc.x = 0.0;
            if (fabs(acc.y) < kSqTolD) acc.y = 0.0;
            P[rem] = acc;
        } else {
            PG[(size_t)d * 9 * na * na + rem] = acc;
        }
    }
}

// D((a2,j),(a1,i)) = sum_pairs exp(i q.R) m(i,j) / sqrt(m1 m2) and its gradient with respect
// to 2 pi q; polar: the long-range blocks and, at Gamma along [1,0,0] (the mesh's default
// direction), the non-analytic term.
__global__ void __launch_bounds__(256) k_dynmat(HarmDev h) {
    const int iq = blockIdx.x, nb = h.nb, na = h.na;
    const double *qr = h.qirr + 3 * iq;
    double qv[3];
    for (int d = 0; d < 3; ++d) {
        qv[d] = qr[d] * kTwoPiD;
        if (fabs(qv[d]) < 1e-13) qv[d] = 0.0;
    }
    const bool gamma = qr[0] * qr[0] + qr[1] * qr[1] + qr[2] * qr[2] < kSqTolD;
    double2 *D = h.D + (size_t)iq * nb * nb;
    double2 *G = h.Gd + (size_t)iq * 3 * nb * nb;
    // non-analytic term along u = [1,0,0]: zq(i,a) = Z(i,0,a), f0 = (1 / eps(0,0)) 4 pi / V
    const double fna = h.polar == 3 ? (1.0 / h.eps[0]) * 4.0 * kPiD / h.volume : 0.0;
    for (int el = threadIdx.x; el < nb * nb; el += blockDim.x) {
        const int ii = el % nb, jj = el / nb;  // D[ii + nb jj]
        const int a2 = ii / 3, j = ii % 3, a1 = jj / 3, i = jj % 3;
        const double ms = h.ism[a1] * h.ism[a2];
        double2 dsum = make_double2(0.0, 0.0), g[3] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
        for (int p = h.pair_ptr[a1 * na + a2]; p < h.pair_ptr[a1 * na + a2 + 1]; ++p) {
            const double *lv = h.lv + 3 * p;
            const double qdotr = lv[0] * qv[0] + lv[1] * qv[1] + lv[2] * qv[2];
            double sn, cs;
            sincos(qdotr, &sn, &cs);
            const double mm = h.m[9 * p + i + 3 * j];
            const double2 val = make_double2(cs * mm * ms, sn * mm * ms);
            dsum = cadd(dsum, val);
            for (int d = 0; d < 3; ++d) g[d] = cadd(g[d], make_double2(-lv[d] * val.y, lv[d] * val.x));
        }
        if (h.polar == 3) {
            const size_t e = ((size_t)a1 * na + a2) * 9 + i + 3 * j;
            double2 p = h.P[(size_t)iq * 9 * na * na + e];
            if (gamma) p.x += h.Z[a1 * 9 + i] * h.Z[a2 * 9 + j] * fna;
            dsum = cadd(dsum, cscale(p, ms));
            for (int d = 0; d < 3; ++d)
                g[d] = cadd(g[d], cscale(h.PG[(size_t)iq * 27 * na * na + (size_t)d * 9 * na * na + e], ms));
        }
        D[el] = dsum;
        for (int d = 0; d < 3; ++d) G[(size_t)d * nb * nb + el] = g[d];
    }
}

__device__ __forceinline__ double negsqrt(double x) { return x >= 0 ? sqrt(x) : -sqrt(-x); }

// Cyclic complex Jacobi on the n x n Hermitian matrix A (column-major, global memory) by one
// warp: the phase of a_pq goes into column q, then a real rotation zeroes the off-diagonal;
// eigenvectors accumulate in V. Every lane reads the same a_pq, a_pp, a_qq and derives the
// same rotation. Returns false when 100 sweeps do not converge.
__device__ bool warp_jacobi(int n, double2 *A, double2 *V, double *w) {
    const int lane = threadIdx.x & 31;
    for (int k = lane; k < n * n; k += 32) V[k] = make_double2((k % n) == (k / n) ? 1.0 : 0.0, 0.0);
    double scale = 0.0;
    for (int k = lane; k < n * n; k += 32) scale += cnorm(A[k]);
    for (int o = 16; o > 0; o >>= 1) scale += __shfl_xor_sync(0xffffffffu, scale, o);
    __syncwarp();
    if (scale == 0.0) {
        for (int k = lane; k < n; k += 32) w[k] = 0.0;
        __syncwarp();
        return true;
    }
    bool conv = false;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int k = lane; k < n * n; k += 32)
            if ((k % n) != (k / n)) off += cnorm(A[k]);
        for (int o = 16; o > 0; o >>= 1) off += __shfl_xor_sync(0xffffffffu, off, o);
        if (off <= 1e-30 * scale) {
            conv = true;
            break;
        }
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double2 g = A[p + (size_t)n * q];
                const double ag = hypot(g.x, g.y);
                if (ag <= 1e-300) continue;
                const double2 u = make_double2(g.x / ag, g.y / ag);
                const double app = A[p + (size_t)n * p].x, aqq = A[q + (size_t)n * q].x;
                const double tau = (aqq - app) / (2.0 * ag);
                const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                const double cs = 1.0 / sqrt(1.0 + t * t);
                const double sn = t * cs;
                const double2 jqp = cscale(cconj(u), -sn), jqq = cscale(cconj(u), cs);
                __syncwarp();
                for (int k = lane; k < n; k += 32) {  // A <- A J
                    const double2 akp = A[k + (size_t)n * p], akq = A[k + (size_t)n * q];
                    A[k + (size_t)n * p] = cadd(cscale(akp, cs), cmul(akq, jqp));
                    A[k + (size_t)n * q] = cadd(cscale(akp, sn), cmul(akq, jqq));
                }
                __syncwarp();
                for (int k = lane; k < n; k += 32) {  // A <- J^H A
                    const double2 apk = A[p + (size_t)n * k], aqk = A[q + (size_t)n * k];
                    A[p + (size_t)n * k] = cadd(cscale(apk, cs), cmul(cconj(jqp), aqk));
                    A[q + (size_t)n * k] = cadd(cscale(apk, sn), cmul(cconj(jqq), aqk));
                }
                __syncwarp();
                if (lane == 0) {
                    A[p + (size_t)n * q] = make_double2(0.0, 0.0);
                    A[q + (size_t)n * p] = make_double2(0.0, 0.0);
                    A[p + (size_t)n * p].y = 0.0;
                    A[q + (size_t)n * q].y = 0.0;
                }
                for (int k = lane; k < n; k += 32) {  // V <- V J
                    const double2 vkp = V[k + (size_t)n * p], vkq = V[k + (size_t)n * q];
                    V[k + (size_t)n * p] = cadd(cscale(vkp, cs), cmul(vkq, jqp));
                    V[k + (size_t)n * q] = cadd(cscale(vkp, sn), cmul(vkq, jqq));
                }
                __syncwarp();
            }
    }
    for (int k = lane; k < n; k += 32) w[k] = A[k + (size_t)n * k].x;
    __syncwarp();
    return conv;
}

// Stable sort of n < 128 keys into ord (by lane 0; the others wait at the caller's syncwarp).
__device__ void stable_order(int n, const double *key, int *ord) {
    for (int i = 0; i < n; ++i) ord[i] = i;
    for (int i = 1; i < n; ++i) {
        const int x = ord[i];
        int j = i - 1;
        while (j >= 0 && key[ord[j]] > key[x]) {
            ord[j + 1] = ord[j];
            --j;
        }
        ord[j + 1] = x;
    }
}

constexpr int kEigWarps = 1;  // one warp per CTA: the points spread over the SMs, each with its own FP64 pipe
constexpr int kMaxModes = 128;

__global__ void __launch_bounds__(32 * kEigWarps) k_eigen(HarmDev h) {
    __shared__ int s_ord[kEigWarps][kMaxModes];
    __shared__ double s_key[kEigWarps][kMaxModes];
    __shared__ int s_sub[kEigWarps][kMaxModes];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int iq = blockIdx.x * kEigWarps + wid;
    if (iq >= h.nirr) return;
    const int n = h.nb;
    int *ord = s_ord[wid];
    double *key = s_key[wid];
    int *sub = s_sub[wid];
    double2 *A = h.D + (size_t)iq * n * n;
    double2 *V = h.V + (size_t)iq * n * n;
    const double2 *G = h.Gd + (size_t)iq * 3 * n * n;
    double *w = h.w + (size_t)iq * n;
    double *om = h.om + (size_t)iq * n;
    double2 *E = h.egv + (size_t)iq * n * n;  // E[b * n + r]
    // Hermitise against rounding
    for (int k = lane; k < n * n; k += 32) {
        const int i = k % n, j = k / n;
        if (i <= j) {
            const double2 a = A[i + (size_t)n * j], b = cconj(A[j + (size_t)n * i]);
            const double2 s = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
            A[i + (size_t)n * j] = s;
            A[j + (size_t)n * i] = cconj(s);
        }
    }
    __syncwarp();
    if (!warp_jacobi(n, A, V, w)) {
        if (lane == 0) atomicExch(h.status, (int32_t)kDevLinalg);
        return;
    }
    const double *qr = h.qirr + 3 * iq;
    if (lane == 0) {
        if (qr[0] * qr[0] + qr[1] * qr[1] + qr[2] * qr[2] < kSqTolD) {  // acoustic modes at Gamma
            for (int b = 0; b < n; ++b) key[b] = fabs(w[b]);
            stable_order(n, key, ord);
            for (int i = 0; i < min(3, n); ++i) w[ord[i]] = 0.0;
        }
        for (int b = 0; b < n; ++b) key[b] = negsqrt(w[b]);
        stable_order(n, key, ord);
        for (int b = 0; b < n; ++b) om[b] = negsqrt(w[ord[b]]);
    }
    __syncwarp();
    for (int k = lane; k < n * n; k += 32) {
        const int b = k / n, r = k % n;
        E[k] = V[r + (size_t)n * ord[b]];
    }
    __syncwarp();
    // degenerate subspaces (contiguous, within lo_freqtol of the first): the velocity
    // operator along a fixed generic direction diagonalised inside each
    const double dir[3] = {1.0, 1.33, 1.45624623};
    for (int b0 = 0; b0 < n;) {
        int b1 = b0 + 1;
        while (b1 < n && fabs(om[b1] - om[b0]) < kFreqTolH) ++b1;
        const int k = b1 - b0;
        if (k > 1) {
            double2 *Pm = h.S + (size_t)iq * (2 * n * n + n);  // k x k, column-major
            double2 *U = Pm + k * k;                           // k x k
            double *pw = (double *)(U + k * k);
            for (int xy = lane; xy < k * k; xy += 32) {
                const int x = xy % k, y = xy / k;
                double2 s = make_double2(0.0, 0.0);
                for (int d = 0; d < 3; ++d)
                    for (int r = 0; r < n; ++r) {
                        double2 gy = make_double2(0.0, 0.0);
                        for (int cc = 0; cc < n; ++cc)
                            gy = cadd(gy, cmul(G[(size_t)d * n * n + r + (size_t)n * cc], E[(size_t)(b0 + y) * n + cc]));
                        s = cadd(s, cscale(cmul(cconj(E[(size_t)(b0 + x) * n + r]), gy), dir[d]));
                    }
                Pm[x + k * y] = s;
            }
            __syncwarp();
            for (int xy = lane; xy < k * k; xy += 32) {
                const int x = xy % k, y = xy / k;
                if (x <= y) {
                    const double2 a = Pm[x + k * y], b = cconj(Pm[y + k * x]);
                    const double2 s = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
                    Pm[x + k * y] = s;
                    Pm[y + k * x] = cconj(s);
                }
            }
            __syncwarp();
            if (!warp_jacobi(k, Pm, U, pw)) {
                if (lane == 0) atomicExch(h.status, (int32_t)kDevLinalg);
                return;
            }
            if (lane == 0) stable_order(k, pw, ord);
            __syncwarp();
            // sub = E_sub U[:, po]: each lane one component r for all y, from a private copy
            for (int r = lane; r < n; r += 32) {
                double2 old[kMaxModes];
                for (int x = 0; x < k; ++x) old[x] = E[(size_t)(b0 + x) * n + r];
                for (int y = 0; y < k; ++y) {
                    double2 s = make_double2(0.0, 0.0);
                    for (int x = 0; x < k; ++x) s = cadd(s, cmul(old[x], U[x + k * ord[y]]));
                    E[(size_t)(b0 + y) * n + r] = s;
                }
            }
            __syncwarp();
        }
        b0 = b1;
    }
    // Hellmann-Feynman values <e_b|dD/dk_d|e_b> into V as scratch [b*3 + d]
    double *hf = (double *)V;
    for (int bd = lane; bd < 3 * n; bd += 32) {
        const int b = bd / 3, d = bd % 3;
        double2 s = make_double2(0.0, 0.0);
        for (int r = 0; r < n; ++r) {
            double2 gy = make_double2(0.0, 0.0);
            for (int cc = 0; cc < n; ++cc)
                gy = cadd(gy, cmul(G[(size_t)d * n * n + r + (size_t)n * cc], E[(size_t)b * n + cc]));
            s = cadd(s, cmul(cconj(E[(size_t)b * n + r]), gy));
        }
        hf[bd] = s.x;
    }
    __syncwarp();
    if (lane == 0) {  // a mode joins the first subspace holding a mode within lo_freqtol of it
        int nsub = 0;
        for (int b = 0; b < n; ++b) {
            sub[b] = -1;
            for (int a = 0; a < b && sub[b] < 0; ++a)
                if (fabs(om[a] - om[b]) < kFreqTolH) sub[b] = sub[a];
            if (sub[b] < 0) sub[b] = nsub++;
        }
    }
    __syncwarp();
    double *vel = h.vel + (size_t)iq * n * 3;
    for (int b = lane; b < n; b += 32) {
        double mv[3] = {0.0, 0.0, 0.0};
        int cnt = 0;
        for (int a = 0; a < n; ++a)
            if (sub[a] == sub[b]) {
                ++cnt;
                for (int d = 0; d < 3; ++d) mv[d] += hf[a * 3 + d];
            }
        for (int d = 0; d < 3; ++d) vel[b * 3 + d] = om[b] > kFreqTolH ? (mv[d] / cnt) / (2.0 * om[b]) : 0.0;
        int l = 0;
        int32_t *dm = h.degen_mode + ((size_t)iq * n + b) * n;
        for (int b2 = 0; b2 < n; ++b2) {
            if (fabs(om[b] - om[b2]) < kFreqTolH) dm[l++] = b2 + 1;
        }
        for (int b2 = l; b2 < n; ++b2) dm[b2] = 0;
        h.degen[(size_t)iq * n + b] = l;
    }
}

// ---- up to kEigCtaModes modes: one CTA of kEigCtaThreads per irreducible point ----
// GB300 issues FP64 at 2 lanes per clock per SM and the work of one point is a chain of
// dependent FP64 steps, so a point's time is its latency: the CTA spreads each step over
// 4 warps, keeps every matrix in shared memory, and runs the Jacobi sweeps in parallel
// order (cta_jacobi). The products of the subspace gauge and of the Hellmann-Feynman
// velocities are split into G E first (one task per (direction, component, mode)) and the
// sandwich after, with the summation order of the warp kernel's single loops.
constexpr int kEigCtaModes = 24;
constexpr int kEigCtaThreads = 128;

// Sum of v over the CTA, the same value in every thread (red: 32 doubles of shared memory).
__device__ double cta_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();  // red is free
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0.0;
    for (int i = 0; i < nw; ++i) s += red[i];
    return s;
}

// The Hermitian eigenproblem of the n x n matrix A (column-major, shared memory, n <= 32)
// by the CTA: the rotations of the cyclic Jacobi (warp_jacobi) in parallel order. Each step
// rotates the m/2 disjoint pairs (p, q) of a round-robin tournament over m = n rounded up to
// even indices (an index >= n pairs with nothing), thread i deriving pair i's rotation from
// the same snapshot of A (a pair's 2 x 2 block is touched by no other pair of the step),
// then A <- A J, A <- J^H A and V <- V J for all pairs at once; m - 1 steps make a sweep.
// The sweeps to convergence are the cyclic order's (a numpy emulation of both orders on
// random Hermitian matrices, n = 3 to 24) and the eigenpairs agree to rounding (degenerate
// subspaces up to their basis). rot: 64 doubles, pq: (m - 1) m / 2 short2, red: 32 doubles.
// Returns false when 100 sweeps do not converge.
__device__ bool cta_jacobi(int n, double2 *A, double2 *V, double *w, double *rot, short2 *pq, double *red) {
    const int tid = threadIdx.x, T = blockDim.x;
    const int m = (n + 1) & ~1, half = m / 2;
    for (int k = tid; k < n * n; k += T) V[k] = make_double2((k % n) == (k / n) ? 1.0 : 0.0, 0.0);
    for (int i = tid; i < (m - 1) * half; i += T) {  // circle method: slot 0 stays, the others rotate
        const int st = i / half, j = i % half;
        const int a = j == 0 ? 0 : 1 + (j - 1 + st) % (m - 1);
        const int b = 1 + (m - 2 - j + st) % (m - 1);
        pq[i] = make_short2((short)min(a, b), (short)max(a, b));
    }
    double part = 0.0;
    for (int k = tid; k < n * n; k += T) part += cnorm(A[k]);
    const double scale = cta_sum(part, red);
    if (scale == 0.0) {
        for (int k = tid; k < n; k += T) w[k] = 0.0;
        __syncthreads();
        return true;
    }
    bool conv = false;
    for (int sweep = 0; sweep < 100; ++sweep) {
        part = 0.0;
        for (int k = tid; k < n * n; k += T)
            if ((k % n) != (k / n)) part += cnorm(A[k]);
        if (cta_sum(part, red) <= 1e-30 * scale) {
            conv = true;
            break;
        }
        for (int st = 0; st < m - 1; ++st) {
            const short2 *ps = pq + st * half;
            if (tid < half) {
                const int p = ps[tid].x, q = ps[tid].y;
                double cs = 1.0, sn = 0.0, ux = 1.0, uy = 0.0;
                if (q < n) {
                    const double2 g = A[p + (size_t)n * q];
                    const double ag = hypot(g.x, g.y);
                    if (ag > 1e-300) {
                        ux = g.x / ag;
                        uy = g.y / ag;
                        const double app = A[p + (size_t)n * p].x, aqq = A[q + (size_t)n * q].x;
                        const double tau = (aqq - app) / (2.0 * ag);
                        const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        cs = 1.0 / sqrt(1.0 + t * t);
                        sn = t * cs;
                    }
                }
                rot[4 * tid] = cs;
                rot[4 * tid + 1] = sn;
                rot[4 * tid + 2] = ux;
                rot[4 * tid + 3] = uy;
            }
            __syncthreads();
            for (int task = tid; task < half * n; task += T) {  // A <- A J, V <- V J
                const int i = task / n, k = task % n;
                const int p = ps[i].x, q = ps[i].y;
                if (q >= n) continue;
                const double cs = rot[4 * i], sn = rot[4 * i + 1];
                const double2 u = make_double2(rot[4 * i + 2], rot[4 * i + 3]);
                const double2 jqp = cscale(cconj(u), -sn), jqq = cscale(cconj(u), cs);
                const double2 akp = A[k + (size_t)n * p], akq = A[k + (size_t)n * q];
                A[k + (size_t)n * p] = cadd(cscale(akp, cs), cmul(akq, jqp));
                A[k + (size_t)n * q] = cadd(cscale(akp, sn), cmul(akq, jqq));
                const double2 vkp = V[k + (size_t)n * p], vkq = V[k + (size_t)n * q];
                V[k + (size_t)n * p] = cadd(cscale(vkp, cs), cmul(vkq, jqp));
                V[k + (size_t)n * q] = cadd(cscale(vkp, sn), cmul(vkq, jqq));
            }
            __syncthreads();
            for (int task = tid; task < half * n; task += T) {  // A <- J^H A
                const int i = task / n, k = task % n;
                const int p = ps[i].x, q = ps[i].y;
                if (q >= n) continue;
                const double cs = rot[4 * i], sn = rot[4 * i + 1];
                const double2 u = make_double2(rot[4 * i + 2], rot[4 * i + 3]);
                const double2 jqp = cscale(cconj(u), -sn), jqq = cscale(cconj(u), cs);
                const double2 apk = A[p + (size_t)n * k], aqk = A[q + (size_t)n * k];
                A[p + (size_t)n * k] = cadd(cscale(apk, cs), cmul(cconj(jqp), aqk));
                A[q + (size_t)n * k] = cadd(cscale(apk, sn), cmul(cconj(jqq), aqk));
            }
            __syncthreads();
            if (tid < half) {
                const int p = ps[tid].x, q = ps[tid].y;
                if (q < n) {
                    A[p + (size_t)n * q] = make_double2(0.0, 0.0);
                    A[q + (size_t)n * p] = make_double2(0.0, 0.0);
                    A[p + (size_t)n * p].y = 0.0;
                    A[q + (size_t)n * q].y = 0.0;
                }
            }
            __syncthreads();
        }
    }
    for (int k = tid; k < n; k += T) w[k] = A[k + (size_t)n * k].x;
    __syncthreads();
    return conv;
}

// Shared memory of k_eigen_cta for n modes (bytes).
inline size_t eigen_cta_smem(int n) {
    const size_t nn = (size_t)n * n, m = (size_t)((n + 1) & ~1);
    return sizeof(double2) * 8 * nn                      // A, V, E, GE (3 nn), Pm, U
           + sizeof(double) * (64 + 32 + 2 * (size_t)n + 3 * (size_t)n)  // rot, red, key, pw, hf
           + sizeof(int) * 2 * (size_t)n                 // ord, sub
           + sizeof(short2) * (m - 1) * (m / 2) + 16;
}

__global__ void __launch_bounds__(kEigCtaThreads) k_eigen_cta(HarmDev h) {
    extern __shared__ double2 s_cta[];
    const int iq = blockIdx.x, n = h.nb, tid = threadIdx.x, T = blockDim.x;
    const size_t nn = (size_t)n * n;
    double2 *A = s_cta, *V = A + nn, *E = V + nn, *GE = E + nn, *Pm = GE + 3 * nn, *U = Pm + nn;
    double *rot = reinterpret_cast<double *>(U + nn), *red = rot + 64, *key = red + 32, *pw = key + n, *hf = pw + n;
    int *ord = reinterpret_cast<int *>(hf + 3 * n), *sub = ord + n;
    short2 *pq = reinterpret_cast<short2 *>(sub + n);
    const double2 *Ag = h.D + (size_t)iq * nn;
    const double2 *G = h.Gd + (size_t)iq * 3 * nn;
    double *w = h.w + (size_t)iq * n;
    double *om = h.om + (size_t)iq * n;
    // Hermitise against rounding
    for (int k = tid; k < (int)nn; k += T) {
        const int i = k % n, j = k / n, i0 = min(i, j), j0 = max(i, j);  // the pair (i0, j0), i0 <= j0
        const double2 a = Ag[i0 + (size_t)n * j0], b = cconj(Ag[j0 + (size_t)n * i0]);
        const double2 sm = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
        A[k] = i <= j ? sm : cconj(sm);
    }
    __syncthreads();
    if (!cta_jacobi(n, A, V, w, rot, pq, red)) {
        if (tid == 0) atomicExch(h.status, (int32_t)kDevLinalg);
        return;
    }
    const double *qr = h.qirr + 3 * iq;
    if (tid == 0) {
        if (qr[0] * qr[0] + qr[1] * qr[1] + qr[2] * qr[2] < kSqTolD) {  // acoustic modes at Gamma
            for (int b = 0; b < n; ++b) key[b] = fabs(w[b]);
            stable_order(n, key, ord);
            for (int i = 0; i < min(3, n); ++i) w[ord[i]] = 0.0;
        }
        for (int b = 0; b < n; ++b) key[b] = negsqrt(w[b]);
        stable_order(n, key, ord);
        for (int b = 0; b < n; ++b) om[b] = negsqrt(w[ord[b]]);
    }
    __syncthreads();
    for (int k = tid; k < (int)nn; k += T) {
        const int b = k / n, r = k % n;
        E[k] = V[r + (size_t)n * ord[b]];
    }
    __syncthreads();
    // degenerate subspaces (contiguous, within lo_freqtol of the first): the velocity
    // operator along a fixed generic direction diagonalised inside each
    const double dir[3] = {1.0, 1.33, 1.45624623};
    for (int b0 = 0; b0 < n;) {
        int b1 = b0 + 1;
        while (b1 < n && fabs(om[b1] - om[b0]) < kFreqTolH) ++b1;
        const int k = b1 - b0;
        if (k > 1) {
            // GE[(d n + r) k + y] = sum_cc G_d[r, cc] E[b0 + y][cc]
            for (int t = tid; t < 3 * n * k; t += T) {
                const int y = t % k, dr = t / k, d = dr / n, r = dr % n;
                double2 gy = make_double2(0.0, 0.0);
                for (int cc = 0; cc < n; ++cc)
                    gy = cadd(gy, cmul(G[(size_t)d * nn + r + (size_t)n * cc], E[(size_t)(b0 + y) * n + cc]));
                GE[t] = gy;
            }
            __syncthreads();
            for (int xy = tid; xy < k * k; xy += T) {
                const int x = xy % k, y = xy / k;
                double2 sm = make_double2(0.0, 0.0);
                for (int d = 0; d < 3; ++d)
                    for (int r = 0; r < n; ++r)
                        sm = cadd(sm, cscale(cmul(cconj(E[(size_t)(b0 + x) * n + r]), GE[(size_t)(d * n + r) * k + y]),
                                             dir[d]));
                Pm[x + k * y] = sm;
            }
            __syncthreads();
            for (int xy = tid; xy < k * k; xy += T) {
                const int x = xy % k, y = xy / k;
                if (x <= y) {
                    const double2 a = Pm[x + k * y], b = cconj(Pm[y + k * x]);
                    const double2 sm = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
                    Pm[x + k * y] = sm;
                    Pm[y + k * x] = cconj(sm);
                }
            }
            __syncthreads();
            if (!cta_jacobi(k, Pm, U, pw, rot, pq, red)) {
                if (tid == 0) atomicExch(h.status, (int32_t)kDevLinalg);
                return;
            }
            if (tid == 0) stable_order(k, pw, ord);
            // the subspace's rows of E, before the rotation, into GE as scratch
            for (int t = tid; t < k * n; t += T) GE[t] = E[(size_t)b0 * n + t];
            __syncthreads();
            // sub = E_sub U[:, po]
            for (int t = tid; t < k * n; t += T) {
                const int y = t / n, r = t % n;
                double2 sm = make_double2(0.0, 0.0);
                for (int x = 0; x < k; ++x) sm = cadd(sm, cmul(GE[(size_t)x * n + r], U[x + k * ord[y]]));
                E[(size_t)(b0 + y) * n + r] = sm;
            }
            __syncthreads();
        }
        b0 = b1;
    }
    // Hellmann-Feynman values <e_b|dD/dk_d|e_b>: GE[(d n + r) n + b] = sum_cc G_d[r, cc] E[b][cc]
    for (int t = tid; t < 3 * (int)nn; t += T) {
        const int b = t % n, dr = t / n, d = dr / n, r = dr % n;
        double2 gy = make_double2(0.0, 0.0);
        for (int cc = 0; cc < n; ++cc) gy = cadd(gy, cmul(G[(size_t)d * nn + r + (size_t)n * cc], E[(size_t)b * n + cc]));
        GE[t] = gy;
    }
    __syncthreads();
    for (int bd = tid; bd < 3 * n; bd += T) {
        const int b = bd / 3, d = bd % 3;
        double2 sm = make_double2(0.0, 0.0);
        for (int r = 0; r < n; ++r) sm = cadd(sm, cmul(cconj(E[(size_t)b * n + r]), GE[(size_t)(d * n + r) * n + b]));
        hf[bd] = sm.x;
    }
    if (tid == 0) {  // a mode joins the first subspace holding a mode within lo_freqtol of it
        int nsub = 0;
        for (int b = 0; b < n; ++b) {
            sub[b] = -1;
            for (int a = 0; a < b && sub[b] < 0; ++a)
                if (fabs(om[a] - om[b]) < kFreqTolH) sub[b] = sub[a];
            if (sub[b] < 0) sub[b] = nsub++;
        }
    }
    __syncthreads();
    double *vel = h.vel + (size_t)iq * n * 3;
    for (int b = tid; b < n; b += T) {
        double mv[3] = {0.0, 0.0, 0.0};
        int cnt = 0;
        for (int a = 0; a < n; ++a)
            if (sub[a] == sub[b]) {
                ++cnt;
                for (int d = 0; d < 3; ++d) mv[d] += hf[a * 3 + d];
            }
        for (int d = 0; d < 3; ++d) vel[b * 3 + d] = om[b] > kFreqTolH ? (mv[d] / cnt) / (2.0 * om[b]) : 0.0;
        int l = 0;
        int32_t *dm = h.degen_mode + ((size_t)iq * n + b) * n;
        for (int b2 = 0; b2 < n; ++b2) {
            if (fabs(om[b] - om[b2]) < kFreqTolH) dm[l++] = b2 + 1;
        }
        for (int b2 = l; b2 < n; ++b2) dm[b2] = 0;
        h.degen[(size_t)iq * n + b] = l;
    }
    double2 *Eg = h.egv + (size_t)iq * nn;  // E[b * n + r]
    for (int k = tid; k < (int)nn; k += T) Eg[k] = E[k];
}

struct UnfoldDev {
    int na, nb, nfull, nirr;
    const int32_t *full_irr, *full_op, *irr_full;  // 1-based, signed operation
    const double *q_full;                          // [nfull*3]
    const double *op_cart;                         // [nop*9] column-major
    const int32_t *fmap;                           // [nop*na] 0-based
    const double *shift;                           // [nop*na*3]
    const double *om_i, *vel_i;
    const double2 *egv_i;
    const int32_t *deg_i, *dm_i;
    double *om, *vel;
    double2 *egv;
    int32_t *deg, *dm;
};

__global__ void k_unfold(UnfoldDev u) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int nb = u.nb, na = u.na;
    if (t >= (int64_t)u.nfull * nb * na) return;
    const int q = (int)(t / ((int64_t)nb * na)), rem = (int)(t % ((int64_t)nb * na));
    const int b = rem / na, a2 = rem % na;
    const int i = u.full_irr[q] - 1, iop = u.full_op[q], o = abs(iop) - 1;
    const double *m = u.op_cart + 9 * o;
    const double *qi = u.q_full + 3 * (u.irr_full[i] - 1);
    if (a2 == 0) {
        u.om[(size_t)q * nb + b] = u.om_i[(size_t)i * nb + b];
        u.deg[(size_t)q * nb + b] = u.deg_i[(size_t)i * nb + b];
        for (int c = 0; c < nb; ++c) u.dm[((size_t)q * nb + b) * nb + c] = u.dm_i[((size_t)i * nb + b) * nb + c];
        const double *v = u.vel_i + ((size_t)i * nb + b) * 3;
        const double sg = iop > 0 ? 1.0 : -1.0;
        for (int d = 0; d < 3; ++d)
            u.vel[((size_t)q * nb + b) * 3 + d] = sg * (m[d] * v[0] + m[d + 3] * v[1] + m[d + 6] * v[2]);
    }
    const int a1 = u.fmap[o * na + a2];
    const double *v0 = u.shift + ((size_t)o * na + a2) * 3;
    const double arg = -(v0[0] * qi[0] + v0[1] * qi[1] + v0[2] * qi[2]) * kTwoPiD;
    double sn, cs;
    sincos(arg, &sn, &cs);
    const double2 ph = make_double2(cs, sn);
    const double2 *e = u.egv_i + ((size_t)i * nb + b) * nb + 3 * a2;
    for (int x = 0; x < 3; ++x) {
        double2 s = make_double2(0.0, 0.0);
        for (int y = 0; y < 3; ++y) s = cadd(s, cscale(e[y], m[x + 3 * y]));
        s = cmul(s, ph);
        if (iop < 0) s = cconj(s);
        u.egv[((size_t)q * nb + b) * nb + 3 * a1 + x] = s;
    }
}

// Device buffers of one call, from the library's memory pool on the legacy stream (a pool
// keeps the memory between calls, where cudaMalloc and cudaFree cost tens of microseconds
// each for the 30-odd buffers of the stage).
template <typename T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    ~DBuf() {
        if (p) cudaFreeAsync(p, 0);
    }
    cudaError_t alloc(size_t count) {
        n = count;
        if (!count) return cudaSuccess;
        cudaMemPool_t pool = shared_device_pool(dev_of_call());
        return pool ? cudaMallocFromPoolAsync(reinterpret_cast<void **>(&p), sizeof(T) * count, pool, 0)
                    : cudaMalloc(&p, sizeof(T) * count);
    }
    cudaError_t up(const T *src, size_t count) {
        cudaError_t e = alloc(count);
        if (e != cudaSuccess || !count) return e;
        return cudaMemcpyAsync(p, src, sizeof(T) * count, cudaMemcpyHostToDevice, 0);
    }
    static int dev_of_call() {
        int d = 0;
        cudaGetDevice(&d);
        return d;
    }
};

}  // namespace

int build_phonons_device(const Crystal &c, const FC2 &fc, const QMesh &qp, int device, Phonons &ph,
                         std::vector<double> &irr_dyngrad) {
    const int na = c.na, nb = 3 * na, ni = qp.n_irr, nf = qp.n_full, nop = (int)c.ops.size();
    if (nb > kMaxModes) return set_error(kErrParam, "device harmonic stage: at most 128 modes");
    PhaseTimer pt("harmonic stage (device)");
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return set_error(kErrDevice, "device harmonic stage: cannot select the device");
    }
    // pairs grouped by atom pair, file order inside
    std::vector<int32_t> pptr((size_t)na * na + 1, 0);
    for (const auto &p : fc.pairs) ++pptr[(size_t)p.a1 * na + p.a2 + 1];
    for (size_t k = 1; k < pptr.size(); ++k) pptr[k] += pptr[k - 1];
    std::vector<int32_t> fill(pptr.begin(), pptr.end() - 1);
    std::vector<double> lv(fc.pairs.size() * 3), mm(fc.pairs.size() * 9);
    for (const auto &p : fc.pairs) {
        const int at = fill[(size_t)p.a1 * na + p.a2]++;
        for (int d = 0; d < 3; ++d) lv[(size_t)at * 3 + d] = p.lv[d];
        for (int e = 0; e < 9; ++e) mm[(size_t)at * 9 + e] = p.m[e];
    }
    std::vector<double> qirr((size_t)ni * 3), rc((size_t)na * 3), G((size_t)fc.G.size() * 3);
    for (int i = 0; i < ni; ++i)
        for (int d = 0; d < 3; ++d) qirr[(size_t)i * 3 + d] = qp.q_full[qp.irr_full[i] - 1][d];
    for (int a = 0; a < na; ++a)
        for (int d = 0; d < 3; ++d) rc[(size_t)a * 3 + d] = c.rcart[a][d];
    for (size_t g = 0; g < fc.G.size(); ++g)
        for (int d = 0; d < 3; ++d) G[g * 3 + d] = fc.G[g][d];
    std::vector<int32_t> fmap;
    std::vector<double> shift;
    int st = op_atom_maps(c, fmap, shift);
    if (st) return st;
    std::vector<double> opc((size_t)nop * 9), qf((size_t)nf * 3);
    for (int o = 0; o < nop; ++o) std::memcpy(&opc[(size_t)o * 9], c.ops[o].m.a, sizeof(double) * 9);
    for (int q = 0; q < nf; ++q)
        for (int d = 0; d < 3; ++d) qf[(size_t)q * 3 + d] = qp.q_full[q][d];

    pt.mark("host tables");
    const bool polar = fc.polar == 3;
    const int np2 = na * (na + 1) / 2;
    DBuf<int32_t> d_pptr, d_status, d_deg, d_dm, d_degf, d_dmf, d_fmap, d_fi, d_fo, d_if;
    DBuf<double> d_lv, d_m, d_ism, d_G, d_eps, d_Z, d_Zon, d_rc, d_q, d_w, d_om, d_vel, d_omf, d_velf, d_opc, d_shift,
        d_qf;
    DBuf<double2> d_dl, d_P, d_PG, d_D, d_Gd, d_V, d_S, d_egv, d_egvf;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    chk(d_pptr.up(pptr.data(), pptr.size()));
    chk(d_lv.up(lv.data(), lv.size()));
    chk(d_m.up(mm.data(), mm.size()));
    chk(d_ism.up(c.invsqrtmass.data(), na));
    chk(d_q.up(qirr.data(), qirr.size()));
    if (polar) {
        chk(d_G.up(G.data(), G.size()));
        chk(d_eps.up(fc.eps.a, 9));
        chk(d_Z.up(fc.Z.data(), fc.Z.size()));
        chk(d_Zon.up(fc.Zonsite.data(), fc.Zonsite.size()));
        chk(d_rc.up(rc.data(), rc.size()));
        chk(d_dl.alloc((size_t)ni * np2 * 36));
        chk(d_P.alloc((size_t)ni * 9 * na * na));
        chk(d_PG.alloc((size_t)ni * 27 * na * na));
    }
    chk(d_D.alloc((size_t)ni * nb * nb));
    chk(d_Gd.alloc((size_t)ni * 3 * nb * nb));
    chk(d_V.alloc((size_t)ni * nb * nb));
    chk(d_S.alloc((size_t)ni * (2 * nb * nb + nb)));
    chk(d_w.alloc((size_t)ni * nb));
    chk(d_om.alloc((size_t)ni * nb));
    chk(d_egv.alloc((size_t)ni * nb * nb));
    chk(d_vel.alloc((size_t)ni * nb * 3));
    chk(d_deg.alloc((size_t)ni * nb));
    chk(d_dm.alloc((size_t)ni * nb * nb));
    chk(d_status.alloc(1));
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("device harmonic stage: ") + cudaGetErrorString(e));
    chk(cudaMemset(d_status.p, 0, sizeof(int32_t)));
    pt.mark("allocations and uploads");
    HarmDev h;
    std::memset(&h, 0, sizeof h);
    h.na = na;
    h.nb = nb;
    h.nirr = ni;
    h.nfull = nf;
    h.nop = nop;
    h.pair_ptr = d_pptr.p;
    h.lv = d_lv.p;
    h.m = d_m.p;
    h.ism = d_ism.p;
    h.polar = fc.polar;
    h.nG = polar ? (int)fc.G.size() : 0;
    h.G = d_G.p;
    h.eps = polar ? d_eps.p : nullptr;
    h.Z = d_Z.p;
    h.Zon = d_Zon.p;
    h.rcart = d_rc.p;
    h.lambda = fc.lambda;
    h.volume = c.volume;
    h.qirr = d_q.p;
    h.dl = d_dl.p;
    h.P = d_P.p;
    h.PG = d_PG.p;
    h.D = d_D.p;
    h.Gd = d_Gd.p;
    h.V = d_V.p;
    h.S = d_S.p;
    h.w = d_w.p;
    h.om = d_om.p;
    h.egv = d_egv.p;
    h.vel = d_vel.p;
    h.degen = d_deg.p;
    h.degen_mode = d_dm.p;
    h.status = d_status.p;
    if (polar) k_longrange<<<ni, 256>>>(h);
    k_dynmat<<<ni, 256>>>(h);
    chk(cudaGetLastError());
    // the gradient at the irreducible points is an output (off-diagonal kappa)
    std::vector<double2> gd((size_t)ni * 3 * nb * nb);
    chk(cudaMemcpy(gd.data(), d_Gd.p, sizeof(double2) * gd.size(), cudaMemcpyDeviceToHost));
    if (nb <= kEigCtaModes) {
        const size_t sm = eigen_cta_smem(nb);
        chk(cudaFuncSetAttribute(k_eigen_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        if (e == cudaSuccess) k_eigen_cta<<<ni, kEigCtaThreads, sm>>>(h);
    } else {
        k_eigen<<<(ni + kEigWarps - 1) / kEigWarps, 32 * kEigWarps>>>(h);
    }
    chk(cudaGetLastError());
    int32_t dst = 0;
    chk(cudaMemcpy(&dst, d_status.p, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("device harmonic stage: ") + cudaGetErrorString(e));
    if (dst) return set_error(kErrLinalg, "device harmonic stage: Jacobi eigensolver did not converge");
    pt.mark("D(q), dD/dq, eigenvectors");
    irr_dyngrad.assign((size_t)ni * 3 * nb * nb * 2, 0.0);
    std::memcpy(irr_dyngrad.data(), gd.data(), sizeof(double) * irr_dyngrad.size());
    // unfold onto the mesh
    std::vector<int32_t> fi(qp.full_irr.begin(), qp.full_irr.end()), fo(qp.full_op.begin(), qp.full_op.end()),
        ifu(qp.irr_full.begin(), qp.irr_full.end());
    chk(d_fi.up(fi.data(), fi.size()));
    chk(d_fo.up(fo.data(), fo.size()));
    chk(d_if.up(ifu.data(), ifu.size()));
    chk(d_qf.up(qf.data(), qf.size()));
    chk(d_opc.up(opc.data(), opc.size()));
    chk(d_fmap.up(fmap.data(), fmap.size()));
    chk(d_shift.up(shift.data(), shift.size()));
    chk(d_omf.alloc((size_t)nf * nb));
    chk(d_velf.alloc((size_t)nf * nb * 3));
    chk(d_egvf.alloc((size_t)nf * nb * nb));
    chk(d_degf.alloc((size_t)nf * nb));
    chk(d_dmf.alloc((size_t)nf * nb * nb));
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("device harmonic stage: ") + cudaGetErrorString(e));
    UnfoldDev u;
    u.na = na;
    u.nb = nb;
    u.nfull = nf;
    u.nirr = ni;
    u.full_irr = d_fi.p;
    u.full_op = d_fo.p;
    u.irr_full = d_if.p;
    u.q_full = d_qf.p;
    u.op_cart = d_opc.p;
    u.fmap = d_fmap.p;
    u.shift = d_shift.p;
    u.om_i = d_om.p;
    u.vel_i = d_vel.p;
    u.egv_i = d_egv.p;
    u.deg_i = d_deg.p;
    u.dm_i = d_dm.p;
    u.om = d_omf.p;
    u.vel = d_velf.p;
    u.egv = d_egvf.p;
    u.deg = d_degf.p;
    u.dm = d_dmf.p;
    pt.mark("unfold uploads");
    const int64_t total = (int64_t)nf * nb * na;
    k_unfold<<<(unsigned)((total + 255) / 256), 256>>>(u);
    chk(cudaGetLastError());
    chk(cudaStreamSynchronize(0));
    pt.mark("unfold");
    ph.n_mode = nb;
    ph.omega.resize((size_t)nf * nb);
    ph.vel.resize((size_t)nf * nb * 3);
    ph.egv.resize((size_t)nf * nb * nb * 2);
    ph.degen.resize((size_t)nf * nb);
    ph.degen_mode.resize((size_t)nf * nb * nb);
    chk(cudaMemcpy(ph.omega.data(), d_omf.p, sizeof(double) * ph.omega.size(), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(ph.vel.data(), d_velf.p, sizeof(double) * ph.vel.size(), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(ph.egv.data(), d_egvf.p, sizeof(double) * ph.egv.size(), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(ph.degen.data(), d_degf.p, sizeof(int32_t) * ph.degen.size(), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(ph.degen_mode.data(), d_dmf.p, sizeof(int32_t) * ph.degen_mode.size(), cudaMemcpyDeviceToHost));
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("device harmonic stage: ") + cudaGetErrorString(e));
    pt.mark("downloads");
    return kOk;
}

}  // namespace tdg
