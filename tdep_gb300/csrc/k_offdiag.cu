// Off-diagonal (coherence) thermal conductivity, get_kappa_offdiag (kappa.f90:77-306).
//
// One CTA per irreducible point. The reference forms, per little-group operation, the
// n^2 x n^2 matrix sum_op conj(egw(:,i)) (x) egw(:,ii) (kappa.f90:171-194) and multiplies it
// by the flattened dD/dq (kappa.f90:200); that product is the sandwich
// egw^H (dPhi/dq) egw with egw = T_op E scaled by m^-1/2 / sqrt(2 w), so the CTA computes it
// as two n x n products per direction: H = G_x egw and V_x += egw^H H, G the mass-weighted
// gradient (the m^-1/2 factors of egw and the m^1/2 factors of the reference's flattened
// gradient cancel). The averaged velocities are chopped and reduced to their real parts
// (kappa.f90:203-213), and each mode pair (j != k) adds
// w_jk v_jk v_jk^T, w_jk = tau_jk f0_jk pref (kappa.f90:246-283); the star rotation
// (kappa.f90:221-231) is linear in v v^T and is applied to the per-point sum on the host.
// FP64 throughout; the work is O(n_irr * |G_q| * 6 n^3), small next to the scattering rates.
// Up to kOffdiagSmemModes modes the operations of a point are spread over CTAs: one CTA per
// (point, operation) forms that operation's three sandwiches (k_offdiag_ops), and one CTA
// per point adds them up in operation order and finishes (k_offdiag_sum). With one CTA per
// point, the points of large little groups (48 operations at Gamma of a cubic cell) set the
// kernel's length on GB300's FP64 pipe.
#include "dev_common.cuh"
#include "tdg_internal.cuh"

namespace tdg {
namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// egw = T_op E (operation o of point q): rows of atom a2 rotated onto atom fmap(a2) with the
// phase exp(-2 pi i v0.q) (type_symmetryoperation.f90:281-289), then scaled by 1/sqrt(2 w).
__device__ void offdiag_egw(const OffdiagArgs &a, int q, int o, double2 *egw) {
    const int n = a.n, nn = n * n;
    const int f = a.irr_full[q];
    const double2 *E = a.egv + (size_t)f * nn;
    const double *om = a.omega + (size_t)f * n;
    const double *qv = a.q_full + (size_t)f * 3;
    const double *R = a.op_cart + 9 * o;
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
        const int b = i / n, rr = i % n, a2 = rr / 3, al = rr % 3;
        const int a1 = a.fmap[o * a.na + a2];
        const double *v0 = a.shift + ((size_t)o * a.na + a2) * 3;
        double sn, cs;
        sincos(-kTwoPiD * (v0[0] * qv[0] + v0[1] * qv[1] + v0[2] * qv[2]), &sn, &cs);
        const double2 *e = E + (size_t)b * n + a2 * 3;
        double2 s = make_double2(0.0, 0.0);
        for (int be = 0; be < 3; ++be) {
            s.x += R[al + 3 * be] * e[be].x;
            s.y += R[al + 3 * be] * e[be].y;
        }
        s = cmul(s, make_double2(cs, sn));
        const double sc = om[b] > kFreqTolD ? 1.0 / sqrt(2.0 * om[b]) : 0.0;
        egw[(size_t)b * n + a1 * 3 + al] = make_double2(s.x * sc, s.y * sc);
    }
}

// V_x (+)= egw^H G_x egw for x = 0..2 (H = G_x egw in between); V starts from its current
// values (accumulate) or from zero.
__device__ void offdiag_sandwich(const OffdiagArgs &a, int q, const double2 *egw, double2 *H, double2 *V,
                                 bool accumulate) {
    const int n = a.n, nn = n * n;
    const double2 *G = a.grad + (size_t)q * 3 * nn;
    for (int x = 0; x < 3; ++x) {
        const double2 *Gx = G + (size_t)x * nn;
        for (int i = threadIdx.x; i < nn; i += blockDim.x) {
            const int b = i / n, r = i % n;
            double2 s = make_double2(0.0, 0.0);
            for (int c = 0; c < n; ++c) {
                const double2 g = Gx[(size_t)c * n + r], w = egw[(size_t)b * n + c];
                s.x += g.x * w.x - g.y * w.y;
                s.y += g.x * w.y + g.y * w.x;
            }
            H[i] = s;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nn; i += blockDim.x) {
            const int j = i / n, kk = i % n;
            double2 s = accumulate ? V[(size_t)x * nn + i] : make_double2(0.0, 0.0);
            for (int r = 0; r < n; ++r) {
                const double2 t = cmulc(egw[(size_t)j * n + r], H[(size_t)kk * n + r]);
                s.x += t.x;
                s.y += t.y;
            }
            V[(size_t)x * nn + i] = s;
        }
        __syncthreads();
    }
}

// The averaged velocities of point q from V (sum over its nop operations), chopped, and the
// point's sum of w v v^T over mode pairs into S[q].
__device__ void offdiag_finish(const OffdiagArgs &a, int q, int nop, const double2 *V) {
    const int n = a.n, nn = n * n;
    const int f = a.irr_full[q];
    const double *om = a.omega + (size_t)f * n;
    const double inv = 1.0 / (double)nop;
    const double *lw = a.lw + (size_t)q * n, *cv = a.cv + (size_t)q * n;
    const double pref = a.irr_weight[q] * a.inv_volume;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
        const int j = i / n, k = i % n;
        double v[3];
        for (int x = 0; x < 3; ++x) {
            const double re = V[(size_t)x * nn + i].x * inv;
            v[x] = fabs(re) < a.chop_tol ? 0.0 : re;
        }
        if (a.vel)
            for (int x = 0; x < 3; ++x) a.vel[((size_t)q * nn + i) * 3 + x] = v[x];
        if (j == k || om[j] < kFreqTolD || om[k] < kFreqTolD || lw[j] < kFreqTolD || lw[k] < kFreqTolD) continue;
        const double t = lw[j] + lw[k], d = om[j] - om[k];
        const double w = t / (t * t + d * d) * (0.5 * (cv[j] + cv[k])) * pref;
        for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) acc[x + 3 * y] += w * v[x] * v[y];
    }
    __shared__ double red[9][8];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    for (int c = 0; c < 9; ++c) {
        double v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[c][wp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        double v = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) v += red[threadIdx.x][i];
        a.S[(size_t)q * 9 + threadIdx.x] = v;
    }
}

// Large cells: one CTA per point, its operations in turn, work arrays in global memory.
__global__ void __launch_bounds__(256) k_offdiag(OffdiagArgs a) {
    const int q = blockIdx.x, nn = a.n * a.n;
    double2 *egw = a.work + (size_t)q * 5 * nn;
    double2 *H = egw + nn, *V = H + nn;
    for (int i = threadIdx.x; i < 3 * nn; i += blockDim.x) V[i] = make_double2(0.0, 0.0);
    const int nop = a.irr_nop[q];
    for (int k = 0; k < nop; ++k) {
        __syncthreads();
        offdiag_egw(a, q, a.irr_ops[(size_t)q * a.n_op + k], egw);
        __syncthreads();
        offdiag_sandwich(a, q, egw, H, V, true);
    }
    __syncthreads();
    offdiag_finish(a, q, nop, V);
}

// One CTA per (point, operation) item: the operation's three sandwiches into part[item].
__global__ void __launch_bounds__(256) k_offdiag_ops(OffdiagArgs a) {
    extern __shared__ double2 sm_offdiag[];
    const int2 it = a.items[blockIdx.x];  // (point, index of the operation in its little group)
    const int nn = a.n * a.n;
    double2 *egw = sm_offdiag, *H = egw + nn;
    offdiag_egw(a, it.x, a.irr_ops[(size_t)it.x * a.n_op + it.y], egw);
    __syncthreads();
    offdiag_sandwich(a, it.x, egw, H, a.part + (size_t)blockIdx.x * 3 * nn, false);
}

// One CTA per point: V = the sum of its items' parts in operation order, then the finish.
__global__ void __launch_bounds__(256) k_offdiag_sum(OffdiagArgs a) {
    extern __shared__ double2 sm_offdiag[];
    const int q = blockIdx.x, nn = a.n * a.n;
    const int i0 = a.item_ptr[q], nop = a.item_ptr[q + 1] - i0;
    double2 *V = sm_offdiag;
    for (int i = threadIdx.x; i < 3 * nn; i += blockDim.x) {
        double2 s = make_double2(0.0, 0.0);
        for (int k = 0; k < nop; ++k) {
            const double2 p = a.part[(size_t)(i0 + k) * 3 * nn + i];
            s.x += p.x;
            s.y += p.y;
        }
        V[i] = s;
    }
    __syncthreads();
    offdiag_finish(a, q, nop, V);
}

}  // namespace

size_t offdiag_work_elems(int n, int n_irr, int n_items) {
    return n <= kOffdiagSmemModes ? (size_t)n_items * 3 * n * n : (size_t)n_irr * 5 * n * n;
}

cudaError_t launch_offdiag(const OffdiagArgs &a, int n_irr, int n_items, cudaStream_t s) {
    if (n_irr <= 0) return cudaSuccess;
    const size_t nn = (size_t)a.n * a.n;
    if (a.n > kOffdiagSmemModes) {
        if (!a.work) return cudaErrorInvalidValue;
        k_offdiag<<<n_irr, 256, 0, s>>>(a);
        return cudaGetLastError();
    }
    if (!a.items || !a.item_ptr || !a.part || n_items < n_irr) return cudaErrorInvalidValue;
    k_offdiag_ops<<<n_items, 256, 2 * nn * sizeof(double2), s>>>(a);
    k_offdiag_sum<<<n_irr, 256, 3 * nn * sizeof(double2), s>>>(a);
    return cudaGetLastError();
}

}  // namespace tdg
