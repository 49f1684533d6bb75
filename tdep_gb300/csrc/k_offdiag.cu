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

__global__ void __launch_bounds__(256) k_offdiag(OffdiagArgs a) {
    extern __shared__ double2 sm_offdiag[];
    const int q = blockIdx.x, n = a.n, nn = n * n;
    double2 *egw = a.n <= kOffdiagSmemModes ? sm_offdiag : a.work + (size_t)q * 5 * nn;
    double2 *H = egw + nn, *V = H + nn;
    const int f = a.irr_full[q];
    const double2 *E = a.egv + (size_t)f * nn;
    const double2 *G = a.grad + (size_t)q * 3 * nn;
    const double *om = a.omega + (size_t)f * n;
    const double *qv = a.q_full + (size_t)f * 3;
    for (int i = threadIdx.x; i < 3 * nn; i += blockDim.x) V[i] = make_double2(0.0, 0.0);
    const int nop = a.irr_nop[q];
    for (int k = 0; k < nop; ++k) {
        const int o = a.irr_ops[(size_t)q * a.n_op + k];
        const double *R = a.op_cart + 9 * o;
        __syncthreads();
        // egw = T_op E: rows of atom a2 rotated onto atom fmap(a2) with the phase
        // exp(-2 pi i v0.q) (type_symmetryoperation.f90:281-289), then scaled
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
        __syncthreads();
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
                double2 s = V[(size_t)x * nn + i];
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
    __syncthreads();
    // velocities and the per-point sum of w v v^T over mode pairs
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

}  // namespace

size_t offdiag_work_elems(int n, int n_irr) { return n <= kOffdiagSmemModes ? 0 : (size_t)n_irr * 5 * n * n; }

cudaError_t launch_offdiag(const OffdiagArgs &a, int n_irr, cudaStream_t s) {
    if (n_irr <= 0) return cudaSuccess;
    const size_t smem = a.n <= kOffdiagSmemModes ? (size_t)5 * a.n * a.n * sizeof(double2) : 0;
    k_offdiag<<<n_irr, 256, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace tdg
