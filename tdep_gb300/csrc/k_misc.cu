// Isotope scattering, the two scattering-matrix symmetrisations and the BTE product.
#include <cuda_runtime.h>

#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr double kIsotopePrefactor = 3.141592653589793 / 4.0;
constexpr double kSqrt2PiInv = 0.398942280401433;
constexpr double kFreqTolD = 1E-9;

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

// symmetrize_scatmat (scattering.f90:296-357): one thread per (row, orbit, mode).
__global__ void k_sym_scatmat(MeshDev m, OrbitDev o, const int32_t *row_q1, double *xi) {
    const int n = m.n_mode;
    const int r = blockIdx.y;
    const int q1 = row_q1[r];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nrep = o.rep_ptr[q1 + 1] - o.rep_ptr[q1];
    if (i >= nrep * n) return;
    const int k = o.rep_ptr[q1] + i / n, b2 = i % n;
    const int cnt = o.cnt[k];
    if (cnt == 0) return;
    const int nu = o.nuniq[k];
    const int32_t *im = o.img + (size_t)k * m.n_op;
    const int32_t *mu = o.mult + (size_t)k * m.n_op;
    double *xr = xi + (int64_t)r * m.n_full * n;
    double buf = 0.0;
    int u = 0;
    for (; u + 4 <= nu; u += 4) {
        const double x0 = xr[(int64_t)im[u] * n + b2], x1 = xr[(int64_t)im[u + 1] * n + b2];
        const double x2 = xr[(int64_t)im[u + 2] * n + b2], x3 = xr[(int64_t)im[u + 3] * n + b2];
        for (int rep = 0; rep < mu[u]; ++rep) buf += x0;
        for (int rep = 0; rep < mu[u + 1]; ++rep) buf += x1;
        for (int rep = 0; rep < mu[u + 2]; ++rep) buf += x2;
        for (int rep = 0; rep < mu[u + 3]; ++rep) buf += x3;
    }
    for (; u < nu; ++u) {
        const double x = xr[(int64_t)im[u] * n + b2];
        for (int rep = 0; rep < mu[u]; ++rep) buf += x;
    }
    buf *= o.rcp[cnt];
    for (u = 0; u < nu; ++u) xr[(int64_t)im[u] * n + b2] = buf;
}

// K8: three dot products per row of Xi (kappa.f90:411-413, the lo_gemv calls).
// Xi streams from HBM once; F (3 x n_col) stays in L2.
__global__ void k_xi_gemv(const double *__restrict__ xi, int64_t n_col, const double *__restrict__ fbb,
                          double *buf) {
    __shared__ double sh[3][32];
    const int r = blockIdx.x;
    const double *row = xi + (int64_t)r * n_col;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    // four independent row loads in flight per thread before they are used
    const int64_t step = blockDim.x;
    int64_t j = threadIdx.x;
    for (; j + 3 * step < n_col; j += 4 * step) {
        double x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = __ldcs(row + j + u * step);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const double *f = fbb + (j + u * step) * 3;
            s0 = fma(x[u], __ldg(f), s0);
            s1 = fma(x[u], __ldg(f + 1), s1);
            s2 = fma(x[u], __ldg(f + 2), s2);
        }
    }
    for (; j < n_col; j += step) {
        const double x = __ldcs(row + j);
        const double *f = fbb + j * 3;
        s0 = fma(x, __ldg(f), s0);
        s1 = fma(x, __ldg(f + 1), s1);
        s2 = fma(x, __ldg(f + 2), s2);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, o);
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
        s2 += __shfl_down_sync(0xffffffffu, s2, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][w] = s0;
        sh[1][w] = s1;
        sh[2][w] = s2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x / 32); ++i) s += sh[threadIdx.x][i];
        buf[(int64_t)r * 3 + threadIdx.x] = s;
    }
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

cudaError_t launch_sym_scatmat(const MeshDev &m, const OrbitDev &o, int32_t n_row, const int32_t *row_q1, double *xi,
                               cudaStream_t s) {
    if (n_row <= 0 || o.max_rep <= 0) return cudaSuccess;
    dim3 grid((unsigned)(((int64_t)o.max_rep * m.n_mode + 127) / 128), (unsigned)n_row);
    k_sym_scatmat<<<grid, 128, 0, s>>>(m, o, row_q1, xi);
    return cudaGetLastError();
}

// foldout (kappa.f90:382-404): F of every full-mesh point from its irreducible point,
// Fbb(q, b) = sign(op) * R_|op| Fn(irr(q), b), one thread per (q, b).
__global__ void k_foldout(int32_t n_full, int32_t n_mode, const int32_t *full_op, const int32_t *full_irr,
                          const double *op_cart, const double *fn, double *fbb) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n_full * n_mode) return;
    const int iq = (int)(i / n_mode), b = (int)(i % n_mode);
    const int iop = full_op[iq];
    const double *m = op_cart + 9 * (abs(iop) - 1);
    const double *v = fn + ((int64_t)full_irr[iq] * n_mode + b) * 3;
    const double sg = iop > 0 ? 1.0 : -1.0;
    for (int d = 0; d < 3; ++d) fbb[i * 3 + d] = sg * (m[d] * v[0] + m[d + 3] * v[1] + m[d + 6] * v[2]);
}

cudaError_t launch_foldout(int32_t n_full, int32_t n_mode, const int32_t *full_op, const int32_t *full_irr,
                           const double *op_cart, const double *fn, double *fbb, cudaStream_t s) {
    const int64_t n = (int64_t)n_full * n_mode;
    if (n <= 0) return cudaSuccess;
    k_foldout<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n_full, n_mode, full_op, full_irr, op_cart, fn, fbb);
    return cudaGetLastError();
}

cudaError_t launch_xi_gemv(const double *xi, int32_t n_row, int64_t n_col, const double *fbb, double *buf,
                           int n_sm, cudaStream_t s) {
    (void)n_sm;
    if (n_row <= 0) return cudaSuccess;
    k_xi_gemv<<<n_row, 256, 0, s>>>(xi, n_col, fbb, buf);
    return cudaGetLastError();
}

}  // namespace tdg
