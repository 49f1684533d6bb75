// Adjoint of the iterative BTE solution (kappa.f90:326-495) with respect to the three-phonon
// scattering matrix: the device parts of tdg_kappa_iter_vjp.
//
// At the converged fixed point F = G(-Q^-1 X T F, F0) (T the foldout of kappa.f90:382-404,
// X = Xi, Q = diag(qs), G the in-place degeneracy averaging and F0 addition of :418-435,
// whose part linear in the update is the degeneracy average D), the cotangent lambda of F
// solves lambda = kbar - T^T X^T Q^-1 D lambda; the scattering matrix then receives the
// rank-3 cotangent W(r, c) = -sum_d z(r, d) (T F)(c, d) with z = Q^-1 D lambda, which is
// mapped back through the row symmetrisations (symmetrize_scatmat, scattering.f90:296-357,
// then symmetrize_and_distribute of the three-phonon terms, scattering_threephonon.f90:
// 143-205, both adjoint: the forward pass applied them in the other order) onto the raw
// three-phonon row terms that the adjoint kernel of k_threephonon consumes.
#include <cuda_runtime.h>

#include "dev_common.cuh"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

// y_part[k][c][d] = sum over the k-th range of rows of X[r][c] z[r][d]: one thread per column
// (coalesced row reads), the rows split over gridDim.y ranges summed in a fixed order by
// k_xit_reduce.
__global__ void k_xit_part(const double *xi, int32_t n_row, int64_t n_col, const double *z, int32_t rows_per,
                           double *part) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int r0 = blockIdx.y * rows_per, r1 = min(n_row, r0 + rows_per);
    if (c >= n_col) return;
    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
    for (int r = r0; r < r1; ++r) {
        const double x = xi[(int64_t)r * n_col + c];
        y0 = fma(x, z[3 * r], y0);
        y1 = fma(x, z[3 * r + 1], y1);
        y2 = fma(x, z[3 * r + 2], y2);
    }
    double *o = part + ((int64_t)blockIdx.y * n_col + c) * 3;
    o[0] = y0;
    o[1] = y1;
    o[2] = y2;
}

__global__ void k_xit_reduce(const double *part, int32_t n_part, int64_t n_col, double *y) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * n_col) return;
    double s = 0.0;
    for (int k = 0; k < n_part; ++k) s += part[(int64_t)k * 3 * n_col + e];
    y[e] = s;
}

// out[r][d] = sum_c X[r][c] f[c][d] in FP64, one warp per row, the lanes' partial sums added
// in a fixed order.
__global__ void k_xi_rowdot(const double *xi, int32_t n_row, int64_t n_col, const double *f, double *out) {
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= n_row) return;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    const double *xr = xi + (int64_t)r * n_col;
    for (int64_t c = lane; c < n_col; c += 32) {
        const double x = xr[c];
        s0 = fma(x, f[3 * c], s0);
        s1 = fma(x, f[3 * c + 1], s1);
        s2 = fma(x, f[3 * c + 2], s2);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, o);
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
        s2 += __shfl_down_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) {
        out[3 * r] = s0;
        out[3 * r + 1] = s1;
        out[3 * r + 2] = s2;
    }
}

// W(r, c) = -z(r) . f(c) for every entry of the scattering matrix.
__global__ void k_xibar_fill(int32_t n_row, int64_t n_col, const double *z, const double *f, double *w) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (c >= n_col) return;
    w[(int64_t)r * n_col + c] = -(z[3 * r] * f[3 * c] + z[3 * r + 1] * f[3 * c + 1] + z[3 * r + 2] * f[3 * c + 2]);
}

// The two row symmetrisations' adjoints on tiles of whole orbits (the layout of k_sym_tile).
// Forward, per orbit and mode: symmetrize_and_distribute sets every image to the
// multiplicity-weighted mean of the images whose raw value is positive (when the row sampled
// the orbit's representative and at least one is); symmetrize_scatmat then sets every image
// to the multiplicity-weighted mean of all images. Adjoint, in the other order: image p
// receives mult_p / cnt times the sum of the images' cotangents, then, where the first
// average applied, mult_p / nn times that sum if its raw value was positive and 0 otherwise.
__global__ void __launch_bounds__(256) k_sym_tile_adjoint(MeshDev m, OrbitDev o, const int32_t *row_q1,
                                                          const double *od_raw, double *w, const uint32_t *sbits) {
    extern __shared__ double adj_sm[];
    __shared__ int wsum[8];
    const int n = m.n_mode, T = o.tile_pts;
    const int r = blockIdx.y, q1 = row_q1[r];
    const int nop = m.irr_nop[q1];
    if (nop <= 1) return;  // every orbit is one point with count 1: both adjoints are the identity
    const int K = min(256, T / nop);
    const int kb = o.rep_ptr[q1], ke = o.rep_ptr[q1 + 1];
    const int k0 = kb + blockIdx.x * K;
    if (k0 >= ke) return;
    const int nk = min(K, ke - k0);
    double *vals = adj_sm;                                 // [T][n] cotangents
    uint32_t *pos = (uint32_t *)(vals + (size_t)T * n);    // [T][n] raw value > 0
    int *pts = (int *)(pos + (size_t)T * n);               // [T]
    int *pmu = pts + T;                                    // [T]
    int *off = pmu + T;                                    // [257]
    const int tid = threadIdx.x;
    const int nu_t = tid < nk ? o.nuniq[k0 + tid] : 0;
    int P = 0;
    const int my = block_exclusive_scan(nu_t, wsum, P);
    if (tid < nk) {
        off[tid] = my;
        const int32_t *im = o.img + (size_t)(k0 + tid) * m.n_op;
        const int32_t *mu = o.mult + (size_t)(k0 + tid) * m.n_op;
        for (int u = 0; u < nu_t; ++u) {
            pts[my + u] = im[u];
            pmu[my + u] = mu[u];
        }
    }
    if (tid == 0) off[nk] = P;
    __syncthreads();
    const int64_t ld = (int64_t)m.n_full * n;
    double *wr = w + (int64_t)r * ld;
    const double *rr = od_raw + (int64_t)r * ld;
    for (int e = tid; e < P * n; e += blockDim.x) {
        const int p = e / n, b2 = e - p * n;
        const int64_t at = (int64_t)pts[p] * n + b2;
        vals[e] = wr[at];
        pos[e] = __double_as_longlong(rr[at]) > 0 ? 1u : 0u;
    }
    __syncthreads();
    const uint32_t *bits = sbits + (size_t)r * ((m.n_full + 31) / 32);
    for (int it = tid; it < nk * n; it += blockDim.x) {
        const int t = it / n, b2 = it - t * n, k = k0 + t;
        const int p0 = off[t], p1 = off[t + 1];
        const int cnt = o.cnt[k];
        if (cnt) {  // symmetrize_scatmat
            double s = 0.0;
            for (int p = p0; p < p1; ++p) s += vals[p * n + b2];
            s *= o.rcp[cnt];
            for (int p = p0; p < p1; ++p) vals[p * n + b2] = s * (double)pmu[p];
        }
        const int q2 = o.rep[k];
        if ((bits[q2 >> 5] >> (q2 & 31)) & 1u) {  // symmetrize_and_distribute, where it applied
            int nn = 0;
            double s = 0.0;
            for (int p = p0; p < p1; ++p) {
                s += vals[p * n + b2];
                if (pos[p * n + b2]) nn += pmu[p];
            }
            if (nn) {
                s *= o.rcp[nn];
                for (int p = p0; p < p1; ++p) vals[p * n + b2] = pos[p * n + b2] ? s * (double)pmu[p] : 0.0;
            }
        }
    }
    __syncthreads();
    for (int e = tid; e < P * n; e += blockDim.x) {
        const int p = e / n, b2 = e - p * n;
        wr[(int64_t)pts[p] * n + b2] = vals[e];
    }
}

}  // namespace

int xit_parts(int32_t n_row) { return n_row < 8 ? 1 : 8; }

cudaError_t launch_xit_gemv(const double *xi, int32_t n_row, int64_t n_col, const double *z, double *part, double *y,
                            cudaStream_t s) {
    if (n_row <= 0 || n_col <= 0) return cudaSuccess;
    const int np = xit_parts(n_row);
    const int per = (n_row + np - 1) / np;
    dim3 grid((unsigned)((n_col + 255) / 256), (unsigned)np);
    k_xit_part<<<grid, 256, 0, s>>>(xi, n_row, n_col, z, per, part);
    k_xit_reduce<<<(unsigned)((3 * n_col + 255) / 256), 256, 0, s>>>(part, np, n_col, y);
    return cudaGetLastError();
}

cudaError_t launch_xi_rowdot(const double *xi, int32_t n_row, int64_t n_col, const double *f, double *out,
                             cudaStream_t s) {
    if (n_row <= 0) return cudaSuccess;
    k_xi_rowdot<<<(unsigned)((n_row + 7) / 8), 256, 0, s>>>(xi, n_row, n_col, f, out);
    return cudaGetLastError();
}

cudaError_t launch_xibar_fill(int32_t n_row, int64_t n_col, const double *z, const double *f, double *w,
                              cudaStream_t s) {
    if (n_row <= 0 || n_col <= 0) return cudaSuccess;
    dim3 grid((unsigned)((n_col + 255) / 256), (unsigned)n_row);
    k_xibar_fill<<<grid, 256, 0, s>>>(n_row, n_col, z, f, w);
    return cudaGetLastError();
}

cudaError_t launch_sym_tile_adjoint(const MeshDev &m, const OrbitDev &o, int32_t n_row, const int32_t *row_q1,
                                    const double *od_raw, double *w, const uint32_t *sbits, cudaStream_t s) {
    if (n_row <= 0 || o.max_tiles <= 0) return cudaSuccess;
    const int T = o.tile_pts, n = m.n_mode;
    const size_t sm = (sizeof(double) + sizeof(uint32_t)) * (size_t)T * n + sizeof(int) * (2 * (size_t)T + 257);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_sym_tile_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    dim3 grid((unsigned)o.max_tiles, (unsigned)n_row);
    k_sym_tile_adjoint<<<grid, 256, sm, s>>>(m, o, row_q1, od_raw, w, sbits);
    return cudaGetLastError();
}

}  // namespace tdg
