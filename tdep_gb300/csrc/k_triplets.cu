// K1: irreducible q-triplet and q-quartet enumeration on integer rotation tables.
//
// For every candidate (q1 irreducible, q2 from the Monte-Carlo sample of q1's rows):
//   q3 = -q1-q2 mod G                          (lo_fftgrid_helper.f90:136-163)
//   skip q3 < q2                               (scattering_threephonon.f90:75)
//   triplet_is_irreducible                     (scattering_threephonon.f90:319-448)
// The reference rotates fractional coordinates in floating point and rounds back to the
// grid; here every rotated index comes from a host-built table rot[op][q], so the whole
// enumeration is integer arithmetic and bit-exact.
// Two passes: count (accepted flag and number of equivalent triplets per candidate),
// exclusive scan, fill. Output order equals candidate order, so results are deterministic.
#include "tdg_internal.cuh"

namespace tdg {

namespace {

constexpr int kMaxOps = 192;

__device__ __forceinline__ void grid_coords(const MeshDev &m, int q, int &i, int &j, int &k) {
    const int n12 = m.grid[1] * m.grid[2];
    i = q / n12;
    j = (q / m.grid[2]) % m.grid[1];
    k = q % m.grid[2];
}

__device__ __forceinline__ int wrap(int x, int n) {
    x %= n;
    return x < 0 ? x + n : x;
}

// q3 = -q1-q2 (0-based full indices).
__device__ __forceinline__ int third_index(const MeshDev &m, int f1, int q2) {
    int i1, j1, k1, i2, j2, k2;
    grid_coords(m, f1, i1, j1, k1);
    grid_coords(m, q2, i2, j2, k2);
    const int i3 = wrap(-i1 - i2, m.grid[0]);
    const int j3 = wrap(-j1 - j2, m.grid[1]);
    const int k3 = wrap(-k1 - k2, m.grid[2]);
    return (i3 * m.grid[1] + j3) * m.grid[2] + k3;
}

// q4 = -q1-q2-q3.
__device__ __forceinline__ int fourth_index(const MeshDev &m, int f1, int q2, int q3) {
    int i1, j1, k1, i2, j2, k2, i3, j3, k3;
    grid_coords(m, f1, i1, j1, k1);
    grid_coords(m, q2, i2, j2, k2);
    grid_coords(m, q3, i3, j3, k3);
    const int i4 = wrap(-i1 - i2 - i3, m.grid[0]);
    const int j4 = wrap(-j1 - j2 - j3, m.grid[1]);
    const int k4 = wrap(-k1 - k2 - k3, m.grid[2]);
    return (i4 * m.grid[1] + j4) * m.grid[2] + k4;
}

// Returns -1 when the triplet is reducible, else the number of distinct equivalent
// triplets; when out != nullptr they are written in operation order (unsorted pairs).
__device__ int triplet_images(const MeshDev &m, int q1, int q2, int q3, int2 *out) {
    const int nop = m.irr_nop[q1];
    const int32_t *ops = m.irr_ops + (size_t)q1 * m.n_op;
    int a[kMaxOps], b[kMaxOps];
    bool isred = false;
    for (int j = 0; j < nop; ++j) {
        const int o = ops[j];
        const int x = m.rot[(size_t)o * m.n_full + q2];
        const int y = m.rot[(size_t)o * m.n_full + q3];
        if (x < 0 || y < 0) {
            a[j] = -1;
            b[j] = -1;
            continue;
        }
        a[j] = x;
        b[j] = y;
        if (min(x, y) > q2) isred = true;
    }
    if (isred) return -1;
    for (int j = 0; j < nop; ++j)
        if (a[j] < 0) {
            a[j] = q2;
            b[j] = q3;
        }
    int cnt = 0;
    for (int j = 0; j < nop; ++j) {
        const int lo = min(a[j], b[j]), hi = max(a[j], b[j]);
        bool uniq = true;
        for (int k = j + 1; k < nop; ++k)
            if (min(a[k], b[k]) == lo && max(a[k], b[k]) == hi) {
                uniq = false;
                break;
            }
        if (uniq) {
            if (out) out[cnt] = make_int2(a[j], b[j]);
            ++cnt;
        }
    }
    return cnt;
}

__device__ __forceinline__ void sort3(int &x, int &y, int &z) {
    if (x > y) { int t = x; x = y; y = t; }
    if (y > z) { int t = y; y = z; z = t; }
    if (x > y) { int t = x; x = y; y = t; }
}

// quartet_is_irreducible (scattering_fourphonon.f90:330-456). Off-grid operations keep
// their original (unsorted) triple replaced by (q2,q3,q4) while their sorted copy stays
// at the sentinel, exactly as the reference's two successive replacement tests do.
__device__ int quartet_images(const MeshDev &m, int q1, int q2, int q3, int q4, int4 *out) {
    const int nop = m.irr_nop[q1];
    const int32_t *ops = m.irr_ops + (size_t)q1 * m.n_op;
    int a[kMaxOps], b[kMaxOps], c[kMaxOps];
    bool isred = false;
    constexpr int kSentinel = -2147483647;
    for (int j = 0; j < nop; ++j) {
        const int o = ops[j];
        const int x = m.rot[(size_t)o * m.n_full + q2];
        const int y = m.rot[(size_t)o * m.n_full + q3];
        const int z = m.rot[(size_t)o * m.n_full + q4];
        if (x < 0 || y < 0 || z < 0) {
            a[j] = kSentinel;
            b[j] = kSentinel;
            c[j] = kSentinel;
            continue;
        }
        a[j] = x;
        b[j] = y;
        c[j] = z;
        int s0 = x, s1 = y, s2 = z;
        sort3(s0, s1, s2);
        if (s0 > q2 || s1 > q3) isred = true;
    }
    if (isred) return -1;
    int cnt = 0;
    for (int j = 0; j < nop; ++j) {
        int s0 = a[j], s1 = b[j], s2 = c[j];
        if (a[j] != kSentinel) sort3(s0, s1, s2);
        bool uniq = true;
        for (int k = j + 1; k < nop; ++k) {
            int t0 = a[k], t1 = b[k], t2 = c[k];
            if (a[k] != kSentinel) sort3(t0, t1, t2);
            if (t0 == s0 && t1 == s1 && t2 == s2) {
                uniq = false;
                break;
            }
        }
        if (uniq) {
            if (out) {
                if (a[j] == kSentinel)
                    out[cnt] = make_int4(q2, q3, q4, 0);
                else
                    out[cnt] = make_int4(a[j], b[j], c[j], 0);
            }
            ++cnt;
        }
    }
    return cnt;
}

__global__ void k_triplet_count(MeshDev m, const int4 *cand, int32_t n_cand, int32_t *n_trip, int32_t *n_red,
                                int32_t *status) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cand) return;
    const int q1 = cand[c].x, q2 = cand[c].y;
    int nt = 0, nr = 0;
    if (q1 < 0 || q1 >= m.n_irr || q2 < 0 || q2 >= m.n_full || m.irr_nop[q1] > kMaxOps) {
        atomicCAS(status, kDevOk, kDevBadIndex);
    } else {
        const int q3 = third_index(m, m.irr_full[q1], q2);
        if (q3 >= q2) {
            const int k = triplet_images(m, q1, q2, q3, nullptr);
            if (k >= 0) {
                nt = 1;
                nr = k;
            }
        }
    }
    n_trip[c] = nt;
    n_red[c] = nr;
}

__global__ void k_triplet_fill(MeshDev m, const int4 *cand, int32_t n_cand, const int32_t *trip_off,
                               const int32_t *red_off, TripletRec *trip, int2 *red) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cand) return;
    if (trip_off[c + 1] == trip_off[c]) return;
    const int q1 = cand[c].x, q2 = cand[c].y;
    const int q3 = third_index(m, m.irr_full[q1], q2);
    const int k = triplet_images(m, q1, q2, q3, red + red_off[c]);
    TripletRec r;
    r.q1 = q1;
    r.q2 = q2;
    r.q3 = q3;
    r.cand = cand[c].z;
    r.red_off = red_off[c];
    r.red_cnt = k;
    trip[trip_off[c]] = r;
}

__global__ void k_quartet_count(MeshDev m, const int4 *cand, int32_t n_cand, int32_t *n_q, int32_t *n_red,
                                int32_t *status) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cand) return;
    const int q1 = cand[c].x, q2 = cand[c].y, q3 = cand[c].z;
    int nq = 0, nr = 0;
    if (q1 < 0 || q1 >= m.n_irr || q2 < 0 || q2 >= m.n_full || q3 < 0 || q3 >= m.n_full ||
        m.irr_nop[q1] > kMaxOps) {
        atomicCAS(status, kDevOk, kDevBadIndex);
    } else if (q3 >= q2) {
        const int q4 = fourth_index(m, m.irr_full[q1], q2, q3);
        if (q4 >= q3) {
            const int k = quartet_images(m, q1, q2, q3, q4, nullptr);
            if (k >= 0) {
                nq = 1;
                nr = k;
            }
        }
    }
    n_q[c] = nq;
    n_red[c] = nr;
}

__global__ void k_quartet_fill(MeshDev m, const int4 *cand, int32_t n_cand, const int32_t *q_off,
                               const int32_t *red_off, QuartetRec *quart, int4 *red) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cand) return;
    if (q_off[c + 1] == q_off[c]) return;
    const int q1 = cand[c].x, q2 = cand[c].y, q3 = cand[c].z;
    const int q4 = fourth_index(m, m.irr_full[q1], q2, q3);
    const int k = quartet_images(m, q1, q2, q3, q4, red + red_off[c]);
    QuartetRec r;
    r.q1 = q1;
    r.q2 = q2;
    r.q3 = q3;
    r.q4 = q4;
    r.cand = cand[c].w;
    r.red_off = red_off[c];
    r.red_cnt = k;
    r.pad = 0;
    quart[q_off[c]] = r;
}

// ---- exclusive scan: per-block scan of 2048 elements, scan of block sums, add ----
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 2 * kScanThreads;

__device__ int32_t block_exclusive_scan(int32_t v, int32_t *sh, int32_t &total) {
    // Hillis-Steele inclusive scan in shared memory, converted to exclusive.
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int off = 1; off < blockDim.x; off <<= 1) {
        const int32_t x = (t >= off) ? sh[t - off] : 0;
        __syncthreads();
        sh[t] += x;
        __syncthreads();
    }
    total = sh[blockDim.x - 1];
    const int32_t incl = sh[t];
    __syncthreads();
    return incl - v;
}

__global__ void k_scan_blocks(const int32_t *in, int32_t *out, int32_t n, int32_t *block_sums) {
    __shared__ int32_t sh[kScanThreads];
    const int64_t base = (int64_t)blockIdx.x * kScanItems;
    const int64_t i0 = base + 2 * threadIdx.x;
    const int32_t a = i0 < n ? in[i0] : 0;
    const int32_t b = i0 + 1 < n ? in[i0 + 1] : 0;
    int32_t total;
    const int32_t ex = block_exclusive_scan(a + b, sh, total);
    if (i0 < n) out[i0] = ex;
    if (i0 + 1 < n) out[i0 + 1] = ex + a;
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int32_t *sums, int32_t nb, int32_t *grand_total) {
    __shared__ int32_t sh[kScanThreads];
    int32_t carry = 0;
    for (int32_t c = 0; c < nb; c += kScanThreads) {
        const int32_t i = c + threadIdx.x;
        const int32_t v = i < nb ? sums[i] : 0;
        int32_t total;
        const int32_t ex = block_exclusive_scan(v, sh, total);
        if (i < nb) sums[i] = ex + carry;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *grand_total = carry;
}

__global__ void k_scan_add(int32_t *out, int32_t n, const int32_t *sums) {
    const int64_t i = (int64_t)blockIdx.x * kScanItems + threadIdx.x;
    const int32_t add = sums[blockIdx.x];
    if (i < n) out[i] += add;
    if (i + kScanThreads < n) out[i + kScanThreads] += add;
}

}  // namespace

namespace {
__global__ void k_build_candidates(const int4 *desc, const int32_t *list, int4 *cand) {
    const int q1 = blockIdx.y;
    const int4 d = desc[q1];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.y; i += gridDim.x * blockDim.x)
        cand[d.z + i] = make_int4(q1, list[d.x + i] - 1, d.w, 0);
}
}  // namespace

cudaError_t launch_build_candidates(const int4 *desc, int32_t n_irr, int32_t max_len, const int32_t *list, int4 *cand,
                                    cudaStream_t s) {
    if (n_irr <= 0 || max_len <= 0) return cudaSuccess;
    dim3 grid((unsigned)((max_len + 255) / 256), (unsigned)n_irr);
    k_build_candidates<<<grid, 256, 0, s>>>(desc, list, cand);
    return cudaGetLastError();
}

size_t exclusive_scan_tmp_elems(int32_t n) { return (size_t)(n + kScanItems - 1) / kScanItems + 1; }

cudaError_t exclusive_scan_i32(const int32_t *in, int32_t *out, int32_t n, int32_t *tmp, cudaStream_t s) {
    const int32_t nb = (n + kScanItems - 1) / kScanItems;
    if (nb == 0) {
        return cudaMemsetAsync(out, 0, sizeof(int32_t), s);
    }
    k_scan_blocks<<<nb, kScanThreads, 0, s>>>(in, out, n, tmp);
    k_scan_sums<<<1, kScanThreads, 0, s>>>(tmp, nb, out + n);
    k_scan_add<<<nb, kScanThreads, 0, s>>>(out, n, tmp);
    return cudaGetLastError();
}

cudaError_t launch_triplet_count(const MeshDev &m, const int4 *cand, int32_t n_cand, int32_t *n_trip,
                                 int32_t *n_red, int32_t *status, cudaStream_t s) {
    if (n_cand <= 0) return cudaSuccess;
    k_triplet_count<<<(n_cand + 127) / 128, 128, 0, s>>>(m, cand, n_cand, n_trip, n_red, status);
    return cudaGetLastError();
}

cudaError_t launch_triplet_fill(const MeshDev &m, const int4 *cand, int32_t n_cand, const int32_t *trip_off,
                                const int32_t *red_off, TripletRec *trip, int2 *red, cudaStream_t s) {
    if (n_cand <= 0) return cudaSuccess;
    k_triplet_fill<<<(n_cand + 127) / 128, 128, 0, s>>>(m, cand, n_cand, trip_off, red_off, trip, red);
    return cudaGetLastError();
}

cudaError_t launch_quartet_count(const MeshDev &m, const int4 *cand, int32_t n_cand, int32_t *n_q,
                                 int32_t *n_red, int32_t *status, cudaStream_t s) {
    if (n_cand <= 0) return cudaSuccess;
    k_quartet_count<<<(n_cand + 127) / 128, 128, 0, s>>>(m, cand, n_cand, n_q, n_red, status);
    return cudaGetLastError();
}

cudaError_t launch_quartet_fill(const MeshDev &m, const int4 *cand, int32_t n_cand, const int32_t *q_off,
                                const int32_t *red_off, QuartetRec *quart, int4 *red, cudaStream_t s) {
    if (n_cand <= 0) return cudaSuccess;
    k_quartet_fill<<<(n_cand + 127) / 128, 128, 0, s>>>(m, cand, n_cand, q_off, red_off, quart, red);
    return cudaGetLastError();
}

}  // namespace tdg
