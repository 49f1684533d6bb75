// C-ABI entry points: context, upload, scattering orchestration and the BTE solve.
//
// tdg_scattering follows lo_scattering_rates%generate (scattering.f90:58-358):
//   init (:85-212)                     be, sigsq, rows            -> host, uploaded
//   per row: isotope (:229-233)        K_iso                       -> device
//            three-phonon (:234-238)   K1 enumerate, K2-4 fused, K5a symmetrise -> device
//            four-phonon (:239-243)    K1 quartets, fused kernel, K5a            -> device
//            boundary (:245-250)       host
//   allreduce + degeneracy (:261-292) host (N_irr x n values)
//   symmetrize_scatmat (:296-357)     K5b -> device
// tdg_kappa follows get_kappa / iterative_solution / symmetrize_kappa (kappa.f90:28-75,
// 308-495) with the Xi product on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/tdep_gb300.h"
#include "host/common.hpp"
#include "tdg_internal.cuh"

using namespace tdg;

namespace {

#define CUDA_TRY(expr)                                                                                 \
    do {                                                                                               \
        cudaError_t e_ = (expr);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return set_error(kErrDevice, std::string(#expr) + ": " + cudaGetErrorString(e_));          \
    } while (0)

// Device memory of a context comes from one stream-ordered pool per device that keeps freed
// blocks (unlimited release threshold): a context created after another one reuses its
// buffers instead of mapping new memory, as a caching allocator does.
// tdg_release_cached_memory returns the cached blocks to the driver. Allocation and free are
// ordered on the stream of the context whose call is running on this thread (PoolScope);
// outside such a call DevBuf falls back to cudaMalloc / cudaFree.
thread_local std::unique_ptr<int32_t[]> tl_slist;  // shared three-phonon samples (tdg_scattering)
thread_local size_t tl_slist_cap = 0;
thread_local cudaStream_t tl_stream = nullptr;
thread_local cudaMemPool_t tl_pool = nullptr;

struct PoolScope {
    cudaStream_t ps;
    cudaMemPool_t pp;
    PoolScope(cudaStream_t s, cudaMemPool_t p) : ps(tl_stream), pp(tl_pool) {
        tl_stream = s;
        tl_pool = p;
    }
    ~PoolScope() {
        tl_stream = ps;
        tl_pool = pp;
    }
};

std::mutex g_pool_mu;
cudaMemPool_t g_pools[64] = {};

cudaMemPool_t device_pool(int dev) {
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> g(g_pool_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        if (cudaMemPoolCreate(&g_pools[dev], &props) != cudaSuccess) {
            cudaGetLastError();
            g_pools[dev] = nullptr;
            return nullptr;
        }
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(g_pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    return g_pools[dev];
}

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t st = nullptr;  // stream of a pool allocation, nullptr for cudaMalloc
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            if (st)
                cudaFreeAsync(p, st);
            else
                cudaFree(p);
        }
        p = nullptr;
        n = 0;
        st = nullptr;
    }
    cudaError_t alloc(size_t count) {
        if (count <= n && p) return cudaSuccess;
        release();
        if (count == 0) count = 1;
        cudaError_t e;
        if (tl_pool && tl_stream) {
            e = cudaMallocFromPoolAsync(reinterpret_cast<void **>(&p), count * sizeof(T), tl_pool, tl_stream);
            if (e == cudaSuccess) st = tl_stream;
        } else {
            e = cudaMalloc(&p, count * sizeof(T));
        }
        if (e == cudaSuccess)
            n = count;
        else
            p = nullptr;
        return e;
    }
    cudaError_t upload(const T *h, size_t count, cudaStream_t s) {
        cudaError_t e = alloc(count);
        if (e != cudaSuccess) return e;
        if (count == 0) return cudaSuccess;
        return copy_async(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s);
    }
};

int gcd_i(int a, int b) { return b == 0 ? a : gcd_i(b, a % b); }

// 2^(-j/64), j = 0..63, for the device exponential; long double keeps the rounding to
// double correct.
std::vector<double> exp2_table() {
    std::vector<double> t(64);
    for (int j = 0; j < 64; ++j) t[j] = (double)std::exp2l(-(long double)j / 64.0L);
    return t;
}

// lo_chop (gottochblandat.f90:1286-1376): snap to 0, +-n/m (m <= 10), +-1/sqrt2, +-sqrt3/2, +-1.
double lo_chop(double x, double tol) {
    if (std::fabs(x) < tol) return 0.0;
    static std::vector<double> wd;
    if (wd.empty()) {
        for (int mm = 2; mm <= 10; ++mm)
            for (int nn = 1; nn < mm; ++nn) wd.push_back((double)nn / mm);
        wd.push_back(0.7071067811865475);
        wd.push_back(0.8660254037844386);
        wd.push_back(1.0);
    }
    for (double w : wd) {
        if (std::fabs(x - w) < tol) return w;
        if (std::fabs(x + w) < tol) return -w;
    }
    return x;
}

}  // namespace

namespace tdg {
thread_local int64_t *tl_xfer = nullptr;
}

struct tdg_ctx {
    int device = 0;
    int64_t xfer[2] = {0, 0};  // host-to-device and device-to-host bytes of calls on this context
    cudaMemPool_t pool = nullptr;  // device_pool(device)
    int n_sm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[10] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int32_t h_tot[2] = {0, 0};  // enumeration totals (a pinned allocation costs more than it saves)
    DevBuf<int32_t> d_full_op;
    DevBuf<double> d_op_cart, d_fn;
    // host copy of the problem
    int na = 0, n = 0, nop = 0, N = 0, nirr = 0;
    int grid[3] = {0, 0, 0};
    double latvec[9], reclat[9], inv_reclat[9], volume = 0;
    std::vector<double> disorder, op_cart, omega, vel, irr_weight;
    std::vector<int32_t> op_recfrac, full_irr, full_op, irr_full, irr_nop, irr_ops, degen, degen_mode;
    int n_fc3 = 0, n_fc4 = 0;
    // device copies
    DevBuf<int32_t> rot, d_irr_full, d_full_irr, d_irr_nop, d_irr_ops;
    DevBuf<double> d_omega, d_vel, d_be, d_sigsq, d_disorder;
    DevBuf<double2> d_egv, d_egvs;
    DevBuf<float2> d_egvs32;
    DevBuf<int32_t> fc3_blk, fc3_lv, fc4_blk, fc4_lv, fc3_abase;
    std::vector<int> fc3_perm;  // device (block-sorted) position -> index in the problem
    DevBuf<double> fc3_mwm, fc4_mwm;
    DevBuf<float> fc3_mwm32, fc4_mwm32;
    // tensor-core fused kernel (9-15 modes, mixed): eigenvector images built on first use;
    // the pretransform plans' layouts (pretransform_plan) built with the force constants,
    // one for the tensor-core kernel and one for the FP32 SIMT kernel (slots 0: no plan),
    // their values refilled by every call (tdg_set_fc3 may change them)
    DevBuf<unsigned char> d_tc_eimg, d_tc_eimg_t;  // E and E^T images (the latter for the adjoint)
    struct Plan {
        DevBuf<uint32_t> word, src;
        DevBuf<float4> pm;
        int slots = 0, threads = 0;
    } tc_plan, simt_plan;
    bool tc_eimg_ready = false, tc_eimg_t_ready = false;
    int last_path = -1;  // 0 SIMT fused kernel, 1 tensor-core fused kernel, 2 large-cell batches
    // fused three-phonon launch of the last scattering call: grid, CTAs per SM used, the
    // runtime's occupancy figure and the register/shared-memory count (-1 before any)
    int last_launch[4] = {-1, -1, -1, -1};
    DevBuf<double2> tw;
    DevBuf<float2> tw32;
    DevBuf<double> d_exp2tab, d_invom;
    DevBuf<float> d_om32, d_sigsq32;
    int L = 1, lmul[3] = {1, 1, 1};
    // scattering state
    int n_row = 0;
    std::vector<int32_t> row_q1, row_b1;
    DevBuf<int32_t> d_row_q1, d_row_b1, d_rowidx;
    DevBuf<double> d_w3, d_w4, d_w3q, d_gamma, d_xi, d_od;
    // orbits of the little groups (built once per context)
    DevBuf<int32_t> d_orb_rep_ptr, d_orb_rep, d_orb_img, d_orb_mult, d_orb_nuniq, d_orb_cnt, d_orb_of;
    DevBuf<double> d_rcp;
    OrbitDev orbits{};
    DevBuf<int32_t> d_status;
    DevBuf<uint32_t> d_sbits;  // per row: bitmap of its sampled q-points (three-phonon)
    bool have_scattering = false;
    std::vector<double> linewidth, qs, F0, Fn;  // irr-point arrays
    // enumeration and sample buffers, kept across calls (they only grow)
    DevBuf<int4> d_cand;
    DevBuf<uint32_t> d_mask;
    DevBuf<int32_t> d_nt, d_nrd, d_toff, d_roff, d_tmp, d_list3, d_rlen;
    DevBuf<int64_t> d_rbeg;
    DevBuf<int4> d_qdesc;
    DevBuf<TripletRec> d_trip;
    DevBuf<int2> d_red;
    // four-phonon enumeration, samples (list a drives the symmetrisation) and kernel scratch
    DevBuf<int4> d_cand4, d_red4;
    DevBuf<uint32_t> d_mask4;
    DevBuf<int32_t> d_nq, d_nrd4, d_qoff, d_roff4, d_tmp4, d_list4a, d_rlen4;
    DevBuf<int64_t> d_rbeg4;
    DevBuf<QuartetRec> d_quart;
    DevBuf<unsigned char> d_scr4;
    // BTE buffers
    DevBuf<double> d_buf, d_part;
    DevBuf<float2> d_fbb;   // F as double-float pairs for the BTE product
    DevBuf<float4> d_xi_df;  // Xi as double-float row pairs (launch_split_xi)
    // state of the last tdg_scattering that the adjoint pass reuses
    PhononDev last_ph{};
    RowsDev last_rows{};
    int32_t last_ntrip = 0;
    bool last_third = false;
    DevBuf<double> d_lam, d_slices, d_mwm_bar;
    // BTE adjoint (tdg_kappa_iter_vjp): cotangent of the raw three-phonon terms of Xi, the
    // recomputed raw terms, and work arrays; fn_iter: c->Fn is an iterative solution
    DevBuf<double> d_xi_bar, d_od_raw, d_gam_tmp, d_zv, d_yv, d_xpart, d_tf, d_xtf;
    bool xi_bar_ready = false, fn_iter = false;
    int last_prec = 0;
    // large-cell path: real-split eigenvector matrices (built once), operand planes, Psi, phases
    DevBuf<__nv_bfloat16> d_bmat, d_lnx;
    DevBuf<float2> d_psi, d_lnph;
    bool bmat_ready = false;
    // The three-phonon kernels of the pipeline (the fused kernel, or the large-cell batches)
    // as a CUDA graph: recorded on the second call with the same key
    // (the first runs it directly, which also sets the kernels' attributes), replayed after.
    struct GraphSlot {
        std::string key;
        int seen = 0;
        bool failed = false;  // capture refused: this key runs directly
        cudaGraphExec_t exec = nullptr;
        int64_t counts[3] = {0, 0, 0};  // direct runs, recordings, replays
    } graph3;
    GraphSlot graph_bte;                  // a chunk of BTE iterations (tdg_kappa)
    int kappa_calls = 0;
    // BTE iteration state on the device
    DevBuf<double> d_fnb, d_scf, d_qs_bte, d_F0, d_bte_part;
    DevBuf<int32_t> d_deg_irr, d_dm_irr;
    DevBuf<BteCtl> d_ctl;
    bool last_ln = false;  // the last tdg_scattering took the large-cell (tensor-core) path
    int last_ln_tune = 324;  // its launch shape (delta row block * 10 + GEMM stages)
    DevBuf<__nv_bfloat16> d_bmat_t;  // transposed real-split matrices (adjoint)
    DevBuf<float> d_ghi, d_glo;      // double-float gradient accumulator (large-cell adjoint)
    int xi_fmt = -1;  // d_xi_df holds the current Xi (1) or nothing (-1)
    // off-diagonal kappa inputs (host copies; uploaded by the first tdg_kappa_offdiag)
    std::vector<double> irr_dyngrad, atom_shift, q_full;
    std::vector<int32_t> op_fmap;
    DevBuf<double2> d_grad, d_odwork;
    DevBuf<int2> d_od_items;
    DevBuf<int32_t> d_od_itemptr;
    int od_items = 0;
    DevBuf<double> d_shift, d_qfull, d_lwcv, d_odS, d_irr_weight;
    DevBuf<int32_t> d_fmap;

    MeshDev mesh() const {
        MeshDev m;
        std::memset(&m, 0, sizeof m);  // kernel-argument bytes are compared as graph keys
        m.n_full = N;
        m.n_irr = nirr;
        m.n_op = nop;
        m.n_mode = n;
        for (int i = 0; i < 3; ++i) m.grid[i] = grid[i];
        m.L = L;
        for (int i = 0; i < 3; ++i) m.lmul[i] = lmul[i];
        m.rot = rot.p;
        m.irr_full = d_irr_full.p;
        m.full_irr = d_full_irr.p;
        m.irr_nop = d_irr_nop.p;
        m.irr_ops = d_irr_ops.p;
        return m;
    }
};

extern "C" int tdg_check_mma(int32_t variant, int32_t n, const float *a, const float *b, float *d) {
    if (!a || !b || !d || variant < 0 || variant > 3 || n < 16 || n > 256 || n % 16 != 0)
        return set_error(kErrParam, "tdg_check_mma: bad argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error(kErrDevice, "no CUDA device available");
    }
    DevBuf<float> da, db, dd;
    DevBuf<int> dst;
    CUDA_TRY(da.upload(a, 128 * 16, nullptr));
    CUDA_TRY(db.upload(b, 16 * (size_t)n, nullptr));
    CUDA_TRY(dd.alloc(128 * (size_t)n));
    CUDA_TRY(dst.alloc(1));
    CUDA_TRY(cudaMemset(dst.p, 0, sizeof(int)));
    CUDA_TRY(launch_mma_check(variant, n, da.p, db.p, dd.p, dst.p, nullptr));
    CUDA_TRY(cudaDeviceSynchronize());
    int st = 0;
    CUDA_TRY(cudaMemcpy(&st, dst.p, sizeof(int), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(d, dd.p, sizeof(float) * 128 * n, cudaMemcpyDeviceToHost));
    if (st) return set_error(kErrDevice, "tdg_check_mma: the MMA did not complete in time");
    return kOk;
}

extern "C" int tdg_check_exp(const double *t, int32_t n, double *out) {
    if (!t || !out || n < 0) return set_error(kErrParam, "tdg_check_exp: bad argument");
    for (int32_t i = 0; i < n; ++i)
        if (!(t[i] >= 0.0 && t[i] <= 40.0)) return set_error(kErrParam, "tdg_check_exp: t outside [0, 40]");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error(kErrDevice, "no CUDA device available");
    }
    DevBuf<double> dt, dout, dtab;
    const std::vector<double> tab = exp2_table();
    CUDA_TRY(dt.upload(t, n, nullptr));
    CUDA_TRY(dtab.upload(tab.data(), tab.size(), nullptr));
    CUDA_TRY(dout.alloc(n));
    CUDA_TRY(launch_exp_neg_check(dt.p, n, dout.p, dtab.p, nullptr));
    CUDA_TRY(cudaMemcpy(out, dout.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return kOk;
}

extern "C" int tdg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

namespace {

int check_problem(const tdg_problem *p) {
    if (!p) return set_error(kErrParam, "null problem");
    if (p->n_atom < 1 || p->n_mode != 3 * p->n_atom) return set_error(kErrBadDim, "n_mode must be 3*n_atom");
    if (p->n_op < 1) return set_error(kErrSymmetry, "no symmetry operations");
    for (int i = 0; i < 3; ++i)
        if (p->grid[i] < 1) return set_error(kErrBadDim, "grid dimensions must be positive");
    if ((int64_t)p->grid[0] * p->grid[1] * p->grid[2] != p->n_full)
        return set_error(kErrBadDim, "n_full != product of the grid dimensions");
    if (p->n_irr < 1 || p->n_irr > p->n_full) return set_error(kErrBadDim, "bad n_irr");
    if (!p->op_cart || !p->op_recfrac || !p->full_irr || !p->full_op || !p->irr_full || !p->irr_weight ||
        !p->irr_nop || !p->irr_ops || !p->omega || !p->egv || !p->vel || !p->degen || !p->degen_mode ||
        !p->mass_disorder)
        return set_error(kErrParam, "null array in problem");
    for (int i = 0; i < p->n_irr; ++i)
        if (p->irr_full[i] < 1 || p->irr_full[i] > p->n_full) return set_error(kErrParam, "irr_full out of range");
    for (int i = 0; i < p->n_full; ++i) {
        if (p->full_irr[i] < 1 || p->full_irr[i] > p->n_irr) return set_error(kErrParam, "full_irr out of range");
        if (p->full_op[i] == 0 || std::abs(p->full_op[i]) > p->n_op)
            return set_error(kErrParam, "full_op out of range");
    }
    for (int i = 0; i < p->n_irr; ++i) {
        if (p->irr_nop[i] < 1 || p->irr_nop[i] > p->n_op) return set_error(kErrParam, "irr_nop out of range");
        if (p->irr_nop[i] > 192) return set_error(kErrParam, "little group larger than 192 operations");
        for (int j = 0; j < p->irr_nop[i]; ++j) {
            const int o = p->irr_ops[(size_t)i * p->n_op + j];
            if (o < 1 || o > p->n_op) return set_error(kErrParam, "irr_ops out of range");
        }
    }
    const size_t nm = (size_t)p->n_full * p->n_mode;
    for (size_t i = 0; i < nm; ++i) {
        if (!std::isfinite(p->omega[i])) return set_error(kErrPhysical, "non-finite frequency");
        if (p->degen[i] < 1 || p->degen[i] > p->n_mode) return set_error(kErrParam, "degeneracy out of range");
        for (int j = 0; j < p->degen[i]; ++j) {
            const int b = p->degen_mode[i * p->n_mode + j];
            if (b < 1 || b > p->n_mode) return set_error(kErrParam, "degenmode out of range");
        }
    }
    if (p->n_fc3 < 0 || p->n_fc4 < 0) return set_error(kErrParam, "negative force-constant count");
    if (p->n_fc3 > 0 && (!p->fc3_atoms || !p->fc3_lv || !p->fc3_mwm)) return set_error(kErrParam, "null fc3 array");
    if (p->n_fc4 > 0 && (!p->fc4_atoms || !p->fc4_lv || !p->fc4_mwm)) return set_error(kErrParam, "null fc4 array");
    for (int t = 0; t < p->n_fc3; ++t)
        for (int k = 0; k < 3; ++k)
            if (p->fc3_atoms[3 * t + k] < 1 || p->fc3_atoms[3 * t + k] > p->n_atom)
                return set_error(kErrParam, "fc3 atom index out of range");
    for (int t = 0; t < p->n_fc4; ++t)
        for (int k = 0; k < 4; ++k)
            if (p->fc4_atoms[4 * t + k] < 1 || p->fc4_atoms[4 * t + k] > p->n_atom)
                return set_error(kErrParam, "fc4 atom index out of range");
    return kOk;
}

}  // namespace

namespace {
// Buffers go back to the pool in the order of the context's stream, which is destroyed last.
void destroy_ctx(tdg_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    PhaseTimer pt("tdg_destroy");
    cudaStream_t s = c->stream;
    if (s) cudaStreamSynchronize(s);
    for (auto &x : c->ev)
        if (x) cudaEventDestroy(x);
    if (c->graph3.exec) cudaGraphExecDestroy(c->graph3.exec);
    if (c->graph_bte.exec) cudaGraphExecDestroy(c->graph_bte.exec);
    delete c;
    pt.mark("device buffers");
    if (s) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    pt.mark("stream");
}
}  // namespace

extern "C" int tdg_last_path(tdg_ctx *c, int32_t *path) {
    if (!c || !path) return set_error(kErrParam, "tdg_last_path: null argument");
    *path = c->last_path;
    return kOk;
}

extern "C" int tdg_last_launch(tdg_ctx *c, int32_t *shape) {
    if (!c || !shape) return set_error(kErrParam, "tdg_last_launch: null argument");
    for (int i = 0; i < 4; ++i) shape[i] = c->last_path == 2 ? -1 : c->last_launch[i];
    return kOk;
}

extern "C" int tdg_graph_counts(tdg_ctx *c, int64_t *counts) {
    if (!c || !counts) return set_error(kErrParam, "tdg_graph_counts: null argument");
    for (int i = 0; i < 3; ++i) counts[i] = c->graph3.counts[i];
    return kOk;
}

extern "C" int tdg_release_cached_memory(int device) {
    cudaMemPool_t pool = device_pool(device);
    if (!pool) return set_error(kErrParam, "tdg_release_cached_memory: no pool for this device");
    int prev = 0;
    CUDA_TRY(cudaGetDevice(&prev));
    CUDA_TRY(cudaSetDevice(device));
    CUDA_TRY(cudaDeviceSynchronize());
    const cudaError_t e = cudaMemPoolTrimTo(pool, 0);
    cudaSetDevice(prev);
    CUDA_TRY(e);
    return kOk;
}

extern "C" int tdg_pool_usage(int device, uint64_t *used, uint64_t *reserved) {
    if (!used || !reserved) return set_error(kErrParam, "tdg_pool_usage: null argument");
    cudaMemPool_t pool = device_pool(device);
    if (!pool) return set_error(kErrParam, "tdg_pool_usage: no pool for this device");
    uint64_t u = 0, r = 0;
    CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u));
    CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r));
    *used = (uint64_t)u;
    *reserved = (uint64_t)r;
    return kOk;
}

extern "C" int tdg_create(tdg_ctx **out, const tdg_problem *p, int device) {
    if (!out) return set_error(kErrParam, "tdg_create: null output");
    *out = nullptr;
    int st = check_problem(p);
    if (st) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error(kErrDevice, "no CUDA device available: the GB300 path has no CPU fallback");
    }
    if (device < 0 || device >= ndev) return set_error(kErrParam, "device index out of range");
    PhaseTimer pt("tdg_create");
    CUDA_TRY(cudaSetDevice(device));
    auto *c = new tdg_ctx();
    c->device = device;
    XferScope xs(c->xfer);
    auto fail = [&](int code) {
        destroy_ctx(c);
        return code;
    };
    int major = 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return fail(set_error(kErrDevice, "device query failed"));
    if (major < 10) return fail(set_error(kErrDevice, "device is not Blackwell (sm_100 family required)"));
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(set_error(kErrDevice, "stream creation failed"));
    c->pool = device_pool(device);
    PoolScope pscope(c->stream, c->pool);
    for (auto &x : c->ev)
        if (cudaEventCreate(&x) != cudaSuccess) return fail(set_error(kErrDevice, "event creation failed"));
    c->na = p->n_atom;
    c->n = p->n_mode;
    c->nop = p->n_op;
    c->N = p->n_full;
    c->nirr = p->n_irr;
    for (int i = 0; i < 3; ++i) c->grid[i] = p->grid[i];
    std::memcpy(c->latvec, p->latvec, sizeof(c->latvec));
    std::memcpy(c->reclat, p->reclat, sizeof(c->reclat));
    std::memcpy(c->inv_reclat, p->inv_reclat, sizeof(c->inv_reclat));
    c->volume = p->volume;
    const size_t nm = (size_t)c->N * c->n;
    c->disorder.assign(p->mass_disorder, p->mass_disorder + c->na);
    c->op_cart.assign(p->op_cart, p->op_cart + 9 * c->nop);
    c->op_recfrac.assign(p->op_recfrac, p->op_recfrac + 9 * c->nop);
    c->omega.assign(p->omega, p->omega + nm);
    c->vel.assign(p->vel, p->vel + nm * 3);
    c->irr_weight.assign(p->irr_weight, p->irr_weight + c->nirr);
    c->full_irr.assign(p->full_irr, p->full_irr + c->N);
    c->full_op.assign(p->full_op, p->full_op + c->N);
    c->irr_full.assign(p->irr_full, p->irr_full + c->nirr);
    c->irr_nop.assign(p->irr_nop, p->irr_nop + c->nirr);
    c->irr_ops.assign(p->irr_ops, p->irr_ops + (size_t)c->nirr * c->nop);
    c->degen.assign(p->degen, p->degen + nm);
    c->degen_mode.assign(p->degen_mode, p->degen_mode + nm * c->n);
    c->n_fc3 = p->n_fc3;
    c->n_fc4 = p->n_fc4;
    c->q_full.assign(p->q_full, p->q_full + 3 * (size_t)c->N);
    if (p->irr_dyngrad && p->op_fmap && p->atom_shift) {
        c->irr_dyngrad.assign(p->irr_dyngrad, p->irr_dyngrad + (size_t)c->nirr * 3 * c->n * c->n * 2);
        c->atom_shift.assign(p->atom_shift, p->atom_shift + (size_t)c->nop * c->na * 3);
        c->op_fmap.resize((size_t)c->nop * c->na);
        for (size_t i = 0; i < c->op_fmap.size(); ++i) {
            c->op_fmap[i] = p->op_fmap[i] - 1;
            if (c->op_fmap[i] < 0 || c->op_fmap[i] >= c->na) return fail(set_error(kErrParam, "op_fmap out of range"));
        }
    }
    c->L = 1;
    for (int i = 0; i < 3; ++i) c->L = c->L / gcd_i(c->L, c->grid[i]) * c->grid[i];
    for (int i = 0; i < 3; ++i) c->lmul[i] = c->L / c->grid[i];

    pt.mark("device and host copies");
    cudaStream_t s = c->stream;
    pt.mark("rotation table");
    std::vector<int32_t> irr_full0(c->nirr), full_irr0(c->N), irr_ops0((size_t)c->nirr * c->nop, 0);
    for (int i = 0; i < c->nirr; ++i) irr_full0[i] = c->irr_full[i] - 1;
    for (int i = 0; i < c->N; ++i) full_irr0[i] = c->full_irr[i] - 1;
    for (size_t i = 0; i < irr_ops0.size(); ++i) irr_ops0[i] = c->irr_ops[i] > 0 ? c->irr_ops[i] - 1 : -1;
    // the eigenvectors go up as stored; the scaled copies (egv(:,b)/sqrt(om),
    // scattering_threephonon.f90:67,93,102) and the rotation table are built on the device
    pt.mark("eigenvector copies");
    // Force constants sorted by atom block (a1,a2,a3).
    const int na = c->na;
    std::vector<int32_t> blk_ptr3(na * na * na + 1, 0), lv3, abase3;
    std::vector<double> mwm3;
    std::vector<float> mwm3f;
    {
        std::vector<int> idx(c->n_fc3);
        std::iota(idx.begin(), idx.end(), 0);
        auto blk = [&](int t) {
            const int32_t *a = p->fc3_atoms + 3 * t;
            return ((a[0] - 1) * na + (a[1] - 1)) * na + (a[2] - 1);
        };
        std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return blk(x) < blk(y); });
        c->fc3_perm = idx;
        for (int t : idx) {
            {
                const int32_t *at = p->fc3_atoms + 3 * t;
                abase3.push_back(((3 * (at[0] - 1)) * c->n + 3 * (at[1] - 1)) * c->n + 3 * (at[2] - 1));
            }
            blk_ptr3[blk(t) + 1]++;
            lv3.insert(lv3.end(), p->fc3_lv + 6 * t, p->fc3_lv + 6 * t + 6);
            for (int k = 0; k < 27; ++k) {
                mwm3.push_back(p->fc3_mwm[27 * t + k]);
                mwm3f.push_back((float)p->fc3_mwm[27 * t + k]);
            }
        }
        for (size_t b = 1; b < blk_ptr3.size(); ++b) blk_ptr3[b] += blk_ptr3[b - 1];
    }
    std::vector<int32_t> blk_ptr4(na * na * na * na + 1, 0), lv4;
    std::vector<double> mwm4;
    std::vector<float> mwm4f;
    {
        std::vector<int> idx(c->n_fc4);
        std::iota(idx.begin(), idx.end(), 0);
        auto blk = [&](int t) {
            const int32_t *a = p->fc4_atoms + 4 * t;
            return (((a[0] - 1) * na + (a[1] - 1)) * na + (a[2] - 1)) * na + (a[3] - 1);
        };
        std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return blk(x) < blk(y); });
        for (int t : idx) {
            blk_ptr4[blk(t) + 1]++;
            lv4.insert(lv4.end(), p->fc4_lv + 9 * t, p->fc4_lv + 9 * t + 9);
            for (int k = 0; k < 81; ++k) {
                mwm4.push_back(p->fc4_mwm[81 * t + k]);
                mwm4f.push_back((float)p->fc4_mwm[81 * t + k]);
            }
        }
        for (size_t b = 1; b < blk_ptr4.size(); ++b) blk_ptr4[b] += blk_ptr4[b - 1];
    }
    std::vector<double2> tw(c->L);
    std::vector<float2> tw32(c->L);
    for (int k = 0; k < c->L; ++k) {
        const double ang = kTwoPi * (double)k / (double)c->L;
        tw[k] = make_double2(std::cos(ang), -std::sin(ang));
        tw32[k] = make_float2((float)tw[k].x, (float)tw[k].y);
    }
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    {
        DevBuf<int32_t> orf;
        chk(orf.upload(p->op_recfrac, (size_t)9 * c->nop, s));
        chk(c->rot.alloc((size_t)c->nop * c->N));
        if (e == cudaSuccess) chk(launch_rot_table(c->grid, c->L, c->N, c->nop, orf.p, c->rot.p, s));
    }
    chk(c->d_irr_full.upload(irr_full0.data(), irr_full0.size(), s));
    chk(c->d_full_irr.upload(full_irr0.data(), full_irr0.size(), s));
    chk(c->d_irr_nop.upload(c->irr_nop.data(), c->irr_nop.size(), s));
    chk(c->d_irr_ops.upload(irr_ops0.data(), irr_ops0.size(), s));
    chk(c->d_omega.upload(c->omega.data(), c->omega.size(), s));
    chk(c->d_vel.upload(c->vel.data(), c->vel.size(), s));
    chk(c->d_egv.upload(reinterpret_cast<const double2 *>(p->egv), nm * c->n, s));
    chk(c->d_egvs.alloc(nm * c->n));
    chk(c->d_egvs32.alloc(nm * c->n));
    if (e == cudaSuccess)
        chk(launch_egv_scaled((int64_t)nm, c->n, c->d_egv.p, c->d_omega.p, c->d_egvs.p, c->d_egvs32.p, s));
    chk(c->d_disorder.upload(c->disorder.data(), c->disorder.size(), s));
    chk(c->fc3_blk.upload(blk_ptr3.data(), blk_ptr3.size(), s));
    auto make_plan = [&](tdg_ctx::Plan &pl, int threads, bool tc_operand) {
        std::vector<uint32_t> pword, psrc;
        pl.threads = threads;
        pl.slots = pretransform_plan(c->n, na * na * na, blk_ptr3.data(), threads, tc_operand, pword, psrc);
        if (pl.slots > 0) {
            chk(pl.word.upload(pword.data(), pword.size(), s));
            chk(pl.src.upload(psrc.data(), psrc.size(), s));
            chk(pl.pm.alloc(pword.size()));
        }
    };
    if (c->n == 9 || c->n == 12 || c->n == 15) make_plan(c->tc_plan, 256, true);
    if (threephonon_plan_fits(c->n, (int)(blk_ptr3.back()))) make_plan(c->simt_plan, threephonon_threads(c->n), false);
    chk(c->fc3_abase.upload(abase3.data(), abase3.size(), s));
    chk(c->fc3_lv.upload(lv3.data(), lv3.size(), s));
    chk(c->fc3_mwm.upload(mwm3.data(), mwm3.size(), s));
    chk(c->fc3_mwm32.upload(mwm3f.data(), mwm3f.size(), s));
    chk(c->fc4_blk.upload(blk_ptr4.data(), blk_ptr4.size(), s));
    chk(c->fc4_lv.upload(lv4.data(), lv4.size(), s));
    chk(c->fc4_mwm.upload(mwm4.data(), mwm4.size(), s));
    chk(c->fc4_mwm32.upload(mwm4f.data(), mwm4f.size(), s));
    chk(c->tw.upload(tw.data(), tw.size(), s));
    chk(c->tw32.upload(tw32.data(), tw32.size(), s));
    const std::vector<double> e2t = exp2_table();
    chk(c->d_exp2tab.upload(e2t.data(), e2t.size(), s));
    {
        // per-mode tables of the kernels' screens: omega in FP32 and 1/omega
        std::vector<float> om32(c->omega.size());
        std::vector<double> invom(c->omega.size());
        for (size_t i = 0; i < c->omega.size(); ++i) {
            om32[i] = (float)c->omega[i];
            invom[i] = c->omega[i] > 0.0 ? 1.0 / c->omega[i] : 0.0;
        }
        chk(c->d_om32.upload(om32.data(), om32.size(), s));
        chk(c->d_invom.upload(invom.data(), invom.size(), s));
    }
    chk(c->d_status.alloc(1));
    chk(cudaStreamSynchronize(s));
    pt.mark("force constants, tables, uploads");
    if (e != cudaSuccess) return fail(set_error(kErrDevice, std::string("upload failed: ") + cudaGetErrorString(e)));
    {
        // Orbit tables: flags, global scan over (q1, q2), fill; representatives per q1.
        const int32_t nflag = c->nirr * c->N;
        if ((int64_t)c->nirr * c->N >= (int64_t)1 << 31) return fail(set_error(kErrBadDim, "mesh too large"));
        DevBuf<int32_t> flag, scan, tmp;
        chk(flag.alloc(nflag));
        chk(scan.alloc(nflag + 1));
        chk(tmp.alloc(exclusive_scan_tmp_elems(nflag)));
        chk(c->d_orb_rep_ptr.alloc(c->nirr + 1));
        chk(c->d_orb_of.alloc(nflag));
        if (e != cudaSuccess) return fail(set_error(kErrDevice, std::string("allocation failed: ") + cudaGetErrorString(e)));
        const MeshDev mesh = c->mesh();
        chk(launch_orbit_flag(mesh, flag.p, s));
        chk(exclusive_scan_i32(flag.p, scan.p, nflag, tmp.p, s));
        int32_t nrep = 0;
        chk(copy_async(&nrep, scan.p + nflag, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        chk(cudaStreamSynchronize(s));
        chk(c->d_orb_rep.alloc(nrep));
        chk(c->d_orb_img.alloc((size_t)nrep * c->nop));
        chk(c->d_orb_cnt.alloc(nrep));
        chk(c->d_orb_mult.alloc((size_t)nrep * c->nop));
        chk(c->d_orb_nuniq.alloc(nrep));
        std::vector<double> rcp(c->nop + 1, 0.0);
        for (int i = 1; i <= c->nop; ++i) rcp[i] = 1.0 / (double)i;
        chk(c->d_rcp.upload(rcp.data(), rcp.size(), s));
        if (e != cudaSuccess) return fail(set_error(kErrDevice, std::string("orbit tables: ") + cudaGetErrorString(e)));
        c->orbits.rep_ptr = c->d_orb_rep_ptr.p;
        c->orbits.rep = c->d_orb_rep.p;
        c->orbits.img = c->d_orb_img.p;
        c->orbits.cnt = c->d_orb_cnt.p;
        c->orbits.mult = c->d_orb_mult.p;
        c->orbits.nuniq = c->d_orb_nuniq.p;
        c->orbits.rcp = c->d_rcp.p;
        c->orbits.orb_of = c->d_orb_of.p;
        chk(launch_orbit_fill(mesh, flag.p, scan.p, c->orbits, s));
        std::vector<int32_t> rp(c->nirr + 1);
        chk(copy_async(rp.data(), c->d_orb_rep_ptr.p, sizeof(int32_t) * rp.size(), cudaMemcpyDeviceToHost, s));
        chk(cudaStreamSynchronize(s));
        if (e != cudaSuccess) return fail(set_error(kErrDevice, std::string("orbit tables: ") + cudaGetErrorString(e)));
        int mx = 0, mt = 0;
        for (int q = 0; q < c->nirr; ++q) {
            mx = std::max(mx, rp[q + 1] - rp[q]);
            mt = std::max(mt, sym_tile_count(rp[q + 1] - rp[q], c->irr_nop[q], c->n));
        }
        c->orbits.max_rep = mx;
        c->orbits.tile_pts = sym_tile_points(c->n);
        c->orbits.max_tiles = mt;
    }
    pt.mark("orbit tables");
    *out = c;
    return kOk;
}

extern "C" void tdg_destroy(tdg_ctx *c) { destroy_ctx(c); }

namespace {

int validate_opts(const tdg_opts *o) {
    if (!o) return set_error(kErrParam, "null options");
    if (o->integrationtype != 1 && o->integrationtype != 2 && o->integrationtype != 6)
        return set_error(kErrParam, "integrationtype must be 1, 2 or 6");
    if (!(o->temperature >= 0) || !std::isfinite(o->temperature)) return set_error(kErrPhysical, "bad temperature");
    if (o->integrationtype == 1 && !(o->sigma > 0)) return set_error(kErrParam, "sigma must be positive");
    if (o->precision != TDG_PREC_FP64 && o->precision != TDG_PREC_MIXED)
        return set_error(kErrParam, "precision must be TDG_PREC_FP64 or TDG_PREC_MIXED");
    if (o->tensor_cores < 0 || o->tensor_cores > 2) return set_error(kErrParam, "tensor_cores must be 0, 1 or 2");
    if (o->tensor_cores == 1 && o->precision != TDG_PREC_MIXED)
        return set_error(kErrParam, "the tensor-core contraction needs precision TDG_PREC_MIXED");
    return kOk;
}

// Row pointers of a CSR sample; with check_values also every entry's range.
int check_list(const char *what, int n_row, const int64_t *ptr, const int32_t *l, int N, bool check_values = true) {
    if (!ptr) return set_error(kErrParam, std::string(what) + ": missing row pointer");
    if (ptr[0] != 0) return set_error(kErrParam, std::string(what) + ": ptr[0] must be 0");
    for (int r = 0; r < n_row; ++r) {
        if (ptr[r + 1] < ptr[r]) return set_error(kErrParam, std::string(what) + ": decreasing row pointer");
        if (ptr[r + 1] == ptr[r]) return set_error(kErrParam, std::string(what) + ": empty q' sample for a row");
    }
    if (ptr[n_row] > 0 && !l) return set_error(kErrParam, std::string(what) + ": missing list");
    if (!check_values) return kOk;
    for (int64_t i = 0; i < ptr[n_row]; ++i)
        if (l[i] < 1 || l[i] > N) return set_error(kErrParam, std::string(what) + ": q' index out of range");
    return kOk;
}

int read_status(tdg_ctx *c) {
    int32_t st = 0;
    CUDA_TRY(copy_async(&st, c->d_status.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (st != kDevOk) return set_error(kErrDevice, "device-side index check failed (status " + std::to_string(st) + ")");
    return kOk;
}

}  // namespace

namespace {
// Buffers and the batch descriptor of the large-cell path (real-split eigenvector matrices
// built once per context; operand planes, Psi and phases for nbmax q-triplets, bounded to
// 2 GB).
int ln_batch_setup(tdg_ctx *c, const MeshDev &mesh, const PhononDev &ph, const RowsDev &rows, const Fc3Dev &fc,
                   int ntrip, LnBatch &b, int &nbmax) {
    cudaStream_t s = c->stream;
    const int n = c->n, N = c->N;
    const int kp = ln_kp(n), mp = ln_mp(n);
    const int64_t plane = (int64_t)kp * mp;
    const size_t per_slot = 4 * (size_t)plane * sizeof(__nv_bfloat16) + (size_t)n * n * n * sizeof(float2) +
                            (size_t)c->n_fc3 * sizeof(float2);
    nbmax = (int)std::max<size_t>(1, std::min<size_t>(256, ((size_t)2 << 30) / per_slot));
    nbmax = std::max(1, std::min(nbmax, ntrip));
    if (!c->bmat_ready) {
        CUDA_TRY(c->d_bmat.alloc((size_t)N * 2 * kp * kp));
        CUDA_TRY(launch_ln_bmat(n, N, c->d_egvs32.p, c->d_bmat.p, false, s));
        c->bmat_ready = true;
    }
    const __nv_bfloat16 *old = c->d_lnx.p;
    CUDA_TRY(c->d_lnx.alloc(4 * (size_t)plane * nbmax));
    CUDA_TRY(c->d_psi.alloc((size_t)nbmax * n * n * n));
    CUDA_TRY(c->d_lnph.alloc((size_t)nbmax * c->n_fc3));
    // padding of the operand planes (component rows a >= n, positions with an index >= n)
    // must read as zero; no kernel writes it
    if (c->d_lnx.p != old) CUDA_TRY(cudaMemsetAsync(c->d_lnx.p, 0, sizeof(__nv_bfloat16) * c->d_lnx.n, s));
    const size_t slots = c->d_lnx.n / (4 * (size_t)plane);
    std::memset(&b, 0, sizeof b);  // kernel-argument bytes are compared as graph keys
    b.delta_bb = 32;
    b.mesh = mesh;
    b.ph = ph;
    b.rows = rows;
    b.fc = fc;
    b.red = c->d_red.p;
    b.cand_mask = c->d_mask.p;
    b.n = n;
    b.plane = plane;
    b.mp = mp;
    b.n_sm = c->n_sm;
    b.xa_hi = c->d_lnx.p;
    b.xa_lo = b.xa_hi + plane * slots;
    b.xb_hi = b.xa_lo + plane * slots;
    b.xb_lo = b.xb_hi + plane * slots;
    b.bmat = c->d_bmat.p;
    b.phase = c->d_lnph.p;
    b.psi = c->d_psi.p;
    b.gamma = c->d_gamma.p;
    b.od = c->d_xi.p;
    b.status = c->d_status.p;
    return kOk;
}
}  // namespace

// Launch shape of the large-cell path packed as one tuning value: delta row block * 10 +
// GEMM pipeline stages.
constexpr int kLnTuneDefault = 324;
void ln_apply_tune(LnBatch &b, int v) {
    b.delta_bb = v / 10 == 16 ? 16 : 32;
    b.gemm_stages = v % 10;
}

bool graphs_enabled() {
    const char *p = std::getenv("TDG_GRAPHS");
    return !(p && std::strcmp(p, "0") == 0);
}

// Runs body on stream s directly, or as the context's recorded graph for this key (see
// tdg_ctx::GraphSlot). A capture the runtime refuses leaves the key on direct runs.
cudaError_t run_graph_region(tdg_ctx *c, tdg_ctx::GraphSlot &g, const std::string &key, cudaStream_t s,
                             const std::function<cudaError_t()> &body, bool may_record = true) {
    if (g.key != key) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        g.key = key;
        g.seen = 0;
        g.failed = false;
    }
    if (g.exec) {
        ++g.counts[2];
        return cudaGraphLaunch(g.exec, s);
    }
    if (g.seen == 0 || g.failed || !may_record || !graphs_enabled()) {
        ++g.seen;
        ++g.counts[0];
        return body();
    }
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGetLastError();
        g.failed = true;
        ++g.counts[0];
        return body();
    }
    const cudaError_t eb = body();
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(s, &graph);
    cudaGraphExec_t exec = nullptr;
    if (eb == cudaSuccess && ee == cudaSuccess && graph) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (eb != cudaSuccess || ee != cudaSuccess || e != cudaSuccess || !exec) {
        // nothing of a failed capture ran: run the work directly from now on
        cudaGetLastError();
        g.failed = true;
        ++g.counts[0];
        return body();
    }
    g.exec = exec;
    ++g.counts[1];
    return cudaGraphLaunch(g.exec, s);
}

// BTE iterations enqueued between two host checks of the convergence flag; iterations after
// convergence in a chunk return at once.
constexpr int kBteChunk = 8;

// Autotuning trials ran on the call's own work: Gamma and Xi start again from zero.
cudaError_t rezero_outputs(tdg_ctx *c, int64_t nr, int64_t ld, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(c->d_xi.p, 0, sizeof(double) * (size_t)nr * ld, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_gamma.p, 0, sizeof(double) * nr, s);
    return e;
}

extern "C" int tdg_scattering(tdg_ctx *c, const tdg_opts *o, const tdg_qlists *ql, double *linewidth, double *qs_out,
                              double *stats) {
    XferScope xs(c ? c->xfer : nullptr);
    PoolScope pscope(c ? c->stream : nullptr, c ? c->pool : nullptr);
    if (!c || !ql || !linewidth) return set_error(kErrParam, "tdg_scattering: null argument");
    PhaseTimer pt("tdg_scattering");
    int st = validate_opts(o);
    if (st) return st;
    CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const int n = c->n, N = c->N, nirr = c->nirr;
    // ---- rows: must be exactly the reference's row set, in order ----
    std::vector<int32_t> exp_q1, exp_b1;
    for (int q1 = 0; q1 < nirr; ++q1) {
        const int f = c->irr_full[q1] - 1;
        for (int b1 = 0; b1 < n; ++b1)
            if (!(c->omega[(size_t)f * n + b1] < kFreqTol)) {
                exp_q1.push_back(q1 + 1);
                exp_b1.push_back(b1 + 1);
            }
    }
    if (ql->n_row != (int)exp_q1.size() || !ql->row_q1 || !ql->row_b1)
        return set_error(kErrParam, "rows do not match the (q1,b1) set with omega >= lo_freqtol");
    for (int r = 0; r < ql->n_row; ++r)
        if (ql->row_q1[r] != exp_q1[r] || ql->row_b1[r] != exp_b1[r])
            return set_error(kErrParam, "rows do not match the (q1,b1) set with omega >= lo_freqtol");
    const int nr = ql->n_row;
    if (o->thirdorder) {
        st = check_list("three-phonon sample", nr, ql->ptr3, ql->list3, N, false);
        if (st) return st;
        if (c->n_fc3 < 1) return set_error(kErrParam, "three-phonon scattering requested without force constants");
        if (n > 18 && o->precision != TDG_PREC_MIXED)
            return set_error(kErrParam, "beyond 18 modes the three-phonon contraction runs on the tensor cores, "
                                        "which needs precision TDG_PREC_MIXED");
        if (ln_kp(n) > 256) return set_error(kErrParam, "the tensor-core contraction supports up to 128 modes");
    }
    if (o->isotope)
        for (int a = 0; a < c->na; ++a)
            if (std::isnan(c->disorder[a]))
                return set_error(kErrParam, "isotope scattering: atom " + std::to_string(a + 1) +
                                                " has no natural isotope distribution in the library's table; "
                                                "give infile.isotopes or switch isotope scattering off");
    if (o->fourthorder) {
        st = check_list("four-phonon sample", nr, ql->ptr4, ql->list4a, N);
        if (st) return st;
        st = check_list("four-phonon sample", nr, ql->ptr4, ql->list4b, N);
        if (st) return st;
        if (c->n_fc4 < 1) return set_error(kErrParam, "four-phonon scattering requested without force constants");
        if (n > 15) return set_error(kErrParam, "this build's four-phonon kernel supports up to 5 atoms");
    }
    c->n_row = nr;
    c->row_q1.assign(ql->row_q1, ql->row_q1 + nr);
    c->row_b1.assign(ql->row_b1, ql->row_b1 + nr);
    pt.mark("argument checks");

    // ---- init block (scattering.f90:126-168) ----
    std::vector<double> be((size_t)nirr * n, 0.0), sigsq((size_t)nirr * n, 0.0), sigavg(n, 0.0);
    double reclat_g[9];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) reclat_g[i + 3 * j] = c->reclat[i + 3 * j] / c->grid[j];
    for (int q1 = 0; q1 < nirr; ++q1) {
        const int f = c->irr_full[q1] - 1;
        for (int b1 = 0; b1 < n; ++b1) {
            const double om = c->omega[(size_t)f * n + b1];
            if (om < kFreqTol) continue;
            be[(size_t)q1 * n + b1] = o->classical ? kKbHartree * o->temperature / om : planck(o->temperature, om);
            const double *v = &c->vel[((size_t)f * n + b1) * 3];
            double sg = 0.0;
            for (int j = 0; j < 3; ++j) {
                double x = 0.0;
                for (int i = 0; i < 3; ++i) x += std::fabs(v[i]) * reclat_g[i + 3 * j];
                sg = std::max(sg, x * x * 0.5);
            }
            sigsq[(size_t)q1 * n + b1] = sg;
            sigavg[b1] += sg * c->irr_weight[q1];
        }
    }
    const double maxavg = *std::max_element(sigavg.begin(), sigavg.end());
    for (double &x : sigsq) x += maxavg * 1e-4;
    PhononDev ph;
    std::memset(&ph, 0, sizeof ph);
    ph.omega = c->d_omega.p;
    ph.egv = c->d_egv.p;
    ph.egvs = c->d_egvs.p;
    ph.egvs32 = c->d_egvs32.p;
    ph.vel = c->d_vel.p;
    std::memcpy(ph.reclat_g, reclat_g, sizeof(reclat_g));
    ph.sigma_fixed = o->sigma * kFreqTHzToHartree;
    ph.thresh_sigma = maxavg * 1e-4;
    ph.integrationtype = o->integrationtype;
    ph.exp2tab = c->d_exp2tab.p;
    ph.inv_omega = c->d_invom.p;
    ph.omega32 = c->d_om32.p;

    std::vector<int32_t> rowidx((size_t)nirr * n, -1), rq1(nr), rb1(nr);
    std::vector<double> w3(nr, 0.0), w4(nr, 0.0), w3q((size_t)nirr * n, 0.0);
    for (int r = 0; r < nr; ++r) {
        rq1[r] = c->row_q1[r] - 1;
        rb1[r] = c->row_b1[r] - 1;
        rowidx[(size_t)rq1[r] * n + rb1[r]] = r;
        if (o->thirdorder) w3[r] = 1.0 / (double)(ql->ptr3[r + 1] - ql->ptr3[r]);
        if (o->fourthorder) w4[r] = 1.0 / (double)(ql->ptr4[r + 1] - ql->ptr4[r]);
        w3q[(size_t)rq1[r] * n + rb1[r]] = w3[r];
    }
    pt.mark("init block");
    // ---- three-phonon samples and candidates ----
    // When all rows of a q1 share one sample (the full grid, or samples given per q1) it is
    // uploaded once per q1 and the candidates (q1, q2, mask of every row of q1) are formed
    // on the device, in sample order. Otherwise the candidates are, per q1, the union of
    // its rows' samples, with the set of rows that sampled q2 as a bit mask. Masks are
    // stored once in a table of distinct masks. A q-point that a row samples k times (the
    // reference's sampler only avoids repeating the previous point, so this happens when the
    // Monte-Carlo grid does not divide the mesh) is counted k times, as the reference does:
    // the j-th copy of a candidate carries the rows that sampled the point at least j times.
    std::vector<int4> cand;                 // union path
    std::vector<uint32_t> masks;            // distinct row masks (4 words each)
    std::vector<int64_t> rbeg(nr, 0);       // per row: start of its sample in the uploaded list
    std::vector<int32_t> rlen(nr, 0);
    // shared path: one sample per q1, in this thread's grow-only host buffer (not zero-filled;
    // the upload from pageable memory has copied it when the call returns)
    size_t slist_n = 0;
    std::vector<int4> qdesc;                // shared path: per q1 (list start, length, first candidate, mask)
    bool shared = true;
    int64_t nc64 = 0;
    if (o->thirdorder) {
        std::vector<int> qr0(nirr + 1, nr);
        for (int r = nr - 1; r >= 0; --r) qr0[rq1[r]] = r;
        for (int q1 = nirr - 1; q1 >= 0; --q1)
            if (qr0[q1] == nr) qr0[q1] = qr0[q1 + 1];
        auto rows_of = [&](int q1, int &r0, int &r1) {
            r0 = qr0[q1];
            r1 = r0;
            while (r1 < nr && rq1[r1] == q1) ++r1;
        };
        // rows of a q1 share one sample when every row's list equals the first row's
        // (compared on all host threads)
        std::vector<char> same(nirr, 1);
        parallel_for(nirr, [&](int64_t q1) {
            int r0, r1;
            rows_of((int)q1, r0, r1);
            for (int r = r0 + 1; r < r1; ++r) {
                const int64_t L = ql->ptr3[r0 + 1] - ql->ptr3[r0];
                if (ql->ptr3[r + 1] - ql->ptr3[r] != L ||
                    std::memcmp(ql->list3 + ql->ptr3[r], ql->list3 + ql->ptr3[r0], sizeof(int32_t) * L) != 0) {
                    same[q1] = 0;
                    return;
                }
            }
        });
        for (int q1 = 0; q1 < nirr; ++q1) shared = shared && same[q1];
        pt.mark("three-phonon sharing test (host)");
        std::vector<std::array<uint32_t, 4>> table;
        auto mask_id = [&](const std::array<uint32_t, 4> &key) {
            for (int t = (int)table.size() - 1; t >= 0 && t >= (int)table.size() - 8; --t)
                if (table[t] == key) return t;
            table.push_back(key);
            return (int)table.size() - 1;
        };
        std::vector<int32_t> stamp(N, -1);
        if (shared) {
            // one list per q1: offsets first, then range checks and the copy in parallel (the
            // other rows' lists are byte-equal to it); a repeated entry becomes a repeated
            // candidate
            qdesc.assign(nirr, make_int4(0, 0, 0, 0));
            std::vector<int64_t> start(nirr + 1, 0);
            for (int q1 = 0; q1 < nirr; ++q1) {
                int r0, r1;
                rows_of(q1, r0, r1);
                const int64_t L = r0 == r1 ? 0 : ql->ptr3[r0 + 1] - ql->ptr3[r0];
                start[q1 + 1] = start[q1] + L;
                if (r0 == r1) continue;
                std::array<uint32_t, 4> key = {0u, 0u, 0u, 0u};
                for (int r = r0; r < r1; ++r) key[rb1[r] >> 5] |= 1u << (rb1[r] & 31);
                qdesc[q1] = make_int4((int32_t)start[q1], (int32_t)L, (int32_t)start[q1], mask_id(key));
                for (int r = r0; r < r1; ++r) {
                    rbeg[r] = start[q1];
                    rlen[r] = (int32_t)L;
                }
            }
            if (start[nirr] >= ((int64_t)1 << 31) - 1)
                return set_error(kErrBadDim, "too many three-phonon candidates for one call");
            slist_n = (size_t)start[nirr];
            if (tl_slist_cap < slist_n) {
                tl_slist.reset(new int32_t[slist_n]);
                tl_slist_cap = slist_n;
            }
            int32_t *slist = tl_slist.get();
            std::atomic<int> bad{0};
            parallel_for(nirr, [&](int64_t q1) {
                const int L = (int)(start[q1 + 1] - start[q1]);
                if (L == 0) return;
                const int32_t *src = ql->list3 + ql->ptr3[qr0[q1]];
                for (int i = 0; i < L; ++i) {
                    const int32_t q2 = src[i];
                    if (q2 < 1 || q2 > N) {
                        bad.store(1);
                        return;
                    }
                    slist[start[q1] + i] = q2;
                }
            });
            if (bad.load() == 1) return set_error(kErrParam, "three-phonon sample: q' index out of range");
            nc64 = start[nirr];
            pt.mark("three-phonon shared samples (host)");
        } else {
            std::atomic<int> bad{0};
            parallel_for(nr, [&](int64_t r) {
                for (int64_t i = ql->ptr3[r]; i < ql->ptr3[r + 1]; ++i)
                    if (ql->list3[i] < 1 || ql->list3[i] > N) bad.store(1);
            });
            if (bad.load()) return set_error(kErrParam, "three-phonon sample: q' index out of range");
            std::vector<uint32_t> mark((size_t)N * 4, 0u);
            std::vector<int32_t> touched, occ(N, 0), row_touched;
            std::vector<std::array<int, 3>> extra;  // (q2, copy index >= 2, b1)
            for (int q1 = 0; q1 < nirr; ++q1) {
                int r0, r1;
                rows_of(q1, r0, r1);
                touched.clear();
                extra.clear();
                for (int r = r0; r < r1; ++r) {
                    const int b1 = rb1[r];
                    rbeg[r] = ql->ptr3[r];
                    rlen[r] = (int32_t)(ql->ptr3[r + 1] - ql->ptr3[r]);
                    row_touched.clear();
                    for (int64_t i = ql->ptr3[r]; i < ql->ptr3[r + 1]; ++i) {
                        const int q2 = ql->list3[i] - 1;
                        if (stamp[q2] == r) {
                            extra.push_back({q2, ++occ[q2], b1});
                            continue;
                        }
                        stamp[q2] = r;
                        occ[q2] = 1;
                        row_touched.push_back(q2);
                        uint32_t *mk = &mark[(size_t)q2 * 4];
                        if (!(mk[0] | mk[1] | mk[2] | mk[3])) touched.push_back(q2);
                        mk[b1 >> 5] |= 1u << (b1 & 31);
                    }
                    for (int q2 : row_touched) occ[q2] = 0;
                }
                std::sort(touched.begin(), touched.end());
                for (int q2 : touched) {
                    uint32_t *mk = &mark[(size_t)q2 * 4];
                    cand.push_back(make_int4(q1, q2, mask_id({mk[0], mk[1], mk[2], mk[3]}), 0));
                    mk[0] = mk[1] = mk[2] = mk[3] = 0u;
                }
                std::sort(extra.begin(), extra.end());
                for (size_t i = 0; i < extra.size();) {
                    std::array<uint32_t, 4> key = {0u, 0u, 0u, 0u};
                    size_t j = i;
                    for (; j < extra.size() && extra[j][0] == extra[i][0] && extra[j][1] == extra[i][1]; ++j)
                        key[extra[j][2] >> 5] |= 1u << (extra[j][2] & 31);
                    cand.push_back(make_int4(q1, extra[i][0], mask_id(key), 0));
                    i = j;
                }
            }
            nc64 = (int64_t)cand.size();
        }
        for (const auto &t : table) masks.insert(masks.end(), t.begin(), t.end());
        if (nc64 >= ((int64_t)1 << 31) - 1 || (int64_t)slist_n >= ((int64_t)1 << 31))
            return set_error(kErrBadDim, "too many three-phonon candidates for one call");
    }
    pt.mark("three-phonon candidates (host)");
    // ---- four-phonon candidates (scattering_fourphonon.f90:88-99): q2 from list a, q3 from
    // list b, q3 >= q2 and q4 = -q1-q2-q3 >= q3, once per q1 with the rows that sampled the
    // pair as a bit mask. Rows of q1 with identical lists share one pass over the pairs;
    // otherwise the pairs of all rows are merged by sorting. A pair that a row forms k times
    // (repeated points in its lists) is counted k times, as in the reference's double loop.
    std::vector<int4> cand4;
    std::vector<uint32_t> masks4;
    std::vector<int64_t> rbeg4;
    std::vector<int32_t> rlen4;
    if (o->fourthorder) {
        std::vector<std::array<uint32_t, 4>> table4;
        auto mask_id4 = [&](const std::array<uint32_t, 4> &key) {
            for (int t = (int)table4.size() - 1; t >= 0 && t >= (int)table4.size() - 8; --t)
                if (table4[t] == key) return t;
            table4.push_back(key);
            return (int)table4.size() - 1;
        };
        const int G0 = c->grid[0], G1 = c->grid[1], G2 = c->grid[2];
        auto wrap = [](int x, int m) {
            x %= m;
            return x < 0 ? x + m : x;
        };
        auto fourth = [&](int f1, int q2, int q3) {
            const int n12 = G1 * G2;
            const int i = wrap(-(f1 / n12) - (q2 / n12) - (q3 / n12), G0);
            const int j = wrap(-((f1 / G2) % G1) - ((q2 / G2) % G1) - ((q3 / G2) % G1), G1);
            const int k = wrap(-(f1 % G2) - (q2 % G2) - (q3 % G2), G2);
            return (i * G1 + j) * G2 + k;
        };
        std::vector<std::pair<int64_t, int>> keys;
        rbeg4.assign(nr, 0);
        rlen4.assign(nr, 0);
        for (int r0 = 0; r0 < nr;) {
            const int q1 = rq1[r0];
            int r1 = r0;
            while (r1 < nr && rq1[r1] == q1) ++r1;
            const int f1 = c->irr_full[q1] - 1;
            bool same = true;
            for (int r = r0; r < r1; ++r) {
                rbeg4[r] = ql->ptr4[r];
                rlen4[r] = (int32_t)(ql->ptr4[r + 1] - ql->ptr4[r]);

                if (r > r0) {
                    const int64_t L = rlen4[r0];
                    same = same && rlen4[r] == L &&
                           std::memcmp(ql->list4a + ql->ptr4[r], ql->list4a + ql->ptr4[r0], sizeof(int32_t) * L) == 0 &&
                           std::memcmp(ql->list4b + ql->ptr4[r], ql->list4b + ql->ptr4[r0], sizeof(int32_t) * L) == 0;
                }
            }
            if (same) {
                std::array<uint32_t, 4> key = {0u, 0u, 0u, 0u};
                for (int r = r0; r < r1; ++r) key[rb1[r] >> 5] |= 1u << (rb1[r] & 31);
                const int id = mask_id4(key);
                const int32_t *la = ql->list4a + ql->ptr4[r0], *lb = ql->list4b + ql->ptr4[r0];
                for (int64_t x = 0; x < rlen4[r0]; ++x)
                    for (int64_t y = 0; y < rlen4[r0]; ++y) {
                        const int q2 = la[x] - 1, q3 = lb[y] - 1;
                        if (q3 < q2 || fourth(f1, q2, q3) < q3) continue;
                        cand4.push_back(make_int4(q1, q2, q3, id));
                    }
            } else {
                keys.clear();
                for (int r = r0; r < r1; ++r) {
                    const int32_t *la = ql->list4a + ql->ptr4[r], *lb = ql->list4b + ql->ptr4[r];
                    for (int64_t x = 0; x < rlen4[r]; ++x)
                        for (int64_t y = 0; y < rlen4[r]; ++y) {
                            const int q2 = la[x] - 1, q3 = lb[y] - 1;
                            if (q3 < q2 || fourth(f1, q2, q3) < q3) continue;
                            keys.emplace_back((int64_t)q2 * N + q3, rb1[r]);
                        }
                }
                std::sort(keys.begin(), keys.end());
                for (size_t i = 0; i < keys.size();) {
                    size_t j = i;
                    while (j < keys.size() && keys[j].first == keys[i].first) ++j;
                    // entries i..j-1: the rows (sorted) that formed this pair, a row once per time
                    // it formed it; copy k goes to the rows with at least k entries
                    for (int k = 1;; ++k) {
                        std::array<uint32_t, 4> key = {0u, 0u, 0u, 0u};
                        bool any = false;
                        for (size_t x = i; x < j;) {
                            size_t y = x;
                            while (y < j && keys[y].second == keys[x].second) ++y;
                            if ((int)(y - x) >= k) {
                                key[keys[x].second >> 5] |= 1u << (keys[x].second & 31);
                                any = true;
                            }
                            x = y;
                        }
                        if (!any) break;
                        cand4.push_back(
                            make_int4(q1, (int)(keys[i].first / N), (int)(keys[i].first % N), mask_id4(key)));
                    }
                    i = j;
                }
            }
            if ((int64_t)cand4.size() >= ((int64_t)1 << 31) - 1)
                return set_error(kErrBadDim, "too many four-phonon candidates for one call");
            r0 = r1;
        }
        for (const auto &t : table4) masks4.insert(masks4.end(), t.begin(), t.end());
        if (ql->ptr4[nr] >= ((int64_t)1 << 31)) return set_error(kErrBadDim, "four-phonon samples too long for one call");
    }
    const int32_t nc4 = (int32_t)cand4.size();
    const int32_t nc = (int32_t)nc64;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    chk(c->d_be.upload(be.data(), be.size(), s));
    chk(c->d_sigsq.upload(sigsq.data(), sigsq.size(), s));
    std::vector<float> sigsq32(sigsq.begin(), sigsq.end());
    chk(c->d_sigsq32.upload(sigsq32.data(), sigsq32.size(), s));
    chk(c->d_rowidx.upload(rowidx.data(), rowidx.size(), s));
    chk(c->d_row_q1.upload(rq1.data(), rq1.size(), s));
    chk(c->d_row_b1.upload(rb1.data(), rb1.size(), s));
    chk(c->d_w3.upload(w3.data(), w3.size(), s));
    chk(c->d_w3q.upload(w3q.data(), w3q.size(), s));
    chk(c->d_w4.upload(w4.data(), w4.size(), s));
    const int64_t ld = (int64_t)N * n;
    const bool fuse_sym = o->thirdorder && !o->fourthorder && !o->isotope;
    if (o->thirdorder) chk(c->d_sbits.alloc((size_t)nr * ((N + 31) / 32)));
    chk(c->d_xi.alloc((size_t)nr * ld));
    chk(c->d_gamma.alloc(nr));
    if (o->thirdorder) {
        chk(c->d_mask.upload(masks.data(), masks.size(), s));
        chk(c->d_nt.alloc(nc + 1));
        chk(c->d_nrd.alloc(nc + 1));
        chk(c->d_toff.alloc(nc + 1));
        chk(c->d_roff.alloc(nc + 1));
        chk(c->d_tmp.alloc(exclusive_scan_tmp_elems(nc)));
        chk(c->d_rbeg.upload(rbeg.data(), rbeg.size(), s));
        chk(c->d_rlen.upload(rlen.data(), rlen.size(), s));
        if (shared) {
            chk(c->d_list3.upload(tl_slist.get(), slist_n, s));
            chk(c->d_qdesc.upload(qdesc.data(), qdesc.size(), s));
            chk(c->d_cand.alloc(nc));
            int maxL = 0;
            for (const auto &d : qdesc) maxL = std::max(maxL, d.y);
            chk(launch_build_candidates(c->d_qdesc.p, nirr, maxL, c->d_list3.p, c->d_cand.p, s));
        } else {
            chk(c->d_cand.upload(cand.data(), cand.size(), s));
            chk(c->d_list3.upload(ql->list3, ql->ptr3[nr], s));
        }
    }
    if (o->fourthorder) {
        chk(c->d_cand4.upload(cand4.data(), cand4.size(), s));
        chk(c->d_mask4.upload(masks4.data(), masks4.size(), s));
        chk(c->d_nq.alloc(nc4 + 1));
        chk(c->d_nrd4.alloc(nc4 + 1));
        chk(c->d_qoff.alloc(nc4 + 1));
        chk(c->d_roff4.alloc(nc4 + 1));
        chk(c->d_tmp4.alloc(exclusive_scan_tmp_elems(nc4)));
        chk(c->d_rbeg4.upload(rbeg4.data(), rbeg4.size(), s));
        chk(c->d_rlen4.upload(rlen4.data(), rlen4.size(), s));
        chk(c->d_list4a.upload(ql->list4a, ql->ptr4[nr], s));
        chk(c->d_od.alloc((size_t)nr * ld));
    }
    chk(cudaStreamSynchronize(s));
    pt.mark("allocations and uploads");
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("allocation/upload failed: ") + cudaGetErrorString(e));
    ph.be = c->d_be.p;
    ph.sigsq = c->d_sigsq.p;
    ph.sigsq32 = c->d_sigsq32.p;
    RowsDev rows;
    std::memset(&rows, 0, sizeof rows);
    rows.n_row = nr;
    rows.rowidx = c->d_rowidx.p;
    rows.weight3 = c->d_w3.p;
    rows.w3q = c->d_w3q.p;
    rows.weight4 = c->d_w4.p;
    const MeshDev mesh = c->mesh();

    // ---- device pipeline; inputs are resident from here on ----
    cudaEvent_t *ev = c->ev;
    int launches = 0;
    // Xi starts at zero and the three-phonon row terms accumulate into it directly: the
    // per-order symmetrisation (od_terms > 0 filter) then runs on Xi in place, and the
    // isotope terms, which the reference adds unsymmetrised, come after it.
    CUDA_TRY(cudaEventRecord(ev[0], s));
    CUDA_TRY(cudaMemsetAsync(c->d_xi.p, 0, sizeof(double) * (size_t)nr * ld, s));
    c->xi_fmt = -1;
    CUDA_TRY(cudaMemsetAsync(c->d_gamma.p, 0, sizeof(double) * nr, s));
    CUDA_TRY(cudaMemsetAsync(c->d_status.p, 0, sizeof(int32_t), s));
    CUDA_TRY(cudaEventRecord(ev[1], s));
    int32_t ntrip = 0, nred = 0;
    if (o->thirdorder) {
        CUDA_TRY(launch_triplet_count(mesh, c->d_cand.p, nc, c->d_nt.p, c->d_nrd.p, c->d_status.p, s));
        CUDA_TRY(exclusive_scan_i32(c->d_nt.p, c->d_toff.p, nc, c->d_tmp.p, s));
        CUDA_TRY(exclusive_scan_i32(c->d_nrd.p, c->d_roff.p, nc, c->d_tmp.p, s));
        launches += 1 + 2 * 3;
        int32_t *tot = c->h_tot;
        CUDA_TRY(copy_async(&tot[0], c->d_toff.p + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(copy_async(&tot[1], c->d_roff.p + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        st = read_status(c);
        if (st) return st;
        ntrip = tot[0];
        nred = tot[1];
        chk(c->d_trip.alloc(ntrip));
        chk(c->d_red.alloc(nred));
        if (e != cudaSuccess) return set_error(kErrDevice, std::string("allocation failed: ") + cudaGetErrorString(e));
        CUDA_TRY(launch_triplet_fill(mesh, c->d_cand.p, nc, c->d_toff.p, c->d_roff.p, c->d_trip.p, c->d_red.p, s));
        ++launches;
        CUDA_TRY(cudaEventRecord(ev[2], s));
        ThreePhArgs a;
        std::memset(&a, 0, sizeof a);
        a.mesh = mesh;
        a.ph = ph;
        a.rows = rows;
        a.fc.n = c->n_fc3;
        a.fc.n_atom = c->na;
        a.fc.blk_ptr = c->fc3_blk.p;
        a.fc.lv = c->fc3_lv.p;
        a.fc.mwm = c->fc3_mwm.p;
        a.fc.mwm32 = c->fc3_mwm32.p;
        a.fc.twiddle = c->tw.p;
        a.fc.twiddle32 = c->tw32.p;
        a.fc.abase = c->fc3_abase.p;
        a.lam = nullptr;
        a.mwm_bar = nullptr;
        a.acc_in_smem = 0;
        a.trip = c->d_trip.p;
        a.n_trip = ntrip;
        a.red = c->d_red.p;
        a.cand_mask = c->d_mask.p;
        a.gamma = c->d_gamma.p;
        a.od = c->d_xi.p;
        a.status = c->d_status.p;
        c->last_ln = n > 18 || o->tensor_cores == 1;
        const char *tc_env = std::getenv("TDG_TC_SMALL");
        const bool use_tc = !c->last_ln && o->tensor_cores != 2 && !(tc_env && tc_env[0] == '0') &&
                            threephonon_tc_supported(n, o->precision, c->n_fc3) && c->tc_plan.slots > 0;
        c->last_path = c->last_ln ? 2 : (use_tc ? 1 : 0);
        if (use_tc) {
            if (!c->tc_eimg_ready) {
                chk(c->d_tc_eimg.alloc((size_t)N * 4096));
                if (e != cudaSuccess)
                    return set_error(kErrDevice, std::string("allocation failed: ") + cudaGetErrorString(e));
                CUDA_TRY(launch_tc_eimg(N, n, c->d_egvs32.p, c->d_tc_eimg.p, s));
                c->tc_eimg_ready = true;
            }
            a.tc_eimg = c->d_tc_eimg.p;
        }
        // the launch shape comes first (autotuner trials run outside any graph), then the
        // three-phonon part of the pipeline runs directly or as the context's graph
        // graph key: every value the recorded launches bake in (kernel-argument bytes, with
        // the device buffers' addresses, and the launch shape)
        std::function<cudaError_t()> body3;
        std::ostringstream gk;
        gk << n << '/' << ntrip << '/' << o->precision << '/' << c->n_sm << '/';
        LnBatch b;
        int nbmax = 0, cps = 0;
        if (c->last_ln) {
            // large-cell path: batches of q-triplets through the tcgen05 contraction
            st = ln_batch_setup(c, mesh, ph, rows, a.fc, ntrip, b, nbmax);
            if (st) return st;
            // launch shape (delta row block, GEMM pipeline depth), timed on the first slots
            {
                const std::string key = tune_key("largecell", n, o->precision, c->device);
                int v = kLnTuneDefault;
                bool tuned = false;
                LnBatch tb = b;
                tb.trip = c->d_trip.p;
                tb.nb = std::min(std::min(nbmax, ntrip), 16);
                CUDA_TRY(tune_pick(key, {324, 164, 323, 163}, kLnTuneDefault,
                                   [&](int cand) {
                                       ln_apply_tune(tb, cand);
                                       return launch_ln_batch(tb, s);
                                   },
                                   s, v, tuned));
                if (tuned) CUDA_TRY(rezero_outputs(c, nr, ld, s));
                ln_apply_tune(b, v);
                c->last_ln_tune = v;
            }
            gk << "ln" << c->last_ln_tune << '/' << nbmax << '/' << (const void *)c->d_trip.p << '/'
               << std::string(reinterpret_cast<const char *>(&b), sizeof b);
            body3 = [&]() -> cudaError_t {
                for (int t0 = 0; t0 < ntrip; t0 += nbmax) {
                    LnBatch bt = b;
                    bt.trip = c->d_trip.p + t0;
                    bt.nb = std::min(nbmax, ntrip - t0);
                    const cudaError_t e = launch_ln_batch(bt, s);
                    if (e != cudaSuccess) return e;
                }
                return cudaSuccess;
            };
            launches += 6 * ((ntrip + nbmax - 1) / std::max(nbmax, 1));
        } else {
            // persistent grid (CTAs per SM), timed on a prefix of the q-triplets
            int occ_api = 0, occ_count = 0;
            const int maxps = use_tc ? threephonon_tc_max_per_sm(n, c->n_fc3, &occ_api, &occ_count)
                                     : threephonon_max_per_sm(n, o->precision, &occ_api, &occ_count);
            std::vector<int> cand;
            for (int v : {maxps, (3 * maxps + 3) / 4, (maxps + 1) / 2})
                if (v >= 1 && std::find(cand.begin(), cand.end(), v) == cand.end()) cand.push_back(v);
            const std::string key = tune_key(use_tc ? "threephonon_tc" : "threephonon", n, o->precision, c->device);
            // the plan of the kernel in use (the SIMT kernel's in FP32 only)
            tdg_ctx::Plan *plan = use_tc ? &c->tc_plan
                                         : (o->precision != TDG_PREC_FP64 && c->simt_plan.slots > 0 ? &c->simt_plan
                                                                                                  : nullptr);
            if (plan) {
                a.plan_pm = plan->pm.p;
                a.plan_word = plan->word.p;
                a.plan_slots = plan->slots;
            }
            auto fused = [&, use_tc, plan](const ThreePhArgs &x, int v) -> cudaError_t {
                if (plan) {
                    const cudaError_t ep =
                        launch_fill_plan(plan->src.p, plan->slots, plan->threads, c->fc3_mwm32.p, plan->pm.p, s);
                    if (ep != cudaSuccess) return ep;
                }
                if (!use_tc) return launch_threephonon(x, o->precision, c->n_sm, v, s);
                return launch_threephonon_tc(x, c->n_sm, v, s);
            };
            bool tuned = false;
            ThreePhArgs ta = a;
            ta.n_trip = std::min(ntrip, std::max(ntrip / 8, 64 * c->n_sm * std::max(maxps, 1)));
            CUDA_TRY(tune_pick(key, cand, 0, [&](int v) { return fused(ta, v); }, s, cps, tuned));
            if (tuned) CUDA_TRY(rezero_outputs(c, nr, ld, s));
            gk << (use_tc ? "t" : "f") << cps << '/' << std::string(reinterpret_cast<const char *>(&a), sizeof a);
            body3 = [&, fused]() { return fused(a, cps); };
            launches += plan ? 2 : 1;
            const int used = (cps > 0 && cps < maxps) ? cps : maxps;
            c->last_launch[0] = (int)std::min<int64_t>((int64_t)c->n_sm * used, std::max(ntrip, 1));
            c->last_launch[1] = used;
            c->last_launch[2] = occ_api;
            c->last_launch[3] = occ_count;
        }
        CUDA_TRY(run_graph_region(c, c->graph3, gk.str(), s, body3));
        // (events recorded inside a graph cannot be timed against the others: ev[3] stays out)
        CUDA_TRY(cudaEventRecord(ev[3], s));
        CUDA_TRY(launch_sample_bits(N, nr, c->d_rbeg.p, c->d_rlen.p, c->d_list3.p, c->d_sbits.p, s));
        ++launches;
        // without four-phonon or isotope terms in between, the three-phonon distribution
        // runs in the same pass as symmetrize_scatmat below
        if (!fuse_sym) {
            CUDA_TRY(launch_sym_tile(mesh, c->orbits, nr, c->d_row_q1.p, c->d_xi.p, c->d_sbits.p, true, false, s));
            ++launches;
        }
    } else {
        CUDA_TRY(cudaEventRecord(ev[2], s));
        CUDA_TRY(cudaEventRecord(ev[3], s));
    }
    CUDA_TRY(cudaEventRecord(ev[7], s));
    // Four-phonon row terms go to their own od buffer: the per-order symmetrisation is not
    // linear (od_terms > 0 filter), so it runs on od alone and then adds od into Xi.
    int32_t nquart = 0, nred4 = 0;
    if (o->fourthorder) {
        CUDA_TRY(cudaMemsetAsync(c->d_od.p, 0, sizeof(double) * (size_t)nr * ld, s));
        CUDA_TRY(launch_quartet_count(mesh, c->d_cand4.p, nc4, c->d_nq.p, c->d_nrd4.p, c->d_status.p, s));
        CUDA_TRY(exclusive_scan_i32(c->d_nq.p, c->d_qoff.p, nc4, c->d_tmp4.p, s));
        CUDA_TRY(exclusive_scan_i32(c->d_nrd4.p, c->d_roff4.p, nc4, c->d_tmp4.p, s));
        launches += 1 + 2 * 3;
        int32_t *tot = c->h_tot;
        CUDA_TRY(copy_async(&tot[0], c->d_qoff.p + nc4, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(copy_async(&tot[1], c->d_roff4.p + nc4, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        st = read_status(c);
        if (st) return st;
        nquart = tot[0];
        nred4 = tot[1];
        const int grid4 = fourphonon_grid(n, o->precision, c->n_sm, nquart);
        if (nquart > 0 && grid4 < 1) return set_error(kErrDevice, "four-phonon kernel configuration failed");
        chk(c->d_quart.alloc(nquart));
        chk(c->d_red4.alloc(nred4));
        chk(c->d_scr4.alloc(fourphonon_scratch_bytes(n, o->precision, grid4)));
        if (e != cudaSuccess) return set_error(kErrDevice, std::string("allocation failed: ") + cudaGetErrorString(e));
        CUDA_TRY(launch_quartet_fill(mesh, c->d_cand4.p, nc4, c->d_qoff.p, c->d_roff4.p, c->d_quart.p, c->d_red4.p, s));
        ++launches;
        CUDA_TRY(cudaEventRecord(ev[8], s));
        FourPhArgs a4;
        a4.mesh = mesh;
        a4.ph = ph;
        a4.rows = rows;
        a4.fc.n = c->n_fc4;
        a4.fc.n_atom = c->na;
        a4.fc.blk_ptr = c->fc4_blk.p;
        a4.fc.lv = c->fc4_lv.p;
        a4.fc.mwm = c->fc4_mwm.p;
        a4.fc.mwm32 = c->fc4_mwm32.p;
        a4.twiddle = c->tw.p;
        a4.twiddle32 = c->tw32.p;
        a4.quart = c->d_quart.p;
        a4.n_quart = nquart;
        a4.red = c->d_red4.p;
        a4.cand_mask = c->d_mask4.p;
        a4.gamma = c->d_gamma.p;
        a4.od = c->d_od.p;
        a4.status = c->d_status.p;
        a4.scratch = c->d_scr4.p;
        CUDA_TRY(launch_fourphonon(a4, o->precision, grid4, s));
        ++launches;
        CUDA_TRY(cudaEventRecord(ev[9], s));
        CUDA_TRY(launch_sym_distribute(mesh, c->orbits, nr, c->d_row_q1.p, c->d_rbeg4.p, c->d_rlen4.p, c->d_list4a.p,
                                       c->d_od.p, c->d_xi.p, s));
        ++launches;
    } else {
        CUDA_TRY(cudaEventRecord(ev[8], s));
        CUDA_TRY(cudaEventRecord(ev[9], s));
    }
    CUDA_TRY(cudaEventRecord(ev[4], s));
    if (o->isotope) {
        CUDA_TRY(launch_isotope(mesh, ph, rows, c->d_row_q1.p, c->d_row_b1.p, c->d_disorder.p, c->na, c->d_gamma.p,
                                c->d_xi.p, s));
        ++launches;
    }
    CUDA_TRY(cudaEventRecord(ev[5], s));
    // ---- gamma to host; symmetrize_scatmat on the device meanwhile ----
    std::vector<double> gamma(nr);
    CUDA_TRY(copy_async(gamma.data(), c->d_gamma.p, sizeof(double) * nr, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(launch_sym_tile(mesh, c->orbits, nr, c->d_row_q1.p, c->d_xi.p, c->d_sbits.p, fuse_sym, true, s));
    ++launches;
    CUDA_TRY(cudaEventRecord(ev[6], s));
    CUDA_TRY(cudaStreamSynchronize(s));
    pt.mark("device pipeline");
    st = read_status(c);
    if (st) return st;
    float ms_total = 0.f, ms_iso = 0.f, ms_k1 = 0.f, ms_fused = 0.f, ms_sym = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms_total, ev[0], ev[6]));
    CUDA_TRY(cudaEventElapsedTime(&ms_iso, ev[4], ev[5]));
    CUDA_TRY(cudaEventElapsedTime(&ms_k1, ev[1], ev[2]));
    CUDA_TRY(cudaEventElapsedTime(&ms_fused, ev[2], ev[3]));
    float ms_s1 = 0.f, ms_s2 = 0.f, ms_s3 = 0.f, ms_k1q = 0.f, ms_f4 = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms_s1, ev[3], ev[7]));
    CUDA_TRY(cudaEventElapsedTime(&ms_k1q, ev[7], ev[8]));
    CUDA_TRY(cudaEventElapsedTime(&ms_f4, ev[8], ev[9]));
    CUDA_TRY(cudaEventElapsedTime(&ms_s3, ev[9], ev[4]));
    CUDA_TRY(cudaEventElapsedTime(&ms_s2, ev[5], ev[6]));
    ms_sym = ms_s1 + ms_s2 + ms_s3;
    ms_k1 += ms_k1q;
    ms_fused += ms_f4;

    // ---- boundary, degeneracy averaging (scattering.f90:244-292) ----
    std::vector<double> buf_lw((size_t)nirr * n, 0.0);
    for (int r = 0; r < nr; ++r) {
        double b = gamma[r];
        if (o->mfp_max > 0.0) {
            const int f = c->irr_full[rq1[r]] - 1;
            const double *v = &c->vel[((size_t)f * n + rb1[r]) * 3];
            const double vn = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (vn > kGroupVelTol) b += vn / o->mfp_max;
        }
        buf_lw[(size_t)rq1[r] * n + rb1[r]] = b;
    }
    c->linewidth.assign((size_t)nirr * n, 0.0);
    c->qs.assign((size_t)nirr * n, 0.0);
    c->F0.assign((size_t)nirr * n * 3, 0.0);
    c->Fn.assign((size_t)nirr * n * 3, 0.0);
    for (int q1 = 0; q1 < nirr; ++q1) {
        const int f = c->irr_full[q1] - 1;
        for (int b1 = 0; b1 < n; ++b1) {
            if (c->omega[(size_t)f * n + b1] < kFreqTol) continue;
            const int dg = c->degen[(size_t)f * n + b1];
            const int32_t *dm = &c->degen_mode[((size_t)f * n + b1) * n];
            double f0 = 0.0;
            for (int j = 0; j < dg; ++j) f0 += buf_lw[(size_t)q1 * n + dm[j] - 1];
            f0 /= (double)dg;
            for (int j = 0; j < dg; ++j) buf_lw[(size_t)q1 * n + dm[j] - 1] = f0;
            const double lw = buf_lw[(size_t)q1 * n + b1];
            c->linewidth[(size_t)q1 * n + b1] = lw;
            c->qs[(size_t)q1 * n + b1] = 2.0 * lw;
            if (lw > kFreqTol) {
                const double *v = &c->vel[((size_t)f * n + b1) * 3];
                for (int d = 0; d < 3; ++d) {
                    const double mfp = v[d] / c->qs[(size_t)q1 * n + b1];
                    c->F0[((size_t)q1 * n + b1) * 3 + d] = mfp;
                    c->Fn[((size_t)q1 * n + b1) * 3 + d] = mfp;
                }
            }
        }
    }
    std::memcpy(linewidth, c->linewidth.data(), sizeof(double) * c->linewidth.size());
    if (qs_out) std::memcpy(qs_out, c->qs.data(), sizeof(double) * c->qs.size());
    if (stats) {
        stats[0] = ntrip;
        stats[1] = nquart;
        stats[2] = ms_total;
        stats[3] = (double)nc + (double)nc4;
        stats[4] = ms_k1;
        stats[5] = ms_fused;
        stats[6] = ms_sym;
        stats[7] = ms_iso;
        stats[8] = launches;
        stats[9] = (double)nred + (double)nred4;
    }
    c->last_ph = ph;
    c->last_rows = rows;
    c->last_ntrip = ntrip;
    c->last_third = o->thirdorder != 0;
    c->last_prec = o->precision;
    c->have_scattering = true;
    c->fn_iter = false;
    c->xi_bar_ready = false;
    pt.mark("linewidths and F0 (host)");
    return kOk;
}

extern "C" int tdg_get_xi(tdg_ctx *c, double *xi) {
    XferScope xs(c ? c->xfer : nullptr);
    PoolScope pscope(c ? c->stream : nullptr, c ? c->pool : nullptr);
    if (!c || !xi) return set_error(kErrParam, "tdg_get_xi: null argument");
    if (!c->have_scattering) return set_error(kErrParam, "tdg_get_xi: call tdg_scattering first");
    CUDA_TRY(cudaSetDevice(c->device));
    const size_t cnt = (size_t)c->n_row * c->N * c->n;
    CUDA_TRY(copy_async(xi, c->d_xi.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return kOk;
}

extern "C" int tdg_triplets(tdg_ctx *c, int32_t q1, const int32_t *sample, int64_t n, int32_t *out, int64_t cap,
                            int64_t *written) {
    XferScope xs(c ? c->xfer : nullptr);
    PoolScope pscope(c ? c->stream : nullptr, c ? c->pool : nullptr);
    if (!c || !sample || !out || !written) return set_error(kErrParam, "tdg_triplets: null argument");
    if (q1 < 1 || q1 > c->nirr) return set_error(kErrParam, "tdg_triplets: q1 out of range");
    if (n < 0 || n > (int64_t)1 << 30) return set_error(kErrParam, "tdg_triplets: bad sample length");
    for (int64_t i = 0; i < n; ++i)
        if (sample[i] < 1 || sample[i] > c->N) return set_error(kErrParam, "tdg_triplets: q' index out of range");
    CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const int32_t nc = (int32_t)n;
    std::vector<int4> cand(nc);
    for (int32_t i = 0; i < nc; ++i) cand[i] = make_int4(q1 - 1, sample[i] - 1, 0, 0);
    DevBuf<int4> d_cand;
    DevBuf<int32_t> d_nt, d_nrd, d_toff, d_roff, d_tmp;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    chk(d_cand.upload(cand.data(), cand.size(), s));
    chk(d_nt.alloc(nc + 1));
    chk(d_nrd.alloc(nc + 1));
    chk(d_toff.alloc(nc + 1));
    chk(d_roff.alloc(nc + 1));
    chk(d_tmp.alloc(exclusive_scan_tmp_elems(nc)));
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("allocation failed: ") + cudaGetErrorString(e));
    const MeshDev mesh = c->mesh();
    CUDA_TRY(cudaMemsetAsync(c->d_status.p, 0, sizeof(int32_t), s));
    CUDA_TRY(launch_triplet_count(mesh, d_cand.p, nc, d_nt.p, d_nrd.p, c->d_status.p, s));
    CUDA_TRY(exclusive_scan_i32(d_nt.p, d_toff.p, nc, d_tmp.p, s));
    CUDA_TRY(exclusive_scan_i32(d_nrd.p, d_roff.p, nc, d_tmp.p, s));
    int32_t tot[2] = {0, 0};
    CUDA_TRY(copy_async(&tot[0], d_toff.p + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(copy_async(&tot[1], d_roff.p + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    int st = read_status(c);
    if (st) return st;
    DevBuf<TripletRec> d_trip;
    DevBuf<int2> d_red;
    // four-phonon enumeration, samples (list a drives the symmetrisation) and kernel scratch
    DevBuf<int4> d_cand4, d_red4;
    DevBuf<uint32_t> d_mask4;
    DevBuf<int32_t> d_nq, d_nrd4, d_qoff, d_roff4, d_tmp4, d_list4a, d_rlen4;
    DevBuf<int64_t> d_rbeg4;
    DevBuf<QuartetRec> d_quart;
    DevBuf<unsigned char> d_scr4;
    chk(d_trip.alloc(tot[0]));
    chk(d_red.alloc(tot[1]));
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("allocation failed: ") + cudaGetErrorString(e));
    CUDA_TRY(launch_triplet_fill(mesh, d_cand.p, nc, d_toff.p, d_roff.p, d_trip.p, d_red.p, s));
    std::vector<TripletRec> trip(tot[0]);
    std::vector<int2> red(tot[1]);
    if (tot[0] > 0)
        CUDA_TRY(copy_async(trip.data(), d_trip.p, sizeof(TripletRec) * tot[0], cudaMemcpyDeviceToHost, s));
    if (tot[1] > 0) CUDA_TRY(copy_async(red.data(), d_red.p, sizeof(int2) * tot[1], cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    int64_t w = 0;
    for (const auto &t : trip) {
        if (w + 3 + 2 * (int64_t)t.red_cnt > cap) return set_error(kErrParam, "tdg_triplets: output capacity too small");
        out[w++] = t.q2 + 1;
        out[w++] = t.q3 + 1;
        out[w++] = t.red_cnt;
        for (int k = 0; k < t.red_cnt; ++k) {
            out[w++] = red[t.red_off + k].x + 1;
            out[w++] = red[t.red_off + k].y + 1;
        }
    }
    *written = w;
    return kOk;
}

namespace {

// get_kappa (kappa.f90:28-75). The reference symmetrises every mode's F (x) v over the
// operations, (1/nop) sum_R (R F) (x) (R v) = (1/nop) sum_R R (F (x) v) R^T; that map is
// linear, so the per-mode tensors are summed first and the operations applied once.
void get_kappa(const tdg_ctx *c, const std::vector<double> &Fn, double T, bool classical, double *kappa) {
    const int n = c->n;
    double M[9] = {0};
    for (int q1 = 0; q1 < c->nirr; ++q1) {
        const int f = c->irr_full[q1] - 1;
        for (int b1 = 0; b1 < n; ++b1) {
            const double om1 = c->omega[(size_t)f * n + b1];
            if (om1 < kFreqTol) continue;
            const double cv = classical ? kKbHartree : harmonic_oscillator_cv(T, om1);
            const double w = cv / c->volume * c->irr_weight[q1];
            const double *F = &Fn[((size_t)q1 * n + b1) * 3];
            const double *v = &c->vel[((size_t)f * n + b1) * 3];
            for (int x = 0; x < 3; ++x)
                for (int y = 0; y < 3; ++y) M[x + 3 * y] += w * F[x] * v[y];
        }
    }
    for (int i = 0; i < 9; ++i) kappa[i] = 0.0;
    for (int j = 0; j < c->nop; ++j) {
        const double *m = &c->op_cart[9 * j];
        for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k)
                    for (int l = 0; l < 3; ++l) s += m[x + 3 * k] * M[k + 3 * l] * m[y + 3 * l];
                kappa[x + 3 * y] += s / c->nop;
            }
    }
    double tol = 0.0;
    for (int k = 0; k < 9; ++k) tol += std::fabs(kappa[k]);
    tol *= 1e-6;
    for (int k = 0; k < 9; ++k) kappa[k] = lo_chop(kappa[k], tol);
}

// symmetrize_kappa (kappa.f90:308-324): average of R kappa R^T over the operations.
void symmetrize_kappa(const tdg_ctx *c, double *kappa) {
    double tmp[9] = {0};
    for (int o = 0; o < c->nop; ++o) {
        const double *m = &c->op_cart[9 * o];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k)
                    for (int l = 0; l < 3; ++l) s += m[i + 3 * k] * kappa[k + 3 * l] * m[j + 3 * l];
                tmp[i + 3 * j] += s;
            }
    }
    double tol = 0.0;
    for (int k = 0; k < 9; ++k) {
        kappa[k] = tmp[k] / c->nop;
        tol += std::fabs(kappa[k]);
    }
    tol *= 1e-6;
    for (int k = 0; k < 9; ++k) kappa[k] = lo_chop(kappa[k], tol);
}

}  // namespace

extern "C" int tdg_kappa(tdg_ctx *c, const tdg_opts *o, int32_t maxiter, double tol, double *kappa_sma,
                         double *kappa_iter, double *fn_out, int32_t *n_iter) {
    XferScope xs(c ? c->xfer : nullptr);
    PoolScope pscope(c ? c->stream : nullptr, c ? c->pool : nullptr);
    if (!c || !kappa_sma || !kappa_iter) return set_error(kErrParam, "tdg_kappa: null argument");
    int st = validate_opts(o);
    if (st) return st;
    if (!c->have_scattering) return set_error(kErrParam, "tdg_kappa: call tdg_scattering first");
    if (maxiter < 0) return set_error(kErrParam, "tdg_kappa: negative iteration count");
    CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const int n = c->n, N = c->N, nirr = c->nirr, nr = c->n_row;
    const bool classical = o->classical != 0;
    const double T = o->temperature;
    if (T < kTemperatureTol) {
        for (int i = 0; i < 9; ++i) kappa_sma[i] = kappa_iter[i] = 0.0;
        if (n_iter) *n_iter = 0;
        return kOk;
    }
    ++c->kappa_calls;
    // Every call starts from Fn = F0, the state sr%generate leaves (scattering.f90:288-289).
    std::vector<double> Fn = c->F0;
    get_kappa(c, Fn, T, classical, kappa_sma);
    int iters = 0;
    if (maxiter > 0) {
        const int64_t ncol = (int64_t)N * n;
        const size_t nfn = (size_t)nirr * n * 3, nbuf = (size_t)nr * 3;
        CUDA_TRY(c->d_fbb.alloc((size_t)ncol * 3));
        // the Xi.F products take Xi as double-float row pairs (k_xi_gemv; floats fail the
        // mixed iteration's convergence test)
        if (c->xi_fmt != 1) {
            CUDA_TRY(c->d_xi_df.alloc(xi_pairs_elems(nr, ncol)));
            CUDA_TRY(launch_split_xi(c->d_xi.p, nr, ncol, c->d_xi_df.p, s));
            c->xi_fmt = 1;
        }
        CUDA_TRY(c->d_buf.alloc(nbuf));
        CUDA_TRY(c->d_part.alloc(xi_gemv_part_elems(nr)));
        CUDA_TRY(c->d_fn.alloc(nfn));
        if (c->d_full_op.n == 0) {
            CUDA_TRY(c->d_full_op.upload(c->full_op.data(), N, s));
            CUDA_TRY(c->d_op_cart.upload(c->op_cart.data(), c->op_cart.size(), s));
        }
        // The whole iteration runs on the device (kappa.f90:382-490): foldout, the three Xi
        // products and the scalar recurrences (k_bte_update), in chunks of kBteChunk
        // iterations between host checks of the done flag; a chunk is replayed as a CUDA
        // graph from its second use. Fn goes up once and comes back once.
        if (c->d_deg_irr.n == 0) {
            std::vector<int32_t> dg((size_t)nirr * n), dm((size_t)nirr * n * n);
            for (int q1 = 0; q1 < nirr; ++q1) {
                const int f = c->irr_full[q1] - 1;
                for (int b1 = 0; b1 < n; ++b1) {
                    dg[(size_t)q1 * n + b1] = c->degen[(size_t)f * n + b1];
                    for (int j = 0; j < n; ++j)
                        dm[((size_t)q1 * n + b1) * n + j] = c->degen_mode[((size_t)f * n + b1) * n + j];
                }
            }
            CUDA_TRY(c->d_deg_irr.upload(dg.data(), dg.size(), s));
            CUDA_TRY(c->d_dm_irr.upload(dm.data(), dm.size(), s));
        }
        CUDA_TRY(c->d_fnb.alloc(nfn));
        CUDA_TRY(c->d_scf.alloc((size_t)maxiter));
        CUDA_TRY(c->d_ctl.alloc(1));
        CUDA_TRY(c->d_bte_part.alloc((size_t)bte_part_elems(nirr)));
        CUDA_TRY(c->d_qs_bte.upload(c->qs.data(), c->qs.size(), s));
        CUDA_TRY(c->d_F0.upload(c->F0.data(), nfn, s));
        CUDA_TRY(copy_async(c->d_fn.p, Fn.data(), sizeof(double) * nfn, cudaMemcpyHostToDevice, s));
        const BteCtl ctl0{0, 0, 0.95};
        CUDA_TRY(copy_async(c->d_ctl.p, &ctl0, sizeof(BteCtl), cudaMemcpyHostToDevice, s));
        BteDev bd;
        std::memset(&bd, 0, sizeof bd);
        bd.n_irr = nirr;
        bd.n_mode = n;
        bd.n_row = nr;
        bd.maxiter = maxiter;
        bd.tol = tol;
        bd.sqtol = kSqTol;
        bd.rowidx = c->d_rowidx.p;
        bd.part = c->d_bte_part.p;
        bd.qs = c->d_qs_bte.p;
        bd.F0 = c->d_F0.p;
        bd.degen = c->d_deg_irr.p;
        bd.degen_mode = c->d_dm_irr.p;
        bd.fn = c->d_fn.p;
        bd.fnb = c->d_fnb.p;
        bd.scf = c->d_scf.p;
        bd.ctl = c->d_ctl.p;
        const int32_t *done = &c->d_ctl.p->done;
        // column split of the Xi products, autotuned per problem size on F0's foldout
        int split = 0;
        {
            CUDA_TRY(launch_foldout(N, n, c->d_full_op.p, c->d_full_irr.p, c->d_op_cart.p, c->d_fn.p, c->d_fbb.p, s));
            // shapes: rows per CTA (4, 8) * 100 + column ranges (the default, twice it)
            const int s0 = xi_gemv_default_split(nr, ncol, c->n_sm), smax = xi_gemv_max_split(ncol);
            std::vector<int> cand;
            for (int rows : {4, 8})
                for (int v : {s0, 2 * s0})
                    if (v <= smax && std::find(cand.begin(), cand.end(), rows * 100 + v) == cand.end())
                        cand.push_back(rows * 100 + v);
            std::ostringstream key;
            key << "xigemv2/r" << nr << "/c" << ncol;
            bool tuned = false;
            CUDA_TRY(tune_pick(tune_key(key.str().c_str(), n, 0, c->device), cand, 400 + s0,
                               [&](int v) {
                                   return launch_xi_gemv(c->d_xi_df.p, nr, ncol, c->d_fbb.p, c->d_part.p,
                                                         c->d_buf.p, c->n_sm, s, nullptr, v);
                               },
                               s, split, tuned));
        }
        auto iterations = [&](int k) -> cudaError_t {
            for (int j = 0; j < k; ++j) {
                cudaError_t e = launch_foldout(N, n, c->d_full_op.p, c->d_full_irr.p, c->d_op_cart.p, c->d_fn.p,
                                               c->d_fbb.p, s, done);
                if (e == cudaSuccess)
                    e = launch_xi_gemv(c->d_xi_df.p, nr, ncol, c->d_fbb.p, c->d_part.p, c->d_buf.p, c->n_sm, s,
                                       done, split);
                if (e == cudaSuccess) e = launch_bte_update(bd, c->d_buf.p, s);
                if (e != cudaSuccess) return e;
            }
            return cudaSuccess;
        };
        BteCtl ctl = ctl0;
        PhaseTimer pt("tdg_kappa");
        for (int it0 = 0; it0 < maxiter; it0 += kBteChunk) {
            const int k = std::min(kBteChunk, maxiter - it0);
            std::ostringstream key;
            key << k << '/' << split << '/' << std::string(reinterpret_cast<const char *>(&bd), sizeof bd)
                << '/'
                << (const void *)c->d_xi_df.p << (const void *)c->d_fbb.p << (const void *)c->d_part.p
                << (const void *)c->d_buf.p << (const void *)c->d_fn.p << ncol;
            // recorded only from the context's second kappa call on: a context that solves
            // once would pay for the recording without replaying it much
            CUDA_TRY(run_graph_region(c, c->graph_bte, key.str(), s, [&]() { return iterations(k); },
                                      c->kappa_calls > 1));
            CUDA_TRY(copy_async(&ctl, c->d_ctl.p, sizeof(BteCtl), cudaMemcpyDeviceToHost, s));
            CUDA_TRY(cudaStreamSynchronize(s));
            pt.mark("iterations (device)");
            if (ctl.done) break;
        }
        iters = ctl.iter;
        CUDA_TRY(copy_async(Fn.data(), c->d_fn.p, sizeof(double) * nfn, cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
    }
    get_kappa(c, Fn, T, classical, kappa_iter);
    symmetrize_kappa(c, kappa_iter);
    symmetrize_kappa(c, kappa_sma);
    c->Fn = Fn;
    c->fn_iter = maxiter > 0;
    c->xi_bar_ready = false;
    if (fn_out) std::memcpy(fn_out, Fn.data(), sizeof(double) * Fn.size());
    if (n_iter) *n_iter = iters;
    return kOk;
}

tdg::CtxView tdg::ctx_view(tdg_ctx *c) {
    CtxView v;
    v.device = c->device;
    v.stream = c->stream;
    v.mesh = c->mesh();
    v.xfer = c->xfer;
    return v;
}

extern "C" int tdg_set_fc3(tdg_ctx *c, const double *fc3_mwm) {
    XferScope xs(c ? c->xfer : nullptr);
    PoolScope pscope(c ? c->stream : nullptr, c ? c->pool : nullptr);
    if (!c || !fc3_mwm) return set_error(kErrParam, "tdg_set_fc3: null argument");
    if (c->n_fc3 < 1) return set_error(kErrParam, "tdg_set_fc3: the context has no third-order force constants");
    const size_t cnt = (size_t)c->n_fc3 * 27;
    for (size_t i = 0; i < cnt; ++i)
        if (!std::isfinite(fc3_mwm[i])) return set_error(kErrPhysical, "tdg_set_fc3: non-finite force constant");
    std::vector<double> m(cnt);
    std::vector<float> mf(cnt);
    for (int sidx = 0; sidx < c->n_fc3; ++sidx) {
        const int t = c->fc3_perm[sidx];
        for (int k = 0; k < 27; ++k) {
            m[(size_t)sidx * 27 + k] = fc3_mwm[(size_t)t * 27 + k];
            mf[(size_t)sidx * 27 + k] = (float)fc3_mwm[(size_t)t * 27 + k];
        }
    }
    CUDA_TRY(cudaSetDevice(c->device));
    CUDA_TRY(c->fc3_mwm.upload(m.data(), cnt, c->stream));
    CUDA_TRY(c->fc3_mwm32.upload(mf.data(), cnt, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->have_scattering = false;
    c->xi_bar_ready = false;
    return kOk;
}

extern "C" int tdg_kappa_sma_vjp(tdg_ctx *c, const tdg_opts *o, const double *kappa_bar, double *lw_bar) {
    XferScope xs(c ? c->xfer : nullptr);
    PoolScope pscope(c ? c->stream : nullptr, c ? c->pool : nullptr);
    if (!c || !kappa_bar || !lw_bar) return set_error(kErrParam, "tdg_kappa_sma_vjp: null argument");
    int st = validate_opts(o);
    if (st) return st;
    if (!c->have_scattering) return set_error(kErrParam, "tdg_kappa_sma_vjp: call tdg_scattering first");
    const int n = c->n;
    // kappa_sma = S(S(M)) with S(X) = (1/nop) sum_R R X R^T (get_kappa, then symmetrize_kappa;
    // lo_chop is taken as the identity). The adjoint of S is (1/nop) sum_R R^T X R.
    auto St = [&](const double *x, double *y) {
        for (int i = 0; i < 9; ++i) y[i] = 0.0;
        for (int j = 0; j < c->nop; ++j) {
            const double *m = &c->op_cart[9 * j];
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    double sum = 0.0;
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) sum += m[a + 3 * k] * x[a + 3 * b] * m[b + 3 * l];
                    y[k + 3 * l] += sum / c->nop;
                }
        }
    };
    double t1[9], Mb[9];
    St(kappa_bar, t1);
    St(t1, Mb);
    const double T = o->temperature;
    for (int q1 = 0; q1 < c->nirr; ++q1) {
        const int f = c->irr_full[q1] - 1;
        for (int b1 = 0; b1 < n; ++b1) {
            double g = 0.0;
            const double om1 = c->omega[(size_t)f * n + b1];
            const double lw = c->linewidth[(size_t)q1 * n + b1];
            if (!(om1 < kFreqTol) && lw > kFreqTol) {
                // M += w F0 (x) v with F0 = v / (2 lw): d M / d lw = -w v (x) v / (2 lw^2)
                const double cv = o->classical ? kKbHartree : harmonic_oscillator_cv(T, om1);
                const double w = cv / c->volume * c->irr_weight[q1];
                const double *v = &c->vel[((size_t)f * n + b1) * 3];
                double vmv = 0.0;
                for (int x = 0; x < 3; ++x)
                    for (int y = 0; y < 3; ++y) vmv += v[x] * Mb[x + 3 * y] * v[y];
                g = -w * vmv / (2.0 * lw * lw);
            }
            lw_bar[(size_t)q1 * n + b1] = g;
        }
    }
    return kOk;
}

namespace {
// tdg_adjoint_fc3 after a large-cell (tensor-core) scattering pass: per batch the forward
// contraction again, W = G conj(Psi) from the delta kernel, the back-contraction with the
// transposed eigenvector matrices into Q, and 2 Re(phase Q) accumulated per force-constant
// entry in double-float.
int adjoint_large_cell(tdg_ctx *c, const std::vector<double> &lam, double *mwm_bar, double *stats) {
    cudaStream_t s = c->stream;
    const int n = c->n, N = c->N, ntrip = c->last_ntrip;
    const int64_t nm = (int64_t)c->n_fc3 * 27;
    CUDA_TRY(c->d_lam.upload(lam.data(), lam.size(), s));
    if (c->d_bmat_t.n == 0) {
        const int kp = ln_kp(n);
        CUDA_TRY(c->d_bmat_t.alloc((size_t)N * 2 * kp * kp));
        CUDA_TRY(launch_ln_bmat(n, N, c->d_egvs32.p, c->d_bmat_t.p, true, s));
    }
    CUDA_TRY(c->d_ghi.alloc(nm));
    CUDA_TRY(c->d_glo.alloc(nm));
    cudaEvent_t *ev = c->ev;
    CUDA_TRY(cudaEventRecord(ev[0], s));
    CUDA_TRY(cudaMemsetAsync(c->d_ghi.p, 0, sizeof(float) * nm, s));
    CUDA_TRY(cudaMemsetAsync(c->d_glo.p, 0, sizeof(float) * nm, s));
    CUDA_TRY(cudaMemsetAsync(c->d_status.p, 0, sizeof(int32_t), s));
    Fc3Dev fc;
    fc.n = c->n_fc3;
    fc.n_atom = c->na;
    fc.blk_ptr = c->fc3_blk.p;
    fc.lv = c->fc3_lv.p;
    fc.mwm = c->fc3_mwm.p;
    fc.mwm32 = c->fc3_mwm32.p;
    fc.twiddle = c->tw.p;
    fc.twiddle32 = c->tw32.p;
    fc.abase = c->fc3_abase.p;
    LnBatch b;
    int nbmax = 0, batches = 0;
    int st = ln_batch_setup(c, c->mesh(), c->last_ph, c->last_rows, fc, std::max(ntrip, 1), b, nbmax);
    if (st) return st;
    ln_apply_tune(b, c->last_ln_tune);
    b.gamma = nullptr;
    b.od = nullptr;
    b.bmat_t = c->d_bmat_t.p;
    b.lam = c->d_lam.p;
    b.grad_hi = c->d_ghi.p;
    b.grad_lo = c->d_glo.p;
    CUDA_TRY(cudaEventRecord(ev[1], s));
    for (int t0 = 0; t0 < ntrip; t0 += nbmax, ++batches) {
        b.trip = c->d_trip.p + t0;
        b.nb = std::min(nbmax, ntrip - t0);
        CUDA_TRY(launch_ln_adjoint_batch(b, s));
    }
    CUDA_TRY(cudaEventRecord(ev[2], s));
    std::vector<float> hi(nm), lo(nm);
    CUDA_TRY(copy_async(hi.data(), c->d_ghi.p, sizeof(float) * nm, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(copy_async(lo.data(), c->d_glo.p, sizeof(float) * nm, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaEventRecord(ev[3], s));
    CUDA_TRY(cudaStreamSynchronize(s));
    st = read_status(c);
    if (st) return st;
    for (int sidx = 0; sidx < c->n_fc3; ++sidx) {
        const int t = c->fc3_perm[sidx];
        for (int k = 0; k < 27; ++k)
            mwm_bar[(size_t)t * 27 + k] = (double)hi[(size_t)sidx * 27 + k] + (double)lo[(size_t)sidx * 27 + k];
    }
    if (stats) {
        float ms_all = 0.f, ms_k = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms_all, ev[0], ev[3]));
        CUDA_TRY(cudaEventElapsedTime(&ms_k, ev[1], ev[2]));
        stats[0] = ms_all;
        stats[1] = ms_k;
        stats[2] = ntrip;
        stats[3] = batches;
    }
    return kOk;
}
}  // namespace

extern "C" int tdg_kappa_iter_vjp(tdg_ctx *c, const tdg_opts *o, const double *kappa_bar, int32_t maxiter,
                                  double tol, double *lw_bar, int32_t *n_iter) {
    XferScope xs(c ? c->xfer : nullptr);
    PoolScope pscope(c ? c->stream : nullptr, c ? c->pool : nullptr);
    if (!c || !kappa_bar || !lw_bar) return set_error(kErrParam, "tdg_kappa_iter_vjp: null argument");
    int st = validate_opts(o);
    if (st) return st;
    if (!c->have_scattering || !c->last_third || !c->fn_iter)
        return set_error(kErrParam, "tdg_kappa_iter_vjp: call tdg_scattering (three-phonon) and tdg_kappa with "
                                    "iterations first");
    if (c->last_ln) return set_error(kErrParam, "tdg_kappa_iter_vjp: not supported on the large-cell path");
    if (maxiter < 1) return set_error(kErrParam, "tdg_kappa_iter_vjp: maxiter must be positive");
    CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const int n = c->n, N = c->N, nirr = c->nirr, nr = c->n_row;
    const int64_t ncol = (int64_t)N * n;
    const double T = o->temperature;
    const bool classical = o->classical != 0;
    // d kappa_iter / d F per irreducible mode: kappa = S(S(sum_r w_r F_r (x) v_r)) (get_kappa,
    // symmetrize_kappa; lo_chop as the identity), so kbar_r = w_r Mb v_r with Mb = S^T S^T kappa_bar.
    auto St = [&](const double *x, double *y) {
        for (int i = 0; i < 9; ++i) y[i] = 0.0;
        for (int j = 0; j < c->nop; ++j) {
            const double *m = &c->op_cart[9 * j];
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    double sum = 0.0;
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) sum += m[a + 3 * k] * x[a + 3 * b] * m[b + 3 * l];
                    y[k + 3 * l] += sum / c->nop;
                }
        }
    };
    double t1[9], Mb[9];
    St(kappa_bar, t1);
    St(t1, Mb);
    const size_t nf = (size_t)nirr * n * 3;
    std::vector<double> kbar(nf, 0.0);
    for (int q1 = 0; q1 < nirr; ++q1) {
        const int f = c->irr_full[q1] - 1;
        for (int b1 = 0; b1 < n; ++b1) {
            const double om1 = c->omega[(size_t)f * n + b1];
            if (om1 < kFreqTol) continue;
            const double cv = classical ? kKbHartree : harmonic_oscillator_cv(T, om1);
            const double w = cv / c->volume * c->irr_weight[q1];
            const double *v = &c->vel[((size_t)f * n + b1) * 3];
            for (int x = 0; x < 3; ++x)
                kbar[((size_t)q1 * n + b1) * 3 + x] = w * (Mb[x] * v[0] + Mb[x + 3] * v[1] + Mb[x + 6] * v[2]);
        }
    }
    // T F on the full mesh (the foldout of kappa.f90:382-404) and X T F
    std::vector<double> tf((size_t)ncol * 3);
    for (int q = 0; q < N; ++q) {
        const int op = c->full_op[q], l = c->full_irr[q] - 1;
        const double *m = &c->op_cart[9 * (std::abs(op) - 1)];
        const double sg = op > 0 ? 1.0 : -1.0;
        for (int b = 0; b < n; ++b) {
            const double *F = &c->Fn[((size_t)l * n + b) * 3];
            for (int x = 0; x < 3; ++x)
                tf[((size_t)q * n + b) * 3 + x] = sg * (m[x] * F[0] + m[x + 3] * F[1] + m[x + 6] * F[2]);
        }
    }
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    chk(c->d_tf.upload(tf.data(), tf.size(), s));
    chk(c->d_xtf.alloc((size_t)nr * 3));
    chk(c->d_zv.alloc((size_t)nr * 3));
    chk(c->d_yv.alloc((size_t)ncol * 3));
    chk(c->d_xpart.alloc((size_t)xit_parts(nr) * 3 * ncol));
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("allocation failed: ") + cudaGetErrorString(e));
    std::vector<double> xtf((size_t)nr * 3), z((size_t)nr * 3), y((size_t)ncol * 3);
    CUDA_TRY(launch_xi_rowdot(c->d_xi.p, nr, ncol, c->d_tf.p, c->d_xtf.p, s));
    CUDA_TRY(copy_async(xtf.data(), c->d_xtf.p, sizeof(double) * xtf.size(), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    // Transpose of distributeF (kappa.f90:418-435). Forward, for b1 = 1..n in turn and in
    // place: every member of the degenerate set of b1 becomes the set's mean, then F0(b1) is
    // added to entry b1, so an F0 added early is averaged again by the later members of its
    // set. Reverse, b1 = n..1: the cotangent of entry b1 goes to F0(b1), then the set's
    // cotangents are replaced by their mean. lam is the cotangent of the result, xb that of
    // the update Fnb, f0b (may be null) that of F0.
    auto distribute_adj = [&](const std::vector<double> &lam, std::vector<double> &xb, std::vector<double> *f0b) {
        xb = lam;
        if (f0b) f0b->assign(lam.size(), 0.0);
        for (int q1 = 0; q1 < nirr; ++q1) {
            const int f = c->irr_full[q1] - 1;
            double *a = &xb[(size_t)q1 * n * 3];
            for (int b1 = n - 1; b1 >= 0; --b1) {
                if (f0b)
                    for (int x = 0; x < 3; ++x) (*f0b)[((size_t)q1 * n + b1) * 3 + x] += a[b1 * 3 + x];
                const int dg = c->degen[(size_t)f * n + b1];
                if (dg == 1) continue;
                const int32_t *dm = &c->degen_mode[((size_t)f * n + b1) * n];
                for (int x = 0; x < 3; ++x) {
                    double sum = 0.0;
                    for (int j = 0; j < dg; ++j) sum += a[(dm[j] - 1) * 3 + x];
                    sum /= (double)dg;
                    for (int j = 0; j < dg; ++j) a[(dm[j] - 1) * 3 + x] = sum;
                }
            }
        }
    };
    // z_r = xb_r / qs_r on the rows (applyXi sets Fnb = -buf / qs, or 0 where qs < lo_freqtol)
    auto make_z = [&](const std::vector<double> &dl) {
        for (int r = 0; r < nr; ++r) {
            const int q1 = c->row_q1[r] - 1, b1 = c->row_b1[r] - 1;
            const double qs = c->qs[(size_t)q1 * n + b1];
            for (int x = 0; x < 3; ++x)
                z[(size_t)r * 3 + x] = qs < kFreqTol ? 0.0 : dl[((size_t)q1 * n + b1) * 3 + x] / qs;
        }
    };
    // adjoint fixed point lambda = kbar - T^T X^T Q^-1 xb(lambda), iterated with the forward
    // pass's mixing schedule and convergence test (kappa.f90:437-490). The test skips entries
    // whose squared norm is below lo_sqtol, a threshold set for F; the cotangents are of the
    // size of c_v / V (1e-8 and below), so the iteration runs on kbar scaled to a largest
    // entry of 1 (the map is linear) and scales back.
    double kscale = 0.0;
    for (double v : kbar) kscale = std::max(kscale, std::fabs(v));
    if (kscale == 0.0) kscale = 1.0;
    for (double &v : kbar) v /= kscale;
    std::vector<double> lam = kbar, nw(nf), dl, f0b;
    std::vector<double> scf;
    double mix = 0.95;
    int it = 0;
    for (it = 1; it <= maxiter; ++it) {
        distribute_adj(lam, dl, nullptr);
        make_z(dl);
        CUDA_TRY(copy_async(c->d_zv.p, z.data(), sizeof(double) * z.size(), cudaMemcpyHostToDevice, s));
        CUDA_TRY(launch_xit_gemv(c->d_xi.p, nr, ncol, c->d_zv.p, c->d_xpart.p, c->d_yv.p, s));
        CUDA_TRY(copy_async(y.data(), c->d_yv.p, sizeof(double) * y.size(), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        nw = kbar;
        for (int q = 0; q < N; ++q) {  // T^T: sum of R^T y over the star, with the sign of the operation
            const int op = c->full_op[q], l = c->full_irr[q] - 1;
            const double *m = &c->op_cart[9 * (std::abs(op) - 1)];
            const double sg = op > 0 ? 1.0 : -1.0;
            for (int b = 0; b < n; ++b) {
                const double *yy = &y[((size_t)q * n + b) * 3];
                for (int x = 0; x < 3; ++x)
                    nw[((size_t)l * n + b) * 3 + x] -= sg * (m[3 * x] * yy[0] + m[3 * x + 1] * yy[1] + m[3 * x + 2] * yy[2]);
            }
        }
        double g0 = 0.0;
        for (size_t i = 0; i < nf; i += 3) {
            double g1 = 0.0, g2 = 0.0;
            for (int x = 0; x < 3; ++x) {
                g1 += (lam[i + x] - nw[i + x]) * (lam[i + x] - nw[i + x]);
                g2 += lam[i + x] * lam[i + x];
            }
            if (g2 > kSqTol) g0 += g1 / g2;
            for (int x = 0; x < 3; ++x) lam[i + x] = lam[i + x] * (1.0 - mix) + mix * nw[i + x];
        }
        scf.push_back(g0 / nirr / n);
        if (it >= 3 && scf[it - 1] + scf[it - 2] + scf[it - 3] < tol) break;
        if (it > 15 && mix > 0.50) mix *= 0.98;
    }
    if (n_iter) *n_iter = std::min(it, maxiter);
    for (double &v : lam) v *= kscale;
    distribute_adj(lam, dl, &f0b);
    make_z(dl);
    // linewidth cotangent: F0 = v / qs (set where linewidth > lo_freqtol) and the 1/qs of the
    // update, qs = 2 linewidth
    for (size_t i = 0; i < (size_t)nirr * n; ++i) lw_bar[i] = 0.0;
    for (int r = 0; r < nr; ++r) {
        const int q1 = c->row_q1[r] - 1, b1 = c->row_b1[r] - 1;
        const size_t i = (size_t)q1 * n + b1;
        const double qs = c->qs[i];
        if (qs < kFreqTol) continue;
        const int f = c->irr_full[q1] - 1;
        const double *v = &c->vel[((size_t)f * n + b1) * 3];
        double g = 0.0;
        for (int x = 0; x < 3; ++x) g += dl[i * 3 + x] * xtf[(size_t)r * 3 + x];
        if (c->linewidth[i] > kFreqTol)
            for (int x = 0; x < 3; ++x) g -= f0b[i * 3 + x] * v[x];
        lw_bar[i] = 2.0 * g / (qs * qs);
    }
    // Xi cotangent W = -z (T F)^T through the adjoint row symmetrisations, given the raw
    // three-phonon terms of a fresh forward pass (the distribution's active entries)
    chk(c->d_xi_bar.alloc((size_t)nr * ncol));
    chk(c->d_od_raw.alloc((size_t)nr * ncol));
    chk(c->d_gam_tmp.alloc((size_t)nr));
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("allocation failed: ") + cudaGetErrorString(e));
    CUDA_TRY(copy_async(c->d_zv.p, z.data(), sizeof(double) * z.size(), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemsetAsync(c->d_od_raw.p, 0, sizeof(double) * (size_t)nr * ncol, s));
    CUDA_TRY(cudaMemsetAsync(c->d_gam_tmp.p, 0, sizeof(double) * nr, s));
    CUDA_TRY(cudaMemsetAsync(c->d_status.p, 0, sizeof(int32_t), s));
    ThreePhArgs a;
    std::memset(&a, 0, sizeof a);
    a.mesh = c->mesh();
    a.ph = c->last_ph;
    a.rows = c->last_rows;
    a.fc.n = c->n_fc3;
    a.fc.n_atom = c->na;
    a.fc.blk_ptr = c->fc3_blk.p;
    a.fc.lv = c->fc3_lv.p;
    a.fc.mwm = c->fc3_mwm.p;
    a.fc.mwm32 = c->fc3_mwm32.p;
    a.fc.twiddle = c->tw.p;
    a.fc.twiddle32 = c->tw32.p;
    a.fc.abase = c->fc3_abase.p;
    a.trip = c->d_trip.p;
    a.n_trip = c->last_ntrip;
    a.red = c->d_red.p;
    a.cand_mask = c->d_mask.p;
    a.gamma = c->d_gam_tmp.p;
    a.od = c->d_od_raw.p;
    a.status = c->d_status.p;
    CUDA_TRY(launch_threephonon(a, c->last_prec, c->n_sm, 0, s));
    CUDA_TRY(launch_xibar_fill(nr, ncol, c->d_zv.p, c->d_tf.p, c->d_xi_bar.p, s));
    CUDA_TRY(launch_sym_tile_adjoint(c->mesh(), c->orbits, nr, c->d_row_q1.p, c->d_od_raw.p, c->d_xi_bar.p,
                                     c->d_sbits.p, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    st = read_status(c);
    if (st) return st;
    c->xi_bar_ready = true;
    return kOk;
}

extern "C" int tdg_adjoint_fc3(tdg_ctx *c, const tdg_opts *o, const double *lw_bar, double *mwm_bar, double *stats) {
    XferScope xs(c ? c->xfer : nullptr);
    PoolScope pscope(c ? c->stream : nullptr, c ? c->pool : nullptr);
    if (!c || !lw_bar || !mwm_bar) return set_error(kErrParam, "tdg_adjoint_fc3: null argument");
    int st = validate_opts(o);
    if (st) return st;
    if (!c->have_scattering || !c->last_third)
        return set_error(kErrParam, "tdg_adjoint_fc3: call tdg_scattering with three-phonon scattering first");
    CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const int n = c->n, nr = c->n_row;
    // linewidth_j is the mean of Gamma over the degenerate set of j (scattering.f90:266-277),
    // so the cotangent of row (q1,b1) collects lw_bar over the set of b1, divided by its size.
    std::vector<double> lam(nr, 0.0);
    for (int r = 0; r < nr; ++r) {
        const int q1 = c->row_q1[r] - 1, b1 = c->row_b1[r] - 1;
        const int f = c->irr_full[q1] - 1;
        const int dg = c->degen[(size_t)f * n + b1];
        const int32_t *dm = &c->degen_mode[((size_t)f * n + b1) * n];
        double acc = 0.0;
        for (int j = 0; j < dg; ++j) acc += lw_bar[(size_t)q1 * n + dm[j] - 1];
        lam[r] = acc / (double)dg;
    }
    const int ntrip = c->last_ntrip;
    if (c->last_ln) {
        if (c->xi_bar_ready)
            return set_error(kErrParam, "tdg_adjoint_fc3: the scattering-matrix cotangent of tdg_kappa_iter_vjp is "
                                        "not supported on the large-cell path");
        return adjoint_large_cell(c, lam, mwm_bar, stats);
    }
    // after the tensor-core forward pass (mixed precision, 9/12/15 modes) the adjoint runs on
    // the tensor cores too; otherwise the SIMT kernel's ADJ variant
    const char *tc_env = std::getenv("TDG_TC_SMALL");
    const bool use_tc = c->last_path == 1 && o->precision != TDG_PREC_FP64 && o->tensor_cores != 2 &&
                        !(tc_env && tc_env[0] == '0') && threephonon_tc_supported(n, o->precision, c->n_fc3) &&
                        c->tc_plan.slots > 0;
    // the CTA's gradient slice lives in shared memory when it is small enough (SIMT)
    const bool acc_smem = !use_tc && (size_t)c->n_fc3 * 27 * sizeof(double) <= 48 * 1024;
    const int grid = use_tc ? threephonon_tc_adjoint_grid(n, c->n_sm, ntrip, c->n_fc3)
                            : threephonon_adjoint_grid(n, o->precision, c->n_sm, ntrip, c->n_fc3, acc_smem);
    if (ntrip > 0 && grid < 1) return set_error(kErrDevice, "adjoint kernel configuration failed");
    const int64_t nm = (int64_t)c->n_fc3 * 27;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    chk(c->d_lam.upload(lam.data(), lam.size(), s));
    chk(c->d_slices.alloc((size_t)std::max(grid, 1) * nm));
    chk(c->d_mwm_bar.alloc(nm));
    if (e != cudaSuccess) return set_error(kErrDevice, std::string("allocation failed: ") + cudaGetErrorString(e));
    cudaEvent_t *ev = c->ev;
    CUDA_TRY(cudaEventRecord(ev[0], s));
    CUDA_TRY(cudaMemsetAsync(c->d_slices.p, 0, sizeof(double) * (size_t)std::max(grid, 1) * nm, s));
    CUDA_TRY(cudaMemsetAsync(c->d_status.p, 0, sizeof(int32_t), s));
    ThreePhArgs a;
    std::memset(&a, 0, sizeof a);
    a.mesh = c->mesh();
    a.ph = c->last_ph;
    a.rows = c->last_rows;
    a.fc.n = c->n_fc3;
    a.fc.n_atom = c->na;
    a.fc.blk_ptr = c->fc3_blk.p;
    a.fc.lv = c->fc3_lv.p;
    a.fc.mwm = c->fc3_mwm.p;
    a.fc.mwm32 = c->fc3_mwm32.p;
    a.fc.twiddle = c->tw.p;
    a.fc.twiddle32 = c->tw32.p;
    a.fc.abase = c->fc3_abase.p;
    a.trip = c->d_trip.p;
    a.n_trip = ntrip;
    a.red = c->d_red.p;
    a.cand_mask = c->d_mask.p;
    a.gamma = nullptr;
    a.od = nullptr;
    a.status = c->d_status.p;
    a.lam = c->d_lam.p;
    a.mwm_bar = c->d_slices.p;
    a.acc_in_smem = acc_smem ? 1 : 0;
    a.xi_bar = c->xi_bar_ready ? c->d_xi_bar.p : nullptr;
    if (use_tc) {
        if (!c->tc_eimg_t_ready) {
            CUDA_TRY(c->d_tc_eimg_t.alloc((size_t)c->N * 4096));
            CUDA_TRY(launch_tc_eimg(c->N, n, c->d_egvs32.p, c->d_tc_eimg_t.p, s, true));
            c->tc_eimg_t_ready = true;
        }
        a.tc_eimg = c->d_tc_eimg.p;
        a.tc_eimg_t = c->d_tc_eimg_t.p;
    }
    tdg_ctx::Plan *plan = use_tc ? &c->tc_plan
                                 : (o->precision != TDG_PREC_FP64 && c->simt_plan.slots > 0 ? &c->simt_plan : nullptr);
    if (plan) {
        CUDA_TRY(launch_fill_plan(plan->src.p, plan->slots, plan->threads, c->fc3_mwm32.p, plan->pm.p, s));
        a.plan_pm = plan->pm.p;
        a.plan_word = plan->word.p;
        a.plan_slots = plan->slots;
    }
    CUDA_TRY(cudaEventRecord(ev[1], s));
    if (use_tc)
        CUDA_TRY(launch_threephonon_tc_adjoint(a, grid, s));
    else
        CUDA_TRY(launch_threephonon_adjoint(a, o->precision, grid, s));
    CUDA_TRY(cudaEventRecord(ev[2], s));
    CUDA_TRY(launch_sum_slices(c->d_slices.p, std::max(grid, 1), nm, o->precision, c->d_mwm_bar.p, s));
    std::vector<double> dev(nm);
    CUDA_TRY(copy_async(dev.data(), c->d_mwm_bar.p, sizeof(double) * nm, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaEventRecord(ev[3], s));
    CUDA_TRY(cudaStreamSynchronize(s));
    st = read_status(c);
    if (st) return st;
    for (int sidx = 0; sidx < c->n_fc3; ++sidx) {
        const int t = c->fc3_perm[sidx];
        for (int k = 0; k < 27; ++k) mwm_bar[(size_t)t * 27 + k] = dev[(size_t)sidx * 27 + k];
    }
    if (stats) {
        float ms_all = 0.f, ms_k = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms_all, ev[0], ev[3]));
        CUDA_TRY(cudaEventElapsedTime(&ms_k, ev[1], ev[2]));
        stats[0] = ms_all;
        stats[1] = ms_k;
        stats[2] = ntrip;
        stats[3] = grid;
    }
    return kOk;
}

extern "C" int tdg_transfer_bytes(tdg_ctx *c, int64_t *h2d, int64_t *d2h) {
    if (!c) return set_error(kErrParam, "tdg_transfer_bytes: null context");
    if (h2d) *h2d = c->xfer[0];
    if (d2h) *d2h = c->xfer[1];
    return kOk;
}

extern "C" int tdg_kappa_offdiag(tdg_ctx *c, const tdg_opts *o, double *kappa_offdiag) {
    XferScope xs(c ? c->xfer : nullptr);
    PoolScope pscope(c ? c->stream : nullptr, c ? c->pool : nullptr);
    if (!c || !kappa_offdiag) return set_error(kErrParam, "tdg_kappa_offdiag: null argument");
    int st = validate_opts(o);
    if (st) return st;
    if (!c->have_scattering) return set_error(kErrParam, "tdg_kappa_offdiag: call tdg_scattering first");
    if (c->irr_dyngrad.empty())
        return set_error(kErrParam, "tdg_kappa_offdiag: the problem has no irr_dyngrad/op_fmap/atom_shift");
    CUDA_TRY(cudaSetDevice(c->device));
    PhaseTimer pt("tdg_kappa_offdiag");
    cudaStream_t s = c->stream;
    const int n = c->n, nirr = c->nirr;
    const size_t nn = (size_t)n * n;
    if (c->d_grad.n == 0) {
        CUDA_TRY(c->d_grad.upload(reinterpret_cast<const double2 *>(c->irr_dyngrad.data()), (size_t)nirr * 3 * nn, s));
        CUDA_TRY(c->d_shift.upload(c->atom_shift.data(), c->atom_shift.size(), s));
        CUDA_TRY(c->d_fmap.upload(c->op_fmap.data(), c->op_fmap.size(), s));
        CUDA_TRY(c->d_qfull.upload(c->q_full.data(), c->q_full.size(), s));
        CUDA_TRY(c->d_irr_weight.upload(c->irr_weight.data(), c->irr_weight.size(), s));
        if (c->d_op_cart.n == 0) CUDA_TRY(c->d_op_cart.upload(c->op_cart.data(), c->op_cart.size(), s));
        // (point, operation) items of the per-operation kernels, point-major
        std::vector<int2> items;
        std::vector<int32_t> iptr(nirr + 1, 0);
        for (int q = 0; q < nirr; ++q) {
            for (int k = 0; k < c->irr_nop[q]; ++k) items.push_back(make_int2(q, k));
            iptr[q + 1] = (int32_t)items.size();
        }
        c->od_items = (int)items.size();
        if (n <= kOffdiagSmemModes) {
            CUDA_TRY(c->d_od_items.upload(items.data(), items.size(), s));
            CUDA_TRY(c->d_od_itemptr.upload(iptr.data(), iptr.size(), s));
        }
        const size_t w = offdiag_work_elems(n, nirr, c->od_items);
        if (w) CUDA_TRY(c->d_odwork.alloc(w));
        CUDA_TRY(c->d_odS.alloc((size_t)nirr * 9));
    }
    // linewidths and heat capacities of the irreducible modes (kappa.f90:252-278)
    std::vector<double> lwcv(2 * (size_t)nirr * n);
    for (int q = 0; q < nirr; ++q) {
        const int f = c->irr_full[q] - 1;
        for (int b = 0; b < n; ++b) {
            lwcv[(size_t)q * n + b] = c->linewidth[(size_t)q * n + b];
            lwcv[(size_t)nirr * n + (size_t)q * n + b] =
                o->classical ? kKbHartree : harmonic_oscillator_cv(o->temperature, c->omega[(size_t)f * n + b]);
        }
    }
    CUDA_TRY(c->d_lwcv.upload(lwcv.data(), lwcv.size(), s));
    pt.mark("uploads");
    OffdiagArgs a{};
    a.n = n;
    a.na = c->na;
    a.n_op = c->nop;
    a.egv = c->d_egv.p;
    a.grad = c->d_grad.p;
    a.omega = c->d_omega.p;
    a.q_full = c->d_qfull.p;
    a.irr_full = c->d_irr_full.p;
    a.irr_nop = c->d_irr_nop.p;
    a.irr_ops = c->d_irr_ops.p;
    a.op_cart = c->d_op_cart.p;
    a.fmap = c->d_fmap.p;
    a.shift = c->d_shift.p;
    a.lw = c->d_lwcv.p;
    a.cv = c->d_lwcv.p + (size_t)nirr * n;
    a.irr_weight = c->d_irr_weight.p;
    a.inv_volume = 1.0 / c->volume;
    a.chop_tol = 1E-10 / (kGroupVelAuToMs / 1000.0);
    a.work = c->d_odwork.p;
    a.part = c->d_odwork.p;
    a.items = c->d_od_items.p;
    a.item_ptr = c->d_od_itemptr.p;
    a.vel = nullptr;
    a.S = c->d_odS.p;
    CUDA_TRY(launch_offdiag(a, nirr, c->od_items, s));
    std::vector<double> S((size_t)nirr * 9);
    CUDA_TRY(copy_async(S.data(), c->d_odS.p, sizeof(double) * S.size(), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    pt.mark("little-group sandwiches (device)");
    // star of each irreducible point: (1/n_star) sum_R R S R^T (kappa.f90:221-231)
    std::vector<double> K((size_t)nirr * 9, 0.0);
    std::vector<int> nstar(nirr, 0);
    for (int f = 0; f < c->N; ++f) {
        const int q = c->full_irr[f] - 1;
        const double *m = &c->op_cart[9 * (std::abs(c->full_op[f]) - 1)];
        const double *Sq = &S[(size_t)q * 9];
        double *Kq = &K[(size_t)q * 9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double v = 0.0;
                for (int k = 0; k < 3; ++k)
                    for (int l = 0; l < 3; ++l) v += m[i + 3 * k] * Sq[k + 3 * l] * m[j + 3 * l];
                Kq[i + 3 * j] += v;
            }
        ++nstar[q];
    }
    double kap[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = 0; q < nirr; ++q)
        for (int k = 0; k < 9; ++k) kap[k] += K[(size_t)q * 9 + k] / nstar[q];
    double tol = 0.0;
    for (int k = 0; k < 9; ++k) tol += std::fabs(kap[k]);
    tol *= 1e-6;
    for (int k = 0; k < 9; ++k) kap[k] = lo_chop(kap[k], tol);
    symmetrize_kappa(c, kap);
    std::memcpy(kappa_offdiag, kap, sizeof(kap));
    pt.mark("stars (host)");
    return kOk;
}

namespace tdg {
cudaMemPool_t shared_device_pool(int device) { return device_pool(device); }
}  // namespace tdg
