// tdg_triplets_static: the irreducible q-triplet enumeration of tdg_triplets (count pass,
// two exclusive scans, fill pass) run entirely in a fixed, file-scope device array, for
// callers that cannot allocate device memory. It calls no cudaMalloc, cudaFree or other
// allocating routine; the array is created with the module and found once per device with
// cudaGetSymbolAddress.
//
// Limits (checked on the host before any device work on the result): a sample of at most
// kMaxSample = 32768 q-points, and at most kMaxPairs = 131072 equivalent triplets in the
// result. A sample without repeated q-points on a mesh of up to 131072 points always stays
// within the second limit (the equivalent triplets of distinct irreducible triplets are
// distinct pairs (q2', q3'), and q3' follows from q2'); a repeated q-point adds its images
// once per repeat, so heavily repeated samples can exceed it and get TDG_ERR_PARAM from
// the check on the count pass. Scratch: about 4.3 MiB per device.
//
// Only the status word must start at zero; every call clears it before the count pass.
// Every other region is written in full before it is read. All calls on one device share
// the array, so calls that overlap in time (from several threads or contexts) race.
#include <mutex>
#include <string>

#include "../../include/tdep_gb300.h"
#include "host/common.hpp"
#include "tdg_internal.cuh"

using namespace tdg;

namespace {

constexpr int32_t kMaxSample = 32768;
constexpr int32_t kMaxPairs = 131072;
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr size_t kCountBytes = align256(sizeof(int32_t) * ((size_t)kMaxSample + 1));
constexpr size_t kTmpBytes = 4096;
constexpr size_t kOffStatus = 0;
constexpr size_t kOffSample = 256;
constexpr size_t kOffCand = kOffSample + align256(sizeof(int32_t) * kMaxSample);
constexpr size_t kOffNt = kOffCand + align256(sizeof(int4) * kMaxSample);
constexpr size_t kOffNrd = kOffNt + kCountBytes;
constexpr size_t kOffToff = kOffNrd + kCountBytes;
constexpr size_t kOffRoff = kOffToff + kCountBytes;
constexpr size_t kOffTmp = kOffRoff + kCountBytes;
constexpr size_t kOffTrip = kOffTmp + kTmpBytes;
constexpr size_t kOffRed = kOffTrip + align256(sizeof(TripletRec) * kMaxSample);
constexpr size_t kOffOut = kOffRed + align256(sizeof(int2) * kMaxPairs);
constexpr size_t kOutInts = 3 * (size_t)kMaxSample + 2 * (size_t)kMaxPairs;
constexpr size_t kScratchBytes = kOffOut + align256(sizeof(int32_t) * kOutInts);
static_assert(kScratchBytes < 5u * 1024 * 1024, "static triplet scratch should stay modest");

static __device__ __align__(256) unsigned char g_triplet_scratch[kScratchBytes];

std::mutex g_setup_mu;
unsigned char *g_scratch[kMaxDevices] = {};

#define CUDA_TRY(expr)                                                                                 \
    do {                                                                                               \
        cudaError_t e_ = (expr);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return set_error(kErrDevice, std::string(#expr) + ": " + cudaGetErrorString(e_));          \
    } while (0)

// Address of the scratch array on `device`, which must be current. Looked up once per
// device; the lookup loads the module, so the first call belongs before any stream capture.
int scratch_for(int device, unsigned char **out) {
    if (device < 0 || device >= kMaxDevices) return set_error(kErrDevice, "tdg_triplets_static: device index too large");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch[device]) {
        if (exclusive_scan_tmp_elems(kMaxSample) * sizeof(int32_t) > kTmpBytes)
            return set_error(kErrDevice, "tdg_triplets_static: scan scratch larger than its reserved region");
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_triplet_scratch);
        if (e != cudaSuccess)
            return set_error(kErrDevice, std::string("tdg_triplets_static: cudaGetSymbolAddress: ") +
                                             cudaGetErrorString(e));
        g_scratch[device] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch[device];
    return kOk;
}

__global__ void k_sample_candidates(int32_t q1, const int32_t *sample, int32_t n, int4 *cand) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) cand[i] = make_int4(q1, sample[i] - 1, 0, 0);
}

// Triplet t starts at 3*t + 2*red_off: every earlier triplet took 3 ints plus two per
// equivalent triplet, and red_off counts exactly those.
__global__ void k_format_triplets(const TripletRec *trip, int32_t n_trip, const int2 *red, int32_t *out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_trip) return;
    const TripletRec r = trip[t];
    int32_t *o = out + 3 * (int64_t)t + 2 * (int64_t)r.red_off;
    o[0] = r.q2 + 1;
    o[1] = r.q3 + 1;
    o[2] = r.red_cnt;
    for (int k = 0; k < r.red_cnt; ++k) {
        const int2 p = red[r.red_off + k];
        o[3 + 2 * k] = p.x + 1;
        o[4 + 2 * k] = p.y + 1;
    }
}

}  // namespace

extern "C" int tdg_triplets_static(tdg_ctx *c, int32_t q1, const int32_t *sample, int64_t n, int32_t *out,
                                   int64_t cap, int64_t *written) {
    if (!c || !out || !written || (n > 0 && !sample)) return set_error(kErrParam, "tdg_triplets_static: null argument");
    if (n < 0) return set_error(kErrParam, "tdg_triplets_static: bad sample length");
    if (n > kMaxSample)
        return set_error(kErrParam, "tdg_triplets_static: sample of " + std::to_string(n) +
                                        " q-points exceeds the static scratch limit of " + std::to_string(kMaxSample));
    const CtxView v = ctx_view(c);
    XferScope xs(v.xfer);
    if (q1 < 1 || q1 > v.mesh.n_irr) return set_error(kErrParam, "tdg_triplets_static: q1 out of range");
    for (int64_t i = 0; i < n; ++i)
        if (sample[i] < 1 || sample[i] > v.mesh.n_full)
            return set_error(kErrParam, "tdg_triplets_static: q' index out of range");
    CUDA_TRY(cudaSetDevice(v.device));
    unsigned char *base = nullptr;
    if (int st = scratch_for(v.device, &base)) return st;
    *written = 0;
    if (n == 0) return kOk;

    const int32_t nc = (int32_t)n;
    const cudaStream_t s = v.stream;
    int32_t *d_status = reinterpret_cast<int32_t *>(base + kOffStatus);
    int32_t *d_sample = reinterpret_cast<int32_t *>(base + kOffSample);
    int4 *d_cand = reinterpret_cast<int4 *>(base + kOffCand);
    int32_t *d_nt = reinterpret_cast<int32_t *>(base + kOffNt);
    int32_t *d_nrd = reinterpret_cast<int32_t *>(base + kOffNrd);
    int32_t *d_toff = reinterpret_cast<int32_t *>(base + kOffToff);
    int32_t *d_roff = reinterpret_cast<int32_t *>(base + kOffRoff);
    int32_t *d_tmp = reinterpret_cast<int32_t *>(base + kOffTmp);
    TripletRec *d_trip = reinterpret_cast<TripletRec *>(base + kOffTrip);
    int2 *d_red = reinterpret_cast<int2 *>(base + kOffRed);
    int32_t *d_out = reinterpret_cast<int32_t *>(base + kOffOut);

    CUDA_TRY(cudaMemsetAsync(d_status, 0, sizeof(int32_t), s));
    CUDA_TRY(copy_async(d_sample, sample, sizeof(int32_t) * nc, cudaMemcpyHostToDevice, s));
    k_sample_candidates<<<(nc + 255) / 256, 256, 0, s>>>(q1 - 1, d_sample, nc, d_cand);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(launch_triplet_count(v.mesh, d_cand, nc, d_nt, d_nrd, d_status, s));
    CUDA_TRY(exclusive_scan_i32(d_nt, d_toff, nc, d_tmp, s));
    CUDA_TRY(exclusive_scan_i32(d_nrd, d_roff, nc, d_tmp, s));
    int32_t h[3] = {0, 0, 0};
    CUDA_TRY(copy_async(&h[0], d_toff + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(copy_async(&h[1], d_roff + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(copy_async(&h[2], d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    if (h[2] != kDevOk)
        return set_error(kErrDevice, "device-side index check failed (status " + std::to_string(h[2]) + ")");
    if (h[1] > kMaxPairs)
        return set_error(kErrParam, "tdg_triplets_static: " + std::to_string(h[1]) +
                                        " equivalent triplets exceed the static scratch limit of " +
                                        std::to_string(kMaxPairs));
    const int64_t w = 3 * (int64_t)h[0] + 2 * (int64_t)h[1];
    if (w > cap) return set_error(kErrParam, "tdg_triplets_static: output capacity too small");
    CUDA_TRY(launch_triplet_fill(v.mesh, d_cand, nc, d_toff, d_roff, d_trip, d_red, s));
    if (h[0] > 0) {
        k_format_triplets<<<(h[0] + 127) / 128, 128, 0, s>>>(d_trip, h[0], d_red, d_out);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(copy_async(out, d_out, sizeof(int32_t) * w, cudaMemcpyDeviceToHost, s));
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    *written = w;
    return kOk;
}
