// Launch-shape autotuner of the scattering kernels.
//
// The choices are tile shapes and grid sizes whose best value depends on the mode count,
// the precision and the device: the persistent grid of the fused three-phonon kernel (CTAs
// per SM), and, on the large-cell path, the row block of the delta kernel and the depth of
// the GEMM's shared-memory pipeline. The first call that needs a decision times every
// candidate on the call's own work with CUDA events on the call's stream (the caller makes
// the trials' outputs disappear afterwards) and keeps the fastest in a process-wide table
// keyed by kernel, mode count, precision, SM count and device name. The table can be
// loaded from and saved to a text file (one "key value" per line): the environment
// variable TDG_TUNE_CACHE names a file that is read before the first decision and
// rewritten after every new one. TDG_AUTOTUNE=0 turns the trials off (every decision takes
// its default); decisions already in the table are still used.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/tdep_gb300.h"
#include "host/common.hpp"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

struct TuneTable {
    std::mutex mu;
    std::map<std::string, int> best;
    bool env_loaded = false;
};

TuneTable &table() {
    static TuneTable t;
    return t;
}

// Parses "key value" lines; blank lines and lines starting with '#' are skipped. Returns
// the number of entries read, or -1 when the file cannot be opened or a line is malformed.
int load_file(const char *path, std::map<std::string, int> &into) {
    std::ifstream f(path);
    if (!f) return -1;
    std::string line;
    int count = 0;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream ss(line);
        std::string key;
        long v;
        std::string rest;
        if (!(ss >> key >> v) || (ss >> rest)) return -1;
        into[key] = (int)v;
        ++count;
    }
    return count;
}

int save_file(const char *path, const std::map<std::string, int> &from) {
    const std::string tmp = std::string(path) + ".tmp";
    {
        std::ofstream f(tmp, std::ios::trunc);
        if (!f) return -1;
        f << "# tdep_gb300 launch-shape decisions: key value\n";
        for (const auto &kv : from) f << kv.first << ' ' << kv.second << '\n';
        if (!f) return -1;
    }
    return std::rename(tmp.c_str(), path) == 0 ? (int)from.size() : -1;
}

void load_env_locked(TuneTable &t) {
    if (t.env_loaded) return;
    t.env_loaded = true;
    const char *p = std::getenv("TDG_TUNE_CACHE");
    if (p && *p) load_file(p, t.best);
}

bool trials_enabled() {
    const char *p = std::getenv("TDG_AUTOTUNE");
    return !(p && std::strcmp(p, "0") == 0);
}

}  // namespace

int resident_ctas(const void *fn, int threads, size_t dyn_bytes, int *api_out, int *count_out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_bytes) != cudaSuccess ||
        cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared) !=
            cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int api = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&api, fn, threads, dyn_bytes) != cudaSuccess) {
        cudaGetLastError();
        api = 0;
    }
    // the same count from the kernel's registers and shared memory: registers in units of 256
    // per warp, shared memory per CTA with the driver's reserve, in units of 128 bytes
    cudaFuncAttributes fa;
    int regs_sm = 0, smem_sm = 0, smem_res = 0, thr_sm = 0;
    int count = 0;
    if (cudaFuncGetAttributes(&fa, fn) == cudaSuccess &&
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&smem_res, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) == cudaSuccess) {
        const int warps = (threads + 31) / 32;
        const long regs_cta = (long)warps * (((long)fa.numRegs * 32 + 255) / 256 * 256);
        const long smem_cta = ((long)dyn_bytes + (long)fa.sharedSizeBytes + smem_res + 127) / 128 * 128;
        const long by_regs = regs_cta > 0 ? regs_sm / regs_cta : 64;
        const long by_smem = smem_cta > 0 ? smem_sm / smem_cta : 64;
        const long by_thr = thr_sm / (warps * 32);
        count = (int)std::min(std::min(by_regs, by_smem), by_thr);
    } else {
        cudaGetLastError();
    }
    if (api_out) *api_out = api;
    if (count_out) *count_out = count;
    return std::max(api, count);
}

std::string tune_key(const char *kernel, int n, int precision, int device) {
    cudaDeviceProp prop;
    std::string name = "unknown";
    int n_sm = 0;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) {
        name = prop.name;
        n_sm = prop.multiProcessorCount;
    } else {
        cudaGetLastError();
    }
    for (char &ch : name)
        if (ch == ' ') ch = '_';
    std::ostringstream k;
    k << kernel << "/n" << n << "/p" << precision << "/sm" << n_sm << "/" << name;
    return k.str();
}

int tune_lookup(const std::string &key, int dflt) {
    TuneTable &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    load_env_locked(t);
    auto it = t.best.find(key);
    return it == t.best.end() ? dflt : it->second;
}

cudaError_t tune_pick(const std::string &key, const std::vector<int> &cand, int dflt,
                      const std::function<cudaError_t(int)> &trial, cudaStream_t s, int &choice, bool &tuned) {
    tuned = false;
    choice = dflt;
    {
        TuneTable &t = table();
        std::lock_guard<std::mutex> lk(t.mu);
        load_env_locked(t);
        auto it = t.best.find(key);
        if (it != t.best.end()) {
            choice = it->second;
            return cudaSuccess;
        }
    }
    if (!trials_enabled() || cand.size() < 2) return cudaSuccess;
    cudaEvent_t e0, e1;
    cudaError_t e;
    if ((e = cudaEventCreate(&e0)) != cudaSuccess) return e;
    if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
        cudaEventDestroy(e0);
        return e;
    }
    std::vector<float> best_ms(cand.size(), 1e30f);
    // one untimed run loads the code and warms the caches; then two timed rounds, the
    // minimum per candidate
    e = trial(cand[0]);
    for (int round = 0; round < 2 && e == cudaSuccess; ++round)
        for (size_t i = 0; i < cand.size() && e == cudaSuccess; ++i) {
            if ((e = cudaEventRecord(e0, s)) != cudaSuccess) break;
            if ((e = trial(cand[i])) != cudaSuccess) break;
            if ((e = cudaEventRecord(e1, s)) != cudaSuccess) break;
            if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
            float ms = 0.f;
            if ((e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) break;
            best_ms[i] = std::min(best_ms[i], ms);
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return e;
    size_t bi = 0;
    for (size_t i = 1; i < cand.size(); ++i)
        if (best_ms[i] < best_ms[bi]) bi = i;
    choice = cand[bi];
    tuned = true;
    TuneTable &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    t.best[key] = choice;
    const char *p = std::getenv("TDG_TUNE_CACHE");
    if (p && *p) save_file(p, t.best);
    return cudaSuccess;
}

}  // namespace tdg

using namespace tdg;

extern "C" int tdg_autotune_load(const char *path) {
    if (!path) return set_error(kErrParam, "tdg_autotune_load: null path");
    std::map<std::string, int> m;
    const int n = load_file(path, m);
    if (n < 0) return set_error(kErrIo, std::string("tdg_autotune_load: cannot read ") + path);
    TuneTable &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    for (const auto &kv : m) t.best[kv.first] = kv.second;
    return kOk;
}

extern "C" int tdg_autotune_save(const char *path) {
    if (!path) return set_error(kErrParam, "tdg_autotune_save: null path");
    TuneTable &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    if (save_file(path, t.best) < 0) return set_error(kErrIo, std::string("tdg_autotune_save: cannot write ") + path);
    return kOk;
}

extern "C" int tdg_autotune_report(char *buf, int64_t cap, int64_t *needed) {
    TuneTable &t = table();
    std::string s;
    {
        std::lock_guard<std::mutex> lk(t.mu);
        load_env_locked(t);
        for (const auto &kv : t.best) s += kv.first + " " + std::to_string(kv.second) + "\n";
    }
    if (needed) *needed = (int64_t)s.size() + 1;
    if (!buf || cap <= 0) return kOk;
    const size_t m = std::min<size_t>(s.size(), (size_t)cap - 1);
    std::memcpy(buf, s.data(), m);
    buf[m] = '\0';
    return kOk;
}

extern "C" int tdg_autotune_clear(void) {
    TuneTable &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    t.best.clear();
    t.env_loaded = true;  // an explicit clear also drops what the environment's file held
    return kOk;
}
