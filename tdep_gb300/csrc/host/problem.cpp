// Host stage of thermal_conductivity: reading the input files and building the flattened
// problem (main.f90:42-181), error reporting and the output file (main.f90:246-294).
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <fstream>
#include <memory>
#include <mutex>
#include <thread>

#include <unistd.h>

#include "../../../include/tdep_gb300.h"
#include "crystal.hpp"

namespace tdg {

namespace {
thread_local std::string g_last_error;
}

namespace {
double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

PhaseTimer::PhaseTimer(const char *scope) : scope_(scope), on_(std::getenv("TDG_TRACE") != nullptr), t_(now_ms()) {}

PhaseTimer::~PhaseTimer() {
    if (!on_) return;
    for (const auto &x : sums_) std::fprintf(stderr, "[tdg] %s %s %.3f ms\n", scope_, x.first, x.second);
}

void PhaseTimer::mark(const char *label) {
    if (!on_) return;
    const double t = now_ms();
    for (auto &x : sums_)
        if (std::strcmp(x.first, label) == 0) {
            x.second += t - t_;
            t_ = t;
            return;
        }
    sums_.emplace_back(label, t - t_);
    t_ = t;
}

int set_error(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
const char *last_error() { return g_last_error.c_str(); }

// gottochblandat_physics.f90:160-186
double planck(double temperature, double omega) {
    if (temperature < kTemperatureTol) return 0.0;
    if (omega < kFreqTol) return 0.0;
    const double x = omega / (kKbHartree * temperature);
    if (x > 1E2) return 0.0;
    return 1.0 / (std::exp(x) - 1.0);
}

// gottochblandat_physics.f90:331-366
double harmonic_oscillator_cv(double temp, double omega) {
    if (omega < kFreqTol) return 0.0;
    if (temp < kTemperatureTol) return 0.0;
    const double x = omega / temp / kKbHartree;
    if (x > 200.0) return 0.0;
    if (x > 21.0) return kKbHartree * x * x * std::exp(-x);
    if (x < 2E-2) return kKbHartree * (1.0 - x * x / 12.0 + x * x * x * x / 240.0);
    const double em1 = std::exp(x) - 1.0;
    return kKbHartree * x * x * std::exp(x) / (em1 * em1);
}

namespace {

// Worker threads of parallel_for, created once (hardware threads - 1; the caller is the last
// one). One job at a time. A job is a shared object that the workers take when they wake;
// indices are claimed in chunks, and the caller returns as soon as every index is done,
// without waiting for the workers that woke late (they find nothing left to claim, so the
// caller's function is never called after it returns). Waiting for every worker to check
// in, as before, cost a wake-up of all threads per parallel_for (about 0.5 ms per call on
// the 16-core Grace host, several calls per problem load).
struct Pool {
    struct Job {
        const std::function<void(int64_t)> *fn = nullptr;
        int64_t n = 0, chunk = 1;
        std::atomic<int64_t> next{0}, done{0};
    };
    std::mutex mu;
    std::condition_variable cv_start;
    std::atomic<bool> busy{false};
    std::shared_ptr<Job> cur;
    uint64_t gen = 0;
    unsigned nw = 0;
    pid_t pid = 0;
    Pool() {
        pid = getpid();
        const unsigned hc = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 64u));
        nw = hc - 1;
        for (unsigned t = 0; t < nw; ++t) std::thread([this] { loop(); }).detach();
    }
    static void work(Job &j) {
        for (;;) {
            const int64_t i0 = j.next.fetch_add(j.chunk);
            if (i0 >= j.n) return;
            const int64_t i1 = std::min(j.n, i0 + j.chunk);
            for (int64_t i = i0; i < i1; ++i) (*j.fn)(i);
            j.done.fetch_add(i1 - i0);
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            std::shared_ptr<Job> j;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_start.wait(lk, [&] { return gen != seen; });
                seen = gen;
                j = cur;
            }
            if (j) work(*j);
        }
    }
    bool run(int64_t count, const std::function<void(int64_t)> &f) {
        if (nw == 0 || getpid() != pid) return false;
        bool idle = false;
        if (!busy.compare_exchange_strong(idle, true)) return false;
        auto j = std::make_shared<Job>();
        j->fn = &f;
        j->n = count;
        j->chunk = std::max<int64_t>(1, count / (8 * (int64_t)(nw + 1)));
        {
            std::lock_guard<std::mutex> lk(mu);
            cur = j;
            ++gen;
        }
        cv_start.notify_all();
        work(*j);
        while (j->done.load() < count) std::this_thread::yield();
        {
            std::lock_guard<std::mutex> lk(mu);
            cur.reset();
        }
        busy = false;
        return true;
    }
};

}  // namespace

bool pool_run(int64_t n, const std::function<void(int64_t)> &f) {
    static Pool *pool = new Pool();  // never destroyed: its threads live as long as the process
    return pool->run(n, f);
}

namespace {

struct ProblemHolder {
    tdg_problem p;  // first member: the C handle points here
    Crystal c;
    QMesh q;
    Phonons ph;
    FC3 f3;
    FC4 f4;
    std::vector<double> op_cart;
    std::vector<int32_t> op_recfrac;
    std::vector<double> q_full;
    std::vector<double> irr_dyngrad, atom_shift;
    std::vector<int32_t> op_fmap;
};

}  // namespace
}  // namespace tdg

extern "C" const char *tdg_last_error(void) { return tdg::last_error(); }
extern "C" const char *tdg_version(void) { return "tdep_gb300 0.1 (sm_103a)"; }

namespace tdg {
namespace {
int problem_load(const char *dir, const int32_t grid[3], int fourthorder, int readiso, int timereversal, int device,
                 tdg_problem **out);
}  // namespace
}  // namespace tdg

extern "C" int tdg_problem_load(const char *dir, const int32_t grid[3], int fourthorder, int readiso,
                                int timereversal, tdg_problem **out) {
    return tdg::problem_load(dir, grid, fourthorder, readiso, timereversal, -1, out);
}

extern "C" int tdg_problem_load_device(const char *dir, const int32_t grid[3], int fourthorder, int readiso,
                                       int timereversal, int32_t device, tdg_problem **out) {
    if (device < 0) return tdg::set_error(tdg::kErrParam, "tdg_problem_load_device: negative device");
    return tdg::problem_load(dir, grid, fourthorder, readiso, timereversal, device, out);
}

namespace tdg {
namespace {
int problem_load(const char *dir, const int32_t grid[3], int fourthorder, int readiso, int timereversal, int device,
                 tdg_problem **out) {
    if (!dir || !grid || !out) return set_error(kErrParam, "tdg_problem_load: null argument");
    *out = nullptr;
    PhaseTimer pt("tdg_problem_load");
    auto h = std::make_unique<ProblemHolder>();
    const std::string d = std::string(dir) + "/";
    int st = read_poscar(d + "infile.ucposcar", h->c);
    if (st) return st;
    if (readiso) {
        st = read_isotopes(d + "infile.isotopes", h->c);
        if (st) return st;
    }
    for (int a = 0; a < h->c.na; ++a)
        if (!(h->c.mass[a] > 0))
            return set_error(kErrParam, "unknown element mass for atom " + std::to_string(a + 1) +
                                            "; provide infile.isotopes and --readiso");
    pt.mark("structure");
    st = find_symmetry(h->c);
    if (st) return st;
    pt.mark("symmetry");
    FC2 fc2;
    st = read_fc2(d + "infile.forceconstant", h->c, fc2);
    if (st) return st;
    st = read_fc3(d + "infile.forceconstant_thirdorder", h->c, h->f3);
    if (st) return st;
    if (fourthorder) {
        st = read_fc4(d + "infile.forceconstant_fourthorder", h->c, h->f4);
        if (st) return st;
    }
    pt.mark("force constants");
    const int g[3] = {grid[0], grid[1], grid[2]};
    st = build_fft_mesh(h->c, g, timereversal != 0, h->q);
    if (st) return st;
    pt.mark("mesh");
    if (device >= 0) {
        st = build_phonons_device(h->c, fc2, h->q, device, h->ph, h->irr_dyngrad);
        if (st) return st;
    } else {
        st = build_phonons(h->c, fc2, h->q, h->ph);
        if (st) return st;
    }
    pt.mark(device >= 0 ? "phonons (device)" : "phonons (host)");
    // off-diagonal kappa inputs: dD/dq at the irreducible points and the atom maps
    {
        const int nb = 3 * h->c.na, ni = h->q.n_irr;
        if (device < 0) {  // (the device stage returns them with the phonons)
            h->irr_dyngrad.assign((size_t)ni * 3 * nb * nb * 2, 0.0);
            parallel_for(ni, [&](int64_t i) {
                std::vector<cplx> g((size_t)3 * nb * nb);
                dyn_gradient(h->c, fc2, h->q.q_full[h->q.irr_full[i] - 1], nb, g.data());
                for (size_t k = 0; k < g.size(); ++k) {
                    h->irr_dyngrad[((size_t)i * 3 * nb * nb + k) * 2] = g[k].real();
                    h->irr_dyngrad[((size_t)i * 3 * nb * nb + k) * 2 + 1] = g[k].imag();
                }
            });
        }
        st = op_atom_maps(h->c, h->op_fmap, h->atom_shift);
        if (st) return st;
        for (auto &x : h->op_fmap) x += 1;
    }

    tdg_problem &p = h->p;
    std::memset(&p, 0, sizeof(p));
    p.n_atom = h->c.na;
    p.n_mode = 3 * h->c.na;
    std::memcpy(p.latvec, h->c.lat.a, sizeof(p.latvec));
    std::memcpy(p.reclat, h->c.reclat.a, sizeof(p.reclat));
    std::memcpy(p.inv_reclat, h->c.inv_reclat.a, sizeof(p.inv_reclat));
    p.volume = h->c.volume;
    p.mass_disorder = h->c.disorder.data();
    p.n_op = (int32_t)h->c.ops.size();
    for (const auto &op : h->c.ops) {
        h->op_cart.insert(h->op_cart.end(), op.m.a, op.m.a + 9);
        h->op_recfrac.insert(h->op_recfrac.end(), op.rfm, op.rfm + 9);
    }
    p.op_cart = h->op_cart.data();
    p.op_recfrac = h->op_recfrac.data();
    for (int i = 0; i < 3; ++i) p.grid[i] = h->q.grid[i];
    p.n_full = h->q.n_full;
    p.n_irr = h->q.n_irr;
    for (const auto &v : h->q.q_full) h->q_full.insert(h->q_full.end(), v.x, v.x + 3);
    p.q_full = h->q_full.data();
    p.full_irr = h->q.full_irr.data();
    p.full_op = h->q.full_op.data();
    p.irr_full = h->q.irr_full.data();
    p.irr_weight = h->q.irr_weight.data();
    p.irr_nop = h->q.irr_nop.data();
    p.irr_ops = h->q.irr_ops.data();
    p.omega = h->ph.omega.data();
    p.egv = h->ph.egv.data();
    p.vel = h->ph.vel.data();
    p.degen = h->ph.degen.data();
    p.degen_mode = h->ph.degen_mode.data();
    p.n_fc3 = h->f3.n();
    p.fc3_atoms = h->f3.atoms.data();
    p.fc3_lv = h->f3.lv.data();
    p.fc3_lvcart = h->f3.lvcart.data();
    p.fc3_mwm = h->f3.mwm.data();
    p.n_fc4 = h->f4.n();
    p.fc4_atoms = h->f4.atoms.data();
    p.fc4_lv = h->f4.lv.data();
    p.fc4_lvcart = h->f4.lvcart.data();
    p.fc4_mwm = h->f4.mwm.data();
    p.irr_dyngrad = h->irr_dyngrad.data();
    p.op_fmap = h->op_fmap.data();
    p.atom_shift = h->atom_shift.data();
    *out = &h.release()->p;
    return kOk;
}
}  // namespace
}  // namespace tdg

extern "C" void tdg_problem_free(tdg_problem *prob) {
    if (!prob) return;
    delete reinterpret_cast<tdg::ProblemHolder *>(prob);
}

namespace {
// Fortran Ew.d edit descriptor: 0.ddddE+ee right-justified in w characters.
std::string fortran_e(double x, int w, int d) {
    char buf[64];
    if (x == 0.0 || !std::isfinite(x)) {
        if (!std::isfinite(x)) {
            std::snprintf(buf, sizeof(buf), "%*s", w, std::string(w, '*').c_str());
            return buf;
        }
        std::string s = "0." + std::string(d, '0') + "E+00";
        std::snprintf(buf, sizeof(buf), "%*s", w, s.c_str());
        return buf;
    }
    // printf gives d.ddd e(e-1); shift to 0.dddd form by formatting d digits.
    char tmp[64];
    std::snprintf(tmp, sizeof(tmp), "%.*e", d - 1, std::fabs(x));
    // tmp = "D.DDDDe+XX"
    std::string t(tmp);
    const size_t epos = t.find('e');
    std::string mant = t.substr(0, epos);
    int ex = std::atoi(t.c_str() + epos + 1) + 1;
    std::string digits;
    for (char ch : mant)
        if (ch != '.') digits += ch;
    char es[16];
    std::snprintf(es, sizeof(es), "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
    std::string s = std::string(x < 0 ? "-" : "") + "0." + digits + es;
    std::snprintf(buf, sizeof(buf), "%*s", w, s.c_str());
    return buf;
}
}  // namespace

extern "C" int tdg_phonon_frequencies(const char *dir, int32_t nq, const double *q, const double *qdir,
                                      double *omega) {
    using namespace tdg;
    if (!dir || nq < 0 || (nq > 0 && (!q || !omega)))
        return set_error(kErrParam, "tdg_phonon_frequencies: null argument");
    const std::string d = std::string(dir) + "/";
    Crystal c;
    int st = read_poscar(d + "infile.ucposcar", c);
    if (st) return st;
    for (int a = 0; a < c.na; ++a)
        if (!(c.mass[a] > 0)) return set_error(kErrParam, "unknown element mass for atom " + std::to_string(a + 1));
    FC2 fc2;
    st = read_fc2(d + "infile.forceconstant", c, fc2);
    if (st) return st;
    std::vector<V3> qv(nq), dv(nq);
    for (int k = 0; k < nq; ++k)
        for (int x = 0; x < 3; ++x) {
            qv[k][x] = q[3 * k + x];
            dv[k][x] = qdir ? qdir[3 * k + x] : (x == 0 ? 1.0 : 0.0);
        }
    return phonon_frequencies(c, fc2, nq, qv.data(), dv.data(), omega);
}

extern "C" int tdg_write_outfile(const char *dir, double temperature, const double *ksma, const double *kiter,
                                 const double *koff) {
    using namespace tdg;
    if (!dir || !ksma || !kiter || !koff) return set_error(kErrParam, "tdg_write_outfile: null argument");
    const std::string path = std::string(dir) + "/outfile.thermal_conductivity";
    std::FILE *u = std::fopen(path.c_str(), "w");
    if (!u) return set_error(kErrIo, "cannot write " + path);
    std::fprintf(u, "# Unit:%15s%s\n", "", "W/m/K");
    std::fprintf(u, "# Temperature:%8s%s\n", "", fortran_e(temperature, 20, 12).c_str());
    auto block = [&](const char *title, const double *m) {
        std::fprintf(u, "%s\n", title);
        std::fprintf(u, "#");
        for (const char *h : {"kxx", "kyy", "kzz", "kxy", "kxz", "kyz"}) std::fprintf(u, " %24s", h);
        std::fprintf(u, "\n ");
        const int idx[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
        for (auto &ij : idx) std::fprintf(u, " %s", fortran_e(m[ij[0] + 3 * ij[1]] * kKappaAuToSI, 24, 12).c_str());
        std::fprintf(u, "\n");
    };
    double coll[9], tot[9];
    for (int i = 0; i < 9; ++i) {
        coll[i] = kiter[i] - ksma[i];
        tot[i] = kiter[i] + koff[i];
    }
    block("# Single mode approximation", ksma);
    block("# Collective contribution", coll);
    block("# Off diagonal (coherence) contribution", koff);
    block("# Total thermal conductivity", tot);
    std::fclose(u);
    return kOk;
}
