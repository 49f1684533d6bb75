// thermal_conductivity host driver over the C-ABI: the call sequence of
// src/thermal_conductivity/main.f90 (read inputs, mesh, phonons, sr%generate,
// get_kappa / iterative_solution / symmetrize_kappa, outfile.thermal_conductivity)
// with the hot path on the GB300 library. Flags follow options.f90.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tdep_gb300.h"

namespace {

constexpr double kEvToHartree = 1.0 / 27.21138602;
constexpr double kBohrToM = 0.52917721067E-10;
constexpr double kHartreeToJoule = 27.21138602 * 1.6021766208E-19;
constexpr double kTimeAuToS = 6.582119514E-16 * 1.6021766208E-19 / kHartreeToJoule;
constexpr double kKappaAuToSI = kHartreeToJoule / kTimeAuToS / kBohrToM;

void usage() {
    std::printf(
        "Usage: thermal_conductivity [-qg n n n] [-qg3ph n n n] [-qg4ph n n n] [--temperature T]\n"
        "       [-it 1|2|6] [--sigma s] [--noisotope] [--readiso] [--fourthorder] [--nothirdorder]\n"
        "       [--classical] [--seed n] [--iterative_tolerance t] [--iterative_maxsteps n]\n"
        "       [--max_mfp m] [--notr] [--mixed] [--device d] [--dir path]\n");
}

int die(int code) {
    std::fprintf(stderr, "thermal_conductivity: %s (code %d)\n", tdg_last_error(), code);
    return code;
}

}  // namespace

int main(int argc, char **argv) {
    int32_t qg[3] = {26, 26, 26}, qg3[3] = {-1, -1, -1}, qg4[3] = {-1, -1, -1};
    tdg_opts o;
    std::memset(&o, 0, sizeof(o));
    o.temperature = 300.0;
    o.integrationtype = 2;
    o.sigma = 1.0;
    o.thirdorder = 1;
    o.isotope = 1;
    o.mfp_max = -1.0;
    o.seed = -1;
    o.precision = TDG_PREC_FP64;
    double itertol = 1e-5;
    int itermax = 200, readiso = 0, timereversal = 1, device = 0;
    std::string dir = ".";
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto need = [&](int k) {
            if (i + k >= argc) {
                usage();
                std::exit(5);
            }
        };
        if (a == "-qg" || a == "--qpoint_grid") {
            need(3);
            for (int d = 0; d < 3; ++d) qg[d] = std::atoi(argv[++i]);
        } else if (a == "-qg3ph" || a == "--qpoint_grid3ph") {
            need(3);
            for (int d = 0; d < 3; ++d) qg3[d] = std::atoi(argv[++i]);
        } else if (a == "-qg4ph" || a == "--qpoint_grid4ph") {
            need(3);
            for (int d = 0; d < 3; ++d) qg4[d] = std::atoi(argv[++i]);
        } else if (a == "--temperature") {
            need(1);
            o.temperature = std::atof(argv[++i]);
        } else if (a == "-it" || a == "--integrationtype") {
            need(1);
            o.integrationtype = std::atoi(argv[++i]);
        } else if (a == "--sigma") {
            need(1);
            o.sigma = std::atof(argv[++i]);
        } else if (a == "--noisotope") {
            o.isotope = 0;
        } else if (a == "--readiso") {
            readiso = 1;
        } else if (a == "--fourthorder") {
            o.fourthorder = 1;
        } else if (a == "--nothirdorder") {
            o.thirdorder = 0;
        } else if (a == "--classical") {
            o.classical = 1;
        } else if (a == "--seed") {
            need(1);
            o.seed = std::atoi(argv[++i]);
        } else if (a == "--iterative_tolerance") {
            need(1);
            itertol = std::atof(argv[++i]);
        } else if (a == "--iterative_maxsteps") {
            need(1);
            itermax = std::atoi(argv[++i]);
        } else if (a == "--max_mfp") {
            need(1);
            o.mfp_max = std::atof(argv[++i]) / kBohrToM;
        } else if (a == "--notr") {
            timereversal = 0;
        } else if (a == "--mixed") {
            o.precision = TDG_PREC_MIXED;
        } else if (a == "--device") {
            need(1);
            device = std::atoi(argv[++i]);
        } else if (a == "--dir") {
            need(1);
            dir = argv[++i];
        } else if (a == "-h" || a == "--help") {
            usage();
            return 0;
        } else {
            std::fprintf(stderr, "unknown option %s\n", a.c_str());
            usage();
            return 5;
        }
    }
    // options.f90:205-235: defaults of the Monte-Carlo grids
    for (int d = 0; d < 3; ++d) {
        o.qg3ph[d] = (qg3[d] < 0 || qg3[d] > qg[d]) ? qg[d] : qg3[d];
        o.qg4ph[d] = (qg4[d] < 0 || qg4[d] > qg[d]) ? qg[d] : qg4[d];
    }
    if (o.seed <= 0) o.seed = (int32_t)(std::chrono::system_clock::now().time_since_epoch().count() % 1000000007) + 1;
    (void)kEvToHartree;

    const auto t0 = std::chrono::steady_clock::now();
    tdg_problem *prob = nullptr;
    int st = tdg_problem_load(dir.c_str(), qg, o.fourthorder, readiso, timereversal, &prob);
    if (st) return die(st);
    double omin = 1e300;
    for (size_t i = 0; i < (size_t)prob->n_full * prob->n_mode; ++i) omin = std::fmin(omin, prob->omega[i]);
    if (omin < -1E-9) {
        std::printf("\n FOUND UNSTABLE MODES. WILL STOP NOW.\n");
        tdg_problem_free(prob);
        return 0;
    }
    std::printf(" ... read inputs, %d x %d x %d mesh, %d irreducible points, %d operations\n", qg[0], qg[1], qg[2],
                prob->n_irr, prob->n_op);
    tdg_ctx *ctx = nullptr;
    st = tdg_create(&ctx, prob, device);
    if (st) return die(st);
    const int cap = prob->n_irr * prob->n_mode;
    const int64_t np3 = (int64_t)o.qg3ph[0] * o.qg3ph[1] * o.qg3ph[2];
    const int64_t np4 = (int64_t)o.qg4ph[0] * o.qg4ph[1] * o.qg4ph[2];
    std::vector<int32_t> rq1(cap), rb1(cap);
    std::vector<int64_t> p3(cap + 1), p4(cap + 1);
    std::vector<int32_t> l3(o.thirdorder ? cap * np3 : 1), l4a(o.fourthorder ? cap * np4 : 1),
        l4b(o.fourthorder ? cap * np4 : 1);
    int32_t nrow = 0;
    st = tdg_mc_qlists(prob, &o, &nrow, rq1.data(), rb1.data(), p3.data(), l3.data(), p4.data(), l4a.data(), l4b.data());
    if (st) return die(st);
    tdg_qlists ql;
    ql.n_row = nrow;
    ql.row_q1 = rq1.data();
    ql.row_b1 = rb1.data();
    ql.ptr3 = o.thirdorder ? p3.data() : nullptr;
    ql.list3 = l3.data();
    ql.ptr4 = o.fourthorder ? p4.data() : nullptr;
    ql.list4a = l4a.data();
    ql.list4b = l4b.data();
    std::vector<double> lw(cap), qs(cap);
    double stats[10];
    const auto t1 = std::chrono::steady_clock::now();
    st = tdg_scattering(ctx, &o, &ql, lw.data(), qs.data(), stats);
    if (st) return die(st);
    const auto t2 = std::chrono::steady_clock::now();
    std::printf(" ... scattering: %.0f irreducible q-triplets in %.3f ms on the device\n", stats[0], stats[2]);
    double ksma[9], kiter[9], koff[9] = {0};
    int32_t nit = 0;
    // main.f90:219-244: single-mode, off-diagonal (coherence) and collective contributions
    st = tdg_kappa_offdiag(ctx, &o, koff);
    if (st) return die(st);
    std::vector<double> fn((size_t)cap * 3);
    st = tdg_kappa(ctx, &o, itermax, itertol, ksma, kiter, fn.data(), &nit);
    if (st) return die(st);
    const auto t3 = std::chrono::steady_clock::now();
    std::printf(" ... iterative solution: %d iterations\n", nit);
    std::printf(" Total thermal conductivity (W/m/K): kxx %.6f kyy %.6f kzz %.6f\n",
                (kiter[0] + koff[0]) * kKappaAuToSI, (kiter[4] + koff[4]) * kKappaAuToSI,
                (kiter[8] + koff[8]) * kKappaAuToSI);
    st = tdg_write_outfile(dir.c_str(), o.temperature, ksma, kiter, koff);
    if (st) return die(st);
    // main.f90:339: the per-mode data of the full mesh
    st = tdg_write_grid_hdf5((dir + "/outfile.thermal_conductivity_grid.hdf5").c_str(), prob, o.temperature, lw.data(),
                             fn.data());
    if (st) return die(st);
    auto ms = [](auto a, auto b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
    std::printf(" Timings (ms): init %.1f  scattering %.1f  kappa %.1f\n", ms(t0, t1), ms(t1, t2), ms(t2, t3));
    tdg_destroy(ctx);
    tdg_problem_free(prob);
    return 0;
}
