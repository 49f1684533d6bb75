// Rows of the scattering matrix and the Monte-Carlo q' samples of every row.
//
// Rows: scattering.f90:170-209 with a single rank (every (q1,b1) with omega >= lo_freqtol).
// Random stream: lo_randomnumbers.f90:203-273. TDEP seeds MT19937-64 with
// init_genrand64 and draws genrand64_real1; that seeding and recurrence are exactly the
// ones of std::mt19937_64 (same multiplier, matrix and tempering constants), so the
// standard engine seeded with the same 64-bit word reproduces TDEP's stream.
// Samples: lo_fftgrid_helper.f90:56-99 (mc_point_to_full, generate_grid).
#include <random>

#include "../../../include/tdep_gb300.h"
#include "crystal.hpp"

namespace tdg {
namespace {

struct McGrid {
    int mc[3], full[3];
    double ratio[3];
    int npoints;
};

McGrid make_grid(const int32_t full[3], const int32_t mc[3]) {
    McGrid g;
    for (int i = 0; i < 3; ++i) {
        g.full[i] = full[i];
        g.mc[i] = std::min(mc[i], full[i]);
        g.ratio[i] = (double)g.full[i] / (double)g.mc[i];
    }
    g.npoints = g.mc[0] * g.mc[1] * g.mc[2];
    return g;
}

// genrand64_real1: 53-bit integer on [0,1] inclusive.
double real1(std::mt19937_64 &rng) { return (double)(rng() >> 11) * (1.0 / (9007199254740992.0 - 1.0)); }

int mc_point_to_full(const McGrid &g, int imc, std::mt19937_64 &rng) {
    // singlet_to_triplet on the MC grid (1-based, last index fastest)
    int k = imc % g.mc[2];
    if (k == 0) k = g.mc[2];
    const int j = ((imc - k) / g.mc[2]) % g.mc[1] + 1;
    const int i = (imc - k - (j - 1) * g.mc[2]) / (g.mc[2] * g.mc[1]) + 1;
    const int gm[3] = {i, j, k};
    int gf[3];
    for (int d = 0; d < 3; ++d) gf[d] = (int)std::ceil(((double)gm[d] - 1.0) * g.ratio[d] + real1(rng) * g.ratio[d]);
    return (gf[0] - 1) * g.full[1] * g.full[2] + (gf[1] - 1) * g.full[2] + gf[2];
}

void generate_grid(const McGrid &g, int32_t *out, std::mt19937_64 &rng) {
    out[0] = mc_point_to_full(g, 1, rng);
    int qprev = out[0], qtest = out[0];
    for (int qi = 2; qi <= g.npoints; ++qi) {
        while (qtest == qprev) qtest = mc_point_to_full(g, qi, rng);
        out[qi - 1] = qtest;
        qprev = qtest;
    }
}

}  // namespace

// 64-bit seed word of init_genrand64(iseed=0, rseed=1/seed).
uint64_t tdep_seed_word(int seed) {
    const double rseed = 1.0 / (double)seed;
    const double f0 = rseed - std::floor(rseed) - 0.5;
    const int64_t s = (int64_t)anint(f0 * 1073741824.0);
    return (uint64_t)s;
}

}  // namespace tdg

extern "C" int tdg_mc_qlists(const tdg_problem *p, const tdg_opts *o, int32_t *n_row, int32_t *row_q1,
                             int32_t *row_b1, int64_t *ptr3, int32_t *list3, int64_t *ptr4, int32_t *list4a,
                             int32_t *list4b) {
    using namespace tdg;
    if (!p || !o || !n_row || !row_q1 || !row_b1) return set_error(kErrParam, "tdg_mc_qlists: null argument");
    if (o->seed <= 0) return set_error(kErrParam, "tdg_mc_qlists: seed must be positive");
    const int nb = p->n_mode;
    int nr = 0;
    for (int q1 = 0; q1 < p->n_irr; ++q1) {
        const int f = p->irr_full[q1] - 1;
        for (int b1 = 0; b1 < nb; ++b1) {
            if (p->omega[(size_t)f * nb + b1] < kFreqTol) continue;
            row_q1[nr] = q1 + 1;
            row_b1[nr] = b1 + 1;
            ++nr;
        }
    }
    *n_row = nr;
    std::mt19937_64 rng(tdep_seed_word(o->seed));
    const McGrid g3 = make_grid(p->grid, o->qg3ph);
    const McGrid g4 = make_grid(p->grid, o->qg4ph);
    if (o->thirdorder && (!ptr3 || !list3)) return set_error(kErrParam, "tdg_mc_qlists: missing third-order lists");
    if (o->fourthorder && (!ptr4 || !list4a || !list4b))
        return set_error(kErrParam, "tdg_mc_qlists: missing fourth-order lists");
    if (ptr3) ptr3[0] = 0;
    if (ptr4) ptr4[0] = 0;
    for (int r = 0; r < nr; ++r) {
        if (o->thirdorder) {
            generate_grid(g3, list3 + (size_t)r * g3.npoints, rng);
            ptr3[r + 1] = (int64_t)(r + 1) * g3.npoints;
        }
        if (o->fourthorder) {
            generate_grid(g4, list4a + (size_t)r * g4.npoints, rng);
            generate_grid(g4, list4b + (size_t)r * g4.npoints, rng);
            ptr4[r + 1] = (int64_t)(r + 1) * g4.npoints;
        }
    }
    return kOk;
}
