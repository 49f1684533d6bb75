// Gamma-centred FFT q-mesh with its irreducible wedge, the map from every point to the
// wedge and the little groups of the irreducible points.
// Follows type_qpointmesh_gridgeneration.f90:8-545 (build_grid for lo_fft_mesh),
// :612-680 (on-grid test, index from coordinate; here exact, on integer coordinates) and
// type_qpointmesh.f90:660-700 (lo_get_small_group_of_qpoint).
#include <algorithm>
#include <numeric>

#include "crystal.hpp"

namespace tdg {

int build_fft_mesh(const Crystal &c, const int grid[3], bool timereversal, QMesh &qp) {
    for (int i = 0; i < 3; ++i)
        if (grid[i] < 1) return set_error(kErrParam, "q-grid dimensions must be positive");
    for (int i = 0; i < 3; ++i) qp.grid[i] = grid[i];
    const int np = grid[0] * grid[1] * grid[2];
    const int nsym = (int)c.ops.size();
    qp.n_full = np;
    PhaseTimer pt("mesh");

    // Points in fractional coordinates, moved to the first zone. The zone test uses the
    // shortest Cartesian vector among the 27 nearest reciprocal lattice translations,
    // with lo_degenvector breaking ties predictably.
    qp.qfrac.assign(np, V3());
    // the same points as integers: qfrac = nq / g exactly
    std::vector<int32_t> nq((size_t)np * 3);
    // Connections: op j maps point i to point connections[i][j] (time reversal: -index).
    // The reference tests in fractional coordinates whether R q is on the mesh and whether
    // R^-1 maps its image back onto q. On integer coordinates the first test is exact:
    // (R q)_i = sum_k R_ik n_k / g_k is on the mesh when num_i = sum_k R_ik n_k (L / g_k), L
    // the least common multiple of the g_k, is a multiple of L / g_i; the second test then
    // always holds (R^-1 is an integer matrix and maps the image's mesh point, which differs
    // from R q by a reciprocal lattice vector, back onto q's).
    const int nc = timereversal ? 2 * nsym : nsym;
    std::vector<int> conn((size_t)np * nc, 0);
    int64_t L = grid[0];
    for (int d = 1; d < 3; ++d) L = L / std::gcd(L, (int64_t)grid[d]) * grid[d];
    const int64_t sg3[3] = {L / grid[0], L / grid[1], L / grid[2]};
    // With equal dimensions (L / g = 1) every image is on the mesh and the wrap needs no
    // division. Each point's row is made right after its first-zone coordinates.
    const bool equal = sg3[0] == 1 && sg3[1] == 1 && sg3[2] == 1;
    auto connect = [&](int64_t i) {
        const int32_t *n = &nq[(size_t)i * 3];
        for (int j = 0; j < nsym; ++j) {
            const int32_t *m = c.ops[j].rfm;
            int64_t gi[3];
            bool on = true;
            if (equal) {
                const int g = grid[0];
                for (int r = 0; r < 3; ++r) {
                    int v = m[r] * n[0] + m[r + 3] * n[1] + m[r + 6] * n[2];
                    while (v < 0) v += g;
                    while (v >= g) v -= g;
                    gi[r] = v;
                }
            } else {
                for (int r = 0; r < 3 && on; ++r) {
                    const int64_t num = m[r] * n[0] * sg3[0] + m[r + 3] * n[1] * sg3[1] + m[r + 6] * n[2] * sg3[2];
                    on = num % sg3[r] == 0;
                    gi[r] = num / sg3[r];
                }
            }
            if (!on) continue;
            for (int tr = 0; tr < (timereversal ? 2 : 1); ++tr) {
                int64_t idx = 0;
                for (int r = 0; r < 3; ++r) {
                    const int64_t v = ((tr ? -gi[r] : gi[r]) % grid[r] + grid[r]) % grid[r];
                    idx = idx * grid[r] + v;
                }
                const int ii = (int)idx + 1;
                conn[(size_t)i * nc + j + tr * nsym] = tr ? -ii : ii;
            }
        }
    };
    parallel_for(np, [&](int64_t l) {  // point l = ((i - 1) g1 + j - 1) g2 + k - 1
        const int k = (int)(l % grid[2]) + 1, j = (int)((l / grid[2]) % grid[1]) + 1,
                  i = (int)(l / ((int64_t)grid[1] * grid[2])) + 1;
        V3 v0;
        v0[0] = (i - 1.0) / grid[0];
        v0[1] = (j - 1.0) / grid[1];
        v0[2] = (k - 1.0) / grid[2];
        double best = 1e300;
        V3 bv = v0;
        int sh[3] = {0, 0, 0};
        for (int a = -1; a <= 1; ++a)
            for (int b = -1; b <= 1; ++b)
                for (int cc = -1; cc <= 1; ++cc) {
                    V3 w;
                    w[0] = v0[0] - a;
                    w[1] = v0[1] - b;
                    w[2] = v0[2] - cc;
                    V3 kc = mul(c.reclat, w);
                    for (int d = 0; d < 3; ++d) kc[d] += kDegenVector[d];
                    const double s = sqnorm(kc);
                    if (s < best - 1e-12) {
                        best = s;
                        bv = w;
                        sh[0] = a;
                        sh[1] = b;
                        sh[2] = cc;
                    }
                }
        qp.qfrac[l] = bv;
        nq[(size_t)l * 3] = i - 1 - sh[0] * grid[0];
        nq[(size_t)l * 3 + 1] = j - 1 - sh[1] * grid[1];
        nq[(size_t)l * 3 + 2] = k - 1 - sh[2] * grid[2];
        connect(l);  // its images under every operation (needs only its own coordinates)
    });

    pt.mark("first zone and connections");
    // Irreducible points: smallest index of every orbit.
    std::vector<int> ind(np, 1);
    for (int i = 0; i < np; ++i)
        for (int j = 0; j < nc; ++j) {
            const int k = std::abs(conn[(size_t)i * nc + j]);
            if (k > i + 1) ind[k - 1] = 0;
        }
    qp.irr_full.clear();
    for (int i = 0; i < np; ++i)
        if (ind[i]) qp.irr_full.push_back(i + 1);
    qp.n_irr = (int)qp.irr_full.size();

    qp.full_irr.assign(np, 0);
    qp.full_op.assign(np, 0);
    for (int k = 0; k < qp.n_irr; ++k) {
        const int base = qp.irr_full[k] - 1;
        for (int j = 0; j < nsym; ++j) {
            const int i = conn[(size_t)base * nc + j];
            if (i == 0) continue;
            if (qp.full_irr[i - 1] != 0) continue;
            qp.full_irr[i - 1] = k + 1;
            qp.full_op[i - 1] = j + 1;
        }
        if (timereversal) {
            for (int j = 0; j < nsym; ++j) {
                const int i = -conn[(size_t)base * nc + j + nsym];
                if (i == 0) continue;
                if (qp.full_irr[i - 1] != 0) continue;
                qp.full_irr[i - 1] = k + 1;
                qp.full_op[i - 1] = -(j + 1);
            }
        }
    }
    for (int i = 0; i < np; ++i)
        if (qp.full_irr[i] == 0) return set_error(kErrSymmetry, "Failed miserably mapping irreducible grid to full");

    qp.irr_weight.assign(qp.n_irr, 0.0);
    for (int i = 0; i < np; ++i) qp.irr_weight[qp.full_irr[i] - 1] += 1.0;
    for (double &w : qp.irr_weight) w /= (double)np;

    qp.q_full.assign(np, V3());
    for (int i = 0; i < np; ++i) {
        V3 r = mul(c.reclat, qp.qfrac[i]);
        for (int d = 0; d < 3; ++d)
            if (std::fabs(r[d]) < 1e-14) r[d] = 0.0;
        qp.q_full[i] = r;
    }

    pt.mark("wedge and q");
    // Little groups of the irreducible points (proper operations, no time reversal).
    qp.irr_nop.assign(qp.n_irr, 0);
    qp.irr_ops.assign((size_t)qp.n_irr * nsym, 0);
    parallel_for(qp.n_irr, [&](int64_t k) {
        const V3 &v0 = qp.q_full[qp.irr_full[k] - 1];
        int ctr = 0;
        for (int i = 0; i < nsym; ++i) {
            V3 rv = mul(c.ops[i].m, v0);
            V3 d;
            for (int x = 0; x < 3; ++x) d[x] = v0[x] - rv[x];
            V3 f = mul(c.inv_reclat, d);
            for (int x = 0; x < 3; ++x) f[x] -= anint(f[x]);
            if (sqnorm(f) < kSqTol) qp.irr_ops[(size_t)k * nsym + ctr++] = i + 1;
        }
        qp.irr_nop[k] = ctr;
    });
    pt.mark("little groups");
    return kOk;
}

}  // namespace tdg
