// Gamma-centred FFT q-mesh with its irreducible wedge, the map from every point to the
// wedge and the little groups of the irreducible points.
// Follows type_qpointmesh_gridgeneration.f90:8-545 (build_grid for lo_fft_mesh),
// :612-680 (on-grid test, index from coordinate) and type_qpointmesh.f90:660-700
// (lo_get_small_group_of_qpoint).
#include <algorithm>

#include "crystal.hpp"

namespace tdg {

namespace {

// lo_clean_fractional_coordinates (gottochblandat.f90:1261-1283) with tol = lo_sqtol.
double clean_frac(double x) {
    double y = x;
    for (int guard = 0; guard < 64; ++guard) {
        if (std::fabs(y) < kSqTol) y = 0.0;
        if (std::fabs(y - 1.0) < kSqTol) y = 0.0;
        if (y > 1.0) y -= 1.0;
        if (y < 0.0) y += 1.0;
        if (y > -kSqTol && y < 1.0) break;
    }
    return y;
}

bool on_grid(const int g[3], const V3 &r) {
    double s = 0;
    for (int j = 0; j < 3; ++j) {
        const double v = r[j] * g[j] + 1.0;
        s += std::fabs(v - anint(v));
    }
    return s < kTol;
}

// 1-based linear index of a fractional coordinate on the grid.
int index_from_coordinate(const int g[3], const V3 &r) {
    int gi[3];
    for (int j = 0; j < 3; ++j) {
        const double v = clean_frac(r[j]) * g[j] + 1.0;
        gi[j] = (int)anint(v);
    }
    for (int j = 0; j < 3; ++j) {
        if (gi[j] > g[j]) gi[j] -= g[j];
        if (gi[j] < 1) gi[j] += g[j];
    }
    return (gi[0] - 1) * g[1] * g[2] + (gi[1] - 1) * g[2] + gi[2];
}

V3 apply_int(const int32_t *m, const V3 &v, double sign) {
    V3 r;
    for (int i = 0; i < 3; ++i) r[i] = sign * (m[i] * v[0] + m[i + 3] * v[1] + m[i + 6] * v[2]);
    return r;
}

void inverse_int(const int32_t *m, int32_t *inv) {
    M3 a;
    for (int k = 0; k < 9; ++k) a.a[k] = m[k];
    M3 b = inverse(a);
    for (int k = 0; k < 9; ++k) inv[k] = (int32_t)anint(b.a[k]);
}

}  // namespace

int build_fft_mesh(const Crystal &c, const int grid[3], bool timereversal, QMesh &qp) {
    for (int i = 0; i < 3; ++i)
        if (grid[i] < 1) return set_error(kErrParam, "q-grid dimensions must be positive");
    for (int i = 0; i < 3; ++i) qp.grid[i] = grid[i];
    const int np = grid[0] * grid[1] * grid[2];
    const int nsym = (int)c.ops.size();
    qp.n_full = np;

    // Points in fractional coordinates, moved to the first zone. The zone test uses the
    // shortest Cartesian vector among the 27 nearest reciprocal lattice translations,
    // with lo_degenvector breaking ties predictably.
    qp.qfrac.assign(np, V3());
    for (int i = 1, l = 0; i <= grid[0]; ++i)
        for (int j = 1; j <= grid[1]; ++j)
            for (int k = 1; k <= grid[2]; ++k, ++l) {
                V3 v0;
                v0[0] = (i - 1.0) / grid[0];
                v0[1] = (j - 1.0) / grid[1];
                v0[2] = (k - 1.0) / grid[2];
                double best = 1e300;
                V3 bv = v0;
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
                            }
                        }
                qp.qfrac[l] = bv;
            }

    // Connections: op j maps point i to point connections[i][j] (time reversal: -index).
    const int nc = timereversal ? 2 * nsym : nsym;
    std::vector<int> conn((size_t)np * nc, 0);
    std::vector<int32_t> irfm(9 * nsym);
    for (int j = 0; j < nsym; ++j) inverse_int(c.ops[j].rfm, &irfm[9 * j]);
    // rows are independent: all host threads (54 ms for 24^3 and 48 operations on one core)
    parallel_for(np, [&](int64_t i) {
        const V3 &v0 = qp.qfrac[i];
        for (int tr = 0; tr < (timereversal ? 2 : 1); ++tr) {
            const double sg = tr ? -1.0 : 1.0;
            for (int j = 0; j < nsym; ++j) {
                V3 v1 = apply_int(c.ops[j].rfm, v0, sg);
                if (!on_grid(grid, v1)) continue;
                const int ii = index_from_coordinate(grid, v1);
                V3 v2 = apply_int(&irfm[9 * j], qp.qfrac[ii - 1], sg);
                if (!on_grid(grid, v2)) continue;
                const int jj = index_from_coordinate(grid, v2);
                if (jj != i + 1) continue;
                conn[(size_t)i * nc + j + tr * nsym] = tr ? -ii : ii;
            }
        }
    });

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

    // Little groups of the irreducible points (proper operations, no time reversal).
    qp.irr_nop.assign(qp.n_irr, 0);
    qp.irr_ops.assign((size_t)qp.n_irr * nsym, 0);
    for (int k = 0; k < qp.n_irr; ++k) {
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
    }
    return kOk;
}

}  // namespace tdg
