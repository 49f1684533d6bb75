// Symmetry-irreducible parameters of the third-order force constants: Phi3 = B x.
//
// The reference's forcemap (src/libolle/type_forcemap*.f90; the tensors are rebuilt from the
// irreducible coefficients in type_forcemap_returntensors.f90:250-362) groups the triplets
// of the third-order force constants into orbits under the space group combined with the
// permutations of the three sites, keeps the components of one representative per orbit
// that its stabiliser leaves free, and builds every other triplet of the orbit by the
// operation that maps the representative onto it. The same construction here: for every
// group element g = (operation, site permutation) the image of each triplet is looked up in
// the triplet list (TDG_ERR_SYMMETRY if the list is not closed under the group), orbits are
// the connected sets, the free components of a representative are the null space of
// sum over its stabiliser of (M_g - 1)^T (M_g - 1) (M_g the 27 x 27 action on the tensor),
// orthonormal, and B_t = M_g B_rep for the first g that takes the representative to t.
// The basis acts on the mass-weighted constants of tdg_problem.fc3_mwm (atoms of one orbit
// have equal masses, so the weighting is constant on an orbit). The acoustic sum rule is not
// imposed on x (force constants that satisfy it keep satisfying it under B B^T).
#include <array>
#include <cmath>
#include <map>
#include <vector>

#include "../../../include/tdep_gb300.h"
#include "common.hpp"

using namespace tdg;

namespace {

struct TripKey {
    std::array<int32_t, 9> v;  // a1, a2, a3, lv2 (3), lv3 (3)
    bool operator<(const TripKey &o) const { return v < o.v; }
};

// Eigen-decomposition of a real symmetric n x n matrix (cyclic Jacobi); a is destroyed,
// w receives the eigenvalues, v the eigenvectors as columns (column-major).
void sym_jacobi(int n, std::vector<double> &a, std::vector<double> &w, std::vector<double> &v) {
    v.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) v[i + (size_t)n * i] = 1.0;
    auto A = [&](int i, int j) -> double & { return a[i + (size_t)n * j]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                tot += A(i, j) * A(i, j);
                if (i != j) off += A(i, j) * A(i, j);
            }
        if (off <= 1e-30 * (tot > 0 ? tot : 1.0)) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A(p, q);
                if (std::fabs(apq) < 1e-300) continue;
                const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - s * akq;
                    A(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - s * aqk;
                    A(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = v[k + (size_t)n * p], vkq = v[k + (size_t)n * q];
                    v[k + (size_t)n * p] = c * vkp - s * vkq;
                    v[k + (size_t)n * q] = s * vkp + c * vkq;
                }
            }
    }
    w.resize(n);
    for (int i = 0; i < n; ++i) w[i] = A(i, i);
}

int find_root(std::vector<int> &par, int x) {
    while (par[x] != x) {
        par[x] = par[par[x]];
        x = par[x];
    }
    return x;
}

}  // namespace

extern "C" int tdg_fc3_irreducible(const tdg_problem *p, int32_t *n_x, int64_t *n_coef, int32_t *t_col0,
                                   int32_t *t_ncol, double *coef, double *x) {
    if (!p || !n_x || !n_coef) return set_error(kErrParam, "tdg_fc3_irreducible: null argument");
    if (p->n_fc3 < 1 || !p->fc3_atoms || !p->fc3_lv || !p->fc3_mwm)
        return set_error(kErrParam, "tdg_fc3_irreducible: the problem has no third-order force constants");
    if (!p->op_cart || !p->op_fmap || !p->atom_shift)
        return set_error(kErrParam, "tdg_fc3_irreducible: the problem lacks the operations' atom maps");
    const int na = p->n_atom, nt = p->n_fc3, nop = p->n_op;
    // real-space fractional rotation W = L^-1 R L and the lattice shift of every atom's image
    M3 L, Li;
    for (int k = 0; k < 9; ++k) L.a[k] = p->latvec[k];
    Li = inverse(L);
    std::vector<std::array<int32_t, 9>> W(nop);
    std::vector<int32_t> shift((size_t)nop * na * 3);
    for (int o = 0; o < nop; ++o) {
        M3 R;
        for (int k = 0; k < 9; ++k) R.a[k] = p->op_cart[(size_t)o * 9 + k];
        const M3 Wd = mul(Li, mul(R, L));
        for (int k = 0; k < 9; ++k) {
            W[o][k] = (int32_t)std::lround(Wd.a[k]);
            if (std::fabs(Wd.a[k] - W[o][k]) > 1e-6) return set_error(kErrSymmetry, "tdg_fc3_irreducible: operation is not a lattice rotation");
        }
        for (int a = 0; a < na; ++a) {
            V3 v0, rv, f;
            for (int d = 0; d < 3; ++d) v0[d] = p->atom_shift[((size_t)o * na + a) * 3 + d];
            rv = mul(R, v0);
            for (int d = 0; d < 3; ++d) rv[d] = -rv[d];  // R r_a + t = r_fmap(a) - R v0
            f = mul(Li, rv);
            for (int d = 0; d < 3; ++d) {
                shift[((size_t)o * na + a) * 3 + d] = (int32_t)std::lround(f[d]);
                if (std::fabs(f[d] - std::lround(f[d])) > 1e-6)
                    return set_error(kErrSymmetry, "tdg_fc3_irreducible: atom shift is not a lattice vector");
            }
        }
    }
    static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    const int ng = nop * 6;
    // 27 x 27 action of every group element on a tensor (component i0 + 3 i1 + 9 i2)
    std::vector<double> M((size_t)ng * 729, 0.0);
    for (int o = 0; o < nop; ++o) {
        const double *R = p->op_cart + (size_t)o * 9;  // column-major: R[r + 3c]
        for (int pi = 0; pi < 6; ++pi) {
            double *Mg = &M[((size_t)o * 6 + pi) * 729];
            for (int k0 = 0; k0 < 3; ++k0)
                for (int k1 = 0; k1 < 3; ++k1)
                    for (int k2 = 0; k2 < 3; ++k2) {
                        int j[3];  // rotated indices of the old sites: old site perm[m] gets k_m
                        j[perm[pi][0]] = k0;
                        j[perm[pi][1]] = k1;
                        j[perm[pi][2]] = k2;
                        const int row = k0 + 3 * k1 + 9 * k2;
                        for (int i0 = 0; i0 < 3; ++i0)
                            for (int i1 = 0; i1 < 3; ++i1)
                                for (int i2 = 0; i2 < 3; ++i2)
                                    Mg[(size_t)row * 27 + i0 + 3 * i1 + 9 * i2] =
                                        R[j[0] + 3 * i0] * R[j[1] + 3 * i1] * R[j[2] + 3 * i2];
                    }
        }
    }
    std::map<TripKey, int> index;
    for (int t = 0; t < nt; ++t) {
        TripKey k;
        for (int s = 0; s < 3; ++s) k.v[s] = p->fc3_atoms[(size_t)t * 3 + s] - 1;
        for (int d = 0; d < 6; ++d) k.v[3 + d] = p->fc3_lv[(size_t)t * 6 + d];
        index[k] = t;
    }
    // image of every triplet under every group element
    std::vector<int32_t> img((size_t)nt * ng);
    for (int t = 0; t < nt; ++t) {
        int at[3], lv[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int s = 0; s < 3; ++s) at[s] = p->fc3_atoms[(size_t)t * 3 + s] - 1;
        for (int d = 0; d < 3; ++d) {
            lv[1][d] = p->fc3_lv[(size_t)t * 6 + d];
            lv[2][d] = p->fc3_lv[(size_t)t * 6 + 3 + d];
        }
        for (int o = 0; o < nop; ++o) {
            int fa[3], pos[3][3];
            for (int s = 0; s < 3; ++s) {
                fa[s] = p->op_fmap[(size_t)o * na + at[s]] - 1;
                for (int r = 0; r < 3; ++r) {
                    int v = shift[((size_t)o * na + at[s]) * 3 + r];
                    for (int c = 0; c < 3; ++c) v += W[o][r + 3 * c] * lv[s][c];
                    pos[s][r] = v;
                }
            }
            for (int pi = 0; pi < 6; ++pi) {
                TripKey k;
                const int s0 = perm[pi][0];
                for (int m = 0; m < 3; ++m) k.v[m] = fa[perm[pi][m]];
                for (int m = 1; m < 3; ++m)
                    for (int r = 0; r < 3; ++r) k.v[3 * m + r] = pos[perm[pi][m]][r] - pos[s0][r];
                auto it = index.find(k);
                if (it == index.end())
                    return set_error(kErrSymmetry, "tdg_fc3_irreducible: the third-order triplets are not closed under "
                                                   "the space group (triplet " + std::to_string(t + 1) + ")");
                img[(size_t)t * ng + o * 6 + pi] = it->second;
            }
        }
    }
    std::vector<int> par(nt);
    for (int t = 0; t < nt; ++t) par[t] = t;
    for (int t = 0; t < nt; ++t)
        for (int g = 0; g < ng; ++g) {
            const int a = find_root(par, t), b = find_root(par, img[(size_t)t * ng + g]);
            if (a != b) par[a > b ? a : b] = a < b ? a : b;
        }
    // representatives (the smallest index of an orbit), the element reaching every member,
    // and the free components of each representative
    std::vector<int> rep(nt), via(nt, -1), orbit_col(nt, -1), orbit_k(nt, 0);
    std::vector<std::vector<double>> basis(nt);
    int32_t ncol = 0;
    int64_t ncoef = 0;
    for (int t = 0; t < nt; ++t) rep[t] = find_root(par, t);
    for (int r = 0; r < nt; ++r) {
        if (rep[r] != r) continue;
        std::vector<double> A(729, 0.0);
        for (int g = 0; g < ng; ++g) {
            const int tg = img[(size_t)r * ng + g];
            if (via[tg] < 0 && rep[tg] == r) via[tg] = g;
            if (tg != r) continue;
            const double *Mg = &M[(size_t)g * 729];
            for (int i = 0; i < 27; ++i)
                for (int j = 0; j < 27; ++j) {
                    double s = 0.0;
                    for (int k = 0; k < 27; ++k) {
                        const double dki = Mg[(size_t)k * 27 + i] - (k == i ? 1.0 : 0.0);
                        const double dkj = Mg[(size_t)k * 27 + j] - (k == j ? 1.0 : 0.0);
                        s += dki * dkj;
                    }
                    A[i + 27 * j] += s;
                }
        }
        std::vector<double> w, V;
        sym_jacobi(27, A, w, V);
        std::vector<double> B;
        for (int c = 0; c < 27; ++c)
            if (std::fabs(w[c]) < 1e-8)
                for (int i = 0; i < 27; ++i) B.push_back(V[i + 27 * c]);  // column c, 27 entries
        const int k = (int)B.size() / 27;
        basis[r] = B;
        orbit_col[r] = ncol;
        orbit_k[r] = k;
        ncol += k;
    }
    for (int t = 0; t < nt; ++t) {
        if (via[t] < 0) return set_error(kErrSymmetry, "tdg_fc3_irreducible: orbit member without a mapping");
        ncoef += 27 * (int64_t)orbit_k[rep[t]];
    }
    *n_x = ncol;
    *n_coef = ncoef;
    if (!t_col0 && !t_ncol && !coef && !x) return kOk;
    if (!t_col0 || !t_ncol || !coef || !x) return set_error(kErrParam, "tdg_fc3_irreducible: output arrays missing");
    int64_t off = 0;
    for (int t = 0; t < nt; ++t) {
        const int r = rep[t], k = orbit_k[r];
        t_col0[t] = orbit_col[r];
        t_ncol[t] = k;
        const double *Mg = &M[(size_t)via[t] * 729];
        // B_t = M_g B_r, stored as 27 rows x k columns
        for (int i = 0; i < 27; ++i)
            for (int c = 0; c < k; ++c) {
                double s = 0.0;
                for (int j = 0; j < 27; ++j) s += Mg[(size_t)i * 27 + j] * basis[r][(size_t)c * 27 + j];
                coef[off + (int64_t)i * k + c] = s;
            }
        off += 27 * (int64_t)k;
    }
    // x: the representatives' components projected on their bases
    for (int r = 0; r < nt; ++r) {
        if (rep[r] != r) continue;
        for (int c = 0; c < orbit_k[r]; ++c) {
            double s = 0.0;
            for (int j = 0; j < 27; ++j) s += basis[r][(size_t)c * 27 + j] * p->fc3_mwm[(size_t)r * 27 + j];
            x[orbit_col[r] + c] = s;
        }
    }
    return kOk;
}
