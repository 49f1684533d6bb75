// Harmonic phonons on every point of the mesh: dynamical matrix and its gradient
// (type_forceconstant_secondorder_dynamicalmatrix.f90:484-788, with the polar
// correction type 3 of :654-714: reciprocal-space Ewald sum and the non-analytic term),
// Hermitian diagonalisation (:113-164), group velocities (:167-200) and the degeneracy
// tables (type_phonon_dispersions.f90:1190-1212).
//
// As in the reference (type_phonon_dispersions_generation.f90:72-170), only the irreducible
// points are diagonalised; every other mesh point takes the frequencies and degeneracy of
// its irreducible point, the rotated velocities and the eigenvectors rotated by
// lo_eigenvector_transformation_matrix (type_symmetryoperation.f90:243-290), conjugated
// under time reversal.
#include <algorithm>
#include <numeric>
#include <thread>

#include "crystal.hpp"

namespace tdg {

int hermitian_jacobi(int n, std::vector<cplx> &a, std::vector<double> &w, std::vector<cplx> &v) {
    // Cyclic Jacobi with complex rotations: for each (p,q) the phase of a_pq is absorbed
    // into column q, then a real Jacobi rotation zeroes the (now real) off-diagonal.
    v.assign((size_t)n * n, cplx(0, 0));
    for (int i = 0; i < n; ++i) v[i + (size_t)n * i] = 1.0;
    auto A = [&](int i, int j) -> cplx & { return a[i + (size_t)n * j]; };
    double scale = 0;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) scale += std::norm(A(i, j));
    if (scale == 0) {
        w.assign(n, 0.0);
        return kOk;
    }
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i)
                if (i != j) off += std::norm(A(i, j));
        if (off <= 1e-30 * scale) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const cplx g = A(p, q);
                const double ag = std::abs(g);
                if (ag <= 1e-300) continue;
                const cplx u = g / ag;
                const double app = A(p, p).real(), aqq = A(q, q).real();
                const double tau = (aqq - app) / (2.0 * ag);
                const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                const double cs = 1.0 / std::sqrt(1.0 + t * t);
                const double sn = t * cs;
                // J = [[c, s], [-conj(u) s, conj(u) c]] acting on columns p, q.
                const cplx jqp = -std::conj(u) * sn, jqq = std::conj(u) * cs;
                for (int k = 0; k < n; ++k) {  // A <- A J
                    const cplx akp = A(k, p), akq = A(k, q);
                    A(k, p) = akp * cs + akq * jqp;
                    A(k, q) = akp * sn + akq * jqq;
                }
                for (int k = 0; k < n; ++k) {  // A <- J^H A
                    const cplx apk = A(p, k), aqk = A(q, k);
                    A(p, k) = cs * apk + std::conj(jqp) * aqk;
                    A(q, k) = sn * apk + std::conj(jqq) * aqk;
                }
                A(p, q) = 0.0;
                A(q, p) = 0.0;
                A(p, p) = A(p, p).real();
                A(q, q) = A(q, q).real();
                for (int k = 0; k < n; ++k) {  // V <- V J
                    const cplx vkp = v[k + (size_t)n * p], vkq = v[k + (size_t)n * q];
                    v[k + (size_t)n * p] = vkp * cs + vkq * jqp;
                    v[k + (size_t)n * q] = vkp * sn + vkq * jqq;
                }
            }
        if (sweep == 99) return set_error(kErrLinalg, "Jacobi eigensolver did not converge");
    }
    w.resize(n);
    for (int i = 0; i < n; ++i) w[i] = A(i, i).real();
    return kOk;
}

namespace {
inline cplx chop(const cplx &z, double tol) {
    return cplx(std::fabs(z.real()) < tol ? 0.0 : z.real(), std::fabs(z.imag()) < tol ? 0.0 : z.imag());
}
}  // namespace

void longrange_dm(const Crystal &c, const FC2 &fc, const V3 &q, bool onsite, cplx *p, cplx *pg) {
    const int na = fc.na;
    const size_t blk = (size_t)9 * na * na;
    // Pairs a1 <= a2 with tau = r(a2) - r(a1); the reciprocal sum accumulates
    // K K^T exp(-|K|^2_eps / 4 lambda^2) / |K|^2_eps exp(-i K.tau) over K = 2 pi (G + q).
    std::vector<int> pa1, pa2;
    std::vector<V3> tau;
    for (int a1 = 0; a1 < na; ++a1)
        for (int a2 = a1; a2 < na; ++a2) {
            V3 t;
            for (int d = 0; d < 3; ++d) {
                t[d] = c.rcart[a2][d] - c.rcart[a1][d];
                if (std::fabs(t[d]) < kSqTol) t[d] = 0.0;
            }
            pa1.push_back(a1);
            pa2.push_back(a2);
            tau.push_back(t);
        }
    const size_t np = tau.size();
    std::vector<cplx> dl(np * 9, 0.0), dq(pg ? np * 27 : 0, 0.0);
    const double inv4l2 = 1.0 / (4.0 * fc.lambda * fc.lambda);
    for (const V3 &g : fc.G) {
        double K[3];
        for (int d = 0; d < 3; ++d) {
            K[d] = (g[d] + q[d]) * kTwoPi;
            if (std::fabs(K[d]) < kSqTol) K[d] = 0.0;
        }
        if (K[0] * K[0] + K[1] * K[1] + K[2] * K[2] < kSqTol * kSqTol) continue;
        double eK[3];
        for (int i = 0; i < 3; ++i) eK[i] = fc.eps(i, 0) * K[0] + fc.eps(i, 1) * K[1] + fc.eps(i, 2) * K[2];
        const double knorm = K[0] * eK[0] + K[1] * eK[1] + K[2] * eK[2];
        const double inv = 1.0 / knorm;
        const double pchi = std::exp(-knorm * inv4l2) * inv;
        double keps[3];  // d|K|^2_eps/dK (1/|K|^2_eps + 1/4 lambda^2): K^T eps, doubled
        for (int i = 0; i < 3; ++i)
            keps[i] = 2.0 * (K[0] * fc.eps(0, i) + K[1] * fc.eps(1, i) + K[2] * fc.eps(2, i)) * (inv + inv4l2);
        for (size_t ip = 0; ip < np; ++ip) {
            const double kr = -(K[0] * tau[ip][0] + K[1] * tau[ip][1] + K[2] * tau[ip][2]);
            const cplx chi = pchi * cplx(std::cos(kr), std::sin(kr));
            for (int j = 0; j < 3; ++j)
                for (int i = 0; i < 3; ++i) dl[ip * 9 + i + 3 * j] += K[i] * K[j] * chi;
            if (!pg) continue;
            for (int d = 0; d < 3; ++d) {
                const cplx v0 = cplx(-keps[d], -tau[ip][d]);  // i*(-tau_d) - keps_d
                for (int j = 0; j < 3; ++j)
                    for (int i = 0; i < 3; ++i) {
                        const double dkk = (i == d ? K[j] : 0.0) + (j == d ? K[i] : 0.0);
                        dq[(ip * 3 + d) * 9 + i + 3 * j] += (K[i] * K[j] * v0 + dkk) * chi;
                    }
            }
        }
    }
    const double f0 = 4.0 * kPi / c.volume;
    // Hermitian completion of the pair blocks, then the Born charges on both sides.
    std::vector<cplx> d0(blk), g0(pg ? 3 * blk : 0);
    for (size_t ip = 0; ip < np; ++ip) {
        const int a1 = pa1[ip], a2 = pa2[ip];
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) {
                const cplx v = dl[ip * 9 + i + 3 * j] * f0;
                d0[((size_t)a1 * na + a2) * 9 + i + 3 * j] = v;
                if (a1 != a2) d0[((size_t)a2 * na + a1) * 9 + j + 3 * i] = std::conj(v);
                if (!pg) continue;
                for (int d = 0; d < 3; ++d) {
                    const cplx w = dq[(ip * 3 + d) * 9 + i + 3 * j] * f0;
                    g0[d * blk + ((size_t)a1 * na + a2) * 9 + i + 3 * j] = w;
                    if (a1 != a2) g0[d * blk + ((size_t)a2 * na + a1) * 9 + j + 3 * i] = std::conj(w);
                }
            }
    }
    const double *Z = fc.Z.data();
    auto zz = [&](const cplx *src, cplx *dst, int a1, int a2) {
        const cplx *s = src + ((size_t)a1 * na + a2) * 9;
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) {
                cplx acc = 0;
                for (int jj = 0; jj < 3; ++jj)
                    for (int ii = 0; ii < 3; ++ii)
                        acc += Z[(size_t)a1 * 9 + i + 3 * ii] * Z[(size_t)a2 * 9 + j + 3 * jj] * s[ii + 3 * jj];
                dst[((size_t)a1 * na + a2) * 9 + i + 3 * j] = acc;
            }
    };
    for (int a1 = 0; a1 < na; ++a1)
        for (int a2 = 0; a2 < na; ++a2) {
            zz(d0.data(), p, a1, a2);
            if (pg)
                for (int d = 0; d < 3; ++d) zz(g0.data() + d * blk, pg + d * blk, a1, a2);
        }
    if (onsite)
        for (int a = 0; a < na; ++a)
            for (int e = 0; e < 9; ++e) p[((size_t)a * na + a) * 9 + e] += fc.Zonsite[(size_t)a * 9 + e];
    for (size_t e = 0; e < blk; ++e) p[e] = chop(p[e], kSqTol);
}

void nonanalytic_dm(const Crystal &c, const FC2 &fc, const V3 &qdir, double *p) {
    const int na = fc.na;
    const double nq = std::sqrt(sqnorm(qdir));
    double u[3] = {qdir[0] / nq, qdir[1] / nq, qdir[2] / nq};
    double qeq = 0;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) qeq += u[i] * fc.eps(i, j) * u[j];
    const double f0 = (1.0 / qeq) * 4.0 * kPi / c.volume;
    std::vector<double> zq((size_t)3 * na);  // zq(i, a) = sum_k u_k Z(i,k,a)
    for (int a = 0; a < na; ++a)
        for (int i = 0; i < 3; ++i) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += u[k] * fc.Z[(size_t)a * 9 + i + 3 * k];
            zq[(size_t)a * 3 + i] = s;
        }
    for (int a1 = 0; a1 < na; ++a1)
        for (int a2 = 0; a2 < na; ++a2)
            for (int j = 0; j < 3; ++j)
                for (int i = 0; i < 3; ++i)
                    p[((size_t)a1 * na + a2) * 9 + i + 3 * j] = zq[(size_t)a1 * 3 + i] * zq[(size_t)a2 * 3 + j] * f0;
}

namespace {

double negsqrt(double x) { return x >= 0 ? std::sqrt(x) : -std::sqrt(-x); }

// D((a2,j),(a1,i)) = sum_pairs exp(i q.R) m(i,j) / sqrt(m1 m2) and its q gradient G, q
// with 2*pi; D and G column-major, G direction-major. Polar force constants add the
// long-range matrix and, at Gamma with qdir given, the non-analytic term along qdir.
void dyn_matrix(const Crystal &c, const FC2 &fc, const V3 &qr, const V3 *qdir, int nb, cplx *D, cplx *G) {
    V3 qv;
    for (int d = 0; d < 3; ++d) {
        qv[d] = qr[d] * kTwoPi;
        if (std::fabs(qv[d]) < 1e-13) qv[d] = 0.0;
    }
    std::fill(D, D + (size_t)nb * nb, cplx(0, 0));
    std::fill(G, G + (size_t)3 * nb * nb, cplx(0, 0));
    for (const auto &p : fc.pairs) {
        const double qdotr = p.lv[0] * qv[0] + p.lv[1] * qv[1] + p.lv[2] * qv[2];
        const cplx e(std::cos(qdotr), std::sin(qdotr));
        const double ms = c.invsqrtmass[p.a1] * c.invsqrtmass[p.a2];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                const int ii = p.a2 * 3 + j, jj = p.a1 * 3 + i;
                const cplx val = e * p.m[i + 3 * j] * ms;
                D[ii + (size_t)nb * jj] += val;
                for (int d = 0; d < 3; ++d) G[(size_t)d * nb * nb + ii + (size_t)nb * jj] += cplx(0, p.lv[d]) * val;
            }
    }
    if (fc.polar != 3) return;
    const int na = fc.na;
    const size_t blk = (size_t)9 * na * na;
    std::vector<cplx> P(blk), PG(3 * blk);
    longrange_dm(c, fc, qr, true, P.data(), PG.data());
    std::vector<double> NA;
    if (qdir && sqnorm(qr) < kSqTol && sqnorm(*qdir) > kSqTol) {
        NA.resize(blk);
        nonanalytic_dm(c, fc, *qdir, NA.data());
    }
    for (int a1 = 0; a1 < na; ++a1)
        for (int a2 = 0; a2 < na; ++a2) {
            const double ms = c.invsqrtmass[a1] * c.invsqrtmass[a2];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    const size_t e = ((size_t)a1 * na + a2) * 9 + i + 3 * j;
                    const size_t at = (size_t)(a2 * 3 + j) + (size_t)nb * (a1 * 3 + i);
                    D[at] += (P[e] + (NA.empty() ? 0.0 : NA[e])) * ms;
                    for (int d = 0; d < 3; ++d) G[(size_t)d * nb * nb + at] += PG[d * blk + e] * ms;
                }
        }
}

int solve_point(const Crystal &c, const FC2 &fc, const V3 &qr, const V3 *qdir, int nb, double *omega, double *egv,
                double *vel) {
    std::vector<cplx> D((size_t)nb * nb), G((size_t)3 * nb * nb);
    dyn_matrix(c, fc, qr, qdir, nb, D.data(), G.data());
    // Hermitise against rounding before diagonalising.
    for (int i = 0; i < nb; ++i)
        for (int j = i; j < nb; ++j) {
            const cplx s = 0.5 * (D[i + (size_t)nb * j] + std::conj(D[j + (size_t)nb * i]));
            D[i + (size_t)nb * j] = s;
            D[j + (size_t)nb * i] = std::conj(s);
        }
    std::vector<cplx> A = D, V;
    std::vector<double> w;
    int st = hermitian_jacobi(nb, A, w, V);
    if (st) return st;
    // Acoustic modes at Gamma: zero the three smallest |eigenvalues|.
    if (sqnorm(qr) < kSqTol) {
        std::vector<int> idx(nb);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return std::fabs(w[a]) < std::fabs(w[b]); });
        for (int i = 0; i < std::min(3, nb); ++i) w[idx[i]] = 0.0;
    }
    std::vector<int> ord(nb);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return negsqrt(w[a]) < negsqrt(w[b]); });
    std::vector<cplx> E((size_t)nb * nb);
    std::vector<double> om(nb);
    for (int b = 0; b < nb; ++b) {
        om[b] = negsqrt(w[ord[b]]);
        for (int r = 0; r < nb; ++r) E[r + (size_t)nb * b] = V[r + (size_t)nb * ord[b]];
    }
    // Degenerate subspaces: rotate the eigenvectors so that the velocity operator along
    // a fixed generic direction is diagonal inside each subspace (a deterministic gauge);
    // the velocities follow the reference's rule for degenerate subspaces
    // (type_forceconstant_secondorder_dynamicalmatrix.f90:313-360): every mode of a
    // subspace gets, per direction, the mean of the subspace's Hellmann-Feynman values
    // <e|dD/dk|e> / (2 omega), which does not depend on the gauge. Subspaces are the modes
    // within lo_freqtol of one another (return_degenerate_subspaces, :911-980).
    const double dir[3] = {1.0, 1.33, 1.45624623};
    for (int b0 = 0; b0 < nb;) {
        int b1 = b0 + 1;
        while (b1 < nb && std::fabs(om[b1] - om[b0]) < kFreqTol) ++b1;
        const int k = b1 - b0;
        if (k > 1) {
            std::vector<cplx> P((size_t)k * k, 0.0);
            for (int x = 0; x < k; ++x)
                for (int y = 0; y < k; ++y) {
                    cplx s = 0;
                    for (int d = 0; d < 3; ++d)
                        for (int r = 0; r < nb; ++r) {
                            cplx gy = 0;
                            for (int cc = 0; cc < nb; ++cc)
                                gy += G[(size_t)d * nb * nb + r + (size_t)nb * cc] * E[cc + (size_t)nb * (b0 + y)];
                            s += dir[d] * std::conj(E[r + (size_t)nb * (b0 + x)]) * gy;
                        }
                    P[x + (size_t)k * y] = s;
                }
            for (int x = 0; x < k; ++x)
                for (int y = x; y < k; ++y) {
                    const cplx s = 0.5 * (P[x + (size_t)k * y] + std::conj(P[y + (size_t)k * x]));
                    P[x + (size_t)k * y] = s;
                    P[y + (size_t)k * x] = std::conj(s);
                }
            std::vector<double> pw;
            std::vector<cplx> U;
            st = hermitian_jacobi(k, P, pw, U);
            if (st) return st;
            std::vector<int> po(k);
            std::iota(po.begin(), po.end(), 0);
            std::stable_sort(po.begin(), po.end(), [&](int a, int b) { return pw[a] < pw[b]; });
            std::vector<cplx> sub((size_t)nb * k, 0.0);
            for (int y = 0; y < k; ++y)
                for (int r = 0; r < nb; ++r) {
                    cplx s = 0;
                    for (int x = 0; x < k; ++x) s += E[r + (size_t)nb * (b0 + x)] * U[x + (size_t)k * po[y]];
                    sub[r + (size_t)nb * y] = s;
                }
            for (int y = 0; y < k; ++y)
                for (int r = 0; r < nb; ++r) E[r + (size_t)nb * (b0 + y)] = sub[r + (size_t)nb * y];
        }
        b0 = b1;
    }
    std::vector<double> hf((size_t)nb * 3);  // <e_b|dD/dk_d|e_b>
    for (int b = 0; b < nb; ++b) {
        omega[b] = om[b];
        for (int r = 0; r < nb; ++r) {
            egv[((size_t)b * nb + r) * 2] = E[r + (size_t)nb * b].real();
            egv[((size_t)b * nb + r) * 2 + 1] = E[r + (size_t)nb * b].imag();
        }
        for (int d = 0; d < 3; ++d) {
            cplx s = 0;
            for (int r = 0; r < nb; ++r) {
                cplx gy = 0;
                for (int cc = 0; cc < nb; ++cc) gy += G[(size_t)d * nb * nb + r + (size_t)nb * cc] * E[cc + (size_t)nb * b];
                s += std::conj(E[r + (size_t)nb * b]) * gy;
            }
            hf[b * 3 + d] = s.real();
        }
    }
    // subspaces: a mode joins the first subspace holding a mode within lo_freqtol of it
    std::vector<int> sub_of(nb, -1);
    int nsub = 0;
    for (int b = 0; b < nb; ++b) {
        for (int a = 0; a < b && sub_of[b] < 0; ++a)
            if (std::fabs(om[a] - om[b]) < kFreqTol) sub_of[b] = sub_of[a];
        if (sub_of[b] < 0) sub_of[b] = nsub++;
    }
    for (int b = 0; b < nb; ++b) {
        double m[3] = {0, 0, 0};
        int cnt = 0;
        for (int a = 0; a < nb; ++a)
            if (sub_of[a] == sub_of[b]) {
                ++cnt;
                for (int d = 0; d < 3; ++d) m[d] += hf[a * 3 + d];
            }
        for (int d = 0; d < 3; ++d) vel[b * 3 + d] = om[b] > kFreqTol ? (m[d] / cnt) / (2.0 * om[b]) : 0.0;
    }
    return kOk;
}

}  // namespace

void dyn_gradient(const Crystal &c, const FC2 &fc, const V3 &qr, int nb, cplx *g) {
    std::vector<cplx> D((size_t)nb * nb);
    dyn_matrix(c, fc, qr, nullptr, nb, D.data(), g);
}

int phonon_frequencies(const Crystal &c, const FC2 &fc, int nq, const V3 *q, const V3 *qdir, double *omega) {
    const int nb = 3 * c.na;
    std::vector<int> status(nq, kOk);
    parallel_for(nq, [&](int64_t k) {
        std::vector<double> egv((size_t)nb * nb * 2), vel((size_t)nb * 3);
        status[k] = solve_point(c, fc, q[k], qdir ? &qdir[k] : nullptr, nb, omega + (size_t)k * nb, egv.data(),
                                vel.data());
    });
    for (int st : status)
        if (st) return st;
    return kOk;
}

int build_phonons(const Crystal &c, const FC2 &fc, const QMesh &qp, Phonons &ph) {
    V3 kDefaultDir;
    kDefaultDir[0] = 1.0;
    const int nb = 3 * c.na;
    const int np = qp.n_full, ni = qp.n_irr;
    // irreducible points; the mesh takes the default direction [1,0,0] at Gamma
    // (type_phonon_dispersions.f90:1099, 1148)
    std::vector<double> om_i((size_t)ni * nb), egv_i((size_t)ni * nb * nb * 2), vel_i((size_t)ni * nb * 3);
    std::vector<int> status(ni, kOk);
    parallel_for(ni, [&](int64_t i) {
        status[i] = solve_point(c, fc, qp.q_full[qp.irr_full[i] - 1], &kDefaultDir, nb, &om_i[(size_t)i * nb],
                                &egv_i[(size_t)i * nb * nb * 2], &vel_i[(size_t)i * nb * 3]);
    });
    for (int st : status)
        if (st) return st;
    std::vector<int32_t> fmap;
    std::vector<double> shift;
    int st = op_atom_maps(c, fmap, shift);
    if (st) return st;
    return unfold_phonons(c, qp, nb, om_i.data(), egv_i.data(), vel_i.data(), fmap, shift, ph);
}

int unfold_phonons(const Crystal &c, const QMesh &qp, int nb, const double *om_i, const double *egv_i,
                   const double *vel_i, const std::vector<int32_t> &fmap, const std::vector<double> &shift,
                   Phonons &ph) {
    const int np = qp.n_full, ni = qp.n_irr, na = c.na;
    ph.n_mode = nb;
    ph.omega.assign((size_t)np * nb, 0.0);
    ph.egv.assign((size_t)np * nb * nb * 2, 0.0);
    ph.vel.assign((size_t)np * nb * 3, 0.0);
    ph.degen.assign((size_t)np * nb, 0);
    ph.degen_mode.assign((size_t)np * nb * nb, 0);
    // degeneracy of the irreducible points (type_phonon_dispersions.f90:1190-1212), copied
    // onto their stars
    std::vector<int32_t> dg((size_t)ni * nb), dm((size_t)ni * nb * nb, 0);
    for (int i = 0; i < ni; ++i) {
        const double *om = om_i + (size_t)i * nb;
        for (int b1 = 0; b1 < nb; ++b1) {
            int l = 0;
            for (int b2 = 0; b2 < nb; ++b2)
                if (std::fabs(om[b1] - om[b2]) < kFreqTol) dm[((size_t)i * nb + b1) * nb + l++] = b2 + 1;
            dg[(size_t)i * nb + b1] = l;
        }
    }
    parallel_for(np, [&](int64_t q) {
        const int i = qp.full_irr[q] - 1, iop = qp.full_op[q], o = std::abs(iop) - 1;
        const M3 &m = c.ops[o].m;
        const double sg = iop > 0 ? 1.0 : -1.0;
        const V3 &qi = qp.q_full[qp.irr_full[i] - 1];
        std::copy(om_i + (size_t)i * nb, om_i + (size_t)(i + 1) * nb, &ph.omega[(size_t)q * nb]);
        std::copy(&dg[(size_t)i * nb], &dg[(size_t)(i + 1) * nb], &ph.degen[(size_t)q * nb]);
        std::copy(&dm[(size_t)i * nb * nb], &dm[(size_t)(i + 1) * nb * nb], &ph.degen_mode[(size_t)q * nb * nb]);
        for (int b = 0; b < nb; ++b) {
            const double *v = vel_i + ((size_t)i * nb + b) * 3;
            for (int d = 0; d < 3; ++d)
                ph.vel[((size_t)q * nb + b) * 3 + d] = sg * (m(d, 0) * v[0] + m(d, 1) * v[1] + m(d, 2) * v[2]);
        }
        for (int a2 = 0; a2 < na; ++a2) {
            const int a1 = fmap[(size_t)o * na + a2];
            const double *v0 = &shift[((size_t)o * na + a2) * 3];
            const double arg = -(v0[0] * qi[0] + v0[1] * qi[1] + v0[2] * qi[2]) * kTwoPi;
            const cplx ph0(std::cos(arg), std::sin(arg));
            for (int b = 0; b < nb; ++b) {
                const double *e = egv_i + (((size_t)i * nb + b) * nb + 3 * a2) * 2;
                for (int x = 0; x < 3; ++x) {
                    cplx s = 0;
                    for (int y = 0; y < 3; ++y) s += m(x, y) * cplx(e[2 * y], e[2 * y + 1]);
                    s *= ph0;
                    if (iop < 0) s = std::conj(s);
                    double *out = &ph.egv[(((size_t)q * nb + b) * nb + 3 * a1 + x) * 2];
                    out[0] = s.real();
                    out[1] = s.imag();
                }
            }
        }
    });
    return kOk;
}

}  // namespace tdg
