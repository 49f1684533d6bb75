// outfile.thermal_conductivity_grid.hdf5: the per-mode data of the full mesh that
// thermal_conductivity writes after the kappa solve (src/libolle/type_phonon_dispersions.f90:
// 316-641, write_to_hdf5, called at src/thermal_conductivity/main.f90:339), with the final
// prefactor of Fn (omega/T, main.f90:321-327) applied to the per-mode conductivity.
//
// Datasets (C order, the Fortran arrays' dimensions reversed as the Fortran HDF5 interface
// stores them): qpoints, frequencies, group_velocities, eigenvectors_re/_im, lifetimes,
// lattice_vectors, linewidths, mean_free_paths, thermal_conductivity, harmonic_heat_capacity;
// attributes number_of_atoms, number_of_bands, number_of_qpoints, meshtype, temperature.
// The reference's other datasets (Gruneisen parameters, frequency shifts, anharmonic free
// energies, plus/minus scattering rates) are not computed by thermal_conductivity and are
// absent there as well.
#include <cmath>
#include <vector>

#include "../../../include/tdep_gb300.h"
#include "common.hpp"
#include "h5write.hpp"

using namespace tdg;

extern "C" int tdg_write_grid_hdf5(const char *path, const tdg_problem *p, double temperature,
                                   const double *linewidth, const double *fn) {
    if (!path || !p || !linewidth) return set_error(kErrParam, "tdg_write_grid_hdf5: null argument");
    if (!p->omega || !p->vel || !p->egv || !p->q_full || !p->full_irr || !p->full_op || !p->irr_full || !p->op_cart)
        return set_error(kErrParam, "tdg_write_grid_hdf5: problem arrays missing");
    if (!(temperature > 0) || !std::isfinite(temperature))
        return set_error(kErrPhysical, "tdg_write_grid_hdf5: bad temperature");
    const int n = p->n_mode, N = p->n_full, nirr = p->n_irr;
    const double hz = 1.0 / kHbarHartree;  // lo_frequency_Hartree_to_Hz
    // smallest non-zero frequency over the irreducible points (dr%omega_min)
    double omin = 1e300;
    for (int l = 0; l < nirr; ++l)
        for (int j = 0; j < n; ++j) {
            const double w = p->omega[(size_t)(p->irr_full[l] - 1) * n + j];
            if (std::fabs(w) > kFreqTol) omin = std::min(omin, w);
        }
    H5Writer h;
    h.attr_int("number_of_atoms", n / 3);
    h.attr_int("number_of_bands", n);
    h.attr_int("number_of_qpoints", N);
    h.attr_string("meshtype", "FFT");
    const size_t nm = (size_t)N * n;
    std::vector<double> q(p->q_full, p->q_full + (size_t)N * 3);
    h.dataset("qpoints", {(uint64_t)N, 3}, q, "1/A", "q-vector,xyz");
    std::vector<double> f(nm), lt(nm), lw(nm), mfp(nm), cv(nm), vel((size_t)nm * 3), er(nm * n), ei(nm * n);
    for (int i = 0; i < N; ++i) {
        const int l = p->full_irr[i] - 1;
        for (int j = 0; j < n; ++j) {
            const size_t ij = (size_t)i * n + j;
            const double g = linewidth[(size_t)l * n + j];
            f[ij] = p->omega[ij] * hz;
            lt[ij] = g > kFreqTol / 10 ? 0.5 / (g * hz) : 0.0;
            lw[ij] = g * hz;
            const double *v = p->vel + ij * 3;
            double m = 0.0;
            if (g > kFreqTol) {
                m = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * 0.5 / g;
                m = m > kTol ? m * kBohrToM : 0.0;
            }
            mfp[ij] = m;
            cv[ij] = harmonic_oscillator_cv(temperature, p->omega[ij]) * kHartreeToJoule;
            for (int x = 0; x < 3; ++x) vel[ij * 3 + x] = v[x] * kGroupVelAuToMs;
            for (int r = 0; r < n; ++r) {
                er[ij * n + r] = p->egv[(ij * n + r) * 2];
                ei[ij * n + r] = p->egv[(ij * n + r) * 2 + 1];
            }
        }
    }
    h.dataset("frequencies", {(uint64_t)N, (uint64_t)n}, f, "Hz (angular)", "q-vector,mode");
    h.dataset("group_velocities", {(uint64_t)N, (uint64_t)n, 3}, vel, "m/s", "q-vector,mode,xyz");
    h.dataset("eigenvectors_re", {(uint64_t)N, (uint64_t)n, (uint64_t)n}, er, "dimensionless",
              "q-vector,mode,atom-xyz");
    h.dataset("eigenvectors_im", {(uint64_t)N, (uint64_t)n, (uint64_t)n}, ei, "dimensionless",
              "q-vector,mode,atom-xyz");
    h.dataset("lifetimes", {(uint64_t)N, (uint64_t)n}, lt, "s", "q-vector,mode");
    std::vector<double> lat(9);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) lat[a * 3 + b] = p->latvec[a + 3 * b] * kBohrToA;
    h.dataset("lattice_vectors", {3, 3}, lat, "A", "xyz,xyz");
    h.dataset("linewidths", {(uint64_t)N, (uint64_t)n}, lw, "Hz", "q-vector,mode");
    h.dataset("mean_free_paths", {(uint64_t)N, (uint64_t)n}, mfp, "m", "q-vector,mode");
    // per-mode conductivity of every mesh point: kappa_ab, stored [q][mode][b][a]
    std::vector<double> kap(nm * 9, 0.0);
    for (int i = 0; i < N; ++i) {
        const int l = p->full_irr[i] - 1, k = p->full_op[i];
        const double *m = p->op_cart + (size_t)(std::abs(k) - 1) * 9;
        const double sgn = k > 0 ? 1.0 : -1.0;
        const size_t fl = (size_t)(p->irr_full[l] - 1);
        for (int j = 0; j < n; ++j) {
            if (p->omega[(size_t)i * n + j] < omin * 0.5) continue;
            const double om = p->omega[fl * n + j];
            const double *vi = p->vel + (fl * n + j) * 3;
            double u[3], w[3];
            const double g = linewidth[(size_t)l * n + j];
            if (fn) {
                const double *fi = fn + ((size_t)l * n + j) * 3;
                const double pre = om >= kFreqTol ? om / temperature : 1.0;  // main.f90:321-327
                for (int r = 0; r < 3; ++r) {
                    u[r] = sgn * (m[r] * fi[0] + m[r + 3] * fi[1] + m[r + 6] * fi[2]) * pre;
                    w[r] = sgn * (m[r] * vi[0] + m[r + 3] * vi[1] + m[r + 6] * vi[2]);
                }
                const double nb = planck(temperature, om);
                const double f0 = om * (nb + 1.0) * nb / (p->volume * kKbHartree * temperature);
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        kap[(((size_t)i * n + j) * 3 + b) * 3 + a] = f0 * u[a] * w[b] * kKappaAuToSI;
            } else if (g > kFreqTol) {
                for (int r = 0; r < 3; ++r) u[r] = sgn * (m[r] * vi[0] + m[r + 3] * vi[1] + m[r + 6] * vi[2]);
                const double c = harmonic_oscillator_cv(temperature, om) * (1.0 / (2.0 * g)) / p->volume;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        kap[(((size_t)i * n + j) * 3 + b) * 3 + a] = c * u[a] * u[b] * kKappaAuToSI;
            }
        }
    }
    h.dataset("thermal_conductivity", {(uint64_t)N, (uint64_t)n, 3, 3}, kap, "W/mK", "q-vector,mode,xyz,xyz");
    h.attr_double("temperature", temperature);
    h.dataset("harmonic_heat_capacity", {(uint64_t)N, (uint64_t)n}, cv, "J/K", "q-vector,mode");
    return h.write(path);
}
