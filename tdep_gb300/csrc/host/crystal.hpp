// Host-side model of the inputs of thermal_conductivity: crystal structure with its
// symmetry operations, force constants of order 2/3/4, the FFT q-mesh and the harmonic
// phonons. These mirror the libolle types the scattering path consumes.
#pragma once

#include "common.hpp"

namespace tdg {

struct SymOp {
    M3 m;              // Cartesian rotation (op%m)
    int32_t fm[9];     // integer rotation of fractional real-space coordinates
    int32_t rfm[9];    // integer rotation of fractional reciprocal coordinates (op%rfm)
    V3 tr;             // fractional translation
};

struct Crystal {
    int na = 0;
    M3 lat;            // latticevectors (columns), Bohr
    M3 inv_lat;
    M3 reclat;         // reciprocal_latticevectors (columns), a_i.b_j = delta_ij
    M3 inv_reclat;
    double volume = 0;
    std::vector<V3> frac;             // fractional positions
    std::vector<V3> rcart;            // Cartesian positions
    std::vector<int> species;         // 0-based species index
    std::vector<std::string> symbols; // per species
    std::vector<double> mass;         // electron masses
    std::vector<double> invsqrtmass;
    std::vector<double> disorder;     // isotope mass-disorder parameter
    std::vector<SymOp> ops;

    V3 frac_to_cart(const V3 &v) const { return mul(lat, v); }
};

// type_crystalstructure_io.f90:9 (readfromfile). Masses from standard atomic weights.
int read_poscar(const std::string &path, Crystal &c);
// type_crystalstructure_io.f90:921-957 (readisotopefromfile).
int read_isotopes(const std::string &path, Crystal &c);
// Space-group operations of the cell: lattice rotations that map the crystal onto
// itself with some fractional translation. Identity first.
int find_symmetry(Crystal &c);

// Atom maps of the operations (op%fmap, type_symmetryoperation.f90:811-900): operation o
// takes atom a onto atom fmap[o*na + a] (0-based), and shift[o*na + a] is the lattice vector
// op^-1(r(fmap(a)) - tr) - r(a) in Cartesian Bohr, the vector whose phase enters
// lo_eigenvector_transformation_matrix (type_symmetryoperation.f90:243-290).
int op_atom_maps(const Crystal &c, std::vector<int32_t> &fmap, std::vector<double> &shift);

struct FC2Pair {
    int a1, a2;        // 0-based
    V3 lv;             // Cartesian lattice vector, Bohr
    double m[9];       // Hartree/Bohr^2, m(i,j) at i + 3j
};
struct FC2 {
    int na = 0;
    std::vector<FC2Pair> pairs;
    int polar = 0;                 // loto%correctiontype: 0 none, 3 reciprocal-space Ewald sum
    M3 eps;                        // dielectric tensor
    double lambda = 0;             // Ewald coupling parameter
    std::vector<double> Z;         // Born charges Z(i,j,a) at a*9 + i + 3j
    std::vector<double> Zonsite;   // onsite correction, same layout
    std::vector<V3> G;             // reciprocal lattice vectors (1/Bohr, no 2*pi) in the Ewald sphere
};
// type_forceconstant_secondorder_io.f90:136-246. For polar materials (correction type 3,
// the only one the reference accepts) it also reads the dielectric tensor, the Ewald
// parameter and the Born charges, and sets up the long-range term
// (type_forceconstant_secondorder_loto.f90:10-99).
// The decimal real at p (leading blanks skipped; *end after it), correctly rounded as
// strtod: digits and power of ten exact in one FP64 operation (Clinger's fast path: at most
// 2^53 after dropping trailing zeros, 10^-22..10^22), otherwise strtod. False when p holds
// no number.
bool parse_real(const char *p, const char **end, double *x);
int read_fc2(const std::string &path, const Crystal &c, FC2 &fc);

// Long-range dipole-dipole dynamical matrix, reciprocal-space sum only
// (lo_longrange_electrostatics_dynmat.f90:12-360 with reconly): P(i,j,a1,a2) at
// ((a1*na + a2)*9 + i + 3j), Hartree/Bohr^2, no masses; q Cartesian in 1/Bohr without 2*pi.
// With pg != nullptr also its gradient with respect to 2*pi*q, direction-major.
void longrange_dm(const Crystal &c, const FC2 &fc, const V3 &q, bool onsite, cplx *p, cplx *pg);
// Non-analytic term at Gamma along qdir (type_forceconstant_secondorder_loto.f90:130-163),
// same layout as longrange_dm, real.
void nonanalytic_dm(const Crystal &c, const FC2 &fc, const V3 &qdir, double *p);

// Frequencies (Hartree) at arbitrary Cartesian points q (1/Bohr, no 2*pi); at Gamma the
// non-analytic term is taken along qdir[k] unless qdir[k] is zero
// (type_phonon_dispersions.f90:1083-1190). omega is nq*3*na.
int phonon_frequencies(const Crystal &c, const FC2 &fc, int nq, const V3 *q, const V3 *qdir, double *omega);

struct FC3 {
    std::vector<int32_t> atoms;    // n*3, 1-based
    std::vector<int32_t> lv;       // n*6 fractional integer (lv2, lv3)
    std::vector<double> lvcart;    // n*6 Cartesian (lv2, lv3)
    std::vector<double> mwm;       // n*27
    int n() const { return (int)(atoms.size() / 3); }
};
// type_forceconstant_thirdorder.f90:243-311.
int read_fc3(const std::string &path, const Crystal &c, FC3 &fc);

struct FC4 {
    std::vector<int32_t> atoms;    // n*4
    std::vector<int32_t> lv;       // n*9
    std::vector<double> lvcart;    // n*9
    std::vector<double> mwm;       // n*81
    int n() const { return (int)(atoms.size() / 4); }
};
// type_forceconstant_fourthorder.f90:259-330.
int read_fc4(const std::string &path, const Crystal &c, FC4 &fc);

struct QMesh {
    int grid[3] = {0, 0, 0};
    int n_full = 0, n_irr = 0;
    std::vector<V3> q_full;               // Cartesian, folded to the first zone
    std::vector<V3> qfrac;                // fractional (folded)
    std::vector<int32_t> full_irr;        // 1-based
    std::vector<int32_t> full_op;         // signed 1-based
    std::vector<int32_t> irr_full;        // 1-based
    std::vector<double> irr_weight;
    std::vector<int32_t> irr_nop;
    std::vector<int32_t> irr_ops;         // n_irr * n_op, 0-padded, 1-based
};
// type_qpointmesh_gridgeneration.f90:8-545 for the Gamma-centred FFT mesh.
int build_fft_mesh(const Crystal &c, const int grid[3], bool timereversal, QMesh &qp);

struct Phonons {
    int n_mode = 0;
    std::vector<double> omega;    // n_full*n
    std::vector<double> egv;      // n_full*n*n*2
    std::vector<double> vel;      // n_full*n*3
    std::vector<int32_t> degen;   // n_full*n
    std::vector<int32_t> degen_mode; // n_full*n*n
};
// D(q) (type_forceconstant_secondorder_dynamicalmatrix.f90:484-788), Hermitian
// diagonalisation and group velocities at the irreducible points, unfolded onto the mesh
// with the degeneracy tables (unfold_phonons).
int build_phonons(const Crystal &c, const FC2 &fc, const QMesh &qp, Phonons &ph);
// The full mesh from the irreducible points' frequencies, eigenvectors ([q][b][r] complex)
// and velocities (type_phonon_dispersions_generation.f90:117-170): frequencies and
// degeneracy tables copied, velocities rotated (negated under time reversal), eigenvectors
// rotated by lo_eigenvector_transformation_matrix (type_symmetryoperation.f90:243-290) and
// conjugated under time reversal; fmap and shift as op_atom_maps gives them.
int unfold_phonons(const Crystal &c, const QMesh &qp, int nb, const double *om_i, const double *egv_i,
                   const double *vel_i, const std::vector<int32_t> &fmap, const std::vector<double> &shift,
                   Phonons &ph);

// The same on the GPU `device` (k_harmonic.cu): D(q) and dD/dq at the irreducible points, the
// Jacobi eigensolver, the subspace gauge, velocities and degeneracy, the unfold; irr_dyngrad
// receives dD/dq at the irreducible points in the layout of dyn_gradient ([i][x][c][r] complex).
// Allocates and frees its own device memory.
int build_phonons_device(const Crystal &c, const FC2 &fc, const QMesh &qp, int device, Phonons &ph,
                         std::vector<double> &irr_dyngrad);

// Gradient of the mass-weighted dynamical matrix at the Cartesian point q (1/Bohr without
// 2*pi, as QMesh::q_full) (type_forceconstant_secondorder_dynamicalmatrix.f90:484-788,
// non-polar branch), derivative with respect to 2*pi*q: g[(x*nb + c)*nb + r] = dD(r, c)/dq_x.
void dyn_gradient(const Crystal &c, const FC2 &fc, const V3 &qr, int nb, cplx *g);

// Complex Hermitian Jacobi eigensolver: a is n x n column-major, overwritten.
// Eigenvalues unsorted in w, eigenvectors as columns of v.
int hermitian_jacobi(int n, std::vector<cplx> &a, std::vector<double> &w, std::vector<cplx> &v);

}  // namespace tdg
