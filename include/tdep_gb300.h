/*
 * tdep_gb300.h -- C-ABI of the GB300 (sm_103a) three/four-phonon scattering path.
 *
 * The entry points replace the Fortran call sequence of TDEP's thermal_conductivity
 * program around its scattering hot path:
 *
 *   src/thermal_conductivity/main.f90:191      call sr%generate(qp, dr, uc, fct, fcf, opts, ...)
 *   src/thermal_conductivity/scattering.f90:58 subroutine generate            -> tdg_scattering
 *   src/thermal_conductivity/main.f90:219,231  get_kappa / iterative_solution -> tdg_kappa
 *   src/thermal_conductivity/kappa.f90:326     subroutine iterative_solution  -> tdg_kappa
 *
 * Conventions (all arrays are caller-owned host memory; the library copies what it needs
 * and never frees or retains caller pointers):
 *   - indices that TDEP stores 1-based (q-points, operations, modes in degeneracy tables,
 *     atoms) are passed 1-based exactly as stored in the Fortran types;
 *   - 3x3 matrices are column-major (Fortran order);
 *   - complex numbers are interleaved (re, im) doubles;
 *   - units are TDEP's internal atomic units (Hartree, Bohr, electron masses).
 *
 * Every entry returns an int status. The codes reuse src/libolle/konstanter.f90:160-172:
 *   0 ok, 1 bad dimension, 2 linear algebra, 3 unphysical value, 4 symmetry,
 *   5 bad parameter, 6 IO; plus TDG_ERR_DEVICE (8) for a CUDA error or a device-side
 *   check that failed. The message of the last error is returned by tdg_last_error().
 *
 * One context per host thread; calls are synchronous; a context is not re-entrant.
 */
#ifndef TDEP_GB300_H
#define TDEP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TDG_OK 0
#define TDG_ERR_BADDIM 1
#define TDG_ERR_LINALG 2
#define TDG_ERR_PHYSICAL 3
#define TDG_ERR_SYMMETRY 4
#define TDG_ERR_PARAM 5
#define TDG_ERR_IO 6
#define TDG_ERR_DEVICE 8

#define TDG_PREC_FP64 0  /* FP64 everywhere                                          */
#define TDG_PREC_MIXED 1 /* FP32 pretransform/contraction, FP64 weights and sums     */

/*
 * The flattened inputs of lo_scattering_rates%generate (scattering.f90:58): the crystal
 * (uc), the FFT q-mesh (qp), the harmonic phonons on the full mesh (dr%aq, dr%iq) and the
 * third/fourth-order force constants (fct, fcf). A Fortran caller fills it from its
 * derived types; the C++ host stage (tdg_problem_load) fills it from infile.* files.
 */
typedef struct tdg_problem {
    /* crystal: type_crystalstructure */
    int32_t n_atom;            /* uc%na                                                  */
    int32_t n_mode;            /* 3*uc%na                                                */
    double latvec[9];          /* uc%latticevectors, column j = a_j, Bohr                 */
    double reclat[9];          /* uc%reciprocal_latticevectors, a_i.b_j = delta_ij, 1/Bohr */
    double inv_reclat[9];      /* uc%inv_reciprocal_latticevectors                         */
    double volume;             /* uc%volume, Bohr^3                                        */
    const double *mass_disorder; /* [n_atom] uc%isotope(:)%disorderparameter               */
    /* symmetry: uc%sym%op(1:n_op) */
    int32_t n_op;
    const double *op_cart;     /* [n_op*9] op%m, Cartesian rotation, column-major          */
    const int32_t *op_recfrac; /* [n_op*9] op%rfm, integer rotation of fractional
                                  reciprocal coordinates, column-major                     */
    /* FFT mesh: type_qpointmesh (lo_fft_mesh) */
    int32_t grid[3];           /* qp%griddensity                                            */
    int32_t n_full;            /* qp%n_full_point = grid[0]*grid[1]*grid[2]                 */
    int32_t n_irr;             /* qp%n_irr_point                                            */
    const double *q_full;      /* [n_full*3] qp%ap(:)%r, Cartesian, 1/Bohr without 2*pi     */
    const int32_t *full_irr;   /* [n_full] qp%ap(:)%irreducible_index (1-based)             */
    const int32_t *full_op;    /* [n_full] qp%ap(:)%operation_from_irreducible (signed)     */
    const int32_t *irr_full;   /* [n_irr] qp%ip(:)%full_index (1-based)                     */
    const double *irr_weight;  /* [n_irr] qp%ip(:)%integration_weight                       */
    const int32_t *irr_nop;    /* [n_irr] qp%ip(:)%n_invariant_operation                    */
    const int32_t *irr_ops;    /* [n_irr*n_op] qp%ip(:)%invariant_operation, 0-padded       */
    /* harmonic phonons on the full mesh: dr%aq(:) (dr%iq(i) == dr%aq(irr_full(i)))        */
    const double *omega;       /* [n_full*n_mode] omega, Hartree, mode fastest              */
    const double *egv;         /* [n_full*n_mode*n_mode*2] egv(:,b), element r of mode b at
                                  ((q*n_mode + b)*n_mode + r)*2 (+1 for imaginary part)     */
    const double *vel;         /* [n_full*n_mode*3] vel(:,b) at (q*n_mode + b)*3 + xyz      */
    const int32_t *degen;      /* [n_full*n_mode] degeneracy(b)                              */
    const int32_t *degen_mode; /* [n_full*n_mode*n_mode] degenmode(j,b) at
                                  (q*n_mode + b)*n_mode + j, 1-based                         */
    /* third order: type_forceconstant_thirdorder, triplets of all atoms concatenated      */
    int32_t n_fc3;
    const int32_t *fc3_atoms;  /* [n_fc3*3] i1,i2,i3 (1-based)                               */
    const int32_t *fc3_lv;     /* [n_fc3*6] lv2, lv3 in integer fractional coordinates       */
    const double *fc3_lvcart;  /* [n_fc3*6] lv2, lv3 Cartesian, Bohr                         */
    const double *fc3_mwm;     /* [n_fc3*27] mwm(i,j,k) at i + 3j + 9k (0-based, Fortran)    */
    /* fourth order: type_forceconstant_fourthorder                                         */
    int32_t n_fc4;
    const int32_t *fc4_atoms;  /* [n_fc4*4] i1..i4 (1-based)                                 */
    const int32_t *fc4_lv;     /* [n_fc4*9] lv2, lv3, lv4, integer fractional                */
    const double *fc4_lvcart;  /* [n_fc4*9] lv2, lv3, lv4 Cartesian, Bohr                    */
    const double *fc4_mwm;     /* [n_fc4*81] mwm(i,j,k,l) at i + 3j + 9k + 27l               */
    /* off-diagonal (coherence) kappa, get_kappa_offdiag (kappa.f90:77-306); only
       tdg_kappa_offdiag reads these, and they may be NULL when it is not called            */
    const double *irr_dyngrad; /* [n_irr*3*n_mode*n_mode*2] gradient of the mass-weighted
                                  dynamical matrix at the irreducible points
                                  (fc%dynamicalmatrix(..., dynamical_matrix_gradient), d/d(2*pi*q),
                                  Cartesian): element (r, c) of direction x of point i at
                                  (((i*3 + x)*n_mode + c)*n_mode + r)*2 (+1 imaginary part)       */
    const int32_t *op_fmap;    /* [n_op*n_atom] op%fmap: operation o takes atom a onto atom
                                  op_fmap[o*n_atom + a] (1-based)                                */
    const double *atom_shift;  /* [n_op*n_atom*3] lattice vector op^-1(r(fmap(a)) - tr) - r(a),
                                  Cartesian Bohr (the v0 of lo_eigenvector_transformation_matrix,
                                  type_symmetryoperation.f90:243-290)                           */
} tdg_problem;

/* The hot-path subset of lo_opts (src/thermal_conductivity/options.f90). */
typedef struct tdg_opts {
    double temperature;        /* --temperature, K                                          */
    int32_t integrationtype;   /* -it 1 (fixed Gaussian), 2 (adaptive), 6 (velocity diff)   */
    double sigma;              /* --sigma, THz, used with -it 1                              */
    int32_t thirdorder;        /* not --nothirdorder                                          */
    int32_t fourthorder;       /* --fourthorder                                               */
    int32_t isotope;           /* not --noisotope                                             */
    int32_t classical;         /* --classical                                                 */
    double mfp_max;            /* --max_mfp converted to Bohr; <= 0 disables boundary term    */
    int32_t qg3ph[3];          /* -qg3ph after defaulting (options.f90:205-235)               */
    int32_t qg4ph[3];          /* -qg4ph after defaulting                                     */
    int32_t seed;              /* --seed (> 0)                                                */
    int32_t precision;         /* TDG_PREC_FP64 or TDG_PREC_MIXED                             */
    int32_t tensor_cores;      /* no reference counterpart: 0 = automatic (mixed precision:
                                  the tcgen05 fused kernel for 9, 12 and 15 modes, the tcgen05
                                  large-cell contraction for more than 18 modes), 1 = always
                                  the large-cell contraction (mixed precision only), 2 = the
                                  FP32 SIMT fused kernel up to 18 modes                       */
} tdg_opts;

/*
 * Scattering-matrix rows: (q1, b1) over irreducible q1 ascending, modes ascending, skipping
 * omega < lo_freqtol (scattering.f90:170-209 with one rank). Monte-Carlo q' samples are per
 * row in CSR form: row r uses list[ptr[r] .. ptr[r+1]) with weight 1/(ptr[r+1]-ptr[r]).
 * For four-phonon each row has two samples of equal length (list4a, list4b).
 */
typedef struct tdg_qlists {
    int32_t n_row;
    const int32_t *row_q1;     /* [n_row] irreducible index (1-based)                          */
    const int32_t *row_b1;     /* [n_row] mode (1-based)                                       */
    const int64_t *ptr3;       /* [n_row+1] or NULL when third order is off                    */
    const int32_t *list3;      /* q' (1-based full index)                                      */
    const int64_t *ptr4;       /* [n_row+1] or NULL when fourth order is off                   */
    const int32_t *list4a;
    const int32_t *list4b;
} tdg_qlists;

typedef struct tdg_ctx tdg_ctx;

/* Last error message of this thread (static storage, never NULL). */
const char *tdg_last_error(void);

/* Library version string. */
const char *tdg_version(void);

/* Number of CUDA devices visible (0 without a GPU); never fails. */
int tdg_device_count(void);

/* Diagnostic: one 128 x n x 16 tile through the tcgen05 tensor cores with BF16 hi/lo
 * operand splits, d = a b (a 128 x 16 and b 16 x n row-major floats, n a multiple of 16 up
 * to 256); variant 0..3 selects the shared-memory operand layout. No reference counterpart. */
int tdg_check_mma(int32_t variant, int32_t n, const float *a, const float *b, float *d);

/* Diagnostic, no counterpart in the reference: evaluates on the current device the FP64
 * exponential the delta weights use, out[i] = exp(-t[i]) for 0 <= t[i] <= 40 (the range
 * of lo_gauss inside its 8-sigma window), so tests can bound its error. */
int tdg_check_exp(const double *t, int32_t n, double *out);

/* Create a context on CUDA device `device` and upload the problem (replaces the
 * allocations of scattering.f90:85-212). Fails with TDG_ERR_DEVICE without a GPU. */
int tdg_create(tdg_ctx **out, const tdg_problem *prob, int device);

void tdg_destroy(tdg_ctx *ctx);

/*
 * Device memory of the contexts comes from a stream-ordered pool per device that keeps the
 * blocks tdg_destroy frees, so that later contexts reuse them (a caching allocator; no
 * reference counterpart). This returns the cached blocks of `device` to the driver; call it
 * when no context of that device is alive.
 */
int tdg_release_cached_memory(int device);

/* Bytes of that pool in use by live buffers and reserved from the driver (diagnostic, no
 * reference counterpart). */
int tdg_pool_usage(int device, uint64_t *used, uint64_t *reserved);

/* Natural isotope composition of an element (replaces naturaldistribution,
 * src/libolle/type_crystalstructure.f90:1522): returns the number of isotopes and fills
 * abundance[] and mass[] (amu) when cap allows, -count when cap is too small, 0 when the
 * library has no table entry for the symbol (such an atom needs infile.isotopes for
 * isotope scattering). */
int tdg_natural_isotopes(const char *symbol, int32_t cap, double *abundance, double *mass);

/*
 * CUDA graphs (no reference counterpart): the three-phonon kernels of tdg_scattering (the
 * fused kernel, or the launches of the large-cell batches) run directly on the first call
 * with a given configuration, are recorded as a CUDA graph on the
 * second and replayed on later calls with the same configuration and device buffers (the
 * data in the buffers may change). TDG_GRAPHS=0 runs it directly every time. counts[0..2]
 * receive the context's direct runs, recordings and replays of that part.
 */
int tdg_graph_counts(tdg_ctx *ctx, int64_t *counts);

/* Which three-phonon path the context's last tdg_scattering took (no reference
 * counterpart): 0 the SIMT fused kernel (FP64, or FP32 contraction), 1 the tcgen05 fused
 * kernel (9, 12 or 15 modes, mixed precision), 2 the large-cell batches (tcgen05), -1 none
 * yet. The environment variable TDG_TC_SMALL=0 turns path 1 off. */
int tdg_last_path(tdg_ctx *ctx, int32_t *path);

/* Launch shape of the fused three-phonon kernel in the context's last tdg_scattering (no
 * reference counterpart): shape[0] the grid (CTAs), shape[1] the CTAs per SM it was sized
 * for, shape[2] the CUDA runtime's occupancy figure for one SM, shape[3] the count from the
 * kernel's registers and shared memory; all -1 before the first call and on the large-cell
 * path. */
int tdg_last_launch(tdg_ctx *ctx, int32_t *shape);

/*
 * Launch-shape autotuner (no reference counterpart). The first scattering call that needs a
 * launch shape for its mode count, precision and device (the persistent grid of the fused
 * three-phonon kernel; the delta kernel's row block and the GEMM pipeline depth of the
 * large-cell path) times each candidate on its own work and keeps the fastest in a
 * process-wide table; results do not depend on the choice beyond floating-point summation
 * order. Environment: TDG_AUTOTUNE=0 turns the trials off (defaults, or decisions already
 * in the table); TDG_TUNE_CACHE=<file> is read before the first decision and rewritten
 * after each new one.
 *   tdg_autotune_load   adds the "key value" lines of a file to the table (TDG_ERR_IO if
 *                       it cannot be read or a line is malformed);
 *   tdg_autotune_save   writes the table to a file;
 *   tdg_autotune_report writes the table as text ("key value\n" lines, NUL-terminated,
 *                       truncated to cap bytes); *needed (if not NULL) gets the full size;
 *   tdg_autotune_clear  empties the table.
 */
int tdg_autotune_load(const char *path);
int tdg_autotune_save(const char *path);
int tdg_autotune_report(char *buf, int64_t cap, int64_t *needed);
int tdg_autotune_clear(void);

/*
 * Rows and Monte-Carlo q' samples, generated on the host exactly as the reference does:
 * MT19937-64 seeded by init_genrand64(iseed=0, rseed=1/seed) (lo_randomnumbers.f90:203-236),
 * one stratified sample per row and order (lo_fftgrid_helper.f90:56-99), consumed row by
 * row in the order isotope, three-phonon, four-phonon (scattering.f90:227-243).
 * Writes n_row and the rows into the caller's arrays (capacity n_irr*n_mode) and the
 * samples into list3 (capacity n_row*prod(qg3ph)) / list4a, list4b (n_row*prod(qg4ph)).
 * Any list pointer may be NULL when that order is off. CPU only.
 */
int tdg_mc_qlists(const tdg_problem *prob, const tdg_opts *opts, int32_t *n_row,
                  int32_t *row_q1, int32_t *row_b1, int64_t *ptr3, int32_t *list3,
                  int64_t *ptr4, int32_t *list4a, int32_t *list4b);

/*
 * The scattering rates (scattering.f90:58-358): isotope, three-phonon, four-phonon and
 * boundary linewidths for every row, degeneracy averaging, and the symmetrised
 * scattering matrix Xi, which stays in device memory for tdg_kappa.
 * Outputs (n_irr*n_mode, mode fastest, zero for skipped modes):
 *   linewidth  dr%iq(:)%linewidth (Hartree)
 *   qs         dr%iq(:)%qs = 2*linewidth
 * stats (may be NULL, 10 doubles): [0] accepted irreducible q-triplets, [1] q-quartets,
 *   [2] device time of the pipeline in ms (inputs resident), [3] candidates (q-pairs for
 *   three-phonon plus q-triples for four-phonon), [4] enumeration ms, [5] fused three- and
 *   four-phonon kernel ms, [6] symmetrisation ms, [7] isotope ms, [8] kernel launches,
 *   [9] equivalent-triplet and -quartet entries.
 * Four-phonon scattering supports up to 5 atoms (15 modes) in the primitive cell,
 * three-phonon up to 6 atoms.
 */
int tdg_scattering(tdg_ctx *ctx, const tdg_opts *opts, const tdg_qlists *lists,
                   double *linewidth, double *qs, double *stats);

/* Copy the device-resident scattering matrix (n_row x n_full*n_mode, row-major, FP64). */
int tdg_get_xi(tdg_ctx *ctx, double *xi);

/*
 * Bytes copied host-to-device (*h2d) and device-to-host (*d2h) by all calls on this context
 * since tdg_create, that call included. Instrumentation with no reference counterpart: the
 * reference keeps everything in host memory.
 */
int tdg_transfer_bytes(tdg_ctx *ctx, int64_t *h2d, int64_t *d2h);

/*
 * Irreducible q-triplets of one sample, enumerated on the device (kernel K1). Replaces the
 * per-candidate q3 index and triplet_is_irreducible of scattering_threephonon.f90:72-77,
 * 319-448. q1 is the irreducible index (1-based) and sample holds full-mesh indices
 * (1-based). For every accepted q2, in sample order, writes q2, q3, k and the k
 * equivalent pairs (q2', q3') in operation order (all 1-based) into out. *written
 * receives the number of ints; TDG_ERR_PARAM when cap is too small.
 */
int tdg_triplets(tdg_ctx *ctx, int32_t q1, const int32_t *sample, int64_t n, int32_t *out, int64_t cap,
                 int64_t *written);

/*
 * tdg_triplets without device allocation: same arguments and same output, bit for bit.
 * This entry point has no counterpart in the reference; it exists for callers that
 * cannot call cudaMalloc at the time of the call. Its device scratch is one fixed
 * file-scope array (about 4.3 MiB per device) instead of per-call allocations, so it
 * calls no cudaMalloc, cudaFree or other allocating routine.
 * Limits: n <= 32768 q-points, and at most 131072 equivalent triplets in the result.
 * A sample without repeated q-points meets the second limit on every mesh of up to 131072
 * points: the equivalent triplets of distinct irreducible triplets are distinct pairs
 * (q2', q3'), and q3' follows from q2'. Repeated q-points (Monte Carlo samples may repeat
 * one) add their images once per repeat, so in general the count is bounded only by n times
 * the largest image count. Beyond either limit: TDG_ERR_PARAM with a message naming the
 * limit, before any device work on the result.
 * The first call on each device looks the array up (cudaGetSymbolAddress, which loads the
 * module); make that first call before any stream capture. Only the status word of the
 * scratch must start at zero, and each call clears it itself. All calls on one device
 * share the array: calls that overlap in time (several threads or contexts on the same
 * device) race, so the caller serialises them.
 */
int tdg_triplets_static(tdg_ctx *ctx, int32_t q1, const int32_t *sample, int64_t n, int32_t *out, int64_t cap,
                        int64_t *written);

/*
 * Symmetry-irreducible parameters of the third-order force constants, Phi3 = B x (the
 * construction of the reference's forcemap, type_forcemap_returntensors.f90:250-362: orbits
 * of the triplets under the space group and the site permutations, the components a
 * representative's stabiliser leaves free, and the operation that maps the representative
 * onto each member). B acts on the mass-weighted constants fc3_mwm; each orbit's columns are
 * orthonormal on its representative. Call with t_col0, t_ncol, coef and x all NULL to get
 * n_x (parameters) and n_coef (doubles of coef); then: t_col0[t], t_ncol[t] give the columns
 * of triplet t, coef holds for every triplet (in order) a 27 x t_ncol[t] block, row c =
 * component i + 3j + 9k, and x the parameters of the problem's own constants (B^T on the
 * representatives). TDG_ERR_SYMMETRY when the triplet list is not closed under the group.
 * The problem must carry op_fmap and atom_shift (tdg_problem_load fills them).
 */
int tdg_fc3_irreducible(const tdg_problem *prob, int32_t *n_x, int64_t *n_coef, int32_t *t_col0, int32_t *t_ncol,
                        double *coef, double *x);

/*
 * Differentiation with respect to the third-order force constants. None of the three entry
 * points below has a counterpart in the reference; they serve d(kappa)/d(Phi3) and
 * d(Gamma)/d(Phi3).
 *
 * tdg_set_fc3: replace the mass-weighted third-order force constants of a context,
 * fc3_mwm[n_fc3*27] in the layout of tdg_problem.fc3_mwm (same triplets as at
 * tdg_create). The scattering state is invalidated (call tdg_scattering again).
 */
int tdg_set_fc3(tdg_ctx *ctx, const double *fc3_mwm);

/*
 * tdg_kappa_sma_vjp: lw_bar[n_irr*n_mode] = (d kappa_sma / d linewidth)^T kappa_bar for the
 * kappa_sma of tdg_kappa (get_kappa then symmetrize_kappa; lo_chop is taken as the
 * identity), at the linewidths of the last tdg_scattering. kappa_bar is 3x3 column-major.
 */
int tdg_kappa_sma_vjp(tdg_ctx *ctx, const tdg_opts *opts, const double *kappa_bar, double *lw_bar);

/*
 * tdg_adjoint_fc3: mwm_bar[n_fc3*27] = (d linewidth / d fc3_mwm)^T lw_bar, the vector-Jacobian
 * product of the three-phonon part of the linewidths (the only part that depends on Phi3)
 * over the rows, samples and q-triplets of the last tdg_scattering, which must have run with
 * the same opts (opts->precision may differ). Psi is recomputed per q-triplet instead of
 * stored. After a large-cell pass (the tensor-core contraction: more than 18 modes, or
 * forced with opts->tensor_cores) the adjoint runs per batch on the same path, with the
 * back-contraction on the tensor cores and the gradient accumulated in double-float.
 * Layout of mwm_bar as tdg_problem.fc3_mwm; divide by sqrt(m_i m_j m_k) for the derivative
 * with respect to the unweighted force constants. stats (may be NULL, 4 doubles): [0] ms of
 * the whole pass, [1] ms of the adjoint kernels, [2] q-triplets, [3] CTAs of the shared-
 * memory kernel or batches of the large-cell path.
 */
int tdg_adjoint_fc3(tdg_ctx *ctx, const tdg_opts *opts, const double *lw_bar, double *mwm_bar, double *stats);

/*
 * Vector-Jacobian product of kappa_iter (iterative_solution + symmetrize_kappa,
 * kappa.f90:326-495) for the cotangent kappa_bar (3x3 column-major), no reference
 * counterpart. At the converged solution of the last tdg_kappa call (maxiter > 0) it solves
 * the transposed fixed point lambda = kbar - T^T Xi^T Q^-1 D lambda on the device (maxiter
 * and tol as for tdg_kappa, the same mixing schedule; *n_iter receives the iterations),
 * writes the cotangent of the linewidths to lw_bar [n_irr*n_mode] (through qs = 2 linewidth
 * and F0 = v / qs) and keeps on the device the cotangent of the three-phonon terms of Xi,
 * mapped back through the row symmetrisations. The next tdg_adjoint_fc3 adds that term, so
 * tdg_adjoint_fc3(lw_bar) then returns d(kappa_bar : kappa_iter) / d fc3_mwm. The stored term
 * lasts until the next tdg_scattering, tdg_kappa or tdg_set_fc3. Shared-memory kernel path
 * only (up to 18 modes); the active entries of the reference's od_terms > 0 averaging are
 * taken from a fresh forward pass of the raw three-phonon terms.
 */
int tdg_kappa_iter_vjp(tdg_ctx *ctx, const tdg_opts *opts, const double *kappa_bar, int32_t maxiter, double tol,
                       double *lw_bar, int32_t *n_iter);

/*
 * Thermal conductivity from the current scattering state (main.f90:216-244):
 * kappa_sma (get_kappa, kappa.f90:28-75), the iterative BTE (kappa.f90:326-495) with
 * maxiter steps and tolerance tol, kappa_iter, both symmetrised (kappa.f90:308-324).
 * All tensors 3x3 column-major in atomic units (multiply by lo_kappa_au_to_SI for W/m/K).
 * fn_out (may be NULL): final Fn, [n_irr*n_mode*3]. n_iter receives the iteration count.
 */
int tdg_kappa(tdg_ctx *ctx, const tdg_opts *opts, int32_t maxiter, double tol,
              double *kappa_sma, double *kappa_iter, double *fn_out, int32_t *n_iter);

/*
 * Off-diagonal (coherence) thermal conductivity, get_kappa_offdiag (kappa.f90:77-306)
 * followed by symmetrize_kappa (main.f90:243), from the linewidths of the last
 * tdg_scattering: per irreducible point the off-diagonal group velocities
 * Re <e_i|dD/dq|e_j> / (2 sqrt(w_i w_j)) averaged over the little group with the eigenvector
 * transformation matrices, rotated over the star, and summed with the Lorentzian
 * (G_i + G_j) / ((G_i + G_j)^2 + (w_i - w_j)^2). Needs irr_dyngrad, op_fmap and atom_shift
 * in the problem given to tdg_create. kappa_offdiag: 3x3 column-major, atomic units.
 * The reference keeps only the real part of each velocity matrix element, which depends on
 * the phases of the eigenvectors: the result is that formula on the problem's eigenvectors.
 */
int tdg_kappa_offdiag(tdg_ctx *ctx, const tdg_opts *opts, double *kappa_offdiag);

/*
 * Host stage of thermal_conductivity (main.f90:42-181) for the C++ driver and tests:
 * reads infile.ucposcar, infile.forceconstant, infile.forceconstant_thirdorder and, when
 * fourthorder != 0, infile.forceconstant_fourthorder from `dir` (masses from infile.isotopes
 * when readiso != 0), finds the symmetry operations, builds the FFT mesh `grid` and the
 * harmonic phonons: the irreducible points are diagonalised and the rest of the mesh takes
 * their rotated eigenvectors (type_phonon_dispersions_generation.f90:72-170). The returned
 * problem owns its arrays; free with tdg_problem_free.
 */
int tdg_problem_load(const char *dir, const int32_t grid[3], int fourthorder, int readiso,
                     int timereversal, tdg_problem **out);
/*
 * The same with the harmonic stage on GPU `device` (no reference counterpart; it replaces the
 * host work of tdg_problem_load inside main.f90:42-181): D(q) and dD/dq at the irreducible
 * points with the polar Ewald sum, a batched Jacobi eigensolver, the degenerate-subspace
 * gauge, velocities and degeneracy tables, and the unfold onto the mesh, in FP64; at most 128
 * modes. The readers, the symmetry search and the mesh stay on the host. Results equal
 * tdg_problem_load's to rounding. Allocates and frees its own device memory.
 */
int tdg_problem_load_device(const char *dir, const int32_t grid[3], int fourthorder, int readiso,
                            int timereversal, int32_t device, tdg_problem **out);
void tdg_problem_free(tdg_problem *prob);

/*
 * Harmonic frequencies (Hartree, ascending) at nq Cartesian points q[3*k..] (1/Bohr,
 * without 2*pi) from infile.ucposcar and infile.forceconstant in `dir`, polar
 * force constants included: the per-point stage of phonon_dispersion_relations
 * (lo_phonon_bandstructure_on_path.f90:203-217 -> type_phonon_dispersions.f90:1083-1190).
 * At Gamma the non-analytic term is taken along qdir[3*k..] (NULL: [1,0,0] for every
 * point; a zero direction leaves it out). omega holds nq*3*na values. Host only.
 */
int tdg_phonon_frequencies(const char *dir, int32_t nq, const double *q, const double *qdir,
                           double *omega);

/*
 * outfile.thermal_conductivity_grid.hdf5 (type_phonon_dispersions.f90:316-641, written by
 * main.f90:339): the per-mode data of the full mesh in HDF5, without libhdf5 (the library
 * writes the file format itself). linewidth [n_irr*n_mode] as tdg_scattering returns it
 * (Hartree); fn [n_irr*n_mode*3] the final Fn of tdg_kappa, or NULL for the relaxation-time
 * form of the per-mode conductivity. The dataset thermal_conductivity summed over points and
 * modes and divided by number_of_qpoints is kappa_iter (W/m/K), as the reference's own test
 * checks (tests/thermal_conductivity/test_thermal_conductivity.py:24-40).
 */
int tdg_write_grid_hdf5(const char *path, const tdg_problem *prob, double temperature, const double *linewidth,
                        const double *fn);

/* Writes outfile.thermal_conductivity (main.f90:246-294) into `dir`. Tensors in a.u. */
int tdg_write_outfile(const char *dir, double temperature, const double *kappa_sma,
                      const double *kappa_iter, const double *kappa_offdiag);

#ifdef __cplusplus
}
#endif

#endif /* TDEP_GB300_H */
