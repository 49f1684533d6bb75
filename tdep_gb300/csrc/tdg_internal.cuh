// Internal device-side declarations shared by the kernels and the C-ABI layer.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <string>
#include <vector>

struct tdg_ctx;

namespace tdg {

// Host<->device byte counter of the context whose entry point runs on this thread
// ([0] host to device, [1] device to host); XferScope sets it for the span of a call.
extern thread_local int64_t *tl_xfer;

struct XferScope {
    int64_t *prev;
    explicit XferScope(int64_t *counter) : prev(tl_xfer) { tl_xfer = counter; }
    ~XferScope() { tl_xfer = prev; }
};

// cudaMemcpyAsync that adds host<->device bytes to the active counter.
inline cudaError_t copy_async(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
    if (tl_xfer) {
        if (kind == cudaMemcpyHostToDevice) tl_xfer[0] += (int64_t)bytes;
        if (kind == cudaMemcpyDeviceToHost) tl_xfer[1] += (int64_t)bytes;
    }
    return cudaMemcpyAsync(dst, src, bytes, kind, s);
}


// Work item of the three-phonon kernel: one accepted irreducible q-triplet.
struct TripletRec {
    int32_t q1;       // irreducible index of q1 (0-based)
    int32_t q2, q3;   // full-mesh indices (0-based)
    int32_t cand;     // index of its row mask (bit b1 set when row (q1,b1) samples q2)
    int32_t red_off;  // first equivalent triplet in the red list
    int32_t red_cnt;  // number of equivalent triplets (size(red_triplet,2))
};

// Work item of the four-phonon kernel: one accepted irreducible q-quartet.
struct QuartetRec {
    int32_t q1, q2, q3, q4;
    int32_t cand;
    int32_t red_off, red_cnt;
    int32_t pad;
};

// Mesh description shared by the kernels.
struct MeshDev {
    int32_t n_full, n_irr, n_op, n_mode;
    int32_t grid[3];
    int32_t L;          // lcm of the grid dimensions
    int32_t lmul[3];    // L / grid[d]
    const int32_t *rot;      // [n_op * n_full] image of each point, -1 when off grid
    const int32_t *irr_full; // [n_irr] 0-based
    const int32_t *full_irr; // [n_full] 0-based
    const int32_t *irr_nop;  // [n_irr]
    const int32_t *irr_ops;  // [n_irr * n_op] 0-based operation indices
};

// Phonon/occupation data on the device.
struct PhononDev {
    const double *omega;     // [n_full*n]
    const double2 *egv;      // [n_full*n*n], (q, b, r)
    const double2 *egvs;     // egv / sqrt(omega), 0 where omega < lo_freqtol
    const float2 *egvs32;    // same in FP32 (mixed precision)
    const double *vel;       // [n_full*n*3]
    const double *be;        // [n_irr*n]
    const double *sigsq;     // [n_irr*n]
    double reclat_g[9];      // sr%reclat: reciprocal lattice / grid, column-major
    double sigma_fixed;      // integrationtype 1, Hartree
    double thresh_sigma;     // integrationtype 6
    int32_t integrationtype;
    const double *exp2tab;   // [64] 2^(-j/64), the table of exp_neg
    const double *inv_omega; // [n_full*n] 1/omega, 0 where omega <= 0
    const float *omega32;    // [n_full*n] omega in FP32 (screens)
    const float *sigsq32;    // [n_irr*n] sigsq in FP32 (screens)
};

// exp(-t), 0 <= t <= 40, on the device (diagnostic for tests): out[i] = exp_neg(t[i]).
cudaError_t launch_exp_neg_check(const double *t, int32_t n, double *out, const double *tab, cudaStream_t s);

// Rows of the scattering matrix.
struct RowsDev {
    int32_t n_row;
    const int32_t *rowidx;    // [n_irr*n] row of (q1,b1), -1 when absent
    const double *weight3;    // [n_row] 1/len of the row's three-phonon sample
    const double *weight4;    // [n_row] 1/len of the row's four-phonon sample
    const double *w3q;        // [n_irr*n] weight3 of the row of (q1,b1), 0 when absent
};

struct Fc3Dev {
    int32_t n;                // number of force-constant triplets
    int32_t n_atom;
    const int32_t *blk_ptr;   // [n_atom^3 + 1] triplets sorted by atom block (a1,a2,a3)
    const int32_t *lv;        // [n*6] integer lattice vectors lv2, lv3
    const double *mwm;        // [n*27]
    const float *mwm32;       // [n*27]
    const double2 *twiddle;   // [L] exp(-2 pi i K / L)
    const float2 *twiddle32;
    const int32_t *abase;     // [n] ((3 a1) n + 3 a2) n + 3 a3: element (0,0,0) of the triplet's
                              // atom block in the n^3 pretransformed tensor
};

struct Fc4Dev {
    int32_t n;
    int32_t n_atom;
    const int32_t *blk_ptr;   // [n_atom^4 + 1]
    const int32_t *lv;        // [n*9]
    const double *mwm;        // [n*81]
    const float *mwm32;
};

// Device status word: kernels record the first failed check here.
enum DevStatus : int32_t { kDevOk = 0, kDevBadIndex = 1, kDevOverflow = 2, kDevTimeout = 3, kDevLinalg = 4 };

// ---- launch wrappers (each returns cudaError_t of the launch) ----
// K1: count/fill passes of the irreducible-triplet enumeration.
cudaError_t launch_triplet_count(const MeshDev &m, const int4 *cand, int32_t n_cand, int32_t *n_trip,
                                 int32_t *n_red, int32_t *status, cudaStream_t s);
cudaError_t launch_triplet_fill(const MeshDev &m, const int4 *cand, int32_t n_cand, const int32_t *trip_off,
                                const int32_t *red_off, TripletRec *trip, int2 *red, cudaStream_t s);
cudaError_t launch_quartet_count(const MeshDev &m, const int4 *cand, int32_t n_cand, int32_t *n_quart,
                                 int32_t *n_red, int32_t *status, cudaStream_t s);
cudaError_t launch_quartet_fill(const MeshDev &m, const int4 *cand, int32_t n_cand, const int32_t *q_off,
                                const int32_t *red_off, QuartetRec *quart, int4 *red, cudaStream_t s);
// Exclusive scan of int32 (n <= 2^31), result in out; total in out[n].
cudaError_t exclusive_scan_i32(const int32_t *in, int32_t *out, int32_t n, int32_t *tmp, cudaStream_t s);
size_t exclusive_scan_tmp_elems(int32_t n);

// K2+K3+K4: fused pretransform, contraction and delta/Bose accumulation.
struct ThreePhArgs {
    MeshDev mesh;
    PhononDev ph;
    RowsDev rows;
    Fc3Dev fc;
    const TripletRec *trip;
    int32_t n_trip;
    const int2 *red;
    const uint32_t *cand_mask;  // [n_mask*4] distinct row masks, indexed by TripletRec::cand
    double *gamma;              // [n_row]
    double *od;                 // [n_row * n_full*n]
    int32_t *status;
    // adjoint only: cotangent of each row's Gamma and one accumulation slice of
    // d L / d mwm ([fc.n * 27]) per CTA
    const double *lam;
    double *mwm_bar;            // FP64 slices, zeroed before the launch
    int32_t acc_in_smem;        // accumulate the CTA's slice in shared memory, store it once
    const double *xi_bar;       // adjoint only, may be null: cotangent of the raw three-phonon
                                // row terms of Xi ([n_row * n_full*n], tdg_kappa_iter_vjp)
    // pretransform plan of the fused kernel launched (pretransform_plan; FP32 force constants):
    // plan_slots x (its threads) values, 4 force constants per slot, and words; plan_slots 0:
    // none (the SIMT kernel then walks the blocks; the tensor-core kernel requires the plan)
    const float4 *plan_pm;
    const uint32_t *plan_word;
    int32_t plan_slots;
    // tensor-core kernel only (k_threephonon_tc): real-split eigenvector images of every mesh
    // point (4 KB each)
    const unsigned char *tc_eimg;
    // tensor-core adjoint only: the images of the transposed eigenvector matrices (E^T)
    const unsigned char *tc_eimg_t;
};
// ctas_per_sm: persistent grid of n_sm * ctas_per_sm CTAs (0 or more than fit: as many as fit).
cudaError_t launch_threephonon(const ThreePhArgs &a, int precision, int n_sm, int ctas_per_sm, cudaStream_t s);
// CTAs of the fused kernel per SM (resident_ctas; 0 if the configuration is not supported);
// api and count (may be null) receive resident_ctas's two figures.
int threephonon_max_per_sm(int n, int precision, int *api = nullptr, int *count = nullptr);
// Adjoint of the three-phonon Gamma with respect to mwm: recomputes Psi per q-triplet and
// accumulates 2 Re(phase * Q) into a.mwm_bar (one slice per CTA of the returned grid).
int threephonon_adjoint_grid(int n, int precision, int n_sm, int n_trip, int n_fc, bool acc_in_smem);
cudaError_t launch_threephonon_adjoint(const ThreePhArgs &a, int precision, int grid, cudaStream_t s);
// out[e] = sum over g < n_slice of slices[g * n + e] in FP64, in slice order; the slices hold
// doubles for precision 0 (FP64) and floats otherwise (the mixed adjoint).
cudaError_t launch_sum_slices(const double *slices, int32_t n_slice, int64_t n, int precision, double *out,
                              cudaStream_t s);
size_t threephonon_smem_bytes(int n, int precision, int n_fc);
// Tensor-core fused kernel for 9, 12 or 15 modes in mixed precision (k_threephonon_tc.cu).
bool threephonon_tc_supported(int n, int precision, int n_fc);
// CTAs per SM of the tensor-core kernel (resident_ctas, at most 8 for the tensor memory);
// api and count (may be null) receive resident_ctas's two figures.
int threephonon_tc_max_per_sm(int n, int n_fc, int *api = nullptr, int *count = nullptr);
cudaError_t launch_threephonon_tc(const ThreePhArgs &a, int n_sm, int ctas_per_sm, cudaStream_t s);
// Its adjoint (the ADJ variant of k_threephonon_tc: Psi again, W = G conj(Psi), the back-
// contraction through E3^T, E2^T, E1^T on the tensor cores, 2 Re(phase Q) into a.mwm_bar as
// float slices, one per CTA of the returned grid; a.acc_in_smem is not used).
int threephonon_tc_adjoint_grid(int n, int n_sm, int n_trip, int n_fc);
cudaError_t launch_threephonon_tc_adjoint(const ThreePhArgs &a, int grid, cudaStream_t s);
// Pretransform plan of a fused kernel for n modes and the force-constant blocks blk_ptr
// (n_blk + 1 offsets, host memory): the elements (atom triple, ijk) dealt out to the threads
// of a CTA, slot-major ([slot][thread]); word = first phase-factor index | (code + 1) << 16
// on an element's last slot, code = the tensor-core operand's byte offset / 2 (tc_operand)
// or the index of P(a, b, c) in the SIMT kernel's n^3 array; src = first triplet | ijk << 16
// | valid triplets << 21. Returns the slot count (a multiple of 8), 0 if the set does not fit.
int pretransform_plan(int n, int n_blk, const int32_t *blk_ptr, int threads, bool tc_operand,
                      std::vector<uint32_t> &word, std::vector<uint32_t> &src);
// The plan's values from the FP32 force constants ([n_fc * 27]), slots x threads float4.
cudaError_t launch_fill_plan(const uint32_t *src, int slots, int threads, const float *mwm32, float4 *pm,
                             cudaStream_t s);
// Threads per CTA of the fused SIMT kernel for n modes, and whether its FP32 passes can take
// a pretransform plan for n_fc force-constant triplets (all phase factors at once).
int threephonon_threads(int n);
bool threephonon_plan_fits(int n, int n_fc);
// Real-split eigenvector images (n <= 16).
// transpose: the image of E^T (rows modes, columns components) for the adjoint.
cudaError_t launch_tc_eimg(int32_t n_full, int32_t n, const float2 *egvs32, unsigned char *out, cudaStream_t s,
                           bool transpose = false);
// Adjoint of the BTE (k_bte_adjoint.cu): y = X^T z (FP64, 3 right-hand sides, part holds
// xit_parts(n_row) * 3 * n_col doubles), out = X f row by row, W = -z f^T, and the adjoint
// of the row symmetrisations on W given the raw three-phonon terms od_raw.
int xit_parts(int32_t n_row);
cudaError_t launch_xit_gemv(const double *xi, int32_t n_row, int64_t n_col, const double *z, double *part, double *y,
                            cudaStream_t s);
cudaError_t launch_xi_rowdot(const double *xi, int32_t n_row, int64_t n_col, const double *f, double *out,
                             cudaStream_t s);
cudaError_t launch_xibar_fill(int32_t n_row, int64_t n_col, const double *z, const double *f, double *w,
                              cudaStream_t s);

struct FourPhArgs {
    MeshDev mesh;
    PhononDev ph;
    RowsDev rows;
    Fc4Dev fc;
    const double2 *twiddle;
    const float2 *twiddle32;
    const QuartetRec *quart;
    int32_t n_quart;
    const int4 *red;
    const uint32_t *cand_mask;
    double *gamma;
    double *od;
    int32_t *status;
    void *scratch;              // fourphonon_scratch_bytes(): one n^4 slice per CTA
};
// Grid of the four-phonon kernel and the device scratch it needs (bytes); 0 when the mode
// count is not supported.
int fourphonon_grid(int n, int precision, int n_sm, int n_quart);
size_t fourphonon_scratch_bytes(int n, int precision, int grid);
cudaError_t launch_fourphonon(const FourPhArgs &a, int precision, int grid, cudaStream_t s);

// Large-cell three-phonon path (tcgen05 contraction), one batch of q-triplets.
struct LnBatch {
    MeshDev mesh;
    PhononDev ph;
    RowsDev rows;
    Fc3Dev fc;
    const TripletRec *trip;  // first q-triplet of the batch
    int nb;                  // q-triplets (slots) in the batch
    const int2 *red;
    const uint32_t *cand_mask;
    int n;
    int64_t plane;           // elements of one operand plane per slot: ln_kp(n) * mp
    int mp;                  // ln_mp(n): M tiles of 128 rows (8 x by 16 y) times 128
    int n_sm = 0;            // SMs of the device (persistent GEMM grid)
    int delta_bb = 32;       // rows b2 per block of the delta kernel (16 or 32)
    int gemm_stages = 0;     // shared-memory pipeline stages of the GEMM (0: the most that fit, at most 4)
    __nv_bfloat16 *xa_hi, *xa_lo, *xb_hi, *xb_lo;  // operand planes (hi/lo), zero-initialised
    const __nv_bfloat16 *bmat;                     // launch_ln_bmat
    float2 *phase;           // [nb * fc.n]
    float2 *psi;             // [nb * n^3]
    double *gamma, *od;
    int32_t *status;
    // adjoint (launch_ln_adjoint_batch): transposed matrices, row cotangents and the
    // double-float gradient accumulator [n_fc * 27] in block-sorted order
    const __nv_bfloat16 *bmat_t = nullptr;
    const double *lam = nullptr;
    float *grad_hi = nullptr, *grad_lo = nullptr;
};
int ln_kp(int n);
int ln_mp(int n);
size_t ln_gemm_smem(int kp);
// Real-split eigenvector matrices of every mesh point: n_q * 2 * ln_kp(n)^2 BF16 (hi, lo);
// transposed for the adjoint's back-contraction.
cudaError_t launch_ln_bmat(int n, int n_q, const float2 *egvs32, __nv_bfloat16 *bmat, bool transpose,
                           cudaStream_t s);
cudaError_t launch_ln_batch(const LnBatch &b, cudaStream_t s);
// Adjoint of one batch: forward contraction, W = G conj(Psi), back-contraction with E^T into Q,
// gradient of the mass-weighted force constants added into grad_hi/grad_lo.
cudaError_t launch_ln_adjoint_batch(const LnBatch &b, cudaStream_t s);

// Isotope scattering (scattering_isotope.f90): adds into gamma and xi.
cudaError_t launch_isotope(const MeshDev &m, const PhononDev &ph, const RowsDev &rows, const int32_t *row_q1,
                           const int32_t *row_b1, const double *disorder, int32_t n_atom, double *gamma,
                           double *xi, cudaStream_t s);

// Context tables built on the device: the rotation table rot[op][q] (integer rotation of
// fractional reciprocal coordinates on the mesh, -1 off the mesh) and the eigenvectors
// scaled by 1/sqrt(omega) in FP64 and FP32.
cudaError_t launch_rot_table(const int32_t grid[3], int L, int n_full, int n_op, const int32_t *op_recfrac,
                             int32_t *rot, cudaStream_t s);
cudaError_t launch_egv_scaled(int64_t nm, int n, const double2 *egv, const double *omega, double2 *egvs,
                              float2 *egvs32, cudaStream_t s);

// Orbits of the little group of every irreducible q1 on the mesh (built once per context).
struct OrbitDev {
    const int32_t *rep_ptr;  // [n_irr+1] first representative of q1
    const int32_t *rep;      // [n_rep] representative q2 (smallest member of its orbit)
    const int32_t *img;      // [n_rep * n_op] distinct on-grid images, first appearance order
    const int32_t *mult;     // [n_rep * n_op] number of operations giving each image
    const int32_t *nuniq;    // [n_rep] number of distinct images
    const int32_t *cnt;      // [n_rep] number of on-grid operations (sum of mult)
    const int32_t *orb_of;   // [n_irr * n_full] representative index of q2, -1 otherwise
    const double *rcp;       // [n_op+1] 1/i, replaces the FP64 divisions by counts
    int32_t max_rep;         // largest number of representatives of one q1
    int32_t tile_pts;        // sym_tile_points(n_mode)
    int32_t max_tiles;       // largest sym_tile_count over the q1
};
cudaError_t launch_orbit_flag(const MeshDev &m, int32_t *flag, cudaStream_t s);
cudaError_t launch_orbit_fill(const MeshDev &m, const int32_t *flag, const int32_t *scan, OrbitDev &o,
                              cudaStream_t s);
// K5a: symmetrize_and_distribute of one order in place on od, then xi += od when xi is
// not null (scattering_threephonon.f90:143-205).
// Row r's sample is list[rbeg[r] .. rbeg[r] + rlen[r]).
cudaError_t launch_sym_distribute(const MeshDev &m, const OrbitDev &o, int32_t n_row, const int32_t *row_q1,
                                  const int64_t *rbeg, const int32_t *rlen, const int32_t *list, double *od, double *xi,
                                  cudaStream_t s);
// Candidates of q1 when all its rows share one sample: desc[q1] = (start in list, length,
// first candidate, mask id); cand[desc.z + i] = (q1, list[desc.x + i] - 1, desc.w, 0).
cudaError_t launch_build_candidates(const int4 *desc, int32_t n_irr, int32_t max_len, const int32_t *list, int4 *cand,
                                    cudaStream_t s);
// K5b: symmetrize_and_distribute of the three-phonon terms in place on xi (dist, orbits
// whose representative the row sampled per sbits, launch_sample_bits) and/or
// symmetrize_scatmat (scat, scattering.f90:296-357), on tiles of whole orbits.
int sym_tile_points(int n_mode);
int sym_tile_count(int n_rep, int n_ops, int n_mode);
cudaError_t launch_sample_bits(int32_t n_full, int32_t n_row, const int64_t *rbeg, const int32_t *rlen,
                               const int32_t *list, uint32_t *bits, cudaStream_t s);
cudaError_t launch_sym_tile(const MeshDev &m, const OrbitDev &o, int32_t n_row, const int32_t *row_q1, double *xi,
                            const uint32_t *sbits, bool dist, bool scat, cudaStream_t s);
// Adjoint of symmetrize_scatmat then symmetrize_and_distribute (three-phonon terms) on the
// cotangent w in place, the distribution's active entries given by the raw terms od_raw.
cudaError_t launch_sym_tile_adjoint(const MeshDev &m, const OrbitDev &o, int32_t n_row, const int32_t *row_q1,
                                    const double *od_raw, double *w, const uint32_t *sbits, cudaStream_t s);
// K8: buf[r*3+a] = sum_j xi[r, j] * fbb[j*3 + a] on the FP32 pipe, xi and fbb as (hi, lo)
// float pairs accumulated in double-float. launch_split_xi converts the FP64 Xi into row
// pairs (xi_pairs_elems(n_row, n_col) float4: hi of rows 2p and 2p + 1, lo of both); part:
// xi_gemv_part_elems(n_row) doubles.
size_t xi_pairs_elems(int32_t n_row, int64_t n_col);
cudaError_t launch_split_xi(const double *xi, int32_t n_row, int64_t n_col, float4 *out, cudaStream_t s);
size_t xi_gemv_part_elems(int32_t n_row);
// shape: rows per CTA (4 or 8) * 100 + column ranges per row group (0: 4 rows and a default
// split sized for about two waves).
cudaError_t launch_xi_gemv(const float4 *xi, int32_t n_row, int64_t n_col, const float2 *fbb, double *part,
                           double *buf, int n_sm, cudaStream_t s, const int32_t *skip = nullptr, int shape = 0);
int xi_gemv_default_split(int32_t n_row, int64_t n_col, int n_sm);
int xi_gemv_max_split(int64_t n_col);

// One-tile tcgen05 self-check: d (128 x n) = a (128 x 16) b (16 x n) through BF16 hi/lo
// splits; variant selects the operand layout reading (diagnostic).
cudaError_t launch_mma_check(int variant, int n, const float *a, const float *b, float *d, int *status,
                             cudaStream_t s);

// foldout of the BTE: fbb[(q*n + b)*3 + d] = sign * (R fn[(irr(q)*n + b)*3 ..])_d, with
// full_op signed 1-based operations (negative: time reversal) and full_irr 0-based; stored
// as (hi, lo) float pairs (the Xi.F element format).
cudaError_t launch_foldout(int32_t n_full, int32_t n_mode, const int32_t *full_op, const int32_t *full_irr,
                           const double *op_cart, const double *fn, float2 *fbb, cudaStream_t s,
                           const int32_t *skip = nullptr);

// Device state of the BTE iteration (kappa.f90:326-495): the iteration counter, the mixing
// factor and the done flag, which every kernel of an iteration checks first.
struct BteCtl {
    int32_t done, iter;
    double mixing;
};
struct BteDev {
    int32_t n_irr, n_mode, n_row, maxiter;
    double tol, sqtol;
    const int32_t *rowidx;            // [n_irr*n] row of (q1, b1), -1 without one
    const double *qs;                 // [n_irr*n]
    const double *F0;                 // [n_irr*n*3]
    const int32_t *degen;             // [n_irr*n] degenerate-subspace sizes at the irreducible points
    const int32_t *degen_mode;        // [n_irr*n*n] its modes, 1-based
    double *fn, *fnb;                 // [n_irr*n*3] current F and the new one
    double *scf;                      // [maxiter] relative changes
    double *part;                     // [bte_part_elems(n_irr)] partial sums of the change
    BteCtl *ctl;
};
cudaError_t launch_bte_update(const BteDev &d, const double *buf, cudaStream_t s);
int bte_part_elems(int32_t n_irr);

// What an entry point compiled outside the context's own file needs of a context.
// Off-diagonal kappa (k_offdiag.cu). Index tables 0-based.
constexpr int kOffdiagSmemModes = 18;  // up to this many modes the work arrays live in shared memory
struct OffdiagArgs {
    int32_t n, na, n_op;
    const double2 *egv;       // full-mesh eigenvectors, element r of mode b of point f at (f*n + b)*n + r
    const double2 *grad;      // [n_irr][3][n][n] dD/dq, element (r, c) at (x*n + c)*n + r
    const double *omega;      // [n_full][n]
    const double *q_full;     // [n_full][3] Cartesian, 1/Bohr without 2*pi
    const int32_t *irr_full;  // [n_irr]
    const int32_t *irr_nop;   // [n_irr]
    const int32_t *irr_ops;   // [n_irr][n_op]
    const double *op_cart;    // [n_op][9]
    const int32_t *fmap;      // [n_op][na]
    const double *shift;      // [n_op][na][3]
    const double *lw;         // [n_irr][n] linewidths
    const double *cv;         // [n_irr][n] heat capacities (k_B when classical)
    const double *irr_weight; // [n_irr]
    double inv_volume;
    double chop_tol;          // velocity components below this become 0 (kappa.f90:209)
    double2 *work;            // beyond kOffdiagSmemModes modes: offdiag_work_elems(n, n_irr, 0)
    // up to kOffdiagSmemModes modes: the (point, operation index) items, point-major in
    // operation order, the first item of each point ([n_irr + 1]) and the items' parts
    // ([n_items][3][n][n], offdiag_work_elems(n, n_irr, n_items))
    const int2 *items;
    const int32_t *item_ptr;
    double2 *part;
    double *vel;              // optional [n_irr][n][n][3] off-diagonal velocities
    double *S;                // [n_irr][9] sum over mode pairs of w v v^T, column-major
};
size_t offdiag_work_elems(int n, int n_irr, int n_items);
cudaError_t launch_offdiag(const OffdiagArgs &a, int n_irr, int n_items, cudaStream_t s);

struct CtxView {
    int device;
    cudaStream_t stream;
    MeshDev mesh;
    int64_t *xfer;  // the context's transfer counter
};
CtxView ctx_view(tdg_ctx *c);


// The library's stream-ordered memory pool of a device (keeps what is freed; contexts and the
// device harmonic stage allocate from it), or nullptr.
cudaMemPool_t shared_device_pool(int device);

// ---- launch-shape autotuner (autotune.cu) ----
// Key of a decision: kernel name, mode count, precision, SM count and device name.
std::string tune_key(const char *kernel, int n, int precision, int device);
// The table's decision for key, or dflt.
int tune_lookup(const std::string &key, int dflt);
// The decision for key: from the table, or (trials enabled, two or more candidates) the
// candidate whose trial(c) ran fastest on stream s, which is then recorded; otherwise dflt.
// tuned is true when trials ran (their outputs are the caller's to discard).
cudaError_t tune_pick(const std::string &key, const std::vector<int> &cand, int dflt,
                      const std::function<cudaError_t(int)> &trial, cudaStream_t s, int &choice, bool &tuned);
// Resident CTAs per SM of kernel fn with `threads` threads and dyn_bytes of dynamic shared
// memory (the attribute is set, with the largest shared-memory carveout): the larger of the
// runtime's occupancy figure (api_out) and the count from the kernel's registers and shared
// memory (count_out); 0 when neither is available. A persistent grid sized from it that is
// larger than what fits only queues the surplus CTAs.
int resident_ctas(const void *fn, int threads, size_t dyn_bytes, int *api_out, int *count_out);

}  // namespace tdg
