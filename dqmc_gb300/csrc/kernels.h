// Host-side launch interface of the device kernels (internal to the library).
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include "common.cuh"

enum SliceMode : int {
  SLICE_LEFT_B = 0,      // M <- B_l M        (multiply_B_left!)
  SLICE_RIGHT_B = 1,     // M <- M B_l        (multiply_B_right!)
  SLICE_LEFT_BINV = 2,   // M <- B_l^-1 M     (multiply_B_inv_left!)
  SLICE_RIGHT_BINV = 3,  // M <- M B_l^-1     (multiply_B_inv_right!)
  SLICE_LEFT_BDAG = 4,   // M <- B_l^dag M    (multiply_daggered_B_left!)
  SLICE_EFF_RIGHT = 5,   // M <- M Hb_half Ha_half           (effective_greens2greens!, right part)
  SLICE_EFF_LEFT_INV = 6 // M <- Ha_half^-1 Hb_half^-1 M     (effective_greens2greens!, left part)
};

// ---- slice matrices (k_slice.cu) ----
size_t evtab_entry_bytes();
cudaError_t launch_build_evtab(const double* phi, void* evtab, int N, int M, double lambda_dtau, cudaStream_t st);
// Applies `count` slices (0-based first, stepping by `step`) to the columns
// of A (left modes), then scales column c by colscale[c] when colscale != 0.
cudaError_t launch_apply_cols(cplx* A, int n, const ModelConst& mc, const void* evtab, int first_slice0,
                              int count, int step, int mode, const double* colscale, cudaStream_t st);
// Applies `count` slices to the rows of A (right modes).
cudaError_t launch_apply_rows(cplx* A, int n, const ModelConst& mc, const void* evtab, int first_slice0,
                              int count, int step, int mode, cudaStream_t st);

// ---- local updates (k_local.cu) ----
struct LocalUpdateArgs {
  cplx* G;
  double* phi;             // (3, N, M)
  void* evtab;             // (N, M) interaction entries, kept in sync with phi (may be null)
  int slice0;              // 0-based slice
  const double* delta;     // (3, N) proposal shifts of this call
  const double* unif;      // (N) Metropolis uniforms of this call
  uint8_t* acc_out;        // (N) or null
  cplx* det_out;           // (N) or null
  double* pacc_out;        // (N) or null
  double* action;          // running boson action (device scalar)
  int* n_acc;              // running accepted count (device scalar)
  cplx* Acol;              // scratch (n, 4)
  cplx* Brow;              // scratch (4, n)
  GridBarrier* bar;
  int* err;
  ModelConst mc;
};
cudaError_t launch_local_updates(const LocalUpdateArgs& a, int sm_count, cudaStream_t st, int max_grid = 0);
// delayed rank-k form: pending factors X (n x 4k, column-major) and Y (4k x n,
// row j at Y + j*n); state[0] = next site of the slice, state[1] = pending accepts
// Per-site data of one slice, prepared once before its first delayed round
// (the old field of a site cannot change before its own visit).
struct SitePrep {
  cplx delta[16];          // Delta_i = e^{+dtau V(phi_i)} e^{-dtau V(phi_i + delta_i)} - I, row-major
  EvEntry ev;              // interaction entries of the proposed field
  double diff[3];          // proposed minus old field
  double dsA, dsQ, dsB;    // boson action difference, space-neighbour coupling excluded
  double pad[2];
};
// state (2 ints, nullable): delayed-round state of the slice, zeroed here
cudaError_t launch_local_prepare(const LocalUpdateArgs& a, SitePrep* prep, int* state, cudaStream_t st);
// BF16 slices of the operands of an m x n x K split-BF16 product in its
// scratch block: As S x (m x Kp), Bre / Bim S x (n x Kp) (K contiguous, Kp =
// 2 Kpad), row scales sA (m), column scales sB (n)
struct OzSlices {
  __nv_bfloat16 *As, *Bre, *Bim;
  double *sA, *sB;
  int m, n, Kpad, S, bits;
};
struct DelayedArgs {
  cplx* X;
  cplx* Y;
  int* state;
  int k;
  const SitePrep* prep;    // (N) from launch_local_prepare for this slice
  cplx* blk;               // (N, 16) cache of the diagonal blocks G_cur[j + rN, j + cN]
  int* pub;                // (N) acceptances of the current round folded into site j's data
  OzSlices sl;             // mixed form: the flush's slices, cut by the owners at the round's end
                           // (sl.As null: the flush slices X and Y itself)
};
cudaError_t launch_local_delayed(const LocalUpdateArgs& a, const DelayedArgs& d, int sm_count, cudaStream_t st,
                                 int max_grid = 0);
// Sets the WHILE condition of a captured round loop (see local_updates_dev):
// another round while state[0] < N, state[2] < max_rounds and *err == 0.
cudaError_t launch_round_cond(cudaGraphConditionalHandle hc, int* state, int N, int max_rounds, const int* err,
                              unsigned long long* rounds_total, cudaStream_t st);


// ---- dense linear algebra (k_linalg.cu) ----
// C = alpha * op(A) * op(B) + beta * C, all n x n column-major; op: 'N', 'C' (conjugate transpose)
// optional diagonal scalings: rowscale (applied to rows of op(A)), colscale (to columns of op(B)).
// active: optional device count p of pending rank-4 factors; when given, the
// product uses only the first 4p columns of op(A) / rows of op(B), and does
// nothing when p == 0 (the delayed-update flush).
cudaError_t launch_zgemm(int m, int nn, int k, char opA, char opB, cplx alpha, const cplx* A, int lda,
                         const cplx* B, int ldb, cplx beta, cplx* C, int ldc, const double* rowscale,
                         const double* colscale, cudaStream_t st, const int* active = nullptr);

struct QRWork {
  double* vn1;       // (2n) partial column norms, reciprocals at [n + j]
  double* vn2;       // (2n) norms at the last recomputation, reciprocals at [n + j]
  int* order;        // (n) logical position -> physical column
  cplx* tau;         // (n)
  double* beta;      // (n) real diagonal of R in logical order
  cplx* V;           // (n, n) Householder vectors, column k = v_k (v_k[k] = 1, zero above)
  double* cand_v;    // (grid) per-CTA pivot candidates: norm
  int* cand_q;       // (grid) and logical position
  GridBarrier* bar;
  int* err;
};
// Column-pivoted Householder QR of A (n x n) in place (LAPACK geqp3 semantics
// without physical column swaps).  On return the upper part of A (rows <=
// logical position of each physical column) holds R in physical column
// order; V/tau hold the reflectors; order/beta the pivots and diag(R).
// max_grid > 0 caps the cooperative grid (chains sharing the GPU)
cudaError_t launch_qrp(cplx* A, int n, QRWork& w, int sm_count, cudaStream_t st, int max_grid = 0);
// After launch_qrp: D[k] = |beta[k]|, T (physical layout) = D^-1 R with zeros below.
cudaError_t launch_qrp_finalize(cplx* A, cplx* T, double* D, int n, const QRWork& w, cudaStream_t st);
// X (m x n) <- X * Q  with Q = H_0 ... H_{n-1} (reflectors in w).  Also used
// with X = I to form Q explicitly.  conj_transpose_q: X <- X * Q^H.
cudaError_t launch_apply_q_right(cplx* X, int m, int n, const QRWork& w, bool conj_transpose_q, cudaStream_t st);
// Upper-triangular solves with the logical-order factor Rhat of a QR (unit
// scaled: That = D^-1 R), using the physical-layout T from launch_qrp_finalize:
//   left:  Y <- That^-1 Y       (Y is n x m)
//   right: Y <- Y That^-1       (Y is m x n)
// Row/column permutation by the pivot order is applied by the caller with
// launch_permute.
// order == nullptr: T itself is upper triangular; rdiag != nullptr: 1 / diagonal (else the diagonal of T)
cudaError_t launch_trsm_left_upper(const cplx* T, const int* order, const cplx* rdiag, cplx* Y, int n, int m,
                                   cudaStream_t st);
// rows j0..j0+b of the m columns of Y <- (b x b diagonal block of T at j0)^-1 (.) (b <= 128):
// lower: unit lower triangular; else upper with reciprocal diagonal rdiag
cudaError_t launch_trsm_diag_block(const cplx* T, int ldT, const cplx* rdiag, cplx* Y, int ldY, int j0, int b, int m,
                                   bool lower, cudaStream_t st);
// Y <- L^-1 Y, L unit lower triangular (strictly lower part of Lc)
cudaError_t launch_trsm_left_lower_unit(const cplx* Lc, cplx* Y, int n, int m, cudaStream_t st);
// Results of the LU with partial pivoting P A = L U (zgetrf semantics).
struct LUWork {
  int* perm;         // (n) row perm[i] of A is row i of P A
  cplx* udiag;       // (n) diagonal of U
  cplx* rdiag;       // (n) 1 / diagonal of U
};
// Unblocked cooperative LU (small n): U in A's strict upper part, L in Lb's strict lower part.
struct LUKernel {
  int* perm;
  cplx* udiag;
  cplx* rdiag;
  int* pivrow;       // (2) pivot row of the next step, by step parity
  GridBarrier* bar;
  int* err;
};
cudaError_t launch_lup(cplx* A, cplx* Lb, int n, LUKernel& w, int sm_count, cudaStream_t st, int max_grid = 0);
// compact-WY block jb..jb+b of the reflectors in V/tau: Vb ((n-jb) x b), trd (b) (tau, 1 for identity reflectors)
cudaError_t launch_wy_prep(const cplx* V, const cplx* tau, int n, int jb, int b, cplx* Vb, cplx* trd,
                           cudaStream_t st);
// Blocked LU (in place): panel factorisation of columns [p0, p0+b) (b <= LU_PB) over rows [p0, n)
constexpr int LU_PB = 64;
struct LUPanel {
  int* piv;            // (n) pivot row of each step
  double* cand_v;      // (grid) per-CTA pivot candidates: |Re| + |Im|
  int* cand_r;         // (grid) and row
  cplx* cand_rows;     // (grid, LU_PB) the candidate rows' panel values
  cplx* rowk;          // (2, LU_PB) row k of the step, by step parity
  GridBarrier* bar;
  int* err;
};
// cluster >= 8: the panel on one thread-block cluster of that many CTAs (16 or
// 8; the cooperative grid when no cluster can be scheduled); 0: the grid
cudaError_t launch_lu_panel(cplx* A, int n, int p0, int b, LUPanel& w, int sm_count, cudaStream_t st,
                            int max_grid = 0, int cluster = 0);
// the panel's row exchanges applied to the columns outside [p0, p0+b) and to perm
cudaError_t launch_lu_apply_swaps(cplx* A, int n, int p0, int b, const int* piv, int* perm, cudaStream_t st);
cudaError_t launch_lu_diag(const cplx* A, int n, cplx* udiag, cplx* rdiag, cudaStream_t st);
cudaError_t launch_iota(int* p, int n, cudaStream_t st);
// C = A + B (count complex entries)
cudaError_t launch_add(const cplx* A, const cplx* B, cplx* C, size_t count, cudaStream_t st);
// D-scale separation: s = [1/max(Dl,1), min(Dl,1), 1/max(Dr,1), min(Dr,1)] (4n)
cudaError_t launch_split_scales(const double* Dl, const double* Dr, int n, double* s, cudaStream_t st);
// out[0] = sum log|udiag| + sum log max(Dl,1) + sum log max(Dr,1)
cudaError_t launch_lu_logdet(const cplx* udiag, const double* Dl, const double* Dr, int n, double* out,
                             cudaStream_t st);
cudaError_t launch_trsm_right_upper(const cplx* T, const int* order, cplx* Y, int m, int n, cudaStream_t st);
// dst = src with rows (by_rows) or columns permuted: dst[order[k]] = src[k] (scatter) when scatter, else gather.
cudaError_t launch_permute(const cplx* src, cplx* dst, int rows, int cols, const int* order, bool by_rows,
                           bool scatter, cudaStream_t st);
// A += diag(d) (d real)
cudaError_t launch_add_diag(cplx* A, int n, const double* d, cudaStream_t st);
// A <- I
cudaError_t launch_set_identity(cplx* A, int n, cudaStream_t st);
// out[0] = sum_k log(x[k]) (one deterministic single-CTA reduction)
cudaError_t launch_sum_log(const double* x, int n, double* out, cudaStream_t st);
// max |A - B| over n*n entries -> out
cudaError_t launch_max_absdiff(const cplx* A, const cplx* B, size_t count, double* out, cudaStream_t st,
                               bool reset = true);
// d[0..n) = v
cudaError_t launch_fill(double* d, int n, double v, cudaStream_t st);
// A (rows x cols) scaled: A[r,c] *= rowscale[r] (if non-null) * colscale[c] (if non-null); rowscale may be inverted
cudaError_t launch_scale(cplx* A, int rows, int cols, const double* rowscale, bool invert_rows,
                         const double* colscale, bool invert_cols, cudaStream_t st);
cudaError_t launch_conj_transpose(const cplx* A, cplx* B, int n, cudaStream_t st);

// ---- diagnostics (k_diag.cu) ----
cudaError_t measure_peak_fp64(int device, double* tflops);

// ---- split-precision complex GEMM (k_ozaki.cu) ----
bool ozaki_plan(int K, int target_bits, int* S, int* bits);
size_t ozaki_scratch_bytes(int m, int n, int K, int S);
// where launch_ozaki_zgemm keeps the slices of an m x n x K product in scratch
OzSlices ozaki_slices(void* scratch, int m, int n, int K, int S, int bits);
cudaError_t launch_ozaki_zgemm(int m, int nn, int k, char opA, char opB, cplx alpha, const cplx* A, int lda,
                               const cplx* B, int ldb, cplx beta, cplx* C, int ldc, const double* rowscale,
                               const double* colscale, int S, int bits, void* scratch, size_t scratch_bytes,
                               unsigned long long* acc, size_t acc_bytes, cudaStream_t st,
                               const int* active = nullptr, int splitk = 1, int* kernels = nullptr,
                               int* err = nullptr, bool persistent = true, bool presliced = false);

// ---- adjoint force (k_force.cu) ----
// grad[:, :, slice0] = d log|det M| / d phi[:, :, slice0] from G of that slice
// ---- equal-time correlators (k_measure.cu) ----
// out (6 L^2 doubles): P+ and P- (L x L real), C+ and C- (L x L complex) of the true G
cudaError_t launch_equal_time_corr(const cplx* G, int L, double* out, cudaStream_t st);
// out (2 L^2 doubles): P+ and P- summed over the `slices` matrices of Gt0 (stride n^2)
cudaError_t launch_zfpc(const cplx* Gt0, int slices, int L, double* out, cudaStream_t st);
// out (4 L^2 doubles): C+ and C- (L x L complex) of the equal-time G, G(tau, 0) and -G(0, tau)
cudaError_t launch_zfcdc(const cplx* G, const cplx* Gt0, const cplx* G0t, int slices, int L, double* out,
                         cudaStream_t st);
// out (4 L^2 doubles): Lambda_xx and Lambda_yy (L x L complex); thop[dir][band] hopping amplitudes
cudaError_t launch_zfccc(const cplx* G, const cplx* Gt0, const cplx* G0t, int slices, int L, const double thop[2][2],
                         double* out, cudaStream_t st);

cudaError_t launch_force_slice(const cplx* G, const double* phi, double* grad, int N, int slice0, double lambda_dtau,
                               cudaStream_t st);
// phi[a, :, :] += shift[a] for a = 0..2 (field of N sites x M slices)
cudaError_t launch_shift_field(double* phi, size_t NM, double s0, double s1, double s2, cudaStream_t st);
