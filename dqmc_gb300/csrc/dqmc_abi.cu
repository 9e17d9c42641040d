// Host engine and C ABI of the GB300 DQMC sweep library.
//
// The engine keeps the reference's state machine on the host (which slice,
// which direction, when to stabilise: src/stack.jl:391-499) and runs every
// matrix operation on the device, on one CUDA stream per handle.  All device
// memory is allocated once in dqmc_create.
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <utility>
#include <string>
#include <initializer_list>
#include <array>
#include <vector>
#include <array>

#include "../../include/dqmc_gpu.h"
#include "common.cuh"
#include "kernels.h"

#define DQMC_VERSION_STRING "dqmc_gb300 0.2 (sm_103a, FP64 + split-BF16 tensor-core form)"

struct TimedSpan {
  cudaEvent_t a, b;
  int kind;
};

struct dqmc_handle {
  dqmc_params p{};
  ModelConst mc{};
  int L = 0, N = 0, n = 0, M = 0, s = 0, ne = 0;
  cudaStream_t st = nullptr;
  int sm_count = 0;
  int device = 0;
  int coop_cap = 0;            // > 0: cap of the cooperative grids (chains sharing the GPU)
  // ---- device state ----
  double* phi = nullptr;       // (3, N, M)
  void* evtab = nullptr;       // (N, M) EvEntry
  cplx* G = nullptr;
  cplx* Gtmp = nullptr;        // greens_temp
  cplx* u_stack = nullptr;     // ne x (n x n)
  double* d_stack = nullptr;   // ne x n
  cplx* t_stack = nullptr;     // ne x (n x n)
  cplx *Ul = nullptr, *Ur = nullptr, *Tl = nullptr, *Tr = nullptr;
  double *Dl = nullptr, *Dr = nullptr;
  cplx *W1 = nullptr, *W2 = nullptr, *W3 = nullptr, *W4 = nullptr;
  double *D1 = nullptr, *d2 = nullptr;
  int* ord1 = nullptr;
  QRWork qr{};
  // mixed form: split-BF16 GEMM scratch and slicing
  void* oz_scratch = nullptr;
  size_t oz_bytes = 0;
  unsigned long long* oz_acc = nullptr;   // split-K integer sums, zero between products
  size_t oz_acc_bytes = 0;
  int oz_target = 40;   // mantissa bits kept per operand
  // local updates
  double* delta_d = nullptr;
  double* unif_d = nullptr;
  int stream_cap = 0;          // update calls the stream buffers hold
  uint8_t* acc_d = nullptr;
  cplx* det_d = nullptr;
  double* pacc_d = nullptr;
  int out_cap = 0;
  double* action_d = nullptr;
  int* nacc_d = nullptr;
  cplx* Acol = nullptr;
  cplx* Brow = nullptr;
  // delayed updates: pending factors and {next site, pending count}
  int delay = 1;
  cplx* Xd = nullptr;
  cplx* Yd = nullptr;
  int* dstate = nullptr;
  SitePrep* prep = nullptr;   // (N) per-site constants of the slice being updated
  cplx* blk = nullptr;        // (N, 16) cached diagonal blocks of G_cur
  int* pub = nullptr;         // (N) per-site publication counters of the delayed rounds
  int greens_method = DQMC_GREENS_SCALES;
  LUWork lu{};                // LU of the D-scale separated calculate_greens
  LUPanel lup{};              // blocked LU: pivots and per-step candidate copies
  cplx* lu_L = nullptr;       // (n x n) unit lower factor of the unblocked LU (strict lower part)
  int* lu_pivrow = nullptr;   // (2) unblocked LU: next pivot row by step parity
  double* lu_scales = nullptr;   // (4n) 1/max(Dl,1), min(Dl,1), 1/max(Dr,1), min(Dr,1)
  // block sizes of the mixed-form factorisations and the LU panel grid
  // (DQMC_TUNE="wy=128,trsm=64,lu_grid=64,lu_small=576" overrides; lu_grid 0
  // = one CTA per SM; n <= lu_small takes the unblocked LU).  Defaults
  // measured at L=16 on GB300: WY 32/64/128 -> 213/128/102 ms per sweep,
  // triangular solves 32/64/128 -> 119/97/107 ms, LU panel grid 32/64/152 ->
  // 186/184/194 ms; LU per sweep blocked/unblocked: n = 144 9.0/5.8 ms,
  // n = 576 39.8/33.9 ms, n = 1024 184/232 ms.
  int wy_block = 128, trsm_block = 64, lu_grid = 64, lu_small = 576;
  // LU panels on one thread-block cluster of this many CTAs (16 or 8; 0: the
  // cooperative grid of lu_grid CTAs; DQMC_TUNE "lu_cluster=").  The grid is
  // the default: at n = 1024 both took about 0.3 ms per panel (the cluster's
  // FP64 work on 16 SMs offsets its cheaper barriers) and 141 ms of LU per sweep
  int lu_cluster = 0;
  cplx* wy_v = nullptr;       // mixed form: (n x kWyMax) reflector block
  cplx* wy_s = nullptr;       // (kWyMax^2) Vb^H Vb
  cplx* wy_z = nullptr;       // (kWyMax x n) T Vb^H W
  cplx* wy_t = nullptr;       // (kWyMax) tau of the block
  double* force_d = nullptr;   // (3, N, M) d log|det M| / d phi
  // time-displaced measurement: work matrices and B-chain stacks in one block,
  // and G(tau, 0) / G(0, tau) buffers for host or absent outputs (allocated on
  // the first measurement and kept until dqmc_destroy)
  void* tdgf_ws = nullptr;
  cplx* tdgf_a = nullptr;
  cplx* tdgf_b = nullptr;
  double* etc_d = nullptr;     // (6 N) equal-time correlators P+, P-, C+, C-
  // global updates: backup of stack, G, field and interaction table (allocated on first use)
  cplx *gb_u = nullptr, *gb_t = nullptr, *gb_G = nullptr;
  double *gb_d = nullptr, *gb_phi = nullptr;
  void* gb_evtab = nullptr;
  GridBarrier* bar = nullptr;
  int* err_d = nullptr;
  double* scal_d = nullptr;    // scalars: [0] sum log d2, [1] absdiff, [2] saved sum log d2, [3] instability max
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;   // brackets of the last enqueued sweep
  int pending_calls = 0;
  // ---- host state ----
  int current_slice = 0;
  int direction = 1;
  bool initialized = false;
  double max_instability = 0.0;
  std::string last_error;
  // timing
  bool timing = false;
  // CUDA graphs of whole sweeps, one per (start slice, direction, calls, flags output)
  struct SweepGraph {
    int slice0 = 0, dir0 = 0, n_calls = 0, acc = 0, slice1 = 0, dir1 = 0;
    cudaGraphExec_t exec = nullptr;
    int64_t cnt[DQMC_NKINDS] = {};
    double flops[DQMC_NKINDS] = {}, bytes[DQMC_NKINDS] = {};
    int64_t launches = 0;
    int while_nodes = 0;      // captured round loops (one body each in the counts above)
  };
  std::vector<SweepGraph> graphs;
  bool graphs_off = false;    // capture refused once: direct launches from then on
  // delayed rounds inside a captured sweep: a WHILE node repeats [round, flush]
  // only while sites remain; its body is captured on st_body
  cudaStream_t st_body = nullptr;
  bool while_off = false;     // conditional nodes refused once: fixed round count from then on
  int64_t graph_epoch = 0;    // advanced whenever the captured launches may have gone stale
  int capture_while = 0;      // WHILE nodes added in the capture in progress
  int pending_while = 0;      // WHILE nodes of the enqueued sweep
  unsigned long long rounds_seen = 0;   // device round counter at the last sweep_finish
  int64_t body_cnt[DQMC_NKINDS] = {};   // launches, flops and bytes of one round body
  double body_flops[DQMC_NKINDS] = {}, body_bytes[DQMC_NKINDS] = {};
  int64_t body_launches = 0;
  cudaEvent_t done = nullptr; // end of the last enqueued sweep (batch pipelining)
  std::vector<TimedSpan> spans;
  std::vector<cudaEvent_t> event_pool;
  size_t event_next = 0;
  double ms[DQMC_NKINDS] = {};
  int64_t cnt[DQMC_NKINDS] = {};
  double flops[DQMC_NKINDS] = {};
  double bytes[DQMC_NKINDS] = {};
  int64_t launches = 0;
};

void fill_model_const(const dqmc_params& p, ModelConst& m);

namespace {

int set_err(dqmc_handle* h, int code, const std::string& msg) {
  if (h) h->last_error = msg;
  return code;
}

#define CU(call)                                                                               \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return set_err(h, DQMC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
  } while (0)

#define CHK(expr)                 \
  do {                            \
    int r_ = (expr);              \
    if (r_ != DQMC_OK) return r_; \
  } while (0)

cudaEvent_t next_event(dqmc_handle* h) {
  if (h->event_next >= h->event_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    h->event_pool.push_back(e);
  }
  return h->event_pool[h->event_next++];
}

// One kernel launch: counted, its algorithmic work accumulated, and bracketed
// by CUDA events on the handle's stream when timing is enabled.
struct KSpan {
  dqmc_handle* h;
  int kind;
  cudaEvent_t a = nullptr;
  KSpan(dqmc_handle* hh, int k, double fl, double by) : h(hh), kind(k) {
    if (h->timing) {
      a = next_event(h);
      cudaEventRecord(a, h->st);
    }
    h->cnt[kind]++;
    h->flops[kind] += fl;
    h->bytes[kind] += by;
    h->launches++;
  }
  ~KSpan() {
    if (h->timing) {
      cudaEvent_t b = next_event(h);
      cudaEventRecord(b, h->st);
      h->spans.push_back({a, b, kind});
    }
  }
};

#define LAUNCH(kind, fl, by, call)      \
  do {                                  \
    KSpan ks_(h, kind, (fl), (by));     \
    CU(call);                           \
  } while (0)

// Resolves recorded spans into accumulated milliseconds (stream must be idle).
void resolve_spans(dqmc_handle* h) {
  for (auto& sp : h->spans) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, sp.a, sp.b) == cudaSuccess) h->ms[sp.kind] += t;
  }
  h->spans.clear();
  h->event_next = 0;
}

int check_device_error(dqmc_handle* h) {
  int e = 0;
  CU(cudaMemcpyAsync(&e, h->err_d, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CU(cudaStreamSynchronize(h->st));
  if (e == 0) return DQMC_OK;
  CU(cudaMemsetAsync(h->err_d, 0, sizeof(int), h->st));
  if (e & DQMC_KERR_BARRIER_TIMEOUT) return set_err(h, DQMC_ERR_TIMEOUT, "device barrier timed out");
  if (e & DQMC_KERR_SINGULAR) return set_err(h, DQMC_ERR_SINGULAR, "singular 4x4 M in a local update");
  if (e & DQMC_KERR_NONFINITE) return set_err(h, DQMC_ERR_NONFINITE, "non-finite determinant ratio");
  return set_err(h, DQMC_ERR_CUDA, "device error flag " + std::to_string(e));
}

int read_instability(dqmc_handle* h);

int sync(dqmc_handle* h) {
  CU(cudaStreamSynchronize(h->st));
  if (h->timing) resolve_spans(h);
  CHK(check_device_error(h));
  return read_instability(h);
}

size_t nn_bytes(const dqmc_handle* h) { return (size_t)h->n * h->n * sizeof(cplx); }
// algorithmic work models (real FP64 flops; bytes of one pass over the operands)
double n2(const dqmc_handle* h) { return (double)h->n * h->n; }
double n3(const dqmc_handle* h) { return (double)h->n * h->n * h->n; }
double gemm_flops(double m, double nn, double k) { return 8.0 * m * nn * k; }
double gemm_bytes(double m, double nn, double k) { return 16.0 * (m * k + k * nn + 2.0 * m * nn); }
cplx* ustk(dqmc_handle* h, int k) { return h->u_stack + (size_t)k * h->n * h->n; }
cplx* tstk(dqmc_handle* h, int k) { return h->t_stack + (size_t)k * h->n * h->n; }
double* dstk(dqmc_handle* h, int k) { return h->d_stack + (size_t)k * h->n; }

int copy_nn(dqmc_handle* h, cplx* dst, const cplx* src) {
  CU(cudaMemcpyAsync(dst, src, nn_bytes(h), cudaMemcpyDeviceToDevice, h->st));
  return DQMC_OK;
}

int set_identity(dqmc_handle* h, cplx* A) {
  LAUNCH(DQMC_K_MISC, 0.0, 16.0 * n2(h), launch_set_identity(A, h->n, h->st));
  return DQMC_OK;
}

int set_ones(dqmc_handle* h, double* d) {
  LAUNCH(DQMC_K_MISC, 0.0, 8.0 * h->n, launch_fill(d, h->n, 1.0, h->st));
  return DQMC_OK;
}

// ---- slice matrices ---------------------------------------------------------
int apply_cols(dqmc_handle* h, cplx* A, int first0, int count, int step, int mode, const double* colscale) {
  const double per = (mode == SLICE_EFF_LEFT_INV) ? 32.0 : 74.0;
  LAUNCH(DQMC_K_SLICE_COLS, per * n2(h) * count, 32.0 * n2(h),
         launch_apply_cols(A, h->n, h->mc, h->evtab, first0, count, step, mode, colscale, h->st));
  return DQMC_OK;
}
int apply_rows(dqmc_handle* h, cplx* A, int first0, int count, int step, int mode) {
  const double per = (mode == SLICE_EFF_RIGHT) ? 32.0 : 74.0;
  LAUNCH(DQMC_K_SLICE_ROWS, per * n2(h) * count, 32.0 * n2(h),
         launch_apply_rows(A, h->n, h->mc, h->evtab, first0, count, step, mode, h->st));
  return DQMC_OK;
}

// wrap_greens! (src/stack.jl:316-325); slice is 1-based.
int wrap_greens(dqmc_handle* h, cplx* gf, int slice, int direction) {
  if (direction == -1) {
    CHK(apply_cols(h, gf, slice - 2, 1, 1, SLICE_LEFT_BINV, nullptr));
    CHK(apply_rows(h, gf, slice - 2, 1, 1, SLICE_RIGHT_B));
  } else {
    CHK(apply_cols(h, gf, slice - 1, 1, 1, SLICE_LEFT_B, nullptr));
    CHK(apply_rows(h, gf, slice - 1, 1, 1, SLICE_RIGHT_BINV));
  }
  return DQMC_OK;
}

// ---- dense kernels with their work models ----------------------------------
// tensor flops of one split-BF16 complex GEMM: S(S+1)/2 slice pairs x 2 real GEMMs with K' = 2K
double ozaki_tensor_flops(double m, double nn, double k, int S) {
  const double kp = 2.0 * std::ceil(k / 16.0) * 16.0;
  return S * (S + 1) / 2.0 * 2.0 * 2.0 * m * nn * kp;
}
int zgemm_general(dqmc_handle* h, int m, int nn, int k, char opA, char opB, cplx alpha, const cplx* A, int lda,
                  const cplx* B, int ldb, cplx beta, cplx* C, int ldc, const double* rs, const double* cs,
                  bool allow_split, int kind = -1, const int* active = nullptr, bool presliced = false) {
  if (allow_split && h->p.precision == DQMC_PREC_MIXED) {
    int S = 0, bits = 0;
    if (!ozaki_plan(k, h->oz_target, &S, &bits)) return set_err(h, DQMC_ERR_ARG, "no exact slicing for this K");
    // few output tiles and a long K: split K over more CTAs (exact integer partial sums)
    const int tiles = ((m + 63) / 64) * ((nn + 63) / 64);
    int splitk = 1;
    if (!active && tiles * 2 < h->sm_count && k >= 256) {
      splitk = (h->sm_count + tiles - 1) / tiles;
      if (splitk > k / 64) splitk = k / 64;
    }
    int kernels = 3;
    LAUNCH(kind >= 0 ? kind : DQMC_K_OZGEMM, ozaki_tensor_flops(m, nn, k, S), gemm_bytes(m, nn, k),
           launch_ozaki_zgemm(m, nn, k, opA, opB, alpha, A, lda, B, ldb, beta, C, ldc, rs, cs, S, bits,
                              h->oz_scratch, h->oz_bytes, h->oz_acc, h->oz_acc_bytes, h->st, active, splitk,
                              &kernels, h->err_d, h->coop_cap == 0, presliced));
    h->launches += kernels - 1;   // slicing kernels and the split-K finaliser
    return DQMC_OK;
  }
  LAUNCH(kind >= 0 ? kind : DQMC_K_GEMM, gemm_flops(m, nn, k), gemm_bytes(m, nn, k),
         launch_zgemm(m, nn, k, opA, opB, alpha, A, lda, B, ldb, beta, C, ldc, rs, cs, h->st, active));
  return DQMC_OK;
}
// n x n x n product of the stabilisation (split-BF16 in the mixed form)
int gemm(dqmc_handle* h, char opA, char opB, const cplx* A, const cplx* B, cplx* C, const double* rs = nullptr,
         const double* cs = nullptr) {
  const int n = h->n;
  return zgemm_general(h, n, n, n, opA, opB, cmake(1, 0), A, n, B, n, cmake(0, 0), C, n, rs, cs, true);
}
// pivoted QR of A (destroyed) -> T (physical layout), D; reflectors in h->qr
int qrp(dqmc_handle* h, cplx* A, cplx* T, double* D) {
  LAUNCH(DQMC_K_QRP, 16.0 / 3.0 * n3(h), 32.0 * n2(h), launch_qrp(A, h->n, h->qr, h->sm_count, h->st, h->coop_cap));
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_qrp_finalize(A, T, D, h->n, h->qr, h->st));
  return DQMC_OK;
}
// X <- X Q with the reflectors of the last qrp (one register-resident pass per row)
int apply_q(dqmc_handle* h, cplx* X) {
  LAUNCH(DQMC_K_APPLYQ, 8.0 * n3(h), 40.0 * n2(h), launch_apply_q_right(X, h->n, h->n, h->qr, false, h->st));
  return DQMC_OK;
}
int trsm_left(dqmc_handle* h, const cplx* T, const int* order, cplx* Y) {
  LAUNCH(DQMC_K_TRSM, 4.0 * n3(h), 40.0 * n2(h), launch_trsm_left_upper(T, order, nullptr, Y, h->n, h->n, h->st));
  return DQMC_OK;
}
int trsm_right(dqmc_handle* h, const cplx* T, const int* order, cplx* Y) {
  LAUNCH(DQMC_K_TRSM, 4.0 * n3(h), 40.0 * n2(h), launch_trsm_right_upper(T, order, Y, h->n, h->n, h->st));
  return DQMC_OK;
}
int permute(dqmc_handle* h, const cplx* src, cplx* dst, const int* order, bool by_rows, bool scatter) {
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_permute(src, dst, h->n, h->n, order, by_rows, scatter, h->st));
  return DQMC_OK;
}

// Q = H_0 ... H_{n-1} formed explicitly from the reflectors of the last qrp
// in compact-WY blocks of h->wy_block reflectors, backward (W <- B_j W, B_j =
// I - V_j T_j V_j^H, T_j^-1 = diag(1/tau) + striu(V_j^H V_j)), the products as
// split-BF16 GEMMs (mixed form).  Before step j, W differs from I only in
// rows and columns >= (j+1) b, so every product acts on W[jb:, jb:].
constexpr int kWyMax = 128;   // largest compact-WY block (buffer sizes; k_trsm_diag_block limit)
int form_q_wy(dqmc_handle* h, cplx* W) {
  const int n = h->n, b = h->wy_block;
  CHK(set_identity(h, W));
  for (int jb = ((n - 1) / b) * b; jb >= 0; jb -= b) {
    const int m = n - jb, bs = m < b ? m : b;
    LAUNCH(DQMC_K_APPLYQ, 0.0, 32.0 * m * bs, launch_wy_prep(h->qr.V, h->qr.tau, n, jb, bs, h->wy_v, h->wy_t, h->st));
    // S = Vb^H Vb, Z = Vb^H W[jb:, jb:]
    CHK(zgemm_general(h, bs, bs, m, 'C', 'N', cmake(1, 0), h->wy_v, m, h->wy_v, m, cmake(0, 0), h->wy_s, bs, nullptr,
                      nullptr, true, DQMC_K_APPLYQ));
    CHK(zgemm_general(h, bs, m, m, 'C', 'N', cmake(1, 0), h->wy_v, m, W + (size_t)jb * n + jb, n, cmake(0, 0),
                      h->wy_z, bs, nullptr, nullptr, true, DQMC_K_APPLYQ));
    // Z <- T Z: solve T^-1 Y = Z (upper: strict part S, diagonal 1/tau)
    LAUNCH(DQMC_K_APPLYQ, 4.0 * bs * bs * m, 32.0 * bs * m,
           launch_trsm_diag_block(h->wy_s, bs, h->wy_t, h->wy_z, bs, 0, bs, m, false, h->st));
    // W[jb:, jb:] -= Vb Z
    CHK(zgemm_general(h, m, m, bs, 'N', 'N', cmake(-1, 0), h->wy_v, m, h->wy_z, bs, cmake(1, 0),
                      W + (size_t)jb * n + jb, n, nullptr, nullptr, true, DQMC_K_APPLYQ));
  }
  return DQMC_OK;
}

// ---- UDT ------------------------------------------------------------------
// decompose_udt! (src/linalg.jl:20-39) of A (destroyed): U (explicit), D, T.
int decompose_udt(dqmc_handle* h, cplx* A, cplx* U, double* D, cplx* T) {
  CHK(qrp(h, A, T, D));
  if (h->p.precision == DQMC_PREC_MIXED) return form_q_wy(h, U);
  CHK(set_identity(h, U));
  CHK(apply_q(h, U));
  return DQMC_OK;
}

// add_slice_sequence_left (src/stack.jl:278-293); idx 1-based.
int add_slice_sequence_left(dqmc_handle* h, int idx) {
  const int k = idx - 1;
  CHK(copy_nn(h, h->W1, ustk(h, k)));
  CHK(apply_cols(h, h->W1, (idx - 1) * h->s, h->s, 1, SLICE_LEFT_B, dstk(h, k)));
  CHK(decompose_udt(h, h->W1, ustk(h, k + 1), dstk(h, k + 1), h->W2));
  CHK(gemm(h, 'N', 'N', h->W2, tstk(h, k), tstk(h, k + 1)));
  return DQMC_OK;
}

// add_slice_sequence_right (src/stack.jl:299-313); idx 1-based.
int add_slice_sequence_right(dqmc_handle* h, int idx) {
  const int k = idx - 1;
  CHK(copy_nn(h, h->W1, ustk(h, k + 1)));
  CHK(apply_cols(h, h->W1, idx * h->s - 1, h->s, -1, SLICE_LEFT_BDAG, dstk(h, k + 1)));
  CHK(decompose_udt(h, h->W1, ustk(h, k), dstk(h, k), h->W2));
  CHK(gemm(h, 'N', 'N', h->W2, tstk(h, k + 1), tstk(h, k)));
  return DQMC_OK;
}

// calculate_greens + calculate_logdet (src/stack.jl:338-385) on the device
// copies Ul, Dl, Tl, Ur, Dr, Tr, written into `out`; log|det G| left in
// scal_d[0].
//
// Same decomposition steps as the reference (two pivoted QRs), but every
// inverse is taken through the triangular factors instead of LU:
//   T1 = That1 P1^T  =>  T1^-1 = P1 That1^-1,   (T1 Ur^dag)^-1 = Ur T1^-1,
// so  tmp = U^dag (T1 Ur^dag)^-1 + D1 = (U^dag Ur) P1 That1^-1 + D1  and
//   G = (t2 T1 Ur^dag)^-1 diag(1/d2) (U u)^dag
//     = Ur P1 That1^-1 P2 That2^-1 diag(1/d2) (U Q2)^dag.
// log|det G| = -sum log d2 (|det| of the unitary and unit-triangular
// factors is 1).
int calculate_greens_two_qr(dqmc_handle* h, cplx* out) {
  const int n = h->n;
  // 1. X = Dl (Tl Tr^dag) Dr
  CHK(gemm(h, 'N', 'C', h->Tl, h->Tr, h->W1, h->Dl, h->Dr));
  // 2. X = Q1 D1 T1
  CHK(qrp(h, h->W1, h->W2, h->D1));
  CU(cudaMemcpyAsync(h->ord1, h->qr.order, n * sizeof(int), cudaMemcpyDeviceToDevice, h->st));
  // 3. U = Ul Q1
  CHK(copy_nn(h, h->W3, h->Ul));
  CHK(apply_q(h, h->W3));
  // 4. tmp = (U^dag Ur) P1 That1^-1 + diag(D1)
  CHK(gemm(h, 'C', 'N', h->W3, h->Ur, h->W4));
  CHK(permute(h, h->W4, h->W1, h->ord1, false, false));
  CHK(trsm_right(h, h->W2, h->ord1, h->W1));
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n, launch_add_diag(h->W1, n, h->D1, h->st));
  // 5. tmp = Q2 d2 t2
  CHK(qrp(h, h->W1, h->W4, h->d2));
  // 6. U Q2
  CHK(apply_q(h, h->W3));
  // 7. G = Ur P1 That1^-1 P2 That2^-1 diag(1/d2) (U Q2)^dag
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_conj_transpose(h->W3, h->W1, n, h->st));
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_scale(h->W1, n, n, h->d2, true, nullptr, false, h->st));
  CHK(trsm_left(h, h->W4, h->qr.order, h->W1));
  CHK(permute(h, h->W1, h->W3, h->qr.order, true, true));
  CHK(trsm_left(h, h->W2, h->ord1, h->W3));
  CHK(permute(h, h->W3, h->W1, h->ord1, true, true));
  CHK(gemm(h, 'N', 'N', h->Ur, h->W1, out));
  LAUNCH(DQMC_K_MISC, 0.0, 8.0 * n, launch_sum_log(h->d2, n, h->scal_d, h->st));
  return DQMC_OK;
}

// Y <- T^-1 Y (n x n) in blocks of h->trsm_block rows: FP64 solves of the
// diagonal blocks, the off-diagonal updates as split-BF16 GEMMs.  lower: T
// unit lower triangular (strict lower part), forward; else upper with the
// reciprocal diagonal rdiag, backward.
int trsm_blocked(dqmc_handle* h, const cplx* T, const cplx* rdiag, cplx* Y, bool lower) {
  const int n = h->n, b = h->trsm_block;
  const int nb = (n + b - 1) / b;
  for (int t = 0; t < nb; ++t) {
    const int blk = lower ? t : nb - 1 - t;
    const int j0 = blk * b, bs = (j0 + b <= n) ? b : n - j0;
    LAUNCH(DQMC_K_TRSM, 4.0 * bs * bs * n, 32.0 * bs * n,
           launch_trsm_diag_block(T, n, rdiag, Y, n, j0, bs, n, lower, h->st));
    if (lower && j0 + bs < n) {
      // Y[j0+bs:, :] -= T[j0+bs:, j0:j0+bs] Y[j0:j0+bs, :]
      CHK(zgemm_general(h, n - j0 - bs, n, bs, 'N', 'N', cmake(-1, 0), T + (size_t)j0 * n + j0 + bs, n, Y + j0, n,
                        cmake(1, 0), Y + j0 + bs, n, nullptr, nullptr, true, DQMC_K_TRSM));
    } else if (!lower && j0 > 0) {
      // Y[:j0, :] -= T[:j0, j0:j0+bs] Y[j0:j0+bs, :]
      CHK(zgemm_general(h, j0, n, bs, 'N', 'N', cmake(-1, 0), T + (size_t)j0 * n, n, Y + j0, n, cmake(1, 0), Y, n,
                        nullptr, nullptr, true, DQMC_K_TRSM));
    }
  }
  return DQMC_OK;
}

// zgetrf of A (n x n, in place: L strict lower, U upper) in panels of LU_PB
// columns: panel factorisation with partial pivoting, the panel's row
// exchanges on the other columns, U12 = L11^-1 A12, A22 -= L21 U12 (a GEMM,
// split-BF16 in the mixed form).  lu.perm, lu.udiag, lu.rdiag on return.
// For n <= lu_small the unblocked cooperative LU runs instead (one launch;
// L then in lu_L).  *Lm receives the matrix whose strict lower part is L.
int lu_blocked(dqmc_handle* h, cplx* A, const cplx** Lm) {
  const int n = h->n;
  if (n <= h->lu_small) {
    LUKernel w{h->lu.perm, h->lu.udiag, h->lu.rdiag, h->lu_pivrow, h->qr.bar, h->err_d};
    LAUNCH(DQMC_K_LU, 8.0 * n3(h) / 3.0, 32.0 * n2(h), launch_lup(A, h->lu_L, n, w, h->sm_count, h->st, h->coop_cap));
    *Lm = h->lu_L;
    return DQMC_OK;
  }
  *Lm = A;
  LAUNCH(DQMC_K_LU, 0.0, 4.0 * n, launch_iota(h->lu.perm, n, h->st));
  for (int p0 = 0; p0 < n; p0 += LU_PB) {
    const int b = n - p0 < LU_PB ? n - p0 : LU_PB;
    const int m = n - p0 - b;
    int lu_cap = h->coop_cap;
    if (h->lu_grid > 0 && (lu_cap == 0 || h->lu_grid < lu_cap)) lu_cap = h->lu_grid;
    LAUNCH(DQMC_K_LU, 8.0 * (n - p0) * b * b / 2.0, 32.0 * (n - p0) * b,
           launch_lu_panel(A, n, p0, b, h->lup, h->sm_count, h->st, lu_cap, h->lu_cluster));
    LAUNCH(DQMC_K_LU, 0.0, 64.0 * b * n, launch_lu_apply_swaps(A, n, p0, b, h->lup.piv, h->lu.perm, h->st));
    if (m > 0) {
      LAUNCH(DQMC_K_LU, 4.0 * b * b * m, 32.0 * b * m,
             launch_trsm_diag_block(A, n, nullptr, A + (size_t)(p0 + b) * n, n, p0, b, m, true, h->st));
      CHK(zgemm_general(h, m, m, b, 'N', 'N', cmake(-1, 0), A + (size_t)p0 * n + p0 + b, n,
                        A + (size_t)(p0 + b) * n + p0, n, cmake(1, 0), A + (size_t)(p0 + b) * n + p0 + b, n, nullptr,
                        nullptr, true, DQMC_K_LU));
    }
  }
  LAUNCH(DQMC_K_LU, 0.0, 32.0 * n, launch_lu_diag(A, n, h->lu.udiag, h->lu.rdiag, h->st));
  return DQMC_OK;
}

// D-scale separated calculate_greens: with D = Dmax Dmin, Dmax = max(D, 1),
//   I + Ul Dl Tl Tr^dag Dr Ur^dag = Ul Dlmax M Drmax Ur^dag,
//   M = Dlmax^-1 (Ul^dag Ur) Drmax^-1 + Dlmin (Tl Tr^dag) Drmin,
// whose entries carry no large scales; M = P^T L U by one LU with partial
// pivoting, so G = (Ur Drmax^-1) U^-1 L^-1 P (Dlmax^-1 Ul^dag) and
// log|det G| = -(sum log|U_ii| + sum log Dlmax + sum log Drmax).
int calculate_greens_scales(dqmc_handle* h, cplx* out) {
  const int n = h->n;
  double* s = h->lu_scales;   // [1/Dlmax, Dlmin, 1/Drmax, Drmin]
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n, launch_split_scales(h->Dl, h->Dr, n, s, h->st));
  // M = diag(1/Dlmax) Ul^dag Ur diag(1/Drmax) + diag(Dlmin) Tl Tr^dag diag(Drmin)
  CHK(zgemm_general(h, n, n, n, 'C', 'N', cmake(1, 0), h->Ul, n, h->Ur, n, cmake(0, 0), h->W1, n, s, s + 2 * n, true));
  CHK(zgemm_general(h, n, n, n, 'N', 'C', cmake(1, 0), h->Tl, n, h->Tr, n, cmake(1, 0), h->W1, n, s + n, s + 3 * n,
                    true));
  // P M = L U in place in W1 (L strict lower, U upper; lu.udiag, lu.rdiag, lu.perm)
  const cplx* Lm = nullptr;
  CHK(lu_blocked(h, h->W1, &Lm));
  // right-hand side P diag(1/Dlmax) Ul^dag
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_conj_transpose(h->Ul, h->W4, n, h->st));
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_scale(h->W4, n, n, s, false, nullptr, false, h->st));
  CHK(permute(h, h->W4, h->W3, h->lu.perm, true, false));
  // U^-1 L^-1 (.), then diag(1/Drmax)
  if (h->p.precision == DQMC_PREC_MIXED) {
    CHK(trsm_blocked(h, Lm, nullptr, h->W3, true));
    CHK(trsm_blocked(h, h->W1, h->lu.rdiag, h->W3, false));
  } else {
    LAUNCH(DQMC_K_TRSM, 4.0 * n3(h), 40.0 * n2(h), launch_trsm_left_lower_unit(Lm, h->W3, n, n, h->st));
    LAUNCH(DQMC_K_TRSM, 4.0 * n3(h), 40.0 * n2(h), launch_trsm_left_upper(h->W1, nullptr, h->lu.rdiag, h->W3, n, n,
                                                                           h->st));
  }
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_scale(h->W3, n, n, s + 2 * n, false, nullptr, false, h->st));
  // G = Ur (.)
  CHK(gemm(h, 'N', 'N', h->Ur, h->W3, out));
  // scal_d[0] = -log|det G|, the convention of the two-QR form (sum log d2)
  LAUNCH(DQMC_K_MISC, 0.0, 24.0 * n, launch_lu_logdet(h->lu.udiag, h->Dl, h->Dr, n, h->scal_d, h->st));
  return DQMC_OK;
}

int calculate_greens_into(dqmc_handle* h, cplx* out) {
  return h->greens_method == DQMC_GREENS_TWO_QR ? calculate_greens_two_qr(h, out) : calculate_greens_scales(h, out);
}

int calculate_greens(dqmc_handle* h) { return calculate_greens_into(h, h->G); }

int save_logdet(dqmc_handle* h) {
  // scal_d[0] = sum log d2  ->  scal_d[2] = log_det = -sum log d2
  CU(cudaMemcpyAsync(h->scal_d + 2, h->scal_d, sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  return DQMC_OK;
}

int set_l(dqmc_handle* h, int k) {
  CHK(copy_nn(h, h->Ul, ustk(h, k)));
  CHK(copy_nn(h, h->Tl, tstk(h, k)));
  CU(cudaMemcpyAsync(h->Dl, dstk(h, k), h->n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  return DQMC_OK;
}
int set_r(dqmc_handle* h, int k) {
  CHK(copy_nn(h, h->Ur, ustk(h, k)));
  CHK(copy_nn(h, h->Tr, tstk(h, k)));
  CU(cudaMemcpyAsync(h->Dr, dstk(h, k), h->n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  return DQMC_OK;
}
int stack_identity(dqmc_handle* h, int k) {
  CHK(set_identity(h, ustk(h, k)));
  CHK(set_identity(h, tstk(h, k)));
  CHK(set_ones(h, dstk(h, k)));
  return DQMC_OK;
}

// max |G_wrapped - G_fresh| of this stabilisation folded into the running
// maximum scal_d[3] on the device (read when the call finishes).
int instability_check(dqmc_handle* h) {
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h),
         launch_max_absdiff(h->Gtmp, h->G, (size_t)h->n * h->n, h->scal_d + 3, h->st, false));
  return DQMC_OK;
}

// Reads the running instability maximum (stream must be idle).
int read_instability(dqmc_handle* h) {
  double d = 0.0;
  CU(cudaMemcpyAsync(&d, h->scal_d + 3, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaStreamSynchronize(h->st));
  if (!(d <= h->max_instability)) h->max_instability = d;
  if (!std::isfinite(d)) return set_err(h, DQMC_ERR_NONFINITE, "non-finite Green's function");
  return DQMC_OK;
}

// build_stack (src/stack.jl:251-272)
int build_stack(dqmc_handle* h) {
  CHK(stack_identity(h, 0));
  for (int i = 1; i <= h->ne - 1; ++i) CHK(add_slice_sequence_left(h, i));
  h->current_slice = h->M + 1;
  h->direction = -1;
  return DQMC_OK;
}

// propagate (src/stack.jl:391-499)
int propagate(dqmc_handle* h) {
  const int s = h->s, M = h->M;
  if (h->direction == 1) {
    if (h->current_slice % s == 0) {
      h->current_slice += 1;
      if (h->current_slice == 1) {
        CHK(set_r(h, 0));
        CHK(stack_identity(h, 0));
        CHK(set_l(h, 0));
        CHK(calculate_greens(h));
        CHK(save_logdet(h));
      } else if (h->current_slice > 1 && h->current_slice <= M) {
        int idx = (h->current_slice - 1) / s;
        CHK(set_r(h, idx));
        CHK(add_slice_sequence_left(h, idx));
        CHK(set_l(h, idx));
        if (h->p.all_checks) {
          CHK(copy_nn(h, h->Gtmp, h->G));
          CHK(wrap_greens(h, h->Gtmp, h->current_slice - 1, 1));
        }
        CHK(calculate_greens(h));
        if (h->p.all_checks) CHK(instability_check(h));
      } else {
        CHK(add_slice_sequence_left(h, h->ne - 1));
        h->direction = -1;
        h->current_slice = M + 1;
        return propagate(h);
      }
    } else {
      CHK(wrap_greens(h, h->G, h->current_slice, 1));
      h->current_slice += 1;
    }
  } else {
    if ((h->current_slice - 1) % s == 0) {
      h->current_slice -= 1;
      if (h->current_slice == M) {
        const int e = h->ne - 1;
        CHK(set_l(h, e));
        CHK(stack_identity(h, e));
        CHK(set_r(h, e));
        CHK(calculate_greens(h));
        CHK(save_logdet(h));
        CHK(wrap_greens(h, h->G, h->current_slice + 1, -1));
      } else if (h->current_slice > 0 && h->current_slice < M) {
        int idx = h->current_slice / s + 1;
        CHK(set_l(h, idx - 1));
        CHK(add_slice_sequence_right(h, idx));
        CHK(set_r(h, idx - 1));
        if (h->p.all_checks) CHK(copy_nn(h, h->Gtmp, h->G));
        CHK(calculate_greens(h));
        if (h->p.all_checks) CHK(instability_check(h));
        CHK(wrap_greens(h, h->G, h->current_slice + 1, -1));
      } else {
        CHK(add_slice_sequence_right(h, 1));
        h->direction = 1;
        h->current_slice = 0;
        return propagate(h);
      }
    } else {
      CHK(wrap_greens(h, h->G, h->current_slice, -1));
      h->current_slice -= 1;
    }
  }
  return DQMC_OK;
}

// calc_boson_action (src/action.jl:1-52) on a host copy of the field.
double boson_action_host(const dqmc_handle* h, const std::vector<double>& phi) {
  const int L = h->L, N = h->N, M = h->M;
  const double dt = h->p.delta_tau, c = h->p.c, r = h->p.r, u = h->p.u;
  auto at = [&](int a, int site, int sl) { return phi[(size_t)3 * ((size_t)N * sl + site) + a]; };
  double S = 0.0, St = 0.0, Ss = 0.0, Sm = 0.0;
  for (int sl = 0; sl < M; ++sl)
    for (int x = 0; x < L; ++x)
      for (int y = 0; y < L; ++y) {
        int site = y + L * x;
        int up = (y + 1) % L + L * x, right = y + L * ((x + 1) % L);
        int later = (sl + 1) % M;
        double sq = 0.0;
        for (int a = 0; a < 3; ++a) {
          double v = at(a, site, sl);
          double dtm = v - at(a, site, later);
          double dy = v - at(a, up, sl);
          double dx = v - at(a, right, sl);
          St += dtm * dtm;
          Ss += dy * dy + dx * dx;
          sq += v * v;
        }
        Sm += dt * r / 2.0 * sq + dt * u / 4.0 * sq * sq;
      }
  S = 0.5 / dt * 1.0 / (c * c) * St + dt * 0.5 * Ss + Sm;
  return S;
}

// d S_boson / d phi (src/action.jl:1-52): temporal, spatial (4 neighbours),
// mass and quartic terms.
void boson_gradient_host(const dqmc_handle* h, const std::vector<double>& phi, double* out) {
  const int L = h->L, N = h->N, M = h->M;
  const double dt = h->p.delta_tau, c = h->p.c, r = h->p.r, u = h->p.u;
  auto at = [&](int a, int site, int sl) { return phi[(size_t)3 * ((size_t)N * sl + site) + a]; };
  for (int sl = 0; sl < M; ++sl)
    for (int x = 0; x < L; ++x)
      for (int y = 0; y < L; ++y) {
        const int s = y + L * x;
        const int nbs[4] = {(y + 1) % L + L * x, y + L * ((x + 1) % L), (y - 1 + L) % L + L * x,
                            y + L * ((x - 1 + L) % L)};
        double sq = 0.0;
        for (int a = 0; a < 3; ++a) sq += at(a, s, sl) * at(a, s, sl);
        for (int a = 0; a < 3; ++a) {
          const double v = at(a, s, sl);
          double g = (2 * v - at(a, s, (sl + 1) % M) - at(a, s, (sl - 1 + M) % M)) / (dt * c * c);
          double nsum = 0.0;
          for (int q = 0; q < 4; ++q) nsum += at(a, nbs[q], sl);
          g += dt * (4 * v - nsum);
          g += dt * (r * v + u * sq * v);
          out[(size_t)3 * ((size_t)N * sl + s) + a] = g;
        }
      }
}

// Captured sweeps hold the device addresses of the handle's buffers: they are
// dropped whenever one of those addresses changes.
void clear_graphs(dqmc_handle* h) {
  for (auto& g : h->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  h->graphs.clear();
  ++h->graph_epoch;   // graphs of a batch that hold this chain's launches are stale too
}

int ensure_stream_capacity(dqmc_handle* h, int calls) {
  if (calls <= h->stream_cap) return DQMC_OK;
  clear_graphs(h);
  if (h->delta_d) cudaFree(h->delta_d);
  if (h->unif_d) cudaFree(h->unif_d);
  h->delta_d = nullptr;
  h->unif_d = nullptr;
  h->stream_cap = 0;
  CU(cudaMalloc(&h->delta_d, (size_t)calls * 3 * h->N * sizeof(double)));
  CU(cudaMalloc(&h->unif_d, (size_t)calls * h->N * sizeof(double)));
  h->stream_cap = calls;
  return DQMC_OK;
}

int ensure_out_capacity(dqmc_handle* h, int calls) {
  if (calls <= h->out_cap) return DQMC_OK;
  clear_graphs(h);
  if (h->acc_d) cudaFree(h->acc_d);
  if (h->det_d) cudaFree(h->det_d);
  if (h->pacc_d) cudaFree(h->pacc_d);
  h->acc_d = nullptr; h->det_d = nullptr; h->pacc_d = nullptr;
  h->out_cap = 0;
  CU(cudaMalloc(&h->acc_d, (size_t)calls * h->N));
  CU(cudaMalloc(&h->det_d, (size_t)calls * h->N * sizeof(cplx)));
  CU(cudaMalloc(&h->pacc_d, (size_t)calls * h->N * sizeof(double)));
  h->out_cap = calls;
  return DQMC_OK;
}

// Inside a stream capture: appends a WHILE node whose body is one delayed
// round and its flush followed by k_round_cond, which continues the loop while
// sites of the slice remain (at most max_rounds times).  A slice then runs
// only the rounds that carry work instead of the fixed bound.  Returns
// kWhileRefused, with the capture untouched, when the runtime refuses
// conditional nodes; the caller then captures the fixed round count.
constexpr int kWhileRefused = 1;   // internal: conditional nodes refused (never returned by the ABI)

template <class Round>
int capture_round_loop(dqmc_handle* h, int max_rounds, Round&& round) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  if (cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess || !g) {
    cudaGetLastError();
    h->while_off = true;
    return kWhileRefused;
  }
  cudaGraphConditionalHandle hc;
  if (cudaGraphConditionalHandleCreate(&hc, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
    cudaGetLastError();
    h->while_off = true;
    return kWhileRefused;
  }
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hc;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp) != cudaSuccess) {
    cudaGetLastError();
    h->while_off = true;
    return kWhileRefused;
  }
  CU(cudaStreamUpdateCaptureDependencies(h->st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  if (!h->st_body) CU(cudaStreamCreateWithFlags(&h->st_body, cudaStreamNonBlocking));
  CU(cudaStreamBeginCaptureToGraph(h->st_body, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                   cudaStreamCaptureModeThreadLocal));
  // the body's launches go to st_body; its counts are those of one round
  int64_t c0[DQMC_NKINDS]; double f0[DQMC_NKINDS], b0[DQMC_NKINDS];
  for (int q = 0; q < DQMC_NKINDS; ++q) { c0[q] = h->cnt[q]; f0[q] = h->flops[q]; b0[q] = h->bytes[q]; }
  const int64_t l0 = h->launches;
  cudaStream_t main_st = h->st;
  h->st = h->st_body;
  int rc = round();
  if (rc == DQMC_OK) {
    KSpan ks_(h, DQMC_K_LOCAL, 0.0, 0.0);
    if (launch_round_cond(hc, h->dstate, h->N, max_rounds, h->err_d,
                          reinterpret_cast<unsigned long long*>(h->dstate + 4), h->st) != cudaSuccess)
      rc = set_err(h, DQMC_ERR_CUDA, "round condition launch failed");
  }
  h->st = main_st;
  cudaGraph_t body = nullptr;
  const bool ended = cudaStreamEndCapture(h->st_body, &body) == cudaSuccess;
  if (rc != DQMC_OK) return rc;
  if (!ended) return set_err(h, DQMC_ERR_CUDA, "capture of the round loop body failed");
  for (int q = 0; q < DQMC_NKINDS; ++q) {
    h->body_cnt[q] = h->cnt[q] - c0[q]; h->body_flops[q] = h->flops[q] - f0[q]; h->body_bytes[q] = h->bytes[q] - b0[q];
  }
  h->body_launches = h->launches - l0;
  ++h->capture_while;
  return DQMC_OK;
}

// local_updates (src/local_updates.jl:1-38) on device streams; outputs to
// device arrays (may be null).  delay <= 1: immediate rank-4 updates in one
// cooperative launch.  delay = k > 1: rounds of [local kernel until k accepts
// are pending, flush G += X Y (FP64 or split-BF16 GEMM)]; the
// number of rounds is the bound ceil(N/k) + 1 and rounds with nothing left
// return at once on a device-side flag, so the host never waits.
int local_updates_dev(dqmc_handle* h, const double* delta_dev, const double* unif_dev, uint8_t* acc_dev,
                      cplx* det_dev, double* pacc_dev) {
  if (h->current_slice < 1 || h->current_slice > h->M)
    return set_err(h, DQMC_ERR_STATE, "local_updates needs 1 <= current_slice <= M (call dqmc_init)");
  LocalUpdateArgs a{};
  a.G = h->G;
  a.phi = h->phi;
  a.evtab = h->evtab;
  a.slice0 = h->current_slice - 1;
  a.delta = delta_dev;
  a.unif = unif_dev;
  a.acc_out = acc_dev;
  a.det_out = det_dev;
  a.pacc_out = pacc_dev;
  a.action = h->action_d;
  a.n_acc = h->nacc_d;
  a.Acol = h->Acol;
  a.Brow = h->Brow;
  a.bar = h->bar;
  a.err = h->err_d;
  a.mc = h->mc;
  if (h->delay <= 1) {
    // flops/bytes of the local updates depend on the acceptances; the caller
    // derives them from the accepted count (32 n^2 flops and bytes per accept)
    LAUNCH(DQMC_K_LOCAL, 0.0, 0.0, launch_local_updates(a, h->sm_count, h->st, h->coop_cap));
    return DQMC_OK;
  }
  const int n = h->n, k = h->delay;
  DelayedArgs d{h->Xd, h->Yd, h->dstate, k, h->prep, h->blk, h->pub, {}};
  // mixed form: the delayed kernel cuts the flush's slices at the round's end
  bool presliced = false;
  if (h->p.precision == DQMC_PREC_MIXED) {
    int S = 0, bits = 0;
    if (ozaki_plan(4 * k, h->oz_target, &S, &bits) && ozaki_scratch_bytes(n, n, 4 * k, S) <= h->oz_bytes) {
      d.sl = ozaki_slices(h->oz_scratch, n, n, 4 * k, S, bits);
      presliced = true;
    }
  }
  LAUNCH(DQMC_K_LOCAL, 0.0, 0.0, launch_local_prepare(a, h->prep, h->dstate, h->st));
  const int rounds = (h->N + k - 1) / k + 1;
  auto round = [&]() -> int {
    LAUNCH(DQMC_K_LOCAL, 0.0, 0.0, launch_local_delayed(a, d, h->sm_count, h->st, h->coop_cap));
    // flush G += X Y over the 4p pending columns (p read on the device; no
    // work when p = 0); the next round clears p
    return zgemm_general(h, n, n, 4 * k, 'N', 'T', cmake(1, 0), h->Xd, n, h->Yd, n, cmake(1, 0), h->G, n, nullptr,
                         nullptr, true, DQMC_K_FLUSH, h->dstate + 1, presliced);
  };
  // the WHILE node only for a chain that has the GPU to itself: with chains
  // in flight together (coop_cap > 0) it cost a batch of 64 chains 28% of its
  // throughput (24.4 against 33.6 chain-sweeps/s with the fixed round count)
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CU(cudaStreamIsCapturing(h->st, &cs));
  if (cs == cudaStreamCaptureStatusActive && !h->while_off && h->coop_cap == 0) {
    const int r = capture_round_loop(h, rounds, round);
    if (r != kWhileRefused) return r;
  }
  for (int r = 0; r < rounds; ++r) CHK(round());
  return DQMC_OK;
}

int read_nacc(dqmc_handle* h, int* out) {
  CU(cudaMemcpyAsync(out, h->nacc_d, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CU(cudaStreamSynchronize(h->st));
  return DQMC_OK;
}

void host_model_constants(dqmc_handle* h) { fill_model_const(h->p, h->mc); }

void free_all(dqmc_handle* h) {
  void* ptrs[] = {h->phi, h->evtab, h->G, h->Gtmp, h->u_stack, h->d_stack, h->t_stack, h->Ul, h->Ur, h->Tl,
                  h->Tr, h->Dl, h->Dr, h->W1, h->W2, h->W3, h->W4, h->D1, h->d2, h->ord1, h->qr.vn1,
                  h->qr.vn2, h->qr.order, h->qr.tau, h->qr.beta, h->qr.V, h->qr.bar, h->qr.cand_v, h->qr.cand_q, h->delta_d, h->unif_d,
                  h->acc_d, h->det_d, h->pacc_d, h->action_d, h->nacc_d, h->Acol, h->Brow, h->bar, h->err_d,
                  h->scal_d, h->oz_scratch, h->oz_acc, h->Xd, h->Yd, h->dstate, h->prep, h->blk, h->pub, h->lu.perm, h->lu.udiag, h->lu.rdiag, h->lup.piv, h->lup.cand_rows, h->lup.rowk, h->lu_L, h->lu_pivrow, h->lu_scales, h->wy_v, h->wy_s, h->wy_z, h->wy_t, h->force_d, h->etc_d, h->tdgf_ws, h->tdgf_a, h->tdgf_b, h->gb_u, h->gb_t, h->gb_G, h->gb_d, h->gb_phi, h->gb_evtab};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  clear_graphs(h);
  if (h->done) cudaEventDestroy(h->done);
  for (auto e : h->event_pool) cudaEventDestroy(e);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->st_body) cudaStreamDestroy(h->st_body);
  if (h->st) cudaStreamDestroy(h->st);
}

int upload_nn(dqmc_handle* h, cplx* dst, const double* src) {
  CU(cudaMemcpyAsync(dst, src, nn_bytes(h), cudaMemcpyHostToDevice, h->st));
  return DQMC_OK;
}
int download_nn(dqmc_handle* h, double* dst, const cplx* src) {
  CU(cudaMemcpyAsync(dst, src, nn_bytes(h), cudaMemcpyDeviceToHost, h->st));
  return DQMC_OK;
}

}  // namespace

// Device constants of the model from the ABI parameters (also used by the
// handle-free entry point).
void fill_model_const(const dqmc_params& p, ModelConst& m) {
  m.L = p.L; m.N = p.L * p.L; m.n = 4 * m.N; m.M = p.slices;
  m.dtau = p.delta_tau; m.lambda = p.lambda; m.r = p.r; m.c = p.c; m.u = p.u;
  m.mu[0] = p.mu1; m.mu[1] = p.mu2;
  // t[bond dir, band] = reshape(hoppings, 2, 2): t[0][b] horizontal, t[1][b] vertical
  const double th[2] = {p.hoppings[0], p.hoppings[2]};
  const double tv[2] = {p.hoppings[1], p.hoppings[3]};
  for (int b = 0; b < 2; ++b) {
    // cosh(fac * -t), sinh(fac * -t) with fac = -prefac * dtau (src/hoppings_checkerboard.jl:46-51)
    double ff = -1.0 * p.delta_tau, fh = -0.5 * p.delta_tau;
    m.ch_f[b] = std::cosh(ff * -th[b]); m.sh_f[b] = std::sinh(ff * -th[b]);
    m.cv_f[b] = std::cosh(ff * -tv[b]); m.sv_f[b] = std::sinh(ff * -tv[b]);
    m.ch_h[b] = std::cosh(fh * -th[b]); m.sh_h[b] = std::sinh(fh * -th[b]);
    m.cv_h[b] = std::cosh(fh * -tv[b]); m.sv_h[b] = std::sinh(fh * -tv[b]);
    // chkr_mu = exp(-dtau * -mu), chkr_mu_inv = exp(dtau * -mu) (src/hoppings_checkerboard.jl:122-127)
    double mu = b == 0 ? p.mu1 : p.mu2;
    m.emu[b] = std::exp(-p.delta_tau * -mu);
    m.emu_inv[b] = std::exp(p.delta_tau * -mu);
  }
}

// ===========================================================================
// C ABI
// ===========================================================================
// ---- time-displaced Green's functions (src/fermion_measurements.jl:1343-1523) ----
namespace tdgf {

// Work matrices of one measurement (allocated per call).
struct Work {
  cplx* m[8] = {};            // n x n temporaries
  double* v[4] = {};          // n vectors
  double* s4 = nullptr;       // (4n) split scales
  double* neg = nullptr;      // (n) -1
};

// X <- A^-1 X: LU with partial pivoting of a copy of A, then P, L^-1, U^-1.
int solve_left(dqmc_handle* h, const cplx* A, cplx* X, cplx* wa, cplx* wb) {
  const int n = h->n;
  CHK(copy_nn(h, wa, A));
  const cplx* Lm = nullptr;
  CHK(lu_blocked(h, wa, &Lm));
  CHK(permute(h, X, wb, h->lu.perm, true, false));
  if (h->p.precision == DQMC_PREC_MIXED) {
    CHK(trsm_blocked(h, Lm, nullptr, wb, true));
    CHK(trsm_blocked(h, wa, h->lu.rdiag, wb, false));
  } else {
    LAUNCH(DQMC_K_TRSM, 4.0 * n3(h), 40.0 * n2(h), launch_trsm_left_lower_unit(Lm, wb, n, n, h->st));
    LAUNCH(DQMC_K_TRSM, 4.0 * n3(h), 40.0 * n2(h), launch_trsm_left_upper(wa, nullptr, h->lu.rdiag, wb, n, n, h->st));
  }
  return copy_nn(h, X, wb);
}

int scale(dqmc_handle* h, cplx* A, const double* rs, bool inv_r, const double* cs, bool inv_c) {
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_scale(A, h->n, h->n, rs, inv_r, cs, inv_c, h->st));
  return DQMC_OK;
}
int ctrans(dqmc_handle* h, const cplx* A, cplx* B) {
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_conj_transpose(A, B, h->n, h->st));
  return DQMC_OK;
}
int diag_of(dqmc_handle* h, cplx* X, const double* d, bool inv) {   // X = diag(d) or diag(1/d)
  CHK(set_identity(h, X));
  return scale(h, X, d, inv, nullptr, false);
}

// calc_Bchain_udts! (src/fermion_measurements.jl:1411-1488) into us/ds/ts
// (nr entries each, in the reference's order after its reverse for RIGHT).
int bchain_udts(dqmc_handle* h, Work& w, bool invert, bool right, cplx* us, double* ds, cplx* ts) {
  const int n = h->n, s = h->s, nr = h->M / h->s;
  const size_t nn = (size_t)n * n;
  const bool rightmult = (right && !invert) || (!right && invert);
  const int mode = !invert ? (right ? SLICE_RIGHT_B : SLICE_LEFT_B) : (right ? SLICE_LEFT_BINV : SLICE_RIGHT_BINV);
  const bool rows = mode == SLICE_RIGHT_B || mode == SLICE_RIGHT_BINV;
  cplx* cur = w.m[0];
  cplx* tmp = w.m[1];
  for (int i = 0; i < nr; ++i) {
    const int ridx = right ? nr - 1 - i : i;          // range processed
    const int pos = right ? nr - 1 - i : i;           // slot after the reverse
    const int prev = right ? pos + 1 : pos - 1;
    if (i == 0) CHK(set_identity(h, cur));
    else CHK(copy_nn(h, cur, rightmult ? ts + (size_t)prev * nn : us + (size_t)prev * nn));
    const int first0 = right ? (ridx + 1) * s - 1 : ridx * s, step = right ? -1 : 1;
    if (rows) CHK(apply_rows(h, cur, first0, s, step, mode));
    else CHK(apply_cols(h, cur, first0, s, step, mode, nullptr));
    if (i != 0) {
      const double* dp = ds + (size_t)prev * n;
      CHK(rightmult ? scale(h, cur, dp, false, nullptr, false) : scale(h, cur, nullptr, false, dp, false));
    }
    cplx* u = us + (size_t)pos * nn;
    cplx* t = ts + (size_t)pos * nn;
    double* d = ds + (size_t)pos * n;
    if (!rightmult) {
      CHK(decompose_udt(h, cur, u, d, tmp));
      if (i == 0) CHK(copy_nn(h, t, tmp));
      else CHK(gemm(h, 'N', 'N', tmp, ts + (size_t)prev * nn, t));
    } else {
      CHK(decompose_udt(h, cur, tmp, d, t));
      if (i == 0) CHK(copy_nn(h, u, tmp));
      else CHK(gemm(h, 'N', 'N', us + (size_t)prev * nn, tmp, u));
    }
  }
  return DQMC_OK;
}

// inv_one_plus_udt_scalettar! (src/linalg.jl:310-339): res = [1 + U D T]^-1
int inv_one_plus_udt(dqmc_handle* h, Work& w, const cplx* U, const double* D, const cplx* T, cplx* res) {
  const int n = h->n;
  cplx *l = w.m[2], *r = w.m[3], *u = w.m[4], *t = w.m[5], *wa = w.m[6], *wb = w.m[7];
  double* s = w.s4;   // [1/max(D,1), min(D,1), ...]
  double* d = w.v[0];
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n, launch_split_scales(D, D, n, s, h->st));
  CHK(diag_of(h, l, s, false));                       // l = T \ Diagonal(1/Dp)
  CHK(solve_left(h, T, l, wa, wb));
  CHK(copy_nn(h, r, U));                              // r = U Diagonal(Dm) + l
  CHK(scale(h, r, nullptr, false, s + n, false));
  LAUNCH(DQMC_K_MISC, 0.0, 48.0 * n2(h), launch_add(r, l, r, (size_t)n * n, h->st));
  CHK(decompose_udt(h, r, u, d, t));                  // r = u d t
  CHK(diag_of(h, r, d, true));                        // r = t \ Diagonal(1/d)
  CHK(solve_left(h, t, r, wa, wb));
  CHK(gemm(h, 'N', 'C', r, u, l));                    // l = r u'
  CHK(scale(h, l, s, false, nullptr, false));         // l = Diagonal(1/Dp) l
  CHK(decompose_udt(h, l, u, d, t));                  // l = u d t
  CHK(copy_nn(h, l, u));                              // l = T \ u
  CHK(solve_left(h, T, l, wa, wb));
  CHK(scale(h, l, nullptr, false, d, false));         // l = l Diagonal(d)
  return gemm(h, 'N', 'N', l, t, res);                // res = l t
}

// inv_sum_udts_scalettar! (src/linalg.jl:512-567): res = [Ua Da Ta + Ub Db Tb]^-1
int inv_sum_udts(dqmc_handle* h, Work& w, const cplx* Ua, const double* Da, const cplx* Ta, const cplx* Ub,
                 const double* Db, const cplx* Tb, cplx* res) {
  const int n = h->n;
  cplx *m1 = w.m[2], *m2 = w.m[3], *u = w.m[4], *t = w.m[5], *wa = w.m[6], *wb = w.m[7];
  double* s = w.s4;   // [1/Dap, Dam, 1/Dbp, Dbm]
  double* d = w.v[0];
  LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n, launch_split_scales(Da, Db, n, s, h->st));
  // mat1 = Ta / Tb = (Tb' \ Ta')'
  CHK(ctrans(h, Ta, m2));
  CHK(ctrans(h, Tb, u));
  CHK(solve_left(h, u, m2, wa, wb));
  CHK(ctrans(h, m2, m1));
  CHK(scale(h, m1, s + n, false, s + 2 * n, false));  // Dam[j] / Dbp[k]
  // mat2 = Diagonal(1/Dap) Ua' Ub Diagonal(Dbm); mat1 += mat2
  CHK(zgemm_general(h, n, n, n, 'C', 'N', cmake(1, 0), Ua, n, Ub, n, cmake(0, 0), m2, n, s, s + 3 * n, true));
  LAUNCH(DQMC_K_MISC, 0.0, 48.0 * n2(h), launch_add(m1, m2, m1, (size_t)n * n, h->st));
  CHK(decompose_udt(h, m1, u, d, t));                 // mat1 = U D T
  CHK(scale(h, t, d, false, nullptr, false));         // T = Diagonal(D) T
  CHK(ctrans(h, u, m1));                              // mat1 = T \ U'
  CHK(solve_left(h, t, m1, wa, wb));
  CHK(scale(h, m1, s + 2 * n, false, s, false));      // mat1 / Dbp[j] / Dap[k]
  CHK(decompose_udt(h, m1, u, d, t));                 // mat1 = U D T
  CHK(copy_nn(h, m1, u));                             // mat1 = Tb \ U
  CHK(solve_left(h, Tb, m1, wa, wb));
  CHK(gemm(h, 'N', 'C', t, Ua, m2));                  // mat2 = T Ua'
  CHK(scale(h, m1, nullptr, false, d, false));        // res = (mat1 Diagonal(D)) mat2
  return gemm(h, 'N', 'N', m1, m2, res);
}

int effective_to_true(dqmc_handle* h, cplx* G) {
  CHK(apply_rows(h, G, 0, 1, 1, SLICE_EFF_RIGHT));
  return apply_cols(h, G, 0, 1, 1, SLICE_EFF_LEFT_INV, nullptr);
}

// measure_tdgfs! (src/fermion_measurements.jl:1343-1403) into device arrays
// Gt0 and G0t of M n x n matrices (slice tau at offset (tau-1) n^2).
int measure(dqmc_handle* h, cplx* Gt0, cplx* G0t) {
  const int n = h->n, s = h->s, M = h->M, nr = M / s;
  const size_t nn = (size_t)n * n;
  Work w;
  cplx* st_u[4] = {}; cplx* st_t[4] = {}; double* st_d[4] = {};
  // one block, carved in the same order on every call: 8 work matrices, 4 + 4 + 1
  // vectors, and the four B-chain stacks (U, T, D); allocated once per handle
  size_t off = 0;
  std::vector<std::pair<void**, size_t>> parts;
  for (int k = 0; k < 8; ++k) parts.push_back({(void**)&w.m[k], nn * sizeof(cplx)});
  for (int k = 0; k < 4; ++k) parts.push_back({(void**)&w.v[k], n * sizeof(double)});
  parts.push_back({(void**)&w.s4, 4 * n * sizeof(double)});
  parts.push_back({(void**)&w.neg, n * sizeof(double)});
  for (int k = 0; k < 4; ++k) {
    parts.push_back({(void**)&st_u[k], nr * nn * sizeof(cplx)});
    parts.push_back({(void**)&st_t[k], nr * nn * sizeof(cplx)});
    parts.push_back({(void**)&st_d[k], (size_t)nr * n * sizeof(double)});
  }
  for (auto& pt : parts) off += (pt.second + 255) / 256 * 256;
  if (!h->tdgf_ws && cudaMalloc(&h->tdgf_ws, off) != cudaSuccess) {
    h->tdgf_ws = nullptr;
    return DQMC_ERR_CUDA;
  }
  off = 0;
  for (auto& pt : parts) {
    *pt.first = static_cast<char*>(h->tdgf_ws) + off;
    off += (pt.second + 255) / 256 * 256;
  }
  int rc = DQMC_OK;
  auto body = [&]() -> int {
    // stacks: 0 = B(tau,1)^-1 (LEFT, inverse), 1 = B(beta,tau) (RIGHT), 2 = B(tau,1) (LEFT), 3 = B(beta,tau)^-1 (RIGHT, inverse)
    CHK(bchain_udts(h, w, true, false, st_u[0], st_d[0], st_t[0]));
    CHK(bchain_udts(h, w, false, true, st_u[1], st_d[1], st_t[1]));
    CHK(bchain_udts(h, w, false, false, st_u[2], st_d[2], st_t[2]));
    CHK(bchain_udts(h, w, true, true, st_u[3], st_d[3], st_t[3]));
    auto U = [&](int k, int i) { return st_u[k] + (size_t)i * nn; };
    auto T = [&](int k, int i) { return st_t[k] + (size_t)i * nn; };
    auto D = [&](int k, int i) { return st_d[k] + (size_t)i * n; };
    for (int i = 0; i < nr; ++i) {
      const int tau = 1 + i * s;
      cplx* g1 = Gt0 + (size_t)(tau - 1) * nn;
      cplx* g2 = G0t + (size_t)(tau - 1) * nn;
      if (i != 0) {
        CHK(inv_sum_udts(h, w, U(0, i - 1), D(0, i - 1), T(0, i - 1), U(1, i), D(1, i), T(1, i), g1));
        CHK(inv_sum_udts(h, w, U(2, i - 1), D(2, i - 1), T(2, i - 1), U(3, i), D(3, i), T(3, i), g2));
      } else {
        CHK(inv_one_plus_udt(h, w, U(1, 0), D(1, 0), T(1, 0), g1));
        CHK(inv_one_plus_udt(h, w, U(3, 0), D(3, 0), T(3, 0), g2));
      }
      CHK(effective_to_true(h, g1));
      CHK(effective_to_true(h, g2));
    }
    // fill_tdgf! (src/fermion_measurements.jl:1497-1523)
    const int Mhalf = M / 2 + 1;
    for (int tau = Mhalf; tau <= M; ++tau) {
      if ((tau - 1) % s == 0) continue;
      cplx* a = Gt0 + (size_t)(tau - 1) * nn;
      cplx* b = G0t + (size_t)(tau - 1) * nn;
      CHK(copy_nn(h, a, a - nn));
      CHK(apply_cols(h, a, tau - 1, 1, 1, SLICE_LEFT_B, nullptr));
      CHK(copy_nn(h, b, b - nn));
      CHK(apply_rows(h, b, tau - 1, 1, 1, SLICE_RIGHT_BINV));
    }
    for (int tau = Mhalf - 1; tau >= 1; --tau) {
      if ((tau - 1) % s == 0) continue;
      cplx* a = Gt0 + (size_t)(tau - 1) * nn;
      cplx* b = G0t + (size_t)(tau - 1) * nn;
      CHK(copy_nn(h, a, a + nn));
      CHK(apply_cols(h, a, tau, 1, 1, SLICE_LEFT_BINV, nullptr));
      CHK(copy_nn(h, b, b + nn));
      CHK(apply_rows(h, b, tau, 1, 1, SLICE_RIGHT_B));
    }
    // G0t *= -1
    LAUNCH(DQMC_K_MISC, 0.0, 8.0 * n, launch_fill(w.neg, n, -1.0, h->st));
    LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h) * M,
           launch_scale(G0t, n, (int)((size_t)n * M), w.neg, false, nullptr, false, h->st));
    return DQMC_OK;
  };
  // zero blocks as allocate_tdgfs! (src/fermion_measurements.jl:1247-1248):
  // when M/2 is not a multiple of safe_mult, fill_tdgf! propagates from a
  // slice it has not filled yet, which the reference holds as zeros
  if (rc == DQMC_OK && (cudaMemsetAsync(Gt0, 0, (size_t)M * nn * sizeof(cplx), h->st) != cudaSuccess ||
                        cudaMemsetAsync(G0t, 0, (size_t)M * nn * sizeof(cplx), h->st) != cudaSuccess))
    rc = DQMC_ERR_CUDA;
  if (rc == DQMC_OK) rc = body();
  return rc;
}

// G(tau, 0) and G(0, tau) buffers of the handle for host or absent outputs
int output_buffers(dqmc_handle* h, cplx** a, cplx** b) {
  const size_t bytes = (size_t)h->M * h->n * h->n * sizeof(cplx);
  if (!h->tdgf_a && cudaMalloc(&h->tdgf_a, bytes) != cudaSuccess) { h->tdgf_a = nullptr; return DQMC_ERR_CUDA; }
  if (!h->tdgf_b && cudaMalloc(&h->tdgf_b, bytes) != cudaSuccess) { h->tdgf_b = nullptr; return DQMC_ERR_CUDA; }
  *a = h->tdgf_a;
  *b = h->tdgf_b;
  return DQMC_OK;
}

}  // namespace tdgf

static bool all_device_accessible(std::initializer_list<const void*> ps) {
  for (const void* p : ps)
    if (!device_accessible(p)) return false;
  return true;
}

// The measurement hook's true G of the current slice into dst:
// wrap_greens(G, current_slice, +1), then effective -> true
// (src/dqmc_framework.jl:378-381, src/fermion_measurements.jl:1125-1142).

static int hook_true_greens(dqmc_handle* h, cplx* dst) {
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  if (h->current_slice < 1 || h->current_slice > h->M) return set_err(h, DQMC_ERR_STATE, "no current slice");
  CHK(copy_nn(h, dst, h->G));
  CHK(wrap_greens(h, dst, h->current_slice, 1));
  CHK(apply_rows(h, dst, 0, 1, 1, SLICE_EFF_RIGHT));
  return apply_cols(h, dst, 0, 1, 1, SLICE_EFF_LEFT_INV, nullptr);
}

extern "C" {

const char* dqmc_version(void) { return DQMC_VERSION_STRING; }

const char* dqmc_last_error(const dqmc_handle* h) { return h ? h->last_error.c_str() : "null handle"; }

int dqmc_create(const dqmc_params* p, dqmc_handle** out) {
  if (!p || !out) return DQMC_ERR_ARG;
  *out = nullptr;
  if (p->L < 2 || p->L % 2 != 0) return DQMC_ERR_ARG;                 // CBAssaad needs even L
  if (p->slices < 1 || p->safe_mult < 1 || p->slices % p->safe_mult != 0) return DQMC_ERR_ARG;
  if (p->opdim != 3) return DQMC_ERR_ARG;
  if (p->precision != DQMC_PREC_FP64 && p->precision != DQMC_PREC_MIXED) return DQMC_ERR_ARG;
  if (p->ozaki_bits < 0 || p->ozaki_bits > 60 || p->delay < 0 || p->delay > 64) return DQMC_ERR_ARG;
  if (4 * p->L * p->L > 1024) return DQMC_ERR_ARG;                     // register-resident QR columns
  if (p->device >= 0 && cudaSetDevice(p->device) != cudaSuccess) return DQMC_ERR_CUDA;
  dqmc_handle* h = new dqmc_handle();
  h->p = *p;
  if (const char* tune = std::getenv("DQMC_TUNE")) {
    int v = 0;
    if (const char* q = std::strstr(tune, "wy=")) if (std::sscanf(q + 3, "%d", &v) == 1 && v >= 16 && v <= kWyMax) h->wy_block = v;
    if (const char* q = std::strstr(tune, "trsm=")) if (std::sscanf(q + 5, "%d", &v) == 1 && v >= 16 && v <= 128) h->trsm_block = v;
    if (const char* q = std::strstr(tune, "lu_grid=")) if (std::sscanf(q + 8, "%d", &v) == 1 && v >= 0) h->lu_grid = v;
    if (const char* q = std::strstr(tune, "lu_small=")) if (std::sscanf(q + 9, "%d", &v) == 1 && v >= 0) h->lu_small = v;
    if (const char* q = std::strstr(tune, "lu_cluster=")) if (std::sscanf(q + 11, "%d", &v) == 1 && (v == 0 || v == 8 || v == 16)) h->lu_cluster = v;
  }
  h->L = p->L; h->N = p->L * p->L; h->n = 4 * h->N; h->M = p->slices; h->s = p->safe_mult;
  h->ne = h->M / h->s + 1;
  host_model_constants(h);
  auto fail = [&](int code) { free_all(h); delete h; return code; };
  if (cudaGetDevice(&h->device) != cudaSuccess) return fail(DQMC_ERR_CUDA);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess) return fail(DQMC_ERR_CUDA);
  h->sm_count = prop.multiProcessorCount;
  if (!prop.cooperativeLaunch) return fail(DQMC_ERR_CUDA);
  // inflight > 1 on a single chain: cooperative grids capped as for one of
  // that many chains sharing the GPU (a batch chain's launch shapes)
  if (p->inflight > 1) h->coop_cap = h->sm_count / p->inflight > 0 ? h->sm_count / p->inflight : 1;
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) return fail(DQMC_ERR_CUDA);
  const size_t n = h->n, N = h->N, M = h->M, ne = h->ne;
  const size_t nn = n * n * sizeof(cplx);
  bool ok = true;
  auto A = [&](void** ptr, size_t bytes) {
    if (ok && cudaMalloc(ptr, bytes) != cudaSuccess) ok = false;
    if (ok) cudaMemset(*ptr, 0, bytes);
  };
  A((void**)&h->phi, 3 * N * M * sizeof(double));
  A(&h->evtab, N * M * evtab_entry_bytes());
  A((void**)&h->G, nn); A((void**)&h->Gtmp, nn);
  A((void**)&h->u_stack, ne * nn); A((void**)&h->t_stack, ne * nn);
  A((void**)&h->d_stack, ne * n * sizeof(double));
  A((void**)&h->Ul, nn); A((void**)&h->Ur, nn); A((void**)&h->Tl, nn); A((void**)&h->Tr, nn);
  A((void**)&h->Dl, n * sizeof(double)); A((void**)&h->Dr, n * sizeof(double));
  A((void**)&h->W1, nn); A((void**)&h->W2, nn); A((void**)&h->W3, nn); A((void**)&h->W4, nn);
  A((void**)&h->D1, n * sizeof(double)); A((void**)&h->d2, n * sizeof(double));
  A((void**)&h->ord1, n * sizeof(int));
  A((void**)&h->qr.vn1, 2 * n * sizeof(double)); A((void**)&h->qr.vn2, 2 * n * sizeof(double));
  A((void**)&h->qr.order, n * sizeof(int)); A((void**)&h->qr.tau, n * sizeof(cplx));
  A((void**)&h->qr.beta, n * sizeof(double)); A((void**)&h->qr.V, nn);
  A((void**)&h->qr.bar, sizeof(GridBarrier));
  A((void**)&h->qr.cand_v, 1024 * sizeof(double)); A((void**)&h->qr.cand_q, 1024 * sizeof(int));
  A((void**)&h->action_d, sizeof(double)); A((void**)&h->nacc_d, 2 * sizeof(int));
  A((void**)&h->Acol, 4 * n * sizeof(cplx)); A((void**)&h->Brow, 4 * n * sizeof(cplx));
  A((void**)&h->bar, sizeof(GridBarrier)); A((void**)&h->err_d, sizeof(int));
  A((void**)&h->scal_d, 8 * sizeof(double));
  h->greens_method = p->greens_method == DQMC_GREENS_TWO_QR ? DQMC_GREENS_TWO_QR : DQMC_GREENS_SCALES;
  A((void**)&h->lu.perm, n * sizeof(int)); A((void**)&h->lu.udiag, n * sizeof(cplx));
  A((void**)&h->lu.rdiag, n * sizeof(cplx));
  A((void**)&h->lu_scales, 4 * n * sizeof(double));
  A((void**)&h->lu_L, n * n * sizeof(cplx)); A((void**)&h->lu_pivrow, 2 * sizeof(int));
  A((void**)&h->lup.piv, n * sizeof(int));
  A((void**)&h->lup.cand_rows, (size_t)1024 * LU_PB * sizeof(cplx));
  A((void**)&h->lup.rowk, (size_t)2 * LU_PB * sizeof(cplx));
  h->lup.cand_v = h->qr.cand_v;
  h->lup.cand_r = h->qr.cand_q;
  h->lup.bar = h->qr.bar;
  h->lup.err = h->err_d;
  h->delay = p->delay > 1 ? p->delay : 1;
  if (h->delay > 1) {
    A((void**)&h->Xd, (size_t)4 * h->delay * n * sizeof(cplx));
    A((void**)&h->Yd, (size_t)4 * h->delay * n * sizeof(cplx));
    A((void**)&h->dstate, 8 * sizeof(int));   // [0] next site, [1] pending, [2] rounds, [4..5] u64 rounds run
    A((void**)&h->prep, (size_t)h->N * sizeof(SitePrep));
    A((void**)&h->blk, (size_t)16 * h->N * sizeof(cplx));
    A((void**)&h->pub, (size_t)h->N * sizeof(int));
  }
  if (p->precision == DQMC_PREC_MIXED) {
    A((void**)&h->wy_v, (size_t)n * kWyMax * sizeof(cplx));
    A((void**)&h->wy_s, (size_t)kWyMax * kWyMax * sizeof(cplx));
    A((void**)&h->wy_z, (size_t)kWyMax * n * sizeof(cplx));
    A((void**)&h->wy_t, (size_t)kWyMax * sizeof(cplx));
    h->oz_target = p->ozaki_bits > 0 ? p->ozaki_bits : 40;
    // the largest products are n x n x n; the flush (K = 4k) needs fewer slices
    int S = 0, bits = 0;
    if (!ozaki_plan((int)n, h->oz_target, &S, &bits)) return fail(DQMC_ERR_ARG);
    size_t need = ozaki_scratch_bytes((int)n, (int)n, (int)n, S);
    if (h->delay > 1 && ozaki_plan(4 * h->delay, h->oz_target, &S, &bits)) {
      size_t f = ozaki_scratch_bytes((int)n, (int)n, 4 * h->delay, S);
      if (f > need) need = f;
    }
    h->oz_bytes = need;
    A(&h->oz_scratch, h->oz_bytes);
    // split K is taken for fewer than sm_count / 2 output tiles of 64 x 64
    const size_t tiles = (size_t)(h->sm_count / 2 + 1);
    h->oz_acc_bytes = std::min((size_t)n * n, tiles * 64 * 64) * 2 * sizeof(unsigned long long);
    A((void**)&h->oz_acc, h->oz_acc_bytes);
  }
  if (!ok) return fail(DQMC_ERR_CUDA);
  h->qr.err = h->err_d;
  if (cudaDeviceSynchronize() != cudaSuccess) return fail(DQMC_ERR_CUDA);
  *out = h;
  return DQMC_OK;
}

int dqmc_destroy(dqmc_handle* h) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  cudaStreamSynchronize(h->st);
  free_all(h);
  delete h;
  return DQMC_OK;
}

int dqmc_set_field(dqmc_handle* h, const double* phi) {
  if (h) cudaSetDevice(h->device);
  if (!h || !phi) return DQMC_ERR_ARG;
  CU(cudaMemcpyAsync(h->phi, phi, (size_t)3 * h->N * h->M * sizeof(double), cudaMemcpyHostToDevice, h->st));
  LAUNCH(DQMC_K_MISC, 0.0, 56.0 * h->N * h->M,
         launch_build_evtab(h->phi, h->evtab, h->N, h->M, h->p.lambda * h->p.delta_tau, h->st));
  h->initialized = false;
  return sync(h);
}

int dqmc_get_field(dqmc_handle* h, double* phi) {
  if (h) cudaSetDevice(h->device);
  if (!h || !phi) return DQMC_ERR_ARG;
  CU(cudaMemcpyAsync(phi, h->phi, (size_t)3 * h->N * h->M * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  return sync(h);
}

int dqmc_init(dqmc_handle* h) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  std::vector<double> phi((size_t)3 * h->N * h->M);
  CU(cudaMemcpyAsync(phi.data(), h->phi, phi.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaStreamSynchronize(h->st));
  double S = boson_action_host(h, phi);
  CU(cudaMemcpyAsync(h->action_d, &S, sizeof(double), cudaMemcpyHostToDevice, h->st));
  CU(cudaMemsetAsync(h->nacc_d, 0, sizeof(int), h->st));
  h->max_instability = 0.0;
  CU(cudaMemsetAsync(h->scal_d + 3, 0, sizeof(double), h->st));
  CHK(build_stack(h));
  CHK(propagate(h));
  h->initialized = true;
  return sync(h);
}

int dqmc_propagate(dqmc_handle* h) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  CHK(propagate(h));
  return sync(h);
}

int dqmc_get_state(dqmc_handle* h, int32_t* slice, int32_t* direction) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  if (slice) *slice = h->current_slice;
  if (direction) *direction = h->direction;
  return DQMC_OK;
}

static int local_updates_host(dqmc_handle* h, const double* delta, const double* unif, uint8_t* accepted,
                              double* detratio, double* p_acc, double* acc_rate) {
  if (!delta || !unif) return set_err(h, DQMC_ERR_ARG, "delta and unif are required");
  CHK(ensure_stream_capacity(h, 1));
  CHK(ensure_out_capacity(h, 1));
  CU(cudaMemcpyAsync(h->delta_d, delta, (size_t)3 * h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CU(cudaMemcpyAsync(h->unif_d, unif, (size_t)h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
  int before = 0;
  CHK(read_nacc(h, &before));
  CHK(local_updates_dev(h, h->delta_d, h->unif_d, h->acc_d, h->det_d, h->pacc_d));
  if (accepted) CU(cudaMemcpyAsync(accepted, h->acc_d, h->N, cudaMemcpyDeviceToHost, h->st));
  if (detratio) CU(cudaMemcpyAsync(detratio, h->det_d, h->N * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
  if (p_acc) CU(cudaMemcpyAsync(p_acc, h->pacc_d, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CHK(sync(h));
  if (acc_rate) {
    int after = 0;
    CHK(read_nacc(h, &after));
    *acc_rate = (double)(after - before) / h->N;
  }
  return DQMC_OK;
}

int dqmc_local_updates(dqmc_handle* h, const double* delta, const double* unif, uint8_t* accepted,
                       double* detratio, double* p_acc, double* acc_rate) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  return local_updates_host(h, delta, unif, accepted, detratio, p_acc, acc_rate);
}

int dqmc_update(dqmc_handle* h, const double* delta, const double* unif, uint8_t* accepted, double* detratio,
                double* p_acc, double* acc_rate) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  CHK(propagate(h));
  return local_updates_host(h, delta, unif, accepted, detratio, p_acc, acc_rate);
}

// Enqueues n_calls update() calls on the handle's stream without waiting.
// n_calls update() calls (propagate + local updates) enqueued on the stream.
static int sweep_body(dqmc_handle* h, int n_calls, const double* delta_dev, const double* unif_dev,
                      uint8_t* acc_dev) {
  const size_t N = h->N;
  for (int c = 0; c < n_calls; ++c) {
    CHK(propagate(h));
    CHK(local_updates_dev(h, delta_dev + (size_t)c * 3 * N, unif_dev + (size_t)c * N,
                          acc_dev ? acc_dev + (size_t)c * N : nullptr, nullptr, nullptr));
  }
  return DQMC_OK;
}

// Captures the sweep from the current state into a CUDA graph (streams in the
// handle's own buffers).  The host state is left as before the capture (no
// work has run); the caller launches the graph and moves the state to the
// graph's end state.  Returns null (and stops trying) if capture is refused.
static dqmc_handle::SweepGraph* capture_sweep(dqmc_handle* h, int n_calls, bool acc) {
  dqmc_handle::SweepGraph g;
  g.slice0 = h->current_slice; g.dir0 = h->direction; g.n_calls = n_calls; g.acc = acc ? 1 : 0;
  int64_t cnt0[DQMC_NKINDS]; double fl0[DQMC_NKINDS], by0[DQMC_NKINDS];
  for (int k = 0; k < DQMC_NKINDS; ++k) { cnt0[k] = h->cnt[k]; fl0[k] = h->flops[k]; by0[k] = h->bytes[k]; }
  const int64_t l0 = h->launches;
  cudaGetLastError();
  h->capture_while = 0;
  bool ok = cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  int rc = DQMC_OK;
  cudaGraph_t graph = nullptr;
  if (ok) {
    rc = sweep_body(h, n_calls, h->delta_d, h->unif_d, acc ? h->acc_d : nullptr);
    ok = cudaStreamEndCapture(h->st, &graph) == cudaSuccess && rc == DQMC_OK && graph;
  }
  if (ok) ok = cudaGraphInstantiate(&g.exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  g.slice1 = h->current_slice; g.dir1 = h->direction;
  for (int k = 0; k < DQMC_NKINDS; ++k) {
    g.cnt[k] = h->cnt[k] - cnt0[k]; g.flops[k] = h->flops[k] - fl0[k]; g.bytes[k] = h->bytes[k] - by0[k];
    h->cnt[k] = cnt0[k]; h->flops[k] = fl0[k]; h->bytes[k] = by0[k];
  }
  g.launches = h->launches - l0;
  g.while_nodes = h->capture_while;
  h->launches = l0;
  h->current_slice = g.slice0; h->direction = g.dir0;
  cudaGetLastError();
  if (!ok) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    h->graphs_off = true;
    h->last_error.clear();
    return nullptr;
  }
  h->graphs.push_back(g);
  return &h->graphs.back();
}

static int sweep_enqueue(dqmc_handle* h, int n_calls, const double* delta_dev, const double* unif_dev,
                         uint8_t* acc_dev) {
  // graphs need the streams at fixed addresses: reserve before the first event
  const bool graphed = !h->timing && !h->graphs_off;
  if (graphed) {
    CHK(ensure_stream_capacity(h, n_calls));
    if (acc_dev) CHK(ensure_out_capacity(h, n_calls));
  }
  CU(cudaMemcpyAsync(h->nacc_d + 1, h->nacc_d, sizeof(int), cudaMemcpyDeviceToDevice, h->st));
  CU(cudaMemsetAsync(h->scal_d + 3, 0, sizeof(double), h->st));
  h->max_instability = 0.0;
  if (!h->ev0) {
    CU(cudaEventCreate(&h->ev0));
    CU(cudaEventCreate(&h->ev1));
  }
  CU(cudaEventRecord(h->ev0, h->st));
  dqmc_handle::SweepGraph* g = nullptr;
  if (graphed) {
    const size_t N = h->N;
    if (delta_dev != h->delta_d)
      CU(cudaMemcpyAsync(h->delta_d, delta_dev, (size_t)n_calls * 3 * N * sizeof(double), cudaMemcpyDeviceToDevice,
                         h->st));
    if (unif_dev != h->unif_d)
      CU(cudaMemcpyAsync(h->unif_d, unif_dev, (size_t)n_calls * N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    for (auto& x : h->graphs)
      if (x.slice0 == h->current_slice && x.dir0 == h->direction && x.n_calls == n_calls &&
          x.acc == (acc_dev ? 1 : 0))
        g = &x;
    if (!g) g = capture_sweep(h, n_calls, acc_dev != nullptr);
  }
  h->pending_while = 0;
  if (g) {
    CU(cudaGraphLaunch(g->exec, h->st));
    h->pending_while = g->while_nodes;
    h->current_slice = g->slice1;
    h->direction = g->dir1;
    for (int k = 0; k < DQMC_NKINDS; ++k) { h->cnt[k] += g->cnt[k]; h->flops[k] += g->flops[k]; h->bytes[k] += g->bytes[k]; }
    h->launches += g->launches;
    if (acc_dev && acc_dev != h->acc_d)
      CU(cudaMemcpyAsync(acc_dev, h->acc_d, (size_t)n_calls * h->N, cudaMemcpyDeviceToDevice, h->st));
  } else {
    CHK(sweep_body(h, n_calls, delta_dev, unif_dev, acc_dev));
  }
  CU(cudaEventRecord(h->ev1, h->st));
  h->pending_calls = n_calls;
  return DQMC_OK;
}

// Waits for an enqueued sweep and fills the statistics.
static int sweep_finish(dqmc_handle* h, dqmc_stats* stats) {
  CHK(sync(h));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  int cnt[2] = {0, 0};
  unsigned long long rounds = 0;
  CU(cudaMemcpyAsync(cnt, h->nacc_d, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  if (h->pending_while > 0)
    CU(cudaMemcpyAsync(&rounds, h->dstate + 4, sizeof(rounds), cudaMemcpyDeviceToHost, h->st));
  CU(cudaStreamSynchronize(h->st));
  if (h->pending_while > 0) {
    // the graph's counts hold one round body per WHILE node (a WHILE node
    // runs its body at least once): add the rounds that ran beyond those
    const int64_t extra = (int64_t)(rounds - h->rounds_seen) - h->pending_while;
    h->rounds_seen = rounds;
    for (int q = 0; q < DQMC_NKINDS; ++q) {
      h->cnt[q] += extra * h->body_cnt[q];
      h->flops[q] += (double)extra * h->body_flops[q];
      h->bytes[q] += (double)extra * h->body_bytes[q];
    }
    h->launches += extra * h->body_launches;
    h->pending_while = 0;
  }
  if (stats) {
    stats->proposals = (int64_t)h->pending_calls * h->N;
    stats->accepted = cnt[0] - cnt[1];
    stats->acc_rate = stats->proposals ? (double)stats->accepted / stats->proposals : 0.0;
    stats->max_instability = h->max_instability;
    stats->device_ms = ms;
  }
  h->pending_calls = 0;
  return DQMC_OK;
}

static int sweep_impl(dqmc_handle* h, int n_calls, const double* delta_dev, const double* unif_dev,
                      uint8_t* acc_dev, dqmc_stats* stats) {
  CHK(sweep_enqueue(h, n_calls, delta_dev, unif_dev, acc_dev));
  return sweep_finish(h, stats);
}

int dqmc_sweep(dqmc_handle* h, int32_t n_calls, const double* delta_stream, const double* unif_stream,
               uint8_t* accepted, dqmc_stats* stats) {
  if (h) cudaSetDevice(h->device);
  if (!h || n_calls < 0 || !delta_stream || !unif_stream) return DQMC_ERR_ARG;
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  if (n_calls == 0) return DQMC_OK;
  CHK(ensure_stream_capacity(h, n_calls));
  CHK(ensure_out_capacity(h, n_calls));
  CU(cudaMemcpyAsync(h->delta_d, delta_stream, (size_t)n_calls * 3 * h->N * sizeof(double),
                     cudaMemcpyHostToDevice, h->st));
  CU(cudaMemcpyAsync(h->unif_d, unif_stream, (size_t)n_calls * h->N * sizeof(double), cudaMemcpyHostToDevice,
                     h->st));
  CHK(sweep_impl(h, n_calls, h->delta_d, h->unif_d, accepted ? h->acc_d : nullptr, stats));
  if (accepted) {
    CU(cudaMemcpyAsync(accepted, h->acc_d, (size_t)n_calls * h->N, cudaMemcpyDeviceToHost, h->st));
    return sync(h);
  }
  return DQMC_OK;
}

int dqmc_sweep_device(dqmc_handle* h, int32_t n_calls, const double* delta_stream_dev,
                      const double* unif_stream_dev, uint8_t* accepted_dev, dqmc_stats* stats) {
  if (h) cudaSetDevice(h->device);
  if (!h || n_calls < 0 || !delta_stream_dev || !unif_stream_dev) return DQMC_ERR_ARG;
  if (!all_device_accessible({delta_stream_dev, unif_stream_dev, accepted_dev}))
    return set_err(h, DQMC_ERR_ARG, "stream or accept pointer is not device memory");
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  if (n_calls == 0) return DQMC_OK;
  return sweep_impl(h, n_calls, delta_stream_dev, unif_stream_dev, accepted_dev, stats);
}

// ---- batches of independent chains ----------------------------------------
struct dqmc_batch {
  std::vector<dqmc_handle*> chains;
  int inflight = 1;   // chains swept at the same time
  // the whole batch sweep as one CUDA graph: every chain's launches on its
  // own stream, chain q after chain q - inflight, forked from and joined
  // into st0; one graph per (calls, start state of every chain)
  struct BatchGraph {
    int n_calls = 0;
    std::vector<int> slice0, dir0, slice1, dir1;
    std::vector<std::array<int64_t, DQMC_NKINDS>> cnt;
    std::vector<std::array<double, DQMC_NKINDS>> flops, bytes;
    std::vector<int64_t> launches;
    std::vector<int64_t> epoch;   // every chain's graph_epoch at the capture
    cudaGraphExec_t exec = nullptr;
  };
  std::vector<BatchGraph> graphs;
  bool graphs_off = false;
  cudaStream_t st0 = nullptr;
  cudaEvent_t fork = nullptr;
};

// Chains in flight per batch: enough to fill the SMs while each chain's
// latency-bound kernels keep a useful share of them (measured optimum ~8-12).
// Chains in flight: 8 by default (64 chains of L in {6..12} on GB300 gave
// 18.6 / 24.4 / 22.9 / 19.8 / 13.2 / 7.8 chain-sweeps/s for 4 / 8 / 12 / 19 /
// 32 / 64: beyond ~8 the capped cooperative grids compete for the SMs).
static int batch_inflight(int count, int requested) {
  const int k = requested > 0 ? requested : 8;
  return count < k ? count : k;
}

int dqmc_batch_create(const dqmc_params* params, int32_t count, dqmc_batch** out) {
  if (!params || !out || count < 1) return DQMC_ERR_ARG;
  *out = nullptr;
  dqmc_batch* b = new dqmc_batch();
  b->inflight = batch_inflight(count, params[0].inflight);
  for (int i = 0; i < count; ++i) {
    dqmc_handle* h = nullptr;
    int rc = dqmc_create(&params[i], &h);
    if (rc != DQMC_OK) {
      for (auto c : b->chains) dqmc_destroy(c);
      delete b;
      return rc;
    }
    // the chains in flight can all be resident at once: their cooperative
    // grids add up to at most one CTA per SM
    h->coop_cap = h->sm_count / b->inflight > 0 ? h->sm_count / b->inflight : 1;
    b->chains.push_back(h);
  }
  *out = b;
  return DQMC_OK;
}

int dqmc_batch_destroy(dqmc_batch* b) {
  if (!b) return DQMC_ERR_ARG;
  if (!b->chains.empty()) cudaSetDevice(b->chains[0]->device);
  for (auto& g : b->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->st0) cudaStreamDestroy(b->st0);
  for (auto c : b->chains) dqmc_destroy(c);
  delete b;
  return DQMC_OK;
}

// Captures the batch sweep from the chains' current states into one graph
// (order: the launch order of the chains).  The chains' host states are left
// as before (nothing has run).  Returns null, and stops trying for this
// batch, if the capture is refused.
static dqmc_batch::BatchGraph* batch_capture(dqmc_batch* b, int n_calls, const std::vector<int>& order) {
  const int C = (int)b->chains.size();
  dqmc_batch::BatchGraph g;
  g.n_calls = n_calls;
  g.slice0.resize(C); g.dir0.resize(C); g.slice1.resize(C); g.dir1.resize(C);
  g.cnt.resize(C); g.flops.resize(C); g.bytes.resize(C); g.launches.resize(C); g.epoch.resize(C);
  std::vector<std::array<int64_t, DQMC_NKINDS>> c0(C);
  std::vector<std::array<double, DQMC_NKINDS>> f0(C), b0(C);
  std::vector<int64_t> l0(C);
  for (int i = 0; i < C; ++i) {
    dqmc_handle* h = b->chains[i];
    g.slice0[i] = h->current_slice; g.dir0[i] = h->direction; g.epoch[i] = h->graph_epoch;
    for (int k = 0; k < DQMC_NKINDS; ++k) { c0[i][k] = h->cnt[k]; f0[i][k] = h->flops[k]; b0[i][k] = h->bytes[k]; }
    l0[i] = h->launches;
    h->capture_while = 0;
  }
  cudaGetLastError();
  bool ok = cudaStreamBeginCapture(b->st0, cudaStreamCaptureModeThreadLocal) == cudaSuccess &&
            cudaEventRecord(b->fork, b->st0) == cudaSuccess;
  int rc = DQMC_OK;
  for (int q = 0; ok && q < C; ++q) {
    dqmc_handle* h = b->chains[order[q]];
    ok = cudaStreamWaitEvent(h->st, b->fork, 0) == cudaSuccess;
    if (ok && q >= b->inflight)
      ok = cudaStreamWaitEvent(h->st, b->chains[order[q - b->inflight]]->done, 0) == cudaSuccess;
    if (ok) rc = sweep_body(h, n_calls, h->delta_d, h->unif_d, nullptr);
    ok = ok && rc == DQMC_OK && h->capture_while == 0 && cudaEventRecord(h->done, h->st) == cudaSuccess;
  }
  for (int q = 0; ok && q < C; ++q) ok = cudaStreamWaitEvent(b->st0, b->chains[order[q]]->done, 0) == cudaSuccess;
  cudaGraph_t graph = nullptr;
  const bool ended = cudaStreamEndCapture(b->st0, &graph) == cudaSuccess;
  ok = ok && ended && graph;
  if (ok) ok = cudaGraphInstantiate(&g.exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  for (int i = 0; i < C; ++i) {
    dqmc_handle* h = b->chains[i];
    g.slice1[i] = h->current_slice; g.dir1[i] = h->direction;
    for (int k = 0; k < DQMC_NKINDS; ++k) {
      g.cnt[i][k] = h->cnt[k] - c0[i][k]; g.flops[i][k] = h->flops[k] - f0[i][k]; g.bytes[i][k] = h->bytes[k] - b0[i][k];
      h->cnt[k] = c0[i][k]; h->flops[k] = f0[i][k]; h->bytes[k] = b0[i][k];
    }
    g.launches[i] = h->launches - l0[i];
    h->launches = l0[i];
    h->current_slice = g.slice0[i]; h->direction = g.dir0[i];
    h->last_error.clear();
  }
  cudaGetLastError();
  if (!ok) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    b->graphs_off = true;
    return nullptr;
  }
  b->graphs.push_back(std::move(g));
  return &b->graphs.back();
}

// The batch sweep as one graph launch on st0 (streams copied into each
// chain's own buffers first).  Returns kBatchUngraphed, with nothing
// enqueued, when the chains are not graphed (timing on, capture refused).
constexpr int kBatchUngraphed = 1;
static int batch_graph_sweep(dqmc_batch* b, int n_calls, const std::vector<int>& order,
                             const double* const* delta_dev, const double* const* unif_dev) {
  const int C = (int)b->chains.size();
  dqmc_handle* h = b->chains[0];   // error reports (CU, CHK) go to the first chain
  if (b->graphs_off) return kBatchUngraphed;
  for (auto c : b->chains)
    if (c->timing || c->graphs_off || c->device != h->device) return kBatchUngraphed;
  cudaSetDevice(h->device);
  if (!b->st0) CU(cudaStreamCreateWithFlags(&b->st0, cudaStreamNonBlocking));
  if (!b->fork) CU(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  for (auto c : b->chains) {
    CHK(ensure_stream_capacity(c, n_calls));
    if (!c->done) CU(cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming));
    if (!c->ev0) {
      CU(cudaEventCreate(&c->ev0));
      CU(cudaEventCreate(&c->ev1));
    }
    CU(cudaStreamSynchronize(c->st));   // work queued on a chain's own stream ends before the graph
  }
  dqmc_batch::BatchGraph* g = nullptr;
  for (auto& x : b->graphs) {
    if (x.n_calls != n_calls) continue;
    bool same = true;
    for (int i = 0; i < C && same; ++i)
      same = x.slice0[i] == b->chains[i]->current_slice && x.dir0[i] == b->chains[i]->direction &&
             x.epoch[i] == b->chains[i]->graph_epoch;
    if (same) { g = &x; break; }
  }
  if (!g) g = batch_capture(b, n_calls, order);
  if (!g) return kBatchUngraphed;
  // per chain, on st0 before the graph: the streams into the chain's buffers,
  // the acceptance counter snapshot, the instability maximum reset
  for (int i = 0; i < C; ++i) {
    dqmc_handle* c = b->chains[i];
    const size_t N = c->N;
    if (delta_dev[i] != c->delta_d)
      CU(cudaMemcpyAsync(c->delta_d, delta_dev[i], (size_t)n_calls * 3 * N * sizeof(double), cudaMemcpyDeviceToDevice,
                         b->st0));
    if (unif_dev[i] != c->unif_d)
      CU(cudaMemcpyAsync(c->unif_d, unif_dev[i], (size_t)n_calls * N * sizeof(double), cudaMemcpyDeviceToDevice,
                         b->st0));
    CU(cudaMemcpyAsync(c->nacc_d + 1, c->nacc_d, sizeof(int), cudaMemcpyDeviceToDevice, b->st0));
    CU(cudaMemsetAsync(c->scal_d + 3, 0, sizeof(double), b->st0));
    c->max_instability = 0.0;
    CU(cudaEventRecord(c->ev0, b->st0));
  }
  CU(cudaGraphLaunch(g->exec, b->st0));
  for (int i = 0; i < C; ++i) {
    dqmc_handle* c = b->chains[i];
    CU(cudaEventRecord(c->ev1, b->st0));
    c->current_slice = g->slice1[i];
    c->direction = g->dir1[i];
    for (int k = 0; k < DQMC_NKINDS; ++k) {
      c->cnt[k] += g->cnt[i][k]; c->flops[k] += g->flops[i][k]; c->bytes[k] += g->bytes[i][k];
    }
    c->launches += g->launches[i];
    c->pending_calls = n_calls;
    c->pending_while = 0;
  }
  CU(cudaStreamSynchronize(b->st0));
  return DQMC_OK;
}

int dqmc_batch_handle(dqmc_batch* b, int32_t i, dqmc_handle** h) {
  if (!b || !h || i < 0 || i >= (int)b->chains.size()) return DQMC_ERR_ARG;
  *h = b->chains[i];
  return DQMC_OK;
}

// Largest chains first; chain q starts once chain q - inflight has finished,
// so `inflight` chains run at a time, each with its capped cooperative grids.
// The whole batch sweep is one graph launch (batch_graph_sweep); launch by
// launch (timing on) every chain's sweep is enqueued on its own stream.
int dqmc_batch_sweep(dqmc_batch* b, int32_t n_calls, const double* const* delta_dev, const double* const* unif_dev,
                     dqmc_stats* stats) {
  if (!b || n_calls < 0 || !delta_dev || !unif_dev) return DQMC_ERR_ARG;
  const int C = (int)b->chains.size();
  for (int i = 0; i < C; ++i) {
    dqmc_handle* h = b->chains[i];
    if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init on every chain first");
    if (!delta_dev[i] || !unif_dev[i]) return DQMC_ERR_ARG;
    if (!all_device_accessible({delta_dev[i], unif_dev[i]}))
      return set_err(h, DQMC_ERR_ARG, "stream pointer is not device memory");
  }
  std::vector<int> order(C);
  for (int i = 0; i < C; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->chains[x]->n > b->chains[y]->n; });
  int rc = DQMC_OK;
  const int gr = batch_graph_sweep(b, n_calls, order, delta_dev, unif_dev);
  if (gr != kBatchUngraphed) {
    if (gr != DQMC_OK) return gr;
    for (int q = 0; q < C; ++q) {
      dqmc_handle* h = b->chains[order[q]];
      int r = sweep_finish(h, stats ? &stats[order[q]] : nullptr);
      if (r != DQMC_OK && rc == DQMC_OK) rc = r;
    }
    return rc;
  }
  // launch by launch: chain q's stream waits on the end event of chain q - inflight
  for (int q = 0; q < C; ++q) {
    dqmc_handle* h = b->chains[order[q]];
    cudaSetDevice(h->device);
    if (!h->done) CU(cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming));
    if (q >= b->inflight) CU(cudaStreamWaitEvent(h->st, b->chains[order[q - b->inflight]]->done, 0));
    const int i = order[q];
    CHK(sweep_enqueue(h, n_calls, delta_dev[i], unif_dev[i], nullptr));
    CU(cudaEventRecord(h->done, h->st));
  }
  for (int q = 0; q < C; ++q) {
    dqmc_handle* h = b->chains[order[q]];
    cudaSetDevice(h->device);
    int r = sweep_finish(h, stats ? &stats[order[q]] : nullptr);
    if (r != DQMC_OK && rc == DQMC_OK) rc = r;
  }
  return rc;
}

int dqmc_get_greens(dqmc_handle* h, double* out, int32_t* slice, int32_t* direction) {
  if (h) cudaSetDevice(h->device);
  if (!h || !out) return DQMC_ERR_ARG;
  CHK(download_nn(h, out, h->G));
  if (slice) *slice = h->current_slice;
  if (direction) *direction = h->direction;
  return sync(h);
}

int dqmc_set_greens(dqmc_handle* h, const double* in) {
  if (h) cudaSetDevice(h->device);
  if (!h || !in) return DQMC_ERR_ARG;
  CHK(upload_nn(h, h->G, in));
  return sync(h);
}

int dqmc_wrap_greens(dqmc_handle* h, double* inout, int32_t slice, int32_t direction) {
  if (h) cudaSetDevice(h->device);
  if (!h || !inout || (direction != 1 && direction != -1)) return DQMC_ERR_ARG;
  int sl0 = direction == 1 ? slice : slice - 1;
  if (sl0 < 1 || sl0 > h->M) return set_err(h, DQMC_ERR_ARG, "slice out of range");
  CHK(upload_nn(h, h->Gtmp, inout));
  CHK(wrap_greens(h, h->Gtmp, slice, direction));
  CHK(download_nn(h, inout, h->Gtmp));
  return sync(h);
}

int dqmc_multiply_B(dqmc_handle* h, int32_t which, int32_t slice, double* inout) {
  if (h) cudaSetDevice(h->device);
  if (!h || !inout || which < 0 || which > 4) return DQMC_ERR_ARG;
  if (slice < 1 || slice > h->M) return set_err(h, DQMC_ERR_ARG, "slice out of range");
  CHK(upload_nn(h, h->Gtmp, inout));
  if (which == DQMC_B_RIGHT || which == DQMC_B_INV_RIGHT)
    CHK(apply_rows(h, h->Gtmp, slice - 1, 1, 1, which));
  else
    CHK(apply_cols(h, h->Gtmp, slice - 1, 1, 1, which, nullptr));
  CHK(download_nn(h, inout, h->Gtmp));
  return sync(h);
}

int dqmc_calculate_greens_udt(dqmc_handle* h, const double* Ul, const double* Dl, const double* Tl,
                              const double* Ur, const double* Dr, const double* Tr, double* G, double* logdet) {
  if (h) cudaSetDevice(h->device);
  if (!h || !Ul || !Dl || !Tl || !Ur || !Dr || !Tr || !G) return DQMC_ERR_ARG;
  const size_t dn = h->n * sizeof(double);
  CHK(upload_nn(h, h->Ul, Ul));
  CHK(upload_nn(h, h->Tl, Tl));
  CHK(upload_nn(h, h->Ur, Ur));
  CHK(upload_nn(h, h->Tr, Tr));
  CU(cudaMemcpyAsync(h->Dl, Dl, dn, cudaMemcpyHostToDevice, h->st));
  CU(cudaMemcpyAsync(h->Dr, Dr, dn, cudaMemcpyHostToDevice, h->st));
  CHK(calculate_greens_into(h, h->Gtmp));
  CHK(download_nn(h, G, h->Gtmp));
  double sl = 0.0;
  CU(cudaMemcpyAsync(&sl, h->scal_d, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CHK(sync(h));
  if (logdet) *logdet = -sl;
  return DQMC_OK;
}

int dqmc_decompose_udt(dqmc_handle* h, const double* A, double* U, double* D, double* T) {
  if (h) cudaSetDevice(h->device);
  if (!h || !A || !U || !D || !T) return DQMC_ERR_ARG;
  CHK(upload_nn(h, h->W1, A));
  CHK(decompose_udt(h, h->W1, h->W3, h->D1, h->W2));
  CHK(download_nn(h, U, h->W3));
  CHK(download_nn(h, T, h->W2));
  CU(cudaMemcpyAsync(D, h->D1, h->n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  return sync(h);
}

int dqmc_logdet(dqmc_handle* h, double* logdet) {
  if (h) cudaSetDevice(h->device);
  if (!h || !logdet) return DQMC_ERR_ARG;
  double sl = 0.0;
  CU(cudaMemcpyAsync(&sl, h->scal_d + 2, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CHK(sync(h));
  *logdet = -sl;
  return DQMC_OK;
}

// calc_greens_and_logdet (src/fermion_measurements.jl:1061-1101): the B chains
// B(slice)^dag ... B(M)^dag and B(slice-1) ... B(1) as UDTs, stabilised every
// safe_mult slices (calc_Bchain_dagger / calc_Bchain, :964-1058).
int dqmc_calc_greens(dqmc_handle* h, int32_t slice, double* out, double* logdet) {
  if (h) cudaSetDevice(h->device);
  if (!h || !out) return DQMC_ERR_ARG;
  if (slice < 1 || slice > h->M) return set_err(h, DQMC_ERR_ARG, "slice out of range");
  const int n = h->n, s = h->s;
  // chain helper: U, D, T accumulate into (Ux, Dx, Tx) buffers
  auto chain = [&](int start, int stop, bool dagger, cplx* Ux, double* Dx, cplx* Tx) -> int {
    CHK(set_identity(h, Ux));
    CHK(set_identity(h, Tx));
    CHK(set_ones(h, Dx));
    auto flush = [&]() -> int {
      LAUNCH(DQMC_K_MISC, 0.0, 32.0 * n2(h), launch_scale(Ux, n, n, nullptr, false, Dx, false, h->st));
      CHK(copy_nn(h, h->W1, Ux));
      CHK(decompose_udt(h, h->W1, Ux, Dx, h->W2));
      CHK(gemm(h, 'N', 'N', h->W2, Tx, h->W4));
      CHK(copy_nn(h, Tx, h->W4));
      return DQMC_OK;
    };
    if (!dagger) {
      for (int k = start; k <= stop; ++k) {
        CHK(apply_cols(h, Ux, k - 1, 1, 1, SLICE_LEFT_B, nullptr));
        if (k % s == 0 || k == stop) CHK(flush());
      }
    } else {
      for (int k = stop; k >= start; --k) {
        CHK(apply_cols(h, Ux, k - 1, 1, 1, SLICE_LEFT_BDAG, nullptr));
        if (k % s == 0 || k == start) CHK(flush());
      }
    }
    return DQMC_OK;
  };
  // Ur, Dr, Tr = B(slice)^dag ... B(M)^dag ; Ul, Dl, Tl = B(slice-1) ... B(1)
  CHK(chain(slice, h->M, true, h->Ur, h->Dr, h->Tr));
  if (slice - 1 >= 1) {
    CHK(chain(1, slice - 1, false, h->Ul, h->Dl, h->Tl));
  } else {
    CHK(set_identity(h, h->Ul));
    CHK(set_identity(h, h->Tl));
    CHK(set_ones(h, h->Dl));
  }
  CHK(calculate_greens_into(h, h->Gtmp));
  CHK(download_nn(h, out, h->Gtmp));
  double sl = 0.0;
  CU(cudaMemcpyAsync(&sl, h->scal_d, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CHK(sync(h));
  if (logdet) *logdet = -sl;
  // the stack copies Ul..Tr were overwritten: restore nothing (propagate re-reads them from the stack)
  return DQMC_OK;
}

// Backup buffers of the global moves (stack, G, field, interaction table),
// allocated on first use.
static int ensure_global_backup(dqmc_handle* h) {
  if (h->gb_u) return DQMC_OK;
  const size_t stack_c = (size_t)h->ne * h->n * h->n, NM = (size_t)h->N * h->M;
  CU(cudaMalloc(&h->gb_u, stack_c * sizeof(cplx)));
  CU(cudaMalloc(&h->gb_t, stack_c * sizeof(cplx)));
  CU(cudaMalloc(&h->gb_d, (size_t)h->ne * h->n * sizeof(double)));
  CU(cudaMalloc(&h->gb_G, nn_bytes(h)));
  CU(cudaMalloc(&h->gb_phi, 3 * NM * sizeof(double)));
  CU(cudaMalloc(&h->gb_evtab, NM * evtab_entry_bytes()));
  return DQMC_OK;
}

int dqmc_global_update(dqmc_handle* h, const double* shift, double u, int32_t* accepted, double* p_acc) {
  if (h) cudaSetDevice(h->device);
  if (!h || !shift) return DQMC_ERR_ARG;
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  if (h->current_slice != h->M || h->direction != -1)
    return set_err(h, DQMC_ERR_STATE, "dqmc_global_update needs the state (slice M, direction -1)");
  const size_t NM = (size_t)h->N * h->M;
  CHK(ensure_global_backup(h));
  double S_old = 0.0, ldsum_old = 0.0;
  CU(cudaMemcpyAsync(&S_old, h->action_d, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaMemcpyAsync(&ldsum_old, h->scal_d + 2, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CHK(sync(h));
  // back up (stack and G by pointer swap, field and table by copy), shift, rebuild
  clear_graphs(h);
  std::swap(h->u_stack, h->gb_u);
  std::swap(h->t_stack, h->gb_t);
  std::swap(h->d_stack, h->gb_d);
  std::swap(h->G, h->gb_G);
  CU(cudaMemcpyAsync(h->gb_phi, h->phi, 3 * NM * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  CU(cudaMemcpyAsync(h->gb_evtab, h->evtab, NM * evtab_entry_bytes(), cudaMemcpyDeviceToDevice, h->st));
  LAUNCH(DQMC_K_MISC, 0.0, 0.0, launch_shift_field(h->phi, NM, shift[0], shift[1], shift[2], h->st));
  LAUNCH(DQMC_K_MISC, 0.0, 0.0,
         launch_build_evtab(h->phi, h->evtab, h->N, h->M, h->p.lambda * h->p.delta_tau, h->st));
  CHK(build_stack(h));
  CHK(propagate(h));
  std::vector<double> phi(3 * NM);
  double ldsum_new = 0.0;
  CU(cudaMemcpyAsync(phi.data(), h->phi, phi.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaMemcpyAsync(&ldsum_new, h->scal_d + 2, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CHK(sync(h));
  const double S_new = boson_action_host(h, phi);
  // log det G = -sum log d2; p_fermion = exp(logdetG_old - logdetG_new)
  const double p_boson = std::exp(-(S_new - S_old));
  const double p_fermion = std::exp(-ldsum_old + ldsum_new);
  const double p = p_boson * p_fermion;
  const bool acc = p > 1.0 || u < p;
  if (acc) {
    CU(cudaMemcpyAsync(h->action_d, &S_new, sizeof(double), cudaMemcpyHostToDevice, h->st));
  } else {
    std::swap(h->u_stack, h->gb_u);
    std::swap(h->t_stack, h->gb_t);
    std::swap(h->d_stack, h->gb_d);
    std::swap(h->G, h->gb_G);
    CU(cudaMemcpyAsync(h->phi, h->gb_phi, 3 * NM * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    CU(cudaMemcpyAsync(h->evtab, h->gb_evtab, NM * evtab_entry_bytes(), cudaMemcpyDeviceToDevice, h->st));
    CU(cudaMemcpyAsync(h->scal_d + 2, &ldsum_old, sizeof(double), cudaMemcpyHostToDevice, h->st));
  }
  CHK(sync(h));
  if (accepted) *accepted = acc ? 1 : 0;
  if (p_acc) *p_acc = p;
  return DQMC_OK;
}

// d log|det M| / d phi into h->force_d from the per-slice G of one down pass
// (slices M, M-1, ..., 1) starting at the state (M, -1); the state is left
// at (1, -1).
static int force_down_pass(dqmc_handle* h) {
  const size_t cnt = (size_t)3 * h->N * h->M;
  if (!h->force_d) CU(cudaMalloc(&h->force_d, cnt * sizeof(double)));
  const double ld = h->p.lambda * h->p.delta_tau;
  for (int c = 0; c < h->M; ++c) {
    if (c > 0) CHK(propagate(h));
    LAUNCH(DQMC_K_MISC, 0.0, 0.0, launch_force_slice(h->G, h->phi, h->force_d, h->N, h->current_slice - 1, ld, h->st));
  }
  return DQMC_OK;
}

// Hybrid Monte Carlo move on the effective action S_eff = S_b - log|det M|
// (the log-weight of the reference's global update, src/global_updates.jl:18-58):
// leapfrog with the adjoint force -dS_eff/dphi = dlog|det M|/dphi - dS_b/dphi,
// then a Metropolis test on dH.  The field lives on the host between the
// steps (3 N M doubles); every step uploads it, rebuilds the stack and takes
// the force from one down pass.
int dqmc_hmc_update(dqmc_handle* h, const double* momenta, int32_t n_steps, double eps, double u,
                    int32_t* accepted, double* delta_H) {
  if (h) cudaSetDevice(h->device);
  if (!h || !momenta || n_steps < 1 || !(eps > 0.0) || !std::isfinite(eps)) return DQMC_ERR_ARG;
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  if (h->current_slice != h->M || h->direction != -1)
    return set_err(h, DQMC_ERR_STATE, "dqmc_hmc_update needs the state (slice M, direction -1)");
  const size_t NM = (size_t)h->N * h->M, cnt = 3 * NM;
  CHK(ensure_global_backup(h));
  std::vector<double> phi(cnt), pi(momenta, momenta + cnt), gl(cnt), gb(cnt);
  double S_old = 0.0, ldsum_old = 0.0;
  CU(cudaMemcpyAsync(phi.data(), h->phi, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaMemcpyAsync(&S_old, h->action_d, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaMemcpyAsync(&ldsum_old, h->scal_d + 2, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CHK(sync(h));
  // H = |pi|^2 / 2 + S_b - log|det M|, with log|det M| = -log det G = sum log d2
  double kin_old = 0.0;
  for (double v : pi) kin_old += 0.5 * v * v;
  const double H_old = kin_old + S_old - ldsum_old;
  // back up (stack and G by pointer swap, field and table by copy)
  clear_graphs(h);
  std::swap(h->u_stack, h->gb_u);
  std::swap(h->t_stack, h->gb_t);
  std::swap(h->d_stack, h->gb_d);
  std::swap(h->G, h->gb_G);
  CU(cudaMemcpyAsync(h->gb_phi, h->phi, cnt * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  CU(cudaMemcpyAsync(h->gb_evtab, h->evtab, NM * evtab_entry_bytes(), cudaMemcpyDeviceToDevice, h->st));
  // the force at the start: the backed-up stack's G is the current one, so
  // the first down pass runs on a rebuilt copy of the same field
  auto rebuild = [&]() -> int {
    CU(cudaMemcpyAsync(h->phi, phi.data(), cnt * sizeof(double), cudaMemcpyHostToDevice, h->st));
    LAUNCH(DQMC_K_MISC, 0.0, 0.0,
           launch_build_evtab(h->phi, h->evtab, h->N, h->M, h->p.lambda * h->p.delta_tau, h->st));
    CHK(build_stack(h));
    return propagate(h);
  };
  auto force = [&]() -> int {   // F = dlog|det M|/dphi - dS_b/dphi at the field `phi`
    CHK(force_down_pass(h));
    CU(cudaMemcpyAsync(gl.data(), h->force_d, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CHK(sync(h));
    boson_gradient_host(h, phi, gb.data());
    return DQMC_OK;
  };
  int rc = rebuild();
  if (rc == DQMC_OK) rc = force();
  for (int st = 0; rc == DQMC_OK && st < n_steps; ++st) {
    for (size_t k = 0; k < cnt; ++k) pi[k] += 0.5 * eps * (gl[k] - gb[k]);
    for (size_t k = 0; k < cnt; ++k) phi[k] += eps * pi[k];
    rc = rebuild();
    if (rc == DQMC_OK) rc = force();
    if (rc == DQMC_OK)
      for (size_t k = 0; k < cnt; ++k) pi[k] += 0.5 * eps * (gl[k] - gb[k]);
  }
  // the state (M, -1) of the final field, its action and log|det M|
  if (rc == DQMC_OK) rc = rebuild();
  double ldsum_new = 0.0;
  if (rc == DQMC_OK) {
    CU(cudaMemcpyAsync(&ldsum_new, h->scal_d + 2, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    rc = sync(h);
  }
  const double S_new = boson_action_host(h, phi);
  double kin_new = 0.0;
  for (double v : pi) kin_new += 0.5 * v * v;
  const double dH = kin_new + S_new - ldsum_new - H_old;
  const bool ok = rc == DQMC_OK && std::isfinite(dH);
  const double p = ok ? std::exp(-dH) : 0.0;
  const bool acc = ok && (p > 1.0 || u < p);
  if (acc) {
    CU(cudaMemcpyAsync(h->action_d, &S_new, sizeof(double), cudaMemcpyHostToDevice, h->st));
  } else {
    std::swap(h->u_stack, h->gb_u);
    std::swap(h->t_stack, h->gb_t);
    std::swap(h->d_stack, h->gb_d);
    std::swap(h->G, h->gb_G);
    CU(cudaMemcpyAsync(h->phi, h->gb_phi, cnt * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    CU(cudaMemcpyAsync(h->evtab, h->gb_evtab, NM * evtab_entry_bytes(), cudaMemcpyDeviceToDevice, h->st));
    CU(cudaMemcpyAsync(h->scal_d + 2, &ldsum_old, sizeof(double), cudaMemcpyHostToDevice, h->st));
    h->current_slice = h->M;
    h->direction = -1;
  }
  CHK(sync(h));
  if (rc != DQMC_OK) return rc;
  if (accepted) *accepted = acc ? 1 : 0;
  if (delta_H) *delta_H = dH;
  return DQMC_OK;
}

int dqmc_force(dqmc_handle* h, double* grad_logdet, double* grad_boson) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  if (h->current_slice != h->M || h->direction != -1)
    return set_err(h, DQMC_ERR_STATE, "dqmc_force needs the state (slice M, direction -1)");
  const size_t cnt = (size_t)3 * h->N * h->M;
  CHK(force_down_pass(h));
  // back to (M, -1): turnaround at 0 and the up pass
  while (!(h->current_slice == h->M && h->direction == -1)) CHK(propagate(h));
  if (grad_logdet) CU(cudaMemcpyAsync(grad_logdet, h->force_d, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CHK(sync(h));
  if (grad_boson) {
    std::vector<double> phi(cnt);
    CU(cudaMemcpyAsync(phi.data(), h->phi, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CHK(sync(h));
    boson_gradient_host(h, phi, grad_boson);
  }
  return DQMC_OK;
}

int dqmc_boson_action(dqmc_handle* h, double* S) {
  if (h) cudaSetDevice(h->device);
  if (!h || !S) return DQMC_ERR_ARG;
  CU(cudaMemcpyAsync(S, h->action_d, sizeof(double), cudaMemcpyDeviceToHost, h->st));
  return sync(h);
}

int dqmc_calc_boson_action(dqmc_handle* h, double* S) {
  if (h) cudaSetDevice(h->device);
  if (!h || !S) return DQMC_ERR_ARG;
  std::vector<double> phi((size_t)3 * h->N * h->M);
  CU(cudaMemcpyAsync(phi.data(), h->phi, phi.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CHK(sync(h));
  *S = boson_action_host(h, phi);
  return DQMC_OK;
}

int dqmc_measure_equal_time(dqmc_handle* h, const double* greens, double* etpc_plus, double* etpc_minus,
                             double* etcdc_plus, double* etcdc_minus, int32_t device_ptrs) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  if (device_ptrs && !all_device_accessible({greens, etpc_plus, etpc_minus, etcdc_plus, etcdc_minus}))
    return set_err(h, DQMC_ERR_ARG, "device_ptrs set but an array is not device memory");
  const int N = h->N;
  const cplx* src = nullptr;
  if (greens) {
    if (device_ptrs) {
      src = reinterpret_cast<const cplx*>(greens);
    } else {
      CU(cudaMemcpyAsync(h->Gtmp, greens, (size_t)h->n * h->n * sizeof(cplx), cudaMemcpyHostToDevice, h->st));
      src = h->Gtmp;
    }
  } else {
    CHK(hook_true_greens(h, h->Gtmp));
    src = h->Gtmp;
  }
  if (!h->etc_d) CU(cudaMalloc(&h->etc_d, (size_t)6 * N * sizeof(double)));
  LAUNCH(DQMC_K_MISC, 0.0, 0.0, launch_equal_time_corr(src, h->L, h->etc_d, h->st));
  const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  double* outs[4] = {etpc_plus, etpc_minus, etcdc_plus, etcdc_minus};
  const size_t off[4] = {0, (size_t)N, (size_t)2 * N, (size_t)4 * N};
  const size_t cnt[4] = {(size_t)N, (size_t)N, (size_t)2 * N, (size_t)2 * N};
  for (int q = 0; q < 4; ++q)
    if (outs[q]) CU(cudaMemcpyAsync(outs[q], h->etc_d + off[q], cnt[q] * sizeof(double), kind, h->st));
  CHK(sync(h));
  return check_device_error(h);
}

int dqmc_measure(dqmc_handle* h, double* greens_out, double* occupation, double* e_kin) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  const int n = h->n, N = h->N, L = h->L;
  if (h->current_slice < 1 || h->current_slice > h->M) return set_err(h, DQMC_ERR_STATE, "no current slice");
  // g = wrap_greens(G, current_slice, +1); effective -> true G
  CHK(copy_nn(h, h->Gtmp, h->G));
  CHK(wrap_greens(h, h->Gtmp, h->current_slice, 1));
  CHK(apply_rows(h, h->Gtmp, 0, 1, 1, 5));   // G Hb_half Ha_half
  CHK(apply_cols(h, h->Gtmp, 0, 1, 1, 6, nullptr));   // Ha_half^-1 Hb_half^-1 G
  std::vector<double> g((size_t)2 * n * n);
  CHK(download_nn(h, g.data(), h->Gtmp));
  CHK(sync(h));
  if (greens_out) std::memcpy(greens_out, g.data(), g.size() * sizeof(double));
  auto Gre = [&](int r, int c) { return g[2 * ((size_t)c * n + r)]; };
  if (occupation) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += 1.0 - Gre(i, i);
    *occupation = s / n;
  }
  if (e_kin) {
    // T = -mu on the diagonal, -t on nearest-neighbour bonds (src/hoppings.jl:23-43);
    // E = sum_ij T_ij (delta_ij - G_ji)
    const double th[2] = {h->p.hoppings[0], h->p.hoppings[2]};
    const double tv[2] = {h->p.hoppings[1], h->p.hoppings[3]};
    double E = 0.0;
    for (int f = 0; f < 4; ++f) {
      int b = f & 1;
      double mu = b == 0 ? h->p.mu1 : h->p.mu2;
      for (int x = 0; x < L; ++x)
        for (int y = 0; y < L; ++y) {
          int src = y + L * x;
          int i = f * N + src;
          E += -mu * (1.0 - Gre(i, i));
          int nbs[4] = {(y + 1) % L + L * x, y + L * ((x + 1) % L), (y - 1 + L) % L + L * x,
                        y + L * ((x - 1 + L) % L)};
          double tt[4] = {tv[b], th[b], tv[b], th[b]};
          for (int q = 0; q < 4; ++q) {
            int j = f * N + nbs[q];   // T[j, i] = -t   ->  term T_ji (delta_ji - G_ij)
            E += -tt[q] * (-(Gre(i, j)));
          }
        }
    }
    *e_kin = E;
  }
  return DQMC_OK;
}

int dqmc_get_timing(dqmc_handle* h, dqmc_timing* t) {
  if (h) cudaSetDevice(h->device);
  if (!h || !t) return DQMC_ERR_ARG;
  CHK(sync(h));
  for (int k = 0; k < DQMC_NKINDS; ++k) {
    t->ms[k] = h->ms[k];
    t->launches[k] = h->cnt[k];
    t->flops[k] = h->flops[k];
    t->bytes[k] = h->bytes[k];
  }
  t->kernel_launches = h->launches;
  return DQMC_OK;
}

int dqmc_gemm_check(dqmc_handle* h, int32_t mode, const double* A, const double* B, double* C) {
  if (h) cudaSetDevice(h->device);
  if (!h || !A || !B || !C || (mode != 0 && mode != 1)) return DQMC_ERR_ARG;
  if (mode == 1 && h->p.precision != DQMC_PREC_MIXED)
    return set_err(h, DQMC_ERR_STATE, "mode 1 needs a handle created with DQMC_PREC_MIXED");
  const int n = h->n;
  CHK(upload_nn(h, h->W1, A));
  CHK(upload_nn(h, h->W2, B));
  CHK(zgemm_general(h, n, n, n, 'N', 'N', cmake(1, 0), h->W1, n, h->W2, n, cmake(0, 0), h->W3, n, nullptr, nullptr,
                    mode == 1));
  CHK(download_nn(h, C, h->W3));
  return sync(h);
}

int dqmc_peak_fp64(int32_t device, double* tflops) {
  if (!tflops || device < 0) return DQMC_ERR_ARG;
  return measure_peak_fp64(device, tflops) == cudaSuccess ? DQMC_OK : DQMC_ERR_CUDA;
}

int dqmc_reset_timing(dqmc_handle* h, int32_t enable) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  CHK(sync(h));
  for (int i = 0; i < DQMC_NKINDS; ++i) { h->ms[i] = 0; h->cnt[i] = 0; h->flops[i] = 0; h->bytes[i] = 0; }
  h->launches = 0;
  h->timing = enable != 0;
  return DQMC_OK;
}

int dqmc_measure_tdgfs(dqmc_handle* h, double* Gt0, double* G0t, int32_t device_ptrs) {
  if (h) cudaSetDevice(h->device);
  if (!h || !Gt0 || !G0t) return DQMC_ERR_ARG;
  if (!h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
  const size_t bytes = (size_t)h->M * h->n * h->n * sizeof(cplx);
  if (device_ptrs && !all_device_accessible({Gt0, G0t}))
    return set_err(h, DQMC_ERR_ARG, "device_ptrs set but an array is not device memory");
  if (device_ptrs) {
    CHK(tdgf::measure(h, reinterpret_cast<cplx*>(Gt0), reinterpret_cast<cplx*>(G0t)));
    return sync(h);
  }
  cplx *a = nullptr, *b = nullptr;
  if (tdgf::output_buffers(h, &a, &b) != DQMC_OK) return set_err(h, DQMC_ERR_CUDA, "out of device memory");
  int rc = tdgf::measure(h, a, b);
  if (rc == DQMC_OK && cudaMemcpyAsync(Gt0, a, bytes, cudaMemcpyDeviceToHost, h->st) != cudaSuccess) rc = DQMC_ERR_CUDA;
  if (rc == DQMC_OK && cudaMemcpyAsync(G0t, b, bytes, cudaMemcpyDeviceToHost, h->st) != cudaSuccess) rc = DQMC_ERR_CUDA;
  if (rc != DQMC_OK) return set_err(h, rc, "time-displaced measurement");
  return sync(h);
}

int dqmc_measure_zfpc(dqmc_handle* h, const double* Gt0, double* zfpc_plus, double* zfpc_minus, int32_t device_ptrs) {
  if (h) cudaSetDevice(h->device);
  if (!h) return DQMC_ERR_ARG;
  if (device_ptrs && !all_device_accessible({Gt0, zfpc_plus, zfpc_minus}))
    return set_err(h, DQMC_ERR_ARG, "device_ptrs set but an array is not device memory");
  const int N = h->N, M = h->M;
  const size_t bytes = (size_t)M * h->n * h->n * sizeof(cplx);
  cplx *g = nullptr, *scratch = nullptr;
  if (Gt0 && device_ptrs) {
    g = reinterpret_cast<cplx*>(const_cast<double*>(Gt0));
  } else {
    if (!Gt0 && !h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
    int rc = tdgf::output_buffers(h, &g, &scratch);
    if (rc == DQMC_OK) {
      if (Gt0) {
        if (cudaMemcpyAsync(g, Gt0, bytes, cudaMemcpyHostToDevice, h->st) != cudaSuccess) rc = DQMC_ERR_CUDA;
      } else {
        rc = tdgf::measure(h, g, scratch);   // G(tau, 0); G(0, tau) is not needed
      }
    }
    if (rc != DQMC_OK) return rc == DQMC_ERR_CUDA ? set_err(h, rc, "device memory for the time-displaced G") : rc;
  }
  if (!h->etc_d) CU(cudaMalloc(&h->etc_d, (size_t)6 * N * sizeof(double)));
  int rc = DQMC_OK;
  if (launch_zfpc(g, M, h->L, h->etc_d, h->st) != cudaSuccess) rc = DQMC_ERR_CUDA;
  ++h->launches;
  const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (rc == DQMC_OK && zfpc_plus &&
      cudaMemcpyAsync(zfpc_plus, h->etc_d, N * sizeof(double), kind, h->st) != cudaSuccess) rc = DQMC_ERR_CUDA;
  if (rc == DQMC_OK && zfpc_minus &&
      cudaMemcpyAsync(zfpc_minus, h->etc_d + N, N * sizeof(double), kind, h->st) != cudaSuccess) rc = DQMC_ERR_CUDA;
  if (rc == DQMC_OK && cudaStreamSynchronize(h->st) != cudaSuccess) rc = DQMC_ERR_CUDA;
  if (rc != DQMC_OK) return set_err(h, rc, "zfpc");
  return check_device_error(h);
}

// Shared body of the zero-frequency charge-density (which = 0) and
// current-current (which = 1) measurements: stages the equal-time G and the
// time-displaced blocks, runs the kernel, copies 2 L^2 complex outputs.
static int zero_frequency_measure(dqmc_handle* h, int which, const double* greens, const double* Gt0,
                                  const double* G0t, double* out0, double* out1, double* sfdensity,
                                  int32_t device_ptrs) {
  if (h) cudaSetDevice(h->device);
  if (!h || (Gt0 == nullptr) != (G0t == nullptr)) return DQMC_ERR_ARG;
  if (device_ptrs && !all_device_accessible({greens, Gt0, G0t, out0, out1}))
    return set_err(h, DQMC_ERR_ARG, "device_ptrs set but an array is not device memory");
  const int N = h->N, M = h->M;
  const size_t nn = (size_t)h->n * h->n, bytes = (size_t)M * nn * sizeof(cplx);
  const bool own = !(Gt0 && device_ptrs);   // time-displaced blocks staged in the handle's buffers
  cplx *gt0 = nullptr, *g0t = nullptr;
  int rc = DQMC_OK;
  if (own) {
    if (!Gt0 && !h->initialized) return set_err(h, DQMC_ERR_STATE, "call dqmc_init first");
    if (tdgf::output_buffers(h, &gt0, &g0t) != DQMC_OK) {
      rc = DQMC_ERR_CUDA;
    } else if (Gt0) {
      if (cudaMemcpyAsync(gt0, Gt0, bytes, cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
          cudaMemcpyAsync(g0t, G0t, bytes, cudaMemcpyHostToDevice, h->st) != cudaSuccess)
        rc = DQMC_ERR_CUDA;
    } else {
      rc = tdgf::measure(h, gt0, g0t);
    }
  } else {
    gt0 = reinterpret_cast<cplx*>(const_cast<double*>(Gt0));
    g0t = reinterpret_cast<cplx*>(const_cast<double*>(G0t));
  }
  // equal-time G: given (host or device) or the measurement hook's
  const cplx* g = nullptr;
  if (rc == DQMC_OK) {
    if (greens && device_ptrs) {
      g = reinterpret_cast<const cplx*>(greens);
    } else if (greens) {
      if (cudaMemcpyAsync(h->Gtmp, greens, nn * sizeof(cplx), cudaMemcpyHostToDevice, h->st) != cudaSuccess)
        rc = DQMC_ERR_CUDA;
      g = h->Gtmp;
    } else {
      rc = hook_true_greens(h, h->Gtmp);
      g = h->Gtmp;
    }
  }
  if (rc == DQMC_OK && !h->etc_d && cudaMalloc(&h->etc_d, (size_t)6 * N * sizeof(double)) != cudaSuccess)
    rc = DQMC_ERR_CUDA;
  if (rc == DQMC_OK) {
    // hopping amplitudes by direction (x, y) and band (X, Y), as the measurement hook's E_kin
    const double thop[2][2] = {{h->p.hoppings[0], h->p.hoppings[2]}, {h->p.hoppings[1], h->p.hoppings[3]}};
    const cudaError_t e = which == 0 ? launch_zfcdc(g, gt0, g0t, M, h->L, h->etc_d, h->st)
                                     : launch_zfccc(g, gt0, g0t, M, h->L, thop, h->etc_d, h->st);
    if (e != cudaSuccess) rc = DQMC_ERR_CUDA;
    ++h->launches;
  }
  const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (rc == DQMC_OK && out0 &&
      cudaMemcpyAsync(out0, h->etc_d, 2 * N * sizeof(double), kind, h->st) != cudaSuccess) rc = DQMC_ERR_CUDA;
  if (rc == DQMC_OK && out1 &&
      cudaMemcpyAsync(out1, h->etc_d + 2 * N, 2 * N * sizeof(double), kind, h->st) != cudaSuccess)
    rc = DQMC_ERR_CUDA;
  std::vector<double> lxx;
  if (rc == DQMC_OK && sfdensity) {
    lxx.resize((size_t)2 * N);
    if (cudaMemcpyAsync(lxx.data(), h->etc_d, 2 * N * sizeof(double), cudaMemcpyDeviceToHost, h->st) != cudaSuccess)
      rc = DQMC_ERR_CUDA;
  }
  if (cudaStreamSynchronize(h->st) != cudaSuccess && rc == DQMC_OK) rc = DQMC_ERR_CUDA;
  if (rc == DQMC_ERR_CUDA) return set_err(h, rc, "zero-frequency measurement: device memory or copy");
  if (rc != DQMC_OK) return rc;
  if (sfdensity) {
    // measure_sfdensity (src/fermion_measurements.jl:911-920): with q the real
    // 2D DFT of Re Lambda_xx (first index y), rho_s = (Re q[0, 1] - Re q[1, 0]) / 4
    const int L = h->L;
    const double w = 2.0 * 3.14159265358979323846 / L;
    double qx = 0.0, qy = 0.0;
    for (int x = 0; x < L; ++x)
      for (int y = 0; y < L; ++y) {
        const double v = lxx[2 * ((size_t)y + (size_t)L * x)];
        qx += v * std::cos(w * x);
        qy += v * std::cos(w * y);
      }
    *sfdensity = 0.25 * (qx - qy);
  }
  return check_device_error(h);
}

int dqmc_measure_zfcdc(dqmc_handle* h, const double* greens, const double* Gt0, const double* G0t,
                       double* zfcdc_plus, double* zfcdc_minus, int32_t device_ptrs) {
  return zero_frequency_measure(h, 0, greens, Gt0, G0t, zfcdc_plus, zfcdc_minus, nullptr, device_ptrs);
}

int dqmc_measure_zfccc(dqmc_handle* h, const double* greens, const double* Gt0, const double* G0t,
                       double* zfccc_xx, double* zfccc_yy, double* sfdensity, int32_t device_ptrs) {
  return zero_frequency_measure(h, 1, greens, Gt0, G0t, zfccc_xx, zfccc_yy, sfdensity, device_ptrs);
}

}  // extern "C"
