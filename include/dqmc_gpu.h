/*
 * dqmc_gpu.h -- C ABI of the GB300 (sm_103a) DQMC sweep library.
 *
 * This is the drop-in boundary for the hot path of carstenbauer/dqmc (the
 * O(3) spin-fermion model, Assaad checkerboard, no B-field): a Julia host
 * binds these symbols with `ccall`, a Python host with ctypes.  Every entry
 * point is `extern "C"`, takes plain pointers and sizes, returns an int
 * status (0 = ok, < 0 = error; see DQMC_ERR_*) and never throws.  The
 * message of the last error of a handle is returned by dqmc_last_error().
 *
 * Conventions shared with the reference:
 *   - G is n x n complex128, column-major (Julia Matrix{ComplexF64}),
 *     n = 4 N, N = L^2, index = flavour * N + site, site = y + L * x;
 *   - the boson field phi is double[3 * N * M], column-major (3, N, M)
 *     (src/parameters.jl:19);
 *   - slice numbers at this boundary are 1-based, as in the reference;
 *   - complex arrays are passed as double* with interleaved (re, im).
 *
 * A handle owns all device memory and one CUDA stream; it is not
 * thread-safe (one host thread drives it), distinct handles are independent.
 */
#ifndef DQMC_GPU_H
#define DQMC_GPU_H

#include <stdint.h>

#if defined(__GNUC__)
#define DQMC_API __attribute__((visibility("default")))
#else
#define DQMC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define DQMC_OK 0
#define DQMC_ERR_ARG (-1)        /* invalid argument / unsupported configuration */
#define DQMC_ERR_CUDA (-2)       /* CUDA runtime error (message has the details) */
#define DQMC_ERR_NONFINITE (-3)  /* NaN/Inf met in G or a determinant ratio */
#define DQMC_ERR_SINGULAR (-4)   /* singular 4x4 M in a local update */
#define DQMC_ERR_TIMEOUT (-5)    /* a device-side wait gave up (bounded spin) */
#define DQMC_ERR_STATE (-6)      /* call not valid in the current state */
#define DQMC_ERR_TOO_LARGE (-7)  /* n = 4 L^2 exceeds the static scratch of dqmc_local_updates_noalloc (1024) */

#define DQMC_PREC_FP64 0         /* plain FP64 everywhere */
#define DQMC_PREC_MIXED 1        /* dense products as split-BF16 tensor-core GEMMs (Ozaki); QR, D scales,
                                    triangular solves, determinant ratios and the wrap stay FP64 */

/* Parameters of the O(3) model; the subset of `Params` (src/parameters.jl:4-80)
 * that the sweep needs.  hoppings[] is the HOPPINGS string
 * "tx_x,ty_x,tx_y,ty_y" (src/lattice.jl:59). */
typedef struct dqmc_params {
  int32_t L;           /* linear lattice size (even, >= 2) */
  int32_t slices;      /* M = beta / delta_tau */
  int32_t safe_mult;   /* stabilisation interval; must divide slices */
  int32_t opdim;       /* must be 3 (O(3) model, 4 flavours) */
  double delta_tau;
  double lambda;       /* Yukawa coupling */
  double r, c, u;      /* boson action couplings */
  double mu1, mu2;     /* chemical potentials of band x and band y */
  double hoppings[4];  /* tx_x, ty_x, tx_y, ty_y */
  int32_t all_checks;  /* compare wrapped and fresh G at each stabilisation (src/stack.jl:416-429) */
  int32_t precision;   /* DQMC_PREC_FP64 or DQMC_PREC_MIXED */
  int32_t device;      /* CUDA device ordinal; -1 = the calling thread's current device */
  int32_t ozaki_bits;  /* mixed form: mantissa bits kept per GEMM operand (0 = default 40); at most what
                          8 slices reach at the product's inner dimension (40 bits at K = 1024) */
  int32_t delay;       /* delayed-update depth k (0 or 1 = immediate rank-4 updates) */
  int32_t greens_method; /* DQMC_GREENS_SCALES (default) or DQMC_GREENS_TWO_QR */
  int32_t inflight;    /* dqmc_batch_create: chains swept at the same time (0 = min(count, 8)); first chain's value.
                          dqmc_create: > 1 caps the cooperative grids as for one of that many batch chains */
  int32_t reserved[1];
} dqmc_params;

/* calculate_greens (src/stack.jl:338-369) formulations; both give
 * G = [I + Ul Dl Tl (Ur Dr Tr)^dag]^-1 and log|det G|:
 *  DQMC_GREENS_SCALES: D-scale separation, D = Dmax Dmin with Dmax = max(D, 1),
 *    G = Ur Drmax^-1 [Dlmax^-1 Ul^dag Ur Drmax^-1 + Dlmin Tl Tr^dag Drmin]^-1 Dlmax^-1 Ul^dag,
 *    the bracket (entries bounded by 1 in scale) inverted through one LU with partial pivoting;
 *  DQMC_GREENS_TWO_QR: the reference's two pivoted QRs (inv_one_plus_two_udts!, src/linalg.jl:237-283). */
#define DQMC_GREENS_SCALES 0
#define DQMC_GREENS_TWO_QR 1

typedef struct dqmc_stats {
  int64_t proposals;        /* site proposals made */
  int64_t accepted;         /* accepted proposals */
  double acc_rate;          /* accepted / proposals */
  double max_instability;   /* max |G_wrapped - G_fresh| seen at stabilisations */
  double device_ms;         /* device time of the call (CUDA events on the handle's stream) */
} dqmc_stats;

/* Kernel kinds of dqmc_timing (one CUDA-event pair per launch when timing is on). */
#define DQMC_K_SLICE_COLS 0   /* B / B^-1 / B^dag applied to columns (left products) */
#define DQMC_K_SLICE_ROWS 1   /* B / B^-1 applied to rows (right products) */
#define DQMC_K_LOCAL 2        /* local updates of one slice (detratio + rank-4 updates) */
#define DQMC_K_GEMM 3         /* complex FP64 GEMM */
#define DQMC_K_QRP 4          /* column-pivoted Householder QR */
#define DQMC_K_APPLYQ 5       /* X <- X Q (reflector application / explicit Q) */
#define DQMC_K_TRSM 6         /* triangular solves with the QR factors */
#define DQMC_K_MISC 7         /* permutations, scalings, reductions, fills */
#define DQMC_K_OZGEMM 8       /* split-BF16 tensor-core complex GEMM (mixed form); flops = tensor flops */
#define DQMC_K_FLUSH 9        /* delayed-update flush G += X Y */
#define DQMC_K_LU 10          /* LU with partial pivoting (D-scale separated calculate_greens) */
#define DQMC_NKINDS 11

typedef struct dqmc_timing {
  double ms[DQMC_NKINDS];           /* accumulated device time per kernel kind */
  int64_t launches[DQMC_NKINDS];    /* launches per kernel kind */
  double flops[DQMC_NKINDS];        /* algorithmic FP64 flops per kernel kind */
  double bytes[DQMC_NKINDS];        /* algorithmic DRAM/L2 bytes per kernel kind */
  int64_t kernel_launches;          /* all kernels launched by the library since the last reset */
} dqmc_timing;

typedef struct dqmc_handle dqmc_handle;

/* ---- lifetime ------------------------------------------------------------ */
/* DQMC(p) (src/dqmc_framework.jl:105-135) + load_lattice / checkerboard setup
 * (src/hoppings_checkerboard.jl:65-136).  Allocates the device state. */
DQMC_API int dqmc_create(const dqmc_params* p, dqmc_handle** out);
DQMC_API int dqmc_destroy(dqmc_handle* h);
DQMC_API const char* dqmc_last_error(const dqmc_handle* h);
/* Library version string. */
DQMC_API const char* dqmc_version(void);

/* ---- field and state ------------------------------------------------------- */
/* p.hsfield = phi (init!(mc, start_conf), src/dqmc_framework.jl:156-163). */
DQMC_API int dqmc_set_field(dqmc_handle* h, const double* phi);
DQMC_API int dqmc_get_field(dqmc_handle* h, double* phi);
/* init! (src/dqmc_framework.jl:156-177): boson action, initialize_stack,
 * build_stack, first propagate.  Leaves the state at (slice M, direction -1). */
DQMC_API int dqmc_init(dqmc_handle* h);
/* propagate (src/stack.jl:391-499). */
DQMC_API int dqmc_propagate(dqmc_handle* h);
/* Current slice / direction (s.current_slice, s.direction). */
DQMC_API int dqmc_get_state(dqmc_handle* h, int32_t* slice, int32_t* direction);

/* ---- local updates ------------------------------------------------------- */
/* local_updates (src/local_updates.jl:1-38) at the current slice with
 * fixed-slot streams: delta[3*N] (proposal shifts phi' = phi + delta, already
 * in [-box, box]) and unif[N] (Metropolis uniforms, used only when p <= 1).
 * Optional outputs (may be NULL): accepted[N], detratio[2*N] (complex),
 * p_acc[N], acc_rate[1]. */
DQMC_API int dqmc_local_updates(dqmc_handle* h, const double* delta, const double* unif, uint8_t* accepted,
                       double* detratio, double* p_acc, double* acc_rate);
/* update (src/dqmc_framework.jl:500-517, global updates off): propagate, then
 * local_updates. */
DQMC_API int dqmc_update(dqmc_handle* h, const double* delta, const double* unif, uint8_t* accepted,
                double* detratio, double* p_acc, double* acc_rate);
/* n_calls consecutive update() calls (one sweep = M calls; the reference's
 * ud-sweep loop `for u in 1:2*p.slices update(mc, i) end`,
 * src/dqmc_framework.jl:259-261).  delta_stream[n_calls*3*N],
 * unif_stream[n_calls*N]; accepted[n_calls*N] may be NULL. */
DQMC_API int dqmc_sweep(dqmc_handle* h, int32_t n_calls, const double* delta_stream, const double* unif_stream,
               uint8_t* accepted, dqmc_stats* stats);
/* Same as dqmc_sweep but reads the streams from device memory (no host
 * copies); device pointers as returned by the caller's allocator. */
DQMC_API int dqmc_sweep_device(dqmc_handle* h, int32_t n_calls, const double* delta_stream_dev,
                      const double* unif_stream_dev, uint8_t* accepted_dev, dqmc_stats* stats);

/* Local updates of one slice for callers that cannot let the library allocate
 * device memory (their allocator owns all GPU memory, or they must stay inside
 * a fixed pre-reserved budget).  No counterpart in the reference: it is the
 * handle-free form of dqmc_local_updates, on buffers the caller owns, all of
 * them DEVICE pointers: greens (n x n complex, updated in place), phi
 * (3 x N x M, updated in place), delta[3*N], unif[N], accepted[N] (may be
 * NULL) and action (one double, incremented by each accepted Delta S).
 * `stream` is a cudaStream_t of the selected device (NULL = legacy default
 * stream).  The call is synchronous: it returns after the stream has
 * finished the update, and it returns DQMC_ERR_ARG on a stream that is being
 * captured, on a stream of another device, and when any array is not device
 * memory.  The calling thread's current device is restored on return.
 *   - It allocates nothing: its scratch (the rank-4 factors, a grid barrier
 *     and an error flag; 128 KB) is one static device array that every GPU
 *     which loads the library holds until exit.  Limit: n = 4 L^2 <= 1024
 *     (L <= 16); larger sizes return DQMC_ERR_TOO_LARGE.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) and keeps it: do not use the library across a
 *     cudaDeviceReset of that device.
 *   - All calls share the array: calls that overlap on the GPU (other host
 *     threads, other streams) race and must be serialised by the caller. */
DQMC_API int dqmc_local_updates_noalloc(const dqmc_params* p, double* greens, double* phi, int32_t slice,
                                        const double* delta, const double* unif, uint8_t* accepted,
                                        double* action, void* stream);

/* ---- batches of independent chains ----------------------------------------- */
/* A batch holds `count` independent chains (params[i] each; sizes may differ),
 * each on its own CUDA stream.  Up to 12 chains run at the same time, with
 * cooperative grids capped so that all of them can be resident on the GPU at
 * once.  dqmc_batch_handle gives the chain's handle for the single-chain calls
 * (set_field, init, greens...).  dqmc_batch_sweep runs n_calls update() calls
 * on every chain (delta_dev[i], unif_dev[i]: device streams of chain i, layouts
 * as in dqmc_sweep), largest chains first, replacing each finished chain by the
 * next one, and returns when all are done; stats has `count` entries (may be NULL).
 * Replaces the reference's SLURM job arrays of independent runs
 * (app/dqmc.jl:48-57) inside one process and one GPU. */
typedef struct dqmc_batch dqmc_batch;
DQMC_API int dqmc_batch_create(const dqmc_params* params, int32_t count, dqmc_batch** out);
DQMC_API int dqmc_batch_destroy(dqmc_batch* b);
DQMC_API int dqmc_batch_handle(dqmc_batch* b, int32_t i, dqmc_handle** h);
DQMC_API int dqmc_batch_sweep(dqmc_batch* b, int32_t n_calls, const double* const* delta_dev,
                              const double* const* unif_dev, dqmc_stats* stats);

/* ---- Green's functions ------------------------------------------------------ */
/* s.greens (effective G at the current slice). out: double[2*n*n]. */
DQMC_API int dqmc_get_greens(dqmc_handle* h, double* out, int32_t* slice, int32_t* direction);
/* Overwrite s.greens (testing and restart). */
DQMC_API int dqmc_set_greens(dqmc_handle* h, const double* in);
/* calc_greens_and_logdet (src/fermion_measurements.jl:1061-1101): G of
 * `slice` computed from scratch with the B chains, plus log|det G|. */
DQMC_API int dqmc_calc_greens(dqmc_handle* h, int32_t slice, double* out, double* logdet);
/* wrap_greens (src/stack.jl:316-332) of a host matrix: inout <- B G B^-1
 * (direction +1) or B^-1 G B (direction -1) at `slice`. */
DQMC_API int dqmc_wrap_greens(dqmc_handle* h, double* inout, int32_t slice, int32_t direction);
/* calculate_greens + calculate_logdet (src/stack.jl:338-385) on given UDTs:
 * G = [1 + Ul Dl Tl (Ur Dr Tr)^dag]^-1.  Matrices n x n complex, D real[n]. */
DQMC_API int dqmc_calculate_greens_udt(dqmc_handle* h, const double* Ul, const double* Dl, const double* Tl,
                              const double* Ur, const double* Dr, const double* Tr, double* G,
                              double* logdet);
/* decompose_udt! (src/linalg.jl:20-39): A = U diag(D) T with pivoted QR. */
DQMC_API int dqmc_decompose_udt(dqmc_handle* h, const double* A, double* U, double* D, double* T);
/* s.log_det after the last fresh G (src/stack.jl:377-385). */
DQMC_API int dqmc_logdet(dqmc_handle* h, double* logdet);

/* ---- slice matrices ---------------------------------------------------------- */
#define DQMC_B_LEFT 0        /* multiply_B_left!       (src/slice_matrices.jl:101) */
#define DQMC_B_RIGHT 1       /* multiply_B_right!      (src/slice_matrices.jl:131) */
#define DQMC_B_INV_LEFT 2    /* multiply_B_inv_left!   (src/slice_matrices.jl:155) */
#define DQMC_B_INV_RIGHT 3   /* multiply_B_inv_right!  (src/slice_matrices.jl:179) */
#define DQMC_B_DAG_LEFT 4    /* multiply_daggered_B_left! (src/slice_matrices.jl:203) */
DQMC_API int dqmc_multiply_B(dqmc_handle* h, int32_t which, int32_t slice, double* inout);

/* ---- boson action and measurements ---------------------------------------- */
/* p.boson_action as maintained by the updates (src/local_updates.jl:34). */
DQMC_API int dqmc_boson_action(dqmc_handle* h, double* S);
/* calc_boson_action (src/action.jl:1-52) recomputed from the current field. */
DQMC_API int dqmc_calc_boson_action(dqmc_handle* h, double* S);
/* Measurement hook _measure_observables! (src/dqmc_framework.jl:371-384):
 * true G = effective_greens2greens!(wrap_greens(G, slice, +1))
 * (src/fermion_measurements.jl:1125-1142) written to greens_out (may be NULL);
 * occupation (src/fermion_measurements.jl:322) and kinetic energy
 * E_kin = sum_ij T_ij <c_i^dag c_j> (not an observable of the reference). */
DQMC_API int dqmc_measure(dqmc_handle* h, double* greens_out, double* occupation, double* e_kin);
/* Equal-time pairing correlators measure_etpc! (src/fermion_measurements.jl:388-424)
 * and charge-density correlators measure_etcdc! (:592-630) of a true G: the
 * n x n column-major complex `greens` if not NULL (as the reference's `greens`
 * argument), else the measurement hook's true G of the current slice.  Outputs
 * (each may be NULL) are L x L column-major, element (y, x) = displacement
 * (x, y) averaged over origins: etpc_plus / etpc_minus real (L^2 doubles),
 * etcdc_plus / etcdc_minus complex (2 L^2 doubles).  device_ptrs != 0: every
 * pointer is a device address on the handle's device. */
DQMC_API int dqmc_measure_equal_time(dqmc_handle* h, const double* greens, double* etpc_plus, double* etpc_minus,
                                     double* etcdc_plus, double* etcdc_minus, int32_t device_ptrs);

/* global_update (src/global_updates.jl:18-58): shift every slice and site of
 * field component k by shift[k] (fixed slot, already in [-box_global,
 * box_global]), rebuild the stack, and accept with
 * p = exp(-(S_new - S_old)) * exp(logdetG_old - logdetG_new) if p > 1 or
 * u < p; a rejection restores field, stack, G and action.  Needs the state
 * (M, -1).  accepted / p_acc may be NULL. */
DQMC_API int dqmc_global_update(dqmc_handle* h, const double* shift, double u, int32_t* accepted, double* p_acc);

/* Hybrid Monte Carlo move (no counterpart in the reference, which has only the
 * field-shift global update of src/global_updates.jl:18-58; the acceptance
 * rule, the restore on rejection and the required state (M, -1) are that
 * update's).  With momenta pi[3*N*M] (fixed slot, standard normal, layout of
 * phi) and H = |pi|^2/2 + S_boson - log|det M|, n_steps leapfrog steps of
 * size eps with the force dlog|det M|/dphi - dS_boson/dphi (dqmc_force),
 * then accept with p = exp(-dH) if p > 1 or u < p.  A rejection restores
 * field, stack, G and action.  accepted / delta_H may be NULL. */
DQMC_API int dqmc_hmc_update(dqmc_handle* h, const double* momenta, int32_t n_steps, double eps, double u,
                             int32_t* accepted, double* delta_H);

/* ---- adjoint force ----------------------------------------------------------- */
/* Gradients of the log-weight parts with respect to every field component
 * (double[3*N*M], layout of phi):
 *   grad_logdet[a,i,l] = d log|det M| / d phi[a,i,l] = -Re tr(G_l[ii] E_i^-1 dE_i/dphi_a),
 *   grad_boson[a,i,l]  = d S_boson / d phi[a,i,l]  (src/action.jl:1-52).
 * M = 1 + B_M ... B_1; G_l is the equal-time G of slice l, taken from the
 * stack (checkpointed UDTs every safe_mult slices, wrapped in between) during
 * one down pass, after which the state returns to (slice M, direction -1).
 * Needs the state (M, -1), i.e. right after dqmc_init or after 2M updates.
 * No counterpart in the reference; either output may be NULL. */
DQMC_API int dqmc_force(dqmc_handle* h, double* grad_logdet, double* grad_boson);

/* ---- time-displaced Green's functions --------------------------------------- */
/* measure_tdgfs! (src/fermion_measurements.jl:1343-1403, with calc_Bchain_udts! :1411-1488,
 * fill_tdgf! :1497-1523, inv_sum_udts_scalettar! and inv_one_plus_udt_scalettar!
 * src/linalg.jl:310-339, 512-567): the time-displaced Green's functions Gt0[tau] = G(tau, 0)
 * and G0t[tau] = -G(0, tau) of the current field for tau = 1..M, each n x n column-major
 * complex at offset (tau - 1) n^2 (2 M n^2 doubles per array).  device_ptrs != 0: Gt0 and
 * G0t are device addresses on the handle's device; otherwise host buffers. */
DQMC_API int dqmc_measure_tdgfs(dqmc_handle* h, double* Gt0, double* G0t, int32_t device_ptrs);
/* measure_zfpc! (src/fermion_measurements.jl:500-541): the pairing correlators of
 * dqmc_measure_equal_time summed over G(tau, 0), tau = 1..M (not divided by M,
 * as in the reference).  Gt0: the M blocks that dqmc_measure_tdgfs writes, or
 * NULL to compute them for the current field on the device.  zfpc_plus /
 * zfpc_minus: L x L real, element (y, x) at y + L x; each may be NULL.
 * device_ptrs != 0: Gt0 and the outputs are device addresses. */
DQMC_API int dqmc_measure_zfpc(dqmc_handle* h, const double* Gt0, double* zfpc_plus, double* zfpc_minus,
                               int32_t device_ptrs);
/* measure_zfcdc! (src/fermion_measurements.jl:688-743, _zfcdc_ev :753-766):
 * zero-frequency charge-density correlators summed over tau = 1..M from the
 * true equal-time G `greens` (NULL: the measurement hook's G), G(tau, 0) in Gt0
 * and the stored -G(0, tau) in G0t as dqmc_measure_tdgfs writes them (both
 * NULL: computed for the current field on the device).  zfcdc_plus /
 * zfcdc_minus: L x L complex (2 L^2 doubles), element (y, x) at y + L x; each
 * may be NULL.  device_ptrs != 0: every pointer is a device address. */
DQMC_API int dqmc_measure_zfcdc(dqmc_handle* h, const double* greens, const double* Gt0, const double* G0t,
                                double* zfcdc_plus, double* zfcdc_minus, int32_t device_ptrs);
/* measure_zfccc! (src/fermion_measurements.jl:814-888): zero-frequency
 * current-current correlators Lambda_xx, Lambda_yy (L x L complex, 2 L^2
 * doubles each, element (y, x) at y + L x), inputs as dqmc_measure_zfcdc; and
 * measure_sfdensity (:911-920) of Lambda_xx into *sfdensity (host double, may
 * be NULL).  device_ptrs != 0: every array pointer is a device address. */
DQMC_API int dqmc_measure_zfccc(dqmc_handle* h, const double* greens, const double* Gt0, const double* G0t,
                                double* zfccc_xx, double* zfccc_yy, double* sfdensity, int32_t device_ptrs);

/* ---- diagnostics ------------------------------------------------------------- */
/* Per-group device times (CUDA events on the handle's stream) and the number
 * of kernels launched since the last reset; enable != 0 turns event timing on. */
DQMC_API int dqmc_get_timing(dqmc_handle* h, dqmc_timing* t);
DQMC_API int dqmc_reset_timing(dqmc_handle* h, int32_t enable);
/* Diagnostic: C = A * B for n x n complex matrices (column-major, interleaved)
 * with the handle's FP64 GEMM kernel (mode 0) or its split-BF16 tensor-core
 * GEMM (mode 1).  No counterpart in the reference. */
DQMC_API int dqmc_gemm_check(dqmc_handle* h, int32_t mode, const double* A, const double* B, double* C);
/* Measures the FP64 FMA throughput of `device` (TFLOP/s, 2 flops per FMA) with
 * a register-resident DFMA kernel: the roofline denominator of the FP64
 * kernels.  No counterpart in the reference (a diagnostic of this library). */
DQMC_API int dqmc_peak_fp64(int32_t device, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* DQMC_GPU_H */
