// Dense complex FP64 linear algebra for the UDT stabilisation.
//
// Reference: src/linalg.jl:20-39 (decompose_udt! = LAPACK zgeqp3 + zungqr),
// src/stack.jl:338-369 (calculate_greens) and src/stack.jl:278-313
// (add_slice_sequence_*).  The column-pivoted Householder QR restates the
// published LAPACK algorithm (zgeqp3/zlaqp2: pivot = first column of maximal
// partial norm, zlarfg reflector, column-norm downdating with the
// sqrt(eps) recomputation guard).  Columns are never moved: a logical ->
// physical order array replaces LAPACK's column swaps, so the triangular
// factor comes out directly in the un-permuted ("T = R[:, invperm(p)]")
// layout that the UDT decomposition needs.
#include <cfloat>
#include <cooperative_groups.h>
#include "common.cuh"
#include "kernels.h"

namespace {

// ---------------------------------------------------------------------------
// GEMM: C = alpha * diag(rs) * op(A) * op(B) * diag(cs) + beta * C
// ---------------------------------------------------------------------------
constexpr int GB_M = 64, GB_N = 64, GB_K = 8;

__device__ __forceinline__ cplx load_op(const cplx* X, int ld, int r, int c, int rows, int cols, char op) {
  // element (r, c) of op(X); op(X) has shape rows x cols
  if (r >= rows || c >= cols) return cmake(0.0, 0.0);
  if (op == 'N') return X[(size_t)c * ld + r];
  cplx v = X[(size_t)r * ld + c];
  return op == 'C' ? cconj(v) : v;
}

__global__ void __launch_bounds__(256) k_zgemm(int m, int nn, int k, char opA, char opB, cplx alpha,
                                              const cplx* __restrict__ A, int lda, const cplx* __restrict__ B,
                                              int ldb, cplx beta, cplx* __restrict__ C, int ldc,
                                              const double* __restrict__ rs, const double* __restrict__ cs,
                                              const int* __restrict__ active) {
  if (active) {
    const int kk = 4 * *active;
    if (kk == 0) return;
    if (kk < k) k = kk;
  }
  __shared__ cplx sA[GB_K][GB_M + 1];
  __shared__ cplx sB[GB_K][GB_N + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int i0 = blockIdx.y * GB_M, j0 = blockIdx.x * GB_N;
  cplx acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = cmake(0.0, 0.0);
  for (int k0 = 0; k0 < k; k0 += GB_K) {
    for (int e = threadIdx.x; e < GB_M * GB_K; e += 256) {
      int kk, ii;
      if (opA == 'N') { ii = e % GB_M; kk = e / GB_M; } else { kk = e % GB_K; ii = e / GB_K; }
      sA[kk][ii] = load_op(A, lda, i0 + ii, k0 + kk, m, k, opA);
      int jj, kb;
      if (opB == 'N') { kb = e % GB_K; jj = e / GB_K; } else { jj = e % GB_N; kb = e / GB_N; }
      sB[kb][jj] = load_op(B, ldb, k0 + kb, j0 + jj, k, nn, opB);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GB_K; ++kk) {
      cplx av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = sA[kk][ty + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) bv[b] = sB[kk][tx + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = cfma(av[a], bv[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    int i = i0 + ty + 16 * a;
    if (i >= m) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      int j = j0 + tx + 16 * b;
      if (j >= nn) continue;
      cplx v = acc[a][b];
      if (rs) v = cscale(v, rs[i]);
      if (cs) v = cscale(v, cs[j]);
      v = cmul(alpha, v);
      cplx* cp = &C[(size_t)j * ldc + i];
      if (beta.x != 0.0 || beta.y != 0.0) v = cfma(beta, *cp, v);
      *cp = v;
    }
  }
}

// ---------------------------------------------------------------------------
// warp / block reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ cplx warp_sum(cplx v) { return cmake(warp_sum(v.x), warp_sum(v.y)); }

// block-wide sum, deterministic (fixed tree); all threads get the result.
__device__ double block_sum(double v, double* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  double t = 0.0;
  for (int q = 0; q < nw; ++q) t += scratch[q];
  return t;
}

// ---------------------------------------------------------------------------
// column-pivoted QR (cooperative, one grid barrier per column step)
// ---------------------------------------------------------------------------
constexpr int QR_THREADS = 256;
constexpr int QR_MAXT = 32;   // elements per lane of one column (n <= 1024)
constexpr int CAND_PER_LANE = 8;   // per-CTA pivot candidates read per lane: grids of at most 256 CTAs

// Candidate of the next pivot: the CTA-local maximum of the partial norms
// and its logical position (ties: smaller position, as LAPACK's idamax).
// Norms are >= +0, so their bit patterns order like their values: the
// comparison runs on the integer units, not the FP64 unit.
__device__ __forceinline__ bool cand_better(double v, int q, double bv, int bq) {
  const long long a = __double_as_longlong(v), b = __double_as_longlong(bv);
  return a > b || (a == b && q < bq);
}

// Complex warp sum with five FP64 adds: after one exchange the low half of
// the warp reduces the real parts and the high half the imaginary parts.
__device__ __forceinline__ cplx warp_sum_c(cplx v) {
  const int lane = threadIdx.x & 31;
  const bool hi = lane & 16;
  double keep = hi ? v.y : v.x;
  const double send = hi ? v.x : v.y;
  keep += __shfl_xor_sync(0xffffffffu, send, 16);
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o);
  return cmake(__shfl_sync(0xffffffffu, keep, 0), __shfl_sync(0xffffffffu, keep, 16));
}

// a -= c v over the column slots of one lane (c = f at r = k, f scal below,
// v_k = 1), stored back; with TAIL the squared norm of the updated rows > k.
template <bool TAIL>
__device__ __forceinline__ double qr_update_column(cplx (&x)[QR_MAXT], cplx* __restrict__ col, const cplx* v, int k,
                                                   int n, int nq, int lane, cplx f, cplx fs) {
  double tp = 0.0;
#pragma unroll
  for (int q = 0; q < QR_MAXT; ++q) {
    if (q >= nq) break;
    const int r = k + lane + 32 * q;
    if (r < n) {
      // four fused multiply-adds per element
      const cplx vr = r == k ? cmake(1.0, 0.0) : v[r];
      const cplx c = r == k ? f : fs;
      x[q] = cmake(fma(-c.x, vr.x, fma(c.y, vr.y, x[q].x)), fma(-c.x, vr.y, fma(-c.y, vr.x, x[q].y)));
      col[r] = x[q];
      if (TAIL && r > k) tp = fma(x[q].x, x[q].x, fma(x[q].y, x[q].y, tp));
    }
  }
  return tp;
}

// sum_{r > k} conj(x_r) a_r over one lane's slots (loads the column into x)
__device__ __forceinline__ cplx qr_load_dot(cplx (&x)[QR_MAXT], const cplx* __restrict__ col, const cplx* v, int k,
                                            int n, int nq, int lane) {
  cplx sp = cmake(0.0, 0.0);
#pragma unroll
  for (int q = 0; q < QR_MAXT; ++q) {
    if (q >= nq) break;
    const int r = k + lane + 32 * q;
    x[q] = cmake(0.0, 0.0);
    if (r < n) {
      x[q] = ldcg_c(&col[r]);
      if (r > k) sp = cfma_conj(v[r], x[q], sp);
    }
  }
  return warp_sum_c(sp);
}

// loads one lane's slots of a column into x (as qr_load_dot, without the dot)
__device__ __forceinline__ void qr_load(cplx (&x)[QR_MAXT], const cplx* __restrict__ col, int k, int n, int nq,
                                        int lane) {
#pragma unroll
  for (int q = 0; q < QR_MAXT; ++q) {
    if (q >= nq) break;
    const int r = k + lane + 32 * q;
    x[q] = r < n ? ldcg_c(&col[r]) : cmake(0.0, 0.0);
  }
}

// sum_{r > k} conj(x_r) a_r over one lane's slots already in x (the order of qr_load_dot)
__device__ __forceinline__ cplx qr_dot(const cplx (&x)[QR_MAXT], const cplx* v, int k, int n, int nq, int lane) {
  cplx sp = cmake(0.0, 0.0);
#pragma unroll
  for (int q = 0; q < QR_MAXT; ++q) {
    if (q >= nq) break;
    const int r = k + lane + 32 * q;
    if (r < n && r > k) sp = cfma_conj(v[r], x[q], sp);
  }
  return warp_sum_c(sp);
}

// One column step after the dot product s0 = sum_{r>k} conj(x_r) a_r:
// a -= tau^H (v^H a) v with v = (1, scal x_{k+1..n}), then the partial norm
// downdate of zlaqp2 with stored reciprocals (vn1, vn2 at [j], 1/vn1, 1/vn2
// at [n + j]); returns the new partial norm.
__device__ __forceinline__ double qr_finish_column(cplx (&x)[QR_MAXT], cplx* __restrict__ col, const cplx* v, int k,
                                                   int n, int nq, int lane, int j, cplx s0, cplx ctau, cplx scal,
                                                   const QRWork& w, double tol3z) {
  const double vn1 = __ldcg(&w.vn1[j]), vn2 = __ldcg(&w.vn2[j]);
  const double inv1 = __ldcg(&w.vn1[n + j]), inv2 = __ldcg(&w.vn2[n + j]);
  // v^H a = a_k + conj(scal) s0
  const cplx ak = cmake(__shfl_sync(0xffffffffu, x[0].x, 0), __shfl_sync(0xffffffffu, x[0].y, 0));
  const cplx s = cfma_conj(scal, s0, ak);
  const cplx f = cmul(ctau, s);     // a_k -= f
  const cplx fs = cmul(f, scal);    // a_r -= f scal x_r, r > k
  // zlaqp2: temp = max(0, 1 - (|a_k|/vn1)^2), temp2 = temp (vn1/vn2)^2;
  // recompute the norm when temp2 <= sqrt(eps), else vn1 *= sqrt(temp)
  double vn1_new = vn1, inv1_new = inv1;
  bool recompute = false;
  if (vn1 != 0.0) {
    const cplx xk = csub(ak, f);
    double temp = 1.0 - (cabs2(xk) * inv1) * inv1;
    temp = temp > 0.0 ? temp : 0.0;
    const double r2 = vn1 * inv2;
    if (temp * r2 * r2 <= tol3z) {
      recompute = true;
    } else {
      const double rs = rsqrt(temp);
      vn1_new = vn1 * temp * rs;
      inv1_new = inv1 * rs;
    }
  }
  if (recompute) {
    const double tail = warp_sum(qr_update_column<true>(x, col, v, k, n, nq, lane, f, fs));
    vn1_new = (k < n - 1) ? sqrt(tail) : 0.0;
    inv1_new = vn1_new > 0.0 ? 1.0 / vn1_new : 0.0;
    if (lane == 0) { w.vn2[j] = vn1_new; w.vn2[n + j] = inv1_new; }
  } else {
    qr_update_column<false>(x, col, v, k, n, nq, lane, f, fs);
  }
  if (lane == 0 && vn1 != 0.0) { w.vn1[j] = vn1_new; w.vn1[n + j] = inv1_new; }
  return vn1_new;
}

__global__ void __launch_bounds__(QR_THREADS) k_qrp(cplx* __restrict__ A, int n, QRWork w) {
  unsigned bar_epoch = 0;
  GridBarrierExit bar_exit(w.bar);
  extern __shared__ double smem_qr[];
  cplx* v = reinterpret_cast<cplx*>(smem_qr);         // (n) pivot column: a_k at k, unscaled x below
  int* order = reinterpret_cast<int*>(v + n);         // (n) logical -> physical
  __shared__ double red[32];
  __shared__ int redi[32];
  __shared__ double nsum[32];
  __shared__ cplx s_tau, s_scal;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int warps = QR_THREADS / 32;
  const int scal_warp = warps - 1;   // holds no column while rem < (warps - 1) * grid
  const int gwarp = blockIdx.x * warps + wid, nwarps = gridDim.x * warps;
  const double tol3z = sqrt(DBL_EPSILON);

  for (int q = threadIdx.x; q < n; q += blockDim.x) order[q] = q;
  // initial column norms (zgeqp3: vn1 = vn2 = ||A(:, j)||) and the first candidates
  double cb = 0.0;
  int cq = n;
  for (int j = gwarp; j < n; j += nwarps) {
    double s = 0.0;
    for (int r = lane; r < n; r += 32) s += cabs2(A[(size_t)j * n + r]);
    s = warp_sum(s);
    const double nv = sqrt(s), iv = nv > 0.0 ? 1.0 / nv : 0.0;
    if (lane == 0) { w.vn1[j] = nv; w.vn2[j] = nv; w.vn1[n + j] = iv; w.vn2[n + j] = iv; }
    if (cand_better(nv, j, cb, cq)) { cb = nv; cq = j; }
  }
  if (lane == 0) { red[wid] = cb; redi[wid] = cq; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = red[0]; int bq = redi[0];
    for (int q = 1; q < warps; ++q)
      if (cand_better(red[q], redi[q], b, bq)) { b = red[q]; bq = redi[q]; }
    w.cand_v[blockIdx.x] = b;
    w.cand_q[blockIdx.x] = bq;
  }
  if (!grid_barrier(w.bar, w.err, bar_epoch)) return;

  const int chunk = (n + gridDim.x - 1) / gridDim.x;   // rows of V written by this CTA
  for (int k = 0; k < n; ++k) {
    const int rem = n - k - 1;
    const int nq = (n - k + 31) >> 5;   // warp-uniform: no FP64 work on fully masked slots
    const int t_first = blockIdx.x + gridDim.x * wid;
    // the first column of this warp, read while the pivot is chosen; if the
    // pivot exchange moves another column to its position, it is read again
    cplx x[QR_MAXT];
    int j_pre = -1;
    if (t_first < rem && wid != scal_warp) {
      j_pre = order[k + 1 + t_first];
      qr_load(x, A + (size_t)j_pre * n, k, n, nq, lane);
    }
    // ---- pivot: best of the per-CTA candidates (first position of maximal norm), warp 0 ----
    if (wid == 0) {
      // all candidate loads in flight at once (grid <= 32 * CAND_PER_LANE), then the compares
      double cvv[CAND_PER_LANE];
      int cqq[CAND_PER_LANE];
#pragma unroll
      for (int u = 0; u < CAND_PER_LANE; ++u) {
        const int c = lane + 32 * u;
        cvv[u] = 0.0;
        cqq[u] = n;
        if (c < (int)gridDim.x) { cvv[u] = __ldcg(&w.cand_v[c]); cqq[u] = __ldcg(&w.cand_q[c]); }
      }
      double best = 0.0;
      int bestq = n;
#pragma unroll
      for (int u = 0; u < CAND_PER_LANE; ++u)
        if (cand_better(cvv[u], cqq[u], best, bestq)) { best = cvv[u]; bestq = cqq[u]; }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        double ob = __shfl_xor_sync(0xffffffffu, best, o);
        int oq = __shfl_xor_sync(0xffffffffu, bestq, o);
        if (cand_better(ob, oq, best, bestq)) { best = ob; bestq = oq; }
      }
      if (lane == 0) {
        if (bestq < k || bestq >= n) bestq = k;   // no candidate: keep the order
        int t = order[k]; order[k] = order[bestq]; order[bestq] = t;
      }
    }
    __syncthreads();
    const int p = order[k];
    // ---- reflector from A[k:n, p] (zlarfg): partial squared norms, 4 loads per thread at n <= 1024 ----
    double xn2 = 0.0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = k + threadIdx.x + u * QR_THREADS;
      if (r < n) {
        cplx x = ldcg_c(&A[(size_t)p * n + r]);
        v[r] = x;
        if (r > k) xn2 = fma(x.x, x.x, fma(x.y, x.y, xn2));
      }
    }
    xn2 = warp_sum(xn2);
    if (lane == 0) nsum[wid] = xn2;
    __syncthreads();
    // ---- one warp forms beta, tau and the reflector scale while the others
    //      start the dot products of their first column (which need neither) ----
    if (wid == scal_warp) {
      double t = lane < warps ? nsum[lane] : 0.0;
#pragma unroll
      for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);   // warps <= 8
      const cplx alpha = v[k];
      double beta;
      cplx tau, scal;
      if (t == 0.0 && alpha.y == 0.0) {
        tau = cmake(0.0, 0.0);
        beta = alpha.x;
        scal = cmake(0.0, 0.0);
      } else {
        const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + t);
        beta = alpha.x >= 0.0 ? -nrm : nrm;
        const double rb = 1.0 / beta;
        tau = cmake((beta - alpha.x) * rb, -alpha.y * rb);
        // scal = 1 / (alpha - beta), formed on (alpha - beta) / nrm (modulus in [1, 2])
        const double an = fabs(rb);
        const cplx dd = cmake((alpha.x - beta) * an, alpha.y * an);
        const double rd = an / (dd.x * dd.x + dd.y * dd.y);
        scal = cmake(dd.x * rd, -dd.y * rd);
      }
      if (lane == 0) {
        s_tau = tau;
        s_scal = scal;
        if (blockIdx.x == 0) { w.tau[k] = tau; w.beta[k] = beta; }
      }
    }
    // ---- apply H_k^H to the remaining columns, downdate their norms ----
    // remaining logical positions k+1..n-1 are dealt round-robin over the CTAs
    // first, so every SM keeps an equal share of the columns as k grows
    double cbest = 0.0;
    int cbq = n;
    cplx s_first = cmake(0.0, 0.0);
    int j_first = -1;
    if (t_first < rem && wid != scal_warp) {
      j_first = order[k + 1 + t_first];
      if (j_first != j_pre) qr_load(x, A + (size_t)j_first * n, k, n, nq, lane);
      s_first = qr_dot(x, v, k, n, nq, lane);
    }
    __syncthreads();   // tau, scal visible
    const cplx ctau = cconj(s_tau), scal = s_scal;
    // rows of V written by this CTA: v = (1, scal x_{k+1..n}), zero above k
    for (int r = blockIdx.x * chunk + threadIdx.x; r < n && r < (blockIdx.x + 1) * chunk; r += blockDim.x)
      w.V[(size_t)k * n + r] = r < k ? cmake(0.0, 0.0) : (r == k ? cmake(1.0, 0.0) : cmul(v[r], scal));
    if (j_first >= 0) {
      const double nv = qr_finish_column(x, A + (size_t)j_first * n, v, k, n, nq, lane, j_first, s_first, ctau, scal,
                                         w, tol3z);
      if (lane == 0 && cand_better(nv, k + 1 + t_first, cbest, cbq)) { cbest = nv; cbq = k + 1 + t_first; }
    }
    // further columns of this warp (more columns than warps), and the scal
    // warp's share when it has one
    for (int t = (wid == scal_warp ? t_first : t_first + gridDim.x * warps); t < rem; t += gridDim.x * warps) {
      const int qpos = k + 1 + t;
      const int j = order[qpos];
      cplx* col = A + (size_t)j * n;
      const cplx s0 = qr_load_dot(x, col, v, k, n, nq, lane);
      const double nv = qr_finish_column(x, col, v, k, n, nq, lane, j, s0, ctau, scal, w, tol3z);
      if (lane == 0 && cand_better(nv, qpos, cbest, cbq)) { cbest = nv; cbq = qpos; }
    }
    // this CTA's candidate for the next pivot (lane 0 of each warp holds its best)
    if (lane == 0) { red[wid] = cbest; redi[wid] = cbq; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = red[0]; int bq = redi[0];
      for (int q = 1; q < warps; ++q)
        if (cand_better(red[q], redi[q], b, bq)) { b = red[q]; bq = redi[q]; }
      w.cand_v[blockIdx.x] = b;
      w.cand_q[blockIdx.x] = bq;
    }
    if (!grid_barrier(w.bar, w.err, bar_epoch)) return;
  }
  if (blockIdx.x == 0)
    for (int q = threadIdx.x; q < n; q += blockDim.x) w.order[q] = order[q];
}

// ---------------------------------------------------------------------------
// LU pivot search helpers: candidates compared on the bit patterns of the
// non-negative |Re| + |Im| (first row of maximal value, as izamax)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool piv_better(double v, int r, double bv, int br) {
  const long long a = __double_as_longlong(v), b = __double_as_longlong(bv);   // v >= 0
  return a > b || (a == b && r < br);
}

__device__ __forceinline__ void warp_argmax(double& best, int& row) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int orow = __shfl_xor_sync(0xffffffffu, row, o);
    if (piv_better(ob, orow, best, row)) { best = ob; row = orow; }
  }
}

// Block j of the compact-WY form of Q = H_0 ... H_{n-1}: Vb (m x b, m = n - jb,
// leading dimension m) = rows jb.. of reflector columns jb..jb+b; a reflector
// with tau = 0 is the identity and is stored as v = 0 with tau' = 1, so that
// T^-1 = diag(1/tau') + striu(Vb^H Vb) stays valid.  trd = tau'.
__global__ void k_wy_prep(const cplx* __restrict__ V, const cplx* __restrict__ tau, int n, int jb, int b,
                          cplx* __restrict__ Vb, cplx* __restrict__ trd) {
  const int m = n - jb;
  const size_t total = (size_t)m * b;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / m), r = (int)(e - (size_t)c * m);
    const cplx t = tau[jb + c];
    const bool ident = t.x == 0.0 && t.y == 0.0;
    Vb[e] = ident ? cmake(0.0, 0.0) : V[(size_t)(jb + c) * n + jb + r];
    if (r == 0) trd[c] = ident ? cmake(1.0, 0.0) : t;
  }
}

// Unblocked LU with partial pivoting (cooperative, one grid barrier per
// column step), for small n where the blocked form's launches dominate:
// P A = L U as LAPACK zgetf2 (pivot: first row of maximal |Re| + |Im|, as
// izamax), rows exchanged physically in the trailing columns.  Column k of
// A is read, never written, in step k: the multipliers go to Lb (strictly
// lower part; earlier columns receive the same row exchanges) and the
// diagonal of U to udiag, so the CTAs need no ordering among themselves
// inside a step.  The owner of column k+1 publishes the next pivot row.
__global__ void __launch_bounds__(QR_THREADS) k_lup(cplx* __restrict__ A, cplx* __restrict__ Lb, int n, LUKernel w) {
  unsigned bar_epoch = 0;
  GridBarrierExit bar_exit(w.bar);
  extern __shared__ double smem_lu[];
  cplx* v = reinterpret_cast<cplx*>(smem_lu);   // (n) column k after the row exchange (rows > k)
  int* perm = reinterpret_cast<int*>(v + n);    // (n) position -> original row
  __shared__ cplx s_rinv;
  __shared__ int s_piv;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int warps = QR_THREADS / 32;
  const int scal_warp = warps - 1;
  for (int q = threadIdx.x; q < n; q += blockDim.x) perm[q] = q;
  if (blockIdx.x == 0 && wid == 0) {
    double best = 0.0;
    int row = n;
    for (int r = lane; r < n; r += 32) {
      const cplx x = A[r];
      const double a = fabs(x.x) + fabs(x.y);
      if (piv_better(a, r, best, row)) { best = a; row = r; }
    }
    warp_argmax(best, row);
    if (lane == 0) w.pivrow[0] = row < n ? row : 0;
  }
  if (!grid_barrier(w.bar, w.err, bar_epoch)) return;

  const int chunk = (n + gridDim.x - 1) / gridDim.x;   // rows of Lb written by this CTA
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) s_piv = __ldcg(&w.pivrow[k & 1]);
    __syncthreads();
    const int p = s_piv;
    const cplx* colk = A + (size_t)k * n;
    const cplx piv = ldcg_c(&colk[p]);
    for (int r = k + 1 + threadIdx.x; r < n; r += blockDim.x) v[r] = ldcg_c(&colk[r == p ? k : r]);
    if (threadIdx.x == 0 && p != k) { const int t = perm[k]; perm[k] = perm[p]; perm[p] = t; }
    if (wid == scal_warp) {
      const bool zero = piv.x == 0.0 && piv.y == 0.0;
      const cplx rinv = zero ? cmake(0.0, 0.0) : cdiv(cmake(1.0, 0.0), piv);
      if (lane == 0) {
        s_rinv = rinv;
        if (blockIdx.x == 0) {
          w.udiag[k] = piv;
          w.rdiag[k] = rinv;
          if (zero) atomicOr(w.err, DQMC_KERR_SINGULAR);
        }
      }
    }
    // the same row exchange in the multiplier columns formed so far
    if (p != k)
      for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < k; j += gridDim.x * blockDim.x) {
        cplx* lj = Lb + (size_t)j * n;
        const cplx a = ldcg_c(&lj[k]), b = ldcg_c(&lj[p]);
        lj[k] = b;
        lj[p] = a;
      }
    __syncthreads();   // v, s_rinv
    const cplx rinv = s_rinv;
    {
      const int r0 = blockIdx.x * chunk, r1 = r0 + chunk < n ? r0 + chunk : n;
      for (int r = (r0 > k + 1 ? r0 : k + 1) + threadIdx.x; r < r1; r += blockDim.x)
        Lb[(size_t)k * n + r] = cmul(v[r], rinv);
    }
    // ---- trailing columns j > k, dealt round-robin over the CTAs ----
    const int rem = n - k - 1;
    const int nq = (rem + 31) >> 5;   // warp-uniform slot count of rows k+1..n-1
    for (int t = blockIdx.x + gridDim.x * wid; t < rem; t += gridDim.x * warps) {
      const int j = k + 1 + t;
      cplx* col = A + (size_t)j * n;
      const cplx u = ldcg_c(&col[p]), wk = ldcg_c(&col[k]);
      cplx x[QR_MAXT];
#pragma unroll
      for (int q = 0; q < QR_MAXT; ++q) {
        if (q >= nq) break;
        const int r = k + 1 + lane + 32 * q;
        x[q] = r < n ? (r == p ? wk : ldcg_c(&col[r])) : cmake(0.0, 0.0);
      }
      const cplx c = cmul(u, rinv);   // a_rj -= (a_rk / piv) u_kj
      double best = 0.0;
      int brow = n;
#pragma unroll
      for (int q = 0; q < QR_MAXT; ++q) {
        if (q >= nq) break;
        const int r = k + 1 + lane + 32 * q;
        if (r < n) {
          const cplx vr = v[r];
          x[q] = cmake(fma(-vr.x, c.x, fma(vr.y, c.y, x[q].x)), fma(-vr.x, c.y, fma(-vr.y, c.x, x[q].y)));
          col[r] = x[q];
          if (t == 0) {
            const double a = fabs(x[q].x) + fabs(x[q].y);
            if (piv_better(a, r, best, brow)) { best = a; brow = r; }
          }
        }
      }
      if (lane == 0) col[k] = u;
      if (t == 0) {   // column k+1: pivot row of the next step
        warp_argmax(best, brow);
        if (lane == 0) w.pivrow[(k + 1) & 1] = brow < n ? brow : k + 1;
      }
    }
    if (!grid_barrier(w.bar, w.err, bar_epoch)) return;
  }
  if (blockIdx.x == 0)
    for (int q = threadIdx.x; q < n; q += blockDim.x) w.perm[q] = perm[q];
}

// ---------------------------------------------------------------------------
// blocked LU with partial pivoting (zgetrf semantics, in place)
// ---------------------------------------------------------------------------
// Panel of LU_PB columns [p0, p0 + b) over rows [p0, n), rows dealt to the CTAs
// in contiguous chunks.  Per column step the CTAs publish their pivot
// candidate (|Re| + |Im|, row, and that row's panel values) and the owner of
// row k publishes row k; after the grid barrier every CTA reads the pivot
// row (the U row) and row k (which moves to the pivot's place) from those
// copies, so no CTA reads a row another one is rewriting.
__global__ void __launch_bounds__(256) k_lu_panel(cplx* __restrict__ A, int n, int p0, int b, LUPanel w) {
  unsigned bar_epoch = 0;
  GridBarrierExit bar_exit(w.bar);
  extern __shared__ double4_16a smem_panel[];
  cplx* prow = reinterpret_cast<cplx*>(smem_panel);   // (own rows, LU_PB): this CTA's rows of the panel
  const int rows = n - p0;
  const int chunk = (rows + gridDim.x - 1) / gridDim.x;
  const int r0 = p0 + blockIdx.x * chunk;
  const int r1 = r0 + chunk < n ? r0 + chunk : n;
  const int nrw = r1 > r0 ? r1 - r0 : 0;
  __shared__ cplx urow[LU_PB], krow[LU_PB];
  __shared__ double s_v[8];
  __shared__ int s_r[8];
  __shared__ int s_p, s_wc;
  __shared__ cplx s_rinv;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int e = threadIdx.x; e < nrw * b; e += blockDim.x) {
    const int rr = e / b, j = e - rr * b;
    prow[rr * LU_PB + j] = ldcg_c(&A[(size_t)(p0 + j) * n + r0 + rr]);
  }
  __syncthreads();

  // candidate of this CTA for panel column jc over its rows >= rlo, published with the row's panel values
  auto publish_candidate = [&](int jc, int rlo) {
    double best = 0.0;
    int brow = n;
    for (int r = (r0 > rlo ? r0 : rlo) + threadIdx.x; r < r1; r += blockDim.x) {
      const cplx x = prow[(r - r0) * LU_PB + jc];
      const double a = fabs(x.x) + fabs(x.y);
      if (piv_better(a, r, best, brow)) { best = a; brow = r; }
    }
    warp_argmax(best, brow);
    if (lane == 0) { s_v[wid] = best; s_r[wid] = brow; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double bv = s_v[0]; int br = s_r[0];
      for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
        if (piv_better(s_v[q], s_r[q], bv, br)) { bv = s_v[q]; br = s_r[q]; }
      w.cand_v[blockIdx.x] = bv;
      w.cand_r[blockIdx.x] = br;
      s_r[0] = br;
    }
    __syncthreads();
    const int br = s_r[0];
    if (br < n)
      for (int j = threadIdx.x; j < b; j += blockDim.x)
        w.cand_rows[(size_t)blockIdx.x * LU_PB + j] = prow[(br - r0) * LU_PB + j];
  };
  auto publish_rowk = [&](int k, int slot) {
    if (r0 <= k && k < r1)
      for (int j = threadIdx.x; j < b; j += blockDim.x) w.rowk[slot * LU_PB + j] = prow[(k - r0) * LU_PB + j];
  };

  publish_candidate(0, p0);
  publish_rowk(p0, 0);
  if (!grid_barrier(w.bar, w.err, bar_epoch)) return;

  for (int kk = 0; kk < b; ++kk) {
    const int k = p0 + kk;
    // ---- pivot: best candidate (first row of maximal |Re| + |Im|) ----
    if (wid == 0) {
      // all candidate loads in flight at once (grid <= 32 * CAND_PER_LANE), then the compares
      double cvv[CAND_PER_LANE];
      int crr[CAND_PER_LANE];
#pragma unroll
      for (int u = 0; u < CAND_PER_LANE; ++u) {
        const int c = lane + 32 * u;
        cvv[u] = 0.0;
        crr[u] = n;
        if (c < (int)gridDim.x) { cvv[u] = __ldcg(&w.cand_v[c]); crr[u] = __ldcg(&w.cand_r[c]); }
      }
      double best = 0.0;
      int brow = n, bc = 0;
#pragma unroll
      for (int u = 0; u < CAND_PER_LANE; ++u)
        if (piv_better(cvv[u], crr[u], best, brow)) { best = cvv[u]; brow = crr[u]; bc = lane + 32 * u; }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int orow = __shfl_xor_sync(0xffffffffu, brow, o), oc = __shfl_xor_sync(0xffffffffu, bc, o);
        if (piv_better(ob, orow, best, brow)) { best = ob; brow = orow; bc = oc; }
      }
      if (lane == 0) { s_p = brow; s_wc = bc; }
    }
    __syncthreads();
    const bool none = s_p >= n;   // all candidates zero: no exchange, singular pivot
    const int p = none ? k : s_p;
    for (int j = threadIdx.x; j < b; j += blockDim.x) {
      const cplx kv = ldcg_c(&w.rowk[(kk & 1) * LU_PB + j]);
      krow[j] = kv;
      urow[j] = none ? kv : ldcg_c(&w.cand_rows[(size_t)s_wc * LU_PB + j]);
    }
    __syncthreads();
    if (wid == 0) {
      // 1 / pivot = conj(pv) / |pv|^2 (the D-scale separated matrix has no large scales)
      const cplx pv = urow[kk];
      const double d2 = pv.x * pv.x + pv.y * pv.y;
      const bool zero = d2 == 0.0;
      const double rd = zero ? 0.0 : 1.0 / d2;
      if (lane == 0) {
        s_rinv = cmake(pv.x * rd, -pv.y * rd);
        if (zero) atomicOr(w.err, DQMC_KERR_SINGULAR);
        if (blockIdx.x == 0) w.piv[k] = p;
      }
    }
    // the exchanged rows: row k <- pivot row (U), row p <- old row k
    if (r0 <= k && k < r1)
      for (int j = threadIdx.x; j < b; j += blockDim.x) prow[(k - r0) * LU_PB + j] = urow[j];
    if (p != k && r0 <= p && p < r1)
      for (int j = threadIdx.x; j < b; j += blockDim.x) prow[(p - r0) * LU_PB + j] = krow[j];
    __syncthreads();
    const cplx rinv = s_rinv;
    // ---- multipliers of the own rows below k, then the rank-1 update of the panel ----
    const int ra = r0 > k + 1 ? r0 : k + 1;
    const int nr = r1 > ra ? r1 - ra : 0;
    for (int t = threadIdx.x; t < nr; t += blockDim.x) {
      cplx* e = &prow[(ra + t - r0) * LU_PB + kk];
      *e = cmul(*e, rinv);
    }
    __syncthreads();
    const int nc = b - kk - 1;
    for (int t = threadIdx.x; t < nr * nc; t += blockDim.x) {
      const int rr = t % nr, jj = kk + 1 + t / nr;
      cplx* rowp = &prow[(ra + rr - r0) * LU_PB];
      const cplx l = rowp[kk], u = urow[jj], x = rowp[jj];
      rowp[jj] = cmake(fma(-l.x, u.x, fma(l.y, u.y, x.x)), fma(-l.x, u.y, fma(-l.y, u.x, x.y)));
    }
    __syncthreads();
    if (kk + 1 < b) {
      publish_candidate(kk + 1, k + 1);
      publish_rowk(k + 1, (kk + 1) & 1);
    }
    if (!grid_barrier(w.bar, w.err, bar_epoch)) return;
  }
  for (int e = threadIdx.x; e < nrw * b; e += blockDim.x) {
    const int rr = e / b, j = e - rr * b;
    A[(size_t)(p0 + j) * n + r0 + rr] = prow[rr * LU_PB + j];
  }
}

// The same panel factorisation on one thread-block cluster of cs CTAs (8 or
// 16, the rows dealt in contiguous chunks): each CTA keeps its candidate (value,
// row and the row's panel values) and, when it holds it, the step's row k in
// its own shared memory, double-buffered by step parity; the others read them
// through distributed shared memory after one cluster barrier per column, in
// place of the grid barrier and the round trips through L2.  Every CTA runs
// the same loop, so every cluster barrier is met by all of them; the last
// barrier of the loop also keeps each CTA's shared memory alive until the
// others have read it.
__global__ void __launch_bounds__(256) k_lu_panel_cluster(cplx* __restrict__ A, int n, int p0, int b, LUPanel w) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int cs = (int)cl.num_blocks(), q = (int)cl.block_rank();
  extern __shared__ double4_16a smem_panel[];
  cplx* prow = reinterpret_cast<cplx*>(smem_panel);   // (own rows, LU_PB): this CTA's rows of the panel
  const int rows = n - p0;
  const int chunk = (rows + cs - 1) / cs;
  const int r0 = p0 + q * chunk;
  const int r1 = r0 + chunk < n ? r0 + chunk : n;
  const int nrw = r1 > r0 ? r1 - r0 : 0;
  __shared__ cplx urow[LU_PB], krow[LU_PB];
  __shared__ cplx c_row[2][LU_PB], k_row[2][LU_PB];
  __shared__ double c_val[2];
  __shared__ int c_r[2];
  __shared__ double s_v[8];
  __shared__ int s_r[8];
  __shared__ int s_p, s_wc;
  __shared__ cplx s_rinv;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int e = threadIdx.x; e < nrw * b; e += blockDim.x) {
    const int rr = e / b, j = e - rr * b;
    prow[rr * LU_PB + j] = ldcg_c(&A[(size_t)(p0 + j) * n + r0 + rr]);
  }
  __syncthreads();

  // candidate of this CTA for panel column jc over its rows >= k (value, row,
  // row values), and row k itself if this CTA holds it, into buffers par
  auto publish = [&](int jc, int k, int par) {
    double best = 0.0;
    int brow = n;
    for (int r = (r0 > k ? r0 : k) + threadIdx.x; r < r1; r += blockDim.x) {
      const cplx x = prow[(r - r0) * LU_PB + jc];
      const double a = fabs(x.x) + fabs(x.y);
      if (piv_better(a, r, best, brow)) { best = a; brow = r; }
    }
    warp_argmax(best, brow);
    if (lane == 0) { s_v[wid] = best; s_r[wid] = brow; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double bv = s_v[0]; int br = s_r[0];
      for (int u = 1; u < (int)(blockDim.x >> 5); ++u)
        if (piv_better(s_v[u], s_r[u], bv, br)) { bv = s_v[u]; br = s_r[u]; }
      c_val[par] = bv;
      c_r[par] = br;
      s_r[0] = br;
    }
    __syncthreads();
    const int br = s_r[0];
    if (br < n)
      for (int j = threadIdx.x; j < b; j += blockDim.x) c_row[par][j] = prow[(br - r0) * LU_PB + j];
    if (r0 <= k && k < r1)
      for (int j = threadIdx.x; j < b; j += blockDim.x) k_row[par][j] = prow[(k - r0) * LU_PB + j];
  };

  publish(0, p0, 0);
  cl.sync();

  for (int kk = 0; kk < b; ++kk) {
    const int k = p0 + kk, par = kk & 1;
    // ---- pivot: best of the cs candidates (first row of maximal |Re| + |Im|) ----
    if (wid == 0) {
      double best = 0.0;
      int brow = n, bc = 0;
      if (lane < cs) {
        best = *cl.map_shared_rank(&c_val[par], lane);
        brow = *cl.map_shared_rank(&c_r[par], lane);
        bc = lane;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int orow = __shfl_xor_sync(0xffffffffu, brow, o), oc = __shfl_xor_sync(0xffffffffu, bc, o);
        if (piv_better(ob, orow, best, brow)) { best = ob; brow = orow; bc = oc; }
      }
      if (lane == 0) { s_p = brow; s_wc = bc; }
    }
    __syncthreads();
    const bool none = s_p >= n;   // all candidates zero: no exchange, singular pivot
    const int p = none ? k : s_p;
    {
      const cplx* kr = cl.map_shared_rank(&k_row[par][0], (unsigned)((k - p0) / chunk));
      const cplx* ur = cl.map_shared_rank(&c_row[par][0], (unsigned)s_wc);
      for (int j = threadIdx.x; j < b; j += blockDim.x) {
        const cplx kv = kr[j];
        krow[j] = kv;
        urow[j] = none ? kv : ur[j];
      }
    }
    __syncthreads();
    if (wid == 0) {
      // 1 / pivot = conj(pv) / |pv|^2 (the D-scale separated matrix has no large scales)
      const cplx pv = urow[kk];
      const double d2 = pv.x * pv.x + pv.y * pv.y;
      const bool zero = d2 == 0.0;
      const double rd = zero ? 0.0 : 1.0 / d2;
      if (lane == 0) {
        s_rinv = cmake(pv.x * rd, -pv.y * rd);
        if (zero) atomicOr(w.err, DQMC_KERR_SINGULAR);
        if (q == 0) w.piv[k] = p;
      }
    }
    // the exchanged rows: row k <- pivot row (U), row p <- old row k
    if (r0 <= k && k < r1)
      for (int j = threadIdx.x; j < b; j += blockDim.x) prow[(k - r0) * LU_PB + j] = urow[j];
    if (p != k && r0 <= p && p < r1)
      for (int j = threadIdx.x; j < b; j += blockDim.x) prow[(p - r0) * LU_PB + j] = krow[j];
    __syncthreads();
    const cplx rinv = s_rinv;
    // ---- multipliers of the own rows below k, then the rank-1 update of the panel ----
    const int ra = r0 > k + 1 ? r0 : k + 1;
    const int nr = r1 > ra ? r1 - ra : 0;
    for (int t = threadIdx.x; t < nr; t += blockDim.x) {
      cplx* e = &prow[(ra + t - r0) * LU_PB + kk];
      *e = cmul(*e, rinv);
    }
    __syncthreads();
    const int nc = b - kk - 1;
    for (int t = threadIdx.x; t < nr * nc; t += blockDim.x) {
      const int rr = t % nr, jj = kk + 1 + t / nr;
      cplx* rowp = &prow[(ra + rr - r0) * LU_PB];
      const cplx l = rowp[kk], u = urow[jj], x = rowp[jj];
      rowp[jj] = cmake(fma(-l.x, u.x, fma(l.y, u.y, x.x)), fma(-l.x, u.y, fma(-l.y, u.x, x.y)));
    }
    __syncthreads();
    if (kk + 1 < b) publish(kk + 1, k + 1, (kk + 1) & 1);
    cl.sync();
  }
  for (int e = threadIdx.x; e < nrw * b; e += blockDim.x) {
    const int rr = e / b, j = e - rr * b;
    A[(size_t)(p0 + j) * n + r0 + rr] = prow[rr * LU_PB + j];
  }
}

// Row exchanges of one panel applied to the columns outside it, and to the
// running permutation: the b exchanges (k, piv[k]) touch at most 2b rows,
// whose net permutation warp 0 works out (panel rows indexed directly, rows
// below the panel found by a ballot over the ones met so far); every column
// is then gathered over those rows.
__global__ void k_lu_apply_swaps(cplx* __restrict__ A, int n, int p0, int b, const int* __restrict__ piv,
                                 int* __restrict__ perm) {
  __shared__ int rowof[2 * LU_PB], src[2 * LU_PB], spiv[LU_PB];
  __shared__ int s_cnt;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    for (int s2 = lane; s2 < b; s2 += 32) {
      rowof[s2] = p0 + s2;
      src[s2] = p0 + s2;
      spiv[s2] = piv[p0 + s2];
    }
    __syncwarp();
    int cnt = b;
    for (int kk = 0; kk < b; ++kk) {
      const int k = p0 + kk, pr = spiv[kk];
      if (pr == k) continue;   // warp-uniform
      int sp = -1;
      if (pr < p0 + b) {
        sp = pr - p0;
      } else {
        for (int base = b; base < cnt && sp < 0; base += 32) {
          const int s2 = base + lane;
          const unsigned hit = __ballot_sync(0xffffffffu, s2 < cnt && rowof[s2] == pr);
          if (hit) sp = base + __ffs(hit) - 1;
        }
        if (sp < 0) {
          sp = cnt++;
          if (lane == 0) { rowof[sp] = pr; src[sp] = pr; }
        }
      }
      __syncwarp();
      if (lane == 0) { const int t = src[kk]; src[kk] = src[sp]; src[sp] = t; }
      __syncwarp();
    }
    if (lane == 0) s_cnt = cnt;
  }
  __syncthreads();
  const int cnt = s_cnt;
  // permutation (block 0): perm[rowof[s]] <- old perm[src[s]]
  if (blockIdx.x == 0) {
    __shared__ int pv[2 * LU_PB];
    for (int s2 = threadIdx.x; s2 < cnt; s2 += blockDim.x) pv[s2] = perm[src[s2]];
    __syncthreads();
    for (int s2 = threadIdx.x; s2 < cnt; s2 += blockDim.x) perm[rowof[s2]] = pv[s2];
  }
  // columns outside the panel, one warp per column
  const int lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  for (int c = blockIdx.x * nw + (threadIdx.x >> 5); c < n; c += gridDim.x * nw) {
    if (c >= p0 && c < p0 + b) continue;
    cplx* col = A + (size_t)c * n;
    cplx v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int s2 = lane + 32 * q;
      if (s2 < cnt) v[q] = ldcg_c(&col[src[s2]]);
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int s2 = lane + 32 * q;
      if (s2 < cnt) col[rowof[s2]] = v[q];
    }
  }
}

// udiag = diag(U) of the in-place LU, rdiag = 1 / udiag
__global__ void k_lu_diag(const cplx* __restrict__ A, int n, cplx* __restrict__ udiag, cplx* __restrict__ rdiag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const cplx d = A[(size_t)i * n + i];
    udiag[i] = d;
    rdiag[i] = (d.x == 0.0 && d.y == 0.0) ? cmake(0.0, 0.0) : cdiv(cmake(1.0, 0.0), d);
  }
}

// C = A + B over count complex entries
__global__ void k_add(const cplx* __restrict__ A, const cplx* __restrict__ B, cplx* __restrict__ C, size_t count) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
    C[e] = cadd(A[e], B[e]);
}

__global__ void k_iota(int* __restrict__ p, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

// D-scale separation helpers: s[0..n) = 1/max(Dl,1), s[n..2n) = min(Dl,1),
// s[2n..3n) = 1/max(Dr,1), s[3n..4n) = min(Dr,1)
__global__ void k_split_scales(const double* __restrict__ Dl, const double* __restrict__ Dr, int n,
                               double* __restrict__ s) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double l = Dl[i], r = Dr[i];
    s[i] = 1.0 / (l > 1.0 ? l : 1.0);
    s[n + i] = l < 1.0 ? l : 1.0;
    s[2 * n + i] = 1.0 / (r > 1.0 ? r : 1.0);
    s[3 * n + i] = r < 1.0 ? r : 1.0;
  }
}

// out[0] = sum_i log|u_i| + log max(Dl_i, 1) + log max(Dr_i, 1)  (single CTA)
__global__ void k_lu_logdet(const cplx* __restrict__ udiag, const double* __restrict__ Dl,
                            const double* __restrict__ Dr, int n, double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double l = Dl[i], r = Dr[i];
    s += 0.5 * log(cabs2(udiag[i])) + log(l > 1.0 ? l : 1.0) + log(r > 1.0 ? r : 1.0);
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) out[0] = s;
}

// T (physical layout) = D^-1 R, zero below the logical diagonal; D = |beta|.
__global__ void k_qrp_finalize(const cplx* __restrict__ A, cplx* __restrict__ T, double* __restrict__ D, int n,
                               const int* __restrict__ order, const double* __restrict__ beta) {
  extern __shared__ int pos[];   // physical -> logical
  for (int q = threadIdx.x; q < n; q += blockDim.x) pos[order[q]] = q;
  __syncthreads();
  const size_t total = (size_t)n * n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    int j = (int)(e / n), r = (int)(e - (size_t)j * n);
    int q = pos[j];
    double d = fabs(beta[r]);
    cplx val;
    if (r < q) val = cscale(A[e], 1.0 / d);
    else if (r == q) val = cmake(beta[r] / d, 0.0);
    else val = cmake(0.0, 0.0);
    T[e] = val;
  }
  if (blockIdx.x == 0)
    for (int q = threadIdx.x; q < n; q += blockDim.x) D[q] = fabs(beta[q]);
}

// X (m x n) <- X * Q (or X * Q^H), one warp per row, row held in registers.
__global__ void __launch_bounds__(128) k_apply_q_right(cplx* __restrict__ X, int m, int n,
                                                      const cplx* __restrict__ V, const cplx* __restrict__ tau,
                                                      int conj_q) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (row >= m) return;
  cplx x[QR_MAXT];
#pragma unroll
  for (int t = 0; t < QR_MAXT; ++t) {
    int c = lane + 32 * t;
    x[t] = c < n ? X[(size_t)c * m + row] : cmake(0.0, 0.0);
  }
  for (int s = 0; s < n; ++s) {
    const int k = conj_q ? (n - 1 - s) : s;
    const cplx* vk = V + (size_t)k * n;
    cplx tk = tau[k];
    if (tk.x == 0.0 && tk.y == 0.0) continue;
    if (conj_q) tk = cconj(tk);
    // X H = X - tau (X v) v^H
    // one accumulator: the FP64 unit's issue rate, not its latency, bounds the chain
    cplx dp = cmake(0.0, 0.0);
    const int t0 = k >> 5, t1 = (n + 31) >> 5;   // warp-uniform range of slots holding columns >= k
#pragma unroll
    for (int t = 0; t < QR_MAXT; ++t) {
      if (t < t0) continue;
      if (t >= t1) break;
      int c = lane + 32 * t;
      if (c >= k && c < n) dp = cfma(x[t], __ldg(&vk[c]), dp);
    }
    cplx d = warp_sum_c(dp);
    cplx f = cmul(tk, d);
#pragma unroll
    for (int t = 0; t < QR_MAXT; ++t) {
      if (t < t0) continue;
      if (t >= t1) break;
      int c = lane + 32 * t;
      if (c >= k && c < n) {
        cplx vc = __ldg(&vk[c]);
        // x_c -= f * conj(v_c) with four fused multiply-adds
        x[t] = cmake(fma(-f.x, vc.x, fma(-f.y, vc.y, x[t].x)), fma(-f.y, vc.x, fma(f.x, vc.y, x[t].y)));
      }
    }
  }
#pragma unroll
  for (int t = 0; t < QR_MAXT; ++t) {
    int c = lane + 32 * t;
    if (c < n) X[(size_t)c * m + row] = x[t];
  }
}

// Y <- That^-1 Y, That[r, q] = T[r, order[q]] upper triangular (logical order).
// One warp per column of Y (column staged in shared memory).
__global__ void __launch_bounds__(128) k_trsm_left_upper(const cplx* __restrict__ T, const int* __restrict__ order,
                                                        const cplx* __restrict__ rdiag, cplx* __restrict__ Y, int n,
                                                        int m) {
  extern __shared__ double smem_t[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int col = blockIdx.x * (blockDim.x / 32) + wid;
  if (col >= m) return;
  cplx* y = reinterpret_cast<cplx*>(smem_t) + (size_t)wid * n;
  cplx* yg = Y + (size_t)col * n;
  for (int r = lane; r < n; r += 32) y[r] = yg[r];
  __syncwarp();
  for (int q = n - 1; q >= 0; --q) {
    const cplx* tq = T + (size_t)(order ? __ldg(&order[q]) : q) * n;
    cplx yq;
    if (rdiag) {
      yq = cmul(y[q], __ldg(&rdiag[q]));
    } else {
      // the unit-scaled factor of a QR has diagonal beta/|beta| = +-1: a sign, not a division
      const cplx d = __ldg(&tq[q]);
      yq = (d.y == 0.0 && fabs(d.x) == 1.0) ? cscale(y[q], d.x) : cdiv(y[q], d);
    }
    __syncwarp();
    if (lane == 0) y[q] = yq;
    for (int r = lane; r < q; r += 32) {
      const cplx t = __ldg(&tq[r]);
      y[r] = cmake(fma(-yq.x, t.x, fma(yq.y, t.y, y[r].x)), fma(-yq.x, t.y, fma(-yq.y, t.x, y[r].y)));
    }
    __syncwarp();
  }
  for (int r = lane; r < n; r += 32) yg[r] = y[r];
}

// Y <- L^-1 Y with L unit lower triangular (strictly lower part of Lc,
// column-major), one warp per column of Y (column staged in shared memory).
__global__ void __launch_bounds__(128) k_trsm_left_lower_unit(const cplx* __restrict__ Lc, cplx* __restrict__ Y, int n,
                                                             int m) {
  extern __shared__ double smem_t[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int col = blockIdx.x * (blockDim.x / 32) + wid;
  if (col >= m) return;
  cplx* y = reinterpret_cast<cplx*>(smem_t) + (size_t)wid * n;
  cplx* yg = Y + (size_t)col * n;
  for (int r = lane; r < n; r += 32) y[r] = yg[r];
  __syncwarp();
  for (int q = 0; q < n - 1; ++q) {
    const cplx* lq = Lc + (size_t)q * n;
    const cplx yq = y[q];
    for (int r = q + 1 + lane; r < n; r += 32) {
      const cplx t = __ldg(&lq[r]);
      y[r] = cmake(fma(-yq.x, t.x, fma(yq.y, t.y, y[r].x)), fma(-yq.x, t.y, fma(-yq.y, t.x, y[r].y)));
    }
    __syncwarp();
  }
  for (int r = lane; r < n; r += 32) yg[r] = y[r];
}

// Diagonal-block solve of a blocked triangular solve: the b x b block of T
// at (j0, j0) (leading dimension ldT) applied to rows j0..j0+b of the m
// columns of Y (leading dimension ldY).  lower: unit lower triangular,
// forward; otherwise upper with the reciprocal diagonal rdiag[j0 + q],
// backward.  Each CTA stages the strict triangle of the block, packed by
// columns, in shared memory once (no L2 round trip inside the dependent
// column steps); each warp solves one column with its b values in registers
// (row lane + 32 i in slot i) and broadcasts y_q by shuffle.
constexpr int TRSM_DB_WARPS = 8;
__device__ __forceinline__ int trsm_pack_lower(int q, int b) { return q * (b - 1) - q * (q - 1) / 2; }
__device__ __forceinline__ int trsm_pack_upper(int q) { return q * (q - 1) / 2; }

__global__ void __launch_bounds__(32 * TRSM_DB_WARPS) k_trsm_diag_block(const cplx* __restrict__ T, int ldT,
                                                                       const cplx* __restrict__ rdiag,
                                                                       cplx* __restrict__ Y, int ldY, int j0, int b,
                                                                       int m, int lower) {
  extern __shared__ double4_16a smem_tdb[];
  cplx* tp = reinterpret_cast<cplx*>(smem_tdb);   // (b (b - 1) / 2) packed strict triangle
  cplx* rd = tp + (size_t)b * (b - 1) / 2;        // (b) reciprocal diagonal (upper)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int bb = b * b;
  for (int e0 = threadIdx.x; e0 < bb; e0 += 8 * blockDim.x) {
    cplx v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = e0 + u * blockDim.x;
      const int q = e / b, r = e - q * b;
      if (e < bb && (lower ? r > q : r < q)) v[u] = __ldg(&T[(size_t)(j0 + q) * ldT + j0 + r]);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = e0 + u * blockDim.x;
      const int q = e / b, r = e - q * b;
      if (e < bb && (lower ? r > q : r < q))
        tp[lower ? trsm_pack_lower(q, b) + (r - q - 1) : trsm_pack_upper(q) + r] = v[u];
    }
  }
  if (!lower)
    for (int q = threadIdx.x; q < b; q += blockDim.x) rd[q] = __ldg(&rdiag[j0 + q]);
  __syncthreads();
  const int col = blockIdx.x * TRSM_DB_WARPS + wid;
  if (col >= m) return;
  cplx* yg = Y + (size_t)col * ldY + j0;
  cplx y[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = lane + 32 * i;
    y[i] = r < b ? yg[r] : cmake(0.0, 0.0);
  }
  auto bcast = [&](int q) {
    const int slot = q >> 5, src = q & 31;
    const cplx v = slot == 0 ? y[0] : slot == 1 ? y[1] : slot == 2 ? y[2] : y[3];
    return cmake(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
  };
  if (lower) {
    for (int q = 0; q < b - 1; ++q) {
      const cplx yq = bcast(q);
      const cplx* tq = tp + trsm_pack_lower(q, b) - q - 1;   // tq[r], r > q
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (32 * i + 31 <= q || 32 * i >= b) continue;   // warp-uniform
        const int r = lane + 32 * i;
        if (r > q && r < b) {
          const cplx t = tq[r];
          y[i] = cmake(fma(-yq.x, t.x, fma(yq.y, t.y, y[i].x)), fma(-yq.x, t.y, fma(-yq.y, t.x, y[i].y)));
        }
      }
    }
  } else {
    for (int q = b - 1; q >= 0; --q) {
      const cplx yq = cmul(bcast(q), rd[q]);
      const cplx* tq = tp + trsm_pack_upper(q);   // tq[r], r < q
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (32 * i > q) continue;   // warp-uniform
        const int r = lane + 32 * i;
        if (r == q) y[i] = yq;
        else if (r < q) {
          const cplx t = tq[r];
          y[i] = cmake(fma(-yq.x, t.x, fma(yq.y, t.y, y[i].x)), fma(-yq.x, t.y, fma(-yq.y, t.x, y[i].y)));
        }
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = lane + 32 * i;
    if (r < b) yg[r] = y[i];
  }
}

// Y <- Y That^-1 (Y is m x n), one warp per row: z That = y, forward over columns.
__global__ void __launch_bounds__(128) k_trsm_right_upper(const cplx* __restrict__ T, const int* __restrict__ order,
                                                         cplx* __restrict__ Y, int m, int n) {
  extern __shared__ double smem_t[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int row = blockIdx.x * (blockDim.x / 32) + wid;
  if (row >= m) return;
  cplx* z = reinterpret_cast<cplx*>(smem_t) + (size_t)wid * n;
  for (int c = lane; c < n; c += 32) z[c] = Y[(size_t)c * m + row];
  __syncwarp();
  for (int q = 0; q < n; ++q) {
    const cplx* tq = T + (size_t)__ldg(&order[q]) * n;
    cplx s = cmake(0.0, 0.0);
    for (int r = lane; r < q; r += 32) s = cfma(z[r], __ldg(&tq[r]), s);
    s = warp_sum(s);
    if (lane == 0) {
      const cplx d = __ldg(&tq[q]);
      const cplx t = csub(z[q], s);
      z[q] = (d.y == 0.0 && fabs(d.x) == 1.0) ? cscale(t, d.x) : cdiv(t, d);
    }
    __syncwarp();
  }
  for (int c = lane; c < n; c += 32) Y[(size_t)c * m + row] = z[c];
}

__global__ void k_permute(const cplx* __restrict__ src, cplx* __restrict__ dst, int rows, int cols,
                          const int* __restrict__ order, int by_rows, int scatter) {
  const size_t total = (size_t)rows * cols;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    int c = (int)(e / rows), r = (int)(e - (size_t)c * rows);
    if (by_rows) {
      if (scatter) dst[(size_t)c * rows + order[r]] = src[e];
      else dst[e] = src[(size_t)c * rows + order[r]];
    } else {
      if (scatter) dst[(size_t)order[c] * rows + r] = src[e];
      else dst[e] = src[(size_t)order[c] * rows + r];
    }
  }
}

__global__ void k_add_diag(cplx* A, int n, const double* d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) A[(size_t)i * n + i].x += d[i];
}

__global__ void k_set_identity(cplx* A, int n) {
  const size_t total = (size_t)n * n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    int c = (int)(e / n), r = (int)(e - (size_t)c * n);
    A[e] = cmake(r == c ? 1.0 : 0.0, 0.0);
  }
}

__global__ void k_scale(cplx* A, int rows, int cols, const double* rs, int inv_r, const double* cs, int inv_c) {
  const size_t total = (size_t)rows * cols;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    int c = (int)(e / rows), r = (int)(e - (size_t)c * rows);
    double f = 1.0;
    if (rs) f = inv_r ? f / rs[r] : f * rs[r];
    if (cs) f = inv_c ? f / cs[c] : f * cs[c];
    A[e] = cscale(A[e], f);
  }
}

__global__ void k_conj_transpose(const cplx* __restrict__ A, cplx* __restrict__ B, int n) {
  __shared__ cplx tile[32][33];
  int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    int c = bx + yy, r = by + threadIdx.x;
    if (c < n && r < n) tile[yy][threadIdx.x] = A[(size_t)c * n + r];
  }
  __syncthreads();
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    int c = by + yy, r = bx + threadIdx.x;   // B[r, c] = conj(A[c, r])
    if (c < n && r < n) B[(size_t)c * n + r] = cconj(tile[threadIdx.x][yy]);
  }
}

// out[0] = sum log(x)  (single CTA, deterministic)
__global__ void k_sum_log(const double* x, int n, double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += log(x[i]);
  s = block_sum(s, red);
  if (threadIdx.x == 0) out[0] = s;
}

__global__ void k_max_absdiff(const cplx* A, const cplx* B, size_t count, double* out) {
  __shared__ double red[32];
  double m = 0.0;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
    cplx d = csub(A[e], B[e]);
    double a = sqrt(cabs2(d));
    if (!(a <= m)) m = a;   // propagates NaN
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double q = __shfl_xor_sync(0xffffffffu, m, o);
    if (!(q <= m)) m = q;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q)
      if (!(red[q] <= t)) t = red[q];
    // combine across CTAs: non-negative doubles order like their bit patterns
    unsigned long long bits = __double_as_longlong(t);
    if (t != t) bits = 0x7ff8000000000000ull;
    atomicMax(reinterpret_cast<unsigned long long*>(out), bits);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline int grid_for(size_t total, int threads = 256, int cap = 4096) {
  size_t g = (total + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > (size_t)cap) g = cap;
  return (int)g;
}

cudaError_t launch_zgemm(int m, int nn, int k, char opA, char opB, cplx alpha, const cplx* A, int lda,
                         const cplx* B, int ldb, cplx beta, cplx* C, int ldc, const double* rowscale,
                         const double* colscale, cudaStream_t st, const int* active) {
  dim3 grid((nn + GB_N - 1) / GB_N, (m + GB_M - 1) / GB_M);
  k_zgemm<<<grid, 256, 0, st>>>(m, nn, k, opA, opB, alpha, A, lda, B, ldb, beta, C, ldc, rowscale, colscale,
                                active);
  return cudaGetLastError();
}

cudaError_t launch_qrp(cplx* A, int n, QRWork& w, int sm_count, cudaStream_t st, int max_grid) {
  if (n > 32 * QR_MAXT) return cudaErrorInvalidValue;
  size_t smem = (size_t)n * (sizeof(cplx) + sizeof(int));
  static SmemLimit smem_limit;
  if (cudaError_t ea = smem_limit.raise((const void*)k_qrp, 64 * 1024); ea != cudaSuccess) return ea;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_qrp, QR_THREADS, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int grid = sm_count;   // one CTA per SM; remaining columns are dealt round-robin over all CTAs
  if (max_grid > 0 && grid > max_grid) grid = max_grid;
  if (grid > 32 * CAND_PER_LANE) grid = 32 * CAND_PER_LANE;
  QRWork copy = w;
  void* args[] = {&A, &n, &copy};
  return cudaLaunchCooperativeKernel((void*)k_qrp, dim3(grid), dim3(QR_THREADS), args, smem, st);
}

cudaError_t launch_qrp_finalize(cplx* A, cplx* T, double* D, int n, const QRWork& w, cudaStream_t st) {
  k_qrp_finalize<<<grid_for((size_t)n * n), 256, n * sizeof(int), st>>>(A, T, D, n, w.order, w.beta);
  return cudaGetLastError();
}

cudaError_t launch_apply_q_right(cplx* X, int m, int n, const QRWork& w, bool conj_transpose_q, cudaStream_t st) {
  if (n > 32 * QR_MAXT) return cudaErrorInvalidValue;
  // one row per warp, 4 warps per CTA: up to 2 CTAs per SM at 256 registers per thread
  int rows_per_cta = 4;
  k_apply_q_right<<<(m + rows_per_cta - 1) / rows_per_cta, 128, 0, st>>>(X, m, n, w.V, w.tau,
                                                                        conj_transpose_q ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_trsm_left_upper(const cplx* T, const int* order, const cplx* rdiag, cplx* Y, int n, int m,
                                   cudaStream_t st) {
  size_t smem = (size_t)4 * n * sizeof(cplx);
  static SmemLimit smem_limit;
  if (cudaError_t ea = smem_limit.raise((const void*)k_trsm_left_upper, 200 * 1024); ea != cudaSuccess) return ea;
  k_trsm_left_upper<<<(m + 3) / 4, 128, smem, st>>>(T, order, rdiag, Y, n, m);
  return cudaGetLastError();
}

cudaError_t launch_trsm_diag_block(const cplx* T, int ldT, const cplx* rdiag, cplx* Y, int ldY, int j0, int b, int m,
                                   bool lower, cudaStream_t st) {
  if (b < 1 || b > 128) return cudaErrorInvalidValue;
  if (!lower && !rdiag) return cudaErrorInvalidValue;
  const size_t smem = ((size_t)b * (b - 1) / 2 + b) * sizeof(cplx);
  static SmemLimit smem_limit;
  constexpr int kMaxTdb = (int)((128 * 127 / 2 + 128) * sizeof(cplx));   // b = 128
  if (cudaError_t ea = smem_limit.raise((const void*)k_trsm_diag_block, kMaxTdb); ea != cudaSuccess) return ea;
  k_trsm_diag_block<<<(m + TRSM_DB_WARPS - 1) / TRSM_DB_WARPS, 32 * TRSM_DB_WARPS, smem, st>>>(
      T, ldT, rdiag, Y, ldY, j0, b, m, lower ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_trsm_left_lower_unit(const cplx* Lc, cplx* Y, int n, int m, cudaStream_t st) {
  size_t smem = (size_t)4 * n * sizeof(cplx);
  static SmemLimit smem_limit;
  if (cudaError_t ea = smem_limit.raise((const void*)k_trsm_left_lower_unit, 200 * 1024); ea != cudaSuccess) return ea;
  k_trsm_left_lower_unit<<<(m + 3) / 4, 128, smem, st>>>(Lc, Y, n, m);
  return cudaGetLastError();
}

cudaError_t launch_wy_prep(const cplx* V, const cplx* tau, int n, int jb, int b, cplx* Vb, cplx* trd,
                           cudaStream_t st) {
  k_wy_prep<<<grid_for((size_t)(n - jb) * b), 256, 0, st>>>(V, tau, n, jb, b, Vb, trd);
  return cudaGetLastError();
}

cudaError_t launch_lup(cplx* A, cplx* Lb, int n, LUKernel& w, int sm_count, cudaStream_t st, int max_grid) {
  if (n > 32 * QR_MAXT) return cudaErrorInvalidValue;
  size_t smem = (size_t)n * (sizeof(cplx) + sizeof(int));
  static SmemLimit smem_limit;
  if (cudaError_t ea = smem_limit.raise((const void*)k_lup, 64 * 1024); ea != cudaSuccess) return ea;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lup, QR_THREADS, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int grid = sm_count;
  if (max_grid > 0 && grid > max_grid) grid = max_grid;
  LUKernel copy = w;
  void* args[] = {&A, &Lb, &n, &copy};
  return cudaLaunchCooperativeKernel((void*)k_lup, dim3(grid), dim3(QR_THREADS), args, smem, st);
}

// One cluster of cs CTAs (16, else 8 when 16 cannot be scheduled); returns
// cudaErrorNotSupported, with nothing launched, when neither fits.
static cudaError_t launch_lu_panel_cluster(cplx* A, int n, int p0, int b, LUPanel& w, int cs, cudaStream_t st) {
  constexpr size_t kMax = 160 * 1024;
  static SmemLimit smem_limit;
  static bool nonportable_set[64] = {};
  int dev = 0;
  if (cudaError_t e = cudaGetDevice(&dev); e != cudaSuccess) return e;
  if (cudaError_t ea = smem_limit.raise((const void*)k_lu_panel_cluster, (int)kMax); ea != cudaSuccess) return ea;
  if (dev >= 0 && dev < 64 && !nonportable_set[dev]) {
    if (cudaError_t e = cudaFuncSetAttribute((const void*)k_lu_panel_cluster,
                                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e != cudaSuccess)
      return e;
    nonportable_set[dev] = true;
  }
  for (int c = cs; c >= 8; c /= 2) {
    const int chunk = (n - p0 + c - 1) / c;
    const size_t smem = (size_t)chunk * LU_PB * sizeof(cplx);
    if (smem > kMax) return cudaErrorNotSupported;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, (const void*)k_lu_panel_cluster, &cfg) != cudaSuccess) {
      cudaGetLastError();
      clusters = 0;
    }
    if (clusters < 1) continue;
    return cudaLaunchKernelEx(&cfg, k_lu_panel_cluster, A, n, p0, b, w);
  }
  return cudaErrorNotSupported;
}

cudaError_t launch_lu_panel(cplx* A, int n, int p0, int b, LUPanel& w, int sm_count, cudaStream_t st, int max_grid,
                            int cluster) {
  if (b < 1 || b > LU_PB) return cudaErrorInvalidValue;
  if (cluster >= 8) {
    const cudaError_t e = launch_lu_panel_cluster(A, n, p0, b, w, cluster, st);
    if (e != cudaErrorNotSupported) return e;
  }
  int grid = sm_count;
  if (max_grid > 0 && grid > max_grid) grid = max_grid;
  if (grid > n - p0) grid = n - p0;
  if (grid > 32 * CAND_PER_LANE) grid = 32 * CAND_PER_LANE;
  const int chunk = (n - p0 + grid - 1) / grid;
  const size_t smem = (size_t)chunk * LU_PB * sizeof(cplx);
  constexpr size_t kMax = 160 * 1024;
  if (smem > kMax) return cudaErrorInvalidValue;   // grid too small for the panel rows
  static SmemLimit smem_limit;
  if (cudaError_t ea = smem_limit.raise((const void*)k_lu_panel, (int)kMax); ea != cudaSuccess) return ea;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lu_panel, 256, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  LUPanel copy = w;
  void* args[] = {&A, &n, &p0, &b, &copy};
  return cudaLaunchCooperativeKernel((void*)k_lu_panel, dim3(grid), dim3(256), args, smem, st);
}

cudaError_t launch_lu_apply_swaps(cplx* A, int n, int p0, int b, const int* piv, int* perm, cudaStream_t st) {
  k_lu_apply_swaps<<<(n + 7) / 8, 256, 0, st>>>(A, n, p0, b, piv, perm);
  return cudaGetLastError();
}

cudaError_t launch_lu_diag(const cplx* A, int n, cplx* udiag, cplx* rdiag, cudaStream_t st) {
  k_lu_diag<<<(n + 255) / 256, 256, 0, st>>>(A, n, udiag, rdiag);
  return cudaGetLastError();
}

cudaError_t launch_add(const cplx* A, const cplx* B, cplx* C, size_t count, cudaStream_t st) {
  k_add<<<grid_for(count), 256, 0, st>>>(A, B, C, count);
  return cudaGetLastError();
}

cudaError_t launch_iota(int* p, int n, cudaStream_t st) {
  k_iota<<<(n + 255) / 256, 256, 0, st>>>(p, n);
  return cudaGetLastError();
}

cudaError_t launch_split_scales(const double* Dl, const double* Dr, int n, double* s, cudaStream_t st) {
  k_split_scales<<<(n + 255) / 256, 256, 0, st>>>(Dl, Dr, n, s);
  return cudaGetLastError();
}

cudaError_t launch_lu_logdet(const cplx* udiag, const double* Dl, const double* Dr, int n, double* out,
                             cudaStream_t st) {
  k_lu_logdet<<<1, 256, 0, st>>>(udiag, Dl, Dr, n, out);
  return cudaGetLastError();
}

cudaError_t launch_trsm_right_upper(const cplx* T, const int* order, cplx* Y, int m, int n, cudaStream_t st) {
  size_t smem = (size_t)4 * n * sizeof(cplx);
  static SmemLimit smem_limit;
  if (cudaError_t ea = smem_limit.raise((const void*)k_trsm_right_upper, 200 * 1024); ea != cudaSuccess) return ea;
  k_trsm_right_upper<<<(m + 3) / 4, 128, smem, st>>>(T, order, Y, m, n);
  return cudaGetLastError();
}

cudaError_t launch_permute(const cplx* src, cplx* dst, int rows, int cols, const int* order, bool by_rows,
                           bool scatter, cudaStream_t st) {
  k_permute<<<grid_for((size_t)rows * cols), 256, 0, st>>>(src, dst, rows, cols, order, by_rows, scatter);
  return cudaGetLastError();
}

cudaError_t launch_add_diag(cplx* A, int n, const double* d, cudaStream_t st) {
  k_add_diag<<<(n + 255) / 256, 256, 0, st>>>(A, n, d);
  return cudaGetLastError();
}

cudaError_t launch_set_identity(cplx* A, int n, cudaStream_t st) {
  k_set_identity<<<grid_for((size_t)n * n), 256, 0, st>>>(A, n);
  return cudaGetLastError();
}

cudaError_t launch_scale(cplx* A, int rows, int cols, const double* rowscale, bool invert_rows,
                         const double* colscale, bool invert_cols, cudaStream_t st) {
  k_scale<<<grid_for((size_t)rows * cols), 256, 0, st>>>(A, rows, cols, rowscale, invert_rows, colscale,
                                                         invert_cols);
  return cudaGetLastError();
}

cudaError_t launch_conj_transpose(const cplx* A, cplx* B, int n, cudaStream_t st) {
  dim3 grid((n + 31) / 32, (n + 31) / 32);
  k_conj_transpose<<<grid, dim3(32, 8), 0, st>>>(A, B, n);
  return cudaGetLastError();
}

cudaError_t launch_sum_log(const double* x, int n, double* out, cudaStream_t st) {
  k_sum_log<<<1, 256, 0, st>>>(x, n, out);
  return cudaGetLastError();
}

__global__ void k_fill(double* d, int n, double v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = v;
}

cudaError_t launch_fill(double* d, int n, double v, cudaStream_t st) {
  k_fill<<<(n + 255) / 256, 256, 0, st>>>(d, n, v);
  return cudaGetLastError();
}

cudaError_t launch_max_absdiff(const cplx* A, const cplx* B, size_t count, double* out, cudaStream_t st, bool reset) {
  if (reset) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
    if (e != cudaSuccess) return e;
  }
  k_max_absdiff<<<grid_for(count, 256, 1024), 256, 0, st>>>(A, B, count, out);
  return cudaGetLastError();
}
