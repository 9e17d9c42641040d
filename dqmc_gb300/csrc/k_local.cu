// Local Metropolis updates of one time slice (plain FP64, rank-4 updates).
//
// Reference: src/local_updates.jl:1-95 (local_updates, calc_detratio,
// update_greens!), src/action.jl:57-100 (calc_boson_action_diff),
// src/interactions.jl:102-141 (interaction_matrix_exp_op!).
//
// One cooperative (co-resident) launch visits all N sites of the slice in
// order.  Every CTA evaluates the 4x4 determinant ratio of the current site
// redundantly from the same 16 entries of G, so all CTAs take the same
// accept/reject decision without communicating.  On acceptance the rank-4
// update G += A B, A = (G[:,c] - I[:,c]) M^-1 (n x 4), B = Delta G[r,:]
// (4 x n), is split over the whole grid in two phases separated by grid
// barriers (phase 1 forms A and B from the unmodified G, phase 2 writes G).
// Rejected sites cost no barrier.
//
// Proposal streams use fixed slots: delta[:, i] and unif[i] belong to site
// i of this call; unif[i] decides only when p_acc <= 1, exactly as
// `p_acc > 1.0 || rand() < p_acc`.
#include "common.cuh"
#include "kernels.h"

namespace {

struct C4 { cplx a[4][4]; };

// exp(-power*dtau*V(op)) for one site (src/interactions.jl:102-141).
__device__ void ev_block(const ModelConst& mc, const double op[3], double power, C4& e, EvEntry* entry) {
  double nrm = sqrt(op[0] * op[0] + op[1] * op[1] + op[2] * op[2]);
  double a = mc.lambda * mc.dtau * nrm;
  double shn = sinh(a) / nrm;
  double C = cosh(a);
  double sh = power * shn;
  cplx S = cmake(-op[0] * sh, op[1] * sh);
  double R = -op[2] * sh;
  cplx z = cmake(0.0, 0.0);
  e.a[0][0] = cmake(C, 0); e.a[0][1] = S;         e.a[0][2] = z;              e.a[0][3] = cmake(R, 0);
  e.a[1][0] = cconj(S);    e.a[1][1] = cmake(C, 0); e.a[1][2] = cmake(-R, 0); e.a[1][3] = z;
  e.a[2][0] = z;           e.a[2][1] = cmake(-R, 0); e.a[2][2] = cmake(C, 0); e.a[2][3] = cconj(S);
  e.a[3][0] = cmake(R, 0); e.a[3][1] = z;           e.a[3][2] = S;            e.a[3][3] = cmake(C, 0);
  if (entry) { entry->C = C; entry->Sr = -op[0] * shn; entry->Si = op[1] * shn; entry->R = -op[2] * shn; }
}

__device__ void mat4_mul(const C4& A, const C4& B, C4& Cm) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      cplx s = cmake(0, 0);
      for (int k = 0; k < 4; ++k) s = cfma(A.a[i][k], B.a[k][j], s);
      Cm.a[i][j] = s;
    }
}

// LU with partial pivoting: determinant and (optionally) inverse of a 4x4.
__device__ cplx mat4_det_inv(const C4& Min, C4* inv, bool* singular) {
  C4 A = Min;
  int piv[4] = {0, 1, 2, 3};
  cplx det = cmake(1.0, 0.0);
  *singular = false;
  for (int k = 0; k < 4; ++k) {
    int p = k;
    double best = cabs2(A.a[k][k]);
    for (int r = k + 1; r < 4; ++r) {
      double v = cabs2(A.a[r][k]);
      if (v > best) { best = v; p = r; }
    }
    if (best == 0.0) { *singular = true; return cmake(0, 0); }
    if (p != k) {
      for (int c = 0; c < 4; ++c) { cplx t = A.a[k][c]; A.a[k][c] = A.a[p][c]; A.a[p][c] = t; }
      int t = piv[k]; piv[k] = piv[p]; piv[p] = t;
      det = cmake(-det.x, -det.y);
    }
    det = cmul(det, A.a[k][k]);
    for (int r = k + 1; r < 4; ++r) {
      cplx l = cdiv(A.a[r][k], A.a[k][k]);
      A.a[r][k] = l;
      for (int c = k + 1; c < 4; ++c) A.a[r][c] = csub(A.a[r][c], cmul(l, A.a[k][c]));
    }
  }
  if (inv) {
    // solve A X = P I column by column
    for (int col = 0; col < 4; ++col) {
      cplx y[4];
      for (int r = 0; r < 4; ++r) y[r] = cmake(piv[r] == col ? 1.0 : 0.0, 0.0);
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < r; ++c) y[r] = csub(y[r], cmul(A.a[r][c], y[c]));
      for (int r = 3; r >= 0; --r) {
        for (int c = r + 1; c < 4; ++c) y[r] = csub(y[r], cmul(A.a[r][c], y[c]));
        y[r] = cdiv(y[r], A.a[r][r]);
      }
      for (int r = 0; r < 4; ++r) inv->a[r][col] = y[r];
    }
  }
  return det;
}

struct SiteDecision {
  int accepted;
  double newop[3];
  double dS;
  double exp_dS;
  cplx det;
  double pacc;
  EvEntry ev_new;
  C4 delta;
  C4 minv;
};

__global__ void __launch_bounds__(256) k_local_updates(LocalUpdateArgs a) {
  const ModelConst& mc = a.mc;
  const int N = mc.N, n = mc.n, M = mc.M, L = mc.L;
  const int l = a.slice0;
  extern __shared__ double smem_local[];
  double* phis = smem_local;  // (3, N): this CTA's copy of phi[:, :, l]
  __shared__ SiteDecision dec;

  for (int k = threadIdx.x; k < 3 * N; k += blockDim.x) phis[k] = a.phi[(size_t)3 * N * l + k];
  __syncthreads();
  const int lt_later = (l + 1) % M, lt_earlier = (l - 1 + M) % M;
  const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t gthreads = (size_t)gridDim.x * blockDim.x;

  for (int i = 0; i < N; ++i) {
    if (threadIdx.x == 0) {
      // ---- boson action difference (src/action.jl:57-100) ----
      double old[3] = {phis[3 * i], phis[3 * i + 1], phis[3 * i + 2]};
      double nw[3];
      for (int c = 0; c < 3; ++c) nw[c] = old[c] + a.delta[3 * i + c];
      double diff[3] = {nw[0] - old[0], nw[1] - old[1], nw[2] - old[2]};
      double old_sq = old[0] * old[0] + old[1] * old[1] + old[2] * old[2];
      double new_sq = nw[0] * nw[0] + nw[1] * nw[1] + nw[2] * nw[2];
      double sq_diff = new_sq - old_sq;
      double pow4_diff = new_sq * new_sq - old_sq * old_sq;
      const double* pe = (lt_earlier == l) ? &phis[3 * i] : &a.phi[((size_t)N * lt_earlier + i) * 3];
      const double* pl = (lt_later == l) ? &phis[3 * i] : &a.phi[((size_t)N * lt_later + i) * 3];
      int y = i % L, x = i / L;
      int nbs[4] = {(y + 1) % L + L * x, y + L * ((x + 1) % L), (y - 1 + L) % L + L * x,
                    y + L * ((x - 1 + L) % L)};
      double tdot = 0.0, sdot = 0.0;
      for (int c = 0; c < 3; ++c) {
        double ot = pl[c] + pe[c];
        double os = 0.0;
        for (int q = 0; q < 4; ++q) os = os + phis[3 * nbs[q] + c];
        tdot += ot * diff[c];
        sdot += os * diff[c];
      }
      double dS = 0.0;
      dS += 1.0 / (mc.dtau * mc.c * mc.c) * (sq_diff - tdot);
      dS += 0.5 * mc.dtau * (4 * sq_diff - 2.0 * sdot);
      dS += mc.dtau * (0.5 * mc.r * sq_diff + 0.25 * mc.u * pow4_diff);
      double exp_dS = exp(-dS);
      // ---- determinant ratio (src/local_updates.jl:42-59) ----
      C4 e1, e2, d, Gii, Mm;
      ev_block(mc, old, -1.0, e1, nullptr);
      EvEntry evn;
      ev_block(mc, nw, 1.0, e2, &evn);
      mat4_mul(e1, e2, d);
      for (int r = 0; r < 4; ++r) d.a[r][r] = csub(d.a[r][r], cmake(1.0, 0.0));
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
          cplx g = ldcg_c(&a.G[(size_t)(i + c * N) * n + i + r * N]);
          Gii.a[r][c] = cmake((r == c ? 1.0 : 0.0) - g.x, -g.y);   // I - G_ii
        }
      mat4_mul(d, Gii, Mm);
      for (int r = 0; r < 4; ++r) Mm.a[r][r] = cadd(Mm.a[r][r], cmake(1.0, 0.0));
      bool singular;
      C4 minv;
      cplx det = mat4_det_inv(Mm, &minv, &singular);
      double pacc = exp_dS * det.x;
      double u = a.unif[i];
      int acc = (pacc > 1.0 || u < pacc) ? 1 : 0;
      if (singular || !isfinite(det.x) || !isfinite(det.y)) {
        acc = 0;
        if (blockIdx.x == 0) atomicOr(a.err, singular ? DQMC_KERR_SINGULAR : DQMC_KERR_NONFINITE);
      }
      dec.accepted = acc;
      for (int c = 0; c < 3; ++c) dec.newop[c] = nw[c];
      dec.dS = dS;
      dec.exp_dS = exp_dS;
      dec.det = det;
      dec.pacc = pacc;
      dec.ev_new = evn;
      dec.delta = d;
      dec.minv = minv;
      if (acc) { phis[3 * i] = nw[0]; phis[3 * i + 1] = nw[1]; phis[3 * i + 2] = nw[2]; }
      if (blockIdx.x == 0) {
        if (a.acc_out) a.acc_out[i] = (uint8_t)acc;
        if (a.det_out) a.det_out[i] = det;
        if (a.pacc_out) a.pacc_out[i] = pacc;
        if (acc) {
          double* pg = &a.phi[((size_t)N * l + i) * 3];
          pg[0] = nw[0]; pg[1] = nw[1]; pg[2] = nw[2];
          if (a.evtab) reinterpret_cast<EvEntry*>(a.evtab)[(size_t)N * l + i] = evn;
          *a.action += -log(exp_dS);
          *a.n_acc += 1;
        }
      }
    }
    __syncthreads();
    const int accepted = dec.accepted;
    // every thread has read the decision before thread 0 may overwrite it
    __syncthreads();
    if (!accepted) continue;

    // ---- phase 1: A = (G[:, cols] - I[:, cols]) M^-1, B = Delta G[rows, :] ----
    for (size_t t = gtid; t < (size_t)2 * n; t += gthreads) {
      if (t < (size_t)n) {
        int r = (int)t;
        cplx g[4];
        for (int k = 0; k < 4; ++k) {
          g[k] = ldcg_c(&a.G[(size_t)(i + k * N) * n + r]);
          if (r == i + k * N) g[k].x -= 1.0;
        }
        for (int c = 0; c < 4; ++c) {
          cplx s = cmake(0, 0);
          for (int k = 0; k < 4; ++k) s = cfma(g[k], dec.minv.a[k][c], s);
          a.Acol[(size_t)c * n + r] = s;
        }
      } else {
        int col = (int)(t - n);
        cplx g[4];
        for (int k = 0; k < 4; ++k) g[k] = ldcg_c(&a.G[(size_t)col * n + i + k * N]);
        for (int r = 0; r < 4; ++r) {
          cplx s = cmake(0, 0);
          for (int k = 0; k < 4; ++k) s = cfma(dec.delta.a[r][k], g[k], s);
          a.Brow[(size_t)r * n + col] = s;
        }
      }
    }
    if (!grid_barrier(a.bar, a.err)) return;
    // ---- phase 2: G += A B (src/local_updates.jl:86-91) ----
    const size_t total = (size_t)n * n;
    for (size_t e = gtid; e < total; e += gthreads) {
      int col = (int)(e / n), r = (int)(e - (size_t)col * n);
      cplx acc = ldcg_c(&a.G[e]);
      for (int k = 0; k < 4; ++k) acc = cfma(ldcg_c(&a.Acol[(size_t)k * n + r]), ldcg_c(&a.Brow[(size_t)k * n + col]), acc);
      a.G[e] = acc;
    }
    if (!grid_barrier(a.bar, a.err)) return;
  }
}

}  // namespace

cudaError_t launch_local_updates(const LocalUpdateArgs& a, int sm_count, cudaStream_t st) {
  size_t smem = (size_t)3 * a.mc.N * sizeof(double);
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_local_updates, 256, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (per_sm > 2) per_sm = 2;
  int grid = sm_count * per_sm;
  size_t need = ((size_t)a.mc.n * a.mc.n + 255) / 256;
  if ((size_t)grid > need) grid = (int)need < 1 ? 1 : (int)need;
  LocalUpdateArgs copy = a;
  void* args[] = {&copy};
  return cudaLaunchCooperativeKernel((void*)k_local_updates, dim3(grid), dim3(256), args, smem, st);
}
