// Local Metropolis updates of one time slice (plain FP64, rank-4 updates).
//
// Reference: src/local_updates.jl:1-95 (local_updates, calc_detratio,
// update_greens!), src/action.jl:57-100 (calc_boson_action_diff),
// src/interactions.jl:102-141 (interaction_matrix_exp_op!).
//
// One cooperative (co-resident) launch visits all N sites of the slice in
// order.  Structure:
//   * prologue: every CTA builds, for all sites in parallel, the 4x4 block
//     Delta_i = e^{+dtau V(phi_i)} e^{-dtau V(phi_i + delta_i)} - I into shared
//     memory (the old field of a site cannot change before its own visit);
//   * per site, warp 0 of every CTA evaluates the ratio redundantly and
//     identically from the same 16 entries of G: lanes build
//     M = I + Delta (I - G_ii) entry-wise, 24 lanes form the permutation
//     expansion of det M, and on acceptance 16 lanes form M^-1 = adj(M)/det;
//     all CTAs therefore take the same decision without communicating;
//   * on acceptance the rank-4 update G += A B, A = (G[:,c] - I[:,c]) M^-1
//     (n x 4), B = Delta G[r,:] (4 x n), runs over the whole grid in two phases
//     separated by grid barriers: phase 1 forms A and B from the unmodified G,
//     phase 2 applies them with warp tiles of 128 rows x 4 columns (A held in
//     registers, B broadcast).  Rejected sites cost no barrier.
//
// Proposal streams use fixed slots: delta[:, i] and unif[i] belong to site
// i of this call; unif[i] decides only when p_acc <= 1, exactly as
// `p_acc > 1.0 || rand() < p_acc`.
#include "common.cuh"
#include "kernels.h"
#include "oz_slice.cuh"

namespace {

// The 24 permutations of (0,1,2,3) and their signs, for det M.
__constant__ unsigned char c_perm[24][4] = {
    {0, 1, 2, 3}, {0, 1, 3, 2}, {0, 2, 1, 3}, {0, 2, 3, 1}, {0, 3, 1, 2}, {0, 3, 2, 1},
    {1, 0, 2, 3}, {1, 0, 3, 2}, {1, 2, 0, 3}, {1, 2, 3, 0}, {1, 3, 0, 2}, {1, 3, 2, 0},
    {2, 0, 1, 3}, {2, 0, 3, 1}, {2, 1, 0, 3}, {2, 1, 3, 0}, {2, 3, 0, 1}, {2, 3, 1, 0},
    {3, 0, 1, 2}, {3, 0, 2, 1}, {3, 1, 0, 2}, {3, 1, 2, 0}, {3, 2, 0, 1}, {3, 2, 1, 0}};
__constant__ signed char c_psign[24] = {1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1, 1,
                                         1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1, 1};

// Interaction block parameters of exp(-power*dtau*V(op)) for one site
// (src/interactions.jl:102-141): C, S, R with S, R scaled by `power`.
__device__ __forceinline__ void ev_params(const ModelConst& mc, const double op[3], double power, double& C,
                                          cplx& S, double& R, double& shn) {
  double nrm = sqrt(op[0] * op[0] + op[1] * op[1] + op[2] * op[2]);
  double a = mc.lambda * mc.dtau * nrm;
  shn = sinh(a) / nrm;
  C = cosh(a);
  double sh = power * shn;
  S = cmake(-op[0] * sh, op[1] * sh);
  R = -op[2] * sh;
}

// Entry (r, c) of the block [[C,S,0,R],[S*,C,-R,0],[0,-R,C,S*],[R,0,S,C]].
__device__ __forceinline__ cplx ev_entry(int r, int c, double C, cplx S, double R) {
  const int code = r * 4 + c;
  switch (code) {
    case 0: case 5: case 10: case 15: return cmake(C, 0.0);
    case 1: case 14: return S;
    case 4: case 11: return cconj(S);
    case 3: case 12: return cmake(R, 0.0);
    case 6: case 9: return cmake(-R, 0.0);
    default: return cmake(0.0, 0.0);
  }
}

__device__ __forceinline__ cplx shfl_c(cplx v, int src) {
  return cmake(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

struct SiteDecision {
  int accepted;
  cplx minv[4][4];
};

constexpr int LU_THREADS = 256;

// Shared-memory layout of both local-update kernels.
struct LocalSmem {
  cplx* delta_all;   // (N, 16): Delta_i row-major
  EvEntry* evnew;    // (N): interaction entries of the proposed field
  double* phis;      // (3, N): this CTA's copy of phi[:, :, l]
};

__device__ LocalSmem local_smem(void* base, int N) {
  LocalSmem s;
  s.delta_all = reinterpret_cast<cplx*>(base);
  s.evnew = reinterpret_cast<EvEntry*>(s.delta_all + 16 * N);
  s.phis = reinterpret_cast<double*>(s.evnew + N);
  return s;
}

// Field copy of slice l and Delta_i = e^{+dtau V(phi_i)} e^{-dtau V(phi_i + delta_i)} - I
// for sites >= first (the old field of a site cannot change before its visit).
__device__ void local_prologue(const LocalUpdateArgs& a, const LocalSmem& sm, int first) {
  const ModelConst& mc = a.mc;
  const int N = mc.N, l = a.slice0;
  for (int k = threadIdx.x; k < 3 * N; k += blockDim.x) sm.phis[k] = a.phi[(size_t)3 * N * l + k];
  for (int i = first + threadIdx.x; i < N; i += blockDim.x) {
    const double* po = &a.phi[((size_t)N * l + i) * 3];
    double old[3] = {po[0], po[1], po[2]};
    double nw[3] = {old[0] + a.delta[3 * i], old[1] + a.delta[3 * i + 1], old[2] + a.delta[3 * i + 2]};
    double C1, R1, s1, C2, R2, s2;
    cplx S1, S2;
    ev_params(mc, old, -1.0, C1, S1, R1, s1);
    ev_params(mc, nw, 1.0, C2, S2, R2, s2);
    EvEntry e;
    e.C = C2; e.Sr = -nw[0] * s2; e.Si = nw[1] * s2; e.R = -nw[2] * s2;
    sm.evnew[i] = e;
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) {
        cplx s = cmake(0.0, 0.0);
        for (int k = 0; k < 4; ++k) s = cfma(ev_entry(r, k, C1, S1, R1), ev_entry(k, c, C2, S2, R2), s);
        if (r == c) s.x -= 1.0;
        sm.delta_all[16 * i + 4 * r + c] = s;
      }
  }
}

// Metropolis decision for site i, executed by warp 0 of every CTA.  g is
// G_cur[i + rN, i + cN] in lane 4r + c (lanes < 16).  Writes dec (accepted
// flag, M^-1), the CTA's field copy, and (CTA 0) the outputs, the field,
// the interaction table, the action and the accepted count.
__device__ void local_decide(const LocalUpdateArgs& a, const LocalSmem& sm, int i, cplx g, SiteDecision& dec) {
  const ModelConst& mc = a.mc;
  const int N = mc.N, M = mc.M, L = mc.L, l = a.slice0;
  const int lane = threadIdx.x & 31;
  const int lt_later = (l + 1) % M, lt_earlier = (l - 1 + M) % M;
  double* phis = sm.phis;
  // ---- boson action difference (src/action.jl:57-100), lane 0 ----
  double dS = 0.0;
  if (lane == 0) {
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
    int nbs[4] = {(y + 1) % L + L * x, y + L * ((x + 1) % L), (y - 1 + L) % L + L * x, y + L * ((x - 1 + L) % L)};
    double tdot = 0.0, sdot = 0.0;
    for (int c = 0; c < 3; ++c) {
      double ot = pl[c] + pe[c];
      double os = 0.0;
      for (int q = 0; q < 4; ++q) os = os + phis[3 * nbs[q] + c];
      tdot += ot * diff[c];
      sdot += os * diff[c];
    }
    dS += 1.0 / (mc.dtau * mc.c * mc.c) * (sq_diff - tdot);
    dS += 0.5 * mc.dtau * (4 * sq_diff - 2.0 * sdot);
    dS += mc.dtau * (0.5 * mc.r * sq_diff + 0.25 * mc.u * pow4_diff);
  }
  dS = __shfl_sync(0xffffffffu, dS, 0);
  // ---- M = I + Delta (I - G_ii), lane 4r+c holds M[r][c] (src/local_updates.jl:49-55) ----
  const int r = (lane >> 2) & 3, c = lane & 3;
  if (lane >= 16) g = cmake(0.0, 0.0);
  cplx mt = cmake((r == c ? 1.0 : 0.0) - g.x, -g.y);   // (I - G_ii)[r][c]
  cplx m = cmake(r == c ? 1.0 : 0.0, 0.0);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    cplx mtk = shfl_c(mt, 4 * k + c);                  // (I - G_ii)[k][c]
    m = cfma(sm.delta_all[16 * i + 4 * r + k], mtk, m);
  }
  // ---- det M by the permutation expansion (24 lanes) ----
  cplx term = cmake(0.0, 0.0);
  {
    const int j = lane < 24 ? lane : 0;
    cplx p = cmake(1.0, 0.0);
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) p = cmul(p, shfl_c(m, 4 * rr + c_perm[j][rr]));
    if (lane < 24) term = cscale(p, (double)c_psign[j]);
  }
  cplx det = term;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) det = cadd(det, shfl_c(det, lane ^ o));
  // lanes associate the sum differently; lane 0's value (the same in every
  // CTA) is the one every lane uses, so all decisions agree bit for bit
  det = shfl_c(det, 0);
  const double exp_dS = exp(-dS);
  const double pacc = exp_dS * det.x;
  const double u = a.unif[i];
  int acc = (pacc > 1.0 || u < pacc) ? 1 : 0;
  const bool bad = !isfinite(det.x) || !isfinite(det.y) || (det.x == 0.0 && det.y == 0.0);
  if (bad) acc = 0;
  // ---- M^-1 = adj(M) / det (lane 4r+c: entry [r][c] = cofactor C[c][r] / det) ----
  if (acc) {
    int rows[3], cols[3];
    for (int t = 0, q = 0; t < 4; ++t) if (t != c) rows[q++] = t;
    for (int t = 0, q = 0; t < 4; ++t) if (t != r) cols[q++] = t;
    cplx e[3][3];
#pragma unroll
    for (int u3 = 0; u3 < 3; ++u3)
#pragma unroll
      for (int v3 = 0; v3 < 3; ++v3) e[u3][v3] = shfl_c(m, (4 * rows[u3] + cols[v3]) & 31);
    cplx d3 = csub(cmul(e[0][0], csub(cmul(e[1][1], e[2][2]), cmul(e[1][2], e[2][1]))),
                   cmul(e[0][1], csub(cmul(e[1][0], e[2][2]), cmul(e[1][2], e[2][0]))));
    d3 = cadd(d3, cmul(e[0][2], csub(cmul(e[1][0], e[2][1]), cmul(e[1][1], e[2][0]))));
    if ((r + c) & 1) d3 = cmake(-d3.x, -d3.y);
    if (lane < 16) dec.minv[r][c] = cdiv(d3, det);
  }
  if (lane == 0) {
    dec.accepted = acc;
    if (acc) {
      for (int q = 0; q < 3; ++q) phis[3 * i + q] += a.delta[3 * i + q];
    }
    if (blockIdx.x == 0) {
      if (bad) atomicOr(a.err, DQMC_KERR_NONFINITE);
      if (a.acc_out) a.acc_out[i] = (uint8_t)acc;
      if (a.det_out) a.det_out[i] = det;
      if (a.pacc_out) a.pacc_out[i] = pacc;
      if (acc) {
        double* pg = &a.phi[((size_t)N * l + i) * 3];
        pg[0] = phis[3 * i]; pg[1] = phis[3 * i + 1]; pg[2] = phis[3 * i + 2];
        if (a.evtab) reinterpret_cast<EvEntry*>(a.evtab)[(size_t)N * l + i] = sm.evnew[i];
        *a.action += -log(exp_dS);
        *a.n_acc += 1;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// immediate rank-4 updates
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(LU_THREADS, 2) k_local_updates(LocalUpdateArgs a) {
  unsigned bar_epoch = 0;
  GridBarrierExit bar_exit(a.bar);
  const ModelConst& mc = a.mc;
  const int N = mc.N, n = mc.n;
  extern __shared__ double4_16a smem_local[];
  const LocalSmem sm = local_smem(smem_local, N);
  __shared__ SiteDecision dec;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  local_prologue(a, sm, 0);
  __syncthreads();
  const int gwarp = blockIdx.x * (LU_THREADS / 32) + wid;
  const int nwarps = gridDim.x * (LU_THREADS / 32);

  for (int i = 0; i < N; ++i) {
    if (wid == 0) {
      const int r = (lane >> 2) & 3, c = lane & 3;
      cplx g = cmake(0.0, 0.0);
      if (lane < 16) g = ldcg_c(&a.G[(size_t)(i + c * N) * n + i + r * N]);
      local_decide(a, sm, i, g, dec);
    }
    __syncthreads();
    const int accepted = dec.accepted;
    if (!accepted) {
      __syncthreads();   // every thread has read the decision before warp 0 overwrites it
      continue;
    }
    // ---- phase 1: A = (G[:, cols] - I[:, cols]) M^-1, B = Delta G[rows, :] ----
    const cplx* Dl = &sm.delta_all[16 * i];
    for (int t = blockIdx.x * LU_THREADS + threadIdx.x; t < 2 * n; t += gridDim.x * LU_THREADS) {
      if (t < n) {
        const int row = t;
        cplx g[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          g[k] = ldcg_c(&a.G[(size_t)(i + k * N) * n + row]);
          if (row == i + k * N) g[k].x -= 1.0;
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          cplx s = cmake(0, 0);
#pragma unroll
          for (int k = 0; k < 4; ++k) s = cfma(g[k], dec.minv[k][c], s);
          a.Acol[(size_t)c * n + row] = s;
        }
      } else {
        const int col = t - n;
        cplx g[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) g[k] = ldcg_c(&a.G[(size_t)col * n + i + k * N]);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          cplx s = cmake(0, 0);
#pragma unroll
          for (int k = 0; k < 4; ++k) s = cfma(Dl[4 * r + k], g[k], s);
          a.Brow[(size_t)r * n + col] = s;
        }
      }
    }
    if (!grid_barrier(a.bar, a.err, bar_epoch)) return;
    // ---- phase 2: G += A B over warp tiles of 128 rows x 4 columns ----
    const int tiles_r = (n + 127) / 128, tiles_c = (n + 3) / 4;
    for (int tile = gwarp; tile < tiles_r * tiles_c; tile += nwarps) {
      const int tr = tile % tiles_r, tc = tile / tiles_r;
      const int r0 = tr * 128 + lane, c0 = tc * 4;
      cplx Av[4][4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int row = r0 + 32 * q;
#pragma unroll
        for (int k = 0; k < 4; ++k) Av[q][k] = row < n ? ldcg_c(&a.Acol[(size_t)k * n + row]) : cmake(0, 0);
      }
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        const int col = c0 + cc;
        if (col >= n) break;
        cplx Bv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) Bv[k] = ldcg_c(&a.Brow[(size_t)k * n + col]);
        cplx* gcol = a.G + (size_t)col * n;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int row = r0 + 32 * q;
          if (row < n) {
            cplx v = ldcg_c(&gcol[row]);
#pragma unroll
            for (int k = 0; k < 4; ++k) v = cfma(Av[q][k], Bv[k], v);
            gcol[row] = v;
          }
        }
      }
    }
    if (!grid_barrier(a.bar, a.err, bar_epoch)) return;
  }
}

// ---------------------------------------------------------------------------
// delayed rank-k updates: G_cur = G + X Y with X (n x 4k), Y (4k x n)
// ---------------------------------------------------------------------------
// On GB300 every FP64 warp instruction occupies a sub-partition's FP64 unit
// for tens of cycles, so the per-site chain is kept short and split over
// warps: the per-site constants come from a prepare kernel run once per
// slice, the 4x4 block G_cur[i + rN, i + cN] is read from a cache that the
// owner CTA of site i keeps current, and the decision runs on three warps
// at once (det and 1/det; the adjugate; the action difference).

// Per-site constants of slice l: one warp per site.  Lanes of even parity
// evaluate the old-field block (power -1), odd lanes the proposed one.
__global__ void __launch_bounds__(128) k_local_prepare(LocalUpdateArgs a, SitePrep* __restrict__ prep, int* state) {
  const ModelConst& mc = a.mc;
  const int N = mc.N, M = mc.M, l = a.slice0;
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 4 + (threadIdx.x >> 5);
  // delayed rounds of this slice start from site 0 with nothing pending
  if (state && blockIdx.x == 0 && threadIdx.x == 0) { state[0] = 0; state[1] = 0; state[2] = 0; }
  if (i >= N) return;
  const double* po = &a.phi[((size_t)N * l + i) * 3];
  const double old[3] = {po[0], po[1], po[2]};
  const double nw[3] = {old[0] + a.delta[3 * i], old[1] + a.delta[3 * i + 1], old[2] + a.delta[3 * i + 2]};
  const bool odd = lane & 1;
  double C, R, shn;
  cplx S;
  const double op[3] = {odd ? nw[0] : old[0], odd ? nw[1] : old[1], odd ? nw[2] : old[2]};
  ev_params(mc, op, odd ? 1.0 : -1.0, C, S, R, shn);
  const double C1 = __shfl_sync(0xffffffffu, C, 0), R1 = __shfl_sync(0xffffffffu, R, 0);
  const double C2 = __shfl_sync(0xffffffffu, C, 1), R2 = __shfl_sync(0xffffffffu, R, 1);
  const cplx S1 = shfl_c(S, 0), S2 = shfl_c(S, 1);
  const double s2 = __shfl_sync(0xffffffffu, shn, 1);
  SitePrep* out = prep + i;
  if (lane < 16) {
    const int r = lane >> 2, c = lane & 3;
    cplx v = cmake(0.0, 0.0);
#pragma unroll
    for (int k = 0; k < 4; ++k) v = cfma(ev_entry(r, k, C1, S1, R1), ev_entry(k, c, C2, S2, R2), v);
    if (r == c) v.x -= 1.0;
    out->delta[lane] = v;
  } else if (lane == 16) {
    EvEntry e;
    e.C = C2; e.Sr = -nw[0] * s2; e.Si = nw[1] * s2; e.R = -nw[2] * s2;
    out->ev = e;
  } else if (lane == 17) {
    // boson action difference (src/action.jl:57-100) without the space-neighbour term
    const int lt_later = (l + 1) % M, lt_earlier = (l - 1 + M) % M;
    const double diff[3] = {nw[0] - old[0], nw[1] - old[1], nw[2] - old[2]};
    const double old_sq = old[0] * old[0] + old[1] * old[1] + old[2] * old[2];
    const double new_sq = nw[0] * nw[0] + nw[1] * nw[1] + nw[2] * nw[2];
    const double sq_diff = new_sq - old_sq;
    const double pow4_diff = new_sq * new_sq - old_sq * old_sq;
    const double* pe = &a.phi[((size_t)N * lt_earlier + i) * 3];
    const double* pl = &a.phi[((size_t)N * lt_later + i) * 3];
    double tdot = 0.0;
    for (int c = 0; c < 3; ++c) tdot += (pl[c] + pe[c]) * diff[c];
    out->diff[0] = diff[0]; out->diff[1] = diff[1]; out->diff[2] = diff[2];
    out->dsA = 1.0 / (mc.dtau * mc.c * mc.c) * (sq_diff - tdot);
    out->dsQ = 4 * sq_diff;
    out->dsB = mc.dtau * (0.5 * mc.r * sq_diff + 0.25 * mc.u * pow4_diff);
  }
}

// det M by the Laplace expansion along rows {0, 1}: the 2x2 minors T_ab of
// rows {0, 1} (lanes 0-5) and B_ab of rows {2, 3} (lanes 6-11), pairs (a, b)
// in the order (0,1) (0,2) (0,3) (1,2) (1,3) (2,3), and
// det = sum_ab (-1)^(a+b+1) T_ab B_(complement of ab); m[r][c] in lane 4r+c.
// The sum is complete in lane 0 (lanes 0-7 take part in it).
__device__ __forceinline__ cplx det_laplace(cplx m, int lane) {
  const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
  const int mi = lane < 12 ? lane : 0;
  const int pr = mi < 6 ? 0 : 2, pp = mi < 6 ? mi : mi - 6;
  const cplx e00 = shfl_c(m, 4 * pr + pa[pp]), e01 = shfl_c(m, 4 * pr + pb[pp]);
  const cplx e10 = shfl_c(m, 4 * (pr + 1) + pa[pp]), e11 = shfl_c(m, 4 * (pr + 1) + pb[pp]);
  const cplx minor = csub(cmul(e00, e11), cmul(e01, e10));
  // lane pp < 6: T_pp times B of the complementary pair (index 5 - pp, in lane 11 - pp)
  const cplx bc = shfl_c(minor, lane < 6 ? 11 - lane : 0);
  cplx term = cmake(0.0, 0.0);
  if (lane < 6) {
    term = cmul(minor, bc);
    if (lane == 1 || lane == 4) term = cmake(-term.x, -term.y);   // (a + b) even: (0,2), (1,3)
  }
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) term = cadd(term, shfl_c(term, lane ^ o));
  return term;
}

// adj(M)[r][c] = cofactor C[c][r] for lane 4r+c (lanes < 16), from the 2x2
// minors of rows {0,1} and {2,3} (Laplace expansion of each 3x3 minor along
// its single row from the other pair); m[r][c] in lane 4r+c.
__device__ __forceinline__ cplx adjugate_entry(cplx m, int lane) {
  // pair index of columns (a, b), a < b: 0:(0,1) 1:(0,2) 2:(0,3) 3:(1,2) 4:(1,3) 5:(2,3)
  const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
  // lanes 0-5: top minors T_ab (rows 0, 1); lanes 6-11: bottom minors B_ab (rows 2, 3)
  const int mi = lane < 12 ? lane : 0;
  const int pr = mi < 6 ? 0 : 2, pp = mi < 6 ? mi : mi - 6;
  const cplx e00 = shfl_c(m, 4 * pr + pa[pp]), e01 = shfl_c(m, 4 * pr + pb[pp]);
  const cplx e10 = shfl_c(m, 4 * (pr + 1) + pa[pp]), e11 = shfl_c(m, 4 * (pr + 1) + pb[pp]);
  const cplx minor = csub(cmul(e00, e11), cmul(e01, e10));
  // lane 4r+c: cofactor with row c and column r removed
  const int r = (lane >> 2) & 3, c = lane & 3;
  const int rr = c, cc = r;                        // removed row / column
  const int other = rr < 2 ? 1 - rr : 5 - rr;      // remaining row of the removed row's pair
  const int base = rr < 2 ? 6 : 0;                 // minors of the complementary pair
  int cols[3];
  for (int t = 0, q = 0; t < 4; ++t) if (t != cc) cols[q++] = t;
  cplx d3 = cmake(0.0, 0.0);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int u = a == 0 ? cols[1] : cols[0];
    const int v = a == 2 ? cols[1] : cols[2];
    const int pidx = u == 0 ? (v - 1) : (u == 1 ? v + 1 : 5);   // (0,1)0 (0,2)1 (0,3)2 (1,2)3 (1,3)4 (2,3)5
    const cplx mn = shfl_c(minor, base + pidx);
    const cplx ent = shfl_c(m, 4 * other + cols[a]);
    const cplx t = cmul(ent, mn);
    d3 = (a == 1) ? csub(d3, t) : cadd(d3, t);
  }
  if ((rr + cc) & 1) d3 = cmake(-d3.x, -d3.y);
  return d3;
}

// The words of site i that the delayed kernel keeps in shared memory: the
// SitePrep (Delta_i, the proposed eV entries, the field difference and the
// prepared action parts), then the Metropolis uniform and the proposal delta.
constexpr int kSiteEv = 32, kSiteDiff = 36, kSiteUnif = 44, kSiteProp = 45, kSiteWords = 48;
static_assert(sizeof(SitePrep) == 44 * sizeof(double), "SitePrep is read as 44 words");
static_assert(offsetof(SitePrep, ev) == kSiteEv * sizeof(double), "SitePrep.ev");
static_assert(offsetof(SitePrep, diff) == kSiteDiff * sizeof(double), "SitePrep.diff");
static_assert(offsetof(SitePrep, dsA) == (kSiteDiff + 3) * sizeof(double), "SitePrep.dsA");
__device__ __forceinline__ double site_word(const LocalUpdateArgs& a, const DelayedArgs& d, int i, int k) {
  if (k < 44) return __ldcg(reinterpret_cast<const double*>(d.prep + i) + k);
  if (k == kSiteUnif) return __ldg(&a.unif[i]);
  return __ldg(&a.delta[3 * i + (k - kSiteProp)]);
}

// Processes sites state[0] .. N-1 until k accepted updates are pending or the
// slice ends; state[0] is left at the next site and state[1] at the number of
// pending factors.  The flush G += X Y (a separate GEMM launch over the first
// 4 state[1] columns) follows every round.
//
// One CTA per SM; CTA b owns sites j = b, b + grid, ...  On each acceptance
// it forms the 4 rows j + rN of the new X columns (one warp, 8 lanes per row)
// and the 4 columns j + cN of the new Y rows (another warp), refreshes the
// cached diagonal block of j, and publishes the number of acceptances it has
// folded into site j.  Deciding site i waits only for that counter of site
// i's owner (no grid-wide barrier per acceptance).  With CACHE the owner
// also keeps its X rows / Y columns in shared memory, so the new factor
// entries need no global loads.
template <bool CACHE>
__global__ void __launch_bounds__(LU_THREADS, 1) k_local_delayed(LocalUpdateArgs a, DelayedArgs d) {
  unsigned bar_epoch = 0;
  GridBarrierExit bar_exit(a.bar);
  const ModelConst& mc = a.mc;
  const int N = mc.N, n = mc.n, L = mc.L, K4 = 4 * d.k;
  __shared__ int s_first, s_ok;
  if (threadIdx.x == 0) s_first = __ldcg(&d.state[0]);
  __syncthreads();
  const int first = s_first;
  // every round follows a flush of the previous round's factors, so nothing
  // is pending at its start; clearing the count here also keeps the flush
  // after a round with no sites left from applying the factors again
  int p = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) d.state[1] = 0;
  if (first >= N) return;   // slice done: nothing to do in this round (uniform over the grid)
  const int owned = (N - blockIdx.x + gridDim.x - 1) / gridDim.x;   // sites j = blockIdx.x + t grid
  extern __shared__ double4_16a smem_local[];
  cplx* s_blk = reinterpret_cast<cplx*>(smem_local);                   // (owned, 16) G_cur blocks
  cplx* s_xn = s_blk + (size_t)16 * owned;                              // (4 sites, 4 x 4) new X rows
  cplx* s_yn = s_xn + 64;                                              // (4 sites, 4 x 4) new Y columns
  cplx* Ysm = s_yn + 64;                                               // (4k x 4): Y[j, i + cN]
  cplx* Xsm = Ysm + (size_t)K4 * 4;                                    // (4 x 4k): X[i + rN, j]
  cplx* s_xrow = Xsm + (size_t)K4 * 4;                                 // CACHE: (owned, 4, 4k) X[j', j + rN]
  cplx* s_ycol = s_xrow + (CACHE ? (size_t)owned * 4 * K4 : 0);        // CACHE: (owned, 4, 4k) Y[j', j + cN]
  double* phis = reinterpret_cast<double*>(s_ycol + (CACHE ? (size_t)owned * 4 * K4 : 0));   // (3, N)
  __shared__ cplx s_adj[2][16];     // adj(M)[r][c] (double-buffered by site parity)
  __shared__ cplx s_det[2];
  __shared__ double s_expds[2];
  // the decision, taken by whichever of the det lane and the exp(-dS) lane
  // finishes second (s_dcnt counts their arrivals), read by all after the
  // barrier: bit 0 accepted, bit 1 non-finite determinant
  __shared__ int s_dcnt[2], s_dec[2];
  __shared__ double s_pacc[2];
  // per site (slot i & 1), read during the previous site's decision: the
  // SitePrep words, the Metropolis uniform and the proposal (site_word), and
  // the site's G_cur block, current if no acceptance came in between
  // (s_gp = the pending count it was read at, -1 if not read).  Three buffers
  // by site (i mod 3): while site i is decided, site i + 1's are written, and
  // a thread still finishing site i - 1 (after its decision barrier, before
  // site i's) reads that site's words, so the three must be distinct.
  __shared__ double s_site[3][kSiteWords];
  __shared__ cplx s_gblk[3][16];
  __shared__ int s_gp[3];
  // CTA 0: exp(-dS) of the round's accepted sites in order; the tracked action
  // gets the same additions -log(exp(-dS)) in the same order once the round
  // ends, off the per-site chain (no read-modify-write of global memory per site)
  __shared__ double s_expq[64];
  // mixed form: every CTA cuts the BF16 slices of its own rows of X and
  // columns of Y (K = 4 pend entries each, zeros up to Kpad) for the flush
  // that follows, so the flush needs no slicing launch
  auto slice_round = [&](int pend) {
    if (d.sl.As == nullptr || pend == 0) return;
    __syncthreads();   // every thread's X / Y entries of the round are stored
    const int K = 4 * pend, ln = threadIdx.x & 31;
    for (int t = threadIdx.x >> 5; t < 8 * owned; t += blockDim.x >> 5) {
      const int ts = t >> 3, sub = (t >> 1) & 3, side = t & 1;
      const int rc = blockIdx.x + ts * gridDim.x + sub * N;
      const cplx* src = side ? d.Y : d.X;
      // with CACHE the entries come from this CTA's shared-memory copies (no L2 round trip)
      const cplx* own = CACHE ? (side ? s_ycol : s_xrow) + (size_t)(4 * ts + sub) * K4 : nullptr;
      oz_slice_vec(d.sl, side, rc, K, [&](int jj) { return CACHE ? own[jj] : ldcg_c(&src[(size_t)jj * n + rc]); },
                   ln);
    }
  };
  auto finish_round = [&](int pend) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && pend > 0) {
      double act = *a.action;
      for (int t = 0; t < pend; ++t) act += -log(s_expq[t]);
      *a.action = act;
      *a.n_acc += pend;
    }
  };
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int l = a.slice0;
  for (int k = threadIdx.x; k < 3 * N; k += blockDim.x) phis[k] = a.phi[(size_t)3 * N * l + k];
  for (int e = threadIdx.x; e < 16 * owned; e += blockDim.x) {
    const int j = blockIdx.x + (e >> 4) * gridDim.x, r = (e >> 2) & 3, c = e & 3;
    s_blk[e] = ldcg_c(&a.G[(size_t)(j + c * N) * n + j + r * N]);
  }
  // publication counters of the owned sites start the round at 0
  for (int t = threadIdx.x; t < owned; t += blockDim.x) d.pub[blockIdx.x + t * gridDim.x] = 0;
  // the first site's words and G block (nothing is pending at the round's start)
  if (threadIdx.x < kSiteWords) s_site[first % 3][threadIdx.x] = site_word(a, d, first, threadIdx.x);
  if (threadIdx.x >= 64 && threadIdx.x < 80) {
    const int e = threadIdx.x - 64, r = e >> 2, c = e & 3;
    s_gblk[first % 3][e] = ldcg_c(&a.G[(size_t)(first + c * N) * n + first + r * N]);
  }
  if (threadIdx.x == 0) { s_gp[first % 3] = 0; s_dcnt[0] = 0; s_dcnt[1] = 0; }
  if (!grid_barrier(a.bar, a.err, bar_epoch)) return;

  // phase-1 role of this warp in the first pass of owned sites
  const int sub = lane >> 3, qg = (lane >> 1) & 3, h = lane & 1;
  const bool isX = (wid & 1) == 0;

  for (int i = first; i < N; ++i) {
    const int J = 4 * p;   // pending columns of X / rows of Y
    const int slot = i & 1;                                       // decision values
    const int rs = i % 3, nrs = rs == 2 ? 0 : rs + 1;             // read-ahead buffers of sites i, i + 1
    const double* sw = s_site[rs];                                // this site's words
    const cplx* sdelta = reinterpret_cast<const cplx*>(sw);      // Delta_i, row-major
    // the block read ahead is current unless an acceptance came in between
    const bool have_g = s_gp[rs] == p;
    // the Metropolis decision from det M and exp(-dS) (src/local_updates.jl:20-30),
    // by the second of the two lanes that produce them
    auto arrive_decide = [&]() {
      __threadfence_block();
      if (atomicAdd(&s_dcnt[slot], 1) == 1) {
        __threadfence_block();
        const cplx dt = s_det[slot];
        const double pa = s_expds[slot] * dt.x;
        const bool bad = !isfinite(dt.x) || !isfinite(dt.y) || (dt.x == 0.0 && dt.y == 0.0);
        const bool ac = !bad && (pa > 1.0 || sw[kSiteUnif] < pa);
        s_pacc[slot] = pa;
        s_dec[slot] = (ac ? 1 : 0) | (bad ? 2 : 0);
        s_dcnt[slot] = 0;
      }
    };
    // ---- otherwise wait until the owner of site i has folded in all p acceptances ----
    if (p > 0 && !have_g) {
      if (threadIdx.x == 0) {
        volatile int* f = d.pub + i;
        int ok = 1;
        long long spins = 0;
        while (*f < p) {
          if ((++spins & 1023) == 0) {
            if (spins > (1ll << 24)) { atomicOr(a.err, 2); ok = 0; break; }
            if (*(volatile int*)a.err & 2) { ok = 0; break; }
          }
        }
        __threadfence();
        s_ok = ok;
      }
      __syncthreads();
      if (!s_ok) return;
    }
    // ---- G entries of the first pass's phase 1 (independent of the decision) ----
    cplx gq_pref = cmake(0.0, 0.0);
    if ((wid >> 1) < owned) {
      const int rc = blockIdx.x + (wid >> 1) * gridDim.x + sub * N;
      if (isX) {
        gq_pref = ldcg_c(&a.G[(size_t)(i + qg * N) * n + rc]);
        if (rc == i + qg * N) gq_pref.x -= 1.0;
      } else {
        gq_pref = ldcg_c(&a.G[(size_t)rc * n + i + qg * N]);
      }
    }
    if (wid == 4 || wid == 6) {
      // ---- M = I + Delta (I - G_cur_ii), lane 4r+c holds M[r][c] (src/local_updates.jl:49-55) ----
      const int r = (lane >> 2) & 3, c = lane & 3;
      cplx g = cmake(0.0, 0.0), drow[4];
      if (lane < 16) {
        g = have_g ? s_gblk[rs][lane] : ldcg_c(&d.blk[(size_t)16 * i + lane]);
#pragma unroll
        for (int k = 0; k < 4; ++k) drow[k] = sdelta[4 * r + k];
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) drow[k] = cmake(0.0, 0.0);
      }
      const cplx mt = cmake((r == c ? 1.0 : 0.0) - g.x, -g.y);   // (I - G_ii)[r][c]
      // M[r][c] = I + sum_k Delta[r][k] (I - G_ii)[k][c], as two independent pairs
      const cplx m01 = cfma(drow[1], shfl_c(mt, 4 + c), cmul(drow[0], shfl_c(mt, c)));
      const cplx m23 = cfma(drow[3], shfl_c(mt, 12 + c), cmul(drow[2], shfl_c(mt, 8 + c)));
      cplx m = cadd(m01, m23);
      if (r == c) m.x += 1.0;
      if (wid == 4) {
        // det M (Laplace expansion by 2x2 minors); lane 0's sum is the one
        // used everywhere, so every CTA decides bit for bit alike
        const cplx det = det_laplace(m, lane);
        if (lane == 0) {
          s_det[slot] = det;
          arrive_decide();
        }
      } else {
        const cplx adj = adjugate_entry(m, lane);
        if (lane < 16) s_adj[slot][lane] = adj;
      }
    } else if (wid == 5) {
      // ---- boson action difference: prepared part + space-neighbour coupling;
      //      lanes 0-2 sum the neighbours' component c = lane (the same four
      //      additions in the same order), lane 0 takes the rest ----
      const int y = i % L, x = i / L;
      const int nbs[4] = {(y + 1) % L + L * x, y + L * ((x + 1) % L), (y - 1 + L) % L + L * x,
                          y + L * ((x - 1 + L) % L)};
      double os = 0.0;
      if (lane < 3)
        for (int q = 0; q < 4; ++q) os = os + phis[3 * nbs[q] + lane];
      const double os1 = __shfl_sync(0xffffffffu, os, 1), os2 = __shfl_sync(0xffffffffu, os, 2);
      if (lane == 0) {
        const double osc[3] = {os, os1, os2};
        double sdot = 0.0;
        for (int c = 0; c < 3; ++c) sdot += osc[c] * sw[kSiteDiff + c];
        double dS = sw[kSiteDiff + 3];
        dS += 0.5 * mc.dtau * (sw[kSiteDiff + 4] - 2.0 * sdot);
        dS += sw[kSiteDiff + 5];
        s_expds[slot] = exp(-dS);
        arrive_decide();
      }
    } else if (wid == 7 && i + 1 < N) {
      // ---- site i + 1's G_cur block, ahead of time: current if site i is
      //      rejected and its owner has folded in all p acceptances by now ----
      int v = p;   // nothing pending: G itself is current
      if (p > 0) {
        if (lane == 0) v = (int)ld_acquire_u32(reinterpret_cast<const unsigned*>(d.pub + i + 1));
        v = __shfl_sync(0xffffffffu, v, 0);
      }
      if (v >= p && lane < 16) {
        const int r = lane >> 2, c = lane & 3, j = i + 1;
        s_gblk[nrs][lane] = p == 0 ? ldcg_c(&a.G[(size_t)(j + c * N) * n + j + r * N])
                                     : ldcg_c(&d.blk[(size_t)16 * j + lane]);
      }
      if (lane == 0) s_gp[nrs] = v >= p ? p : -1;
    }
    if (wid < 4) {
      // ---- site i + 1's words (warp 3), then the pending factor entries
      //      touching site i (128 threads, loads issued together) ----
      // (the words are loaded first and stored last, so that their latency
      // overlaps the staging loads)
      const bool words = wid == 3 && i + 1 < N;
      double w0 = 0.0, w1 = 0.0;
      if (words) {
        w0 = site_word(a, d, i + 1, lane);
        if (lane + 32 < kSiteWords) w1 = site_word(a, d, i + 1, lane + 32);
      }
      constexpr int kStage = 128;
      for (int t = threadIdx.x; t < 4 * J; t += 2 * kStage) {
        const int t2 = t + kStage;
        const int j1 = t >> 2, c1 = t & 3, j2 = t2 >> 2, c2 = t2 & 3;
        const cplx y1 = ldcg_c(&d.Y[(size_t)j1 * n + i + c1 * N]);
        const cplx x1 = ldcg_c(&d.X[(size_t)j1 * n + i + c1 * N]);
        cplx y2 = cmake(0.0, 0.0), x2 = cmake(0.0, 0.0);
        if (t2 < 4 * J) {
          y2 = ldcg_c(&d.Y[(size_t)j2 * n + i + c2 * N]);
          x2 = ldcg_c(&d.X[(size_t)j2 * n + i + c2 * N]);
        }
        Ysm[4 * j1 + c1] = y1;
        Xsm[(size_t)c1 * K4 + j1] = x1;
        if (t2 < 4 * J) {
          Ysm[4 * j2 + c2] = y2;
          Xsm[(size_t)c2 * K4 + j2] = x2;
        }
      }
      if (words) {
        s_site[nrs][lane] = w0;
        if (lane + 32 < kSiteWords) s_site[nrs][lane + 32] = w1;
      }
    }
    __syncthreads();
    // ---- Metropolis decision (the same in every CTA); thread 0 writes its effects ----
    const int dec = s_dec[slot];
    const bool acc = (dec & 1) != 0, bad = (dec & 2) != 0;
    const cplx det = s_det[slot];
    const double exp_dS = s_expds[slot];
    const double pacc = s_pacc[slot];
    if (threadIdx.x == 0) {
      if (acc)
        for (int q = 0; q < 3; ++q) phis[3 * i + q] += sw[kSiteProp + q];
      if (blockIdx.x == 0) {
        if (bad) atomicOr(a.err, DQMC_KERR_NONFINITE);
        if (a.acc_out) a.acc_out[i] = (uint8_t)acc;
        if (a.det_out) a.det_out[i] = det;
        if (a.pacc_out) a.pacc_out[i] = pacc;
        if (acc) {
          double* pg = &a.phi[((size_t)N * l + i) * 3];
          pg[0] = phis[3 * i]; pg[1] = phis[3 * i + 1]; pg[2] = phis[3 * i + 2];
          if (a.evtab) {
            EvEntry ev;
            ev.C = sw[kSiteEv]; ev.Sr = sw[kSiteEv + 1]; ev.Si = sw[kSiteEv + 2]; ev.R = sw[kSiteEv + 3];
            reinterpret_cast<EvEntry*>(a.evtab)[(size_t)N * l + i] = ev;
          }
          s_expq[p] = exp_dS;   // the action and the count are updated at the round's end
        }
      }
    }
    // the decision values are double-buffered by site parity: a rejected site
    // needs no barrier here; an accepted one synchronises in the passes below
    if (!acc) continue;
    // ---- new factor columns: X[:, J+k] = (G_cur[:, i + qN] - I[:, i + qN]) adj(M),
    //      Y[J+k, :] = Delta G_cur[i + qN, :] / det  (X Y = (G_cur - I) M^-1 Delta G_cur) ----
    // owned sites in passes of 4: site t of a pass -> warps 2t (X rows) and 2t+1 (Y columns)
    for (int t0 = 0; t0 < owned; t0 += 4) {
      const int ts = t0 + (wid >> 1);
      if (ts < owned) {
        const int j = blockIdx.x + ts * gridDim.x;
        const int rc = j + sub * N;   // X: row rc; Y: column rc
        cplx gq = gq_pref;
        if (t0 > 0) {
          if (isX) {
            gq = ldcg_c(&a.G[(size_t)(i + qg * N) * n + rc]);
            if (rc == i + qg * N) gq.x -= 1.0;
          } else {
            gq = ldcg_c(&a.G[(size_t)rc * n + i + qg * N]);
          }
        }
        cplx inv = cmake(0.0, 0.0);
        if (!isX) {
          const cplx det = s_det[slot];
          const double rd = 1.0 / (det.x * det.x + det.y * det.y);
          inv = cmake(det.x * rd, -det.y * rd);
        }
        cplx part = cmake(0.0, 0.0);
        const cplx* own = CACHE ? (isX ? s_xrow : s_ycol) + (size_t)(4 * ts + sub) * K4 : nullptr;
        if (isX) {
          if (CACHE) {
            for (int jj = h; jj < J; jj += 2) part = cfma(own[jj], Ysm[4 * jj + qg], part);
          } else {
            for (int jj = h; jj < J; jj += 2) part = cfma(ldcg_c(&d.X[(size_t)jj * n + rc]), Ysm[4 * jj + qg], part);
          }
        } else {
          if (CACHE) {
            for (int jj = h; jj < J; jj += 2) part = cfma(Xsm[(size_t)qg * K4 + jj], own[jj], part);
          } else {
            for (int jj = h; jj < J; jj += 2) part = cfma(Xsm[(size_t)qg * K4 + jj], ldcg_c(&d.Y[(size_t)jj * n + rc]), part);
          }
        }
        part = cadd(part, shfl_c(part, lane ^ 1));
        const cplx gcur = cadd(gq, part);   // G_cur[rc, i + qN] (- delta) or G_cur[i + qN, rc]
        // output k = qg of this lane over q' = 2h, 2h + 1, then the pair sum
        const int ko = qg;
        const cplx g0 = shfl_c(gcur, 8 * sub + 4 * h), g1 = shfl_c(gcur, 8 * sub + 4 * h + 2);
        cplx prod;
        if (isX) prod = cfma(g1, s_adj[slot][4 * (2 * h + 1) + ko], cmul(g0, s_adj[slot][4 * (2 * h) + ko]));
        else prod = cfma(sdelta[4 * ko + 2 * h + 1], g1, cmul(sdelta[4 * ko + 2 * h], g0));
        prod = cadd(prod, shfl_c(prod, lane ^ 1));
        if (!isX) prod = cmul(prod, inv);
        if (h == 0) {
          const int ls = ts - t0;
          if (isX) {
            d.X[(size_t)(J + ko) * n + rc] = prod;
            s_xn[16 * ls + 4 * sub + ko] = prod;        // X_new[j + sub N, k]
          } else {
            d.Y[(size_t)(J + ko) * n + rc] = prod;
            s_yn[16 * ls + 4 * ko + sub] = prod;        // Y_new[k, j + sub N]
          }
          if (CACHE) const_cast<cplx*>(own)[J + ko] = prod;
        }
      }
      __syncthreads();
      // ---- refresh the cached blocks of the pass's sites (needed by later sites only) ----
      if (!(wid & 1)) {
        const int ls = wid >> 1, tsr = t0 + ls;
        const int j = blockIdx.x + tsr * gridDim.x;
        if (tsr < owned && j > i) {
          // entry e = 4r + c of the block: lanes e and e + 16 take k = 0, 1 and
          // k = 2, 3 of X_new[r, k] Y_new[k, c], then add the halves
          const int e = lane & 15, r = e >> 2, c = e & 3, k0 = (lane >> 4) * 2;
          cplx b = lane < 16 ? s_blk[16 * tsr + e] : cmake(0.0, 0.0);
          b = cfma(s_xn[16 * ls + 4 * r + k0], s_yn[16 * ls + 4 * k0 + c], b);
          b = cfma(s_xn[16 * ls + 4 * r + k0 + 1], s_yn[16 * ls + 4 * (k0 + 1) + c], b);
          b = cadd(b, shfl_c(b, lane ^ 16));
          if (lane < 16) {
            s_blk[16 * tsr + e] = b;
            d.blk[(size_t)16 * j + e] = b;
          }
        }
      }
      __syncthreads();   // s_xn / s_yn reused by the next pass; all stores precede the publication
    }
    ++p;
    if (p == d.k || i == N - 1) {
      if (blockIdx.x == 0 && threadIdx.x == 0) { d.state[0] = i + 1; d.state[1] = p; }
      finish_round(p);
      slice_round(p);
      return;   // the flush follows as its own launch
    }
    // ---- publish: the owned later sites now include p acceptances (the CTA
    //      barrier above orders every thread's stores before this fence) ----
    if (threadIdx.x == 0) {
      __threadfence();
      for (int t = 0; t < owned; ++t) {
        const int j = blockIdx.x + t * gridDim.x;
        if (j > i) *(volatile int*)(d.pub + j) = p;
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) { d.state[0] = N; d.state[1] = p; }
  finish_round(p);
  slice_round(p);
}

// Condition of the graph's WHILE node that repeats [delayed round, flush]:
// one more round while sites of the slice remain, at most max_rounds rounds
// per slice (state[2] counts them from the prepare kernel on), and none after
// an error bit is set.  rounds_total counts every round run this way.
__global__ void k_round_cond(cudaGraphConditionalHandle hc, int* state, int N, int max_rounds, const int* err,
                             unsigned long long* rounds_total) {
  if (threadIdx.x == 0) {
    const int it = state[2] + 1;
    state[2] = it;
    const bool more = it < max_rounds && __ldcg(&state[0]) < N && __ldcg(err) == 0;
    cudaGraphSetConditional(hc, more ? 1u : 0u);
    *rounds_total += 1ull;
  }
}

}  // namespace

cudaError_t launch_round_cond(cudaGraphConditionalHandle hc, int* state, int N, int max_rounds, const int* err,
                              unsigned long long* rounds_total, cudaStream_t st) {
  k_round_cond<<<1, 32, 0, st>>>(hc, state, N, max_rounds, err, rounds_total);
  return cudaGetLastError();
}

static size_t local_smem_bytes(int N) {
  return (size_t)N * (16 * sizeof(cplx) + sizeof(EvEntry)) + (size_t)3 * N * sizeof(double);
}

cudaError_t launch_local_prepare(const LocalUpdateArgs& a, SitePrep* prep, int* state, cudaStream_t st) {
  k_local_prepare<<<(a.mc.N + 3) / 4, 128, 0, st>>>(a, prep, state);
  return cudaGetLastError();
}

static size_t local_delayed_smem(int N, int k, int grid, bool cache) {
  const size_t owned = (size_t)(N + grid - 1) / grid;
  size_t c = 16 * owned + 128 + (size_t)2 * 16 * k;
  if (cache) c += 2 * owned * 4 * 4 * (size_t)k;
  return c * sizeof(cplx) + (size_t)3 * N * sizeof(double);
}

cudaError_t launch_local_delayed(const LocalUpdateArgs& a, const DelayedArgs& d, int sm_count, cudaStream_t st,
                                 int max_grid) {
  constexpr size_t kMaxSmem = 200 * 1024;
  const int N = a.mc.N;
  int grid = sm_count;    // one CTA per SM
  if (grid > N) grid = N;
  if (max_grid > 0 && grid > max_grid) grid = max_grid;
  const bool cache = local_delayed_smem(N, d.k, grid, true) <= kMaxSmem;
  const size_t smem = local_delayed_smem(N, d.k, grid, cache);
  if (smem > kMaxSmem) return cudaErrorInvalidValue;
  static SmemLimit limit_cache, limit_plain;
  if (cudaError_t ea = limit_cache.raise((const void*)k_local_delayed<true>, (int)kMaxSmem); ea != cudaSuccess)
    return ea;
  if (cudaError_t ea = limit_plain.raise((const void*)k_local_delayed<false>, (int)kMaxSmem); ea != cudaSuccess)
    return ea;
  const void* fn = cache ? (const void*)k_local_delayed<true> : (const void*)k_local_delayed<false>;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, LU_THREADS, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  LocalUpdateArgs ca = a;
  DelayedArgs cd = d;
  void* args[] = {&ca, &cd};
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(LU_THREADS), args, smem, st);
}

cudaError_t launch_local_updates(const LocalUpdateArgs& a, int sm_count, cudaStream_t st, int max_grid) {
  const size_t smem = local_smem_bytes(a.mc.N);
  static SmemLimit smem_limit;
  if (cudaError_t ea = smem_limit.raise((const void*)k_local_updates, 100 * 1024); ea != cudaSuccess) return ea;
  if (smem > 100 * 1024) return cudaErrorInvalidValue;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_local_updates, LU_THREADS, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (per_sm > 2) per_sm = 2;
  int grid = sm_count * per_sm;
  // small matrices: no more CTAs than warp tiles of the update
  const int n = a.mc.n;
  const int tiles = ((n + 127) / 128) * ((n + 3) / 4);
  const int need = (tiles + (LU_THREADS / 32) - 1) / (LU_THREADS / 32);
  if (grid > need) grid = need < 1 ? 1 : need;
  if (max_grid > 0 && grid > max_grid) grid = max_grid;
  LocalUpdateArgs copy = a;
  void* args[] = {&copy};
  return cudaLaunchCooperativeKernel((void*)k_local_updates, dim3(grid), dim3(LU_THREADS), args, smem, st);
}
