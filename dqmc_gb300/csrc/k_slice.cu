// Slice-matrix application for the Assaad 4-site checkerboard (CBAssaad).
//
// Reference: src/slice_matrices.jl:101-226 (multiply_B_left!, _right!,
// _inv_left!, _inv_right!, multiply_daggered_B_left!), with the constant
// factors of src/hoppings_checkerboard.jl:20-136 and the per-site
// interaction blocks of src/interactions.jl:35-88.
//
//   B = Hb_half * Ha * Hb_half * diag(exp(dtau*mu)) * eV(+1)
//
// The reference applies these five sparse factors as five separate
// sparse x dense products, each writing a full temporary.  Here one CTA
// stages a slab of the matrix in shared memory and applies every factor
// (and, for the stack, several consecutive slices plus the trailing
// diagonal scaling) before writing it back: one read and one write of the
// slab per call.
//   * left application (B*M, B^-1*M, B^dag*M): the slab is a set of whole
//     columns (each column is an independent vector);
//   * right application (M*B, M*B^-1): the slab is a set of whole rows.
// Every factor is block-local: eV couples the 4 flavours of one site,
// a plaquette layer couples the 4 sites of one plaquette within one flavour.
#include "common.cuh"
#include "kernels.h"

namespace {

// Layout of a slab in shared memory: element e of vector v lives at
// buf[e * es + v * vs].
struct Slab {
  cplx* buf;
  int es, vs;
  __device__ cplx& at(int e, int v) const { return buf[e * es + v * vs]; }
};

// y = E x for one site block; E per src/interactions.jl:66-85, optionally
// transposed (right application uses x^T E = (E^T x)^T, E^T = conj(E)),
// with optional diagonal scalings before (pre) and after (post) the block.
__device__ __forceinline__ void apply_ev_site(const Slab& s, int v, int site, int N, double C,
                                              cplx S, double R, bool transpose,
                                              const double* pre, const double* post) {
  cplx x0 = s.at(site, v), x1 = s.at(site + N, v), x2 = s.at(site + 2 * N, v), x3 = s.at(site + 3 * N, v);
  if (pre) { x0 = cscale(x0, pre[0]); x1 = cscale(x1, pre[1]); x2 = cscale(x2, pre[0]); x3 = cscale(x3, pre[1]); }
  cplx Sa = transpose ? cconj(S) : S;   // entry (0,1) and (3,2)
  cplx Sb = cconj(Sa);                   // entry (1,0) and (2,3)
  // row0: C x0 + Sa x1 + R x3
  cplx y0 = cfma(Sa, x1, cmake(C * x0.x + R * x3.x, C * x0.y + R * x3.y));
  // row1: Sb x0 + C x1 - R x2
  cplx y1 = cfma(Sb, x0, cmake(C * x1.x - R * x2.x, C * x1.y - R * x2.y));
  // row2: -R x1 + C x2 + Sb x3
  cplx y2 = cfma(Sb, x3, cmake(C * x2.x - R * x1.x, C * x2.y - R * x1.y));
  // row3: R x0 + Sa x2 + C x3
  cplx y3 = cfma(Sa, x2, cmake(C * x3.x + R * x0.x, C * x3.y + R * x0.y));
  if (post) { y0 = cscale(y0, post[0]); y1 = cscale(y1, post[1]); y2 = cscale(y2, post[0]); y3 = cscale(y3, post[1]); }
  s.at(site, v) = y0; s.at(site + N, v) = y1; s.at(site + 2 * N, v) = y2; s.at(site + 3 * N, v) = y3;
}

// One plaquette layer on one plaquette of one flavour block:
// (x_i, x_j, x_m, x_n) <- P (x_i, x_j, x_m, x_n), P per
// src/hoppings_checkerboard.jl:48-56 with coefficients (cc, cs, sc, ss).
__device__ __forceinline__ void apply_plaquette(const Slab& s, int v, int i, int j, int m, int nn,
                                                double cc, double cs, double sc, double ss) {
  cplx xi = s.at(i, v), xj = s.at(j, v), xm = s.at(m, v), xn = s.at(nn, v);
  cplx yi = cmake(cc * xi.x + cs * xj.x + sc * xm.x + ss * xn.x, cc * xi.y + cs * xj.y + sc * xm.y + ss * xn.y);
  cplx yj = cmake(cs * xi.x + cc * xj.x + ss * xm.x + sc * xn.x, cs * xi.y + cc * xj.y + ss * xm.y + sc * xn.y);
  cplx ym = cmake(sc * xi.x + ss * xj.x + cc * xm.x + cs * xn.x, sc * xi.y + ss * xj.y + cc * xm.y + cs * xn.y);
  cplx yn = cmake(ss * xi.x + sc * xj.x + cs * xm.x + cc * xn.x, ss * xi.y + sc * xj.y + cs * xm.y + cc * xn.y);
  s.at(i, v) = yi; s.at(j, v) = yj; s.at(m, v) = ym; s.at(nn, v) = yn;
}

__device__ void plaquette_layer(const Slab& s, int nvec, const ModelConst& mc, int group, bool half,
                                bool inverse) {
  const int L = mc.L, N = mc.N, L2 = L / 2, P = N / 4;
  const int units = 4 * P * nvec;  // flavours x plaquettes x vectors
  for (int w = threadIdx.x; w < units; w += blockDim.x) {
    int v = w / (4 * P);
    int rem = w - v * 4 * P;
    int f = rem / P;
    int p = rem - f * P;
    int py = p % L2, px = p / L2;
    int y = 2 * py + group, x = 2 * px + group;
    int y1 = (y + 1) % L, x1 = (x + 1) % L;
    int base = f * N;
    int i = base + y + L * x, j = base + y1 + L * x, m = base + y + L * x1, nn = base + y1 + L * x1;
    int b = f & 1;
    double ch = half ? mc.ch_h[b] : mc.ch_f[b];
    double sh = half ? mc.sh_h[b] : mc.sh_f[b];
    double cv = half ? mc.cv_h[b] : mc.cv_f[b];
    double sv = half ? mc.sv_h[b] : mc.sv_f[b];
    if (inverse) { sh = -sh; sv = -sv; }
    apply_plaquette(s, v, i, j, m, nn, ch * cv, ch * sv, sh * cv, sh * sv);
  }
}

// Applies the eV (+mu) factor to all vectors.  mode selects the variant:
//   LEFT_B:     y = mu * E(+1) x             (B = ... mu eV)
//   LEFT_BINV:  y = E(-1) * mu^-1 x
//   LEFT_BDAG:  y = E(+1) * mu x             (B^dag = eV mu ...)
//   RIGHT_B:    y = E(+1)^T * mu x           (row vector: x^T mu eV)
//   RIGHT_BINV: y = mu^-1 * E(-1)^T x        (row vector: x^T eV^-1 mu^-1)
__device__ void ev_layer(const Slab& s, int nvec, const ModelConst& mc, const EvEntry* ev, int mode) {
  const int N = mc.N;
  const int units = N * nvec;
  double pw = (mode == SLICE_LEFT_BINV || mode == SLICE_RIGHT_BINV) ? -1.0 : 1.0;
  bool transpose = (mode == SLICE_RIGHT_B || mode == SLICE_RIGHT_BINV);
  double mup[2] = {mc.emu[0], mc.emu[1]};
  double mui[2] = {mc.emu_inv[0], mc.emu_inv[1]};
  const double* pre = nullptr;
  const double* post = nullptr;
  switch (mode) {
    case SLICE_LEFT_B: post = mup; break;
    case SLICE_LEFT_BINV: pre = mui; break;
    case SLICE_LEFT_BDAG: pre = mup; break;
    case SLICE_RIGHT_B: pre = mup; break;
    case SLICE_RIGHT_BINV: post = mui; break;
  }
  for (int w = threadIdx.x; w < units; w += blockDim.x) {
    int v = w / N;
    int site = w - v * N;
    EvEntry e = ev[site];
    apply_ev_site(s, v, site, N, e.C, cmake(pw * e.Sr, pw * e.Si), pw * e.R, transpose, pre, post);
  }
}

// Full factor sequence of one slice for a given mode (applied in the order
// the reference applies its sparse products).
__device__ void apply_slice(const Slab& s, int nvec, const ModelConst& mc, const EvEntry* ev, int mode) {
  switch (mode) {
    case SLICE_LEFT_B:  // eV, mu, Hb_half, Ha, Hb_half
    case SLICE_RIGHT_B:
      if (mode == SLICE_LEFT_B) { ev_layer(s, nvec, mc, ev, mode); __syncthreads(); }
      plaquette_layer(s, nvec, mc, 1, true, false); __syncthreads();
      plaquette_layer(s, nvec, mc, 0, false, false); __syncthreads();
      plaquette_layer(s, nvec, mc, 1, true, false); __syncthreads();
      if (mode == SLICE_RIGHT_B) { ev_layer(s, nvec, mc, ev, mode); __syncthreads(); }
      break;
    case SLICE_LEFT_BINV:  // Hb_half^-1, Ha^-1, Hb_half^-1, mu^-1, eV^-1
    case SLICE_RIGHT_BINV: // eV^-1, mu^-1, Hb_half^-1, Ha^-1, Hb_half^-1
      if (mode == SLICE_RIGHT_BINV) { ev_layer(s, nvec, mc, ev, mode); __syncthreads(); }
      plaquette_layer(s, nvec, mc, 1, true, true); __syncthreads();
      plaquette_layer(s, nvec, mc, 0, false, true); __syncthreads();
      plaquette_layer(s, nvec, mc, 1, true, true); __syncthreads();
      if (mode == SLICE_LEFT_BINV) { ev_layer(s, nvec, mc, ev, mode); __syncthreads(); }
      break;
    case SLICE_LEFT_BDAG:  // Hb_half^T, Ha^T, Hb_half^T, mu, eV (real symmetric / Hermitian factors)
      plaquette_layer(s, nvec, mc, 1, true, false); __syncthreads();
      plaquette_layer(s, nvec, mc, 0, false, false); __syncthreads();
      plaquette_layer(s, nvec, mc, 1, true, false); __syncthreads();
      ev_layer(s, nvec, mc, ev, mode); __syncthreads();
      break;
    case SLICE_EFF_RIGHT:     // x^T Hb_half Ha_half (src/fermion_measurements.jl:1132-1135)
      plaquette_layer(s, nvec, mc, 1, true, false); __syncthreads();
      plaquette_layer(s, nvec, mc, 0, true, false); __syncthreads();
      break;
    case SLICE_EFF_LEFT_INV:  // Ha_half^-1 Hb_half^-1 x (src/fermion_measurements.jl:1136-1139)
      plaquette_layer(s, nvec, mc, 1, true, true); __syncthreads();
      plaquette_layer(s, nvec, mc, 0, true, true); __syncthreads();
      break;
  }
}

// Left application on whole columns.  Applies, for k = 0..count-1, the
// slice (first + k*step) in `mode`, then optionally scales column c by
// colscale[c] (rmul!(U, Diagonal(d)) of add_slice_sequence_*).
__global__ void k_apply_cols(cplx* __restrict__ A, int n, int cols_per_cta, ModelConst mc,
                             const EvEntry* __restrict__ evtab, int first, int count, int step, int mode,
                             const double* __restrict__ colscale) {
  extern __shared__ double4 smem_raw[];
  cplx* buf = reinterpret_cast<cplx*>(smem_raw);
  EvEntry* ev = reinterpret_cast<EvEntry*>(buf + (size_t)cols_per_cta * n);
  const int c0 = blockIdx.x * cols_per_cta;
  const int nc = min(cols_per_cta, n - c0);
  if (nc <= 0) return;
  const size_t total = (size_t)nc * n;
  const cplx* src = A + (size_t)c0 * n;
  for (size_t e = threadIdx.x; e < total; e += blockDim.x) buf[e] = src[e];
  Slab s{buf, 1, n};
  for (int k = 0; k < count; ++k) {
    int sl = first + k * step;
    __syncthreads();
    for (int i = threadIdx.x; i < mc.N; i += blockDim.x) ev[i] = evtab[(size_t)sl * mc.N + i];
    __syncthreads();
    apply_slice(s, nc, mc, ev, mode);
  }
  cplx* dst = A + (size_t)c0 * n;
  for (size_t e = threadIdx.x; e < total; e += blockDim.x) {
    cplx val = buf[e];
    if (colscale) val = cscale(val, colscale[c0 + e / n]);
    dst[e] = val;
  }
}

// Right application on whole rows: rows [r0, r0+nr) of A, stored in shared
// memory interleaved (element e of row v at buf[e*rows_per_cta + v]).
__global__ void k_apply_rows(cplx* __restrict__ A, int n, int rows_per_cta, ModelConst mc,
                             const EvEntry* __restrict__ evtab, int first, int count, int step, int mode) {
  extern __shared__ double4 smem_raw[];
  cplx* buf = reinterpret_cast<cplx*>(smem_raw);
  EvEntry* ev = reinterpret_cast<EvEntry*>(buf + (size_t)rows_per_cta * n);
  const int R = rows_per_cta;
  const int r0 = blockIdx.x * R;
  const int nr = min(R, n - r0);
  if (nr <= 0) return;
  const size_t total = (size_t)R * n;
  for (size_t e = threadIdx.x; e < total; e += blockDim.x) {
    int c = (int)(e / R), v = (int)(e - (size_t)c * R);
    buf[e] = v < nr ? A[(size_t)c * n + r0 + v] : cmake(0.0, 0.0);
  }
  Slab s{buf, R, 1};
  for (int k = 0; k < count; ++k) {
    int sl = first + k * step;
    __syncthreads();
    for (int i = threadIdx.x; i < mc.N; i += blockDim.x) ev[i] = evtab[(size_t)sl * mc.N + i];
    __syncthreads();
    apply_slice(s, nr, mc, ev, mode);
  }
  __syncthreads();
  for (size_t e = threadIdx.x; e < total; e += blockDim.x) {
    int c = (int)(e / R), v = (int)(e - (size_t)c * R);
    if (v < nr) A[(size_t)c * n + r0 + v] = buf[e];
  }
}

// Per-site interaction entries for every slice from the field
// (src/interactions.jl:52-64, power +1).
__global__ void k_build_evtab(const double* __restrict__ phi, EvEntry* __restrict__ evtab, int N, int M,
                              double lambda_dtau) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * M) return;
  const double* p = phi + 3 * (size_t)idx;   // phi[:, i, l], idx = i + N*l
  double nrm = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
  double a = lambda_dtau * nrm;
  double sh = sinh(a) / nrm;
  EvEntry e;
  e.C = cosh(a);
  e.Sr = -p[0] * sh;
  e.Si = p[1] * sh;
  e.R = -p[2] * sh;
  evtab[idx] = e;
}

}  // namespace

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static int pick_cols_per_cta(int n) {
  // ~32 KB of slab per CTA keeps 4-6 CTAs per SM and >= 2 waves of work.
  int c = 32768 / (16 * n);
  if (c < 1) c = 1;
  if (c > 64) c = 64;
  return c;
}

cudaError_t launch_apply_cols(cplx* A, int n, const ModelConst& mc, const void* evtab, int first_slice0,
                              int count, int step, int mode, const double* colscale, cudaStream_t st) {
  int cpc = pick_cols_per_cta(n);
  int grid = (n + cpc - 1) / cpc;
  size_t smem = (size_t)cpc * n * sizeof(cplx) + (size_t)mc.N * sizeof(EvEntry);
  static SmemLimit smem_limit;
  if (cudaError_t ea = smem_limit.raise((const void*)k_apply_cols, 200 * 1024); ea != cudaSuccess) return ea;
  k_apply_cols<<<grid, 256, smem, st>>>(A, n, cpc, mc, (const EvEntry*)evtab, first_slice0, count, step, mode,
                                         colscale);
  return cudaGetLastError();
}

cudaError_t launch_apply_rows(cplx* A, int n, const ModelConst& mc, const void* evtab, int first_slice0,
                              int count, int step, int mode, cudaStream_t st) {
  int rpc = pick_cols_per_cta(n);
  int grid = (n + rpc - 1) / rpc;
  size_t smem = (size_t)rpc * n * sizeof(cplx) + (size_t)mc.N * sizeof(EvEntry);
  static SmemLimit smem_limit;
  if (cudaError_t ea = smem_limit.raise((const void*)k_apply_rows, 200 * 1024); ea != cudaSuccess) return ea;
  k_apply_rows<<<grid, 256, smem, st>>>(A, n, rpc, mc, (const EvEntry*)evtab, first_slice0, count, step, mode);
  return cudaGetLastError();
}

cudaError_t launch_build_evtab(const double* phi, void* evtab, int N, int M, double lambda_dtau,
                               cudaStream_t st) {
  int total = N * M;
  k_build_evtab<<<(total + 255) / 256, 256, 0, st>>>(phi, (EvEntry*)evtab, N, M, lambda_dtau);
  return cudaGetLastError();
}

size_t evtab_entry_bytes() { return sizeof(EvEntry); }
