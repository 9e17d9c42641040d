// Adjoint force: gradient of log|det M(phi)|, M = 1 + B_M ... B_1, with
// respect to every field component, from the equal-time G of each slice.
//
// Not an operation of the reference; built from its pieces.  With B_l =
// H mu eV_l (src/slice_matrices.jl:101-129) the push-through identity gives
//   d log det M = tr[B_l^-1 (1 - G_{l+1}) dB_l] = -tr[G_l eV_l^-1 deV_l]
// (det of every 4x4 interaction block is 1, src/interactions.jl:66-85), so
//   d log|det M| / d phi[a, i, l] = -Re tr(G_l[ii] E_i^-1 dE_i/dphi_a)
// with G_l[ii] the 4x4 site block of G at slice l and E_i the site's block.
#include "common.cuh"
#include "kernels.h"

namespace {

__device__ __forceinline__ cplx blk(int r, int c, double C, cplx S, double R) {
  switch (r * 4 + c) {
    case 0: case 5: case 10: case 15: return cmake(C, 0.0);
    case 1: case 14: return S;
    case 4: case 11: return cconj(S);
    case 3: case 12: return cmake(R, 0.0);
    case 6: case 9: return cmake(-R, 0.0);
    default: return cmake(0.0, 0.0);
  }
}

__global__ void k_force_slice(const cplx* __restrict__ G, const double* __restrict__ phi, double* __restrict__ grad,
                              int N, int slice0, double lambda_dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int n = 4 * N;
  const double* op = phi + ((size_t)N * slice0 + i) * 3;
  const double nrm = sqrt(op[0] * op[0] + op[1] * op[1] + op[2] * op[2]);
  const double x = lambda_dtau * nrm;
  const double sh = sinh(x) / nrm, C = cosh(x);
  const double dsh = (lambda_dtau * C - sh) / (nrm * nrm);   // (d sh / d op_a) / op_a
  // E^-1 = block with power -1: S -> -S, R -> -R
  const cplx Si = cmake(op[0] * sh, -op[1] * sh);
  const double Ri = op[2] * sh;
  cplx g[4][4];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) g[r][c] = G[(size_t)(i + c * N) * n + i + r * N];
  for (int a = 0; a < 3; ++a) {
    const double dC = lambda_dtau * op[a] * sh;
    const cplx dS = cmake(-op[0] * dsh * op[a] - (a == 0 ? sh : 0.0), op[1] * dsh * op[a] + (a == 1 ? sh : 0.0));
    const double dR = -op[2] * dsh * op[a] - (a == 2 ? sh : 0.0);
    // tr(G E^-1 dE) = sum_{r,c} G[r][c] (E^-1 dE)[c][r]
    cplx tr = cmake(0.0, 0.0);
    for (int c = 0; c < 4; ++c)
      for (int r = 0; r < 4; ++r) {
        cplx p = cmake(0.0, 0.0);
        for (int k = 0; k < 4; ++k) p = cfma(blk(c, k, C, Si, Ri), blk(k, r, dC, dS, dR), p);
        tr = cfma(g[r][c], p, tr);
      }
    grad[((size_t)N * slice0 + i) * 3 + a] = -tr.x;
  }
}

__global__ void k_shift_field(double* phi, size_t NM, double s0, double s1, double s2) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < NM; e += (size_t)gridDim.x * blockDim.x) {
    phi[3 * e] += s0;
    phi[3 * e + 1] += s1;
    phi[3 * e + 2] += s2;
  }
}

}  // namespace

cudaError_t launch_shift_field(double* phi, size_t NM, double s0, double s1, double s2, cudaStream_t st) {
  int grid = (int)((NM + 255) / 256);
  if (grid > 4096) grid = 4096;
  k_shift_field<<<grid, 256, 0, st>>>(phi, NM, s0, s1, s2);
  return cudaGetLastError();
}

cudaError_t launch_force_slice(const cplx* G, const double* phi, double* grad, int N, int slice0, double lambda_dtau,
                               cudaStream_t st) {
  k_force_slice<<<(N + 127) / 128, 128, 0, st>>>(G, phi, grad, N, slice0, lambda_dtau);
  return cudaGetLastError();
}
