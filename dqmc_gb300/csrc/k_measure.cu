// Fermion correlators of true Green's functions (sm_103a).
//
// measure_etpc! (src/fermion_measurements.jl:388-427, expectation value
// _pc_ev :436-451), measure_etcdc! (:580-620, _etcdc_ev :630-643) and
// measure_zfpc! (:486-530, the pairing form summed over G(tau, 0) for
// tau = 1..M) for opdim 3, where G is accessed directly (:23-26).  G is n x n
// column-major with index flavour * N + site (flavours xu, yd, xd, yu), sites
// y + L x with periodic boundaries (siteidx, :7-12).
#include "kernels.h"

namespace {

constexpr int ETC_THREADS = 256;

__device__ __forceinline__ double block_sum_fixed(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();   // red reused by consecutive calls
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < ETC_THREADS / 32; ++w) s += red[w];
  return s;   // valid in thread 0
}

// One CTA per displacement d = y + L x; threads over the origins r0, each
// origin's terms summed over the `slices` matrices (stride n^2) in a fixed
// order, then a fixed-order block sum.  out: P+ (L^2), P- (L^2), and unless
// PAIR_ONLY C+ (L^2 complex), C- (L^2 complex); element (y, x) of each L x L
// array at y + L x (the reference's Pp[y+1, x+1]).
template <bool PAIR_ONLY>
__global__ void __launch_bounds__(ETC_THREADS) k_fermion_corr(const cplx* __restrict__ Gs, int slices, int L,
                                                             double* __restrict__ out) {
  __shared__ double red[ETC_THREADS / 32];
  const int N = L * L, n = 4 * N;
  const int d = blockIdx.x;
  const int x = d / L, y = d - x * L;
  const cplx* G = Gs;
  auto g = [&](int i, int j) { return __ldg(&G[(size_t)j * n + i]); };
  // (j1, j2, j3, j4) flavours of the four pairing terms (0-based xu, yd, xd, yu = 0, 1, 2, 3)
  const int js[4][4] = {{2, 0, 0, 2}, {2, 0, 3, 1}, {1, 3, 0, 2}, {1, 3, 3, 1}};
  double pp = 0.0, pm = 0.0, cpr = 0.0, cpi = 0.0, cmr = 0.0, cmi = 0.0;
  for (int sl = 0; sl < slices; ++sl) {
    G = Gs + (size_t)sl * n * n;
    for (int r0 = threadIdx.x; r0 < N; r0 += blockDim.x) {
      const int x0 = r0 / L, y0 = r0 - x0 * L;
      const int ri = (y0 + y) % L + L * ((x0 + x) % L);
      // pairing: ev_q = Re[G(i1, i4) G(i2, i3) - G(i1, i3) G(i2, i4)]
      double ev[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i1 = js[q][0] * N + ri, i2 = js[q][1] * N + ri, i3 = js[q][2] * N + r0, i4 = js[q][3] * N + r0;
        const cplx a = cmul(g(i1, i4), g(i2, i3)), b = cmul(g(i1, i3), g(i2, i4));
        ev[q] = a.x - b.x;
      }
      pm += ev[0] - ev[1] - ev[2] + ev[3];
      pp += ev[0] + ev[1] + ev[2] + ev[3];
      if (PAIR_ONLY) continue;
      // charge density: flavour a at ri, b at r0 (bands X: a = 0, 2; Y: a = 1, 3),
      // ev = (1 - G(ia, ia)) (1 - G(ib, ib)) + (delta(ia, ib) - G(ib, ia)) G(ia, ib),
      // C- weights equal bands +1 and different bands -1
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const int ia = a * N + ri;
        const cplx gaa = g(ia, ia);
        const cplx ua = cmake(1.0 - gaa.x, -gaa.y);
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int ib = b * N + r0;
          const cplx gbb = g(ib, ib);
          cplx e = cmul(ua, cmake(1.0 - gbb.x, -gbb.y));
          const cplx gba = g(ib, ia);
          const cplx c1 = cmake((ia == ib ? 1.0 : 0.0) - gba.x, -gba.y);
          e = cadd(e, cmul(c1, g(ia, ib)));
          cpr += e.x;
          cpi += e.y;
          if ((a & 1) == (b & 1)) { cmr += e.x; cmi += e.y; }
          else { cmr -= e.x; cmi -= e.y; }
        }
      }
    }
  }
  const double inv = 1.0 / N;
  const double s0 = block_sum_fixed(pp, red), s1 = block_sum_fixed(pm, red);
  if (PAIR_ONLY) {
    if (threadIdx.x == 0) {
      out[d] = s0 * inv;
      out[N + d] = s1 * inv;
    }
    return;
  }
  const double s2 = block_sum_fixed(cpr, red), s3 = block_sum_fixed(cpi, red);
  const double s4 = block_sum_fixed(cmr, red), s5 = block_sum_fixed(cmi, red);
  if (threadIdx.x == 0) {
    out[d] = s0 * inv;
    out[N + d] = s1 * inv;
    out[2 * N + 2 * d] = s2 * inv;
    out[2 * N + 2 * d + 1] = s3 * inv;
    out[4 * N + 2 * d] = s4 * inv;
    out[4 * N + 2 * d + 1] = s5 * inv;
  }
}

}  // namespace

cudaError_t launch_equal_time_corr(const cplx* G, int L, double* out, cudaStream_t st) {
  if (L < 1 || L * L > 1024) return cudaErrorInvalidValue;
  k_fermion_corr<false><<<L * L, ETC_THREADS, 0, st>>>(G, 1, L, out);
  return cudaGetLastError();
}

cudaError_t launch_zfpc(const cplx* Gt0, int slices, int L, double* out, cudaStream_t st) {
  if (L < 1 || L * L > 1024 || slices < 1) return cudaErrorInvalidValue;
  k_fermion_corr<true><<<L * L, ETC_THREADS, 0, st>>>(Gt0, slices, L, out);
  return cudaGetLastError();
}
