// Fermion correlators of true Green's functions (sm_103a).
//
// measure_etpc! (src/fermion_measurements.jl:388-424, expectation value
// _pc_ev :435-449), measure_etcdc! (:592-630, _etcdc_ev :641-653) and
// measure_zfpc! (:500-541, the pairing form summed over G(tau, 0) for
// tau = 1..M), measure_zfcdc! (:688-743, _zfcdc_ev :753-766) and
// measure_zfccc! (:814-888) for opdim 3, where G is accessed directly (:23-26).  G is n x n
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

// Zero-frequency charge-density correlators: one CTA per displacement,
// threads over the origins, summed over tau in a fixed order.  G is the
// equal-time G (as G(tau) and G(0)), Gt0s[tau] = G(tau, 0), G0ts[tau] the
// stored -G(0, tau); flavour a at ri, b at r0,
//   ev = (1 - G(ia, ia)) (1 - G(ib, ib)) - G0t(ib, ia) Gt0(ia, ib).
// out: C+ then C- (L^2 complex each), element (y, x) at y + L x.
__global__ void __launch_bounds__(ETC_THREADS) k_zfcdc(const cplx* __restrict__ G, const cplx* __restrict__ Gt0s,
                                                      const cplx* __restrict__ G0ts, int slices, int L,
                                                      double* __restrict__ out) {
  __shared__ double red[ETC_THREADS / 32];
  const int N = L * L, n = 4 * N;
  const int d = blockIdx.x;
  const int x = d / L, y = d - x * L;
  double cpr = 0.0, cpi = 0.0, cmr = 0.0, cmi = 0.0;
  for (int sl = 0; sl < slices; ++sl) {
    const cplx* Gt0 = Gt0s + (size_t)sl * n * n;
    const cplx* G0t = G0ts + (size_t)sl * n * n;
    for (int r0 = threadIdx.x; r0 < N; r0 += blockDim.x) {
      const int x0 = r0 / L, y0 = r0 - x0 * L;
      const int ri = (y0 + y) % L + L * ((x0 + x) % L);
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const int ia = a * N + ri;
        const cplx gaa = __ldg(&G[(size_t)ia * n + ia]);
        const cplx ua = cmake(1.0 - gaa.x, -gaa.y);
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int ib = b * N + r0;
          const cplx gbb = __ldg(&G[(size_t)ib * n + ib]);
          const cplx u = cmul(ua, cmake(1.0 - gbb.x, -gbb.y));
          const cplx c = cmul(__ldg(&G0t[(size_t)ia * n + ib]), __ldg(&Gt0[(size_t)ib * n + ia]));
          const cplx e = csub(u, c);
          cpr += e.x;
          cpi += e.y;
          if ((a & 1) == (b & 1)) { cmr += e.x; cmi += e.y; }
          else { cmr -= e.x; cmi -= e.y; }
        }
      }
    }
  }
  const double inv = 1.0 / N;
  const double s0 = block_sum_fixed(cpr, red), s1 = block_sum_fixed(cpi, red);
  const double s2 = block_sum_fixed(cmr, red), s3 = block_sum_fixed(cmi, red);
  if (threadIdx.x == 0) {
    out[2 * d] = s0 * inv;
    out[2 * d + 1] = s1 * inv;
    out[2 * N + 2 * d] = s2 * inv;
    out[2 * N + 2 * d + 1] = s3 * inv;
  }
}

// Zero-frequency current-current correlators Lambda_xx (blockIdx.y = 0) and
// Lambda_yy (blockIdx.y = 1): one CTA per displacement and direction, threads
// over the origins, summed over tau in a fixed order.  The hopping matrix is
// band-diagonal with T[j, i] = -t_dir(band) on the bonds i -> i + dir
// (src/hoppings.jl:19-40, accumulated: twice that at L = 2, where +dir and
// -dir reach the same site); thop[dir][band].  out: Lambda_xx then Lambda_yy
// (L^2 complex each, element (y, x) at y + L x), divided by -N.
__global__ void __launch_bounds__(ETC_THREADS) k_zfccc(const cplx* __restrict__ G, const cplx* __restrict__ Gt0s,
                                                      const cplx* __restrict__ G0ts, int slices, int L, double t00,
                                                      double t01, double t10, double t11, double* __restrict__ out) {
  __shared__ double red[ETC_THREADS / 32];
  const int N = L * L, n = 4 * N;
  const int d = blockIdx.x, dir = blockIdx.y;
  const int x = d / L, y = d - x * L;
  const double mult = L == 2 ? 2.0 : 1.0;
  const double tb[2] = {-mult * (dir == 0 ? t00 : t10), -mult * (dir == 0 ? t01 : t11)};   // by band
  const int dx = dir == 0 ? 1 : 0, dy = dir == 0 ? 0 : 1;
  auto at = [&](const cplx* M, int r, int c) { return __ldg(&M[(size_t)c * n + r]); };
  double lr = 0.0, li = 0.0;
  for (int sl = 0; sl < slices; ++sl) {
    const cplx* Gt0 = Gt0s + (size_t)sl * n * n;
    const cplx* G0t = G0ts + (size_t)sl * n * n;
    for (int r0 = threadIdx.x; r0 < N; r0 += blockDim.x) {
      const int x0 = r0 / L, y0 = r0 - x0 * L;
      const int ri = (y0 + y) % L + L * ((x0 + x) % L);
      const int rj = (y0 + y + dy) % L + L * ((x0 + x + dx) % L);
      const int r0p = (y0 + dy) % L + L * ((x0 + dx) % L);
#pragma unroll
      for (int f1 = 0; f1 < 4; ++f1) {
        const int ais = f1 * N + ri, ajs = f1 * N + rj;
        const double tij = tb[f1 & 1], tji = tij;
        // (tij G(ajs, ais) - tji G(ais, ajs)) of G(tau)
        const cplx ga = at(G, ajs, ais), gb = at(G, ais, ajs);
        const cplx u1 = cmake(tij * ga.x - tji * gb.x, tij * ga.y - tji * gb.y);
#pragma unroll
        for (int f2 = 0; f2 < 4; ++f2) {
          const int a0 = f2 * N + r0, a0p = f2 * N + r0p;
          const double t00p = tb[f2 & 1], t0p0 = t00p;
          const cplx gc = at(G, a0p, a0), gd = at(G, a0, a0p);
          const cplx u2 = cmake(t00p * gc.x - t0p0 * gd.x, t00p * gc.y - t0p0 * gd.y);
          cplx e = cmul(u1, u2);
          const cplx c1 = cscale(cmul(at(G0t, a0p, ais), at(Gt0, ajs, a0)), -tij * t00p);
          const cplx c2 = cscale(cmul(at(G0t, a0, ais), at(Gt0, ajs, a0p)), tij * t0p0);
          const cplx c3 = cscale(cmul(at(G0t, a0p, ajs), at(Gt0, ais, a0)), tji * t00p);
          const cplx c4 = cscale(cmul(at(G0t, a0, ajs), at(Gt0, ais, a0p)), -tji * t0p0);
          e = cadd(e, cadd(cadd(c1, c2), cadd(c3, c4)));
          lr += e.x;
          li += e.y;
        }
      }
    }
  }
  const double s0 = block_sum_fixed(lr, red), s1 = block_sum_fixed(li, red);
  if (threadIdx.x == 0) {
    const double inv = -1.0 / N;
    out[2 * N * dir + 2 * d] = s0 * inv;
    out[2 * N * dir + 2 * d + 1] = s1 * inv;
  }
}

}  // namespace

cudaError_t launch_zfccc(const cplx* G, const cplx* Gt0, const cplx* G0t, int slices, int L, const double thop[2][2],
                         double* out, cudaStream_t st) {
  if (L < 2 || L * L > 1024 || slices < 1) return cudaErrorInvalidValue;
  k_zfccc<<<dim3(L * L, 2), ETC_THREADS, 0, st>>>(G, Gt0, G0t, slices, L, thop[0][0], thop[0][1], thop[1][0],
                                                   thop[1][1], out);
  return cudaGetLastError();
}

cudaError_t launch_zfcdc(const cplx* G, const cplx* Gt0, const cplx* G0t, int slices, int L, double* out,
                         cudaStream_t st) {
  if (L < 1 || L * L > 1024 || slices < 1) return cudaErrorInvalidValue;
  k_zfcdc<<<L * L, ETC_THREADS, 0, st>>>(G, Gt0, G0t, slices, L, out);
  return cudaGetLastError();
}

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
