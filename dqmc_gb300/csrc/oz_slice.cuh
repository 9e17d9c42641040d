// Exact slicing of FP64 values into BF16 digits for the split-precision GEMM
// (k_ozaki.cu).  The delayed local-update kernel (k_local.cu) uses the same
// code to slice its own rows of the pending factors at the end of a round.
#pragma once
#include <cuda_bf16.h>
#include "common.cuh"
#include "kernels.h"

// The slicing runs on the integer units.  A row (column) scale is 2^E with
// E the frexp exponent of its largest |Re|/|Im|, taken from the exponent
// fields; x 2^-E (|.| < 1) becomes a 62-bit fixed-point integer built from
// the mantissa, and the S signed digits are cut off it by shifts, each
// rounded half to even: the same digits as rint on the FP64 value, which is
// exact at every step.
__device__ __forceinline__ int expo_field(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// x 2^(62 - E) as an integer (|x| < 2^E); values below 2^(E-62) are dropped
__device__ __forceinline__ long long fixed62(double x, int E) {
  const long long b = __double_as_longlong(x);
  const int ef = (int)((b >> 52) & 0x7FF);
  if (ef == 0) return 0;
  const long long m = (b & 0xFFFFFFFFFFFFFll) | 0x10000000000000ll;   // x = m 2^(ef - 1075)
  const int sh = ef - 1075 - E + 62;                                   // <= 9
  long long X = 0;
  if (sh >= 0) X = m << sh;
  else if (sh > -63) X = m >> (-sh);
  return b < 0 ? -X : X;
}

// next digit: round(X / 2^s) half to even, X <- X - digit 2^s
__device__ __forceinline__ int next_digit(long long& X, int s) {
  if (s <= 0) {
    const long long d = s == 0 ? X : X * (1ll << -s);
    X = 0;
    return (int)d;
  }
  long long q = X >> s;                        // floor
  const long long r = X - (q << s);            // in [0, 2^s)
  const long long half = 1ll << (s - 1);
  if (r > half || (r == half && (q & 1))) ++q;
  X -= q << s;
  return (int)q;
}

// One warp slices vector vec of one side of a product into o: side 0 a row of
// op(A) (As: Re digits in k, Im digits in Kpad + k), side 1 a column of op(B)
// (B'_re = [Re; -Im], B'_im = [Im; Re]); x(k) gives its entries for k < K,
// zeros are written up to Kpad, and the scale 2^E goes to sA / sB.
template <class Get>
__device__ __forceinline__ void oz_slice_vec(const OzSlices& o, int side, int vec, int K, Get x, int lane) {
  int me = 0;
  for (int k = lane; k < K; k += 32) {
    const cplx v = x(k);
    me = max(me, max(expo_field(v.x), expo_field(v.y)));
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) me = max(me, __shfl_xor_sync(0xffffffffu, me, s));
  const int E = me > 0 ? me - 1022 : 0;   // 2^E > max |.| (frexp exponent)
  if (lane == 0) (side ? o.sB : o.sA)[vec] = ldexp(1.0, E);
  const size_t Kp = 2 * (size_t)o.Kpad;
  for (int k = lane; k < o.Kpad; k += 32) {
    const cplx v = k < K ? x(k) : cmake(0.0, 0.0);
    long long xr = fixed62(v.x, E), xi = fixed62(v.y, E);
    for (int p = 0; p < o.S; ++p) {
      const int sft = 62 - (p + 1) * o.bits;
      const int ar = next_digit(xr, sft), ai = next_digit(xi, sft);
      if (side == 0) {
        __nv_bfloat16* a = o.As + (size_t)p * o.m * Kp + (size_t)vec * Kp;
        a[k] = __float2bfloat16_rn((float)ar);
        a[o.Kpad + k] = __float2bfloat16_rn((float)ai);
      } else {
        const size_t base = (size_t)p * o.n * Kp + (size_t)vec * Kp;
        o.Bre[base + k] = __float2bfloat16_rn((float)ar);
        o.Bre[base + o.Kpad + k] = __float2bfloat16_rn((float)-ai);
        o.Bim[base + k] = __float2bfloat16_rn((float)ai);
        o.Bim[base + o.Kpad + k] = __float2bfloat16_rn((float)ar);
      }
    }
  }
}
