// Split-precision complex GEMM on the BF16 tensor cores (Ozaki scheme).
//
//   C = alpha * diag(rs) * op(A) * op(B) * diag(cs) + beta * C     (complex FP64)
//
// GB300 runs FP64 at ~1/1500 of its BF16 tensor rate, so the mixed-precision
// form computes the dense products of the UDT stabilisation and of the
// delayed local-update flush as sums of exact BF16 x BF16 -> FP32 products:
//
//  * every row i of op(A) gets a power-of-two scale sigma_i >= max_k |op(A)_ik|
//    (real and imaginary parts together), every column j of op(B) a scale
//    tau_j; the scaled entries lie in [-1, 1];
//  * each scaled entry x is cut into S slices of B_BITS bits,
//    x ~ sum_p 2^{-B_BITS p} a_p with integers |a_p| <= 2^B_BITS, which BF16
//    holds exactly;
//  * the complex product is two real GEMMs with K' = 2K on stacked operands,
//    A' = [Re A, Im A] and B'_re = [Re B; -Im B], B'_im = [Im B; Re B];
//  * slice pairs (p, q) with p + q = t <= S + 1 are accumulated into one FP32
//    accumulator per t; with K' * S * 2^{2 B_BITS} <= 2^24 every partial sum is
//    an integer below 2^24, so the FP32 accumulation is exact; the groups are
//    combined in FP64 with their weights 2^{-B_BITS t} and the scales.
// The only error is the truncation of the slice expansion (~2^{-B_BITS S}
// relative to sigma_i tau_j K).
//
// The tensor-core products use warp-level mma.sync m16n8k16 (BF16 in, FP32
// accumulate) fed from shared memory with ldmatrix; operands are staged with
// cp.async double buffering.
#include <cuda_bf16.h>
#include <cmath>
#include <type_traits>
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int OZ_BM = 64, OZ_BN = 64, OZ_BK = 32;
constexpr int OZ_THREADS = 256;
constexpr int OZ_LDS = OZ_BK + 8;   // padded shared-memory row (bf16 elements): 80 B, conflict-free ldmatrix
constexpr int OZ_STAGES = 3;        // cp.async pipeline depth (46 KB of static shared memory)

// ---------------------------------------------------------------------------
// split: slices of op(X) scaled per row ("row" side = A) or per column (B side)
// ---------------------------------------------------------------------------
// element (r, c) of op(X) where X is column-major with leading dimension ld
__device__ __forceinline__ cplx op_elem(const cplx* X, int ld, int r, int c, char op) {
  if (op == 'N') return X[(size_t)c * ld + r];
  cplx v = X[(size_t)r * ld + c];
  return op == 'C' ? cconj(v) : v;
}

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

__device__ __forceinline__ int block_max_int(int v, int* red) {
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  int t = 0;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t = max(t, red[q]);
  return t;
}

// A side: op(A) is rows x K; writes S slices of A' (rows x Kp, row-major,
// Kp = 2 * Kpad): row i = [Re op(A)_i,:  Im op(A)_i,:], zero padded.
__global__ void k_oz_split_rows(const cplx* __restrict__ X, int ld, char op, int rows, int K, int Kpad, int S,
                                int bits, __nv_bfloat16* __restrict__ out, double* __restrict__ scale,
                                const int* __restrict__ active) {
  const int i = blockIdx.x;
  if (i >= rows) return;
  if (active) {   // only the first 4p inner indices are live (delayed-update flush)
    const int kk = 4 * *active;
    if (kk == 0) return;
    if (kk < K) K = kk;
  }
  __shared__ int red[32];
  int me = 0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    const cplx v = op_elem(X, ld, i, k, op);
    me = max(me, max(expo_field(v.x), expo_field(v.y)));
  }
  me = block_max_int(me, red);
  const int E = me > 0 ? me - 1022 : 0;   // 2^E > max |.| (frexp exponent)
  if (threadIdx.x == 0) scale[i] = ldexp(1.0, E);
  const size_t Kp = 2 * (size_t)Kpad;
  for (int k = threadIdx.x; k < Kpad; k += blockDim.x) {
    const cplx v = k < K ? op_elem(X, ld, i, k, op) : cmake(0.0, 0.0);
    long long xr = fixed62(v.x, E), xi = fixed62(v.y, E);
    for (int p = 0; p < S; ++p) {
      const int sft = 62 - (p + 1) * bits;
      const int ar = next_digit(xr, sft), ai = next_digit(xi, sft);
      __nv_bfloat16* o = out + (size_t)p * rows * Kp + (size_t)i * Kp;
      o[k] = __float2bfloat16_rn((float)ar);
      o[Kpad + k] = __float2bfloat16_rn((float)ai);
    }
  }
}

// B side: op(B) is K x cols; writes S slices of B'_re and B'_im (cols x Kp,
// K contiguous per column): column j of B'_re = [Re op(B)_:,j ; -Im op(B)_:,j],
// of B'_im = [Im op(B)_:,j ; Re op(B)_:,j].
__global__ void k_oz_split_cols(const cplx* __restrict__ X, int ld, char op, int K, int cols, int Kpad, int S,
                                int bits, __nv_bfloat16* __restrict__ out_re, __nv_bfloat16* __restrict__ out_im,
                                double* __restrict__ scale, const int* __restrict__ active) {
  const int j = blockIdx.x;
  if (j >= cols) return;
  if (active) {
    const int kk = 4 * *active;
    if (kk == 0) return;
    if (kk < K) K = kk;
  }
  __shared__ int red[32];
  int me = 0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    const cplx v = op_elem(X, ld, k, j, op);
    me = max(me, max(expo_field(v.x), expo_field(v.y)));
  }
  me = block_max_int(me, red);
  const int E = me > 0 ? me - 1022 : 0;
  if (threadIdx.x == 0) scale[j] = ldexp(1.0, E);
  const size_t Kp = 2 * (size_t)Kpad;
  for (int k = threadIdx.x; k < Kpad; k += blockDim.x) {
    const cplx v = k < K ? op_elem(X, ld, k, j, op) : cmake(0.0, 0.0);
    long long xr = fixed62(v.x, E), xi = fixed62(v.y, E);
    for (int p = 0; p < S; ++p) {
      const int sft = 62 - (p + 1) * bits;
      const int ar = next_digit(xr, sft), ai = next_digit(xi, sft);
      const size_t base = (size_t)p * cols * Kp + (size_t)j * Kp;
      out_re[base + k] = __float2bfloat16_rn((float)ar);
      out_re[base + Kpad + k] = __float2bfloat16_rn((float)-ai);
      out_im[base + k] = __float2bfloat16_rn((float)ai);
      out_im[base + Kpad + k] = __float2bfloat16_rn((float)ar);
    }
  }
}

// ---------------------------------------------------------------------------
// products
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::); }

__device__ __forceinline__ void ldmatrix_x4(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3, const void* p) {
  unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(s));
}
__device__ __forceinline__ void ldmatrix_x2(unsigned& r0, unsigned& r1, const void* p) {
  unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(s));
}
__device__ __forceinline__ void mma_bf16(float* d, const unsigned* a, const unsigned* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct OzArgs {
  const __nv_bfloat16* As;   // S x (m x Kp), row-major
  const __nv_bfloat16* Bre;  // S x (n x Kp), K contiguous per column
  const __nv_bfloat16* Bim;
  const double* sA;          // (m) row scales
  const double* sB;          // (n) column scales
  int m, n, Kp, S, bits;
  cplx alpha, beta;
  cplx* C;
  int ldc;
  const double* rs;          // optional extra row scaling
  const double* cs;          // optional extra column scaling
  const int* active;         // optional: nothing to do when *active == 0
  int int_combine;           // group sums combined exactly in 64-bit integers
  int kchunk;                // split K: K steps per CTA layer (blockIdx.z); 0 = all
  unsigned long long* acc;   // split K: exact integer sums (m x n x {re, im}), finished by k_oz_finalize
                             // (zero on entry; the finaliser zeroes what it read)
};

// Final scaling and accumulation of one output value (shared by the GEMM and
// the split-K finaliser).
__device__ __forceinline__ void oz_store(const OzArgs& a, int row, int col, double vr, double vi, double wint,
                                         bool plain) {
  double f = a.sA[row] * a.sB[col] * wint;
  if (a.rs) f *= a.rs[row];
  if (a.cs) f *= a.cs[col];
  cplx v = cmake(vr * f, vi * f);
  cplx* cp = &a.C[(size_t)col * a.ldc + row];
  if (plain) {
    // alpha = +-1, beta in {0, 1}: one multiply and at most one add per value
    if (a.alpha.x < 0.0) v = cmake(-v.x, -v.y);
    if (a.beta.x != 0.0) v = cadd(*cp, v);
  } else {
    v = cmul(a.alpha, v);
    if (a.beta.x != 0.0 || a.beta.y != 0.0) v = cfma(a.beta, *cp, v);
  }
  *cp = v;
}

__device__ __forceinline__ bool oz_plain(const OzArgs& a) {
  return (a.alpha.x == 1.0 || a.alpha.x == -1.0) && a.alpha.y == 0.0 && a.beta.y == 0.0 &&
         (a.beta.x == 0.0 || a.beta.x == 1.0);
}

// One CTA: 64 x 64 output tile; 8 warps in a 2 x 4 grid of 32 x 16 warp tiles.
template <bool INT>
__global__ void __launch_bounds__(OZ_THREADS, 2) k_oz_gemm(OzArgs a) {
  if (a.active && *a.active == 0) return;
  __shared__ __align__(16) __nv_bfloat16 sA[OZ_STAGES][OZ_BM * OZ_LDS];
  __shared__ __align__(16) __nv_bfloat16 sBr[OZ_STAGES][OZ_BN * OZ_LDS];
  __shared__ __align__(16) __nv_bfloat16 sBi[OZ_STAGES][OZ_BN * OZ_LDS];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int wm = wid >> 2, wn = wid & 3;          // warp tile origin: rows 32*wm, cols 16*wn
  const int i0 = blockIdx.y * OZ_BM, j0 = blockIdx.x * OZ_BN;
  const size_t Kp = a.Kp;
  const size_t sliceA = (size_t)a.m * Kp, sliceB = (size_t)a.n * Kp;

  // accumulators over the groups: 2 (m16) x 2 (n8) mma tiles x 4 values, re
  // and im; exact 64-bit integers (Horner in 2^bits) or FP64 with weights
  typedef typename std::conditional<INT, long long, double>::type acc_t;
  acc_t accr[2][2][4], acci[2][2][4];
#pragma unroll
  for (int x = 0; x < 2; ++x)
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int z = 0; z < 4; ++z) { accr[x][y][z] = 0; acci[x][y][z] = 0; }

  // staging of one K step of pair (p, q) into buffer `buf`
  auto stage = [&](int buf, int p, int q, int k0) {
    // 64 rows x 32 bf16 = 4 chunks of 16 B per row; 256 threads -> 1 chunk each per operand
    const int r = tid >> 2, ch = tid & 3;
    {
      int gi = i0 + r;
      __nv_bfloat16* dst = &sA[buf][r * OZ_LDS + ch * 8];
      if (gi < a.m) cp_async16(dst, a.As + (size_t)p * sliceA + (size_t)gi * Kp + k0 + ch * 8);
      else *reinterpret_cast<uint4*>(dst) = make_uint4(0, 0, 0, 0);
    }
    {
      int gj = j0 + r;
      __nv_bfloat16* dr = &sBr[buf][r * OZ_LDS + ch * 8];
      __nv_bfloat16* di = &sBi[buf][r * OZ_LDS + ch * 8];
      if (gj < a.n) {
        cp_async16(dr, a.Bre + (size_t)q * sliceB + (size_t)gj * Kp + k0 + ch * 8);
        cp_async16(di, a.Bim + (size_t)q * sliceB + (size_t)gj * Kp + k0 + ch * 8);
      } else {
        *reinterpret_cast<uint4*>(dr) = make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4*>(di) = make_uint4(0, 0, 0, 0);
      }
    }
    cp_async_commit();
  };

  const int ksteps_all = (int)(Kp / OZ_BK);
  const int ks0 = a.kchunk ? (int)blockIdx.z * a.kchunk : 0;
  const int ksteps = a.kchunk ? min(ksteps_all, ks0 + a.kchunk) : ksteps_all;
  // one stream of (group t, slice pair (p, q = t - p), K step) items, staged
  // OZ_STAGES - 1 items ahead across pair and group boundaries
  auto pmin_of = [&](int t) { return t - a.S > 1 ? t - a.S : 1; };
  auto pmax_of = [&](int t) { return t - 1 < a.S ? t - 1 : a.S; };
  auto advance = [&](int& t, int& p, int& ks) {
    if (++ks < ksteps) return;
    ks = ks0;
    if (++p <= pmax_of(t)) return;
    ++t;
    p = pmin_of(t);
  };
  int lt = 2, lp = pmin_of(2), lks = ks0;   // next item to stage
  int ct = 2, cp = pmin_of(2), cks = ks0;   // item being computed
  const bool any = ks0 < ksteps;
  int staged = 0;                           // items staged so far
  for (int pre = 0; any && pre < OZ_STAGES - 1 && lt <= a.S + 1; ++pre) {
    stage(staged % OZ_STAGES, lp - 1, lt - lp - 1, lks * OZ_BK);
    ++staged;
    advance(lt, lp, lks);
  }
  float fr[2][2][4], fi[2][2][4];
#pragma unroll
  for (int x = 0; x < 2; ++x)
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int z = 0; z < 4; ++z) { fr[x][y][z] = 0.f; fi[x][y][z] = 0.f; }
  for (int c = 0; any && ct <= a.S + 1; ++c) {
    const int buf = c % OZ_STAGES;
    // item c is complete when at most (staged - c - 1) later groups are pending
    if (staged - c - 1 >= 1) cp_async_wait_one(); else cp_async_wait_all();
    __syncthreads();
    if (lt <= a.S + 1) {   // the buffer of item c - 1 is free: stage item c + OZ_STAGES - 1
      stage(staged % OZ_STAGES, lp - 1, lt - lp - 1, lks * OZ_BK);
      ++staged;
      advance(lt, lp, lks);
    }
#pragma unroll
    for (int kk = 0; kk < OZ_BK; kk += 16) {
      unsigned af[2][4];
#pragma unroll
      for (int x = 0; x < 2; ++x) {
        // rows 32*wm + 16*x + (lane % 16), k columns kk + 8*(lane / 16)
        const __nv_bfloat16* pa = &sA[buf][(32 * wm + 16 * x + (lane & 15)) * OZ_LDS + kk + 8 * (lane >> 4)];
        ldmatrix_x4(af[x][0], af[x][1], af[x][2], af[x][3], pa);
      }
      unsigned br[2][2], bi[2][2];
#pragma unroll
      for (int y = 0; y < 2; ++y) {
        // columns 16*wn + 8*y + (lane % 8), k rows kk + 8*((lane / 8) % 2)
        const int rowb = 16 * wn + 8 * y + (lane & 7);
        const int kof = kk + 8 * ((lane >> 3) & 1);
        ldmatrix_x2(br[y][0], br[y][1], &sBr[buf][rowb * OZ_LDS + kof]);
        ldmatrix_x2(bi[y][0], bi[y][1], &sBi[buf][rowb * OZ_LDS + kof]);
      }
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
          mma_bf16(fr[x][y], af[x], br[y]);
          mma_bf16(fi[x][y], af[x], bi[y]);
        }
    }
    const int t_done = ct;
    advance(ct, cp, cks);
    if (ct != t_done) {
      // group t_done complete: fold its exact FP32 sums into the accumulators
      if constexpr (INT) {
        const long long step = 1ll << a.bits;
#pragma unroll
        for (int x = 0; x < 2; ++x)
#pragma unroll
          for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int z = 0; z < 4; ++z) {
              accr[x][y][z] = accr[x][y][z] * step + (long long)__float2int_rn(fr[x][y][z]);
              acci[x][y][z] = acci[x][y][z] * step + (long long)__float2int_rn(fi[x][y][z]);
            }
      } else {
        const double wgt = ldexp(1.0, -a.bits * t_done);
#pragma unroll
        for (int x = 0; x < 2; ++x)
#pragma unroll
          for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int z = 0; z < 4; ++z) {
              accr[x][y][z] = fma(wgt, (double)fr[x][y][z], accr[x][y][z]);
              acci[x][y][z] = fma(wgt, (double)fi[x][y][z], acci[x][y][z]);
            }
      }
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
          for (int z = 0; z < 4; ++z) { fr[x][y][z] = 0.f; fi[x][y][z] = 0.f; }
    }
  }
  __syncthreads();
  // integer form: value = acc * 2^{-bits (S + 1)}
  const double wint = INT ? ldexp(1.0, -a.bits * (a.S + 1)) : 1.0;
  const bool plain = oz_plain(a);
  // epilogue: mma C fragment layout (m16n8): value z of lane -> row (lane/4) + 8*(z/2), col 2*(lane%4) + (z%2)
#pragma unroll
  for (int x = 0; x < 2; ++x)
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int z = 0; z < 4; ++z) {
        const int row = i0 + 32 * wm + 16 * x + (lane >> 2) + 8 * (z >> 1);
        const int col = j0 + 16 * wn + 8 * y + 2 * (lane & 3) + (z & 1);
        if (row < a.m && col < a.n) {
          if constexpr (INT) {
            if (a.acc) {
              // split K: integer partial sums add exactly (and in any order)
              unsigned long long* q = a.acc + 2 * ((size_t)col * a.m + row);
              atomicAdd(q, (unsigned long long)accr[x][y][z]);
              atomicAdd(q + 1, (unsigned long long)acci[x][y][z]);
            } else {
              oz_store(a, row, col, __ll2double_rn(accr[x][y][z]), __ll2double_rn(acci[x][y][z]), wint, plain);
            }
          } else {
            oz_store(a, row, col, accr[x][y][z], acci[x][y][z], wint, plain);
          }
        }
      }
}

__global__ void k_oz_finalize(OzArgs a) {
  const double wint = ldexp(1.0, -a.bits * (a.S + 1));
  const bool plain = oz_plain(a);
  const size_t total = (size_t)a.m * a.n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int col = (int)(e / a.m), row = (int)(e - (size_t)col * a.m);
    const long long vr = (long long)a.acc[2 * e], vi = (long long)a.acc[2 * e + 1];
    a.acc[2 * e] = 0ull;
    a.acc[2 * e + 1] = 0ull;
    oz_store(a, row, col, __ll2double_rn(vr), __ll2double_rn(vi), wint, plain);
  }
}

}  // namespace

// Slice count S and width `bits` for a product with inner dimension K and a
// target of `target_bits` mantissa bits: the smallest S whose widest exact
// width bits = floor((24 - log2(K' S)) / 2) (at most 8, the BF16 integer range)
// reaches the target.  Returns false when no S <= 12 does.
bool ozaki_plan(int K, int target_bits, int* S_out, int* bits_out) {
  const double kp = 2.0 * ((K + 15) / 16 * 16);
  for (int S = 2; S <= 12; ++S) {
    int bits = (int)std::floor((24.0 - std::log2(kp * S)) / 2.0);
    if (bits > 8) bits = 8;
    if (bits < 1) return false;
    if (S * bits >= target_bits) {
      *S_out = S;
      *bits_out = bits;
      return true;
    }
  }
  return false;
}

// Scratch: As S*m*Kp, Bre/Bim S*n*Kp bf16, scales m + n doubles.
size_t ozaki_scratch_bytes(int m, int n, int K, int S) {
  const size_t Kpad = ((size_t)K + 15) / 16 * 16;
  const size_t Kp = 2 * Kpad;
  return (size_t)S * Kp * ((size_t)m + 2 * (size_t)n) * sizeof(__nv_bfloat16) + ((size_t)m + n) * sizeof(double) + 256;
}

cudaError_t launch_ozaki_zgemm(int m, int nn, int k, char opA, char opB, cplx alpha, const cplx* A, int lda,
                               const cplx* B, int ldb, cplx beta, cplx* C, int ldc, const double* rowscale,
                               const double* colscale, int S, int bits, void* scratch, size_t scratch_bytes,
                               unsigned long long* acc, size_t acc_bytes, cudaStream_t st, const int* active,
                               int splitk, int* kernels) {
  if (S < 1 || S > 12 || bits < 1 || bits > 8) return cudaErrorInvalidValue;
  const int Kpad = (k + 15) / 16 * 16;
  const size_t Kp = 2 * (size_t)Kpad;
  // exactness of the FP32 group sums: Kp * S * 2^(2 bits) <= 2^24
  if ((double)Kp * S * ldexp(1.0, 2 * bits) > 16777216.0) return cudaErrorInvalidValue;
  if (ozaki_scratch_bytes(m, nn, k, S) > scratch_bytes) return cudaErrorInvalidValue;
  char* base = static_cast<char*>(scratch);
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(base);
  __nv_bfloat16* Bre = As + (size_t)S * m * Kp;
  __nv_bfloat16* Bim = Bre + (size_t)S * nn * Kp;
  double* sA = reinterpret_cast<double*>(Bim + (size_t)S * nn * Kp);
  double* sB = sA + m;
  k_oz_split_rows<<<m, 128, 0, st>>>(A, lda, opA, m, k, Kpad, S, bits, As, sA, active);
  k_oz_split_cols<<<nn, 128, 0, st>>>(B, ldb, opB, k, nn, Kpad, S, bits, Bre, Bim, sB, active);
  OzArgs a;
  a.As = As; a.Bre = Bre; a.Bim = Bim; a.sA = sA; a.sB = sB;
  a.m = m; a.n = nn; a.Kp = (int)Kp; a.S = S; a.bits = bits;
  a.alpha = alpha; a.beta = beta; a.C = C; a.ldc = ldc; a.rs = rowscale; a.cs = colscale; a.active = active;
  // |sum_t g_t 2^{bits (S+1-t)}| < 2^{24 + bits (S-1) + 1}: exact in int64 below 2^63
  a.int_combine = 24 + bits * (S - 1) <= 61 ? 1 : 0;
  a.kchunk = 0;
  a.acc = nullptr;
  dim3 grid((nn + OZ_BN - 1) / OZ_BN, (m + OZ_BM - 1) / OZ_BM);
  const int ksteps = (int)(Kp / OZ_BK);
  if (splitk > 1 && a.int_combine && !active && ksteps > 1 && acc &&
      (size_t)m * nn * 2 * sizeof(unsigned long long) <= acc_bytes) {
    // split K over blockIdx.z: exact 64-bit integer partial sums in acc, which
    // is zero between products (zeroed at allocation, re-zeroed by the finaliser)
    if (splitk > ksteps) splitk = ksteps;
    a.kchunk = (ksteps + splitk - 1) / splitk;
    grid.z = (ksteps + a.kchunk - 1) / a.kchunk;
    a.acc = acc;
  }
  if (kernels) *kernels = a.acc ? 4 : 3;
  if (a.int_combine) k_oz_gemm<true><<<grid, OZ_THREADS, 0, st>>>(a);
  else k_oz_gemm<false><<<grid, OZ_THREADS, 0, st>>>(a);
  if (a.acc) {
    const size_t total = (size_t)m * nn;
    const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    k_oz_finalize<<<blocks, 256, 0, st>>>(a);
  }
  return cudaGetLastError();
}
