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
//    an integer below 2^24, so the FP32 accumulation is exact; the group sums
//    are combined exactly in 64-bit integers (Horner in 2^B_BITS) and the
//    result converted once with its power-of-two weight and the scales.
// The only error is the truncation of the slice expansion (~2^{-B_BITS S}
// relative to sigma_i tau_j K).
//
// The tensor-core products run on tcgen05.mma (kind::f16, BF16 in, FP32
// accumulators in tensor memory), with every operand tile staged by TMA
// (cp.async.bulk.tensor) onto mbarriers; see the engine section below.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>
#include "common.cuh"
#include "kernels.h"
#include "oz_slice.cuh"

namespace {

// ---------------------------------------------------------------------------
// split: slices of op(X) scaled per row ("row" side = A) or per column (B side)
// ---------------------------------------------------------------------------
// element (r, c) of op(X) where X is column-major with leading dimension ld
__device__ __forceinline__ cplx op_elem(const cplx* X, int ld, int r, int c, char op) {
  if (op == 'N') return X[(size_t)c * ld + r];
  cplx v = X[(size_t)r * ld + c];
  return op == 'C' ? cconj(v) : v;
}

// (the digit helpers expo_field, fixed62 and next_digit are in oz_slice.cuh)
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

// Both sides in one launch when each operand vector is contiguous across
// vectors (op(A) = A 'N': element k of row i at A[k lda + i]; op(B) = B^T
// 'T': element k of column j at B[k ldb + j]) and Kpad <= 64, the shape of
// the delayed-update flush: 8 vectors x Kpad elements are loaded with
// coalesced reads into shared memory, then one warp per vector finds its
// scale and cuts its digits (the same digits as k_oz_split_rows/cols).
// blockIdx.y = 0: rows of A; 1: columns of B.
constexpr int OZ_TILED_KMAX = 64;
constexpr int OZ_TILED_V = 8;      // vectors per block: one warp each
__global__ void __launch_bounds__(256) k_oz_split_tiled(const cplx* __restrict__ A, int lda, int m,
                                                        const cplx* __restrict__ B, int ldb, int nn, int K, int Kpad,
                                                        int S, int bits, __nv_bfloat16* __restrict__ As,
                                                        __nv_bfloat16* __restrict__ Bre, __nv_bfloat16* __restrict__ Bim,
                                                        double* __restrict__ sA, double* __restrict__ sB,
                                                        const int* __restrict__ active) {
  __shared__ cplx tile[OZ_TILED_KMAX][OZ_TILED_V + 1];
  const int side = blockIdx.y;
  const cplx* X = side ? B : A;
  const int ld = side ? ldb : lda, cnt = side ? nn : m;
  const int v0 = blockIdx.x * OZ_TILED_V;
  if (v0 >= cnt) return;
  if (active) {   // only the first 4p inner indices are live (delayed-update flush)
    const int kk = 4 * *active;
    if (kk == 0) return;
    if (kk < K) K = kk;
  }
  for (int idx = threadIdx.x; idx < Kpad * OZ_TILED_V; idx += blockDim.x) {
    const int k = idx / OZ_TILED_V, v = idx % OZ_TILED_V;
    tile[k][v] = (k < K && v0 + v < cnt) ? X[(size_t)k * ld + v0 + v] : cmake(0.0, 0.0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const OzSlices o{As, Bre, Bim, sA, sB, m, nn, Kpad, S, bits};
  for (int v = wid; v < OZ_TILED_V; v += blockDim.x >> 5) {
    const int vec = v0 + v;
    if (vec >= cnt) break;
    oz_slice_vec(o, side, vec, K, [&](int k) { return tile[k][v]; }, lane);
  }
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

// alpha v + beta c_old for one output value (the scaled product v):
// alpha = +-1, beta in {0, 1} take one multiply and at most one add.
__device__ __forceinline__ cplx oz_combine(const OzArgs& a, cplx v, cplx c_old, bool plain) {
  if (plain) {
    if (a.alpha.x < 0.0) v = cmake(-v.x, -v.y);
    if (a.beta.x != 0.0) v = cadd(c_old, v);
    return v;
  }
  v = cmul(a.alpha, v);
  if (a.beta.x != 0.0 || a.beta.y != 0.0) v = cfma(a.beta, c_old, v);
  return v;
}

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

// ---------------------------------------------------------------------------
// tcgen05 engine: TMA-staged slices, tensor-core MMAs into TMEM accumulators
// ---------------------------------------------------------------------------
// A CTA computes 128 x 32 complex tiles of C, persistently: one CTA per SM
// takes tiles x, x + grid, ... and the MMAs of a tile run while the epilogue
// of the previous one converts and stores.  Each MMA is
// M = 128, N = 64, K = 16 (kind::f16, BF16 in, FP32 out): its B operand
// stacks the 32 columns of B'_re over the 32 of B'_im, so one accumulator
// holds [Re | Im] of the tile.  Every group t = p + q (2 <= t <= S + 1) has
// its own accumulator of 64 TMEM columns, all S live at once (S <= 8: 512
// columns), so one pass over K serves every slice pair and each K block of
// every slice is staged once:
//   * warp 0 (one lane) streams, per K block of 64 of every tile, the S
//     B-slices (double-buffered) and the S A-slices (a ring of 6) with
//     cp.async.bulk.tensor (128-byte swizzle) onto mbarriers;
//   * warp 1 allocates TMEM, and one lane issues tcgen05.mma for every pair
//     (p, q) with p + q <= S + 1 into group p + q, releasing each A slot and
//     B buffer with tcgen05.commit and marking a tile's accumulators final
//     with a commit; before the first MMA of the next tile it waits until
//     the epilogue has read the accumulators out of TMEM;
//   * warps 2-9 (two per TMEM lane quarter, one half of the columns each)
//     read the S exact FP32 group sums of a tile with tcgen05.ld, release
//     TMEM, combine the sums exactly in 64-bit integers (Horner in 2^bits),
//     then scale and store as before.
// Every wait is bounded; on a timeout the kernel sets an error bit, drains
// what it issued (bounded) and frees its TMEM.
constexpr int TC_BM = 128;                      // rows of C per CTA (TMEM lanes)
constexpr int TC_BN = 32;                       // complex columns of C per CTA (MMA N = 64)
constexpr int TC_BK = 64;                       // BF16 per K block: one 128-byte swizzle row
constexpr int TC_MAXS = 8;                      // S groups x 64 TMEM columns <= 512
constexpr int TC_ARING = 6;                     // A-slice stages (S <= 6: one K block of A in flight)
constexpr int TC_EPI_WARPS = 8;                 // epilogue warps 2-9: two per TMEM lane quarter
constexpr int TC_THREADS = 32 * (2 + TC_EPI_WARPS);   // warp 0 TMA, warp 1 MMA (and TMEM allocation)
constexpr int TC_A_TILE = TC_BM * TC_BK * 2;    // 16 KB
constexpr int TC_B_HALF = TC_BN * TC_BK * 2;    // 4 KB: 32 rows of B'_re or of B'_im
constexpr int TC_B_TILE = 2 * TC_B_HALF;        // 8 KB
// MMA instruction descriptor (kind::f16): D F32 (bits 4-5 = 1), A BF16 (bits
// 7-9 = 1), B BF16 (bits 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(2 * TC_BN) >> 3 << 17) |
                              ((uint32_t)TC_BM >> 4 << 24);

__host__ __device__ constexpr size_t tc_smem_bytes(int S) {
  return 1024 + (size_t)2 * S * TC_B_TILE + (size_t)TC_ARING * TC_A_TILE + 256;
}
__host__ __device__ constexpr uint32_t tc_tmem_cols(int S) {
  return S <= 2 ? 128u : (S <= 4 ? 256u : 512u);
}

// Shared-memory matrix descriptor of a K-major operand tile written by TMA
// with the 128-byte swizzle: start address >> 4 (bits 0-13), leading byte
// offset 16 >> 4 (bits 16-29; unused for this layout), stride byte offset
// 1024 >> 4 between 8-row groups (bits 32-45), descriptor version 1 (bits
// 46-47), layout SWIZZLE_128B = 2 (bits 61-63).  Tiles start on 1024-byte
// boundaries; the K step of 16 BF16 (32 bytes) inside the swizzle row adds
// 2 to the start field.
__device__ __forceinline__ uint64_t tc_desc(uint32_t smem_addr) {
  return (uint64_t)((smem_addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// Waits until the phase of parity `parity` of the barrier has completed; gives
// up after ~2^31 SM cycles (about a second), sets the error bit and *abort.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, volatile int* abort) {
  const long long t0 = clock64();
  for (uint32_t it = 0;; ++it) {
    if (mbar_test(bar, parity)) return true;
    if ((it & 255) == 255) {
      if (*abort) return false;
      if (clock64() - t0 > (1ll << 31)) {
        atomicOr(err, DQMC_KERR_BARRIER_TIMEOUT);
        *abort = 1;
        return false;
      }
    }
  }
}
// Bounded wait used on the abort path only (about 0.1 s, no error reporting).
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_test(bar, parity) && clock64() - t0 < (1ll << 28)) {}
}
// 3-D tiled TMA load (x = K element, y = row, z = slice) into shared memory,
// completing `bytes` of the barrier's transaction count.
__device__ __forceinline__ void tma_load3(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y), "r"(z)
      : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(accumulate)
      : "memory");
}
// arrives on the barrier once every tcgen05.mma issued so far by this thread has completed
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
// 32 TMEM lanes (this warp's quarter) x 16 consecutive 32-bit columns; the
// registers are valid after tc_wait_ld
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// (double)v 2^e, rounded to nearest even exactly as __ll2double_rn(v) * 2^e,
// on the integer units and without branches, for -1022 <= e <= 960 (every
// |v| < 2^63 then gives a normal double): |v| is shifted so that its leading
// one sits at bit 63, the 53 high bits are rounded to nearest even at bit 11,
// and a carry out of the significand steps the biased exponent by addition.
__device__ __forceinline__ double ll_ldexp(long long v, int e) {
  const unsigned long long sgn = (unsigned long long)v & 0x8000000000000000ull;
  const unsigned long long m = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  const int lz = __clzll((long long)m) & 63;   // 64 for m = 0, masked; the select below covers it
  const unsigned long long mn = m << lz;
  unsigned long long q = mn >> 11;
  const unsigned rem = (unsigned)mn & 0x7FFu;
  q += (rem + (unsigned)(q & 1ull)) > 0x400u ? 1ull : 0ull;
  const long long be = 63 - lz + e + 1023;
  const unsigned long long bits = sgn | ((unsigned long long)(be - 1) << 52) + q;
  return m ? __longlong_as_double((long long)bits) : 0.0;
}
// the exponent window in which ll_ldexp is exact for every 64-bit value
__device__ __forceinline__ bool ll_ldexp_safe(int e) { return e >= -1022 && e <= 960; }

struct TcMaps {
  CUtensorMap a, bre, bim;   // (Kp, rows, S) BF16 slices, box (64, 128 | 32, 1), 128-byte swizzle
};

template <bool INT>
__global__ void __launch_bounds__(TC_THREADS, 1) k_oz_gemm_tc(const __grid_constant__ TcMaps maps, OzArgs a,
                                                             int* err) {
  if (a.active && *a.active == 0) return;   // flush with nothing pending (uniform over the grid)
  extern __shared__ uint8_t tc_smem_raw[];
  const uint32_t raw = smem_u32(tc_smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* basep = tc_smem_raw + (base - raw);
  const int S = a.S;
  const uint32_t sB = base;                                     // [2][S] B tiles of 8 KB
  const uint32_t sA = base + 2u * S * TC_B_TILE;                // [TC_ARING] A tiles of 16 KB
  const uint32_t sBar = sA + TC_ARING * TC_A_TILE;              // barriers
  uint64_t* bars = reinterpret_cast<uint64_t*>(basep + (sBar - base));
  // barrier slots: full_b 0-1, empty_b 2-3, full_a FA.., empty_a EA.., a tile's
  // accumulators final ACC, TMEM drained by the epilogue TE, MMA thread done DONE
  constexpr int FA = 4, EA = FA + TC_ARING, ACC = EA + TC_ARING, TE = ACC + 1, DONE = TE + 1, NBAR = DONE + 1;
  auto bar = [&](int k) { return sBar + 8u * k; };
  volatile int* s_abort = reinterpret_cast<volatile int*>(bars + NBAR);
  uint32_t* s_tmem = reinterpret_cast<uint32_t*>(bars + NBAR + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // output tiles, taken persistently: CTA x handles tiles x, x + gridDim.x, ...
  // (tile t: row block t / tiles_x, column block t % tiles_x)
  const int tiles_x = (a.n + TC_BN - 1) / TC_BN;
  const int ntiles = tiles_x * ((a.m + TC_BM - 1) / TC_BM);
  const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const int nkb_all = (a.Kp + TC_BK - 1) / TC_BK;
  const int kb0 = a.kchunk ? (int)blockIdx.z * a.kchunk : 0;
  const int kb1 = a.kchunk ? min(nkb_all, kb0 + a.kchunk) : nkb_all;
  const int nkb = kb1 > kb0 ? kb1 - kb0 : 0;
  const int U = my_tiles * nkb;                                 // K blocks this CTA streams, all tiles
  auto tile_of = [&](int tt, int& i0, int& j0) {
    const int t = (int)blockIdx.x + tt * (int)gridDim.x;
    i0 = (t / tiles_x) * TC_BM;
    j0 = (t % tiles_x) * TC_BN;
  };
  const uint32_t ncols = tc_tmem_cols(S);

  if (threadIdx.x == 0) {
    for (int k = 0; k < 2; ++k) { mbar_init(bar(k), 1); mbar_init(bar(2 + k), 1); }
    for (int k = 0; k < TC_ARING; ++k) { mbar_init(bar(FA + k), 1); mbar_init(bar(EA + k), 1); }
    mbar_init(bar(ACC), 1);
    mbar_init(bar(TE), TC_EPI_WARPS);
    mbar_init(bar(DONE), 1);
    *s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *s_tmem;

  int armed[2 + TC_ARING] = {};   // producer: phases armed per full barrier (B 0-1, A from 2)
  if (warp == 0) {
    // ---- TMA producer: K block u = (tile u / nkb, kb0 + u % nkb) ----
    if (lane == 0 && U > 0) {
      int a_use = 0;
      int b_next = 0;   // next K block whose B slices are to be issued
      // the B slices of block u into buffer u & 1, once it is free;
      // block = false only tests whether it is free
      auto issue_b = [&](int u, bool block) -> bool {
        const int bb = u & 1;
        const uint32_t parity = ((u >> 1) & 1) ^ 1;
        if (block ? !mbar_wait(bar(2 + bb), parity, err, s_abort) : !mbar_test(bar(2 + bb), parity)) return false;
        armed[bb] = u + 1;
        int i0, j0;
        tile_of(u / nkb, i0, j0);
        const int kb = kb0 + u % nkb;
        mbar_expect_tx(bar(bb), (uint32_t)(S * TC_B_TILE));
        for (int q = 0; q < S; ++q) {
          const uint32_t dst = sB + (uint32_t)(bb * S + q) * TC_B_TILE;
          tma_load3(dst, &maps.bre, bar(bb), kb * TC_BK, j0, q);
          tma_load3(dst + TC_B_HALF, &maps.bim, bar(bb), kb * TC_BK, j0, q);
        }
        return true;
      };
      for (int u = 0; u < U && !*s_abort; ++u) {
        if (b_next == u) {
          if (!issue_b(u, true)) break;
          ++b_next;
        }
        int i0, j0;
        tile_of(u / nkb, i0, j0);
        const int kb = kb0 + u % nkb;
        for (int p = 0; p < S; ++p, ++a_use) {
          // the next block's B as early as its buffer is free (without waiting)
          if (b_next == u + 1 && u + 1 < U && issue_b(u + 1, false)) ++b_next;
          const int slot = a_use % TC_ARING;
          if (!mbar_wait(bar(EA + slot), ((a_use / TC_ARING) & 1) ^ 1, err, s_abort)) break;
          armed[2 + slot] = a_use / TC_ARING + 1;
          mbar_expect_tx(bar(FA + slot), (uint32_t)TC_A_TILE);
          tma_load3(sA + (uint32_t)slot * TC_A_TILE, &maps.a, bar(FA + slot), kb * TC_BK, i0, p);
        }
      }
    }
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0) {
      int a_use = 0;
      for (int u = 0; u < U && !*s_abort; ++u) {
        const int tt = u / nkb, kbi = u % nkb, bb = u & 1;
        if (kbi == 0 && tt > 0) {
          // the epilogue has read tile tt - 1's accumulators out of TMEM
          if (!mbar_wait(bar(TE), (tt - 1) & 1, err, s_abort)) break;
          tc_fence_after();
        }
        if (!mbar_wait(bar(bb), (u >> 1) & 1, err, s_abort)) break;
        tc_fence_after();
        bool ok = true;
        for (int p = 0; p < S; ++p, ++a_use) {
          const int slot = a_use % TC_ARING;
          if (!mbar_wait(bar(FA + slot), (a_use / TC_ARING) & 1, err, s_abort)) { ok = false; break; }
          tc_fence_after();
          const uint64_t ad = tc_desc(sA + (uint32_t)slot * TC_A_TILE);
          for (int q = 0; q + p < S; ++q) {
            // pair (p + 1, q + 1) belongs to group t = p + q + 2: accumulator columns (p + q) * 64
            const uint64_t bd = tc_desc(sB + (uint32_t)(bb * S + q) * TC_B_TILE);
            const uint32_t d = tmem + (uint32_t)(p + q) * (2 * TC_BN);
#pragma unroll
            for (int kk = 0; kk < TC_BK / 16; ++kk)
              tc_mma(d, ad + 2u * kk, bd + 2u * kk, (kbi == 0 && p == 0 && kk == 0) ? 0u : 1u);
          }
          tc_commit(bar(EA + slot));  // A slot free once these MMAs have read it
        }
        tc_commit(bar(2 + bb));       // B buffer free
        if (!ok) break;
        if (kbi == nkb - 1) tc_commit(bar(ACC));   // tile tt's accumulators final
      }
      tc_commit(bar(DONE));           // every MMA issued has completed (the abort path waits on it)
    }
  } else if (U > 0) {
    // ---- epilogue: warps 2-9, two per TMEM lane quarter (warp % 4); warp w
    //      takes the 16 columns of half (w - 2) / 4 of each tile ----
    const int quarter = warp & 3;
    const int h = (warp - 2) >> 2;
    const bool fast = INT && oz_plain(a) && !a.rs && !a.cs && !a.acc;
    const bool add = a.beta.x != 0.0;
    const uint32_t tq = tmem + ((uint32_t)(32 * quarter) << 16);
    const double wint = INT ? ldexp(1.0, -a.bits * (S + 1)) : 1.0;
    const bool plain = oz_plain(a);
    for (int tt = 0; tt < my_tiles; ++tt) {
      int i0, j0;
      tile_of(tt, i0, j0);
      const int row = i0 + 32 * quarter + lane;
      const bool waited = mbar_wait(bar(ACC), tt & 1, err, s_abort);
      // tcgen05.ld is warp-collective: the decision must be uniform over the warp
      const bool have = __all_sync(0xffffffffu, waited && !*s_abort);
      if (!have) break;
      tc_fence_after();
      {
        typedef typename std::conditional<INT, long long, double>::type acc_t;
        acc_t ar[16], ai[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) { ar[c] = 0; ai[c] = 0; }
#pragma unroll 1
        for (int g = 0; g < S; ++g) {
          uint32_t ur[16], ui[16];
          tc_ld16(tq + (uint32_t)(g * 2 * TC_BN + 16 * h), ur);
          tc_ld16(tq + (uint32_t)(g * 2 * TC_BN + TC_BN + 16 * h), ui);
          tc_wait_ld();
          float vr[16], vi[16];
#pragma unroll
          for (int c = 0; c < 16; ++c) { vr[c] = __uint_as_float(ur[c]); vi[c] = __uint_as_float(ui[c]); }
          if constexpr (INT) {
            const long long step = 1ll << a.bits;
#pragma unroll
            for (int c = 0; c < 16; ++c) {
              ar[c] = ar[c] * step + (long long)__float2int_rn(vr[c]);
              ai[c] = ai[c] * step + (long long)__float2int_rn(vi[c]);
            }
          } else {
            const double wgt = ldexp(1.0, -a.bits * (g + 2));
#pragma unroll
            for (int c = 0; c < 16; ++c) {
              ar[c] = fma(wgt, (double)vr[c], ar[c]);
              ai[c] = fma(wgt, (double)vi[c], ai[c]);
            }
          }
        }
        // this tile's accumulators are all in registers: TMEM may take the next tile
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(bar(TE));
        if (row < a.m) {
          if (INT && a.acc) {
#pragma unroll
            for (int c = 0; c < 16; ++c) {
              const int col = j0 + 16 * h + c;
              if (col < a.n) {
                unsigned long long* qa = a.acc + 2 * ((size_t)col * a.m + row);
                atomicAdd(qa, (unsigned long long)ar[c]);
                atomicAdd(qa + 1, (unsigned long long)ai[c]);
              }
            }
          } else if (fast) {
            // the scale sA sB 2^-bits(S+1) is a power of two: the value is the
            // exact integer converted with that exponent on the integer units
            // (GB300 issues FP64 at a small fraction of its integer rate); the
            // only FP64 operation left is the addition of the old C (beta = 1)
            const int e_row = expo_field(a.sA[row]) - 1023 - a.bits * (S + 1);
            const bool neg = a.alpha.x < 0.0;
            // two passes of 8 columns: the old C values of a pass are loaded
            // together while the next tile's MMAs run (the arrays are indexed
            // only by unrolled constants, so they stay in registers)
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
              cplx pre[8];
              int e_col[8];
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                const int col = j0 + 16 * h + 8 * hh + c;
                pre[c] = (add && col < a.n) ? a.C[(size_t)col * a.ldc + row] : cmake(0.0, 0.0);
                e_col[c] = col < a.n ? expo_field(a.sB[col]) - 1023 : 0;
              }
              bool safe = true;
#pragma unroll
              for (int c = 0; c < 8; ++c) safe = safe && ll_ldexp_safe(e_row + e_col[c]);
              if (safe) {
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                  const int col = j0 + 16 * h + 8 * hh + c;
                  if (col < a.n) {
                    const long long vr = neg ? -(long long)ar[8 * hh + c] : (long long)ar[8 * hh + c];
                    const long long vi = neg ? -(long long)ai[8 * hh + c] : (long long)ai[8 * hh + c];
                    cplx v = cmake(ll_ldexp(vr, e_row + e_col[c]), ll_ldexp(vi, e_row + e_col[c]));
                    if (add) v = cadd(pre[c], v);
                    a.C[(size_t)col * a.ldc + row] = v;
                  }
                }
              } else {
                // results that may leave the normal range: the FP64 route
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                  const int col = j0 + 16 * h + 8 * hh + c;
                  if (col < a.n) {
                    const long long vr = neg ? -(long long)ar[8 * hh + c] : (long long)ar[8 * hh + c];
                    const long long vi = neg ? -(long long)ai[8 * hh + c] : (long long)ai[8 * hh + c];
                    cplx v = cmake(ldexp(__ll2double_rn(vr), e_row + e_col[c]),
                                   ldexp(__ll2double_rn(vi), e_row + e_col[c]));
                    if (add) v = cadd(pre[c], v);
                    a.C[(size_t)col * a.ldc + row] = v;
                  }
                }
              }
            }
          } else {
            // per pass of 8 columns every load (scales, old C) is issued before
            // the first store, so they are in flight together
            double fr = a.sA[row] * wint;
            if (a.rs) fr *= a.rs[row];
            const bool rd = a.beta.x != 0.0 || a.beta.y != 0.0;
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
              double fc[8];
              cplx cold[8];
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                const int col = j0 + 16 * h + 8 * hh + c;
                fc[c] = 0.0;
                cold[c] = cmake(0.0, 0.0);
                if (col < a.n) {
                  fc[c] = a.sB[col];
                  if (a.cs) fc[c] *= a.cs[col];
                  if (rd) cold[c] = a.C[(size_t)col * a.ldc + row];
                }
              }
#pragma unroll
              for (int c = 0; c < 8; ++c) {
                const int col = j0 + 16 * h + 8 * hh + c;
                if (col < a.n) {
                  const double f = fr * fc[c];
                  double vr, vi;
                  if constexpr (INT) { vr = __ll2double_rn(ar[8 * hh + c]); vi = __ll2double_rn(ai[8 * hh + c]); }
                  else { vr = ar[8 * hh + c]; vi = ai[8 * hh + c]; }
                  a.C[(size_t)col * a.ldc + row] = oz_combine(a, cmake(vr * f, vi * f), cold[c], plain);
                }
              }
            }
          }
        }
      }
    }
  }
  // ---- teardown: on an abort, let issued copies and MMAs finish (bounded) ----
  __syncthreads();
  if (*s_abort) {
    if (threadIdx.x == 32) {
      mbar_drain(bar(DONE), 0);  // the MMA thread's final commit: every MMA it issued has completed
    } else if (threadIdx.x == 0) {
      for (int k = 0; k < 2; ++k)
        if (armed[k]) mbar_drain(bar(k), (armed[k] - 1) & 1);
      for (int k = 0; k < TC_ARING; ++k)
        if (armed[2 + k]) mbar_drain(bar(FA + k), (armed[2 + k] - 1) & 1);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
  }
}

}  // namespace

// Slice count S and width `bits` for a product with inner dimension K and a
// target of `target_bits` mantissa bits: the smallest S whose widest exact
// width bits = floor((24 - log2(K' S)) / 2) (at most 8, the BF16 integer range)
// reaches the target.  Returns false when no S <= 8 does (the product keeps one
// TMEM accumulator of 64 columns per group: 8 groups fill the 512 columns).
bool ozaki_plan(int K, int target_bits, int* S_out, int* bits_out) {
  const double kp = 2.0 * ((K + 15) / 16 * 16);
  for (int S = 2; S <= TC_MAXS; ++S) {
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

OzSlices ozaki_slices(void* scratch, int m, int n, int K, int S, int bits) {
  const int Kpad = (K + 15) / 16 * 16;
  const size_t Kp = 2 * (size_t)Kpad;
  OzSlices o;
  o.As = reinterpret_cast<__nv_bfloat16*>(scratch);
  o.Bre = o.As + (size_t)S * m * Kp;
  o.Bim = o.Bre + (size_t)S * n * Kp;
  o.sA = reinterpret_cast<double*>(o.Bim + (size_t)S * n * Kp);
  o.sB = o.sA + m;
  o.m = m; o.n = n; o.Kpad = Kpad; o.S = S; o.bits = bits;
  return o;
}

// Scratch: As S*m*Kp, Bre/Bim S*n*Kp bf16, scales m + n doubles.
size_t ozaki_scratch_bytes(int m, int n, int K, int S) {
  const size_t Kpad = ((size_t)K + 15) / 16 * 16;
  const size_t Kp = 2 * Kpad;
  return (size_t)S * Kp * ((size_t)m + 2 * (size_t)n) * sizeof(__nv_bfloat16) + ((size_t)m + n) * sizeof(double) + 256;
}

// cuTensorMapEncodeTiled from the driver, looked up once (no link against libcuda).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// SMs of the current device, looked up once per device.
static int sm_count_of_current_device() {
  static int cached[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (!cached[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) return 148;
    cached[dev] = v;
  }
  return cached[dev];
}

// BF16 slices (Kp, rows, S), K contiguous: box of 64 K elements (128 bytes,
// the swizzle span) x box_rows rows x 1 slice, 128-byte swizzle.
static bool encode_slices(CUtensorMap* map, const __nv_bfloat16* base, size_t Kp, int rows, int S, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)S};
  cuuint64_t strides[2] = {(cuuint64_t)(Kp * 2), (cuuint64_t)(Kp * 2 * rows)};
  cuuint32_t box[3] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t launch_ozaki_zgemm(int m, int nn, int k, char opA, char opB, cplx alpha, const cplx* A, int lda,
                               const cplx* B, int ldb, cplx beta, cplx* C, int ldc, const double* rowscale,
                               const double* colscale, int S, int bits, void* scratch, size_t scratch_bytes,
                               unsigned long long* acc, size_t acc_bytes, cudaStream_t st, const int* active,
                               int splitk, int* kernels, int* err, bool persistent, bool presliced) {
  if (S < 1 || S > TC_MAXS || bits < 1 || bits > 8) return cudaErrorInvalidValue;
  const int Kpad = (k + 15) / 16 * 16;
  const size_t Kp = 2 * (size_t)Kpad;
  // exactness of the FP32 group sums: Kp * S * 2^(2 bits) <= 2^24
  if ((double)Kp * S * ldexp(1.0, 2 * bits) > 16777216.0) return cudaErrorInvalidValue;
  if (ozaki_scratch_bytes(m, nn, k, S) > scratch_bytes) return cudaErrorInvalidValue;
  const OzSlices sl = ozaki_slices(scratch, m, nn, k, S, bits);
  __nv_bfloat16 *As = sl.As, *Bre = sl.Bre, *Bim = sl.Bim;
  double *sA = sl.sA, *sB = sl.sB;
  const bool tiled = opA == 'N' && opB == 'T' && Kpad <= OZ_TILED_KMAX;
  if (presliced) {
    // the slices are already in scratch (cut by the delayed local-update kernel)
  } else if (tiled) {
    const int vecs = m > nn ? m : nn;
    k_oz_split_tiled<<<dim3((vecs + OZ_TILED_V - 1) / OZ_TILED_V, 2), 32 * OZ_TILED_V, 0, st>>>(A, lda, m, B, ldb, nn, k, Kpad, S, bits, As, Bre, Bim,
                                                               sA, sB, active);
  } else {
    k_oz_split_rows<<<m, 128, 0, st>>>(A, lda, opA, m, k, Kpad, S, bits, As, sA, active);
    k_oz_split_cols<<<nn, 128, 0, st>>>(B, ldb, opB, k, nn, Kpad, S, bits, Bre, Bim, sB, active);
  }
  OzArgs a;
  a.As = As; a.Bre = Bre; a.Bim = Bim; a.sA = sA; a.sB = sB;
  a.m = m; a.n = nn; a.Kp = (int)Kp; a.S = S; a.bits = bits;
  a.alpha = alpha; a.beta = beta; a.C = C; a.ldc = ldc; a.rs = rowscale; a.cs = colscale; a.active = active;
  // |sum_t g_t 2^{bits (S+1-t)}| < 2^{24 + bits (S-1) + 1}: exact in int64 below 2^63
  a.int_combine = 24 + bits * (S - 1) <= 61 ? 1 : 0;
  a.kchunk = 0;
  a.acc = nullptr;
  if (S > TC_MAXS || !err) return cudaErrorInvalidValue;
  // persistent CTAs: one per SM (each holds the whole TMEM), every CTA takes
  // tiles x, x + grid, ... and overlaps a tile's epilogue with the next tile's
  // MMAs; otherwise one CTA per tile (chains sharing the GPU: short CTAs let
  // the other chains' kernels in between)
  const int ntiles = ((nn + TC_BN - 1) / TC_BN) * ((m + TC_BM - 1) / TC_BM);
  const int sms = sm_count_of_current_device();
  dim3 grid(persistent && ntiles > sms ? sms : ntiles);
  const int ksteps = (int)((Kp + TC_BK - 1) / TC_BK);
  if (splitk > 1 && a.int_combine && !active && ksteps > 1 && acc &&
      (size_t)m * nn * 2 * sizeof(unsigned long long) <= acc_bytes) {
    // split K over blockIdx.z: exact 64-bit integer partial sums in acc, which
    // is zero between products (zeroed at allocation, re-zeroed by the finaliser)
    if (splitk > ksteps) splitk = ksteps;
    a.kchunk = (ksteps + splitk - 1) / splitk;
    grid.z = (ksteps + a.kchunk - 1) / a.kchunk;
    a.acc = acc;
  }
  if (kernels) *kernels = (a.acc ? 4 : 3) - (presliced ? 2 : tiled ? 1 : 0);
  {
    TcMaps maps;
    if (!encode_slices(&maps.a, As, Kp, m, S, TC_BM) || !encode_slices(&maps.bre, Bre, Kp, nn, S, TC_BN) ||
        !encode_slices(&maps.bim, Bim, Kp, nn, S, TC_BN))
      return cudaErrorInvalidValue;
    static SmemLimit limit_int, limit_fp;
    const size_t smem = tc_smem_bytes(S);
    if (a.int_combine) {
      if (cudaError_t e = limit_int.raise((const void*)k_oz_gemm_tc<true>, (int)tc_smem_bytes(TC_MAXS));
          e != cudaSuccess)
        return e;
      k_oz_gemm_tc<true><<<grid, TC_THREADS, smem, st>>>(maps, a, err);
    } else {
      if (cudaError_t e = limit_fp.raise((const void*)k_oz_gemm_tc<false>, (int)tc_smem_bytes(TC_MAXS));
          e != cudaSuccess)
        return e;
      k_oz_gemm_tc<false><<<grid, TC_THREADS, smem, st>>>(maps, a, err);
    }
  }
  if (a.acc) {
    const size_t total = (size_t)m * nn;
    const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    k_oz_finalize<<<blocks, 256, 0, st>>>(a);
  }
  return cudaGetLastError();
}
