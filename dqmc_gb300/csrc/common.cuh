// Shared device helpers for the DQMC sweep kernels (sm_103a).
//
// Complex numbers are stored as double2 {re, im}, layout-compatible with
// Julia's ComplexF64 and C's double _Complex.  Every matrix is column-major
// with leading dimension n (element (r, c) at c*n + r), exactly the layout
// of the reference's `Matrix{ComplexF64}`.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>

#define DQMC_HD __host__ __device__ __forceinline__

typedef double2 cplx;

DQMC_HD cplx cmake(double r, double i) { return make_double2(r, i); }
DQMC_HD cplx cadd(cplx a, cplx b) { return cmake(a.x + b.x, a.y + b.y); }
DQMC_HD cplx csub(cplx a, cplx b) { return cmake(a.x - b.x, a.y - b.y); }
DQMC_HD cplx cmul(cplx a, cplx b) { return cmake(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
DQMC_HD cplx cconj(cplx a) { return cmake(a.x, -a.y); }
DQMC_HD cplx cscale(cplx a, double s) { return cmake(a.x * s, a.y * s); }
// acc + a*b
DQMC_HD cplx cfma(cplx a, cplx b, cplx acc) {
  return cmake(fma(a.x, b.x, fma(-a.y, b.y, acc.x)), fma(a.x, b.y, fma(a.y, b.x, acc.y)));
}
// acc + conj(a)*b
DQMC_HD cplx cfma_conj(cplx a, cplx b, cplx acc) {
  return cmake(fma(a.x, b.x, fma(a.y, b.y, acc.x)), fma(a.x, b.y, fma(-a.y, b.x, acc.y)));
}
DQMC_HD double cabs2(cplx a) { return a.x * a.x + a.y * a.y; }
DQMC_HD cplx cdiv(cplx a, cplx b) {
  // Smith's algorithm (robust complex division)
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return cmake((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    double r = b.x / b.y, d = b.x * r + b.y;
    return cmake((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}

// Model constants needed on the device.  Filled once per handle.
struct ModelConst {
  int L, N, n, M;
  double dtau, lambda, r, c, u;
  double mu[2];          // band x, band y
  // hyperbolic rotation factors of the plaquette layers, per band b (0 = x, 1 = y):
  //   full step (prefactor 1):  ch_f[b] (horizontal), sh_f[b]; cv_f[b] (vertical), sv_f[b]
  //   half step (prefactor 1/2): ch_h, sh_h, cv_h, sv_h
  double ch_f[2], sh_f[2], cv_f[2], sv_f[2];
  double ch_h[2], sh_h[2], cv_h[2], sv_h[2];
  double emu[2], emu_inv[2];  // exp(dtau*mu), exp(-dtau*mu) per band
};

// Per-site interaction entries of one slice: (C, Re S, Im S, R) for power +1
// (src/interactions.jl:52-64).  Power -1 flips the sign of S and R.
struct EvEntry { double C, Sr, Si, R; };

// Cross-CTA barrier for cooperative (co-resident) grids, with a bounded spin.
// On timeout it sets *err (bit 1) and returns false: the kernel must then
// leave its loop and return; it never hangs the device.  count holds the
// arrivals of the launch, exits the CTAs that have left it; both start at
// zero (zeroed at allocation) and the last CTA to leave zeroes them again
// for the next launch on the stream (GridBarrierExit), so the launcher
// needs no memset node per launch.
struct GridBarrier {
  unsigned int count;
  unsigned int exits;
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// count is zeroed before every launch that uses the barrier; the e-th
// barrier of the launch completes when all CTAs have added their arrival,
// i.e. when count reaches e * gridDim.x (no returning atomic, no reset).
__device__ __forceinline__ bool grid_barrier(GridBarrier* b, int* err, unsigned& epoch) {
  __syncthreads();
  __shared__ int s_ok;
  ++epoch;
  if (threadIdx.x == 0) {
    const unsigned target = epoch * gridDim.x;
    __threadfence();
    atomicAdd(&b->count, 1u);
    int ok = 1;
    long long spins = 0;
    while (ld_acquire_u32(&b->count) < target) {
      if ((++spins & 1023) == 0) {
        if (spins > (1ll << 26)) { atomicOr(err, 2); ok = 0; break; }
        if (*(volatile int*)err & 2) { ok = 0; break; }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Declared at the top of a kernel that uses grid_barrier: its destructor runs
// on every return path, after the CTA's last barrier; the last CTA out (all
// others have stopped polling by then) zeroes the barrier.
struct GridBarrierExit {
  GridBarrier* b;
  __device__ __forceinline__ explicit GridBarrierExit(GridBarrier* bar) : b(bar) {}
  __device__ __forceinline__ ~GridBarrierExit() {
    if (threadIdx.x == 0) {
      __threadfence();
      if (atomicAdd(&b->exits, 1u) == gridDim.x - 1) {
        b->count = 0;
        b->exits = 0;
        __threadfence();
      }
    }
  }
};

// Raises a kernel's dynamic shared-memory limit (cudaFuncSetAttribute) once
// per device: the attribute belongs to the device's context, so a process
// driving several GPUs sets it on each.  One static instance per kernel
// launcher; thread-safe.
class SmemLimit {
 public:
  cudaError_t raise(const void* fn, int bytes) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu_);
    if (set_[dev] >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) set_[dev] = bytes;
    return e;
  }

 private:
  static constexpr int kMaxDevices = 64;
  std::mutex mu_;
  int set_[kMaxDevices] = {};
};

// Host-side check of an address a kernel will dereference: device or managed
// memory, or registered host memory mapped at the same address (NULL passes;
// callers check it).  A pageable host array passed as a device address would
// otherwise make the kernel fault.  Allocates nothing.
inline bool device_accessible(const void* p) {
  if (!p) return true;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged ||
         (at.type == cudaMemoryTypeHost && at.devicePointer == p);
}

// Error bits reported by kernels through a device int.
enum {
  DQMC_KERR_BARRIER_TIMEOUT = 2,
  DQMC_KERR_NONFINITE = 4,
  DQMC_KERR_SINGULAR = 8,
  DQMC_KERR_BAD_SHAPE = 16,
};

__device__ __forceinline__ cplx ldcg_c(const cplx* p) { return __ldcg(p); }
