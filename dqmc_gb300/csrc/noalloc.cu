// Local updates without any device allocation.
//
// Some hosts cannot let this library call cudaMalloc: a Julia or C++
// application that hands every byte of GPU memory to its own pool allocator
// (and tracks it there), a service that must run inside a fixed, pre-reserved
// memory budget, or code that runs while allocation is not permitted.  For
// such callers `dqmc_local_updates_noalloc` runs the local-update kernel of
// one time slice on buffers the caller already owns; the only scratch it
// needs (the rank-4 factors A and B of one accepted site, the grid barrier
// and an error flag) lives in the file-scope device array below, which every
// GPU that loads this library holds until the process exits.
#include <initializer_list>
#include <mutex>

#include "../../include/dqmc_gpu.h"
#include "common.cuh"
#include "kernels.h"

void fill_model_const(const dqmc_params& p, ModelConst& m);

namespace {

// Largest supported matrix dimension n = 4 L^2 (L <= 16).
constexpr int kNoAllocMaxN = 1024;
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
  cplx Acol[4 * kNoAllocMaxN];   // A = (G[:, cols] - I[:, cols]) M^-1
  cplx Brow[4 * kNoAllocMaxN];   // B = Delta G[rows, :]
  GridBarrier bar;               // must be zero when a launch starts
  int err;                       // device error bits, cleared per call
  int n_acc;                     // accepted-count accumulator, cleared per call
};

// 128 KB + 16 bytes, shared by every call on a device.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Host side: the device address of g_noalloc_scratch and the SM count, looked
// up once per device (the host-side name of the array is only a stand-in,
// never a device address).  The cached address belongs to the device's
// primary context: the library must not be used across a cudaDeviceReset.
std::mutex g_setup_mu;
NoAllocScratch* g_scratch_dev[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};

int setup_device(int dev, NoAllocScratch** scratch, int* sms) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_dev[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return DQMC_ERR_CUDA;
    int count = 0;
    if (cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DQMC_ERR_CUDA;
    g_sm_count[dev] = count;
    g_scratch_dev[dev] = static_cast<NoAllocScratch*>(ptr);
  }
  *scratch = g_scratch_dev[dev];
  *sms = g_sm_count[dev];
  return DQMC_OK;
}

// Restores the calling thread's current device on every return path: the
// device selection belongs to the host application.
struct DeviceRestore {
  int saved = -1;
  DeviceRestore() {
    if (cudaGetDevice(&saved) != cudaSuccess) saved = -1;
  }
  ~DeviceRestore() {
    if (saved >= 0) cudaSetDevice(saved);
  }
};

int run(const dqmc_params* p, double* greens, double* phi, int32_t slice, const double* delta,
        const double* unif, uint8_t* accepted, double* action, void* stream) {
  if (!p || !greens || !phi || !delta || !unif || !action) return DQMC_ERR_ARG;
  if (p->L < 2 || p->L % 2 != 0 || p->opdim != 3 || p->slices < 1) return DQMC_ERR_ARG;
  if (slice < 1 || slice > p->slices) return DQMC_ERR_ARG;
  if (4 * p->L * p->L > kNoAllocMaxN) return DQMC_ERR_TOO_LARGE;
  if (p->device >= 0 && cudaSetDevice(p->device) != cudaSuccess) return DQMC_ERR_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DQMC_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (st) {
    // a stream of another device would only fail later, as a launch error
    int sdev = -1;
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess) {
      cudaGetLastError();
      return DQMC_ERR_ARG;
    }
    if (sdev != dev) return DQMC_ERR_ARG;
  }
  // the call waits for its own result (a stream synchronisation), which a
  // capturing stream does not allow
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();
    return DQMC_ERR_ARG;
  }
  if (cap != cudaStreamCaptureStatusNone) return DQMC_ERR_ARG;
  // every array is dereferenced by the kernel: a host or foreign pointer is
  // an argument error here, never a memory fault on the GPU
  for (const void* q : {(const void*)greens, (const void*)phi, (const void*)delta, (const void*)unif,
                        (const void*)accepted, (const void*)action})
    if (!device_accessible(q)) return DQMC_ERR_ARG;
  NoAllocScratch* s = nullptr;
  int sms = 0;
  int rc = setup_device(dev, &s, &sms);
  if (rc != DQMC_OK) return rc;
  // the barrier, the error flag and the counter must start at zero; the
  // factor buffers are fully written before they are read
  if (cudaMemsetAsync(&s->bar, 0, sizeof(GridBarrier) + 2 * sizeof(int), st) != cudaSuccess) return DQMC_ERR_CUDA;
  LocalUpdateArgs a{};
  a.G = reinterpret_cast<cplx*>(greens);
  a.phi = phi;
  a.evtab = nullptr;
  a.slice0 = slice - 1;
  a.delta = delta;
  a.unif = unif;
  a.acc_out = accepted;
  a.det_out = nullptr;
  a.pacc_out = nullptr;
  a.action = action;
  a.n_acc = &s->n_acc;
  a.Acol = s->Acol;
  a.Brow = s->Brow;
  a.bar = &s->bar;
  a.err = &s->err;
  fill_model_const(*p, a.mc);
  if (launch_local_updates(a, sms, st) != cudaSuccess) return DQMC_ERR_CUDA;
  int err = 0;
  if (cudaMemcpyAsync(&err, &s->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return DQMC_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return DQMC_ERR_CUDA;
  if (err & DQMC_KERR_BARRIER_TIMEOUT) return DQMC_ERR_TIMEOUT;
  if (err & DQMC_KERR_SINGULAR) return DQMC_ERR_SINGULAR;
  if (err & DQMC_KERR_NONFINITE) return DQMC_ERR_NONFINITE;
  return err ? DQMC_ERR_CUDA : DQMC_OK;
}

}  // namespace

extern "C" int dqmc_local_updates_noalloc(const dqmc_params* p, double* greens, double* phi, int32_t slice,
                                          const double* delta, const double* unif, uint8_t* accepted,
                                          double* action, void* stream) {
  DeviceRestore keep;
  return run(p, greens, phi, slice, delta, unif, accepted, action, stream);
}
