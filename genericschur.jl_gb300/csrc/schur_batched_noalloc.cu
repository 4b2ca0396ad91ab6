// Allocation-free entry point of the batched real Schur decomposition.
//
// Some callers cannot allocate device memory at the point where they want the
// decomposition: code running inside an externally managed memory pool or arena
// (a framework allocator that forbids raw cudaMalloc), plugins of a host program
// that owns all device memory, and sequences being recorded for later replay
// where an allocation would be a side effect outside the recorded work.  This
// entry point serves them: the caller passes only device buffers for inputs and
// outputs and a stream, and the work-queue scratch the kernels need (the sorted
// matrix order and the per-bin ticket counters) lives in a file-scope device array
// of fixed size instead of the context's workspace.
//
// Cost of that choice: every GPU that loads this library holds the array
// (GS_NOALLOC_MAX_BATCH ints plus the counters, about 256 KiB) until the process
// exits; calls share it, so two calls whose work overlaps on the GPU (different
// streams, or the same stream from different host threads without ordering) race
// on it.  The bin-sort kernel rewrites the order and zeroes the counters at the
// start of every call, so nothing from a previous call leaks into the next.
#include <mutex>

#include "../../include/gschur_gb300_noalloc.h"
#include "gs_internal.h"

namespace gsk {
namespace {

// order[GS_NOALLOC_MAX_BATCH] followed by the 3 * kNumBins scheduling words.
static __device__ __align__(256) int g_noalloc_scratch[GS_NOALLOC_MAX_BATCH + 3 * kNumBins];

struct DeviceSetup {
  int* scratch = nullptr;  // device address of g_noalloc_scratch on that device
  int num_sms = 0;
  bool ready = false;
};

constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

// Once per device, with that device current: resolve the array's device address
// (the host-side symbol is only a stand-in and must never reach a kernel) and the
// SM count.  Returns a CUDA error code.
cudaError_t device_setup(int dev, DeviceSetup** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup& s = g_setup[dev];
  if (!s.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    s.scratch = (int*)p;
    s.num_sms = sms;
    s.ready = true;
  }
  *out = &s;
  return cudaSuccess;
}

}  // namespace
}  // namespace gsk

extern "C" int gs_schur_batched_f64_noalloc(void* stream, int64_t count, const int32_t* ns, const int64_t* offs,
                                            const int64_t* woffs, double* A, double* Z, double* wr, double* wi,
                                            int32_t* status, unsigned flags) {
  using namespace gsk;
  if (count < 0 || count > GS_NOALLOC_MAX_BATCH) return GS_BADARG;  // beyond the static scratch
  if (count == 0) return GS_OK;
  const bool wantz = flags & GS_WANTZ;
  if (!ns || !offs || !woffs || !A || !wr || !wi || !status || (wantz && !Z)) return GS_BADARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GS_CUDA;
  DeviceSetup* su = nullptr;
  if (device_setup(dev, &su) != cudaSuccess) return GS_CUDA;
  RealBatch bt{};
  bt.count = (int)count;
  bt.ns = ns;
  bt.offs = (const long long*)offs;
  bt.woffs = (const long long*)woffs;
  bt.A = A;
  bt.Z = wantz ? Z : nullptr;
  bt.wr = wr;
  bt.wi = wi;
  bt.status = status;
  bt.wantz = wantz;
  bt.scale = (flags & GS_SCALE) ? 1 : 0;
  bt.maxiter_mult = 100;
  int* order = su->scratch;
  int* sched = su->scratch + GS_NOALLOC_MAX_BATCH;
  cudaStream_t s = (cudaStream_t)stream;
  if (launch_bin_sort(ns, (int)count, order, sched, s) != cudaSuccess) return GS_CUDA;
  // all size bins on the caller's stream, one after another
  if (launch_schur_batched_real(bt, order, sched, su->num_sms, &s, 1) != cudaSuccess) return GS_CUDA;
  return GS_OK;
}
