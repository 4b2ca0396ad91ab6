// Work-queue construction for the persistent batched kernels: a counting sort of
// the matrices by order, largest first, split into the size bins (bounds: the largest
// order of each bin, ascending).
// Runs on the device so that the whole batched pipeline is graph-capturable and
// needs no host round trip to read the orders.  Orders outside [0, kSmallMax] (possible
// when the orders live in device memory and were never checked on the host) are counted
// in the nearest end bin; the solve kernels see the true order there and write ST_BADARG
// for it without touching the matrix.
#include <algorithm>

#include "gs_internal.h"

namespace gsk {
namespace {

__global__ void __launch_bounds__(1024) k_bin_sort(const int* __restrict__ ns, int count,
                                                   int* __restrict__ order, int* __restrict__ sched,
                                                   BinBounds bounds, const int* status, int code) {
  __shared__ int hist[kSmallMax + 1];
  __shared__ int pos[kSmallMax + 1];
  for (int i = threadIdx.x; i <= kSmallMax; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (int b = threadIdx.x; b < count; b += blockDim.x) {
    if (status && status[b] != code) continue;
    int n = ns[b];
    n = n < 0 ? 0 : (n > kSmallMax ? kSmallMax : n);
    atomicAdd(&hist[n], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    int bin = kNumBins - 1;
    sched[3 * bin] = 0;
    for (int n = kSmallMax; n >= 0; --n) {
      while (bin > 0 && n <= bounds.b[bin - 1]) {
        sched[3 * bin + 1] = run;
        --bin;
        sched[3 * bin] = run;
      }
      pos[n] = run;
      run += hist[n];
    }
    sched[3 * bin + 1] = run;
    while (bin > 0) {  // empty low bins
      --bin;
      sched[3 * bin] = run;
      sched[3 * bin + 1] = run;
    }
    for (int i = 0; i < kNumBins; ++i) sched[3 * i + 2] = 0;
  }
  __syncthreads();
  for (int b = threadIdx.x; b < count; b += blockDim.x) {
    if (status && status[b] != code) continue;
    int n = ns[b];
    n = n < 0 ? 0 : (n > kSmallMax ? kSmallMax : n);
    order[atomicAdd(&pos[n], 1)] = b;
  }
}

__global__ void k_batch_extent(const int* __restrict__ ns, const long long* __restrict__ offs,
                               const long long* __restrict__ woffs, int count, unsigned long long* out) {
  unsigned long long ea = 0, ew = 0;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < count; b += gridDim.x * blockDim.x) {
    int n = ns[b];
    n = n < 0 ? 0 : (n > kSmallMax ? kSmallMax : n);
    const long long a = offs[b] + (long long)n * n, w = woffs[b] + n;
    ea = a > (long long)ea ? (unsigned long long)a : ea;
    ew = w > (long long)ew ? (unsigned long long)w : ew;
  }
  atomicMax(out, ea);
  atomicMax(out + 1, ew);
}

// The queue of a single matrix: order[0] = 0, bin `bin` holds [0, 1), the other bins are
// empty, all ticket counters zero.  meta (when not null) receives iota[0..kSmallMax] in its
// first ints and zeros after, so that ns = meta + m, offs = woffs = (long long*) zeros.
__global__ void k_single_queue(int* order, int* sched, int bin) {
  const int t = threadIdx.x;
  if (t == 0) order[0] = 0;
  if (t < kNumBins) {
    sched[3 * t] = 0;
    sched[3 * t + 1] = (t == bin) ? 1 : 0;
    sched[3 * t + 2] = 0;
  }
}

__global__ void k_single_meta(int* iota, long long* zeros) {
  for (int t = threadIdx.x; t <= kSmallMax; t += blockDim.x) iota[t] = t;
  if (threadIdx.x < 2) zeros[threadIdx.x] = 0;
}

}  // namespace

int default_bin_of(int m) {
  for (int b = 0; b < kNumBins; ++b)
    if (m <= bin_max(b)) return b;
  return kNumBins - 1;
}

cudaError_t launch_single_queue(int bin, int* order, int* sched, cudaStream_t s) {
  k_single_queue<<<1, 32, 0, s>>>(order, sched, bin);
  return cudaGetLastError();
}

cudaError_t launch_single_meta(int* iota, long long* zeros, cudaStream_t s) {
  k_single_meta<<<1, 128, 0, s>>>(iota, zeros);
  return cudaGetLastError();
}

cudaError_t launch_bin_sort(const int* ns, int count, int* order, int* sched, const BinBounds& bounds,
                            cudaStream_t s) {
  k_bin_sort<<<1, 1024, 0, s>>>(ns, count, order, sched, bounds, nullptr, 0);
  return cudaGetLastError();
}

cudaError_t launch_bin_sort_status(const int* ns, int count, const int* status, int code, int* order, int* sched,
                                   const BinBounds& bounds, cudaStream_t s) {
  k_bin_sort<<<1, 1024, 0, s>>>(ns, count, order, sched, bounds, status, code);
  return cudaGetLastError();
}

cudaError_t launch_batch_extent(const int* ns, const long long* offs, const long long* woffs, int count,
                                unsigned long long* out, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_batch_extent<<<std::min(1024, (count + 255) / 256), 256, 0, s>>>(ns, offs, woffs, count, out);
  return cudaGetLastError();
}

cudaError_t launch_bin_sort(const int* ns, int count, int* order, int* sched, cudaStream_t s) {
  BinBounds d;
  for (int i = 0; i < kNumBins; ++i) d.b[i] = bin_max(i);
  return launch_bin_sort(ns, count, order, sched, d, s);
}

BinTuning default_tuning_real() {
  return BinTuning{{32, 64, 96, 128}, {64, 64, 128, 128}, {1, 1, 0, 0}, {0, 0, 0, 0}};
}
BinTuning default_tuning_cplx() {
  return BinTuning{{32, 64, 96, 128}, {64, 64, 128, 128}, {1, 1, 0, 0}, {0, 0, 0, 0}};
}
BinTuning default_tuning_mixed32() {
  return BinTuning{{32, 64, 96, 128}, {64, 64, 128, 128}, {1, 1, 0, 0}, {0, 0, 0, 0}};
}

// Largest dynamic shared memory a CTA may use on sm_103 (227 KiB), less the kernels'
// static shared memory.
static constexpr size_t kMaxDynSmem = 227 * 1024 - 1024;

bool tuning_shape_ok(int kind, int nmax, int nt, int hsmem) {
  bool known = false;
  for (int t : kTuneThreads) known |= (t == nt);
  if (kind == kTuneMixed32 && nt == 160) known = false;
  if (!known || nmax < 1 || nmax > kSmallMax || kind < 0 || kind > kTuneMixed32) return false;
  const size_t b = kind == kTuneCplx ? cplx_bin_smem_bytes(nmax, hsmem)
                                     : (kind == kTuneReal ? real_bin_smem_bytes(nmax, hsmem)
                                                          : real32_bin_smem_bytes(nmax, hsmem));
  return b <= kMaxDynSmem;
}

}  // namespace gsk
