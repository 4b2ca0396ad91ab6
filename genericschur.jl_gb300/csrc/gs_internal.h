// Internal declarations shared by the kernel translation units and the C-ABI.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gsk {

// Largest matrix order handled by the one-CTA-per-matrix kernels.
constexpr int kSmallMax = 128;

// Per-matrix status codes (also the C-ABI return codes).
enum : int { ST_OK = 0, ST_UNCONVERGED = 1, ST_BADARG = 2, ST_CUDA = 3 };

// A ragged batch of column-major matrices in one packed buffer.  Matrix b has
// order ns[b] and starts at element offs[b] of A and Z; its eigenvalues start at
// woffs[b].  All pointers are device pointers.
struct RealBatch {
  int count;
  const int* ns;
  const long long* offs;
  const long long* woffs;
  double* A;       // in: A; out: T (quasi-triangular, standard form)
  double* Z;       // out: Schur vectors (ignored when wantz == 0)
  double* wr;      // out: real parts of the eigenvalues
  double* wi;      // out: imaginary parts
  int* status;     // out: ST_OK / ST_UNCONVERGED per matrix
  int wantz;
  int scale;
  int maxiter_mult;  // maxiter = maxiter_mult * n (reference default 100)
  long long maxiter_abs;  // when > 0, overrides maxiter_mult
};

struct CplxBatch {
  int count;
  const int* ns;
  const long long* offs;
  const long long* woffs;
  double2* A;      // in: A; out: T (upper triangular)
  double2* Z;
  double2* w;
  int* status;
  int wantz;
  int scale;
  int maxiter_mult;  // maxiter = maxiter_mult * n (reference default 100)
  int maxinner_mult; // maxinner = maxinner_mult * n (reference default 30)
  long long maxiter_abs;   // when > 0, overrides maxiter_mult
  long long maxinner_abs;  // when > 0, overrides maxinner_mult
};

// Size bins of the persistent batched kernels.  `sched` holds, per bin, the
// [start, end) range of that bin inside the sorted work order and a queue ticket
// counter: sched[3*bin + {0,1,2}].
constexpr int kNumBins = 4;
__host__ __device__ constexpr int bin_max(int bin) { return 32 * (bin + 1); }  // 32, 64, 96, 128

// Sorting/binning kernel: order[] lists matrix indices grouped by bin, largest
// order first inside a bin; sched[] receives the bin ranges and zeroed counters.
cudaError_t launch_bin_sort(const int* ns, int count, int* order, int* sched, cudaStream_t s);

cudaError_t launch_schur_batched_real(const RealBatch& bt, const int* order, int* sched,
                                      int num_sms, cudaStream_t* streams, int nstreams);
cudaError_t launch_schur_batched_cplx(const CplxBatch& bt, const int* order, int* sched,
                                      int num_sms, cudaStream_t* streams, int nstreams);

}  // namespace gsk
