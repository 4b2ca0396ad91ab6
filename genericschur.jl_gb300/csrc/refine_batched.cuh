// Arguments of the mixed-precision batched real Schur refinement (refine_batched.cu
// describes the method); the FP64-accurate products of each Newton step run on the
// tensor cores (refine_tc.cu), the rest of the step in the bin kernels of
// refine_bin_impl.cuh, instantiated by one translation unit per size bin (refine_bin_r*.cu).
#pragma once
#include <algorithm>

#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {

// Per-matrix status while the refinement runs: awaiting the step's tensor-core products,
// or products done (the rest of the step to come).
constexpr int kStRefining = 8;
constexpr int kStStepReady = 9;
constexpr int kRefineSteps = 6;  // Newton steps before a matrix is handed back
// ticket counters per Newton step: one per size bin, one for the tensor-core products
constexpr int kRefineTicketsPerStep = kNumBins + 1;

struct RefineArgs {
  int count;
  const int* ns;
  const long long* offs;
  const long long* woffs;
  double* A;      // in: A; out: T where the refinement succeeds (else untouched)
  double* Z;      // out: Z (workspace when the caller wants no Z)
  float* T32;     // in: FP32 Schur form; then fp32 of At (Z^T A_s Z) per step
  float* Z32;     // in: FP32 Schur vectors; scratch (fp32 of Z) afterwards
  double* P;      // FP64 scratch (A_s Z, then the new Z)
  double* Q;      // FP64 At = Z^T A_s Z of the step
  float* M;       // FP32 scratch (right-hand sides)
  float* W;       // FP32 scratch (W, then X)
  float* NF;      // FP32 N = (I - Z^T Z) / 2 of the step
  double* wr;
  double* wi;
  int* status;    // in: FP32 status; kStRefining while refined; out: ST_OK, kStFallback,
                  // ST_UNCONVERGED or ST_BADARG
  const int* exps;
  const int* order;
  const int* sched;  // bin ranges of the bin sort (3 ints per bin)
  int* ticket;       // kRefineTicketsPerStep * kRefineSteps zeroed counters
  unsigned char* blk;  // per eigenvalue slot (woffs): 1 where a 2x2 block of T32 starts
  int* exA;            // per eigenvalue slot (woffs): row scale exponents of A
  int* exZ;            // per eigenvalue slot (woffs): column scale exponents of the current Z
  float* xprev;        // per matrix: max|X| of the previous Newton step
  int* err;            // set when a tensor-core wait timed out (the matrix was handed back)
  unsigned long long* stats;  // null, or: refined, handed back, Newton steps, FP64-accurate product FLOPs
  int nofallback;
};

// Scale exponents of the tensor-core products: e with max |x| < 2^e over a row or column,
// or a sentinel for a zero row / column and for one holding Inf or NaN.
constexpr int kExpZeroRow = -100000;
constexpr int kExpBadRow = 100000;
__device__ __forceinline__ int refine_scale_exp(double m) {
  if (m == 0.0) return kExpZeroRow;
  if (!(m <= 1.7976931348623157e308)) return kExpBadRow;
  int e;
  frexp(m, &e);  // m < 2^e
  return e;
}
__device__ __forceinline__ double refine_nanmax(double m, double v) { return (v > m || v != v) ? v : m; }

// Column exponents of an n x n column-major FP64 matrix (n <= 128) by a CTA of NT threads:
// a warp per column, four columns in flight per warp.
template <int NT>
__device__ void refine_col_exps(int n, const double* M, int* out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c0 = 4 * warp; c0 < n; c0 += 4 * (NT / 32)) {
    double v[4][kSmallMax / 32];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int r = 0; r < kSmallMax / 32; ++r) {
        const int k = lane + 32 * r;
        v[u][r] = (c0 + u < n && k < n) ? fabs(M[(size_t)(c0 + u) * n + k]) : 0.0;
      }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      double m = v[u][0];
#pragma unroll
      for (int r = 1; r < kSmallMax / 32; ++r) m = refine_nanmax(m, v[u][r]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = refine_nanmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (lane == 0 && c0 + u < n) out[c0 + u] = refine_scale_exp(m);
    }
  }
}

// Block structure of T32, Z = fp64(Z32), and the status of every matrix for the
// refinement (kStRefining, or handed back when its FP32 Schur did not converge).
cudaError_t launch_refine_init(const RefineArgs& a, int num_sms, cudaStream_t s);
// The tensor-core products of Newton step `step` for every matrix still refined.
cudaError_t launch_refine_tc(const RefineArgs& a, int step, int num_sms, cudaStream_t s);
// The rest of Newton step `step` for one size bin: RM = 2, 4, 6, 8 serves orders <= 16 RM.
template <int RM>
cudaError_t launch_refine_bin(const RefineArgs& a, int bin, int step, int num_sms, cudaStream_t s);

}  // namespace gsk
