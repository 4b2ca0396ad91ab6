// Arguments of the mixed-precision batched real Schur refinement (refine_batched.cu
// describes the method); the bin kernels are in refine_bin_impl.cuh,
// instantiated by one translation unit per size bin (refine_bin_r*.cu).
#pragma once
#include <algorithm>

#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {

struct RefineArgs {
  int count;
  const int* ns;
  const long long* offs;
  const long long* woffs;
  double* A;      // in: A; out: T where the refinement succeeds (else untouched)
  double* Z;      // out: Z (workspace when the caller wants no Z)
  float* T32;     // in: FP32 Schur form; scratch (fp32 of At) afterwards
  float* Z32;     // in: FP32 Schur vectors; scratch (fp32 of Z) afterwards
  double* P;      // FP64 scratch (A Z, then the new Z)
  double* Q;      // FP64 scratch (At)
  float* M;       // FP32 scratch (right-hand sides)
  float* W;       // FP32 scratch (W, then X)
  float* NF;      // FP32 scratch (N)
  double* wr;
  double* wi;
  int* status;    // in: FP32 status; out: ST_OK, kStFallback, ST_UNCONVERGED or ST_BADARG
  const int* exps;
  const int* order;
  const int* sched;  // bin ranges of the bin sort (3 ints per bin)
  int* ticket;       // one zeroed counter per bin
  unsigned long long* stats;  // null, or: refined, handed back, Newton steps, FP64 FLOPs
  int nofallback;
};

// One bin's refinement kernel: RM = 2, 4, 6, 8 serves orders <= 16 RM.
template <int RM>
cudaError_t launch_refine_bin(const RefineArgs& a, int bin, int num_sms, cudaStream_t s);

}  // namespace gsk
