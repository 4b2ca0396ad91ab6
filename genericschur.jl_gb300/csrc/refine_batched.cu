// Batched mixed-precision real Schur (orders <= 128): FP32 Schur pairs refined to FP64.
//
// The FP64 pipe of GB300 issues about one FP64 FMA per SM per cycle pair, the FP32 pipe
// sixty-four times that, so the batched FP64 Francis kernel is bound by FP64 issue
// (the QR sweeps are sequences of short dependent updates).  The mixed form runs the
// same Francis kernel in FP32 and wins FP64 accuracy back with a few dense FP64
// products per matrix, which keep the FP64 pipe busy:
//
//   1. k_mixed_prep   per matrix the power of two 2^e with max|a_ij| 2^-e in [1, 2) and
//                     A32 = fp32(A 2^-e) (the scaling is exact, so FP32 cannot overflow);
//   2. the FP32 batched Schur kernel on A32 -> (T32, Z32), standard form;
//   3. up to six Newton steps of the iteration of Bujanovic, Kressner and Schroeder
//      ("Iterative refinement of Schur decompositions", Numer. Algorithms 2023) with the
//      1x1/2x2 block structure of T32, each step two launches over the matrices still
//      being refined: k_refine_tc (refine_tc.cu), the FP64-accurate products on the
//      tensor cores, then k_refine_bin (refine_bin_impl.cuh, one kernel per size bin,
//      one CTA per matrix), the rest of the step:
//        At = Z^T A_s Z (FP64-accurate),  N = (I - Z^T Z) / 2 (FP64-accurate product, FP32 result);
//        W block-lower solving, for blocks p > q,
//          T_pp W_pq - W_pq T_qq = -L'_pq - sum_{r>p} T_pr W_rq + sum_{r<q} W_pr T_rq,
//        with T / L the block-upper / block-lower parts of At and L' the block-lower part
//        of At + N At + At N  (FP32: anti-diagonal waves of block pairs);
//        X = N + W - W^T;  Z <- Z + Z X.
//      Z (I + X) is orthogonal and (I + X)^T At (I + X) block upper triangular to first
//      order in X.  Products with X or N run in FP32 (their error is eps32 |X| |A|); the
//      products whose small parts are the signal (A Z, Z^T (A Z), Z^T Z) are FP64-accurate.
//      Once max|X| <= 1e-9 the step is the last (the FP32 products then add at most a few
//      eps |A|): T = At + X^T At + At X with the block-lower part set to zero,
//      Z <- Z + Z X, the 2x2 blocks standardised with _gs2x2! (GenericSchur.jl:716-803)
//      at the unit scale of A_s (its thresholds are absolute: at 1e-300, b c underflows),
//      then T and the eigenvalues scaled back by 2^e;
//   4. matrices whose FP32 Schur did not converge, or whose refinement diverges, stops
//      gaining (from the third step on, less than 4x per step) or has not reached the
//      tolerance in six steps (eigenvalues FP32 cannot separate), keep A untouched and
//      are recomputed by the FP64 batched kernel (or reported unconverged).
// The eigenvalue order is the FP32 run's deflation order; the result satisfies the same
// backward-error, orthogonality and standard-form conditions as the FP64 path.
#include <algorithm>

#include "refine_batched.cuh"

namespace gsk {
namespace {

// Per matrix: the scale exponent and the FP32 copy of A 2^-e.
__global__ void __launch_bounds__(256) k_mixed_prep(int count, const int* ns, const long long* offs, const double* A,
                                                    float* A32, int* exps) {
  __shared__ double red[8];
  for (int b = blockIdx.x; b < count; b += gridDim.x) {
    const int n = ns[b];
    if (n < 1 || n > kSmallMax) {
      if (threadIdx.x == 0) exps[b] = 0;
      continue;
    }
    const double* Ab = A + offs[b];
    float* Fb = A32 + offs[b];
    const int nn = n * n;
    double m = 0.0;
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
      const double v = fabs(Ab[i]);
      m = (v > m || v != v) ? v : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double v = __shfl_xor_sync(0xffffffffu, m, o);
      m = (v > m || v != v) ? v : m;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = red[0];
    for (int w = 1; w < 8; ++w) m = (red[w] > m || red[w] != red[w]) ? red[w] : m;
    const int e = (m > 0.0 && m <= 1.7976931348623157e308) ? ilogb(m) : 0;
    const double sc = ldexp(1.0, -e);
    for (int i = threadIdx.x; i < nn; i += blockDim.x) Fb[i] = (float)(Ab[i] * sc);
    if (threadIdx.x == 0) exps[b] = e;
  }
}

// Per matrix, after the FP32 stage: the 2x2 block starts of T32, Z = fp64(Z32), and the
// status for the refinement (kStRefining, or handed back when the FP32 Schur did not
// converge).
__global__ void __launch_bounds__(128) k_refine_init(RefineArgs a) {
  for (int b = blockIdx.x; b < a.count; b += gridDim.x) {
    const int n = a.ns[b];
    if (n < 1 || n > kSmallMax) continue;
    const int st = a.status[b];
    if (st != ST_OK) {
      if (threadIdx.x == 0 && st == ST_UNCONVERGED) {
        if (!a.nofallback) a.status[b] = kStFallback;
        if (a.stats) atomicAdd(a.stats + 1, 1ull);
      }
      continue;
    }
    const long long off = a.offs[b];
    const float* T = a.T32 + off;
    const float* ZF = a.Z32 + off;
    double* Z = a.Z + off;
    unsigned char* blk = a.blk + a.woffs[b];
    // a 2x2 block starts at row i when T(i+1, i) != 0 (standard form: no two in a row)
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      blk[i] = (unsigned char)(i + 1 < n && T[(size_t)i * n + i + 1] != 0.f);
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) Z[idx] = (double)ZF[idx];
    // scale exponents of the tensor-core products: rows of A (fixed), columns of Z
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double* Ai = a.A + off + i;
      double m = 0.0;
      int k = 0;
      for (; k + 8 <= n; k += 8) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = fabs(Ai[(size_t)(k + u) * n]);
#pragma unroll
        for (int u = 0; u < 8; ++u) m = refine_nanmax(m, v[u]);
      }
      for (; k < n; ++k) m = refine_nanmax(m, fabs(Ai[(size_t)k * n]));
      a.exA[a.woffs[b] + i] = refine_scale_exp(m);
    }
    __syncthreads();
    refine_col_exps<128>(n, Z, a.exZ + a.woffs[b]);
    if (threadIdx.x == 0) a.status[b] = kStRefining;
  }
}

}  // namespace

size_t mixed_batched_ws_bytes(long long na, long long nw, bool wantz) {
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t b = 0;
  b += 5 * al(sizeof(float) * (size_t)na);                  // A32/T32, Z32, M, W, NF
  b += 2 * al(sizeof(float) * (size_t)nw);                  // FP32 eigenvalues
  b += (wantz ? 2 : 3) * al(sizeof(double) * (size_t)na);  // P, Q (, Z)
  b += al((size_t)nw);                                     // 2x2 block starts
  b += 2 * al(sizeof(int) * (size_t)nw);                   // scale exponents of A's rows, Z's columns
  return b;
}

cudaError_t launch_refine_init(const RefineArgs& a, int num_sms, cudaStream_t s) {
  k_refine_init<<<std::max(1, std::min(a.count, 16 * num_sms)), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_mixed_batched(const MixedBatch& m, int num_sms, cudaStream_t s, cudaStream_t* aux, int naux,
                                 cudaEvent_t fork, cudaEvent_t* join, const BinTuning& tun64, const BinTuning& tun32) {
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  char* w = static_cast<char*>(m.ws);
  auto take = [&](size_t bytes) { char* p = w; w += al(bytes); return (void*)p; };
  float* A32 = (float*)take(sizeof(float) * (size_t)m.na);
  float* Z32 = (float*)take(sizeof(float) * (size_t)m.na);
  float* M = (float*)take(sizeof(float) * (size_t)m.na);
  float* W = (float*)take(sizeof(float) * (size_t)m.na);
  float* NF = (float*)take(sizeof(float) * (size_t)m.na);
  float* wr32 = (float*)take(sizeof(float) * (size_t)m.nw);
  float* wi32 = (float*)take(sizeof(float) * (size_t)m.nw);
  double* P = (double*)take(sizeof(double) * (size_t)m.na);
  double* Q = (double*)take(sizeof(double) * (size_t)m.na);
  double* Zw = m.Z ? m.Z : (double*)take(sizeof(double) * (size_t)m.na);
  unsigned char* blk = (unsigned char*)take((size_t)m.nw);
  int* exA = (int*)take(sizeof(int) * (size_t)m.nw);
  int* exZ = (int*)take(sizeof(int) * (size_t)m.nw);
  int* exps = m.iws;
  float* xprev = reinterpret_cast<float*>(m.iws + m.count);
  int* order2 = m.iws + 2 * (size_t)m.count;
  int* sched2 = m.iws + 3 * (size_t)m.count;
  int* ticket = sched2 + 3 * kNumBins + 2;  // kRefineTicketsPerStep * kRefineSteps counters
  static_assert(3 * kNumBins + 2 + kRefineTicketsPerStep * kRefineSteps <= kMixedSchedInts,
                "the run's schedule words hold the ticket counters");
  cudaError_t e;
  // 1. bin sort (the default bins: the FP32 table keeps them, the refinement kernels are
  // compiled per default bin) and the FP32 copies
  if ((e = launch_bin_sort(m.ns, m.count, m.order, m.sched, s)) != cudaSuccess) return e;
  k_mixed_prep<<<std::min(m.count, 64 * num_sms), 256, 0, s>>>(m.count, m.ns, m.offs, m.A, A32, exps);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // 2. FP32 Schur pairs
  RealBatchT<float, float> b32{};
  b32.count = m.count; b32.ns = m.ns; b32.offs = m.offs; b32.woffs = m.woffs;
  b32.A = A32; b32.Z = Z32; b32.wr = wr32; b32.wi = wi32; b32.status = m.status;
  b32.wantz = 1; b32.scale = 0; b32.maxiter_mult = 100;
  auto forked = [&](auto body) -> cudaError_t {
    cudaError_t r = cudaEventRecord(fork, s);
    if (r != cudaSuccess) return r;
    for (int i = 0; i < naux; ++i)
      if ((r = cudaStreamWaitEvent(aux[i], fork, 0)) != cudaSuccess) return r;
    if ((r = body()) != cudaSuccess) return r;
    for (int i = 0; i < naux; ++i) {
      if ((r = cudaEventRecord(join[i], aux[i])) != cudaSuccess) return r;
      if ((r = cudaStreamWaitEvent(s, join[i], 0)) != cudaSuccess) return r;
    }
    return cudaSuccess;
  };
  e = forked([&]() { return launch_schur_batched_real32_tuned(b32, m.order, m.sched, num_sms, aux, naux, tun32); });
  if (e != cudaSuccess) return e;
  // 3. refinement, largest matrices first: per Newton step the tensor-core products, then
  // one kernel per default size bin (orders <= 32, 64, 96, 128: row tiles 2, 4, 6, 8 x 16),
  // forked like the Schur bins so that the bins' tails overlap
  if ((e = cudaMemsetAsync(ticket, 0, sizeof(int) * kRefineTicketsPerStep * kRefineSteps, s)) != cudaSuccess)
    return e;
  // under stream capture: external event nodes, so that the graph's replay records them
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if ((e = cudaStreamIsCapturing(s, &cap)) != cudaSuccess) return e;
  const unsigned evflags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
  if (m.ref0 && (e = cudaEventRecordWithFlags(m.ref0, s, evflags)) != cudaSuccess) return e;
  RefineArgs ra{};
  ra.count = m.count; ra.ns = m.ns; ra.offs = m.offs; ra.woffs = m.woffs;
  ra.A = m.A; ra.Z = Zw; ra.T32 = A32; ra.Z32 = Z32; ra.P = P; ra.Q = Q; ra.M = M; ra.W = W; ra.NF = NF;
  ra.wr = m.wr; ra.wi = m.wi; ra.status = m.status; ra.exps = exps; ra.order = m.order; ra.sched = m.sched;
  ra.ticket = ticket; ra.blk = blk; ra.exA = exA; ra.exZ = exZ; ra.xprev = xprev; ra.err = m.tc_err; ra.nofallback = m.nofallback;
  ra.stats = m.stats;
  if ((e = launch_refine_init(ra, num_sms, s)) != cudaSuccess) return e;
  static_assert(kNumBins == 4, "the refinement bins follow the default size bins");
  for (int step = 0; step < kRefineSteps; ++step) {
    if ((e = launch_refine_tc(ra, step, num_sms, s)) != cudaSuccess) return e;
    e = forked([&]() -> cudaError_t {
      cudaError_t r;
      if ((r = launch_refine_bin<8>(ra, 3, step, num_sms, aux[0 % naux])) != cudaSuccess) return r;
      if ((r = launch_refine_bin<6>(ra, 2, step, num_sms, aux[1 % naux])) != cudaSuccess) return r;
      if ((r = launch_refine_bin<4>(ra, 1, step, num_sms, aux[2 % naux])) != cudaSuccess) return r;
      return launch_refine_bin<2>(ra, 0, step, num_sms, aux[3 % naux]);
    });
    if (e != cudaSuccess) return e;
  }
  if (m.ref1 && (e = cudaEventRecordWithFlags(m.ref1, s, evflags)) != cudaSuccess) return e;
  if (m.nofallback) return cudaSuccess;
  // 4. the FP64 kernel on the matrices the refinement handed back
  BinBounds bounds;
  for (int i = 0; i < kNumBins; ++i) bounds.b[i] = tun64.bounds[i];
  if ((e = launch_bin_sort_status(m.ns, m.count, m.status, kStFallback, order2, sched2, bounds, s)) != cudaSuccess)
    return e;
  RealBatchT<double, double> b64{};
  b64.count = m.count; b64.ns = m.ns; b64.offs = m.offs; b64.woffs = m.woffs;
  b64.A = m.A; b64.Z = m.Z; b64.wr = m.wr; b64.wi = m.wi; b64.status = m.status;
  b64.wantz = m.Z != nullptr; b64.scale = m.scale; b64.maxiter_mult = 100;
  return forked([&]() { return launch_schur_batched_real_tuned(b64, order2, sched2, num_sms, aux, naux, tun64); });
}

}  // namespace gsk
