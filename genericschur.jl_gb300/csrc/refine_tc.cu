// FP64-accurate matrix products of the batched mixed-precision refinement on the BF16
// tensor cores (tcgen05), one CTA per matrix of order n <= 128.
//
// Every Newton step of the refinement (refine_batched.cu) needs three products whose
// small parts carry the signal and which therefore must be accurate to FP64 rounding:
//   P  = A_s Z                      (A_s = A 2^-e, the unit-scaled input),
//   At = Z^T P                      (its block-lower part is the Schur residual),
//   G  = Z^T Z                      (N = (I - G) / 2 is the orthogonality correction).
// On GB300 the FP64 pipe runs about 1.2 TFLOP/s while the BF16 tensor cores run about
// 2 PFLOP/s, so these products use the error-free splitting of Ozaki, Ogita, Oishi and
// Rump (Numer. Algorithms 59, 2012) in the tensor-core form of Mukunoki, Ozaki, Ogita and
// Imamura (ISC 2020), sized for n <= 128:
//   * row i of op(X) is scaled by 2^e_i with max_k |x_ik| < 2^e_i, column j of Y by 2^f_j;
//   * the scaled entries are cut into S = 8 slices of 7 bits (56 bits, exact up to the
//     last slice): x = 2^e sum_s q_s 2^{-7 s}, |q_s| <= 127, each slice a BF16 integer;
//   * a slice product summed over k <= 128 is at most 127^2 * 128 < 2^21, and the up to 8
//     slice products of one level s + t add up to less than 2^24, so the tensor core's
//     FP32 accumulation of a whole level is exact in any order;
//   * C_ij = 2^{e_i + f_j} sum_{s + t <= 9} 2^{-7 (s + t)} (level sums), the 8 exact level
//     sums converted to FP64 and added least significant first.  The truncation (2^-56
//     of the row maximum) and the dropped levels (s + t >= 10) stay below the rounding
//     error of an FP64 dot product of the same length.
//
// Kernel k_refine_tc: persistent CTAs of 512 threads (one per SM: the eight level
// accumulators fill the SM's 512 TMEM columns), each taking the matrices still being
// refined from a ticket counter, largest first.  Per product, per 64-column panel of Y:
// chunks of 32 contraction indices are split by all threads straight into shared memory
// in the tensor core's canonical K-major layout (no swizzle; 8 x 8 core matrices of 128
// contiguous bytes, K-adjacent core matrices 128 B apart, 8-row groups 512 B apart),
// double-buffered so that one chunk is split while the MMAs of the previous one run;
// thread 0 issues the 36 slice products per 16-wide K step (tcgen05.mma, M = 128,
// N = 64, K = 16) into the accumulator of their level; after the panel's last chunk the
// sixteen warps (four per TMEM lane quarter, 16 columns each) drain the levels with
// tcgen05.ld.  Every wait is bounded: a timeout hands the matrix to the FP64 kernel
// (status kStFallback), records the error, waits for the CTA's MMAs, frees TMEM and ends
// the CTA.
#include <cstdint>

#include "refine_batched.cuh"
#include "tc_common.cuh"

namespace gsk {
namespace {

using namespace tc;

constexpr int kQBits = 7;                          // bits per slice
constexpr int kQSlices = 8;                        // slices per operand (56 bits)
constexpr int kQLevels = 8;                        // levels s + t = 0 .. 7 (0-based slices)
constexpr int kQM = 128;                           // MMA M (rows of op(X), zero-padded)
constexpr int kQN = 64;                            // MMA N: panel width of Y
constexpr int kQK = 32;                            // contraction indices per chunk
constexpr int kQThreads = 512;
constexpr int kQXSlice = kQM * kQK * 2;            // bytes of one X slice of a chunk (8 KiB)
constexpr int kQYSlice = kQN * kQK * 2;            // bytes of one Y slice of a chunk (4 KiB)
constexpr int kQStage = kQSlices * (kQXSlice + kQYSlice);  // 96 KiB
constexpr int kQSbo = (kQK / 8) * 128;             // bytes between 8-row groups
constexpr uint32_t kQIdesc = idesc_bf16(kQM, kQN);
constexpr int kQExpZero = kExpZeroRow;             // row / column of zeros
constexpr int kQExpBad = kExpBadRow;               // row / column with Inf or NaN
constexpr unsigned long long kQTimeout = 4000000000ull;  // ~2 s of SM clock

struct QCtl {
  uint64_t bar[2];     // MMA completion per stage (tcgen05.commit)
  uint64_t done;       // every MMA of the CTA complete (before TMEM is freed)
  uint32_t tslot;
  int ticket;
  int fail;
  int exA[kQM];        // row exponents of A (the rows of op(X) in A_s Z)
  int exZ[kQM];        // column exponents of Z (rows of Z^T, columns of Z)
  int exP[kQM];        // column exponents of P = A_s Z
};

constexpr size_t kQSmem = 2 * (size_t)kQStage + sizeof(QCtl) + 128;

// floor(|x| 2^(56 - e)) for |x| < 2^e (so below 2^56), from the IEEE bits; its 7-bit
// groups are the slices of |x| 2^-e.
__device__ __forceinline__ unsigned long long fixed56(double x, int e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
  const int be = (int)(b >> 52);
  if (b == 0ull) return 0ull;
  const unsigned long long m = (b & 0xfffffffffffffull) | (be ? (1ull << 52) : 0ull);
  const int ex = be ? be - 1075 : -1074;  // |x| = m 2^ex
  const int sh = ex + 56 - e;             // <= 3
  if (sh >= 0) return m << sh;
  return sh <= -64 ? 0ull : (m >> (-sh));
}

// The integer value of an FP32 word holding an integer of magnitude below 2^24 (a level
// sum), by integer operations: the significand shifted by the exponent, with the sign.
__device__ __forceinline__ long long level_int(uint32_t u) {
  const int e = (int)((u >> 23) & 255u);
  const uint32_t m = (u & 0x7fffffu) | 0x800000u;
  const int mag = e >= 127 ? (int)(m >> (150 - e)) : 0;
  return (long long)((int)u < 0 ? -mag : mag);
}

// Two 7-bit integers q0, q1 (< 128) as a packed BF16 pair (q0 low), exact: in FP32,
// (2^23 + q) - 2^23 = q, and the upper 16 bits of an FP32 integer below 2^8 are its BF16.
__device__ __forceinline__ unsigned bf16x2_q(unsigned q0, unsigned q1) {
  const float f0 = __uint_as_float(0x4B000000u | q0) - 8388608.f;
  const float f1 = __uint_as_float(0x4B000000u | q1) - 8388608.f;
  return __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632);
}

// Eight values of one row (op(X) row i, or Y column j) at k0 .. k0 + 7 -> the 16-byte
// core-matrix row of each slice, at `dst` + s * slice_bytes.  The 56-bit fixed-point
// magnitudes are held as two 28-bit halves of four slices each; the sign is applied to
// every slice.
__device__ __forceinline__ void split8(const double (&v)[8], int e, unsigned char* dst, int slice_bytes) {
  unsigned hi[8], lo[8], sg[4];
  const bool live = e != kQExpZero && e != kQExpBad;
#pragma unroll
  for (int x = 0; x < 8; ++x) {
    const unsigned long long f = live ? fixed56(v[x], e) : 0ull;
    hi[x] = (unsigned)(f >> 28);
    lo[x] = (unsigned)f & 0xfffffffu;
  }
#pragma unroll
  for (int x = 0; x < 4; ++x) {
    const unsigned n0 = (unsigned)(((unsigned long long)__double_as_longlong(v[2 * x])) >> 63);
    const unsigned n1 = (unsigned)(((unsigned long long)__double_as_longlong(v[2 * x + 1])) >> 63);
    sg[x] = (n0 << 15) | (n1 << 31);
  }
#pragma unroll
  for (int s = 0; s < kQSlices; ++s) {
    const int sh = 21 - kQBits * (s & 3);
    unsigned w[4];
#pragma unroll
    for (int x = 0; x < 4; ++x) {
      const unsigned a0 = ((s < 4 ? hi[2 * x] : lo[2 * x]) >> sh) & 127u;
      const unsigned a1 = ((s < 4 ? hi[2 * x + 1] : lo[2 * x + 1]) >> sh) & 127u;
      w[x] = bf16x2_q(a0, a1) ^ sg[x];
    }
    *reinterpret_cast<uint4*>(dst + s * slice_bytes) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__device__ __forceinline__ void zero8(unsigned char* dst, int slice_bytes) {
#pragma unroll
  for (int s = 0; s < kQSlices; ++s) *reinterpret_cast<uint4*>(dst + s * slice_bytes) = make_uint4(0u, 0u, 0u, 0u);
}

// One product C = op(X) Y of n x n column-major FP64 matrices with the exponents of the
// rows of op(X) in ex and of the columns of Y in fy.  XT = 0: op(X) = X, XT = 1:
// op(X) = X^T.  KIND 0: P = C 2^extra; KIND 1: Q = C, F = fp32(C); KIND 2:
// F = fp32((I - C) / 2).  Returns false after a timed-out wait (the CTA must stop).
template <int XT, int KIND>
__device__ bool tc_product(int n, const double* X, const double* Y, const int* ex, const int* fy, int extra,
                           double* Cd, float* Cf, unsigned char* smem, QCtl& ctl, uint32_t tmem,
                           unsigned& gchunk) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nchunks = (n + kQK - 1) / kQK;
  const uint32_t s0 = smem_u32(smem);
  for (int j0 = 0; j0 < n; j0 += kQN) {
    for (int c = 0; c < nchunks; ++c, ++gchunk) {
      const int st = gchunk & 1;
      // the MMAs that last read this stage must be complete before it is overwritten
      if (tid == 0) {
        ctl.fail = 0;
        if (gchunk >= 2 && !mbar_wait(&ctl.bar[st], ((gchunk >> 1) - 1) & 1u, kQTimeout)) ctl.fail = 1;
      }
      __syncthreads();
      if (ctl.fail) return false;
      unsigned char* xs = smem + st * kQStage;
      unsigned char* ys = xs + kQSlices * kQXSlice;
      const int k0 = c * kQK;
      // items: op(X) rows (128 rows x 4 groups of 8 k), then the panel's Y columns (64 x 4);
      // rows of op(X) and columns of Y beyond n only reach outputs that are not stored, so
      // they are skipped; contraction indices beyond n are zero in both operands
      constexpr int kXItems = kQM * (kQK / 8), kItems = kXItems + kQN * (kQK / 8);
      constexpr int kPer = (kItems + kQThreads - 1) / kQThreads;  // 2
      double v[kPer][8];
      int eit[kPer];
      unsigned char* dst[kPer];
      bool live[kPer];
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        const int it = tid + u * kQThreads;
        int row = 0, kg = 0, e = kQExpZero;
        if (it >= kItems) {
          live[u] = false;
          dst[u] = xs;
        } else if (it < kXItems) {
          row = it & (kQM - 1); kg = it >> 7;
          live[u] = row < n;
          dst[u] = xs + (((row >> 3) * (kQK / 8) + kg) * 64 + (row & 7) * 8) * 2;
          if (live[u]) e = ex[row];
        } else {
          const int jt = it - kXItems;
          const int jl = jt & (kQN - 1);
          kg = jt >> 6;
          row = j0 + jl;
          live[u] = row < n;
          dst[u] = ys + (((jl >> 3) * (kQK / 8) + kg) * 64 + (jl & 7) * 8) * 2;
          if (live[u]) e = fy[row];
        }
        eit[u] = e;
        const int kb = k0 + kg * 8;
#pragma unroll
        for (int x = 0; x < 8; ++x) {
          const int k = kb + x;
          double val = 0.0;
          if (live[u] && k < n) {
            if (it < kXItems) val = XT ? X[(size_t)row * n + k] : X[(size_t)k * n + row];
            else val = Y[(size_t)row * n + k];
          }
          v[u][x] = val;
        }
        if (kb >= n) eit[u] = kQExpZero;  // live rows whose k-group lies beyond n: zero slices
      }
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        if (!live[u]) continue;
        const int sb = (tid + u * kQThreads) < kXItems ? kQXSlice : kQYSlice;
        if (eit[u] == kQExpZero) zero8(dst[u], sb);
        else split8(v[u], eit[u], dst[u], sb);
      }
      fence_proxy_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t xa = s0 + st * kQStage, ya = xa + kQSlices * kQXSlice;
        const uint64_t adesc = smem_desc(xa, 128, kQSbo), bdesc = smem_desc(ya, 128, kQSbo);
        // the 36 slice pairs (s, t), s + t = L <= 7, into the accumulator of level L; the
        // level's first pair at the panel's first K step overwrites it (descriptor start
        // addresses are in units of 16 bytes)
#pragma unroll
        for (int L = 0; L < kQLevels; ++L) {
#pragma unroll
          for (int s = 0; s <= L; ++s) {
#pragma unroll
            for (int kk = 0; kk < kQK / 16; ++kk) {
              const uint32_t acc = (c > 0 || kk > 0 || s > 0) ? 1u : 0u;
              tc_mma(tmem + (uint32_t)(L * kQN), adesc + (uint64_t)((s * kQXSlice + kk * 256) >> 4),
                     bdesc + (uint64_t)(((L - s) * kQYSlice + kk * 256) >> 4), kQIdesc, acc);
            }
          }
        }
        tc_commit(&ctl.bar[st]);
      }
    }
    // drain the panel: the last chunk's commit covers every MMA before it
    if (tid == 0) {
      const unsigned last = gchunk - 1;
      ctl.fail = mbar_wait(&ctl.bar[last & 1], (last >> 1) & 1u, kQTimeout) ? 0 : 1;
    }
    __syncthreads();
    if (ctl.fail) return false;
    tc_fence_after();
    {
      const int q = warp & 3, cq = warp >> 2;  // TMEM lane quarter, 16-column quarter of the panel
      const int i = q * 32 + lane;
      const int jb = j0 + cq * 16;
      // G = Z^T Z is symmetric: only the lower triangle is formed (and mirrored)
      const bool need = KIND != 2 || q * 32 + 32 > jb;
      if (jb < n && q * 32 < n && need) {  // warp-uniform
        // the eight exact level sums, as integers, combined in two 64-bit Horner sums of
        // four levels each (below 2^46, so their FP64 conversions are exact)
        long long hs[16], ls[16];
#pragma unroll
        for (int x = 0; x < 16; ++x) { hs[x] = 0; ls[x] = 0; }
        const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cq * 16);
#pragma unroll 1
        for (int L = 0; L < kQLevels; ++L) {  // most significant level first
          uint32_t v[16];
          tc_ld16(tb + L * kQN, v);
          tc_wait_ld();
          if (L < 4) {
#pragma unroll
            for (int x = 0; x < 16; ++x) hs[x] = hs[x] * 128 + level_int(v[x]);
          } else {
#pragma unroll
            for (int x = 0; x < 16; ++x) ls[x] = ls[x] * 128 + level_int(v[x]);
          }
        }
        if (i < n) {
          const int ei = ex[i];
#pragma unroll
          for (int x = 0; x < 16; ++x) {
            const int j = jb + x;
            if (j < n && (KIND != 2 || i >= j)) {
              const int fj = fy[j];
              double r;
              if (ei == kQExpBad || fj == kQExpBad) r = __longlong_as_double(0x7ff8000000000000ll);
              else if (ei == kQExpZero || fj == kQExpZero) r = 0.0;
              else {
                // sum_L lev_L 2^(-7 L) = hs 2^-21 + ls 2^-49, times 2^(e_i + f_j - 14)
                const double sum = fma((double)hs[x], 0x1p-21, (double)ls[x] * 0x1p-49);
                r = ldexp(sum, ei + fj - 2 * kQBits + (KIND == 0 ? extra : 0));
              }
              const size_t o = (size_t)j * n + i;
              if (KIND == 0) Cd[o] = r;
              else if (KIND == 1) { Cd[o] = r; Cf[o] = (float)r; }
              else {
                const float h2 = (float)(0.5 * ((i == j ? 1.0 : 0.0) - r));
                Cf[o] = h2;
                Cf[(size_t)i * n + j] = h2;
              }
            }
          }
        }
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  return true;
}

__global__ void __launch_bounds__(kQThreads, 1) k_refine_tc(RefineArgs a, int step) {
  extern __shared__ __align__(1024) unsigned char smem[];
  QCtl& ctl = *reinterpret_cast<QCtl*>(smem + 2 * kQStage);
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&ctl.bar[0], 1);
    mbar_init(&ctl.bar[1], 1);
    mbar_init(&ctl.done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if ((tid >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&ctl.tslot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = ctl.tslot;
  unsigned gchunk = 0;
  int* ticket = a.ticket + kRefineTicketsPerStep * step + kNumBins;
  // bins largest first: ticket t walks bin 3's range of the order array, then bin 2's, ...
  int total = 0;
  for (int bin = 0; bin < kNumBins; ++bin) total += a.sched[3 * bin + 1] - a.sched[3 * bin];
  for (;;) {
    __syncthreads();
    if (tid == 0) ctl.ticket = atomicAdd(ticket, 1);
    __syncthreads();
    int t = ctl.ticket;
    if (t >= total) break;
    int pos = -1;
    for (int bin = kNumBins - 1; bin >= 0; --bin) {
      const int len = a.sched[3 * bin + 1] - a.sched[3 * bin];
      if (t < len) { pos = a.sched[3 * bin] + t; break; }
      t -= len;
    }
    if (pos < 0) continue;
    const int b = a.order[pos];
    const int n = a.ns[b];
    if (n < 1 || n > kSmallMax || a.status[b] != kStRefining) continue;
    const long long off = a.offs[b];
    const double* A = a.A + off;
    double* P = a.P + off;
    double* Z = a.Z + off;
    {  // the exponents of A's rows (fixed) and Z's columns (from the previous step's update)
      const int* ga = a.exA + a.woffs[b];
      const int* gz = a.exZ + a.woffs[b];
      for (int i = tid; i < n; i += kQThreads) { ctl.exA[i] = ga[i]; ctl.exZ[i] = gz[i]; }
    }
    __syncthreads();
    bool ok = tc_product<0, 0>(n, A, Z, ctl.exA, ctl.exZ, -a.exps[b], P, nullptr, smem, ctl, tmem, gchunk);
    if (ok) {
      refine_col_exps<kQThreads>(n, P, ctl.exP);  // P was written by this CTA before the panel's closing barrier
      __syncthreads();
      ok = tc_product<1, 1>(n, Z, P, ctl.exZ, ctl.exP, 0, a.Q + off, a.T32 + off, smem, ctl, tmem, gchunk);
    }
    if (ok) ok = tc_product<1, 2>(n, Z, Z, ctl.exZ, ctl.exZ, 0, nullptr, a.NF + off, smem, ctl, tmem, gchunk);
    if (ok && tid == 0) a.status[b] = kStStepReady;
    if (!ok) {
      if (tid == 0) {
        a.status[b] = a.nofallback ? ST_UNCONVERGED : kStFallback;
        atomicExch(a.err, 1);
      }
      break;
    }
  }
  // every MMA issued must be complete before TMEM is freed
  if (tid == 0) {
    tc_commit(&ctl.done);
    if (!mbar_wait(&ctl.done, 0, kQTimeout)) atomicExch(a.err, 2);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if ((tid >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

}  // namespace

cudaError_t launch_refine_tc(const RefineArgs& a, int step, int num_sms, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_refine_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kQSmem);
  if (e != cudaSuccess) return e;
  k_refine_tc<<<num_sms, kQThreads, kQSmem, s>>>(a, step);
  return cudaGetLastError();
}

}  // namespace gsk
