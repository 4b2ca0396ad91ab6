// FP64 matrix product on the BF16 tensor cores (tcgen05), by exact splitting.
//
//   C (m x p, column-major, ldc) = op(A) (m x q) * B (q x p),   op(A) = A or A^T.
//
// GB300's FP64 pipe delivers ~1.2 TFLOP/s, while its BF16 tensor cores deliver ~2 PFLOP/s.
// The FP64 products of the mixed-precision Schur refinement (Z^T A Z, Z^T Z) therefore
// run as sums of exact BF16 x BF16 -> FP32 products:
//
// Method: the error-free splitting of Ozaki, Ogita, Oishi and Rump ("Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012), in the variant of
// Mukunoki, Ozaki, Ogita and Imamura ("DGEMM using Tensor Cores, and Its Accurate and
// Reproducible Versions", ISC 2020) that uses low-precision tensor-core inputs with FP32
// accumulation:
//   * row i of op(A) has the scale 2^e_i with max_k |a_ik| < 2^e_i; column j of B
//     likewise 2^f_j;
//   * a_ik = 2^e_i * sum_{s=1..S} q^A_iks 2^{-beta s} with integers |q| < 2^beta
//     (successive truncation of the scaled row; exact up to the last slice);
//   * with beta = 6, every product q^A q^B is below 2^12 and a sum of up to 4096 of them
//     below 2^24: the tensor core's FP32 accumulation of one slice pair over a K-chunk of
//     4096 is exact, whatever its internal order;
//   * C_ij = 2^{e_i + f_j} sum_{s + t <= S + 1} 2^{-beta (s + t)} (Q^A_s Q^B_t)_ij, the
//     exact FP32 chunk sums converted to FP64 and accumulated least significant first.
// With S = 10 (60 bits) and the 55 slice products of s + t <= 11, the slice truncation
// (2^-60 of the row maximum) and the dropped products (level 12 and below) stay below
// the rounding error of an FP64 dot product of the same length.
//
// Kernels:
//   k_absmax  per-row max |x| of both operands (atomicMax on the IEEE bits of |x|, which
//             order like the values and put NaN above Inf);
//   k_exps    the scale exponents (sentinels for zero and non-finite rows);
//   k_split   the S slices of an operand as BF16 integers, written tile by tile in the
//             tensor core's canonical K-major layout (no swizzle: 8 x 8 core matrices of
//             128 contiguous bytes, K-adjacent core matrices 128 B apart, 8-row groups
//             1024 B apart), so that one 128 x 64 tile is one contiguous 16 KiB block;
//   k_gemm_tc one CTA per 128 x 128 tile of C, warp-specialised: warp 0 streams the
//             A/B slice tiles into a 4-stage shared-memory ring with 1-D bulk async
//             copies (cp.async.bulk, completion on mbarriers); warp 1 allocates 256 TMEM
//             columns and issues tcgen05.mma (M = 128, N = 128, K = 16, BF16 in, FP32 out)
//             into one of two TMEM accumulators per (slice pair, K-chunk); warps 2-9 drain
//             the other accumulator with tcgen05.ld and add it into FP64 registers, so the
//             FP64 accumulation overlaps the next product.  Every wait is bounded: a
//             timeout sets the error word, the CTA drains its copies in flight, frees its
//             TMEM and exits.
#include <cstdint>
#include <cuda_bf16.h>

#include "gs_internal.h"
#include "tc_common.cuh"

namespace gsk {
namespace {

constexpr int kTcBeta = 6;        // bits per slice
constexpr int kTcSlices = 10;     // slices per operand (60 bits)
constexpr int kTcBM = 128;        // tile rows (M and N)
constexpr int kTcBK = 64;         // k per stage (one 128-byte core-matrix row pair x 4)
constexpr int kTcChunkBlocks = 64;  // k-blocks per exact chunk: 64 x 64 = 4096
constexpr int kTcStages = 4;
constexpr int kTcTileElems = kTcBM * kTcBK;            // 8192 bf16
constexpr int kTcTileBytes = kTcTileElems * 2;         // 16 KiB
constexpr int kTcThreads = 320;                        // 10 warps
constexpr int kTcEpiWarps = 8;
constexpr int kTcMaxPairs = 64;
constexpr int kExpZero = -100000;  // row of zeros
constexpr int kExpBad = 100000;    // row with Inf/NaN
constexpr unsigned long long kTcTimeoutCycles = 4000000000ull;  // ~2 s at 2 GHz

// --------------------------------------------------------------------------------------
// operand access: element (r, k) of an operand whose rows are the M (or N) index of C
// and whose columns run along the contraction.  tr = 0: column-major X with (r, k) at
// k * ld + r (op(A) = A); tr = 1: (r, k) at r * ld + k (op(A) = A^T, and B seen by its
// columns).
// --------------------------------------------------------------------------------------

template <int TR>
__global__ void __launch_bounds__(256) k_absmax(int R, int K, const double* __restrict__ X, int ld,
                                                unsigned long long* __restrict__ out) {
  const int r0 = blockIdx.x * 64, k0 = blockIdx.y * 256;
  const int kend = min(K, k0 + 256);
  if (TR == 0) {
    __shared__ unsigned long long red[4][64];
    const int rr = threadIdx.x % 64, kk = threadIdx.x / 64;
    const int r = r0 + rr;
    unsigned long long m = 0;
    if (r < R)
      for (int k = k0 + kk; k < kend; k += 4) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(X[(size_t)k * ld + r]));
        m = b > m ? b : m;
      }
    red[kk][rr] = m;
    __syncthreads();
    if (kk == 0 && r < R) {
      for (int x = 1; x < 4; ++x) m = red[x][rr] > m ? red[x][rr] : m;
      if (m) atomicMax(out + r, m);
    }
  } else {
    const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (int rr = w; rr < 64; rr += 8) {
      const int r = r0 + rr;
      if (r >= R) break;
      unsigned long long m = 0;
      for (int k = k0 + lane; k < kend; k += 32) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(X[(size_t)r * ld + k]));
        m = b > m ? b : m;
      }
      for (int o = 16; o; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, m, o);
        m = y > m ? y : m;
      }
      if (lane == 0 && m) atomicMax(out + r, m);
    }
  }
}

__global__ void k_exps(int R, const unsigned long long* __restrict__ amax, int* __restrict__ ex) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const double a = __longlong_as_double((long long)amax[r]);
  int e;
  if (a == 0.0) e = kExpZero;
  else if (!(a <= 1.7976931348623157e308)) e = kExpBad;
  else {
    frexp(a, &e);  // a = f 2^e, f in [0.5, 1): a < 2^e
  }
  ex[r] = e;
}

// |x| 2^(60 - e) truncated to an integer (|x| < 2^e, so below 2^60), from the IEEE bits:
// the 53-bit significand shifted by its exponent.  The 6-bit groups of this integer are
// exactly the successive truncations trunc(y 64^s) mod 64 of y = |x| 2^-e.
__device__ __forceinline__ unsigned long long fixed60(double x, int e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
  const int be = (int)(b >> 52);
  if (be == 0 && (b & 0xfffffffffffffull) == 0) return 0ull;
  const unsigned long long m = (b & 0xfffffffffffffull) | (be ? (1ull << 52) : 0ull);
  const int ex = be ? be - 1075 : -1074;  // x = m 2^ex
  const int sh = ex + 60 - e;             // <= 7
  if (sh >= 0) return m << sh;
  return sh <= -64 ? 0ull : (m >> (-sh));
}

// BF16 bits of the integer q (|q| < 64) with the given sign.
__device__ __forceinline__ unsigned short bf16_int(unsigned q, unsigned neg) {
  if (q == 0u) return 0;
  const int p = 31 - __clz(q);
  return (unsigned short)((neg << 15) | ((unsigned)(127 + p) << 7) | ((q << (7 - p)) & 0x7fu));
}

// Slices of rows [128 rb, 128 rb + 128) x k [64 kb, 64 kb + 64): one CTA per tile, each
// thread one (row, 8-k group) item at a time -> one 16-byte core-matrix row per slice.
// Integer arithmetic only (the FP64 pipe is the scarce resource on this part).
template <int TR>
__global__ void __launch_bounds__(256) k_split(int R, int K, const double* __restrict__ X, int ld,
                                               const int* __restrict__ ex, int Rt, int Kt,
                                               __nv_bfloat16* __restrict__ out) {
  const int rb = blockIdx.x, kb = blockIdx.y;
  const size_t slice_stride = (size_t)Rt * Kt * kTcTileElems;
  __nv_bfloat16* tile = out + ((size_t)rb * Kt + kb) * kTcTileElems;
  for (int it = threadIdx.x; it < kTcBM * (kTcBK / 8); it += 256) {
    const int rl = it % kTcBM, kg = it / kTcBM;
    const int r = rb * kTcBM + rl, kbase = kb * kTcBK + kg * 8;
    unsigned long long f[8];
    unsigned neg[8];
    int e = kExpZero;
    if (r < R) e = ex[r];
    const bool live = (e != kExpZero && e != kExpBad);
#pragma unroll
    for (int x = 0; x < 8; ++x) {
      const int k = kbase + x;
      double v = 0.0;
      if (live && k < K) v = TR ? X[(size_t)r * ld + k] : X[(size_t)k * ld + r];
      f[x] = live ? fixed60(v, e) : 0ull;
      neg[x] = (unsigned)(((unsigned long long)__double_as_longlong(v)) >> 63);
    }
    const size_t off = (size_t)((rl >> 3) * 8 + kg) * 64 + (rl & 7) * 8;
#pragma unroll 1
    for (int s = 0; s < kTcSlices; ++s) {
      const int sh = 60 - kTcBeta * (s + 1);
      unsigned w[4];
#pragma unroll
      for (int x = 0; x < 4; ++x) {
        const unsigned lo = bf16_int((unsigned)(f[2 * x] >> sh) & 63u, neg[2 * x]);
        const unsigned hi = bf16_int((unsigned)(f[2 * x + 1] >> sh) & 63u, neg[2 * x + 1]);
        w[x] = lo | (hi << 16);
      }
      *reinterpret_cast<uint4*>(tile + s * slice_stride + off) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// tcgen05 / mbarrier / bulk-copy primitives: tc_common.cuh
using namespace tc;

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  return tc::mbar_wait(bar, parity, kTcTimeoutCycles);
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, N = 128, M = 128.
constexpr uint32_t kTcIdesc = idesc_bf16(kTcBM, kTcBM);

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accum) {
  tc::tc_mma(dtmem, adesc, bdesc, kTcIdesc, accum);
}

struct TcPairs {
  int npairs;
  unsigned char s[kTcMaxPairs], t[kTcMaxPairs];  // 0-based slice indices, least significant first
};

struct TcArgs {
  int m, p, Rt, Ct, Kt, nchunks;
  const __nv_bfloat16* As;  // slices of op(A): [S][Rt][Kt] tiles
  const __nv_bfloat16* Bs;  // slices of B (by columns): [S][Ct][Kt] tiles
  const int* exA;
  const int* exB;
  double* C;
  int ldc;
  int* err;
};

__global__ void __launch_bounds__(kTcThreads, 1) k_gemm_tc(TcArgs a, TcPairs pr) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* ring = smem;  // kTcStages x (A tile, B tile)
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kTcStages * 2 * kTcTileBytes);
  uint64_t* empty = full + kTcStages;
  uint64_t* accf = empty + kTcStages;
  uint64_t* acce = accf + 2;
  uint64_t* done = acce + 2;  // all MMAs of the CTA complete (before TMEM is freed)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int rb = blockIdx.x % a.Rt, cb = blockIdx.x / a.Rt;
  const int nunits = pr.npairs * a.nchunks;

  if (threadIdx.x == 0) {
    for (int i = 0; i < kTcStages; ++i) {
      mbar_init(full + i, 1);
      mbar_init(empty + i, 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(accf + i, 1);
      mbar_init(acce + i, kTcEpiWarps);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(tslot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  const size_t sliceA = (size_t)a.Rt * a.Kt * kTcTileElems, sliceB = (size_t)a.Ct * a.Kt * kTcTileElems;

  if (warp == 0) {
    // ---- producer
    if (lane == 0) {
      int it = 0;
      int last_fill[kTcStages];
      for (int i = 0; i < kTcStages; ++i) last_fill[i] = -1;
      bool ok = true;
      for (int u = 0; u < nunits && ok; ++u) {
        const int pi = u / a.nchunks, c = u % a.nchunks;
        const __nv_bfloat16* Ab = a.As + pr.s[pi] * sliceA + (size_t)rb * a.Kt * kTcTileElems;
        const __nv_bfloat16* Bb = a.Bs + pr.t[pi] * sliceB + (size_t)cb * a.Kt * kTcTileElems;
        const int kb0 = c * kTcChunkBlocks, kb1 = min(a.Kt, kb0 + kTcChunkBlocks);
        for (int kb = kb0; kb < kb1; ++kb, ++it) {
          const int st = it % kTcStages;
          const uint32_t ph = (uint32_t)(it / kTcStages) & 1u;
          if (*abort_flag || !mbar_wait(empty + st, ph ^ 1u)) { ok = false; break; }
          unsigned char* dA = ring + st * 2 * kTcTileBytes;
          mbar_expect_tx(full + st, 2 * kTcTileBytes);
          bulk_g2s(dA, Ab + (size_t)kb * kTcTileElems, kTcTileBytes, full + st);
          bulk_g2s(dA + kTcTileBytes, Bb + (size_t)kb * kTcTileElems, kTcTileBytes, full + st);
          last_fill[st] = it;
        }
      }
      if (!ok) { *abort_flag = 1; atomicExch(a.err, 1); }
      // drain: every copy issued must have landed before the CTA exits
      for (int i = 0; i < kTcStages; ++i)
        if (last_fill[i] >= 0 && !mbar_wait(full + i, (uint32_t)(last_fill[i] / kTcStages) & 1u)) atomicExch(a.err, 2);
    }
  } else if (warp == 1) {
    // ---- MMA issuer
    if (lane == 0) {
      int it = 0;
      bool ok = true;
      const uint32_t ring0 = smem_u32(ring);
      for (int u = 0; u < nunits && ok; ++u) {
        const int b = u & 1;
        const uint32_t aph = (uint32_t)(u >> 1) & 1u;
        if (*abort_flag || !mbar_wait(acce + b, aph ^ 1u)) { ok = false; break; }
        tc_fence_after();
        const int c = u % a.nchunks;
        const int kb0 = c * kTcChunkBlocks, kb1 = min(a.Kt, kb0 + kTcChunkBlocks);
        for (int kb = kb0; kb < kb1; ++kb, ++it) {
          const int st = it % kTcStages;
          const uint32_t ph = (uint32_t)(it / kTcStages) & 1u;
          if (*abort_flag || !mbar_wait(full + st, ph)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sa = ring0 + st * 2 * kTcTileBytes, sb = sa + kTcTileBytes;
#pragma unroll
          for (int j = 0; j < kTcBK / 16; ++j)
            tc_mma(tmem + b * kTcBM, smem_desc(sa + j * 256, 128, 1024), smem_desc(sb + j * 256, 128, 1024),
                   (kb > kb0 || j > 0) ? 1u : 0u);
          tc_commit(empty + st);
        }
        if (!ok) break;
        tc_commit(accf + b);
      }
      if (!ok) { *abort_flag = 1; atomicExch(a.err, 3); }
      // every MMA issued must have completed before the accumulators are freed
      tc_commit(done);
      if (!mbar_wait(done, 0)) atomicExch(a.err, 5);
    }
  } else {
    // ---- epilogue: warps 2..9; TMEM lane quarter = warp % 4, column half = (warp - 2) / 4
    const int q = warp & 3, h = (warp - 2) >> 2;
    double acc[64];
#pragma unroll
    for (int c = 0; c < 64; ++c) acc[c] = 0.0;
    bool ok = true;
    for (int u = 0; u < nunits; ++u) {
      const int b = u & 1;
      const uint32_t aph = (uint32_t)(u >> 1) & 1u;
      if (*abort_flag || !mbar_wait(accf + b, aph)) { ok = false; break; }
      tc_fence_after();
      const int pi = u / a.nchunks;
      const double sc = ldexp(1.0, -kTcBeta * (pr.s[pi] + pr.t[pi] + 2));
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + b * kTcBM + h * 64;
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        uint32_t v[16];
        tc_ld16(tbase + g * 16, v);
        tc_wait_ld();
#pragma unroll
        for (int x = 0; x < 16; ++x) acc[g * 16 + x] = fma((double)__uint_as_float(v[x]), sc, acc[g * 16 + x]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce + b);
    }
    if (!ok) {
      *abort_flag = 1;
      if (lane == 0) atomicExch(a.err, 4);
    } else {
      const int i = rb * kTcBM + q * 32 + lane;
      if (i < a.m) {
        const int ei = a.exA[i];
#pragma unroll
        for (int c = 0; c < 64; ++c) {
          const int j = cb * kTcBM + h * 64 + c;
          if (j < a.p) {
            const int fj = a.exB[j];
            double r;
            if (ei == kExpBad || fj == kExpBad) r = __longlong_as_double(0x7ff8000000000000ll);
            else if (ei == kExpZero || fj == kExpZero) r = 0.0;
            else r = ldexp(acc[c], ei + fj);
            a.C[(size_t)j * a.ldc + i] = r;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
}

constexpr size_t kTcSmem = (size_t)kTcStages * 2 * kTcTileBytes + 8 * (2 * kTcStages + 5) + 16;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

size_t gemm_tc_ws_bytes(int m, int p, int q) {
  const size_t Rt = (m + kTcBM - 1) / kTcBM, Ct = (p + kTcBM - 1) / kTcBM, Kt = (q + kTcBK - 1) / kTcBK;
  size_t b = 0;
  b += align256(kTcSlices * Rt * Kt * (size_t)kTcTileBytes);
  b += align256(kTcSlices * Ct * Kt * (size_t)kTcTileBytes);
  b += align256(8 * (size_t)(m + p));
  b += align256(4 * (size_t)(m + p));
  b += 256;
  return b;
}

cudaError_t launch_gemm_tc(int m, int p, int q, const double* A, int lda, int transA, const double* B, int ldb,
                           double* C, int ldc, void* ws, cudaStream_t s) {
  if (m <= 0 || p <= 0) return cudaSuccess;
  const int Rt = (m + kTcBM - 1) / kTcBM, Ct = (p + kTcBM - 1) / kTcBM;
  const int Kt = q > 0 ? (q + kTcBK - 1) / kTcBK : 1;
  char* w = static_cast<char*>(ws);
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(w);
  w += align256(kTcSlices * (size_t)Rt * Kt * kTcTileBytes);
  __nv_bfloat16* Bs = reinterpret_cast<__nv_bfloat16*>(w);
  w += align256(kTcSlices * (size_t)Ct * Kt * kTcTileBytes);
  unsigned long long* amax = reinterpret_cast<unsigned long long*>(w);
  w += align256(8 * (size_t)(m + p));
  int* ex = reinterpret_cast<int*>(w);
  w += align256(4 * (size_t)(m + p));
  int* err = reinterpret_cast<int*>(w);
  cudaError_t e = cudaMemsetAsync(amax, 0, 8 * (size_t)(m + p), s);
  if (e != cudaSuccess) return e;
  if (q > 0) {
    dim3 ga((m + 63) / 64, (q + 255) / 256), gb((p + 63) / 64, (q + 255) / 256);
    if (transA) k_absmax<1><<<ga, 256, 0, s>>>(m, q, A, lda, amax);
    else k_absmax<0><<<ga, 256, 0, s>>>(m, q, A, lda, amax);
    k_absmax<1><<<gb, 256, 0, s>>>(p, q, B, ldb, amax + m);
  }
  k_exps<<<(m + p + 255) / 256, 256, 0, s>>>(m + p, amax, ex);
  if (transA) k_split<1><<<dim3(Rt, Kt), 256, 0, s>>>(m, q, A, lda, ex, Rt, Kt, As);
  else k_split<0><<<dim3(Rt, Kt), 256, 0, s>>>(m, q, A, lda, ex, Rt, Kt, As);
  k_split<1><<<dim3(Ct, Kt), 256, 0, s>>>(p, q, B, ldb, ex + m, Ct, Kt, Bs);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  TcPairs pr{};
  for (int L = 2 * kTcSlices; L >= 2; --L)  // least significant level first
    for (int si = 1; si <= kTcSlices; ++si) {
      const int ti = L - si;
      if (ti < 1 || ti > kTcSlices || si + ti > kTcSlices + 1) continue;
      pr.s[pr.npairs] = (unsigned char)(si - 1);
      pr.t[pr.npairs] = (unsigned char)(ti - 1);
      ++pr.npairs;
    }
  TcArgs a{};
  a.m = m; a.p = p; a.Rt = Rt; a.Ct = Ct; a.Kt = Kt;
  a.nchunks = (Kt + kTcChunkBlocks - 1) / kTcChunkBlocks;
  a.As = As; a.Bs = Bs; a.exA = ex; a.exB = ex + m; a.C = C; a.ldc = ldc; a.err = err;
  e = cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
  if (e != cudaSuccess) return e;
  k_gemm_tc<<<Rt * Ct, kTcThreads, kTcSmem, s>>>(a, pr);
  return cudaGetLastError();
}

int* gemm_tc_err_word(int m, int p, int q, void* ws) {
  const int Rt = (m + kTcBM - 1) / kTcBM, Ct = (p + kTcBM - 1) / kTcBM;
  const int Kt = q > 0 ? (q + kTcBK - 1) / kTcBK : 1;
  char* w = static_cast<char*>(ws);
  w += align256(kTcSlices * (size_t)Rt * Kt * kTcTileBytes);
  w += align256(kTcSlices * (size_t)Ct * Kt * kTcTileBytes);
  w += align256(8 * (size_t)(m + p));
  w += align256(4 * (size_t)(m + p));
  return reinterpret_cast<int*>(w);
}

}  // namespace gsk
