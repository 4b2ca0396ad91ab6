// Device code of one bin of the mixed-precision batched real Schur refinement
// (refine_batched.cu describes the method): CTA matrix products, the block Sylvester
// waves, the per-matrix Newton loop and the bin kernel.  Included only by the per-bin
// translation units (refine_bin_r*.cu), so that each compiles one row tile.
#pragma once
#include <cstdlib>
#include "refine_batched.cuh"

namespace gsk {
namespace {

constexpr int kRT = 256;          // threads per CTA (16 x 16 product layout)
constexpr int kKC = 16;           // contraction chunk staged in shared memory
constexpr int kAS = kSmallMax + 4;  // staged op(A) chunk: kKC rows of up to 128 entries
constexpr int kNC = 2;            // columns per thread in one pass
constexpr int kPW = 16 * kNC;     // columns per pass
constexpr int kBS = kPW + 4;      // staged B chunk: kKC rows of kPW entries
constexpr float kMinGain = 4.f;    // from the third step on, a step must shrink max|X| this much
constexpr float kTolFinal = 1e-9f;
constexpr float kTolDiverge = 1e-1f;

struct Smem {
  double a[kKC * kAS];
  double b[kKC * kBS];
  float red[3][kRT / 32];
  double rot[2];
  short bs[kSmallMax + 2];
  unsigned char bid[kSmallMax];
  int nblk;
  int ticket;
};

__device__ __forceinline__ float nanmax(float m, float v) { return (v > m || v != v) ? v : m; }

// max over the CTA of three per-thread values (NaN propagates)
__device__ void cta_max3(float& x, float& y, float& z, Smem& sm) {
  for (int o = 16; o > 0; o >>= 1) {
    x = nanmax(x, __shfl_xor_sync(0xffffffffu, x, o));
    y = nanmax(y, __shfl_xor_sync(0xffffffffu, y, o));
    z = nanmax(z, __shfl_xor_sync(0xffffffffu, z, o));
  }
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { sm.red[0][w] = x; sm.red[1][w] = y; sm.red[2][w] = z; }
  __syncthreads();
  x = sm.red[0][0]; y = sm.red[1][0]; z = sm.red[2][0];
  for (int i = 1; i < kRT / 32; ++i) {
    x = nanmax(x, sm.red[0][i]); y = nanmax(y, sm.red[1][i]); z = nanmax(z, sm.red[2][i]);
  }
}

// ------------------------------------------------------------------------------------
// CTA matrix product C (n x ncols) = sum_{k < kdim} opA(i, k) B(k, j), computed in CT.
// Threads form a 16 x 16 grid; in each pass over kPW columns [j0, j0 + kPW) thread
// (tx, ty) owns rows rb + tx + 16 r (r < RMP) and columns j0 + ty + 16 c (c < kNC) (the
// FP64 pipe, not the register tile, bounds the FP64 products, so the tile stays small
// and nothing spills).  Chunks of kKC contraction indices are staged in shared memory
// (zero beyond n / kdim); the loaders say whether consecutive k are contiguous in memory
// (kfast), which picks the coalesced staging order.  The store functor receives every
// (i, j, value) with i < n, j < ncols of the pass's rows.
// PART 0: all rows; PART 1: rows from the 16-row group holding j0 down (covers i >= j);
// PART 2: rows up to j0 + kPW (covers i <= j + 1), so that a triangle costs about half.
// ------------------------------------------------------------------------------------
template <int RMP, class CT, class LA, class LB, class ST>
__device__ void mm_pass(int n, int ncols, int kdim, int rb, int j0, const LA& la, const LB& lb, const ST& st,
                        Smem& sm) {
  CT* sa = reinterpret_cast<CT*>(sm.a);
  CT* sb = reinterpret_cast<CT*>(sm.b);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int nrow = RMP * 16;
  const int cm = min(kNC, (ncols - j0 + 15) >> 4);
  CT acc[RMP][kNC];
#pragma unroll
  for (int r = 0; r < RMP; ++r)
#pragma unroll
    for (int c = 0; c < kNC; ++c) acc[r][c] = CT(0);
  for (int k0 = 0; k0 < kdim; k0 += kKC) {
    __syncthreads();
    if (la.kfast(k0)) {
      for (int e = tid; e < kKC * nrow; e += kRT) {
        const int kk = e & (kKC - 1), i = rb + (e >> 4), k = k0 + kk;
        sa[kk * kAS + (i - rb)] = (i < n && k < kdim) ? la(i, k) : CT(0);
      }
    } else {
      for (int e = tid; e < kKC * nrow; e += kRT) {
        const int kk = e / nrow, ii = e - kk * nrow, i = rb + ii, k = k0 + kk;
        sa[kk * kAS + ii] = (i < n && k < kdim) ? la(i, k) : CT(0);
      }
    }
    if (lb.kfast(k0)) {
      for (int e = tid; e < kKC * kPW; e += kRT) {
        const int kk = e & (kKC - 1), jj = e >> 4, j = j0 + jj, k = k0 + kk;
        sb[kk * kBS + jj] = (j < ncols && k < kdim) ? lb(k, j) : CT(0);
      }
    } else {
      for (int e = tid; e < kKC * kPW; e += kRT) {
        const int kk = e / kPW, jj = e % kPW, j = j0 + jj, k = k0 + kk;
        sb[kk * kBS + jj] = (j < ncols && k < kdim) ? lb(k, j) : CT(0);
      }
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < kKC; ++kk) {
      CT av[RMP], bv[kNC];
#pragma unroll
      for (int r = 0; r < RMP; ++r) av[r] = sa[kk * kAS + tx + 16 * r];
#pragma unroll
      for (int c = 0; c < kNC; ++c) bv[c] = sb[kk * kBS + ty + 16 * c];
      if (cm == kNC) {
#pragma unroll
        for (int r = 0; r < RMP; ++r)
#pragma unroll
          for (int c = 0; c < kNC; ++c) acc[r][c] = fma(av[r], bv[c], acc[r][c]);
      } else {
#pragma unroll
        for (int r = 0; r < RMP; ++r) acc[r][0] = fma(av[r], bv[0], acc[r][0]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < RMP; ++r)
#pragma unroll
    for (int c = 0; c < kNC; ++c) {
      const int i = rb + tx + 16 * r, j = j0 + ty + 16 * c;
      if (i < n && j < ncols) st(i, j, acc[r][c]);
    }
}

template <int RM, int PART, class CT, class LA, class LB, class ST>
__device__ void cta_mm(int n, int ncols, int kdim, const LA& la, const LB& lb, const ST& st, Smem& sm) {
  for (int j0 = 0; j0 < ncols; j0 += kPW) {
    if constexpr (PART == 0) {
      mm_pass<RM, CT>(n, ncols, kdim, 0, j0, la, lb, st, sm);
    } else {
      const int rb = PART == 1 ? (j0 & ~15) : 0;
      const int re = PART == 1 ? n : min(n, j0 + kPW + 1);
      const int rm = (((re - rb + 15) >> 4) + 1) & ~1;  // even row-group counts only
      switch (rm) {
        case 2: mm_pass<2, CT>(n, ncols, kdim, rb, j0, la, lb, st, sm); break;
        case 4: if constexpr (RM >= 4) mm_pass<4, CT>(n, ncols, kdim, rb, j0, la, lb, st, sm); break;
        case 6: if constexpr (RM >= 6) mm_pass<6, CT>(n, ncols, kdim, rb, j0, la, lb, st, sm); break;
        default: if constexpr (RM >= 8) mm_pass<8, CT>(n, ncols, kdim, rb, j0, la, lb, st, sm); break;
      }
    }
  }
  __syncthreads();
}

// loaders: element (i, k) of op(A) or (k, j) of B over column-major n x n storage
template <class S, class CT>
struct LdN {  // X(r, c), column-major: contiguous along r
  const S* p; int n; CT s;
  __device__ CT operator()(int r, int c) const { return (CT)p[(size_t)c * n + r] * s; }
  __device__ bool kfast(int) const { return false; }
};
template <class S, class CT>
struct LdNB {  // B operand X(k, j), column-major: contiguous along k
  const S* p; int n;
  __device__ CT operator()(int k, int j) const { return (CT)p[(size_t)j * n + k]; }
  __device__ bool kfast(int) const { return true; }
};
template <class S, class CT>
struct LdT {  // X^T(i, k) = X(k, i): contiguous along k
  const S* p; int n;
  __device__ CT operator()(int i, int k) const { return (CT)p[(size_t)i * n + k]; }
  __device__ bool kfast(int) const { return true; }
};
// [X1 | X2](i, k) with k < n from X1, else from X2 (both column-major, or X1 transposed)
struct LdCatA {
  const float* x1; bool t1; const float* x2; int n;
  __device__ float operator()(int i, int k) const {
    if (k < n) return t1 ? x1[(size_t)i * n + k] : x1[(size_t)k * n + i];
    return x2[(size_t)(k - n) * n + i];
  }
  __device__ bool kfast(int k0) const { return k0 < n && t1; }
};
// [Y1; Y2](k, j), both column-major
struct LdCatB {
  const float* y1; const float* y2; int n;
  __device__ float operator()(int k, int j) const {
    return k < n ? y1[(size_t)j * n + k] : y2[(size_t)j * n + (k - n)];
  }
  __device__ bool kfast(int) const { return true; }
};

// Solve the m x m system K x = r (m <= 4) by Gaussian elimination with partial pivoting;
// pivots below `floor` in magnitude are replaced by +-floor (bounded correction for
// eigenvalues that FP32 does not separate; the step then fails the tolerance).
__device__ void small_solve4(int m, float K[4][4], float r[4], float floor) {
  for (int c = 0; c < m; ++c) {
    int piv = c;
    for (int i = c + 1; i < m; ++i)
      if (fabsf(K[i][c]) > fabsf(K[piv][c])) piv = i;
    if (piv != c) {
      for (int j = 0; j < 4; ++j) { const float t = K[c][j]; K[c][j] = K[piv][j]; K[piv][j] = t; }
      const float t = r[c]; r[c] = r[piv]; r[piv] = t;
    }
    if (fabsf(K[c][c]) < floor) K[c][c] = K[c][c] < 0.f ? -floor : floor;
    for (int i = c + 1; i < m; ++i) {
      const float f = K[i][c] / K[c][c];
      for (int j = c; j < m; ++j) K[i][j] -= f * K[c][j];
      r[i] -= f * r[c];
    }
  }
  for (int c = m - 1; c >= 0; --c) {
    float s = r[c];
    for (int j = c + 1; j < m; ++j) s -= K[c][j] * r[j];
    r[c] = s / K[c][c];
  }
}

// Block-lower W from T (block-upper part of Tf) and the right-hand sides R (block-lower
// entries of R), by waves D = p - q = N-1 .. 1: block pair (p, q) needs W_rq, r > p, and
// W_pr, r < q, all of larger D.
__device__ void sylv_waves(int n, int N, const short* bs, const float* Tf, const float* R, float* W, float floor) {
  for (int D = N - 1; D >= 1; --D) {
    for (int q = threadIdx.x; q < N - D; q += kRT) {
      const int p = q + D;
      const int i0 = bs[p], ip = bs[p + 1] - i0, j0 = bs[q], jq = bs[q + 1] - j0;
      float r00 = R[(size_t)j0 * n + i0];
      float r10 = ip == 2 ? R[(size_t)j0 * n + i0 + 1] : 0.f;
      float r01 = jq == 2 ? R[(size_t)(j0 + 1) * n + i0] : 0.f;
      float r11 = (ip == 2 && jq == 2) ? R[(size_t)(j0 + 1) * n + i0 + 1] : 0.f;
      // The two sums run in k order; their loads are issued kU at a time, so that the
      // L1/L2 latency is paid once per kU terms rather than once per term.
      constexpr int kU = 8;
      const float* Ti0 = Tf + i0;       // row i0 of T: stride n
      const float* Wj0 = W + (size_t)j0 * n;
      int k = i0 + ip;
      for (; k + kU <= n; k += kU) {  // - sum_{r>p} T_pr W_rq
        float t0[kU], t1[kU], w0[kU], w1[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          t0[u] = Ti0[(size_t)(k + u) * n];
          t1[u] = ip == 2 ? Ti0[(size_t)(k + u) * n + 1] : 0.f;
          w0[u] = Wj0[k + u];
          w1[u] = jq == 2 ? Wj0[n + k + u] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          r00 -= t0[u] * w0[u]; r01 -= t0[u] * w1[u]; r10 -= t1[u] * w0[u]; r11 -= t1[u] * w1[u];
        }
      }
      for (; k < n; ++k) {
        const float t0 = Ti0[(size_t)k * n], t1 = ip == 2 ? Ti0[(size_t)k * n + 1] : 0.f;
        const float w0 = Wj0[k], w1 = jq == 2 ? Wj0[n + k] : 0.f;
        r00 -= t0 * w0; r01 -= t0 * w1; r10 -= t1 * w0; r11 -= t1 * w1;
      }
      const float* Tj0 = Tf + (size_t)j0 * n;  // column j0 of T
      const float* Wi0 = W + i0;               // row i0 of W: stride n
      k = 0;
      for (; k + kU <= j0; k += kU) {  // + sum_{r<q} W_pr T_rq
        float w0[kU], w1[kU], t0[kU], t1[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          w0[u] = Wi0[(size_t)(k + u) * n];
          w1[u] = ip == 2 ? Wi0[(size_t)(k + u) * n + 1] : 0.f;
          t0[u] = Tj0[k + u];
          t1[u] = jq == 2 ? Tj0[n + k + u] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          r00 += w0[u] * t0[u]; r01 += w0[u] * t1[u]; r10 += w1[u] * t0[u]; r11 += w1[u] * t1[u];
        }
      }
      for (; k < j0; ++k) {
        const float w0 = Wi0[(size_t)k * n], w1 = ip == 2 ? Wi0[(size_t)k * n + 1] : 0.f;
        const float t0 = Tj0[k], t1 = jq == 2 ? Tj0[n + k] : 0.f;
        r00 += w0 * t0; r01 += w0 * t1; r10 += w1 * t0; r11 += w1 * t1;
      }
      // (I_q (x) T_pp - T_qq^T (x) I_p) vec(W_pq) = vec(R), vec index a + ip * b
      const int m = ip * jq;
      float K[4][4], rv[4];
      const float rr[2][2] = {{r00, r01}, {r10, r11}};
      for (int u = 0; u < 4; ++u)
        for (int v = 0; v < 4; ++v) K[u][v] = 0.f;
      for (int b = 0; b < jq; ++b)
        for (int a = 0; a < ip; ++a) {
          const int row = a + ip * b;
          rv[row] = rr[a][b];
          for (int a2 = 0; a2 < ip; ++a2) K[row][a2 + ip * b] += Tf[(size_t)(i0 + a2) * n + i0 + a];
          for (int b2 = 0; b2 < jq; ++b2) K[row][a + ip * b2] -= Tf[(size_t)(j0 + b) * n + j0 + b2];
        }
      small_solve4(m, K, rv, floor);
      for (int b = 0; b < jq; ++b)
        for (int a = 0; a < ip; ++a) W[(size_t)(j0 + b) * n + i0 + a] = rv[a + ip * b];
    }
    __syncthreads();
  }
}


// One Newton step of one matrix: At = Z^T A_s Z and N = (I - Z^T Z) / 2 were formed by
// the tensor-core products of this step (Q in FP64, its FP32 copy in T32, N in NF).
template <int RM>
__device__ void refine_step(const RefineArgs& a, int b, int n, int step, Smem& sm) {
  const int tid = threadIdx.x;
  const long long off = a.offs[b];
  double* A = a.A + off;
  double* Z = a.Z + off;
  double* P = a.P + off;
  double* Q = a.Q + off;
  float* AtF = a.T32 + off;
  float* ZF = a.Z32 + off;
  float* M = a.M + off;
  float* W = a.W + off;
  float* NF = a.NF + off;
  const int nn = n * n;
  const int e = a.exps[b];
  const double usc = ldexp(1.0, e);
  // 1x1 / 2x2 block structure of the FP32 Schur form
  if (tid == 0) {
    const unsigned char* blk = a.blk + a.woffs[b];
    int N = 0, i = 0;
    while (i < n) {
      sm.bs[N++] = (short)i;
      i += (i + 1 < n && blk[i]) ? 2 : 1;
    }
    sm.bs[N] = (short)n;
    sm.nblk = N;
  }
  __syncthreads();
  const int N = sm.nblk;
  for (int p = tid; p < N; p += kRT)
    for (int i = sm.bs[p]; i < sm.bs[p + 1]; ++i) sm.bid[i] = (unsigned char)p;
  __syncthreads();
  const unsigned char* bid = sm.bid;
  const int steps = step + 1;
  bool ok = false, fail = false;
  {
    float tnorm = 0.f, dummy0 = 0.f, dummy1 = 0.f;
    for (int idx = tid; idx < nn; idx += kRT) tnorm = nanmax(tnorm, fabsf(AtF[idx]));
    cta_max3(tnorm, dummy0, dummy1, sm);
    // M = N At + At N (FP32), then the right-hand sides -(L + M) on the block-lower part
    cta_mm<RM, 0, float>(n, n, 2 * n, LdCatA{NF, false, AtF, n}, LdCatB{AtF, NF, n},
                      [&](int i, int j, float v) { M[(size_t)j * n + i] = v; }, sm);
    for (int idx = tid; idx < nn; idx += kRT) {
      const int i = idx % n, j = idx / n;
      if (bid[i] > bid[j]) M[idx] = -(AtF[idx] + M[idx]);
    }
    __syncthreads();
    const float floor = 8.f * 1.2e-7f * (tnorm > 0.f ? tnorm : 1.f);
    sylv_waves(n, N, sm.bs, AtF, M, W, floor);
    // X = N + W - W^T (W block-lower); each block-lower entry's thread writes its mirror
    float xmax = 0.f;
    for (int idx = tid; idx < nn; idx += kRT) {
      const int i = idx % n, j = idx / n;
      if (bid[i] > bid[j]) {
        const float w = W[idx];
        const float x1 = NF[idx] + w, x2 = NF[(size_t)i * n + j] - w;
        W[idx] = x1;
        W[(size_t)i * n + j] = x2;
        xmax = nanmax(xmax, fmaxf(fabsf(x1), fabsf(x2)));
      } else if (bid[i] == bid[j]) {
        W[idx] = NF[idx];
        xmax = nanmax(xmax, fabsf(NF[idx]));
      }
    }
    float d2 = 0.f, d3 = 0.f;
    cta_max3(xmax, d2, d3, sm);
    const float xprev = step > 0 ? a.xprev[b] : 0.f;
    if (!(xmax <= kTolDiverge)) {
      fail = true;
    } else {
      ok = xmax <= kTolFinal;
      if (!ok && (step >= 2 && xmax * kMinGain > xprev)) fail = true;  // stagnating: hand back
      if (!ok && step == kRefineSteps - 1) fail = true;                 // out of steps
    }
    if (!ok && !fail && tid == 0) a.xprev[b] = xmax;
  }
  if (!fail) {
    if (ok) {
      // T = At + X^T At + At X (unit scale; At in FP64 from the tensor-core product), block-lower part zero, into A
      cta_mm<RM, 0, float>(n, n, 2 * n, LdCatA{W, true, AtF, n}, LdCatB{AtF, W, n},
                        [&](int i, int j, float v) {
                          A[(size_t)j * n + i] = bid[i] > bid[j] ? 0.0 : Q[(size_t)j * n + i] + (double)v;
                        },
                        sm);
    }
    // Z <- Z + Z X (product in FP32), through P
    cta_mm<RM, 0, float>(n, n, n, LdN<float, float>{ZF, n, 1.f}, LdNB<float, float>{W, n},
                      [&](int i, int j, float v) { P[(size_t)j * n + i] = Z[(size_t)j * n + i] + (double)v; }, sm);
    for (int idx = tid; idx < nn; idx += kRT) {
      const double z = P[idx];
      Z[idx] = z;
      ZF[idx] = (float)z;
    }
    __syncthreads();
    if (!ok) refine_col_exps<kRT>(n, Z, a.exZ + a.woffs[b]);  // for the next step's products
  }
  const unsigned long long n3 = (unsigned long long)n * n * n;
  if (fail) {
    if (tid == 0) {
      a.status[b] = a.nofallback ? ST_UNCONVERGED : kStFallback;
      if (a.stats) {
        atomicAdd(a.stats + 1, 1ull);
        atomicAdd(a.stats + 2, (unsigned long long)steps);
        atomicAdd(a.stats + 3, 6ull * steps * n3);
      }
    }
    return;
  }
  if (!ok) {  // next Newton step
    if (tid == 0) a.status[b] = kStRefining;
    return;
  }
  // standard form of the 2x2 blocks (_gs2x2!) and the eigenvalues
  double* wr = a.wr + a.woffs[b];
  double* wi = a.wi + a.woffs[b];
  for (int p = 0; p < N; ++p) {
    const int i0 = sm.bs[p];
    if (sm.bs[p + 1] - i0 == 1) {
      if (tid == 0) { wr[i0] = A[(size_t)i0 * n + i0]; wi[i0] = 0.0; }
      continue;
    }
    const int q = i0 + 1;
    if (tid == 0) {
      double aa = A[(size_t)i0 * n + i0], bb = A[(size_t)q * n + i0], cc = A[(size_t)i0 * n + q], dd = A[(size_t)q * n + q];
      double cs, sn, w1r, w1i, w2r, w2i;
      gs2x2(aa, bb, cc, dd, cs, sn, w1r, w1i, w2r, w2i);
      wr[i0] = w1r; wi[i0] = w1i; wr[q] = w2r; wi[q] = w2i;
      A[(size_t)i0 * n + i0] = aa; A[(size_t)q * n + i0] = bb; A[(size_t)i0 * n + q] = cc; A[(size_t)q * n + q] = dd;
      sm.rot[0] = cs; sm.rot[1] = sn;
    }
    __syncthreads();
    const double cs = sm.rot[0], sn = sm.rot[1];
    for (int j = q + 1 + tid; j < n; j += kRT) {  // rows i0, q right of the block
      const double a1 = A[(size_t)j * n + i0], a2 = A[(size_t)j * n + q];
      A[(size_t)j * n + i0] = cs * a1 + sn * a2;
      A[(size_t)j * n + q] = -sn * a1 + cs * a2;
    }
    for (int r = tid; r < n; r += kRT) {  // columns i0, q above the block, and of Z
      if (r < i0) {
        const double a1 = A[(size_t)i0 * n + r], a2 = A[(size_t)q * n + r];
        A[(size_t)i0 * n + r] = cs * a1 + sn * a2;
        A[(size_t)q * n + r] = -sn * a1 + cs * a2;
      }
      const double z1 = Z[(size_t)i0 * n + r], z2 = Z[(size_t)q * n + r];
      Z[(size_t)i0 * n + r] = cs * z1 + sn * z2;
      Z[(size_t)q * n + r] = -sn * z1 + cs * z2;
    }
    __syncthreads();
  }
  __syncthreads();
  if (usc != 1.0) {
    for (int idx = tid; idx < nn; idx += kRT) A[idx] *= usc;
    for (int i = tid; i < n; i += kRT) { wr[i] *= usc; wi[i] *= usc; }
  }
  if (tid == 0) {
    a.status[b] = ST_OK;
    if (a.stats) {  // FP64-accurate product FLOPs: per step A_s Z, Z^T P and Z^T Z (2 n^3 each)
      atomicAdd(a.stats, 1ull);
      atomicAdd(a.stats + 2, (unsigned long long)steps);
      atomicAdd(a.stats + 3, 6ull * steps * n3);
    }
  }
}

// One size bin (orders up to 16 RM), Newton step `step`: persistent CTAs take the bin's
// matrices, largest first, from the step's ticket counter for the bin.
// Three CTAs per SM (80 registers): measured faster than two on the 20,000-matrix batch;
// four spill the product loops.
template <int RM>
__global__ void __launch_bounds__(kRT, 3) k_refine_bin(RefineArgs a, int bin, int step) {
  __shared__ Smem sm;
  const int beg = a.sched[3 * bin], end = a.sched[3 * bin + 1];
  int* ticket = a.ticket + kRefineTicketsPerStep * step + bin;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sm.ticket = beg + atomicAdd(ticket, 1);
    __syncthreads();
    const int t = sm.ticket;
    if (t >= end) break;
    const int b = a.order[t];
    const int n = a.ns[b];
    if (n < 1 || n > kSmallMax) continue;  // empty (ST_OK) or order out of range (ST_BADARG)
    const int st = a.status[b];
    if (st == kStRefining) {  // the step's products are missing (a tensor-core wait timed out)
      if (threadIdx.x == 0) {
        a.status[b] = a.nofallback ? ST_UNCONVERGED : kStFallback;
        if (a.stats) atomicAdd(a.stats + 1, 1ull);
      }
      continue;
    }
    if (st != kStStepReady) continue;
    refine_step<RM>(a, b, n, step, sm);
  }
}

}  // namespace

template <int RM>
cudaError_t launch_refine_bin(const RefineArgs& a, int bin, int step, int num_sms, cudaStream_t s) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_refine_bin<RM>, kRT, 0);
  if (e != cudaSuccess) return e;
  if (const char* ev = std::getenv("GS_REFINE_CTAS")) {  // tuning runs: CTAs per SM
    const int c = std::atoi(ev);
    if (c > 0 && c < per_sm) per_sm = c;
  }
  if (const char* ev = std::getenv("GS_REFINE_CARVEOUT")) {  // tuning runs: shared-memory carveout, percent
    e = cudaFuncSetAttribute(k_refine_bin<RM>, cudaFuncAttributePreferredSharedMemoryCarveout, std::atoi(ev));
    if (e != cudaSuccess) return e;
  }
  k_refine_bin<RM><<<num_sms * (per_sm > 0 ? per_sm : 1), kRT, 0, s>>>(a, bin, step);
  return cudaGetLastError();
}

}  // namespace gsk
