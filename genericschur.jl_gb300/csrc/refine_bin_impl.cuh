// Device code of one bin of the mixed-precision batched real Schur refinement
// (refine_batched.cu describes the method): CTA matrix products, the block Sylvester
// waves, the per-matrix Newton loop and the bin kernel.  Included only by the per-bin
// translation units (refine_bin_r*.cu), so that each compiles one row tile.
#pragma once
#include "refine_batched.cuh"

namespace gsk {
namespace {

constexpr int kRT = 256;          // threads per CTA (16 x 16 product layout)
constexpr int kKC = 32;           // contraction chunk staged in shared memory
constexpr int kAS = kSmallMax + 1;  // staged op(A) chunk: kKC rows of up to 128 entries (odd stride)
constexpr int kNC = 4;            // columns per thread in one pass
constexpr int kPW = 16 * kNC;     // columns per pass
constexpr int kBS = kPW + 1;      // staged B chunk: kKC rows of kPW entries
constexpr float kMinGain = 4.f;    // from the third step on, a step must shrink max|X| this much
constexpr float kTolFinal = 1e-9f;
constexpr float kTolDiverge = 1e-1f;

// Tiles of the block Sylvester solve: about kTile rows each, never splitting a 2x2 block
constexpr int kTile = 16;
constexpr int kMaxTiles = 9;   // orders <= 128 give at most 8 tiles of >= 16 rows
constexpr int kTS = 17;        // largest tile (a 2x2 block may extend one by a row); smem row stride

struct Smem {
  float a[kKC * kAS];          // product staging; the Sylvester solve's tiles
  float b[kKC * kBS];
  float red[3][kRT / 32];
  double rot[2];
  short bs[kSmallMax + 2];
  unsigned char bid[kSmallMax];
  short te[kMaxTiles + 1];     // tile row starts
  short tbk[kMaxTiles + 1];    // tile block starts
  int nblk;
  int ntile;
  int ticket;
};
static_assert(2 * kMaxTiles * kTS * kTS <= kKC * (kAS + kBS),
              "the Sylvester tiles fit in the product staging area");

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
// CTA matrix product C (n x ncols) = sum_{k < kdim} opA(i, k) B(k, j) in FP32.  Threads
// form a 16 x 16 grid; in each pass over kPW columns [j0, j0 + kPW) thread (tx, ty) owns
// rows tx + 16 r (r < RMP) and columns j0 + ty + 16 c (c < kNC).  Chunks of kKC
// contraction indices are staged in shared memory (zero beyond n / kdim); the loaders say
// whether consecutive k are contiguous in memory (kfast), which picks the coalesced
// staging order.  The store functor receives every (i, j, value) with i < n, j < ncols.
// ------------------------------------------------------------------------------------
template <int RMP, class LA, class LB, class ST>
__device__ void mm_pass(int n, int ncols, int kdim, int j0, const LA& la, const LB& lb, const ST& st, Smem& sm) {
  float* sa = sm.a;
  float* sb = sm.b;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  constexpr int nrow = RMP * 16;
  const int cm = min(kNC, (ncols - j0 + 15) >> 4);
  float acc[RMP][kNC];
#pragma unroll
  for (int r = 0; r < RMP; ++r)
#pragma unroll
    for (int c = 0; c < kNC; ++c) acc[r][c] = 0.f;
  for (int k0 = 0; k0 < kdim; k0 += kKC) {
    __syncthreads();
    if (la.kfast(k0)) {
      for (int e = tid; e < kKC * nrow; e += kRT) {
        const int kk = e & (kKC - 1), i = e / kKC, k = k0 + kk;
        sa[kk * kAS + i] = (i < n && k < kdim) ? la(i, k) : 0.f;
      }
    } else {
      for (int e = tid; e < kKC * nrow; e += kRT) {
        const int kk = e / nrow, i = e - kk * nrow, k = k0 + kk;
        sa[kk * kAS + i] = (i < n && k < kdim) ? la(i, k) : 0.f;
      }
    }
    if (lb.kfast(k0)) {
      for (int e = tid; e < kKC * kPW; e += kRT) {
        const int kk = e & (kKC - 1), jj = e / kKC, j = j0 + jj, k = k0 + kk;
        sb[kk * kBS + jj] = (j < ncols && k < kdim) ? lb(k, j) : 0.f;
      }
    } else {
      for (int e = tid; e < kKC * kPW; e += kRT) {
        const int kk = e / kPW, jj = e % kPW, j = j0 + jj, k = k0 + kk;
        sb[kk * kBS + jj] = (j < ncols && k < kdim) ? lb(k, j) : 0.f;
      }
    }
    __syncthreads();
    const int kn = min(kKC, kdim - k0);
#pragma unroll 4
    for (int kk = 0; kk < kn; ++kk) {
      float av[RMP], bv[kNC];
#pragma unroll
      for (int r = 0; r < RMP; ++r) av[r] = sa[kk * kAS + tx + 16 * r];
#pragma unroll
      for (int c = 0; c < kNC; ++c) bv[c] = sb[kk * kBS + ty + 16 * c];
#pragma unroll
      for (int r = 0; r < RMP; ++r)
#pragma unroll
        for (int c = 0; c < kNC; ++c)
          if (c < cm) acc[r][c] = fmaf(av[r], bv[c], acc[r][c]);
    }
  }
#pragma unroll
  for (int r = 0; r < RMP; ++r)
#pragma unroll
    for (int c = 0; c < kNC; ++c) {
      const int i = tx + 16 * r, j = j0 + ty + 16 * c;
      if (i < n && j < ncols) st(i, j, acc[r][c]);
    }
}

template <int RM, class LA, class LB, class ST>
__device__ void cta_mm(int n, int ncols, int kdim, const LA& la, const LB& lb, const ST& st, Smem& sm) {
  for (int j0 = 0; j0 < ncols; j0 += kPW) mm_pass<RM>(n, ncols, kdim, j0, la, lb, st, sm);
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

// Gaussian elimination with partial pivoting on an M x M system held in registers (every
// index is a compile-time constant: the pivot row is brought up by compare-and-swap steps);
// pivots below `floor` in magnitude are replaced by +-floor (a bounded correction for
// eigenvalues that FP32 does not separate; the step then fails the tolerance).
template <int M>
__device__ __forceinline__ void gauss_solve(float (&K)[M][M], float (&r)[M], float floor) {
  float inv[M];
#pragma unroll
  for (int c = 0; c < M; ++c) {
#pragma unroll
    for (int i = c + 1; i < M; ++i) {
      const bool sw = fabsf(K[i][c]) > fabsf(K[c][c]);
#pragma unroll
      for (int j = c; j < M; ++j) {
        const float x = K[c][j], y = K[i][j];
        K[c][j] = sw ? y : x;
        K[i][j] = sw ? x : y;
      }
      const float x = r[c], y = r[i];
      r[c] = sw ? y : x;
      r[i] = sw ? x : y;
    }
    if (fabsf(K[c][c]) < floor) K[c][c] = K[c][c] < 0.f ? -floor : floor;
    inv[c] = __frcp_rn(K[c][c]);  // one reciprocal per pivot, reused by the back substitution
#pragma unroll
    for (int i = c + 1; i < M; ++i) {
      const float f = K[i][c] * inv[c];
#pragma unroll
      for (int j = c; j < M; ++j) K[i][j] -= f * K[c][j];
      r[i] -= f * r[c];
    }
  }
#pragma unroll
  for (int c = M - 1; c >= 0; --c) {
    float v = r[c];
#pragma unroll
    for (int j = c + 1; j < M; ++j) v -= K[c][j] * r[j];
    r[c] = v * inv[c];
  }
}

// Kronecker system of block pair (p, q) of orders IP, JQ:
// (I_q (x) T_pp - T_qq^T (x) I_p) vec(W_pq) = vec(r), vec index a + IP b.  tp / tq: the
// diagonal blocks (row stride ld); r[a][b]: the right-hand side, overwritten by W_pq.
template <int IP, int JQ>
__device__ __forceinline__ void pair_solve_t(const float* tp, const float* tq, int ld, float (&r)[2][2], float floor) {
  constexpr int M = IP * JQ;
  float K[M][M], rv[M];
#pragma unroll
  for (int u = 0; u < M; ++u)
#pragma unroll
    for (int v = 0; v < M; ++v) K[u][v] = 0.f;
#pragma unroll
  for (int b = 0; b < JQ; ++b)
#pragma unroll
    for (int a = 0; a < IP; ++a) {
      const int row = a + IP * b;
      rv[row] = r[a][b];
#pragma unroll
      for (int a2 = 0; a2 < IP; ++a2) K[row][a2 + IP * b] += tp[a * ld + a2];
#pragma unroll
      for (int b2 = 0; b2 < JQ; ++b2) K[row][a + IP * b2] -= tq[b2 * ld + b];
    }
  gauss_solve<M>(K, rv, floor);
#pragma unroll
  for (int b = 0; b < JQ; ++b)
#pragma unroll
    for (int a = 0; a < IP; ++a) r[a][b] = rv[a + IP * b];
}

__device__ __forceinline__ void pair_solve(int ip, int jq, const float* tp, const float* tq, int ld,
                                           float (&r)[2][2], float floor) {
  if (ip == 1 && jq == 1) pair_solve_t<1, 1>(tp, tq, ld, r, floor);
  else if (ip == 2 && jq == 1) pair_solve_t<2, 1>(tp, tq, ld, r, floor);
  else if (ip == 1) pair_solve_t<1, 2>(tp, tq, ld, r, floor);
  else pair_solve_t<2, 2>(tp, tq, ld, r, floor);
}

// Block-lower W of T_pp W_pq - W_pq T_qq = R_pq - sum_{r>p} T_pr W_rq + sum_{r<q} W_pr T_rq
// (T: block-upper part of Tf; R: block-lower entries of R, overwritten) by tiles of about
// kTile rows that never split a 2x2 block.  Tile pairs (P, Q), P >= Q, are solved by
// waves D = P - Q from the bottom-left tile up; the tiles of one wave are solved at once in
// shared memory (the diagonal tiles of T and the wave's tiles of R/W there), block pair by
// block pair along local anti-diagonals, with only the within-tile sums; after each wave,
// the solved tiles' contributions are pushed into the right-hand sides of the tiles that
// need them (R_PQ -= T_{P,S} W_{S,Q} for the solved tile below in the same tile column,
// R_PQ += W_{P,S} T_{S,Q} for the solved tile left in the same tile row).  The long sums of
// the element-wise waves thus become short tile products whose loads are coalesced.
__device__ void sylv_tiled(int n, int N, const short* bs, const unsigned char* bid, const float* Tf, float* R,
                           float* W, float floor, Smem& sm) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    int nt = 0;
    sm.te[0] = 0;
    sm.tbk[0] = 0;
    for (int p = 0; p < N; ++p)
      if (bs[p] - sm.te[nt] >= kTile) {
        ++nt;
        sm.te[nt] = bs[p];
        sm.tbk[nt] = (short)p;
      }
    ++nt;
    sm.te[nt] = (short)n;
    sm.tbk[nt] = (short)N;
    sm.ntile = nt;
  }
  __syncthreads();
  const int nt = sm.ntile;
  float* sT = sm.a;       // diagonal tiles of T: [tile][row * kTS + col]
  float* sW = sT + kMaxTiles * kTS * kTS;            // the wave's tiles of R / W: [Q][row * kTS + col]
  for (int e = tid; e < nt * kTS * kTS; e += kRT) {
    const int t = e / (kTS * kTS), l = e - t * kTS * kTS, li = l / kTS, lj = l - li * kTS;
    const int i = sm.te[t] + li, j = sm.te[t] + lj;
    sT[e] = (i < sm.te[t + 1] && j < sm.te[t + 1]) ? Tf[(size_t)j * n + i] : 0.f;
  }
  for (int D = nt - 1; D >= 0; --D) {
    const int ntl = nt - D;  // tiles (Q + D, Q), Q < ntl
    __syncthreads();
    for (int e = tid; e < ntl * kTS * kTS; e += kRT) {
      const int Q = e / (kTS * kTS), l = e - Q * kTS * kTS, li = l / kTS, lj = l - li * kTS;
      const int i = sm.te[Q + D] + li, j = sm.te[Q] + lj;
      sW[e] = (i < sm.te[Q + D + 1] && j < sm.te[Q + 1]) ? R[(size_t)j * n + i] : 0.f;
    }
    int maxw = 0;
    for (int Q = 0; Q < ntl; ++Q)
      maxw = max(maxw, (sm.tbk[Q + D + 1] - sm.tbk[Q + D]) + (sm.tbk[Q + 1] - sm.tbk[Q]) - 1);
    __syncthreads();
    // local waves: pair (p, q) of tile pair (P, Q) on wave (last block of P - p) + (q - first block of Q)
    for (int w = 0; w < maxw; ++w) {
      for (int task = tid; task < ntl * kTS; task += kRT) {
        const int Q = task / kTS, a = task - Q * kTS, P = Q + D;
        const int pb = sm.tbk[P], pe = sm.tbk[P + 1], qb = sm.tbk[Q], qe = sm.tbk[Q + 1];
        const int p = pe - 1 - a, q = qb + (w - a);
        if (a > w || p < pb || q >= qe) continue;
        if (D == 0 && p <= q) continue;
        const int tP = sm.te[P], tQ = sm.te[Q];
        const int li0 = bs[p] - tP, ip = bs[p + 1] - bs[p], lj0 = bs[q] - tQ, jq = bs[q + 1] - bs[q];
        const int lpe = sm.te[P + 1] - tP;
        float* rw = sW + Q * kTS * kTS;
        const float* tp = sT + P * kTS * kTS;
        const float* tq = sT + Q * kTS * kTS;
        float r[2][2];
        r[0][0] = rw[li0 * kTS + lj0];
        r[1][0] = ip == 2 ? rw[(li0 + 1) * kTS + lj0] : 0.f;
        r[0][1] = jq == 2 ? rw[li0 * kTS + lj0 + 1] : 0.f;
        r[1][1] = (ip == 2 && jq == 2) ? rw[(li0 + 1) * kTS + lj0 + 1] : 0.f;
        for (int k = li0 + ip; k < lpe; ++k) {  // - sum_{r>p} T_pr W_rq within tile P
          const float t0 = tp[li0 * kTS + k], t1 = ip == 2 ? tp[(li0 + 1) * kTS + k] : 0.f;
          const float w0 = rw[k * kTS + lj0], w1 = jq == 2 ? rw[k * kTS + lj0 + 1] : 0.f;
          r[0][0] -= t0 * w0; r[0][1] -= t0 * w1; r[1][0] -= t1 * w0; r[1][1] -= t1 * w1;
        }
        for (int k = 0; k < lj0; ++k) {  // + sum_{r<q} W_pr T_rq within tile Q
          const float w0 = rw[li0 * kTS + k], w1 = ip == 2 ? rw[(li0 + 1) * kTS + k] : 0.f;
          const float t0 = tq[k * kTS + lj0], t1 = jq == 2 ? tq[k * kTS + lj0 + 1] : 0.f;
          r[0][0] += w0 * t0; r[0][1] += w0 * t1; r[1][0] += w1 * t0; r[1][1] += w1 * t1;
        }
        pair_solve(ip, jq, tp + li0 * kTS + li0, tq + lj0 * kTS + lj0, kTS, r, floor);
        for (int b = 0; b < jq; ++b)
          for (int a2 = 0; a2 < ip; ++a2) rw[(li0 + a2) * kTS + lj0 + b] = r[a2][b];
      }
      __syncthreads();
    }
    // the solved tiles to W (block-lower entries)
    for (int e = tid; e < ntl * kTS * kTS; e += kRT) {
      const int Q = e / (kTS * kTS), l = e - Q * kTS * kTS, li = l / kTS, lj = l - li * kTS;
      const int i = sm.te[Q + D] + li, j = sm.te[Q] + lj;
      if (i < sm.te[Q + D + 1] && j < sm.te[Q + 1] && bid[i] > bid[j]) W[(size_t)j * n + i] = sW[e];
    }
    if (D == 0) break;
    // right-looking update, term 1: for each tile column Q < ntl, rows of tiles Q .. Q+D-1:
    // R(i, j) -= sum_{k in tile Q+D} T(i, k) W(k, j)
    {
      int tot = 0;
      for (int Q = 0; Q < ntl; ++Q) tot += (sm.te[Q + D] - sm.te[Q]) * (sm.te[Q + 1] - sm.te[Q]);
      for (int e = tid; e < tot; e += kRT) {
        int Q = 0, l = e;
        for (;; ++Q) {
          const int sz = (sm.te[Q + D] - sm.te[Q]) * (sm.te[Q + 1] - sm.te[Q]);
          if (l < sz) break;
          l -= sz;
        }
        const int rows = sm.te[Q + D] - sm.te[Q];
        const int i = sm.te[Q] + l % rows, lj = l / rows, j = sm.te[Q] + lj;
        const int k0 = sm.te[Q + D], kn = sm.te[Q + D + 1] - k0;
        const float* ws = sW + Q * kTS * kTS + lj;  // W(k0 + kk, j) = ws[kk * kTS]
        float acc = 0.f;
#pragma unroll
        for (int kk = 0; kk < kTS; ++kk)
          if (kk < kn) acc += Tf[(size_t)(k0 + kk) * n + i] * ws[kk * kTS];
        R[(size_t)j * n + i] -= acc;
      }
    }
    __syncthreads();
    // term 2: for each tile row P >= D, columns of tiles P-D+1 .. P:
    // R(i, j) += sum_{k in tile P-D} W(i, k) T(k, j)
    {
      int tot = 0;
      for (int P = D; P < nt; ++P) tot += (sm.te[P + 1] - sm.te[P]) * (sm.te[P + 1] - sm.te[P - D + 1]);
      for (int e = tid; e < tot; e += kRT) {
        int P = D, l = e;
        for (;; ++P) {
          const int sz = (sm.te[P + 1] - sm.te[P]) * (sm.te[P + 1] - sm.te[P - D + 1]);
          if (l < sz) break;
          l -= sz;
        }
        const int rows = sm.te[P + 1] - sm.te[P];
        const int li = l % rows, i = sm.te[P] + li, j = sm.te[P - D + 1] + l / rows;
        const int k0 = sm.te[P - D], kn = sm.te[P - D + 1] - k0;
        const float* ws = sW + (P - D) * kTS * kTS + li * kTS;  // W(i, k0 + kk) = ws[kk]
        const float* tc = Tf + (size_t)j * n + k0;                // T(k0 + kk, j) = tc[kk]
        float acc = 0.f;
#pragma unroll
        for (int kk = 0; kk < kTS; ++kk)
          if (kk < kn) acc += ws[kk] * tc[kk];
        R[(size_t)j * n + i] += acc;
      }
    }
  }
  __syncthreads();
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
    cta_mm<RM>(n, n, 2 * n, LdCatA{NF, false, AtF, n}, LdCatB{AtF, NF, n},
                      [&](int i, int j, float v) { M[(size_t)j * n + i] = v; }, sm);
    for (int idx = tid; idx < nn; idx += kRT) {
      const int i = idx % n, j = idx / n;
      if (bid[i] > bid[j]) M[idx] = -(AtF[idx] + M[idx]);
    }
    __syncthreads();
    const float floor = 8.f * 1.2e-7f * (tnorm > 0.f ? tnorm : 1.f);
    sylv_tiled(n, N, sm.bs, bid, AtF, M, W, floor, sm);
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
      cta_mm<RM>(n, n, 2 * n, LdCatA{W, true, AtF, n}, LdCatB{AtF, W, n},
                        [&](int i, int j, float v) {
                          A[(size_t)j * n + i] = bid[i] > bid[j] ? 0.0 : Q[(size_t)j * n + i] + (double)v;
                        },
                        sm);
    }
    // Z <- Z + Z X (product in FP32), through P
    cta_mm<RM>(n, n, n, LdN<float, float>{ZF, n, 1.f}, LdNB<float, float>{W, n},
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
// Three CTAs per SM (80 registers): measured faster than two or one (also with the L1 share
// raised for the Sylvester waves) on the 20,000-matrix batch; four spill the product loops.
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
  k_refine_bin<RM><<<num_sms * (per_sm > 0 ? per_sm : 1), kRT, 0, s>>>(a, bin, step);
  return cudaGetLastError();
}

}  // namespace gsk
