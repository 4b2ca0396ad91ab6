// FP64 refinement of an approximate real Schur pair (the mixed-precision form).
//
// Given orthogonal Z (to working accuracy) and At = Z^T A Z = T + L, with T block
// upper triangular in the 1x1/2x2 block structure of the low-precision Schur form and
// L the (small) block-lower remainder, one Newton step looks for Q = I + S,
// S = W - W^T skew with W block-lower, such that Q^T At Q is block upper triangular
// to first order.  The block-lower part of T S - S T + L must vanish, which for
// block rows p > q reads
//     T_pp W_pq - W_pq T_qq = -L_pq - sum_{r>p} T_pr W_rq + sum_{r<q} W_pr T_rq,
// a block triangular Sylvester equation (the iteration of Bujanovic, Kressner and
// Schroeder, "Iterative refinement of Schur decompositions", Numer. Algorithms 2023),
// solved in 32-row tiles (k_sylv_tile).
// Z is then updated to Z (I + S), which departs from orthogonality by O(|S|^2); a
// Newton-Schulz step Z <- Z (3 I - Z^T Z) / 2 follows whenever |S| is above 1e-8.
// Products with the small corrections S and (I - Z^T Z)/2 run in FP32 (their error is
// second order); Z^T A Z and Z^T Z, whose small parts are the signal, run in FP64.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

// Solve the small system M x = r (m <= 4) with partial pivoting; tiny pivots are
// replaced by +-floor so that (nearly) equal eigenvalues give a bounded correction.
__device__ void small_solve(int m, double M[4][4], double r[4], double floor) {
  for (int c = 0; c < m; ++c) {
    int piv = c;
    for (int i = c + 1; i < m; ++i)
      if (fabs(M[i][c]) > fabs(M[piv][c])) piv = i;
    if (piv != c) {
      for (int j = 0; j < m; ++j) { double t = M[c][j]; M[c][j] = M[piv][j]; M[piv][j] = t; }
      double t = r[c]; r[c] = r[piv]; r[piv] = t;
    }
    if (fabs(M[c][c]) < floor) M[c][c] = (M[c][c] < 0.0) ? -floor : floor;
    for (int i = c + 1; i < m; ++i) {
      const double f = M[i][c] / M[c][c];
      for (int j = c; j < m; ++j) M[i][j] -= f * M[c][j];
      r[i] -= f * r[c];
    }
  }
  for (int c = m - 1; c >= 0; --c) {
    double s = r[c];
    for (int j = c + 1; j < m; ++j) s -= M[c][j] * r[j];
    r[c] = s / M[c][c];
  }
}

// Tiled block Sylvester solve.  The scalar index range is cut into tiles of at most
// kSt rows that never split a 2x2 block (ts[t] = first row of tile t, tbk[t] = its first
// block; ts[nT] = n, tbk[nT] = N).  Tile pair (P, Q), P >= Q, needs the tiles (R, Q),
// R > P, and (P, R), R < Q, so the pairs go by levels D = P - Q from nT-1 down to 0,
// one pair of launches per level:
//   1. rhs = -L_PQ - sum_{R>P} T_PR W_RQ + sum_{R<Q} W_PR T_RQ: the nT-1-D tile
//      products of every pair of the level are split over CTAs of kSplit products
//      (k_sylv_rhs), whose partial tiles the solve step adds in a fixed order;
//   2. the block pairs inside the tile pair by local anti-diagonal waves (k_sylv_solve).
// At: Z^T A Z (block-upper part T, block-lower part L), W: the block-lower solution.
constexpr int kSt = 32;

// Level D, step 1: partial right-hand sides.  CTA (pair, chunk) adds the tile products
// with indices [chunk * kSplit, ...) of the pair's list  R = P+1..nT-1 (minus T_PR W_RQ),
// then R = 0..Q-1 (plus W_PR T_RQ), into part[pair][chunk] (32 x 32, column-major).
constexpr int kSplit = 4;  // tile products per CTA

__global__ void __launch_bounds__(256) k_sylv_rhs(int n, int nT, int D, const double* __restrict__ At,
                                                  const double* __restrict__ W, const int* __restrict__ ts,
                                                  double* __restrict__ part, int nchunk) {
  __shared__ double Ta[kSt][kSt + 1];
  __shared__ double Tb[kSt][kSt + 1];
  const int Q = blockIdx.x, P = Q + D, chunk = blockIdx.y;
  const int tid = threadIdx.x;
  const int p0 = ts[P], pw = ts[P + 1] - p0, q0 = ts[Q], qw = ts[Q + 1] - q0;
  const int r = tid % kSt, cb = tid / kSt;
  const int nprod = nT - 1 - D;  // (nT-1-P) + Q
  const int n1 = nT - 1 - P;     // products of the first sum
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int t = chunk * kSplit; t < min(nprod, (chunk + 1) * kSplit); ++t) {
    const bool first = t < n1;
    const int R = first ? P + 1 + t : t - n1;
    const int r0 = ts[R], rw = ts[R + 1] - r0;
    for (int idx = tid; idx < kSt * kSt; idx += 256) {
      const int x = idx % kSt, y = idx / kSt;
      if (first) {
        Ta[x][y] = (x < pw && y < rw) ? At[(size_t)(r0 + y) * n + p0 + x] : 0.0;  // T_PR
        Tb[x][y] = (x < rw && y < qw) ? W[(size_t)(q0 + y) * n + r0 + x] : 0.0;   // W_RQ
      } else {
        Ta[x][y] = (x < pw && y < rw) ? W[(size_t)(r0 + y) * n + p0 + x] : 0.0;   // W_PR
        Tb[x][y] = (x < rw && y < qw) ? At[(size_t)(q0 + y) * n + r0 + x] : 0.0;  // T_RQ
      }
    }
    __syncthreads();
    const double sg = first ? -1.0 : 1.0;
#pragma unroll 8
    for (int kk = 0; kk < kSt; ++kk) {
      const double a = sg * Ta[r][kk];
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[k] = fma(a, Tb[kk][cb + 8 * k], acc[k]);
    }
    __syncthreads();
  }
  double* out = part + ((size_t)Q * nchunk + chunk) * (kSt * kSt);
#pragma unroll
  for (int k = 0; k < 4; ++k) out[(cb + 8 * k) * kSt + r] = acc[k];
}

// Level D, step 2: one CTA per tile pair sums its partials (fixed order) and -L_PQ,
// then solves the block pairs inside the tile pair by local anti-diagonal waves, warp
// per block pair (the in-tile sums over the lanes, lane 0 solves the <= 4x4 Kronecker
// system (I (x) T_pp - T_qq^T (x) I) vec(W_pq) = rhs).
__global__ void __launch_bounds__(256) k_sylv_solve(int n, int nT, int D, const double* __restrict__ At,
                                                    double* __restrict__ W, const int* __restrict__ bs,
                                                    const int* __restrict__ bz, const int* __restrict__ blk,
                                                    const int* __restrict__ ts, const int* __restrict__ tbk,
                                                    const double* __restrict__ part, int nchunk, double floor) {
  __shared__ double Ta[kSt][kSt + 1];
  __shared__ double Tb[kSt][kSt + 1];
  __shared__ double Wl[kSt][kSt + 1];
  const int Q = blockIdx.x, P = Q + D;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int p0 = ts[P], pw = ts[P + 1] - p0, q0 = ts[Q], qw = ts[Q + 1] - q0;
  const int nused = (nT - 1 - D + kSplit - 1) / kSplit;
  for (int idx = tid; idx < kSt * kSt; idx += 256) {
    const int x = idx % kSt, y = idx / kSt;
    double v = (x < pw && y < qw) ? -At[(size_t)(q0 + y) * n + p0 + x] : 0.0;
    for (int c = 0; c < nused; ++c) v += part[((size_t)Q * nchunk + c) * (kSt * kSt) + y * kSt + x];
    Wl[x][y] = v;
    Ta[x][y] = (x < pw && y < pw) ? At[(size_t)(p0 + y) * n + p0 + x] : 0.0;  // T_PP
    Tb[x][y] = (x < qw && y < qw) ? At[(size_t)(q0 + y) * n + q0 + x] : 0.0;  // T_QQ
  }
  __syncthreads();
  const int pb0 = tbk[P], pb1 = tbk[P + 1], qb0 = tbk[Q], qb1 = tbk[Q + 1];
  const int np = pb1 - pb0, nq = qb1 - qb0;
  for (int d = 0; d < np + nq - 1; ++d) {
    for (int i = warp; i < np; i += 8) {
      const int j = d - i;
      if (j < 0 || j >= nq) continue;
      const int p = pb1 - 1 - i, q = qb0 + j;
      if (P == Q && p <= q) continue;
      const int sp = bs[p] - p0, zp = bz[p], sq = bs[q] - q0, zq = bz[q];
      double s2[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
      for (int k = sp + zp + lane; k < pw; k += 32)
        for (int a = 0; a < zp; ++a)
          for (int b = 0; b < zq; ++b) s2[a][b] -= Ta[sp + a][k] * Wl[k][sq + b];
      for (int k = lane; k < sq; k += 32)
        for (int a = 0; a < zp; ++a)
          for (int b = 0; b < zq; ++b) s2[a][b] += Wl[sp + a][k] * Tb[k][sq + b];
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
          for (int o = 16; o > 0; o >>= 1) s2[a][b] += __shfl_xor_sync(0xffffffffu, s2[a][b], o);
      if (lane == 0) {
        const int m = zp * zq;
        double M[4][4] = {{0}}, rr[4];
        for (int b = 0; b < zq; ++b)
          for (int a = 0; a < zp; ++a) rr[a + b * zp] = Wl[sp + a][sq + b] + s2[a][b];
        for (int b = 0; b < zq; ++b)
          for (int a = 0; a < zp; ++a) {
            const int row = a + b * zp;
            for (int a2 = 0; a2 < zp; ++a2) M[row][a2 + b * zp] += Ta[sp + a][sp + a2];
            for (int b2 = 0; b2 < zq; ++b2) M[row][a + b2 * zp] -= Tb[sq + b2][sq + b];
          }
        small_solve(m, M, rr, floor);
        for (int b = 0; b < zq; ++b)
          for (int a = 0; a < zp; ++a) Wl[sp + a][sq + b] = rr[a + b * zp];
      }
      __syncwarp();
    }
    __syncthreads();
  }
  // write the tile back: block-lower entries only (the diagonal tile keeps zeros elsewhere)
  for (int idx = tid; idx < kSt * kSt; idx += 256) {
    const int x = idx % kSt, y = idx / kSt;
    if (x < pw && y < qw) {
      const bool lower = blk[p0 + x] > blk[q0 + y];
      W[(size_t)(q0 + y) * n + p0 + x] = lower ? Wl[x][y] : 0.0;
    }
  }
}

// S = W - W^T (+ I when add_identity), and block-lower norm accumulation helpers.
__global__ void k_skew(int n, const double* __restrict__ W, double* __restrict__ S, double add_identity) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int i = idx % n, j = idx / n;
  S[idx] = W[idx] - W[(size_t)i * n + j] + (i == j ? add_identity : 0.0);
}

// E = I + S + S2/2 in place over S2.
__global__ void k_exp2(int n, const double* __restrict__ S, double* __restrict__ S2) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int i = idx % n, j = idx / n;
  S2[idx] = (i == j ? 1.0 : 0.0) + S[idx] + 0.5 * S2[idx];
}

// Newton-Schulz correction: X <- (I - X) / 2  (X = Z^T Z on entry)
__global__ void k_ns_factor(int n, double* X) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int i = idx % n, j = idx / n;
  X[idx] = (i == j ? 0.5 : 0.0) - 0.5 * X[idx];
}

// Z += P (P an FP32 product)
__global__ void k_add_f32(double* __restrict__ Z, const float* __restrict__ P, size_t cnt) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (size_t)gridDim.x * blockDim.x)
    Z[i] += (double)P[i];
}

// sum of squares of the block-lower part (entries (i, j) with block(i) > block(j)) and of all
// entries, into out[0], out[1] (atomics on doubles: the norms only steer the iteration).
__global__ void k_lower_norm(int n, const double* __restrict__ At, const int* __restrict__ blk, double* out) {
  double sl = 0.0, sa = 0.0;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (size_t)n * n;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int i = idx % n, j = idx / n;
    const double v = At[idx];
    sa += v * v;
    if (blk[i] > blk[j]) sl += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sl += __shfl_xor_sync(0xffffffffu, sl, o);
    sa += __shfl_xor_sync(0xffffffffu, sa, o);
  }
  if ((threadIdx.x & 31) == 0) { atomicAdd(&out[0], sl); atomicAdd(&out[1], sa); }
}

// T = block-upper part of At (zero below the block diagonal).
__global__ void k_block_triu(int n, const double* __restrict__ At, const int* __restrict__ blk, double* __restrict__ T) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int i = idx % n, j = idx / n;
  T[idx] = (blk[i] > blk[j]) ? 0.0 : At[idx];
}

// Standardise every 2x2 diagonal block with _gs2x2! (GenericSchur.jl:716-803): the
// rotations of different blocks act on disjoint index pairs.  Phase 0: compute
// (cs, sn) and the eigenvalues; phase 1: rows; phase 2: columns of T and Z.
__global__ void k_std_blocks(int n, int N, const int* __restrict__ bs, const int* __restrict__ bz, double* T,
                             double* Z, double* cs_sn, double* wr, double* wi, int phase) {
  const int b = blockIdx.x;
  if (b >= N) return;
  const int s = bs[b], z = bz[b];
  if (z == 1) {
    if (phase == 0 && threadIdx.x == 0) { wr[s] = T[(size_t)s * n + s]; wi[s] = 0.0; }
    return;
  }
  const int p = s, q = s + 1;
  if (phase == 0) {
    if (threadIdx.x == 0) {
      double a = T[(size_t)p * n + p], bb = T[(size_t)q * n + p], c = T[(size_t)p * n + q], d = T[(size_t)q * n + q];
      double cs, sn, w1r, w1i, w2r, w2i;
      gs2x2(a, bb, c, d, cs, sn, w1r, w1i, w2r, w2i);
      cs_sn[4 * b] = cs; cs_sn[4 * b + 1] = sn;
      wr[p] = w1r; wi[p] = w1i; wr[q] = w2r; wi[q] = w2i;
      cs_sn[4 * b + 2] = a;  // keep the standardised block to write it back exactly
      (void)bb; (void)c;
      T[(size_t)p * n + p] = a; T[(size_t)q * n + p] = bb; T[(size_t)p * n + q] = c; T[(size_t)q * n + q] = d;
    }
    return;
  }
  const double cs = cs_sn[4 * b], sn = cs_sn[4 * b + 1];
  if (phase == 1) {
    // rows p, q of T, columns outside the block
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      if (j == p || j == q) continue;
      const double a1 = T[(size_t)j * n + p], a2 = T[(size_t)j * n + q];
      T[(size_t)j * n + p] = cs * a1 + sn * a2;
      T[(size_t)j * n + q] = -sn * a1 + cs * a2;
    }
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      if (i != p && i != q) {
        const double a1 = T[(size_t)p * n + i], a2 = T[(size_t)q * n + i];
        T[(size_t)p * n + i] = cs * a1 + sn * a2;
        T[(size_t)q * n + i] = -sn * a1 + cs * a2;
      }
      if (Z) {
        const double z1 = Z[(size_t)p * n + i], z2 = Z[(size_t)q * n + i];
        Z[(size_t)p * n + i] = cs * z1 + sn * z2;
        Z[(size_t)q * n + i] = -sn * z1 + cs * z2;
      }
    }
  }
}

template <class S, class D>
__global__ void k_convert(const S* __restrict__ src, D* __restrict__ dst, size_t count, double scale) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (D)((double)src[i] * scale);
}

}  // namespace

template <class S, class D>
cudaError_t convert_array(const S* src, D* dst, size_t count, double scale, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  k_convert<S, D><<<1024, 256, 0, s>>>(src, dst, count, scale);
  return cudaGetLastError();
}
template cudaError_t convert_array<double, float>(const double*, float*, size_t, double, cudaStream_t);
template cudaError_t convert_array<float, double>(const float*, double*, size_t, double, cudaStream_t);
template cudaError_t convert_array<double, double>(const double*, double*, size_t, double, cudaStream_t);

int sylv_tiles(int n, const int* blk_host, int* ts, int* tbk) {
  int nT = 0, t = 0;
  while (t < n) {
    int e = t + kSt < n ? t + kSt : n;
    if (e < n && blk_host[e] == blk_host[e - 1]) --e;  // never split a 2x2 block
    ts[nT] = t;
    tbk[nT] = blk_host[t];
    ++nT;
    t = e;
  }
  ts[nT] = n;
  tbk[nT] = blk_host[n - 1] + 1;
  return nT;
}

size_t sylv_part_elems(int nT) {
  const int nchunk = (nT + kSplit - 1) / kSplit;
  return (size_t)nT * nchunk * kSt * kSt;
}

cudaError_t launch_sylv_tiled(int n, int nT, const double* At, double* W, const int* bs, const int* bz,
                              const int* blk, const int* ts, const int* tbk, double* part, double floor,
                              cudaStream_t s) {
  const int nchunk = (nT + kSplit - 1) / kSplit;
  for (int D = nT - 1; D >= 0; --D) {
    const int nprod = nT - 1 - D;
    if (nprod > 0) {
      dim3 g(nT - D, (nprod + kSplit - 1) / kSplit);
      k_sylv_rhs<<<g, 256, 0, s>>>(n, nT, D, At, W, ts, part, nchunk);
    }
    k_sylv_solve<<<nT - D, 256, 0, s>>>(n, nT, D, At, W, bs, bz, blk, ts, tbk, part, nchunk, floor);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_refine_elementwise(int op, int n, const double* a, double* b, double x, cudaStream_t s) {
  const size_t tot = (size_t)n * n;
  const unsigned g = (unsigned)((tot + 255) / 256);
  switch (op) {
    case 0: k_skew<<<g, 256, 0, s>>>(n, a, b, x); break;
    case 1: k_exp2<<<g, 256, 0, s>>>(n, a, b); break;
    case 2: k_ns_factor<<<g, 256, 0, s>>>(n, b); break;
    default: break;
  }
  return cudaGetLastError();
}

// X += P1 - P2 (two FP32 products)
__global__ void k_add_diff_f32(double* __restrict__ X, const float* __restrict__ P1, const float* __restrict__ P2,
                               size_t cnt) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (size_t)gridDim.x * blockDim.x)
    X[i] += (double)P1[i] - (double)P2[i];
}

cudaError_t launch_add_diff_f32(double* X, const float* P1, const float* P2, size_t cnt, cudaStream_t s) {
  k_add_diff_f32<<<1024, 256, 0, s>>>(X, P1, P2, cnt);
  return cudaGetLastError();
}

// X -= P (an FP32 product)
__global__ void k_sub_f32(double* __restrict__ X, const float* __restrict__ P, size_t cnt) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (size_t)gridDim.x * blockDim.x)
    X[i] -= (double)P[i];
}

cudaError_t launch_sub_f32(double* X, const float* P, size_t cnt, cudaStream_t s) {
  k_sub_f32<<<1024, 256, 0, s>>>(X, P, cnt);
  return cudaGetLastError();
}

cudaError_t launch_add_f32(double* Z, const float* P, size_t cnt, cudaStream_t s) {
  k_add_f32<<<1024, 256, 0, s>>>(Z, P, cnt);
  return cudaGetLastError();
}

cudaError_t launch_lower_norm(int n, const double* At, const int* blk, double* out, int num_sms, cudaStream_t s) {
  k_lower_norm<<<4 * num_sms, 256, 0, s>>>(n, At, blk, out);
  return cudaGetLastError();
}

cudaError_t launch_block_triu(int n, const double* At, const int* blk, double* T, cudaStream_t s) {
  const size_t tot = (size_t)n * n;
  k_block_triu<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, At, blk, T);
  return cudaGetLastError();
}

cudaError_t launch_std_blocks(int n, int N, const int* bs, const int* bz, double* T, double* Z, double* cs_sn,
                              double* wr, double* wi, cudaStream_t s) {
  for (int ph = 0; ph < 3; ++ph) {
    k_std_blocks<<<N, 128, 0, s>>>(n, N, bs, bz, T, Z, cs_sn, wr, wi, ph);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace gsk
