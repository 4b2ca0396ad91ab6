// Eigenvectors of a complex Schur pair of any order (the n > 128 path).
//
// Right eigenvector ki (_geigvecs!, vectors.jl:45-131): x_ki = 1, x_i = 0 for i > ki,
// and for i < ki
//     (T[i,i] - T[ki,ki]) x_i = -sum_{i<k<=ki} T[i,k] x_k,
// with the shifted diagonal floored at smin = max(eps |T[ki,ki]|_1, n safemin) as in
// _usolve! (util.jl:128-293); then v = Z x, scaled by 1/max|v|_1 and normalised by
// _enormalize! (util.jl:572-592).  All n systems together form an upper-triangular X
// with T X - X diag(T) = 0 column by column, solved here in 32x32 tiles: tile (I, J)
// (I <= J, eigenvectors of column tile J, rows of row tile I) needs the tiles (K, J),
// K > I, so the tiles are processed by levels L = J - I, one launch per level, each
// tile by one CTA: the right-hand side -sum_K T_IK X_KJ is accumulated from tiles
// staged in shared memory, then each of the 32 columns is back-substituted through
// T_II by one thread.
//
// Left eigenvectors (_gleigvecs!, vectors.jl:372-460: A^H y = conj(lambda) y) are the
// right eigenvectors of W = P T^H P (P the index reversal, W upper triangular):
// y = P x.  The xLATRS-style rescaling of _usolve!/_cusolve! is not carried out for
// n > 128 (the systems are solved directly with the floored diagonal); a column
// whose solution overflows (non-finite entries) makes the call return GS_UNCONVERGED,
// where the reference would have rescaled it instead.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kEb = 32;    // tile order
constexpr int kEt = 256;   // threads per CTA

// smin of eigenvalue lam (vectors.jl:61, 73)
__device__ __forceinline__ double ev_smin(double2 lam, int n) {
  return fmax(kEps * zabs1(lam), kSafemin * (double)n);
}

// 1 / d for the floored shifted diagonal d (complex), via conj(d) / |d|^2
__device__ __forceinline__ double2 zrecip(double2 d) {
  const double r = 1.0 / fma(d.x, d.x, d.y * d.y);
  return make_double2(d.x * r, -d.y * r);
}

// W = P T^H P (reversal), or a plain copy of T, upper triangle only; lower triangle zero.
__global__ void k_prep_w(int n, const double2* __restrict__ T, double2* __restrict__ W, int reverse) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int i = idx % n, j = idx / n;
  double2 v = make_double2(0.0, 0.0);
  if (i <= j) v = reverse ? zconj(T[(size_t)(n - 1 - i) * n + (n - 1 - j)]) : T[idx];
  W[idx] = v;
}

// Level 0: the diagonal tiles.  Thread c (< tile width) owns eigenvector ki = j0 + c.
__global__ void __launch_bounds__(kEt) k_ev_diag(int n, const double2* __restrict__ W, double2* __restrict__ X) {
  __shared__ double2 Ts[kEb][kEb + 1];
  const int j0 = blockIdx.x * kEb;
  const int w = min(kEb, n - j0);
  for (int idx = threadIdx.x; idx < kEb * kEb; idx += kEt) {
    const int r = idx % kEb, c = idx / kEb;
    Ts[r][c] = (r < w && c < w) ? W[(size_t)(j0 + c) * n + j0 + r] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (c >= w) return;
  const double2 lam = Ts[c][c];
  const double smin = ev_smin(lam, n);
  double2 x[kEb];
#pragma unroll
  for (int r = 0; r < kEb; ++r) x[r] = (r < c) ? zneg(Ts[r][c]) : make_double2(r == c ? 1.0 : 0.0, 0.0);
  for (int r = c - 1; r >= 0; --r) {
    double2 d = zsub(Ts[r][r], lam);
    if (zabs1(d) < smin) d = make_double2(smin, 0.0);
    const double2 xr = zmul(x[r], zrecip(d));
    x[r] = xr;
    for (int k = 0; k < r; ++k) x[k] = zfms(Ts[k][r], xr, x[k]);
  }
  for (int r = 0; r < kEb; ++r)
    if (r < w) X[(size_t)(j0 + c) * n + j0 + r] = x[r];
}

// Level L >= 1: tile (I, J = I + L).  rhs = -sum_{K=I+1..J} W_IK X_KJ, then column
// back-substitution through W_II.
__global__ void __launch_bounds__(kEt) k_ev_level(int n, int nt, int L, const double2* __restrict__ W,
                                                  double2* __restrict__ X) {
  __shared__ double2 As[kEb][kEb + 1];
  __shared__ double2 Bs[kEb][kEb + 1];
  __shared__ double2 R[kEb][kEb + 1];
  const int I = blockIdx.x, J = I + L;
  if (J >= nt) return;
  const int i0 = I * kEb, j0 = J * kEb;
  const int wi = min(kEb, n - i0), wj = min(kEb, n - j0);
  const int tid = threadIdx.x;
  // each thread owns 4 outputs: rows r = tid % 32, columns c = tid / 32 + 8 q
  const int r = tid % kEb, cb = tid / kEb;
  double2 acc[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = make_double2(0.0, 0.0);
  for (int K = I + 1; K <= J; ++K) {
    const int k0 = K * kEb, wk = min(kEb, n - k0);
    for (int idx = tid; idx < kEb * kEb; idx += kEt) {
      const int a = idx % kEb, b = idx / kEb;
      As[a][b] = (a < wi && b < wk) ? W[(size_t)(k0 + b) * n + i0 + a] : make_double2(0.0, 0.0);
      Bs[a][b] = (a < wk && b < wj) ? X[(size_t)(j0 + b) * n + k0 + a] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kEb; ++k) {
      const double2 a = As[r][k];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = zfma(a, Bs[k][cb + 8 * q], acc[q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) R[r][cb + 8 * q] = zneg(acc[q]);
  for (int idx = tid; idx < kEb * kEb; idx += kEt) {
    const int a = idx % kEb, b = idx / kEb;
    As[a][b] = (a < wi && b < wi) ? W[(size_t)(i0 + b) * n + i0 + a] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int c = tid;
  if (c < wj) {
    const double2 lam = W[(size_t)(j0 + c) * n + j0 + c];
    const double smin = ev_smin(lam, n);
    for (int rr = wi - 1; rr >= 0; --rr) {
      double2 d = zsub(As[rr][rr], lam);
      if (zabs1(d) < smin) d = make_double2(smin, 0.0);
      const double2 xr = zmul(R[rr][c], zrecip(d));
      R[rr][c] = xr;
      for (int k = 0; k < rr; ++k) R[k][c] = zfms(As[k][rr], xr, R[k][c]);
    }
    for (int rr = 0; rr < wi; ++rr) X[(size_t)(j0 + c) * n + i0 + rr] = R[rr][c];
  }
}

// C = Z X restricted to the nonzero triangle of X (upper: rows <= column; with
// reverse, X is stored for W and Y = P X: column ki of the left vectors is
// Z (P x^{(n-1-ki)})).  64x64 output tiles, 256 threads, 4x4 per thread.
__global__ void __launch_bounds__(256) k_ev_gemm(int n, const double2* __restrict__ Z, const double2* __restrict__ X,
                                                 double2* __restrict__ V, int reverse) {
  __shared__ double2 Zs[16][64 + 1];
  __shared__ double2 Xs[16][64 + 1];
  const int tid = threadIdx.x;
  const int tr = tid % 16, tc = tid / 16;
  const int r0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
  double2 acc[4][4];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0.0, 0.0);
  // output column ki = c0 + cc uses X column (reverse ? n-1-ki : ki) with entries at
  // rows k (reverse: row n-1-k of X holds the coefficient of Z column k)
  const int kmax = reverse ? n : min(n, c0 + 64);
  const int kmin = reverse ? max(0, c0) : 0;
  for (int k0 = kmin - (kmin % 16); k0 < kmax; k0 += 16) {
    for (int idx = tid; idx < 16 * 64; idx += 256) {
      const int kk = idx / 64, ii = idx % 64;
      const int k = k0 + kk;
      const int row = r0 + ii;
      Zs[kk][ii] = (row < n && k < n) ? (Z ? Z[(size_t)k * n + row] : make_double2(row == k ? 1.0 : 0.0, 0.0))
                                      : make_double2(0.0, 0.0);
      const int col = c0 + ii;
      double2 xv = make_double2(0.0, 0.0);
      if (col < n && k < n) {
        if (!reverse) xv = (k <= col) ? X[(size_t)col * n + k] : make_double2(0.0, 0.0);
        else {
          const int xc = n - 1 - col, xr = n - 1 - k;
          xv = (xr <= xc) ? X[(size_t)xc * n + xr] : make_double2(0.0, 0.0);
        }
      }
      Xs[kk][ii] = xv;
    }
    __syncthreads();
    for (int kk = 0; kk < 16; ++kk) {
      double2 a[4], b[4];
      for (int x = 0; x < 4; ++x) a[x] = Zs[kk][tr + 16 * x];
      for (int y = 0; y < 4; ++y) b[y] = Xs[kk][tc + 16 * y];
      for (int x = 0; x < 4; ++x)
        for (int y = 0; y < 4; ++y) acc[x][y] = zfma(a[x], b[y], acc[x][y]);
    }
    __syncthreads();
  }
  for (int x = 0; x < 4; ++x)
    for (int y = 0; y < 4; ++y) {
      const int i = r0 + tr + 16 * x, j = c0 + tc + 16 * y;
      if (i < n && j < n) V[(size_t)j * n + i] = acc[x][y];
    }
}

// Per column: scale by 1/max|v|_1, then (normalize) _enormalize!.  Warp per column;
// cmap (optional) maps eigenvector ki to its output column.  bad[0] counts columns
// with non-finite entries.
__global__ void k_ev_normalize(int n, double2* __restrict__ V, int normalize, int* bad) {
  const int lane = threadIdx.x & 31;
  const int col = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (col >= n) return;
  double2* v = V + (size_t)col * n;
  double t0 = 0.0;
  for (int r = lane; r < n; r += 32) t0 = fmax(t0, zabs1(v[r]));
  for (int o = 16; o > 0; o >>= 1) t0 = fmax(t0, __shfl_xor_sync(0xffffffffu, t0, o));
  if (!(t0 > 0.0) || !(t0 < 1.0e308)) {
    if (lane == 0) atomicAdd(bad, 1);
    return;
  }
  const double remax = 1.0 / t0;
  double ss = 0.0, best = -1.0;
  int ib = 0;
  for (int r = lane; r < n; r += 32) {
    const double2 x = zscal(v[r], remax);
    v[r] = x;
    const double a2 = x.x * x.x + x.y * x.y;
    ss += a2;
    if (a2 > best) { best = a2; ib = r; }
  }
  if (!normalize) return;
  for (int o = 16; o > 0; o >>= 1) {
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, ib, o);
    if (ob > best || (ob == best && oi < ib)) { best = ob; ib = oi; }
  }
  const double2 vi0 = v[ib];
  const double s = 1.0 / sqrt(ss);
  const double2 f = zscal(zconj(vi0), s / sqrt(best));
  __syncwarp();
  for (int r = lane; r < n; r += 32) {
    double2 x = zmul(v[r], f);
    if (r == ib) x.y = 0.0;
    v[r] = x;
  }
}

// Scatter columns through a column map (real input: eigenvector ki of the
// triangularised pair goes to output column cmap[ki]).
__global__ void k_ev_scatter(int n, const double2* __restrict__ src, double2* __restrict__ dst, const int* cmap) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int i = idx % n, j = idx / n;
  dst[(size_t)cmap[j] * n + i] = src[idx];
}

}  // namespace

size_t eigvecs_large_ws_elems(int n) { return 3 * (size_t)n * n; }

cudaError_t launch_enormalize(int n, int m, double2* V, int normalize, int* bad, cudaStream_t s) {
  // columns of V (n x m, ld n): 1 / max|v|_1, then _enormalize! when normalize
  k_ev_normalize<<<(m + 7) / 8, 256, 0, s>>>(n, V, normalize, bad);
  return cudaGetLastError();
}

cudaError_t launch_eigvecs_large(int n, const double2* T, const double2* Z, double2* VR, double2* VL, int normalize,
                                 const int* cmap, double2* ws, int* bad, cudaStream_t s) {
  const size_t nn = (size_t)n * n;
  double2* W = ws;
  double2* X = ws + nn;
  double2* tmp = ws + 2 * nn;
  const int nt = (n + kEb - 1) / kEb;
  const unsigned g1 = (unsigned)((nn + 255) / 256);
  for (int pass = 0; pass < 2; ++pass) {
    double2* V = pass == 0 ? VR : VL;
    if (!V) continue;
    const int rev = pass == 1;
    k_prep_w<<<g1, 256, 0, s>>>(n, T, W, rev);
    cudaError_t e = cudaMemsetAsync(X, 0, nn * sizeof(double2), s);
    if (e != cudaSuccess) return e;
    k_ev_diag<<<nt, kEt, 0, s>>>(n, W, X);
    for (int L = 1; L < nt; ++L) k_ev_level<<<nt - L, kEt, 0, s>>>(n, nt, L, W, X);
    dim3 gg((n + 63) / 64, (n + 63) / 64);
    double2* out = cmap ? tmp : V;
    k_ev_gemm<<<gg, 256, 0, s>>>(n, Z, X, out, rev);
    k_ev_normalize<<<(n + 7) / 8, 256, 0, s>>>(n, out, normalize, bad);
    if (cmap) k_ev_scatter<<<g1, 256, 0, s>>>(n, out, V, cmap);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace gsk
