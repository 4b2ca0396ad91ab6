// Kernels of the large-matrix (n > 128) Schur path: multishift bulge chasing with
// delayed far updates, the deflation scan, and a tiled GEMM used to apply the
// orthogonal factors of small diagonal blocks to the rest of H and Z.
//
// A sweep on the active block [ilo, ihi] chases B double-shift bulges in a chain
// spaced three rows apart: at sweep step t bulge b sits at k = ilo + t - 3b.  The
// reflectors of one step have disjoint supports, so they are all computed from the
// state at the start of the step (one lane each) and applied left-then-right
// (P H P with P the product of the commuting reflectors).  Each reflector follows
// doubleShiftQR! (GenericSchur.jl:877-949): a bulge enters at k = ilo from the
// start vector of its shift pair (855-862 with m = istart), moves down with 3-element
// reflectors, and leaves with a 2-element one at k = ihi-1.
//
// A sweep runs in chunks of w steps.  The chase kernel (one CTA) keeps the window
// [wlo, whi] that the chunk's bulges occupy in shared memory, updates it and logs
// the reflectors; the far kernel then applies the logged reflectors, step by step,
// to the columns right of the window (rows wlo..whi), the rows above it (columns
// wlo..whi) and to Z (all rows, columns wlo..whi).
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

template <class T> __device__ __forceinline__ T tabs(T x) { return x < T(0) ? -x : x; }

// Real reflector of length 2/3 in type T (householder.jl:12-54 semantics).
template <class T>
__device__ __forceinline__ T refl_t(T& a, T& x1, T& x2, int nr) {
  return reflector_fast(a, x1, x2, nr);
}

}  // namespace

template <class T>
__global__ void __launch_bounds__(256) k_chase_chunk(ChaseArgs<T> ca) {
  extern __shared__ unsigned char smraw[];
  T* W = (T*)smraw;
  const int nw = ca.whi - ca.wlo + 1;
  const int ldw = nw | 1;
  __shared__ T rf[kMaxBulges][5];
  __shared__ int rk[kMaxBulges];
  __shared__ int rn[kMaxBulges];
  const int tid = threadIdx.x;
  const int n = ca.n;
  T* H = ca.H;
  // load the window
  for (int idx = tid; idx < nw * nw; idx += blockDim.x) {
    const int i = idx % nw, j = idx / nw;
    W[i + j * ldw] = H[(size_t)(ca.wlo - 1 + j) * n + (ca.wlo - 1 + i)];
  }
  __syncthreads();
#define WW(i, j) W[((i) - ca.wlo) + ((j) - ca.wlo) * ldw]
  for (int s = 0; s < ca.w; ++s) {
    const int t = ca.t0 + s;
    if (tid < ca.B) {
      const int b = tid;
      const int k = ca.ilo + t - 3 * b;
      int nr = 0;
      T r[5] = {T(0), T(0), T(0), T(0), T(0)};
      if (k >= ca.ilo && k <= ca.ihi - 1) {
        nr = min(3, ca.ihi - k + 1);
        T a, x1, x2 = T(0);
        if (k == ca.ilo) {
          // start vector of the shift pair (GenericSchur.jl:855-862 at m = istart)
          const T r1r = ca.shifts[4 * b + 0], r1i = ca.shifts[4 * b + 1];
          const T r2r = ca.shifts[4 * b + 2], r2i = ca.shifts[4 * b + 3];
          const int m = k;
          T h21s = WW(m + 1, m);
          T sc = tabs(WW(m, m) - r2r) + tabs(r2i) + tabs(h21s);
          if (sc == T(0)) sc = T(1);
          h21s /= sc;
          a = h21s * WW(m, m + 1) + (WW(m, m) - r1r) * ((WW(m, m) - r2r) / sc) - r1i * (r2i / sc);
          x1 = h21s * (WW(m, m) + WW(m + 1, m + 1) - r1r - r2r);
          x2 = (nr == 3) ? h21s * WW(m + 2, m + 1) : T(0);
          const T sn = tabs(a) + tabs(x1) + tabs(x2);
          if (sn != T(0)) { a /= sn; x1 /= sn; x2 /= sn; }
        } else {
          a = WW(k, k - 1); x1 = WW(k + 1, k - 1); x2 = (nr == 3) ? WW(k + 2, k - 1) : T(0);
        }
        const T t1 = refl_t<T>(a, x1, x2, nr);
        if (k > ca.ilo) {
          WW(k, k - 1) = a;
          WW(k + 1, k - 1) = T(0);
          if (nr == 3) WW(k + 2, k - 1) = T(0);
        }
        r[0] = t1; r[1] = t1 * x1; r[2] = t1 * x2; r[3] = x1; r[4] = x2;
      }
      rk[b] = nr ? k : 0;
      rn[b] = nr;
      for (int q = 0; q < 5; ++q) rf[b][q] = r[q];
      const size_t li = (size_t)s * ca.B + b;
      ca.logk[li] = nr ? k : 0;
      for (int q = 0; q < 5; ++q) ca.logr[li * 5 + q] = r[q];
    }
    __syncthreads();
    // left updates inside the window: bulge b, column j >= k_b
    for (int idx = tid; idx < ca.B * nw; idx += blockDim.x) {
      const int b = idx / nw, j = ca.wlo + idx % nw;
      const int k = rk[b], nr = rn[b];
      if (!nr || j < k) continue;
      T* h = &WW(k, j);
      const T ss = (nr == 3) ? fma(rf[b][4], h[2], fma(rf[b][3], h[1], h[0])) : fma(rf[b][3], h[1], h[0]);
      h[0] = fma(-ss, rf[b][0], h[0]);
      h[1] = fma(-ss, rf[b][1], h[1]);
      if (nr == 3) h[2] = fma(-ss, rf[b][2], h[2]);
    }
    __syncthreads();
    // right updates inside the window: bulge b, row i <= min(k_b + 3, ihi)
    for (int idx = tid; idx < ca.B * nw; idx += blockDim.x) {
      const int b = idx / nw, i = ca.wlo + idx % nw;
      const int k = rk[b], nr = rn[b];
      if (!nr || i > min(k + 3, ca.ihi)) continue;
      T& h0 = WW(i, k);
      T& h1 = WW(i, k + 1);
      if (nr == 3) {
        T& h2 = WW(i, k + 2);
        const T ss = fma(rf[b][4], h2, fma(rf[b][3], h1, h0));
        h0 = fma(-ss, rf[b][0], h0);
        h1 = fma(-ss, rf[b][1], h1);
        h2 = fma(-ss, rf[b][2], h2);
      } else {
        const T ss = fma(rf[b][3], h1, h0);
        h0 = fma(-ss, rf[b][0], h0);
        h1 = fma(-ss, rf[b][1], h1);
      }
    }
    __syncthreads();
  }
#undef WW
  for (int idx = tid; idx < nw * nw; idx += blockDim.x) {
    const int i = idx % nw, j = idx / nw;
    H[(size_t)(ca.wlo - 1 + j) * n + (ca.wlo - 1 + i)] = W[i + j * ldw];
  }
}

// Far updates of one chunk.  blockIdx.x enumerates tiles of kFarTile columns right of
// the window (left updates on H), then tiles of kFarTile rows above the window
// (right updates on H), then tiles of rows of Z (right updates on Z).
template <class T>
__global__ void __launch_bounds__(256) k_chase_far(ChaseArgs<T> ca, int nleft, int nright, int nz) {
  extern __shared__ unsigned char smraw[];
  const int nw = ca.whi - ca.wlo + 1;
  const int steps = ca.w;
  T* lr = (T*)smraw;                                    // steps*B*5 reflector scalars
  int* lk = (int*)(lr + (size_t)steps * ca.B * 5);      // steps*B positions
  T* seg = (T*)(lk + (((size_t)steps * ca.B + 1) & ~size_t(1)));  // segment
  const int tid = threadIdx.x;
  const int n = ca.n;
  for (int idx = tid; idx < steps * ca.B * 5; idx += blockDim.x) lr[idx] = ca.logr[idx];
  for (int idx = tid; idx < steps * ca.B; idx += blockDim.x) lk[idx] = ca.logk[idx];
  int tile = blockIdx.x;
  if (tile < nleft) {
    // columns c0.. c0+kFarTile-1 right of the window, rows wlo..whi: segment[nw][kFarTile]
    const int c0 = ca.whi + 1 + tile * kFarTile;
    const int nc = min(kFarTile, n - c0 + 1);
    for (int idx = tid; idx < nw * kFarTile; idx += blockDim.x) {
      const int i = idx % nw, c = idx / nw;
      seg[i + c * nw] = (c < nc) ? ca.H[(size_t)(c0 - 1 + c) * n + (ca.wlo - 1 + i)] : T(0);
    }
    __syncthreads();
    for (int s = 0; s < steps; ++s) {
      for (int idx = tid; idx < ca.B * kFarTile; idx += blockDim.x) {
        const int b = idx / kFarTile, c = idx % kFarTile;
        const int k = lk[s * ca.B + b];
        if (!k || c >= nc) continue;
        const T* r = &lr[(s * ca.B + b) * 5];
        const bool three = (k <= ca.ihi - 2);
        T* h = &seg[(k - ca.wlo) + c * nw];
        const T ss = three ? fma(r[4], h[2], fma(r[3], h[1], h[0])) : fma(r[3], h[1], h[0]);
        h[0] = fma(-ss, r[0], h[0]);
        h[1] = fma(-ss, r[1], h[1]);
        if (three) h[2] = fma(-ss, r[2], h[2]);
      }
      __syncthreads();
    }
    for (int idx = tid; idx < nw * kFarTile; idx += blockDim.x) {
      const int i = idx % nw, c = idx / nw;
      if (c < nc) ca.H[(size_t)(c0 - 1 + c) * n + (ca.wlo - 1 + i)] = seg[i + c * nw];
    }
    return;
  }
  tile -= nleft;
  T* M;
  int r0, nrw;
  if (tile < nright) {
    M = ca.H;
    r0 = 1 + tile * kFarTile;
    nrw = min(kFarTile, ca.wlo - r0);
  } else {
    tile -= nright;
    M = ca.Z;
    r0 = 1 + tile * kFarTile;
    nrw = min(kFarTile, n - r0 + 1);
  }
  // rows r0..r0+nrw-1, columns wlo..whi: segment[kFarTile][nw] (row index fastest)
  for (int idx = tid; idx < kFarTile * nw; idx += blockDim.x) {
    const int i = idx % kFarTile, j = idx / kFarTile;
    seg[i + j * kFarTile] = (i < nrw) ? M[(size_t)(ca.wlo - 1 + j) * n + (r0 - 1 + i)] : T(0);
  }
  __syncthreads();
  for (int s = 0; s < steps; ++s) {
    for (int idx = tid; idx < ca.B * kFarTile; idx += blockDim.x) {
      const int b = idx / kFarTile, i = idx % kFarTile;
      const int k = lk[s * ca.B + b];
      if (!k || i >= nrw) continue;
      const T* r = &lr[(s * ca.B + b) * 5];
      const bool three = (k <= ca.ihi - 2);
      T* h = &seg[i + (k - ca.wlo) * kFarTile];
      const T ss = three ? fma(r[4], h[2 * kFarTile], fma(r[3], h[kFarTile], h[0])) : fma(r[3], h[kFarTile], h[0]);
      h[0] = fma(-ss, r[0], h[0]);
      h[kFarTile] = fma(-ss, r[1], h[kFarTile]);
      if (three) h[2 * kFarTile] = fma(-ss, r[2], h[2 * kFarTile]);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < kFarTile * nw; idx += blockDim.x) {
    const int i = idx % kFarTile, j = idx / kFarTile;
    if (i < nrw) M[(size_t)(ca.wlo - 1 + j) * n + (r0 - 1 + i)] = seg[i + j * kFarTile];
  }
}

// Deflation scan on [ilo+1, ihi] (GenericSchur.jl:563-600): the largest k with a
// negligible H[k,k-1] goes to out[0] (0 if none); that entry is zeroed by the host
// driver's next step.
template <class T>
__global__ void k_deflation_scan(const T* __restrict__ H, int n, int ilo, int ihi, int* out) {
  const int k = ilo + 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (k > ihi) return;
  const T eps = sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-07);
  const T fmn = sizeof(T) == 8 ? T(2.2250738585072014e-308) : T(1.17549435e-38);
  const T smallnum = fmn * ((T)n / eps);
#define HG(i, j) H[(size_t)((j) - 1) * n + ((i) - 1)]
  bool split = false;
  const T hk = HG(k, k - 1);
  if (tabs(hk) < smallnum) {
    split = true;
  } else {
    const T hkk = HG(k, k), hkm1 = HG(k - 1, k - 1);
    T t = tabs(hkm1) + tabs(hkk);
    if (t == T(0)) {
      if (k > 2) t += tabs(HG(k - 1, k - 2));
      if (k + 1 <= n) t += tabs(HG(k + 1, k));
    }
    const T ahkkm1 = tabs(hk);
    if (ahkkm1 <= t * eps) {
      const T ahkm1k = tabs(HG(k - 1, k));
      const T ab = fmax(ahkkm1, ahkm1k), ba = fmin(ahkkm1, ahkm1k);
      const T aa = fmax(tabs(hkk), tabs(hkm1 - hkk)), bb = fmin(tabs(hkk), tabs(hkm1 - hkk));
      const T s = aa + bb;
      if (ba * (ab / s) <= fmax(smallnum, eps * (bb * (aa / s)))) split = true;
    }
  }
#undef HG
  if (split) atomicMax(out, k);
}

// C (m x p, ldc) = op(A) (m x q) * B (q x p); op(A) = A or A^T.  64x64 tiles,
// 256 threads, 4x4 outputs per thread, k-slabs of 16 staged in shared memory.
template <class T>
__global__ void __launch_bounds__(256) k_gemm(int m, int p, int q, const T* __restrict__ A, int lda, int transA,
                                              const T* __restrict__ B, int ldb, T* __restrict__ C, int ldc) {
  __shared__ T As[16][64 + 1];
  __shared__ T Bs[16][64 + 1];
  const int tid = threadIdx.x;
  const int tr = tid % 16, tc = tid / 16;  // 16 x 16 threads, 4 x 4 each
  const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
  T acc[4][4];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
  for (int k0 = 0; k0 < q; k0 += 16) {
    for (int idx = tid; idx < 16 * 64; idx += 256) {
      const int kk = idx / 64, ii = idx % 64;
      const int i = i0 + ii, k = k0 + kk;
      T av = T(0);
      if (i < m && k < q) av = transA ? A[(size_t)i * lda + k] : A[(size_t)k * lda + i];
      As[kk][ii] = av;
      const int j = j0 + ii;
      Bs[kk][ii] = (j < p && k < q) ? B[(size_t)j * ldb + k] : T(0);
    }
    __syncthreads();
    for (int kk = 0; kk < 16; ++kk) {
      T a[4], b[4];
      for (int x = 0; x < 4; ++x) a[x] = As[kk][tr + 16 * x];
      for (int y = 0; y < 4; ++y) b[y] = Bs[kk][tc + 16 * y];
      for (int x = 0; x < 4; ++x)
        for (int y = 0; y < 4; ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
    }
    __syncthreads();
  }
  for (int x = 0; x < 4; ++x)
    for (int y = 0; y < 4; ++y) {
      const int i = i0 + tr + 16 * x, j = j0 + tc + 16 * y;
      if (i < m && j < p) C[(size_t)j * ldc + i] = acc[x][y];
    }
}

template <class T>
cudaError_t launch_gemm(int m, int p, int q, const T* A, int lda, int transA, const T* B, int ldb, T* C, int ldc,
                        cudaStream_t s) {
  if (m <= 0 || p <= 0) return cudaSuccess;
  dim3 g((m + 63) / 64, (p + 63) / 64);
  k_gemm<T><<<g, 256, 0, s>>>(m, p, q, A, lda, transA, B, ldb, C, ldc);
  return cudaGetLastError();
}

template <class T>
size_t chase_smem_bytes(int nw) { return sizeof(T) * (size_t)nw * (nw | 1); }

template <class T>
size_t far_smem_bytes(int nw, int w, int B) {
  const size_t steps = w;
  return sizeof(T) * steps * B * 5 + sizeof(int) * ((steps * B + 1) & ~size_t(1)) + sizeof(T) * (size_t)nw * kFarTile;
}

template <class T>
cudaError_t launch_chase_chunk(const ChaseArgs<T>& ca, int num_sms, cudaStream_t s) {
  const int nw = ca.whi - ca.wlo + 1;
  size_t sm = chase_smem_bytes<T>(nw);
  cudaError_t e = cudaFuncSetAttribute(k_chase_chunk<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_chase_chunk<T><<<1, 256, sm, s>>>(ca);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int nleft = (ca.n - ca.whi + kFarTile - 1) / kFarTile;
  const int nright = (ca.wlo - 1 + kFarTile - 1) / kFarTile;
  const int nz = ca.Z ? (ca.n + kFarTile - 1) / kFarTile : 0;
  const int tiles = nleft + nright + nz;
  if (tiles == 0) return cudaSuccess;
  sm = far_smem_bytes<T>(nw, ca.w, ca.B);
  e = cudaFuncSetAttribute(k_chase_far<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_chase_far<T><<<tiles, 256, sm, s>>>(ca, nleft, nright, nz);
  (void)num_sms;
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_deflation_scan(const T* H, int n, int ilo, int ihi, int* out, cudaStream_t s) {
  const int cnt = ihi - ilo;
  if (cnt <= 0) return cudaSuccess;
  k_deflation_scan<T><<<(cnt + 255) / 256, 256, 0, s>>>(H, n, ilo, ihi, out);
  return cudaGetLastError();
}

template cudaError_t launch_chase_chunk<double>(const ChaseArgs<double>&, int, cudaStream_t);
template cudaError_t launch_chase_chunk<float>(const ChaseArgs<float>&, int, cudaStream_t);
template cudaError_t launch_deflation_scan<double>(const double*, int, int, int, int*, cudaStream_t);
template cudaError_t launch_deflation_scan<float>(const float*, int, int, int, int*, cudaStream_t);
template cudaError_t launch_gemm<double>(int, int, int, const double*, int, int, const double*, int, double*, int,
                                         cudaStream_t);
template cudaError_t launch_gemm<float>(int, int, int, const float*, int, int, const float*, int, float*, int,
                                        cudaStream_t);

}  // namespace gsk
