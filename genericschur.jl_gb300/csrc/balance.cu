// Balancing (balance!, src/balance.jl:33-185) and the Balancer's action on
// eigenvectors (lmul!/ldiv!, src/balance.jl:189-261), as used by eigen!
// (src/pirates.jl:63-89).
//
// Permutation search: each step of the reference looks for the last row (first
// column) of the active block whose off-diagonal entries inside the block are all
// zero.  Here one grid pass marks every row (column) that has a nonzero off-diagonal
// entry, a one-CTA pass picks the candidate, and the host swaps and repeats -- one
// step per permutation found, so dense matrices cost two passes.
//
// Scaling: the reference's Gauss-Seidel sweeps (row/column i rescaled by a power of
// two before i+1 is looked at) are kept in order, so one persistent CTA runs them:
// per i two block reductions (the maxima, then the scaled sums of squares giving the
// 2-norms c, r), the power-of-two search on thread 0, and the rescaling of row i
// (columns ilo..n) and column i (rows 1..ihi) by all threads.  A sweep limit turns a
// non-terminating case into an error status instead of a hang.
#include <type_traits>
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

template <class S> __device__ __forceinline__ bool bz(S x);
template <> __device__ __forceinline__ bool bz<double>(double x) { return x == 0.0; }
template <> __device__ __forceinline__ bool bz<double2>(double2 x) { return x.x == 0.0 && x.y == 0.0; }
template <class S> __device__ __forceinline__ double babs(S x);
template <> __device__ __forceinline__ double babs<double>(double x) { return fabs(x); }
template <> __device__ __forceinline__ double babs<double2>(double2 x) { return hypot(x.x, x.y); }
// _findamax (src/norm1est.jl:76-99) compares |x| for real entries and |x|^2 =
// re*re + im*im (unfused) for complex ones, returning the square root of the largest.
template <class S> __device__ __forceinline__ double babs2(S x);
template <> __device__ __forceinline__ double babs2<double>(double x) { return fabs(x); }
template <> __device__ __forceinline__ double babs2<double2>(double2 x) {
  return __dadd_rn(__dmul_rn(x.x, x.x), __dmul_rn(x.y, x.y));
}
template <class S> __device__ __forceinline__ S bscale(S x, double f);
template <> __device__ __forceinline__ double bscale<double>(double x, double f) { return x * f; }
template <> __device__ __forceinline__ double2 bscale<double2>(double2 x, double f) { return make_double2(x.x * f, x.y * f); }

// flag[i] = 1 if row i (rows == 1) or column i (rows == 0) of the block [lo, hi] has a
// nonzero off-diagonal entry inside the block (1-based indices).
template <class S>
__global__ void k_bal_mark(const S* __restrict__ A, int lda, int lo, int hi, int rows, int* __restrict__ flag) {
  const int m = hi - lo + 1;
  const size_t tot = (size_t)m * m;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int i = lo + (int)(idx % m), j = lo + (int)(idx / m);
    if (i == j) continue;
    if (!bz(A[(size_t)(j - 1) * lda + (i - 1)])) flag[rows ? i : j] = 1;
  }
}

// out[0] = the last (rows == 1) / first (rows == 0) index in [lo, hi] without a flag, or 0.
__global__ void k_bal_pick(const int* __restrict__ flag, int lo, int hi, int rows, int* out) {
  __shared__ int best;
  if (threadIdx.x == 0) best = rows ? 0 : 0x7fffffff;
  __syncthreads();
  for (int i = lo + threadIdx.x; i <= hi; i += blockDim.x)
    if (!flag[i]) {
      if (rows) atomicMax(&best, i);
      else atomicMin(&best, i);
    }
  __syncthreads();
  if (threadIdx.x == 0) out[0] = (best == 0x7fffffff) ? 0 : best;
}

// swap columns p, q over rows 1..rows and rows p, q over columns c0..n
template <class S>
__global__ void k_bal_swap(S* A, int lda, int n, int p, int q, int rows, int c0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < rows) {
    S a = A[(size_t)(p - 1) * lda + t], b = A[(size_t)(q - 1) * lda + t];
    A[(size_t)(p - 1) * lda + t] = b;
    A[(size_t)(q - 1) * lda + t] = a;
  }
  const int c = c0 + t;
  if (c <= n) {
    S a = A[(size_t)(c - 1) * lda + (p - 1)], b = A[(size_t)(c - 1) * lda + (q - 1)];
    A[(size_t)(c - 1) * lda + (p - 1)] = b;
    A[(size_t)(c - 1) * lda + (q - 1)] = a;
  }
}

constexpr int kBalT = 512;

template <int NT>
__device__ __forceinline__ void bmax2(double& a, double& b, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { red[w] = a; red[32 + w] = b; }
  __syncthreads();
  a = red[0]; b = red[32];
  for (int q = 1; q < NT / 32; ++q) { a = fmax(a, red[q]); b = fmax(b, red[32 + q]); }
  __syncthreads();
}
template <int NT>
__device__ __forceinline__ void bsum2(double& a, double& b, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { red[w] = a; red[32 + w] = b; }
  __syncthreads();
  a = red[0]; b = red[32];
  for (int q = 1; q < NT / 32; ++q) { a += red[q]; b += red[32 + q]; }
  __syncthreads();
}

// Scaling sweeps on the block [ilo, ihi] (balance.jl:135-181, algo :pr with p = 1).
// D[i-1] *= f per accepted rescaling; st[0] = 0 (ok), 2 (NaN), 3 (sweep limit);
// st[1] = 1 if some factor differed from 1 (the Balancer is not trivial).
template <class S>
__global__ void __launch_bounds__(kBalT) k_bal_scale(S* A, int lda, int n, int ilo, int ihi, double* D, int* st,
                                                     long long max_sweeps) {
  __shared__ double red[64];
  __shared__ double sh_f;
  __shared__ int sh_apply, sh_conv, sh_err, sh_nontriv;
  const int tid = threadIdx.x;
  const double beta = 2.0, factor = 0.95;
  const double sfmin1 = kFmin / kEps;
  const double sfmin2 = sfmin1 * beta;
  const double sfmax2 = 1.0 / sfmin2;
  const int m = ihi - ilo + 1;
  if (tid == 0) { sh_err = 0; sh_nontriv = 0; }
  long long sweeps = 0;
  for (;;) {
    if (tid == 0) sh_conv = 1;
    __syncthreads();
    if (++sweeps > max_sweeps) {
      if (tid == 0) sh_err = 3;
      break;
    }
    for (int i = ilo; i <= ihi; ++i) {
      const S* col = A + (size_t)(i - 1) * lda + (ilo - 1);
      const S* row = A + (size_t)(ilo - 1) * lda + (i - 1);
      double mc = 0.0, mr = 0.0, qc = 0.0, qr = 0.0;
      for (int k = tid; k < m; k += kBalT) {
        mc = fmax(mc, babs(col[k]));
        mr = fmax(mr, babs(row[(size_t)k * lda]));
        if constexpr (!std::is_same<S, double>::value) {
          qc = fmax(qc, babs2(col[k]));
          qr = fmax(qr, babs2(row[(size_t)k * lda]));
        }
      }
      bmax2<kBalT>(mc, mr, red);
      if constexpr (!std::is_same<S, double>::value) bmax2<kBalT>(qc, qr, red);
      double sc = 0.0, sr = 0.0;
      const double ic = mc > 0.0 ? 1.0 / mc : 0.0, ir = mr > 0.0 ? 1.0 / mr : 0.0;
      for (int k = tid; k < m; k += kBalT) {
        const double x = babs(col[k]) * ic, y = babs(row[(size_t)k * lda]) * ir;
        sc = fma(x, x, sc);
        sr = fma(y, y, sr);
      }
      bsum2<kBalT>(sc, sr, red);
      if (tid == 0) {
        double c = mc * sqrt(sc), r = mr * sqrt(sr);
        double ca = mc, ra = mr;
        if constexpr (!std::is_same<S, double>::value) { ca = sqrt(qc); ra = sqrt(qr); }
        int apply = 0;
        double f = 1.0;
        if (c != 0.0 && r != 0.0) {
          double g = r / beta;
          const double s = c + r;
          bool bad = false;
          while (c < r / beta) {
            if (c >= g || fmax(fmax(f, c), ca) >= sfmax2 || fmin(fmin(r, g), ra) <= sfmin2) break;
            const double chk = c + f + ca + r + g + ra;
            if (chk != chk) { bad = true; break; }
            f *= beta; c *= beta; ca *= beta; r /= beta; g /= beta; ra /= beta;
          }
          if (bad) {
            sh_err = 2;
          } else {
            g = c / beta;
            while (r <= c / beta) {
              if (g < r || fmax(r, ra) >= sfmax2 || fmin(fmin(f, c), fmin(g, ca)) <= sfmin2) break;
              f /= beta; c /= beta; g /= beta; ca /= beta; r *= beta; ra *= beta;
            }
            if (f != 1.0) sh_nontriv = 1;
            if (!(c + r >= factor * s)) {
              apply = 1;
              sh_conv = 0;
              D[i - 1] *= f;
            }
          }
        }
        sh_f = f;
        sh_apply = apply;
      }
      __syncthreads();
      if (sh_err) break;
      if (sh_apply) {
        const double f = sh_f, rf = 1.0 / f;
        for (int j = ilo + tid; j <= n; j += kBalT) {
          S* p = A + (size_t)(j - 1) * lda + (i - 1);
          *p = bscale(*p, rf);
        }
        __syncthreads();
        for (int j = 1 + tid; j <= ihi; j += kBalT) {
          S* p = A + (size_t)(i - 1) * lda + (j - 1);
          *p = bscale(*p, f);
        }
      }
      __syncthreads();
    }
    if (sh_err || sh_conv) break;
  }
  if (tid == 0) {
    st[0] = sh_err;
    st[1] = sh_nontriv;
  }
}

// V[r, :] <- d_r V[src[r], :] with d = D or 1/D (n x m complex, ld ldv): the scaling and
// the composed row permutation of lmul!/ldiv! in one gather (into W).
__global__ void k_bal_apply(int n, int m, const double2* __restrict__ V, int ldv, double2* __restrict__ W,
                            const int* __restrict__ src, const double* __restrict__ D, int scale, int inverse) {
  const size_t tot = (size_t)n * m;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx % n), j = (int)(idx / n);
    const int s = src[r];
    double2 v = V[(size_t)j * ldv + s];
    if (scale) {
      const double d = inverse ? 1.0 / D[s] : D[s];
      v = make_double2(v.x * d, v.y * d);
    }
    W[(size_t)j * n + r] = v;
  }
}

// rconde_j = |vl_j^H vr_j| / (|vl_j|_2 |vr_j|_2) (pirates.jl:107-113), warp per column.
__global__ void k_rconde(int n, int m, const double2* __restrict__ VL, const double2* __restrict__ VR, double* out) {
  const int lane = threadIdx.x & 31;
  const int col = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (col >= m) return;
  const double2* l = VL + (size_t)col * n;
  const double2* r = VR + (size_t)col * n;
  double dr = 0.0, di = 0.0, nl = 0.0, nr = 0.0;
  for (int i = lane; i < n; i += 32) {
    const double2 a = l[i], b = r[i];
    dr += a.x * b.x + a.y * b.y;  // conj(a) b
    di += a.x * b.y - a.y * b.x;
    nl += a.x * a.x + a.y * a.y;
    nr += b.x * b.x + b.y * b.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    dr += __shfl_xor_sync(0xffffffffu, dr, o);
    di += __shfl_xor_sync(0xffffffffu, di, o);
    nl += __shfl_xor_sync(0xffffffffu, nl, o);
    nr += __shfl_xor_sync(0xffffffffu, nr, o);
  }
  if (lane == 0) out[col] = hypot(dr, di) / (sqrt(nl) * sqrt(nr));
}

}  // namespace

cudaError_t launch_rconde(int n, int m, const double2* VL, const double2* VR, double* out, cudaStream_t s) {
  k_rconde<<<(m + 7) / 8, 256, 0, s>>>(n, m, VL, VR, out);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_bal_mark(const S* A, int lda, int lo, int hi, int rows, int* flag, int num_sms, cudaStream_t s) {
  k_bal_mark<S><<<4 * num_sms, 256, 0, s>>>(A, lda, lo, hi, rows, flag);
  return cudaGetLastError();
}
cudaError_t launch_bal_pick(const int* flag, int lo, int hi, int rows, int* out, cudaStream_t s) {
  k_bal_pick<<<1, 1024, 0, s>>>(flag, lo, hi, rows, out);
  return cudaGetLastError();
}
template <class S>
cudaError_t launch_bal_swap(S* A, int lda, int n, int p, int q, int rows, int c0, cudaStream_t s) {
  const int cnt = std::max(rows, n - c0 + 1);
  if (cnt <= 0) return cudaSuccess;
  k_bal_swap<S><<<(cnt + 255) / 256, 256, 0, s>>>(A, lda, n, p, q, rows, c0);
  return cudaGetLastError();
}
template <class S>
cudaError_t launch_bal_scale(S* A, int lda, int n, int ilo, int ihi, double* D, int* st, cudaStream_t s) {
  k_bal_scale<S><<<1, kBalT, 0, s>>>(A, lda, n, ilo, ihi, D, st, 100000);
  return cudaGetLastError();
}
cudaError_t launch_bal_apply(int n, int m, const double2* V, int ldv, double2* W, const int* src, const double* D,
                             int scale, int inverse, int num_sms, cudaStream_t s) {
  k_bal_apply<<<4 * num_sms, 256, 0, s>>>(n, m, V, ldv, W, src, D, scale, inverse);
  return cudaGetLastError();
}

template cudaError_t launch_bal_mark<double>(const double*, int, int, int, int, int*, int, cudaStream_t);
template cudaError_t launch_bal_mark<double2>(const double2*, int, int, int, int, int*, int, cudaStream_t);
template cudaError_t launch_bal_swap<double>(double*, int, int, int, int, int, int, cudaStream_t);
template cudaError_t launch_bal_swap<double2>(double2*, int, int, int, int, int, int, cudaStream_t);
template cudaError_t launch_bal_scale<double>(double*, int, int, int, int, double*, int*, cudaStream_t);
template cudaError_t launch_bal_scale<double2>(double2*, int, int, int, int, double*, int*, cudaStream_t);

}  // namespace gsk
