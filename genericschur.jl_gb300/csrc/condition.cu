// Condition estimators of a Schur form: eigvalscond and subspacesep (src/ordschur.jl:84-140).
//
// Both rest on the triangular Sylvester solves trsylvester! (A X - X B = scale C) and
// adjtrsylvester! (A^H X - X B^H = scale C) of src/sylvester.jl:11-139, A and B upper
// triangular (only their upper triangles are read).  X(k, l) needs X(k', l) for k' > k and
// X(k, l') for l' < l, so the solve runs in 32 x 32 tiles by anti-diagonal levels of the
// tile grid, one launch per level, one CTA per tile (k_trsyl_level):
//   1. rhs = C_KL - sum_{K' > K} A_KK' X_K'L + sum_{L' < L} X_KL' B_L'L over 32-wide panels
//      staged in shared memory (FP64 FMA bound: 8 m p (m + p) / 2 real flops per solve
//      for complex data);
//   2. the tile's own triangular system by element waves along its anti-diagonals (warp 0),
//      with the reference's perturbation of small diagonal differences to smin.
// The adjoint solve is the forward one on P A^H P, P B^H P and P C P (P the reversal
// permutation): k_adj_copy builds the first two, the third is an index map.  With possign
// (A X + X B = scale C) the B terms change sign.
// The reference rescales the whole right-hand side when an entry would overflow
// (scaloc = 1 / |v|_1 when |a11|_1 < 1 < |v|_1 and |v|_1 > bignum |a11|_1).  The tiled
// solve flags that case (and any non-finite entry) instead; the host then reruns the
// solve in the reference's element order with that rescaling (k_trsyl_exact, one CTA).
// norm1est! (src/norm1est.jl:21-99) runs on the host over these solves with the vector
// steps below (fills, sign vectors, one-norm and _findamax in one deterministic CTA).
#include "gs_internal.h"
#include "device_common.cuh"

namespace gsk {
namespace {

constexpr int kTs = 32;   // tile edge
constexpr int kSyT = 256; // threads of the tile CTAs
constexpr int kN1T = 1024;

template <class S> struct Sc;
template <> struct Sc<double> {
  static __device__ __forceinline__ double zero() { return 0.0; }
  static __device__ __forceinline__ double from(double r) { return r; }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ double fnma(double a, double b, double c) { return ::fma(-a, b, c); }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __device__ __forceinline__ double conj(double a) { return a; }
  static __device__ __forceinline__ double abs1(double a) { return fabs(a); }
  static __device__ __forceinline__ double mod(double a) { return fabs(a); }
  static __device__ __forceinline__ double key(double a) { return fabs(a); }  // _findamax's key
  static __device__ __forceinline__ double keyroot(double k) { return k; }
  static __device__ __forceinline__ double scal(double a, double s) { return a * s; }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ bool finite(double a) { return isfinite(a); }
  static __device__ __forceinline__ double shfl_xor(double a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
};
template <> struct Sc<double2> {
  static __device__ __forceinline__ double2 zero() { return make_double2(0.0, 0.0); }
  static __device__ __forceinline__ double2 from(double r) { return make_double2(r, 0.0); }
  static __device__ __forceinline__ double2 fma(double2 a, double2 b, double2 c) { return zfma(a, b, c); }
  static __device__ __forceinline__ double2 fnma(double2 a, double2 b, double2 c) { return zfms(a, b, c); }
  static __device__ __forceinline__ double2 add(double2 a, double2 b) { return zadd(a, b); }
  static __device__ __forceinline__ double2 sub(double2 a, double2 b) { return zsub(a, b); }
  static __device__ __forceinline__ double2 conj(double2 a) { return zconj(a); }
  static __device__ __forceinline__ double abs1(double2 a) { return fabs(a.x) + fabs(a.y); }
  static __device__ __forceinline__ double mod(double2 a) { return hypot(a.x, a.y); }
  static __device__ __forceinline__ double key(double2 a) { return __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)); }
  static __device__ __forceinline__ double keyroot(double k) { return sqrt(k); }
  static __device__ __forceinline__ double2 scal(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
  static __device__ __forceinline__ double2 div(double2 a, double2 b) { return zdiv(a, b); }
  static __device__ __forceinline__ bool finite(double2 a) { return isfinite(a.x) && isfinite(a.y); }
  static __device__ __forceinline__ double2 shfl_xor(double2 a, int o) {
    return make_double2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
  }
};

template <class S> __device__ __forceinline__ S* cptr(const SylvArgs<S>& P, int i, int j) {
  return P.flip ? P.C + (size_t)(P.m - 1 - i) + (size_t)(P.p - 1 - j) * P.ldc : P.C + i + (size_t)j * P.ldc;
}

// Entrywise max modulus of a rows x cols block (Julia's norm(M, Inf) of a matrix), as the
// bits of a non-negative double (NaN orders above Inf).
template <class S>
__global__ void k_cond_maxabs(const S* __restrict__ M, int ld, int rows, int cols, unsigned long long* out) {
  using O = Sc<S>;
  double v = 0.0;
  const size_t tot = (size_t)rows * cols;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const double a = fabs(O::mod(M[(e % rows) + (e / rows) * (size_t)ld]));
    if (a > v || a != a) v = a;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, v, o);
    if (w > v || w != w) v = w;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(v));
}

// Ap = P M^H P for the m x m block M (ld): Ap(i, j) = conj(M(m-1-j, m-1-i)).
template <class S>
__global__ void k_adj_copy(const S* __restrict__ M, int ld, int m, S* __restrict__ Ap) {
  const size_t tot = (size_t)m * m;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % m), j = (int)(e / m);
    Ap[e] = Sc<S>::conj(M[(size_t)(m - 1 - j) + (size_t)(m - 1 - i) * ld]);
  }
}

// One anti-diagonal level d of the tile grid: tiles (K, L) with (mT - 1 - K) + L = d,
// L = Lmin + blockIdx.x.  Dynamic shared memory: three 32 x 33 scalar panels.
template <class S>
__global__ void __launch_bounds__(kSyT) k_trsyl_level(SylvArgs<S> P, int d, int Lmin) {
  using O = Sc<S>;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  S(*Pa)[kTs + 1] = reinterpret_cast<S(*)[kTs + 1]>(sm_raw);
  S(*Pb)[kTs + 1] = Pa + kTs;
  S(*R)[kTs + 1] = Pb + kTs;
  const int t = threadIdx.x;
  const int L = Lmin + blockIdx.x;
  const int K = P.mT - 1 - d + L;
  const int r0 = K * kTs, c0 = L * kTs;
  const int mloc = min(kTs, P.m - r0), ploc = min(kTs, P.p - c0);
  const int cc = t >> 3, rb = (t & 7) * 4;
  S acc[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = (rb + q < mloc && cc < ploc) ? *cptr(P, r0 + rb + q, c0 + cc) : O::zero();
  // - sum over the row tiles below: A(r0.., jb..) X(jb.., c0..)
  for (int jb = r0 + kTs; jb < P.m; jb += kTs) {
    const int jl = min(kTs, P.m - jb);
    for (int e = t; e < kTs * kTs; e += kSyT) {
      const int i = e & (kTs - 1), j = e >> 5;
      Pa[i][j] = (i < mloc && j < jl) ? P.A[(size_t)(r0 + i) + (size_t)(jb + j) * P.lda] : O::zero();
      Pb[i][j] = (i < jl && j < ploc) ? *cptr(P, jb + i, c0 + j) : O::zero();
    }
    __syncthreads();
#pragma unroll 4
    for (int j = 0; j < kTs; ++j) {
      const S x = Pb[j][cc];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = O::fnma(Pa[rb + q][j], x, acc[q]);
    }
    __syncthreads();
  }
  // + sum over the column tiles to the left: X(r0.., jb..) B(jb.., c0..)
  for (int jb = 0; jb < c0; jb += kTs) {
    for (int e = t; e < kTs * kTs; e += kSyT) {
      const int i = e & (kTs - 1), j = e >> 5;
      Pa[i][j] = (i < mloc) ? *cptr(P, r0 + i, jb + j) : O::zero();
      Pb[i][j] = (j < ploc) ? P.B[(size_t)(jb + i) + (size_t)(c0 + j) * P.ldb] : O::zero();
    }
    __syncthreads();
    if (P.pos) {
#pragma unroll 4
      for (int j = 0; j < kTs; ++j) {
        const S b = Pb[j][cc];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = O::fnma(Pa[rb + q][j], b, acc[q]);
      }
    } else {
#pragma unroll 4
      for (int j = 0; j < kTs; ++j) {
        const S b = Pb[j][cc];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = O::fma(Pa[rb + q][j], b, acc[q]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) R[rb + q][cc] = acc[q];
  // diagonal blocks (upper triangles)
  for (int e = t; e < kTs * kTs; e += kSyT) {
    const int i = e & (kTs - 1), j = e >> 5;
    Pa[i][j] = (i <= j && j < mloc) ? P.A[(size_t)(r0 + i) + (size_t)(r0 + j) * P.lda] : O::zero();
    Pb[i][j] = (i <= j && j < ploc) ? P.B[(size_t)(c0 + i) + (size_t)(c0 + j) * P.ldb] : O::zero();
  }
  __syncthreads();
  if (t < 32) {
    // element waves: element (k, l) on wave (mloc - 1 - k) + l; lane = l
    const int l = t;
    int fl = 0;
    for (int w = 0; w < mloc + ploc - 1; ++w) {
      const int kk = w - l;
      if (l < ploc && kk >= 0 && kk < mloc) {
        const int k = mloc - 1 - kk;
        S suml = O::zero(), sumr = O::zero();
        for (int j = k + 1; j < mloc; ++j) suml = O::fma(Pa[k][j], R[j][l], suml);
        for (int j = 0; j < l; ++j) sumr = O::fma(R[k][j], Pb[j][l], sumr);
        const S v = O::sub(R[k][l], P.pos ? O::add(suml, sumr) : O::sub(suml, sumr));
        S a11 = P.pos ? O::add(Pa[k][k], Pb[l][l]) : O::sub(Pa[k][k], Pb[l][l]);
        double da11 = O::abs1(a11);
        if (P.le ? (da11 <= P.smin) : (da11 < P.smin)) {
          a11 = O::from(P.smin);
          da11 = P.smin;
          fl |= 1;
        }
        const double db = O::abs1(v);
        if (da11 < 1.0 && db > 1.0 && db > P.bignum * da11) fl |= 2;
        const S x = O::div(v, a11);
        if (!O::finite(x)) fl |= 4;
        R[k][l] = x;
      }
      __syncwarp();
    }
    fl = __reduce_or_sync(0xffffffffu, fl);
    if (t == 0 && fl) atomicOr(P.flag, fl);
  }
  __syncthreads();
  for (int e = t; e < kTs * kTs; e += kSyT) {
    const int i = e & (kTs - 1), j = e >> 5;
    if (i < mloc && j < ploc) *cptr(P, r0 + i, c0 + j) = R[i][j];
  }
}

template <class S>
__device__ __forceinline__ S block_sum_s(S v, S* red) {
  using O = Sc<S>;
  for (int o = 16; o > 0; o >>= 1) v = O::add(v, O::shfl_xor(v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  S r = red[0];
  for (int q = 1; q < (int)(blockDim.x >> 5); ++q) r = O::add(r, red[q]);
  return r;
}

// The reference's element order (l ascending, k descending) with its overflow rescaling
// of the whole right-hand side; one CTA.  out[0] = scale.
template <class S>
__global__ void __launch_bounds__(kSyT) k_trsyl_exact(SylvArgs<S> P, double* out) {
  using O = Sc<S>;
  __shared__ S red[kSyT / 32];
  __shared__ S sh_x;
  __shared__ double sh_scaloc;
  const int t = threadIdx.x;
  double scale = 1.0;
  int fl = 0;
  for (int l = 0; l < P.p; ++l)
    for (int k = P.m - 1; k >= 0; --k) {
      S suml = O::zero(), sumr = O::zero();
      for (int j = k + 1 + t; j < P.m; j += kSyT) suml = O::fma(P.A[(size_t)k + (size_t)j * P.lda], *cptr(P, j, l), suml);
      for (int j = t; j < l; j += kSyT) sumr = O::fma(*cptr(P, k, j), P.B[(size_t)j + (size_t)l * P.ldb], sumr);
      suml = block_sum_s(suml, red);
      sumr = block_sum_s(sumr, red);
      if (t == 0) {
        const S v = O::sub(*cptr(P, k, l), P.pos ? O::add(suml, sumr) : O::sub(suml, sumr));
        S a11 = P.pos ? O::add(P.A[(size_t)k + (size_t)k * P.lda], P.B[(size_t)l + (size_t)l * P.ldb])
                      : O::sub(P.A[(size_t)k + (size_t)k * P.lda], P.B[(size_t)l + (size_t)l * P.ldb]);
        double da11 = O::abs1(a11);
        if (P.le ? (da11 <= P.smin) : (da11 < P.smin)) {
          a11 = O::from(P.smin);
          da11 = P.smin;
          fl |= 1;
        }
        double scaloc = 1.0;
        const double db = O::abs1(v);
        if (da11 < 1.0 && db > 1.0 && db > P.bignum * da11) scaloc = 1.0 / db;
        sh_x = O::div(O::scal(v, scaloc), a11);
        sh_scaloc = scaloc;
      }
      __syncthreads();
      const double scaloc = sh_scaloc;
      if (scaloc != 1.0) {
        for (size_t e = t; e < (size_t)P.m * P.p; e += kSyT) {
          S* c = cptr(P, (int)(e % P.m), (int)(e / P.m));
          *c = O::scal(*c, scaloc);
        }
        scale *= scaloc;
        __syncthreads();
      }
      if (t == 0) *cptr(P, k, l) = sh_x;
      __syncthreads();
    }
  if (t == 0) {
    out[0] = scale;
    if (fl) atomicOr(P.flag, fl);
  }
}

// ---- norm1est! vector steps ----------------------------------------------------
template <class S>
__global__ void k_n1_fill(S* x, long long N, double v) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    x[i] = Sc<S>::from(v);
}
template <class S>
__global__ void k_n1_unit(S* x, long long N, long long j0) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    x[i] = Sc<S>::from(i == j0 ? 1.0 : 0.0);
}
// v_i = (-1)^i (1 + i / (N - 1)), 0-based (norm1est.jl:63-68)
template <class S>
__global__ void k_n1_alt(S* x, long long N) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const double v = 1.0 + (double)i / (double)(N - 1);
    x[i] = Sc<S>::from((i & 1) ? -v : v);
  }
}
// x_i <- x_i / |x_i| where |x_i| > tiny, else 1 (norm1est.jl:30-37)
template <class S>
__global__ void k_n1_sign(S* x, long long N, double tiny) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const double a = Sc<S>::mod(x[i]);
    x[i] = a > tiny ? Sc<S>::scal(x[i], 1.0 / a) : Sc<S>::from(1.0);
  }
}

// One CTA: out[0] = sum |x_i|; out[1] = _findamax value, out[2] = its first index,
// out[3] = |x[jlast]| (jlast >= 0).
template <class S>
__global__ void __launch_bounds__(kN1T) k_n1_stats(const S* __restrict__ x, long long N, long long jlast, double* out) {
  using O = Sc<S>;
  __shared__ double rs[kN1T / 32], rk[kN1T / 32];
  __shared__ long long ri[kN1T / 32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  double s = 0.0, kmax = -1.0;
  long long imax = -1;
  for (long long i = t; i < N; i += kN1T) {
    s += O::mod(x[i]);
    const double k = O::key(x[i]);
    if (imax < 0 || k > kmax) { kmax = k; imax = i; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    const double k2 = __shfl_xor_sync(0xffffffffu, kmax, o);
    const long long i2 = __shfl_xor_sync(0xffffffffu, imax, o);
    if (i2 >= 0 && (imax < 0 || k2 > kmax || (k2 == kmax && i2 < imax))) { kmax = k2; imax = i2; }
  }
  if (lane == 0) { rs[w] = s; rk[w] = kmax; ri[w] = imax; }
  __syncthreads();
  if (t == 0) {
    double S0 = rs[0], K0 = rk[0];
    long long I0 = ri[0];
    for (int q = 1; q < kN1T / 32; ++q) {
      S0 += rs[q];
      if (ri[q] >= 0 && (I0 < 0 || rk[q] > K0 || (rk[q] == K0 && ri[q] < I0))) { K0 = rk[q]; I0 = ri[q]; }
    }
    out[0] = S0;
    out[1] = O::keyroot(K0);
    out[2] = (double)I0;
    out[3] = jlast >= 0 ? O::mod(x[jlast]) : 0.0;
  }
}

// Frobenius norm of x (N scalars) without overflow: max |component|, then the scaled sum
// of squares (one CTA).
template <class S>
__global__ void __launch_bounds__(kN1T) k_cond_fro(const S* __restrict__ x, long long N, double* out) {
  __shared__ double red[kN1T / 32];
  const double* xr = reinterpret_cast<const double*>(x);
  const long long M = N * (long long)(sizeof(S) / sizeof(double));
  const int t = threadIdx.x;
  double mx = 0.0;
  for (long long i = t; i < M; i += kN1T) mx = fmax(mx, fabs(xr[i]));
  mx = block_max<kN1T>(mx, red);
  double ss = 0.0;
  if (mx > 0.0 && isfinite(mx)) {
    const double inv = 1.0 / mx;
    for (long long i = t; i < M; i += kN1T) {
      const double v = xr[i] * inv;
      ss = fma(v, v, ss);
    }
  }
  ss = block_sum<kN1T>(ss, red);
  if (t == 0) out[0] = (mx > 0.0 && isfinite(mx)) ? mx * sqrt(ss) : mx;
}

int grid_for(size_t work, int nsm) {
  const size_t g = (work + 255) / 256;
  return (int)std::max<size_t>(1, std::min<size_t>(g, (size_t)nsm * 8));
}

}  // namespace

template <class S>
cudaError_t launch_cond_maxabs(const S* M, int ld, int rows, int cols, unsigned long long* out, int nsm, cudaStream_t s) {
  if ((size_t)rows * cols == 0) return cudaSuccess;
  k_cond_maxabs<S><<<grid_for((size_t)rows * cols, nsm), 256, 0, s>>>(M, ld, rows, cols, out);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_adj_copy(const S* M, int ld, int m, S* Ap, int nsm, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  k_adj_copy<S><<<grid_for((size_t)m * m, nsm), 256, 0, s>>>(M, ld, m, Ap);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_trsyl_levels(const SylvArgs<S>& P, cudaStream_t s) {
  const size_t smem = 3 * kTs * (kTs + 1) * sizeof(S);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_trsyl_level<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  for (int d = 0; d <= P.mT + P.pT - 2; ++d) {
    const int Lmin = std::max(0, d - (P.mT - 1)), Lmax = std::min(P.pT - 1, d);
    k_trsyl_level<S><<<Lmax - Lmin + 1, kSyT, smem, s>>>(P, d, Lmin);
  }
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_trsyl_exact(const SylvArgs<S>& P, double* out, cudaStream_t s) {
  k_trsyl_exact<S><<<1, kSyT, 0, s>>>(P, out);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_n1_step(int op, S* x, long long N, double arg, int nsm, cudaStream_t s) {
  const int g = grid_for((size_t)N, nsm);
  switch (op) {
    case N1_FILL: k_n1_fill<S><<<g, 256, 0, s>>>(x, N, arg); break;
    case N1_UNIT: k_n1_unit<S><<<g, 256, 0, s>>>(x, N, (long long)arg); break;
    case N1_ALT: k_n1_alt<S><<<g, 256, 0, s>>>(x, N); break;
    case N1_SIGN: k_n1_sign<S><<<g, 256, 0, s>>>(x, N, arg); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_n1_stats(const S* x, long long N, long long jlast, double* out, cudaStream_t s) {
  k_n1_stats<S><<<1, kN1T, 0, s>>>(x, N, jlast, out);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_cond_fro(const S* x, long long N, double* out, cudaStream_t s) {
  k_cond_fro<S><<<1, kN1T, 0, s>>>(x, N, out);
  return cudaGetLastError();
}

#define GS_COND_INST(S)                                                                                       \
  template cudaError_t launch_cond_maxabs<S>(const S*, int, int, int, unsigned long long*, int, cudaStream_t); \
  template cudaError_t launch_adj_copy<S>(const S*, int, int, S*, int, cudaStream_t);                         \
  template cudaError_t launch_trsyl_levels<S>(const SylvArgs<S>&, cudaStream_t);                              \
  template cudaError_t launch_trsyl_exact<S>(const SylvArgs<S>&, double*, cudaStream_t);                      \
  template cudaError_t launch_n1_step<S>(int, S*, long long, double, int, cudaStream_t);                      \
  template cudaError_t launch_n1_stats<S>(const S*, long long, long long, double*, cudaStream_t);             \
  template cudaError_t launch_cond_fro<S>(const S*, long long, double*, cudaStream_t);
GS_COND_INST(double)
GS_COND_INST(double2)
#undef GS_COND_INST

}  // namespace gsk
