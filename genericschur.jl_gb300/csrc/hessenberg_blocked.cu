// Blocked Householder Hessenberg reduction of one large matrix (n > 128), with the
// Schur vectors Z = H(1) H(2) ... accumulated alongside.
//
// Reference semantics: _hessenberg! (hessenberg.jl:3-17) generates reflector i from
// column i of the matrix updated by reflectors 1..i-1 (_reflector!, householder.jl:12-54)
// and applies it from both sides; _materializeQ (hessenberg.jl:150-166) forms
// Q = H(1) ... H(n-2).  The blocked form below produces the same reflectors in exact
// arithmetic, with most of the work moved into matrix products (the compact-WY panel
// scheme of LAPACK's xGEHRD/xLAHR2, restated):
//
// For a panel of nb columns starting at c0, with Q_j = H_0 ... H_{j-1} = I - V_j T_j V_j^T
// and Y_j = A V_j T_j (A the matrix at the start of the panel):
//   column c = c0 + j of Q_j^T A Q_j is  b = A e_c - Y_j V_j^T e_c, then on rows > c0
//   b <- b - V_j T_j^T V_j^T b;  the reflector of b[c+1:] gives (tau_j, v_j);
//   Y[:, j] = tau_j (A v_j - Y_j (V_j^T v_j)),  T[:j, j] = -tau_j T_j V_j^T v_j, T[j,j] = tau_j.
// After the panel the trailing columns k >= c0 + nb become (I - V T^T V^T)(A - Y V^T) and
// Z <- Z - (Z V) T V^T: seven matrix products per panel (k_gemm_ex, split over K where
// one output dimension is the panel width).
//
// The panel itself is one cooperative launch (all CTAs resident) with four grid barriers
// per column:
//   P1  b = A[:,c] - Y V[c,:]^T (rows), partial sums of V^T b            | barrier
//   P2  w = V^T b, u = T^T w (each CTA), b -= V u on rows > c0, and the
//       (scale, sum of squares) pairs of b[c+2:] (one-pass, no overflow)   | barrier
//   P3  the reflector (every CTA reduces the same partials in the same
//       order, so all agree), v into V[:, j] and A[:, c], partials of V^T v | barrier
//   P4  A[:, c+1:] v over (32-row block, column chunk) warp tasks          | barrier
//   P5  Y[:, j] and T[:, j]; fused with the next column's P1.
// Every row is owned by the same thread in every row phase, so a thread's own b and Y
// entries need no barrier.  Barrier waits give up after ~4 s and raise an error word.
#include <algorithm>
#include <cstdlib>

#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kHbNT = 256;       // threads per CTA of the panel kernel
constexpr int kHbNbMax = 32;     // panel width
constexpr int kGT = 64;          // GEMM tile edge

template <class T> struct HbLim;
template <> struct HbLim<double> {
  static __device__ __forceinline__ double big() { return 1.7976931348623157e308; }
  static __device__ __forceinline__ double fmin() { return 2.2250738585072014e-308; }
  static __device__ __forceinline__ double eps() { return 2.220446049250313e-16; }
};
template <> struct HbLim<float> {
  static __device__ __forceinline__ float big() { return 3.40282347e38f; }
  static __device__ __forceinline__ float fmin() { return 1.17549435e-38f; }
  static __device__ __forceinline__ float eps() { return 1.1920929e-07f; }
};

struct HbCtl {
  unsigned count, gen;
  int err;
};

// Grid barrier of a cooperative launch: arrival counter + generation word; the wait
// gives up after ~4 s (then every later barrier of the launch is skipped).
__device__ void hb_barrier(HbCtl* ctl, unsigned nblocks) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = &ctl->gen;
    volatile int* verr = &ctl->err;
    if (*verr == 0) {
      const unsigned g = *vgen;
      __threadfence();
      if (atomicAdd(&ctl->count, 1u) == nblocks - 1) {
        ctl->count = 0;
        __threadfence();
        atomicAdd(&ctl->gen, 1u);
      } else {
        long long it = 0;
        while (*vgen == g) {
          if (++it > (1LL << 25)) { atomicOr(&ctl->err, 1); break; }
          __nanosleep(128);
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
}

// Sum of squares kept as S * 4^E with E an exponent (frexp) and S < 4 * count: adding a
// value or merging two sums needs only exponent arithmetic and exact power-of-two
// scaling, no division; overflow and underflow cannot occur.  Inf/NaN give NaN.
template <class T>
struct Ssq {
  int E;
  T S;
};
template <class T>
__device__ __forceinline__ void ssq_init(Ssq<T>& q) { q.E = -(1 << 20); q.S = T(0); }
template <class T>
__device__ __forceinline__ void ssq_add(Ssq<T>& q, T a) {
  if (a == T(0)) return;
  if (!(fabs(a) <= HbLim<T>::big())) { q.E = 1 << 20; q.S = a - a; return; }
  int e;
  const T m = frexp(a, &e);  // |m| in [0.5, 1)
  if (e > q.E) {
    q.S = ldexp(q.S, 2 * (q.E - e)) + m * m;
    q.E = e;
  } else {
    const T x = ldexp(m, e - q.E);
    q.S = fma(x, x, q.S);
  }
}
template <class T>
__device__ __forceinline__ void ssq_merge(Ssq<T>& q, int E2, T S2) {
  if (S2 == T(0) && E2 < (1 << 20)) return;
  if (E2 > q.E) {
    q.S = ldexp(q.S, 2 * (q.E - E2)) + S2;
    q.E = E2;
  } else {
    q.S += ldexp(S2, 2 * (E2 - q.E));
  }
}

// Warp sum, identical in every lane (xor butterfly: each step adds a commutative pair).
template <class T>
__device__ __forceinline__ T warp_sum(T x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// dst[i] = sum_g part[g * kHbNbMax + i], i < cnt: lane = value, warps over g with stride
// 8, then the 8 warp sums in order -- the same order in every CTA.  scr: 8 x 32.
template <class T>
__device__ void grid_sum_vec(const T* __restrict__ part, int G, int cnt, T* scr, T* dst) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T acc = T(0);
  if (lane < cnt)
    for (int g = wid; g < G; g += kHbNT / 32) acc += part[(size_t)g * kHbNbMax + lane];
  scr[wid * 32 + lane] = acc;
  __syncthreads();
  if (threadIdx.x < cnt) {
    T sum = T(0);
    for (int w = 0; w < kHbNT / 32; ++w) sum += scr[w * 32 + threadIdx.x];
    dst[threadIdx.x] = sum;
  }
  __syncthreads();
}

// CTA partial: part[i] = sum over warps of scr[w][i] (each warp's lane i holds acc).
template <class T>
__device__ void cta_partial(T acc, int cnt, T* scr, T* part) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  scr[wid * 32 + lane] = acc;
  __syncthreads();
  if (threadIdx.x < cnt) {
    T sum = T(0);
    for (int w = 0; w < kHbNT / 32; ++w) sum += scr[w * 32 + threadIdx.x];
    part[threadIdx.x] = sum;
  }
  __syncthreads();
}

template <class T>
struct HbArgs {
  int n, c0, nb;
  T* A;
  int lda;
  T* Y;       // n x kHbNbMax, ld n
  T* V;       // n x kHbNbMax, ld n
  T* Tm;      // kHbNbMax x kHbNbMax, ld kHbNbMax (written by CTA 0 at the end of the panel)
  T* b;       // n
  T* partW;   // G x kHbNbMax
  T* partT;   // G x kHbNbMax
  T* partN;   // G x 2 (E as a value, S)
  T* mvp;     // CS x n
  int CS;
  T* tau_out;
  HbCtl* ctl;
};

template <class T>
__global__ void __launch_bounds__(kHbNT, 2) k_hess_panel(HbArgs<T> a) {
  __shared__ T scr[(kHbNT / 32) * 32];
  __shared__ T mred[kHbNT / 32][32];
  __shared__ T vc[kHbNbMax], wv[kHbNbMax], uv[kHbNbMax], tv[kHbNbMax];
  __shared__ T Ts[kHbNbMax][kHbNbMax + 1];  // this panel's T, the same in every CTA
  __shared__ int sE[kHbNT / 32];
  __shared__ T sS[kHbNT / 32];
  __shared__ T refl[4];
  const int n = a.n, c0 = a.c0, G = gridDim.x, bid = blockIdx.x, tid = threadIdx.x;
  const size_t ldv = (size_t)n;
  const int lane = tid & 31, wid = tid >> 5;
  // rows of this CTA: r = bid + G * (wid + 8 m), one row per warp at a time, lane = i
  const int rstep = G * (kHbNT / 32);
  const int rfirst = bid + G * wid;
  for (int x = tid; x < kHbNbMax * (kHbNbMax + 1); x += kHbNT) (&Ts[0][0])[x] = T(0);
  __syncthreads();
  T tau_prev = T(0);
  for (int j = 0; j <= a.nb; ++j) {
    const int c = c0 + j;
    // ---------------- P5 of column j-1 (Y, T) fused with P1 of column j
    if (j > 0) {
      grid_sum_vec<T>(a.partT, G, j - 1, scr, tv);
      if (tid < j - 1) {
        // T[i, j-1] = -tau (T t)_i, T upper triangular: sum over k = i .. j-2
        T s = T(0);
        for (int k = tid; k < j - 1; ++k) s = fma(Ts[tid][k], tv[k], s);
        Ts[tid][j - 1] = -tau_prev * s;
      }
      if (tid == 0) Ts[j - 1][j - 1] = tau_prev;
    }
    if (j < a.nb && tid < j) vc[tid] = a.V[(size_t)c + tid * ldv];
    __syncthreads();
    T accw = T(0);
    for (int r = rfirst; r < n; r += rstep) {
      T y = T(0);
      if (j > 0) {
        const int jj = j - 1;
        T term = T(0);
        for (int cs = lane; cs < a.CS; cs += 32) term += a.mvp[(size_t)cs * n + r];
        if (lane < jj) term = fma(-a.Y[r + lane * ldv], tv[lane], term);
        y = tau_prev * warp_sum(term);
        if (lane == 0) a.Y[r + jj * ldv] = y;
      }
      if (j < a.nb) {
        T yi = T(0);
        if (lane < j) yi = (lane == j - 1) ? y : a.Y[r + lane * ldv];
        const T bb = a.A[(size_t)c * a.lda + r] - warp_sum(yi * (lane < j ? vc[lane] : T(0)));
        if (lane == 0) a.b[r] = bb;
        if (r >= c0 + 1 && lane < j) accw = fma(a.V[r + lane * ldv], bb, accw);
      }
    }
    if (j == a.nb) {
      __syncthreads();
      if (bid == 0)
        for (int x = tid; x < kHbNbMax * kHbNbMax; x += kHbNT) a.Tm[x] = Ts[x % kHbNbMax][x / kHbNbMax];
      break;
    }
    cta_partial<T>(accw, j, scr, a.partW + (size_t)bid * kHbNbMax);
    hb_barrier(a.ctl, G);
    // ---------------- P2: w = V^T b, u = T^T w, b -= V u (rows > c0), sum of squares of b[c+2:]
    grid_sum_vec<T>(a.partW, G, j, scr, wv);
    if (tid < j) {
      T s = T(0);
      for (int k = 0; k <= tid; ++k) s = fma(Ts[k][tid], wv[k], s);
      uv[tid] = s;
    }
    __syncthreads();
    Ssq<T> q;
    ssq_init(q);
    for (int r = rfirst; r < n; r += rstep) {
      if (r >= c0 + 1) {
        const T vu = (lane < j) ? a.V[r + lane * ldv] * uv[lane] : T(0);
        const T bb = a.b[r] - warp_sum(vu);
        if (lane == 0) {
          a.b[r] = bb;
          if (r >= c + 2) ssq_add(q, bb);
        }
      }
    }
    if (lane == 0) { sE[wid] = q.E; sS[wid] = q.S; }
    __syncthreads();
    if (tid == 0) {
      Ssq<T> m;
      ssq_init(m);
      for (int w = 0; w < kHbNT / 32; ++w) ssq_merge(m, sE[w], sS[w]);
      a.partN[2 * bid] = (T)m.E;
      a.partN[2 * bid + 1] = m.S;
    }
    hb_barrier(a.ctl, G);
    // ---------------- P3: the reflector of b[c+1:], v into V[:, j] and A[:, c]
    {
      Ssq<T> m;
      ssq_init(m);
      for (int g = tid; g < G; g += kHbNT) ssq_merge(m, (int)a.partN[2 * g], a.partN[2 * g + 1]);
      for (int o = 16; o > 0; o >>= 1) {
        const int E2 = __shfl_down_sync(0xffffffffu, m.E, o);
        const T S2 = __shfl_down_sync(0xffffffffu, m.S, o);
        if (lane < o) ssq_merge(m, E2, S2);
      }
      if (lane == 0) { sE[wid] = m.E; sS[wid] = m.S; }
      __syncthreads();
      if (tid == 0) {
        Ssq<T> t;
        ssq_init(t);
        for (int w = 0; w < kHbNT / 32; ++w) ssq_merge(t, sE[w], sS[w]);
        const T xnorm = (t.S == T(0)) ? T(0) : ldexp(sqrt(t.S), t.E);
        T alpha = a.b[c + 1];
        T tau = T(0), beta = alpha, f = T(0);
        if (xnorm != T(0)) {
          const T sfmin = T(2) * HbLim<T>::fmin() / HbLim<T>::eps();
          const T rsfmin = T(1) / sfmin;
          T xn = xnorm;
          beta = -copysign(hypot(alpha, xn), alpha);
          int kount = 0;
          T fs = T(1);
          if (fabs(beta) < sfmin) {
            do {
              ++kount;
              beta *= rsfmin;
              alpha *= rsfmin;
              xn *= rsfmin;
              fs *= rsfmin;
            } while (fabs(beta) < sfmin && kount < 20);
            beta = -copysign(hypot(alpha, xn), alpha);
          }
          tau = (beta - alpha) / beta;
          f = fs * (T(1) / (alpha - beta));
          for (int k = 0; k < kount; ++k) beta *= sfmin;
        }
        refl[0] = tau;
        refl[1] = beta;
        refl[2] = f;
      }
      __syncthreads();
    }
    const T tau = refl[0], beta = refl[1], f = refl[2];
    T acct = T(0);
    for (int r = rfirst; r < n; r += rstep) {
      T v;
      if (r <= c) {
        v = T(0);
        if (lane == 0) a.A[(size_t)c * a.lda + r] = a.b[r];
      } else if (r == c + 1) {
        v = T(1);
        if (lane == 0) a.A[(size_t)c * a.lda + r] = (tau != T(0)) ? beta : a.b[r];
      } else {
        const T br = a.b[r];
        v = (tau != T(0)) ? br * f : T(0);
        if (lane == 0) a.A[(size_t)c * a.lda + r] = (tau != T(0)) ? v : br;
      }
      if (lane == 0) a.V[r + j * ldv] = v;
      if (r >= c + 1 && lane < j) acct = fma(a.V[r + lane * ldv], v, acct);
    }
    if (bid == 0 && tid == 0 && a.tau_out) a.tau_out[c] = tau;
    cta_partial<T>(acct, j, scr, a.partT + (size_t)bid * kHbNbMax);
    tau_prev = tau;
    hb_barrier(a.ctl, G);
    // ---------------- P4: matvec partials mvp[cs][r] = sum_{k in chunk cs} A[r, k] v[k]
    // CTA task = (32-row block, column chunk); its 8 warps split the chunk's columns and
    // add their partial rows in shared memory.
    {
      const int m = n - c - 1;
      const int RB = (n + 31) / 32;
      const int CSe = a.CS;
      const T* vcol = a.V + j * ldv;
      for (int task = bid; task < RB * CSe; task += G) {
        const int rb = task % RB, cs = task / RB;
        const int k0 = c + 1 + (int)((long long)cs * m / CSe), k1 = c + 1 + (int)((long long)(cs + 1) * m / CSe);
        const int kw0 = k0 + (int)((long long)wid * (k1 - k0) / (kHbNT / 32));
        const int kw1 = k0 + (int)((long long)(wid + 1) * (k1 - k0) / (kHbNT / 32));
        const int r = rb * 32 + lane;
        T acc = T(0);
        if (r < n) {
          const T* col = a.A + (size_t)kw0 * a.lda + r;
          int k = kw0;
          for (; k + 7 < kw1; k += 8, col += 8 * (size_t)a.lda) {
            T x[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) x[u] = col[u * (size_t)a.lda];
#pragma unroll
            for (int u = 0; u < 8; ++u) acc = fma(x[u], vcol[k + u], acc);
          }
          for (; k < kw1; ++k, col += a.lda) acc = fma(*col, vcol[k], acc);
        }
        mred[wid][lane] = acc;
        __syncthreads();
        if (wid == 0 && r < n) {
          T sum = T(0);
#pragma unroll
          for (int w = 0; w < kHbNT / 32; ++w) sum += mred[w][lane];
          a.mvp[(size_t)cs * n + r] = sum;
        }
        __syncthreads();
      }
    }
    hb_barrier(a.ctl, G);
  }
}

// C (M x N, ldc) = beta C + alpha op(A) op(B); op(A) is M x K, op(B) is K x N.  64 x 64
// tiles, 256 threads with 4 x 4 outputs each, k-slabs of 16 in shared memory.  With
// gridDim.z > 1 the K range is split and each slice writes alpha * its partial product
// into P[z] (M x N, ld M) for k_gemm_reduce.
template <class T>
__global__ void __launch_bounds__(256) k_gemm_ex(int M, int N, int K, T alpha, const T* __restrict__ A, int lda,
                                                int tA, const T* __restrict__ B, int ldb, int tB, T beta,
                                                T* __restrict__ C, int ldc, T* __restrict__ P) {
  __shared__ T As[16][kGT + 1];
  __shared__ T Bs[16][kGT + 1];
  const int tid = threadIdx.x;
  const int tr = tid % 16, tc = tid / 16;
  const int i0 = blockIdx.x * kGT, j0 = blockIdx.y * kGT;
  const int S = gridDim.z, z = blockIdx.z;
  const int kb = (int)((long long)K * z / S), ke = (int)((long long)K * (z + 1) / S);
  T acc[4][4];
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) acc[x][y] = T(0);
  for (int k0 = kb; k0 < ke; k0 += 16) {
    for (int idx = tid; idx < 16 * kGT; idx += 256) {
      int kk, ii;
      // coalesced order: along the operand's contiguous dimension
      if (tA) { kk = idx % 16; ii = idx / 16; } else { ii = idx % kGT; kk = idx / kGT; }
      const int i = i0 + ii, k = k0 + kk;
      T av = T(0);
      if (i < M && k < ke) av = tA ? A[(size_t)i * lda + k] : A[(size_t)k * lda + i];
      As[kk][ii] = av;
    }
    for (int idx = tid; idx < 16 * kGT; idx += 256) {
      int kk, jj;
      if (tB) { jj = idx % kGT; kk = idx / kGT; } else { kk = idx % 16; jj = idx / 16; }
      const int jx = j0 + jj, k = k0 + kk;
      T bv = T(0);
      if (jx < N && k < ke) bv = tB ? B[(size_t)k * ldb + jx] : B[(size_t)jx * ldb + k];
      Bs[kk][jj] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      T av[4], bv[4];
#pragma unroll
      for (int x = 0; x < 4; ++x) av[x] = As[kk][tr + 16 * x];
#pragma unroll
      for (int y = 0; y < 4; ++y) bv[y] = Bs[kk][tc + 16 * y];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) acc[x][y] = fma(av[x], bv[y], acc[x][y]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      const int i = i0 + tr + 16 * x, jx = j0 + tc + 16 * y;
      if (i < M && jx < N) {
        if (S == 1) {
          T* cp = C + (size_t)jx * ldc + i;
          *cp = (beta == T(0)) ? alpha * acc[x][y] : fma(alpha, acc[x][y], beta * *cp);
        } else {
          P[((size_t)z * N + jx) * M + i] = alpha * acc[x][y];
        }
      }
    }
}

template <class T>
__global__ void k_gemm_reduce(int M, int N, int S, const T* __restrict__ P, T beta, T* __restrict__ C, int ldc) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)M * N) return;
  const int i = (int)(idx % M), jx = (int)(idx / M);
  T s = T(0);
  for (int z = 0; z < S; ++z) s += P[(size_t)z * M * N + idx];
  T* cp = C + (size_t)jx * ldc + i;
  *cp = (beta == T(0)) ? s : beta * *cp + s;
}

template <class T>
__global__ void k_hb_identity(int n, T* Z, int ldz) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int r = (int)(idx % n), c = (int)(idx / n);
  Z[(size_t)c * ldz + r] = (r == c) ? T(1) : T(0);
}

constexpr int kSplitMax = 16;

template <class T>
cudaError_t gemm_ex(int M, int N, int K, T alpha, const T* A, int lda, int tA, const T* B, int ldb, int tB, T beta,
                    T* C, int ldc, T* P, size_t pcap, int num_sms, cudaStream_t s) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  const int tiles = ((M + kGT - 1) / kGT) * ((N + kGT - 1) / kGT);
  int S = 1;
  if (K > 512 && tiles < 2 * num_sms) {
    S = std::min(kSplitMax, std::max(1, (2 * num_sms + tiles - 1) / tiles));
    S = std::min(S, std::max(1, K / 256));
    while (S > 1 && (size_t)S * M * N > pcap) --S;
  }
  dim3 g((M + kGT - 1) / kGT, (N + kGT - 1) / kGT, S);
  k_gemm_ex<T><<<g, 256, 0, s>>>(M, N, K, alpha, A, lda, tA, B, ldb, tB, beta, C, ldc, P);
  if (S > 1) {
    const size_t tot = (size_t)M * N;
    k_gemm_reduce<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(M, N, S, P, beta, C, ldc);
  }
  return cudaGetLastError();
}

size_t al(size_t x) { return (x + 63) & ~size_t(63); }

}  // namespace

constexpr int kHbMaxCtas = 512;  // 2 CTAs per SM on up to 256 SMs

// Workspace in elements of T for order n.
size_t hess_blocked_ws_elems(int n) {
  const size_t G = kHbMaxCtas;
  const size_t W = G * (kHbNT / 32), RB = ((size_t)n + 31) / 32;
  const size_t CS = std::max<size_t>(1, W / std::max<size_t>(RB, 1));
  size_t e = 0;
  e += 2 * al((size_t)n * kHbNbMax);           // Y, V
  e += al(kHbNbMax * kHbNbMax);                // T
  e += al(n);                                  // b
  e += 2 * al(G * kHbNbMax) + al(2 * G);       // partials
  e += al(CS * n);                             // matvec partials
  e += 2 * al((size_t)kHbNbMax * n);           // W, W2 (nb x n)
  e += 2 * al((size_t)n * kHbNbMax);           // X, X2 (n x nb)
  e += al((size_t)kSplitMax * kHbNbMax * n);   // split-K partials
  e += 64;                                     // barrier control
  return e;
}

template <class T>
cudaError_t hessenberg_blocked(int n, T* A, int lda, T* Z, int ldz, T* tau_out, T* ws, int num_sms, int* err_host,
                               cudaStream_t s) {
  if (err_host) *err_host = 0;
  if (n <= 0) return cudaSuccess;
  cudaError_t e;
  if (Z) {
    const size_t tot = (size_t)n * n;
    k_hb_identity<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, Z, ldz);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (n < 3) return cudaSuccess;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hess_panel<T>, kHbNT, 0);
  if (e != cudaSuccess) return e;
  const int G = std::min(kHbMaxCtas, num_sms * std::max(1, std::min(per_sm, 2)));
  const int RB = (n + 31) / 32;
  const int CSmax = std::max(1, (kHbMaxCtas * (kHbNT / 32)) / std::max(RB, 1));
  T* p = ws;
  T* Y = p; p += al((size_t)n * kHbNbMax);
  T* V = p; p += al((size_t)n * kHbNbMax);
  T* Tm = p; p += al(kHbNbMax * kHbNbMax);
  T* b = p; p += al(n);
  const size_t Gc = kHbMaxCtas;
  T* partW = p; p += al(Gc * kHbNbMax);
  T* partT = p; p += al(Gc * kHbNbMax);
  T* partN = p; p += al(2 * Gc);
  T* mvp = p; p += al((size_t)CSmax * n);
  T* Wb = p; p += al((size_t)kHbNbMax * n);
  T* W2 = p; p += al((size_t)kHbNbMax * n);
  T* X = p; p += al((size_t)n * kHbNbMax);
  T* X2 = p; p += al((size_t)n * kHbNbMax);
  T* P = p; p += al((size_t)kSplitMax * kHbNbMax * n);
  HbCtl* ctl = reinterpret_cast<HbCtl*>(p);
  const size_t pcap = (size_t)kSplitMax * kHbNbMax * n;
  if ((e = cudaMemsetAsync(ctl, 0, sizeof(HbCtl), s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(Y, 0, sizeof(T) * 2 * al((size_t)n * kHbNbMax), s)) != cudaSuccess) return e;
  for (int c0 = 0; c0 < n - 2; c0 += kHbNbMax) {
    const int w = std::min(kHbNbMax, n - 2 - c0);
    HbArgs<T> a;
    a.n = n; a.c0 = c0; a.nb = w; a.A = A; a.lda = lda; a.Y = Y; a.V = V; a.Tm = Tm; a.b = b;
    a.partW = partW; a.partT = partT; a.partN = partN; a.mvp = mvp;
    a.CS = std::max(1, std::min(CSmax, std::min(G / std::max(RB, 1), n - c0 - 1)));
    a.tau_out = tau_out; a.ctl = ctl;
    void* args[] = {&a};
    if ((e = cudaLaunchCooperativeKernel((const void*)k_hess_panel<T>, dim3(G), dim3(kHbNT), args, 0, s)) !=
        cudaSuccess)
      return e;
    const int k = c0 + w, mt = n - k, m1 = n - c0 - 1;
    // A[:, k:] -= Y V[k:, :]^T
    if (mt > 0) {
      if ((e = gemm_ex<T>(n, mt, w, T(-1), Y, n, 0, V + k, n, 1, T(1), A + (size_t)k * lda, lda, P, pcap, num_sms,
                          s)) != cudaSuccess)
        return e;
      // W = V[c0+1:, :]^T A[c0+1:, k:];  W2 = T^T W;  A[c0+1:, k:] -= V[c0+1:, :] W2
      if ((e = gemm_ex<T>(w, mt, m1, T(1), V + c0 + 1, n, 1, A + (size_t)k * lda + c0 + 1, lda, 0, T(0), Wb, w, P,
                          pcap, num_sms, s)) != cudaSuccess)
        return e;
      if ((e = gemm_ex<T>(w, mt, w, T(1), Tm, kHbNbMax, 1, Wb, w, 0, T(0), W2, w, P, pcap, num_sms, s)) !=
          cudaSuccess)
        return e;
      if ((e = gemm_ex<T>(m1, mt, w, T(-1), V + c0 + 1, n, 0, W2, w, 0, T(1), A + (size_t)k * lda + c0 + 1, lda,
                          P, pcap, num_sms, s)) != cudaSuccess)
        return e;
    }
    if (Z) {
      // X = Z[:, c0+1:] V[c0+1:, :];  X2 = X T;  Z[:, c0+1:] -= X2 V[c0+1:, :]^T
      if ((e = gemm_ex<T>(n, w, m1, T(1), Z + (size_t)(c0 + 1) * ldz, ldz, 0, V + c0 + 1, n, 0, T(0), X, n, P, pcap,
                          num_sms, s)) != cudaSuccess)
        return e;
      if ((e = gemm_ex<T>(n, w, w, T(1), X, n, 0, Tm, kHbNbMax, 0, T(0), X2, n, P, pcap, num_sms, s)) !=
          cudaSuccess)
        return e;
      if ((e = gemm_ex<T>(n, m1, w, T(-1), X2, n, 0, V + c0 + 1, n, 1, T(1), Z + (size_t)(c0 + 1) * ldz, ldz, P,
                          pcap, num_sms, s)) != cudaSuccess)
        return e;
    }
  }
  if (err_host) {
    HbCtl h{};
    if ((e = cudaMemcpyAsync(&h, ctl, sizeof(HbCtl), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    *err_host = h.err;
  }
  return cudaSuccess;
}

int hess_blocked_min(size_t tsize) {
  if (const char* ev = std::getenv("GS_HESS_BLOCKED_MIN")) return std::atoi(ev);
  // FP32: the panel's per-column latency (~30 us at n = 4096) is far below the unblocked
  // reduction's three passes per column.  FP64: the trailing products (5 n^3 flops on the
  // FP64 pipe) cost more than the unblocked reduction's fused rank-2 passes saves.
  return tsize == sizeof(float) ? 256 : (1 << 30);
}

template cudaError_t hessenberg_blocked<double>(int, double*, int, double*, int, double*, double*, int, int*,
                                                cudaStream_t);
template cudaError_t hessenberg_blocked<float>(int, float*, int, float*, int, float*, float*, int, int*, cudaStream_t);

}  // namespace gsk
