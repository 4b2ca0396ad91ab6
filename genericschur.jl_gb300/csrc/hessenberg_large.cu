// Householder Hessenberg reduction of one large matrix (n > 128) on the whole GPU,
// with the Schur vectors Z = H(1) H(2) ... accumulated alongside.
//
// Reference semantics: _hessenberg! (hessenberg.jl:3-17) applies reflector i as
// lmul!(H', A[i+1:n, i+1:n]) then rmul!(A[:, i+1:n], H) (householder.jl:140-172);
// _materializeQ (hessenberg.jl:150-166) forms Q from the same reflectors.  Per
// column i the two one-sided updates are fused into one rank-2 update using
//   v = u^T A[i+1:n, i+1:n],  w = A[:, i+1:n] u - tau (v.u) u,
//   A <- A - tau u v^T - tau w u^T   (the u v^T term on rows i+1..n only),
// which is algebraically the left-then-right sequence.  Each column costs two
// launches: a read pass over A and Z producing tiled partial sums, whose last CTA
// (ticket counter, no waiting) adds the per-tile parts of u^T A u in a fixed order;
// and the update pass, which sums the partials it needs, and whose last CTA computes
// the next column's reflector.  Everything is deterministic.
#include <algorithm>

#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kTile = 64;   // tile edge of the partial-sum pass
constexpr int kHT = 256;    // threads per CTA of the streaming passes
constexpr int kUpdColsMax = 256;  // columns per CTA of the update pass (at most)

template <class T> __device__ __forceinline__ T tsqrt(T x);
template <> __device__ __forceinline__ double tsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float tsqrt<float>(float x) { return sqrtf(x); }
template <class T> __device__ __forceinline__ T thypot(T a, T b);
template <> __device__ __forceinline__ double thypot<double>(double a, double b) { return hypot(a, b); }
template <> __device__ __forceinline__ float thypot<float>(float a, float b) { return hypotf(a, b); }
template <class T> struct Lim;
template <> struct Lim<double> {
  static __device__ __forceinline__ double fmin() { return 2.2250738585072014e-308; }
  static __device__ __forceinline__ double eps() { return 2.220446049250313e-16; }
  static __device__ __forceinline__ double safe_hi() { return 1.0e150; }
  static __device__ __forceinline__ double safe_lo() { return 1.0e-150; }
};
template <> struct Lim<float> {
  static __device__ __forceinline__ float fmin() { return 1.17549435e-38f; }
  static __device__ __forceinline__ float eps() { return 1.1920929e-07f; }
  static __device__ __forceinline__ float safe_hi() { return 1.0e18f; }
  static __device__ __forceinline__ float safe_lo() { return 1.0e-18f; }
};

template <class T, int NT>
__device__ T blk_max(T v, T* red) {
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v || w != w) ? w : v;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  v = red[0];
  for (int i = 1; i < NT / 32; ++i) { T w = red[i]; v = (w > v || w != w) ? w : v; }
  __syncthreads();
  return v;
}
template <class T, int NT>
__device__ T blk_sum(T v, T* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  v = red[0];
  for (int i = 1; i < NT / 32; ++i) v += red[i];
  __syncthreads();
  return v;
}

// Reflector for column i (0-based column c = i-1, rows i..n-1 0-based), householder.jl:12-54.
// Writes beta / the essential part into A, the full vector u (zeros above row i) into
// u[], and tau into st[0].
template <class T, int NT>
__device__ void hess_reflector(int n, T* A, int lda, int i, T* u, T* st, T* tau_out, T* red) {
  const int tid = threadIdx.x;
  T* col = A + (size_t)(i - 1) * lda + i;  // rows i+1..n (1-based) of column i
  const int m = n - i;
  T lmax = 0;
  for (int r = 1 + tid; r < m; r += NT) lmax = fmax(lmax, fabs(col[r]));
  const T big = blk_max<T, NT>(lmax, red);
  T tau = 0;
  T alpha = col[0];
  if (big != T(0)) {
    const bool safe = (big < Lim<T>::safe_hi() && big > Lim<T>::safe_lo());
    const T sc = safe ? T(1) : T(1) / big;
    T ls = 0;
    for (int r = 1 + tid; r < m; r += NT) { const T t = col[r] * sc; ls = fma(t, t, ls); }
    const T ssq = blk_sum<T, NT>(ls, red);
    T xnorm = safe ? tsqrt(ssq) : big * tsqrt(ssq);
    const T sfmin = T(2) * Lim<T>::fmin() / Lim<T>::eps();
    T beta = -copysign(thypot(alpha, xnorm), alpha);
    int kount = 0;
    if (fabs(beta) < sfmin) {
      const T rsfmin = T(1) / sfmin;
      T bb = beta;
      do { ++kount; bb *= rsfmin; alpha *= rsfmin; } while (fabs(bb) < sfmin && kount < 20);
      for (int r = 1 + tid; r < m; r += NT) {
        T t = col[r];
        for (int q = 0; q < kount; ++q) t *= rsfmin;
        col[r] = t;
      }
      __syncthreads();
      T lm2 = 0;
      for (int r = 1 + tid; r < m; r += NT) lm2 = fmax(lm2, fabs(col[r]));
      const T big2 = blk_max<T, NT>(lm2, red);
      const T sc2 = big2 > T(0) ? T(1) / big2 : T(0);
      T ls2 = 0;
      for (int r = 1 + tid; r < m; r += NT) { const T t = col[r] * sc2; ls2 = fma(t, t, ls2); }
      xnorm = big2 * tsqrt(blk_sum<T, NT>(ls2, red));
      beta = -copysign(thypot(alpha, xnorm), alpha);
    }
    tau = (beta - alpha) / beta;
    const T t = T(1) / (alpha - beta);
    for (int r = 1 + tid; r < m; r += NT) col[r] *= t;
    for (int q = 0; q < kount; ++q) beta *= sfmin;
    __syncthreads();
    if (tid == 0) col[0] = beta;
  }
  // u over all n rows: zeros for rows 1..i, 1 at row i+1, x below
  for (int r = tid; r < n; r += NT) u[r] = (r < i) ? T(0) : (r == i ? T(1) : (tau != T(0) ? col[r - i] : T(0)));
  if (tid == 0) {
    st[0] = tau;
    if (tau_out) tau_out[i - 1] = tau;
  }
}

template <class T, int NT>
__global__ void __launch_bounds__(NT) k_hess_reflector(int n, T* A, int lda, int i, T* u, T* st, T* tau_out) {
  __shared__ T red[32];
  hess_reflector<T, NT>(n, A, lda, i, u, st, tau_out, red);
}

// Partial sums over a strip of A (rows r0..r0+63, column tiles ct, ct + ncs, ...,
// columns >= i+1): pw[ct][r] = sum over the strip of A[r,c] u_c, pv[rt][c] = sum over
// the strip's rows of u_r A[r,c]; the same strip of Z gives pz[ct][r].  The strip's part
// of u^T A u goes to pdot[rt * ncs + ct]; the last CTA to finish adds those parts in a
// fixed order into st[1].
template <class T>
__global__ void __launch_bounds__(kHT) k_hess_partials(int n, const T* __restrict__ A, int lda,
                                                      const T* __restrict__ Z, int ldz, int i,
                                                      const T* __restrict__ u, T* __restrict__ st,
                                                      T* __restrict__ pw, T* __restrict__ pv, T* __restrict__ pz,
                                                      T* __restrict__ pdot, unsigned* __restrict__ ticket) {
  __shared__ T tile[kTile][kTile + 1];
  __shared__ T us[kTile];
  __shared__ T ur[kTile];
  __shared__ T rs[4][kTile];
  __shared__ T cs[4][kTile];
  __shared__ T wd[2];
  __shared__ T wsum[kHT / 32];
  __shared__ bool last;
  const int tid = threadIdx.x;
  const int ct = blockIdx.x, rt = blockIdx.y, ncs = gridDim.x;
  const int r0 = rt * kTile;
  const int which = blockIdx.z;     // 0: A, 1: Z (the grid has no Z slice without Z)
  const T* M = which ? Z : A;
  const int ld = which ? ldz : lda;
  for (int t = tid; t < kTile; t += kHT) ur[t] = (r0 + t < n) ? u[r0 + t] : T(0);
  const int q = tid & 63, g = tid >> 6;
  T sr_tot = T(0);  // row partial of row r0 + q over the strip (threads g == 0 keep it)
  for (int c0 = i + ct * kTile; c0 < n; c0 += ncs * kTile) {
    for (int t = tid; t < kTile; t += kHT) us[t] = (c0 + t < n) ? u[c0 + t] : T(0);
    for (int t = tid; t < kTile * kTile; t += kHT) {
      const int rr = t % kTile, cc = t / kTile;
      const int r = r0 + rr, c = c0 + cc;
      tile[rr][cc] = (r < n && c < n) ? M[(size_t)c * ld + r] : T(0);
    }
    __syncthreads();
    // row partials (4 threads per row) and, for A, column partials (4 threads per column)
    T sr = 0, sc = 0;
    for (int k = g; k < kTile; k += 4) sr = fma(tile[q][k], us[k], sr);
    if (which == 0)
      for (int k = g; k < kTile; k += 4) sc = fma(ur[k], tile[k][q], sc);
    rs[g][q] = sr;
    cs[g][q] = sc;
    __syncthreads();
    if (tid < kTile) {
      sr_tot += rs[0][tid] + rs[1][tid] + rs[2][tid] + rs[3][tid];
      if (which == 0 && c0 + tid < n)
        pv[(size_t)rt * n + c0 + tid] = cs[0][tid] + cs[1][tid] + cs[2][tid] + cs[3][tid];
    }
    __syncthreads();
  }
  T tdot = T(0);
  if (tid < kTile) {
    if (r0 + tid < n) (which ? pz : pw)[(size_t)ct * n + r0 + tid] = sr_tot;
    if (which == 0) tdot = ur[tid] * sr_tot;  // this strip's part of u^T A u
  }
  for (int o = 16; o > 0; o >>= 1) tdot += __shfl_xor_sync(0xffffffffu, tdot, o);
  if (tid < kTile && (tid & 31) == 0) wd[tid >> 5] = tdot;
  __syncthreads();
  if (which == 0 && tid == 0) pdot[(size_t)rt * ncs + ct] = wd[0] + wd[1];
  __threadfence();
  __syncthreads();
  if (tid == 0) last = (atomicAdd(ticket, 1u) == gridDim.x * gridDim.y * gridDim.z - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  const int ntile = gridDim.x * gridDim.y;
  T acc = T(0);
  for (int t = tid; t < ntile; t += kHT) acc += pdot[t];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((tid & 31) == 0) wsum[tid >> 5] = acc;
  __syncthreads();
  if (tid == 0) {
    T d = T(0);
    for (int w = 0; w < kHT / 32; ++w) d += wsum[w];
    st[1] = d;
    *ticket = 0u;
  }
}

// A[r,c] -= tau (u_r v_c + w_r u_c), Z[r,c] -= tau z_r u_c, for c >= i+1 (0-based c >= i),
// with v_c = sum of the column partials (staged per CTA for its column range) and
// w_r = sum of the row partials - tau (u^T A u) u_r.  The last CTA to finish computes
// the reflector of column i+1 for the next step.
template <class T>
__global__ void __launch_bounds__(kHT) k_hess_update(int n, T* __restrict__ A, int lda, T* __restrict__ Z, int ldz,
                                                    int i, T* __restrict__ u, T* __restrict__ st,
                                                    const T* __restrict__ pv, int nrt, const T* __restrict__ pw,
                                                    const T* __restrict__ pz, int nct, unsigned* __restrict__ ticket,
                                                    T* tau_out, int cpc) {
  __shared__ T vs[kUpdColsMax];
  __shared__ T red[32];
  __shared__ bool last;
  const T tau = st[0];
  const int tid = threadIdx.x;
  const int which = blockIdx.z;
  const int cb = i + blockIdx.y * cpc, ce = min(n, cb + cpc);
  if (tau != T(0)) {
    if (which == 0)
      for (int c = cb + tid; c < ce; c += kHT) {
        T sv = T(0);
        for (int t = 0; t < nrt; ++t) sv += pv[(size_t)t * n + c];
        vs[c - cb] = sv;
      }
    __syncthreads();
    const T* part = which ? pz : pw;
    T* M = which ? Z : A;
    const int ld = which ? ldz : lda;
    const T dot = st[1];
    for (int r = blockIdx.x * kHT + tid; r < n; r += gridDim.x * kHT) {
      T w = T(0);
      for (int t = 0; t < nct; ++t) w += part[(size_t)t * n + r];
      const T ur = u[r];
      if (which == 0) w = fma(-tau * dot, ur, w);
      const T tw = tau * w, tu = tau * ur;
      // four columns per round: the four loads are issued before any store
      T* p = M + (size_t)cb * ld + r;
      int c = cb;
      for (; c + 3 < ce; c += 4, p += 4 * (size_t)ld) {
        T a0 = p[0], a1 = p[ld], a2 = p[2 * (size_t)ld], a3 = p[3 * (size_t)ld];
        if (which == 0) {
          a0 = fma(-tu, vs[c - cb], a0);
          a1 = fma(-tu, vs[c + 1 - cb], a1);
          a2 = fma(-tu, vs[c + 2 - cb], a2);
          a3 = fma(-tu, vs[c + 3 - cb], a3);
        }
        p[0] = fma(-tw, u[c], a0);
        p[ld] = fma(-tw, u[c + 1], a1);
        p[2 * (size_t)ld] = fma(-tw, u[c + 2], a2);
        p[3 * (size_t)ld] = fma(-tw, u[c + 3], a3);
      }
      for (; c < ce; ++c, p += ld) {
        T a0 = *p;
        if (which == 0) a0 = fma(-tu, vs[c - cb], a0);
        *p = fma(-tw, u[c], a0);
      }
    }
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last = (atomicAdd(ticket, 1u) == gridDim.x * gridDim.y * gridDim.z - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (tid == 0) *ticket = 0u;
  if (i + 1 <= n - 2) hess_reflector<T, kHT>(n, A, lda, i + 1, u, st, tau_out, red);
}

template <class T>
__global__ void k_set_identity(int n, T* Z, int ldz) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int r = idx % n, c = idx / n;
  Z[(size_t)c * ldz + r] = (r == c) ? T(1) : T(0);
}

}  // namespace

// Workspace (elements of T): u n, st 8, pw/pz/pv nt*n each, pdot nt*nt, two tickets.
size_t hess_large_ws_elems(int n) {
  const size_t nt = (size_t)(n + kTile - 1) / kTile;
  return (size_t)n + 8 + 3 * nt * n + nt * nt + 16;
}

template <class T>
cudaError_t hessenberg_large(int n, T* A, int lda, T* Z, int ldz, T* tau_out, T* ws, cudaStream_t s) {
  const int nt = (n + kTile - 1) / kTile;
  T* u = ws;
  T* st = u + n;
  T* pw = st + 8;
  T* pz = pw + (size_t)nt * n;
  T* pv = pz + (size_t)nt * n;
  T* pdot = pv + (size_t)nt * n;
  unsigned* tickets = (unsigned*)(pdot + (size_t)nt * nt);
  cudaError_t e = cudaMemsetAsync(tickets, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  if (Z) {
    const size_t tot = (size_t)n * n;
    k_set_identity<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, Z, ldz);
  }
  if (n >= 3) k_hess_reflector<T, 512><<<1, 512, 0, s>>>(n, A, lda, 1, u, st, tau_out);
  for (int i = 1; i <= n - 2; ++i) {
    // partials: row strips of 64 x ncs column tiles, about 1024 CTAs over A and Z
    const int nctile = (n - i + kTile - 1) / kTile;
    const int ncs = std::max(1, std::min(nctile, 1024 / (nt * (Z ? 2 : 1))));
    dim3 g1(ncs, nt, Z ? 2 : 1);
    k_hess_partials<T><<<g1, kHT, 0, s>>>(n, A, lda, Z, ldz, i, u, st, pw, pv, pz, pdot, tickets);
    // update: up to 4 row blocks x column blocks of cpc columns, about 512 CTAs
    const int rows = std::min((n + kHT - 1) / kHT, 4);
    int cpc = (int)(((long long)(n - i) * rows * (Z ? 2 : 1) + 511) / 512);
    cpc = std::max(32, std::min(kUpdColsMax, (cpc + 31) / 32 * 32));
    const int ncb = (n - i + cpc - 1) / cpc;
    dim3 g2(rows, ncb, Z ? 2 : 1);
    k_hess_update<T><<<g2, kHT, 0, s>>>(n, A, lda, Z, ldz, i, u, st, pv, nt, pw, pz, ncs, tickets + 1, tau_out, cpc);
  }
  return cudaGetLastError();
}

template cudaError_t hessenberg_large<double>(int, double*, int, double*, int, double*, double*, cudaStream_t);
template cudaError_t hessenberg_large<float>(int, float*, int, float*, int, float*, float*, cudaStream_t);

}  // namespace gsk
