// Batched real Schur decomposition, one CTA per matrix (n <= 128), FP64 (and an FP32
// instance of the same code for the FP32 stage of the mixed-precision form).
//
// Each CTA pulls matrix indices from its size bin's work queue (a ticket counter
// in global memory) and runs, for one matrix:
//   1. load + _scale! (util.jl:14-29);
//   2. Householder Hessenberg reduction (hessenberg.jl:3-17; reflector as in
//      householder.jl:12-54, lmul!/rmul! as householder.jl:140-172), in shared
//      memory for the small bins and in the L2-resident output buffer for the
//      large ones;
//   3. Q formation (hessenberg.jl:150-166) straight into the Z output, each thread
//      owning whole rows of Z so that Z never needs a barrier;
//   4. the real double-shift Francis iteration of gschur!(H::Hessenberg{<:Real}, Z)
//      (GenericSchur.jl:513-699) with doubleShiftQR! (837-952) and _gs2x2!
//      (716-803) on a packed copy of H in shared memory (column j keeps rows
//      1..j+3: the Hessenberg part and the two rows of the 3x3 bulge), which lets
//      three 128x128 matrices share one SM;
//   5. T, eigenvalues and status written back, undoing the scaling.
//
// Bulge chase, one barrier per step: warp 0 owns the near-diagonal block of step k
// (left update of columns k..k+2, right update of rows k..k+3) and then computes
// the reflector of step k+1 from column k, while the other warps apply step k to
// the far columns (k+3..n) and far rows (1..k-1).  The two sets are disjoint, and
// everything step k+1 reads was written by one side or the other before the
// barrier.  Each sweep's reflectors are logged and applied to the Z rows in one
// streaming pass afterwards (every thread owns rows of Z).
#include <type_traits>

#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

template <class T>
struct Refl {
  T t1, t2, t3, v2, v3;
};

template <class T>
struct Ctl {
  T v[3];        // start vector of the sweep
  Refl<T> r[2];  // reflector of the current step / the next step
  T s[4];        // shifts r1r, r1i, r2r, r2i
  T g[2];        // Givens cs, sn of a 2x2 deflation
  T blk[4];      // standardised 2x2 block
  int split;
  int mx;
};

// Packed QR layout: column j (1-based) holds rows 1..j+3.
__host__ __device__ __forceinline__ int rpk(int j) { return ((j - 1) * (j + 6)) >> 1; }

#define AA(i, j) A[((i) - 1) + ((j) - 1) * lda]
#define HH(i, j) H[rpk(j) + (i) - 1]

template <class T, int NT>
__device__ void hessenberg_real(int n, T* A, int lda, T* tau, T* red) {
  const int tid = threadIdx.x;
  const T sfmin = T(2) * Prec<T>::fmin / Prec<T>::eps;
  for (int i = 1; i <= n - 2; ++i) {
    const int m = n - i;          // reflector length: rows i+1..n
    T* col = &AA(i + 1, i);  // col[0] = alpha, col[1..m-1] = x
    T lmax = T(0);
    for (int r = 1 + tid; r < m; r += NT) lmax = fmax(lmax, fabs(col[r]));
    const T big = block_max<NT>(lmax, red);
    T tau_i = T(0);
    if (big != T(0)) {
      const bool safe = (big < Prec<T>::safe_hi && big > Prec<T>::safe_lo);
      const T sc = safe ? T(1) : T(1) / big;
      T ls = T(0);
      for (int r = 1 + tid; r < m; r += NT) { const T t = col[r] * sc; ls = fma(t, t, ls); }
      const T ssq = block_sum<NT>(ls, red);
      T xnorm = safe ? sqrt(ssq) : big * sqrt(ssq);
      T alpha = col[0];
      T beta = -copysign(hypot(alpha, xnorm), alpha);
      int kount = 0;
      if (fabs(beta) < sfmin) {
        // underflow guard (householder.jl:25-42): rescale x, alpha and beta
        const T rsfmin = T(1) / sfmin;
        T bb = beta;
        do { ++kount; bb *= rsfmin; alpha *= rsfmin; } while (fabs(bb) < sfmin && kount < 20);
        __syncthreads();
        for (int r = 1 + tid; r < m; r += NT) {
          T t = col[r];
          for (int q = 0; q < kount; ++q) t *= rsfmin;
          col[r] = t;
        }
        __syncthreads();
        T lm2 = T(0);
        for (int r = 1 + tid; r < m; r += NT) lm2 = fmax(lm2, fabs(col[r]));
        const T big2 = block_max<NT>(lm2, red);
        const T sc2 = (big2 > T(0)) ? T(1) / big2 : T(0);
        T ls2 = T(0);
        for (int r = 1 + tid; r < m; r += NT) { const T t = col[r] * sc2; ls2 = fma(t, t, ls2); }
        const T ssq2 = block_sum<NT>(ls2, red);
        xnorm = big2 * sqrt(ssq2);
        beta = -copysign(hypot(alpha, xnorm), alpha);
      }
      tau_i = (beta - alpha) / beta;
      const T t = T(1) / (alpha - beta);
      for (int r = 1 + tid; r < m; r += NT) col[r] *= t;
      for (int q = 0; q < kount; ++q) beta *= sfmin;
      __syncthreads();
      if (tid == 0) col[0] = beta;
    }
    if (tid == 0) tau[i - 1] = tau_i;
    __syncthreads();
    if (tau_i == T(0)) continue;
    // lmul!(H', A[i+1:n, i+1:n]): one column per thread
    for (int j = i + 1 + tid; j <= n; j += NT) {
      T* hj = &AA(i + 1, j);
      T va0 = hj[0], va1 = T(0);
      int r = 1;
      for (; r + 1 < m; r += 2) { va0 = fma(col[r], hj[r], va0); va1 = fma(col[r + 1], hj[r + 1], va1); }
      if (r < m) va0 = fma(col[r], hj[r], va0);
      const T va = (va0 + va1) * tau_i;
      hj[0] -= va;
      for (r = 1; r < m; ++r) hj[r] = fma(-va, col[r], hj[r]);
    }
    __syncthreads();
    // rmul!(A[:, i+1:n], H): one row per thread
    for (int r = tid; r < n; r += NT) {
      T* hr = &A[r + i * lda];  // row r+1, column i+1
      T x0 = hr[0], x1 = T(0);
      int q = 1;
      for (; q + 1 < m; q += 2) { x0 = fma(hr[q * lda], col[q], x0); x1 = fma(hr[(q + 1) * lda], col[q + 1], x1); }
      if (q < m) x0 = fma(hr[q * lda], col[q], x0);
      const T x = (x0 + x1) * tau_i;
      hr[0] -= x;
      for (q = 1; q < m; ++q) hr[q * lda] = fma(-x, col[q], hr[q * lda]);
    }
    __syncthreads();
  }
}

// Apply reflector r (order 3) from the left to column j, rows k..k+2 of packed H.
template <class T>
__device__ __forceinline__ void left3(T* H, int k, int j, const Refl<T>& r) {
  T* h = &HH(k, j);
  const T ss = fma(r.v3, h[2], fma(r.v2, h[1], h[0]));
  h[0] = fma(-ss, r.t1, h[0]);
  h[1] = fma(-ss, r.t2, h[1]);
  h[2] = fma(-ss, r.t3, h[2]);
}
// ... from the right to row i, columns k..k+2.
template <class T>
__device__ __forceinline__ void right3(T* H, int k, int i, const Refl<T>& r) {
  T& h0 = HH(i, k);
  T& h1 = HH(i, k + 1);
  T& h2 = HH(i, k + 2);
  const T ss = fma(r.v3, h2, fma(r.v2, h1, h0));
  h0 = fma(-ss, r.t1, h0);
  h1 = fma(-ss, r.t2, h1);
  h2 = fma(-ss, r.t3, h2);
}
template <class T>
__device__ __forceinline__ void left2(T* H, int k, int j, const Refl<T>& r) {
  T* h = &HH(k, j);
  const T ss = fma(r.v2, h[1], h[0]);
  h[0] = fma(-ss, r.t1, h[0]);
  h[1] = fma(-ss, r.t2, h[1]);
}
template <class T>
__device__ __forceinline__ void right2(T* H, int k, int i, const Refl<T>& r) {
  T& h0 = HH(i, k);
  T& h1 = HH(i, k + 1);
  const T ss = fma(r.v2, h1, h0);
  h0 = fma(-ss, r.t1, h0);
  h1 = fma(-ss, r.t2, h1);
}

// Reflector of chase step k (> mx) from column k-1, writing beta and the zeros
// back into H (GenericSchur.jl:882-895); logged for the Z pass.
template <class T>
__device__ __forceinline__ void make_refl(T* H, int k, int iend, Refl<T>& out, T* lg) {
  const int nr = min(3, iend - k + 1);
  T a = HH(k, k - 1), x1 = HH(k + 1, k - 1), x2 = (nr == 3) ? HH(k + 2, k - 1) : T(0);
  const T t1 = reflector_fast(a, x1, x2, nr);
  HH(k, k - 1) = a;
  HH(k + 1, k - 1) = T(0);
  if (k < iend - 1) HH(k + 2, k - 1) = T(0);
  out.t1 = t1; out.v2 = x1; out.v3 = x2; out.t2 = t1 * x1; out.t3 = t1 * x2;
  T* l = lg + 5 * (k - 1);
  l[0] = t1; l[1] = out.t2; l[2] = out.t3; l[3] = x1; l[4] = x2;
}

// nmax: the largest order the launch sized shared memory for.  Orders come from device
// memory (GS_DEVICE calls are not checked on the host), so an order outside [0, nmax]
// gets ST_BADARG before anything is read or written.
template <class T, class W, int NT, bool HSMEM>
__device__ void solve_real(const RealBatchT<T, W>& bt, int b, int nmax, T* smem, Ctl<T>& c) {
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int n = bt.ns[b];
  if (n <= 0 || n > nmax) {
    if (tid == 0) bt.status[b] = (n == 0) ? ST_OK : ST_BADARG;
    return;
  }
  T* __restrict__ Ag = bt.A + bt.offs[b];
  T* __restrict__ Zg = bt.wantz ? bt.Z + bt.offs[b] : nullptr;
  W* __restrict__ wr = bt.wr + bt.woffs[b];
  W* __restrict__ wi = bt.wi + bt.woffs[b];
  const int lda = HSMEM ? (n | 1) : n;
  const int hsz = HSMEM ? n * lda : rpk(n + 1);  // full (Hessenberg phase) or packed (QR phase)
  const int hreg = max(hsz, rpk(n + 1));
  T* H = smem;                      // packed H of the QR phase (and the full matrix before it, HSMEM)
  T* tau = H + hreg;                // n-1 reflector scalars
  T* lg = tau + n;                  // 5 per chase step: t1, t2, t3, v2, v3
  T* red = lg + 5 * n;              // reduction scratch (32)
  T* A = HSMEM ? smem : Ag;         // where the Hessenberg reduction runs

  // ---- 1. load and scale --------------------------------------------------
  double amax = 0.0;
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    const T a = Ag[idx];
    if (HSMEM) A[i + j * lda] = a;
    const double aa = fabs((double)a);
    amax = (aa > amax || aa != aa) ? aa : amax;
  }
  amax = (double)block_max<NT>((T)amax, red);
  __syncthreads();
  const double smlnum = sqrt((double)Prec<T>::fmin) / (double)Prec<T>::eps;
  const double bignum = 1.0 / smlnum;
  bool scaled = false;
  double cscale = 1.0;
  if (bt.scale) {
    if (amax > 0.0 && amax < smlnum) { scaled = true; cscale = smlnum; }
    else if (amax > bignum) { scaled = true; cscale = bignum; }
  }
  if (scaled) {
    double mul[8];
    const int nf = safescale_factors(amax, cscale, mul);
    for (int f = 0; f < nf; ++f)
      for (int idx = tid; idx < n * n; idx += NT) {
        const int i = idx % n, j = idx / n;
        A[i + j * lda] = (T)((double)A[i + j * lda] * mul[f]);
      }
    __syncthreads();
  }

  // ---- 2. Hessenberg reduction ------------------------------------------------
  hessenberg_real<T, NT>(n, A, lda, tau, red);

  // ---- 3. Q formation into Z (row-owner threads, no barriers) ------------------
  if (Zg) {
    for (int r = tid; r < n; r += NT)
      for (int j = 0; j < n; ++j) Zg[r + (long long)j * n] = (r == j) ? T(1) : T(0);
    for (int i = 1; i <= n - 2; ++i) {
      const T t = tau[i - 1];
      if (t == T(0)) continue;
      const int m = n - i;
      const T* col = &AA(i + 1, i);
      for (int r = tid; r < n; r += NT) {
        T* zr = Zg + r + (long long)i * n;  // Z[r+1, i+1]
        T s0 = zr[0], s1 = T(0);
        int q = 1;
        for (; q + 1 < m; q += 2) { s0 = fma(zr[q * n], col[q], s0); s1 = fma(zr[(q + 1) * n], col[q + 1], s1); }
        if (q < m) s0 = fma(zr[q * n], col[q], s0);
        const T s = (s0 + s1) * t;
        zr[0] -= s;
        for (q = 1; q < m; ++q) zr[q * n] = fma(-s, col[q], zr[q * n]);
      }
    }
  }
  __syncthreads();

  // ---- 4. pack H (Hessenberg part + bulge rows) into shared memory ----------------
  if (HSMEM) {
    // the full matrix occupies the same shared memory: route through the output buffer
    for (int idx = tid; idx < n * n; idx += NT) {
      const int i = idx % n, j = idx / n;
      Ag[idx] = A[i + j * lda];
    }
    __syncthreads();
  }
  for (int j = 1; j <= n; ++j)
    for (int i = 1 + tid; i <= j + 3; i += NT)
      HH(i, j) = (i <= min(j + 1, n)) ? Ag[(i - 1) + (long long)(j - 1) * n] : T(0);
  __syncthreads();

  // ---- 5. Francis double-shift QR on packed H ------------------------------------------
  const T eps = Prec<T>::eps;
  const T smallnum = Prec<T>::fmin * ((T)n / eps);
  const long long maxiter = bt.maxiter_abs > 0 ? bt.maxiter_abs : (long long)bt.maxiter_mult * n;
  long long iter = 0;
  int status = ST_OK;
  int iend = n;
  while (iend >= 1) {
    int istart = 1;
    int iterqr = 0;
    bool deflate = false;
    for (;;) {
      ++iter;
      if (iter > maxiter) { status = ST_UNCONVERGED; break; }
      // deflation scan (GenericSchur.jl:563-600): largest k with a negligible H[k,k-1]
      if (tid == 0) c.split = 0;
      __syncthreads();
      for (int k = istart + 1 + tid; k <= iend; k += NT) {
        bool split = false;
        const T hk = HH(k, k - 1);
        if (fabs(hk) < smallnum) {
          split = true;
        } else {
          const T hkk = HH(k, k), hkm1 = HH(k - 1, k - 1);
          T t = fabs(hkm1) + fabs(hkk);
          if (t == T(0)) {
            if (k > 2) t += fabs(HH(k - 1, k - 2));
            if (k + 1 <= n) t += fabs(HH(k + 1, k));
          }
          const T ahkkm1 = fabs(hk);
          if (ahkkm1 <= t * eps) {
            const T ahkm1k = fabs(HH(k - 1, k));
            const T ab = fmax(ahkkm1, ahkm1k), ba = fmin(ahkkm1, ahkm1k);
            const T aa = fmax(fabs(hkk), fabs(hkm1 - hkk)), bb = fmin(fabs(hkk), fabs(hkm1 - hkk));
            const T s = aa + bb;
            if (ba * (ab / s) <= fmax(smallnum, eps * (bb * (aa / s)))) split = true;
          }
        }
        if (split) atomicMax(&c.split, k);
      }
      __syncthreads();
      istart = (c.split > 0) ? c.split : 1;
      if (istart > 1 && tid == 0) HH(istart, istart - 1) = T(0);
      if (istart >= iend - 1) { deflate = true; break; }
      ++iterqr;
      __syncthreads();
      // shifts (GenericSchur.jl:614-665)
      if (tid == 0) {
        T h11, h12, h21, h22;
        if (iterqr == 10) {
          const T s = fabs(HH(istart + 1, istart)) + fabs(HH(istart + 2, istart + 1));
          h11 = T(0.75) * s + HH(istart, istart); h12 = T(-0.4375) * s; h21 = s; h22 = h11;
        } else if (iterqr == 20) {
          const T s = fabs(HH(iend, iend - 1)) + fabs(HH(iend - 1, iend - 2));
          h11 = T(0.75) * s + HH(iend, iend); h12 = T(-0.4375) * s; h21 = s; h22 = h11;
        } else {
          h11 = HH(iend - 1, iend - 1); h21 = HH(iend, iend - 1);
          h12 = HH(iend - 1, iend); h22 = HH(iend, iend);
        }
        const T s = fabs(h11) + fabs(h12) + fabs(h21) + fabs(h22);
        T r1r, r2r, r1i, r2i;
        if (s == T(0)) {
          r1r = r2r = r1i = r2i = T(0);
        } else {
          h11 /= s; h12 /= s; h21 /= s; h22 /= s;
          const T tr = (h11 + h22) / T(2);
          const T d = (h11 - tr) * (h22 - tr) - h12 * h21;
          const T rtd = sqrt(fabs(d));
          if (d >= T(0)) {
            r1r = tr * s; r2r = r1r; r1i = rtd * s; r2i = -r1i;
          } else {
            r1r = tr + rtd; r2r = tr - rtd;
            if (fabs(r1r - h22) <= fabs(r2r - h22)) { r1r *= s; r2r = r1r; }
            else { r2r *= s; r1r = r2r; }
            r1i = r2i = T(0);
          }
        }
        c.s[0] = r1r; c.s[1] = r1i; c.s[2] = r2r; c.s[3] = r2i;
        c.mx = istart;
      }
      __syncthreads();
      // start row (GenericSchur.jl:850-872): largest m with two small subdiagonals
      {
        const T r1r = c.s[0], r1i = c.s[1], r2r = c.s[2], r2i = c.s[3];
        for (int m = istart + 1 + tid; m <= iend - 2; m += NT) {
          T h21s = HH(m + 1, m);
          T s = fabs(HH(m, m) - r2r) + fabs(r2i) + fabs(h21s);
          h21s /= s;
          T v0 = h21s * HH(m, m + 1) + (HH(m, m) - r1r) * ((HH(m, m) - r2r) / s) - r1i * (r2i / s);
          T v1 = h21s * (HH(m, m) + HH(m + 1, m + 1) - r1r - r2r);
          T v2 = h21s * HH(m + 2, m + 1);
          s = fabs(v0) + fabs(v1) + fabs(v2);
          v0 /= s; v1 /= s; v2 /= s;
          if (fabs(HH(m, m - 1)) * (fabs(v1) + fabs(v2)) <=
              eps * fabs(v0) * (fabs(HH(m - 1, m - 1)) + fabs(HH(m, m)) + fabs(HH(m + 1, m + 1))))
            atomicMax(&c.mx, m);
        }
      }
      __syncthreads();
      const int mx = c.mx;
      // reflector of the first step from the start vector
      if (tid == 0) {
        const T r1r = c.s[0], r1i = c.s[1], r2r = c.s[2], r2i = c.s[3];
        const int m = mx;
        T h21s = HH(m + 1, m);
        T s = fabs(HH(m, m) - r2r) + fabs(r2i) + fabs(h21s);
        h21s /= s;
        T v0 = h21s * HH(m, m + 1) + (HH(m, m) - r1r) * ((HH(m, m) - r2r) / s) - r1i * (r2i / s);
        T v1 = h21s * (HH(m, m) + HH(m + 1, m + 1) - r1r - r2r);
        T v2 = h21s * HH(m + 2, m + 1);
        s = fabs(v0) + fabs(v1) + fabs(v2);
        v0 /= s; v1 /= s; v2 /= s;
        const int nr = min(3, iend - mx + 1);
        const T t1 = reflector_fast(v0, v1, v2, nr);
        if (mx > istart) HH(mx, mx - 1) *= (T(1) - t1);
        Refl<T>& r = c.r[0];
        r.t1 = t1; r.v2 = v1; r.v3 = v2; r.t2 = t1 * v1; r.t3 = t1 * v2;
        T* l = lg + 5 * (mx - 1);
        l[0] = t1; l[1] = r.t2; l[2] = r.t3; l[3] = v1; l[4] = v2;
      }
      __syncthreads();
      // bulge chase (GenericSchur.jl:877-949), steps with a 3-element reflector
      int cur = 0;
      for (int k = mx; k <= iend - 2; ++k) {
        const Refl<T> r = c.r[cur];
        if (warp == 0) {
          // near block: left on columns k..k+2, then right on rows k..min(k+3, iend)
          if (lane < 3) left3(H, k, k + lane, r);
          __syncwarp();
          if (lane < 4 && k + lane <= iend) right3(H, k, k + lane, r);
          __syncwarp();
          if (lane == 0) make_refl(H, k + 1, iend, c.r[cur ^ 1], lg);
        } else {
          // one task list: far columns k+3..n (left), then far rows 1..k-1 (right)
          const int ft = tid - 32;
          constexpr int NF = NT - 32;
          const int nl = n - k - 2;
          const int ntask = nl + k - 1;
          for (int t = ft; t < ntask; t += NF) {
            if (t < nl) left3(H, k, k + 3 + t, r);
            else right3(H, k, t - nl + 1, r);
          }
        }
        __syncthreads();
        cur ^= 1;
      }
      // last step: 2-element reflector at k = iend-1 (left on columns k..n, right on rows 1..iend)
      {
        const int k = iend - 1;
        const Refl<T> r = c.r[cur];
        for (int j = k + tid; j <= n; j += NT) left2(H, k, j, r);
        __syncthreads();
        for (int i = 1 + tid; i <= iend; i += NT) right2(H, k, i, r);
      }
      __syncthreads();
      // apply the sweep's reflectors to the Z rows each thread owns
      if (Zg) {
        for (int r = tid; r < n; r += NT) {
          T* zr = Zg + r;
          T z0 = zr[(long long)(mx - 1) * n], z1 = zr[(long long)mx * n];
          for (int k = mx; k <= iend - 1; ++k) {
            const T* l = lg + 5 * (k - 1);
            if (k <= iend - 2) {
              const T z2 = zr[(long long)(k + 1) * n];
              const T ss = fma(l[4], z2, fma(l[3], z1, z0));
              zr[(long long)(k - 1) * n] = fma(-ss, l[0], z0);
              z0 = fma(-ss, l[1], z1);
              z1 = fma(-ss, l[2], z2);
            } else {
              const T ss = fma(l[3], z1, z0);
              zr[(long long)(k - 1) * n] = fma(-ss, l[0], z0);
              zr[(long long)k * n] = fma(-ss, l[1], z1);
            }
          }
        }
      }
    }
    if (status != ST_OK) break;
    __syncthreads();
    if (deflate && istart >= iend) {
      if (tid == 0) { wr[iend - 1] = (W)HH(iend, iend); wi[iend - 1] = W(0); }
    } else if (deflate && istart + 1 == iend) {
      const int p = iend - 1, q = iend;
      if (tid == 0) {
        double a = HH(p, p), bq = HH(p, q), cc = HH(q, p), d = HH(q, q), cs, sn, w1r, w1i, w2r, w2i;
        gs2x2(a, bq, cc, d, cs, sn, w1r, w1i, w2r, w2i);
        wr[q - 1] = (W)w2r; wi[q - 1] = (W)w2i; wr[p - 1] = (W)w1r; wi[p - 1] = (W)w1i;
        c.g[0] = (T)cs; c.g[1] = (T)sn;
        c.blk[0] = (T)a; c.blk[1] = (T)bq; c.blk[2] = (T)cc; c.blk[3] = (T)d;
      }
      __syncthreads();
      const T cs = c.g[0], sn = c.g[1];
      for (int j = q + 1 + tid; j <= n; j += NT) {  // lmul!(G, HH[:, istart:n]) beyond the block
        const T a1 = HH(p, j), a2 = HH(q, j);
        HH(p, j) = cs * a1 + sn * a2;
        HH(q, j) = -sn * a1 + cs * a2;
      }
      for (int r = 1 + tid; r <= p - 1; r += NT) {  // rmul!(HH[1:iend, :], G') above the block
        const T a1 = HH(r, p), a2 = HH(r, q);
        HH(r, p) = cs * a1 + sn * a2;
        HH(r, q) = -sn * a1 + cs * a2;
      }
      if (Zg)
        for (int r = tid; r < n; r += NT) {
          T* zp = Zg + r + (long long)(p - 1) * n;
          const T a1 = zp[0], a2 = zp[n];
          zp[0] = cs * a1 + sn * a2;
          zp[n] = -sn * a1 + cs * a2;
        }
      if (tid == 0) {
        HH(p, p) = c.blk[0]; HH(p, q) = c.blk[1]; HH(q, p) = c.blk[2]; HH(q, q) = c.blk[3];
        if (iend > 2) HH(iend - 1, iend - 2) = T(0);
      }
    }
    iend = istart - 1;
    __syncthreads();
  }
  __syncthreads();

  // ---- 6. write back -----------------------------------------------------------
  double mul[8];
  int nf = 0;
  if (scaled) nf = safescale_factors(cscale, amax, mul);
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    double v = (i > j + 1) ? 0.0 : (double)HH(i + 1, j + 1);
    for (int f = 0; f < nf; ++f) v *= mul[f];
    Ag[idx] = (T)v;
  }
  if (scaled)
    for (int i = tid; i < n; i += NT) {
      double a = wr[i], bq = wi[i];
      for (int f = 0; f < nf; ++f) { a *= mul[f]; bq *= mul[f]; }
      wr[i] = (W)a; wi[i] = (W)bq;
    }
  if (tid == 0) bt.status[b] = status;
  __syncthreads();
}
#undef AA
#undef HH

template <class T, class W, int NT, bool HSMEM>
__global__ void __launch_bounds__(NT) k_schur_real(RealBatchT<T, W> bt, const int* __restrict__ order,
                                                   int* __restrict__ sched, int bin, int nmax) {
  extern __shared__ double smem_raw[];
  T* smem = (T*)smem_raw;
  __shared__ Ctl<T> c;
  __shared__ int s_job;
  const int start = sched[3 * bin], end = sched[3 * bin + 1];
  for (;;) {
    if (threadIdx.x == 0) s_job = start + atomicAdd(&sched[3 * bin + 2], 1);
    __syncthreads();
    const int job = s_job;
    __syncthreads();
    if (job >= end) break;
    solve_real<T, W, NT, HSMEM>(bt, order[job], nmax, smem, c);
  }
}

// Dynamic shared memory of one CTA for orders up to nmax: the packed H of the QR phase
// (or the full matrix of the Hessenberg phase, hsmem), tau, the reflector log and the
// reduction scratch.
size_t bin_smem_elems(int nmax, bool hsmem) {
  const size_t full = hsmem ? (size_t)nmax * (nmax | 1) : 0;
  const size_t hreg = full > (size_t)rpk(nmax + 1) ? full : (size_t)rpk(nmax + 1);
  return hreg + 6 * (size_t)nmax + 32;
}

template <class T, class W, int NT, bool HSMEM>
cudaError_t launch_bin(const RealBatchT<T, W>& bt, const int* order, int* sched, int bin, int nmax, int ctas,
                       int num_sms, cudaStream_t s) {
  const size_t smem = sizeof(T) * bin_smem_elems(nmax, HSMEM);
  cudaError_t e = cudaFuncSetAttribute(k_schur_real<T, W, NT, HSMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_schur_real<T, W, NT, HSMEM>, NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (ctas > 0 && per_sm > ctas) per_sm = ctas;
  k_schur_real<T, W, NT, HSMEM><<<num_sms * per_sm, NT, smem, s>>>(bt, order, sched, bin, nmax);
  return cudaGetLastError();
}

// One bin with the requested shape.  FP64 compiles every shape of kTuneThreads with
// and without the shared-memory Hessenberg phase, the FP32 kernel with FP32 eigenvalues
// (Float32 batches and the FP32 stage of the mixed form) the same but 160 threads, the
// FP32 kernel with FP64 eigenvalues (the large path's small solves) the default shapes.
template <class T, class W>
cudaError_t launch_shape(const RealBatchT<T, W>& bt, const int* order, int* sched, int bin, int nmax, int nt,
                         int hsmem, int ctas, int num_sms, cudaStream_t s) {
#define GS_SHAPE(NTV, HS) \
  if (nt == NTV && (hsmem != 0) == HS) return launch_bin<T, W, NTV, HS>(bt, order, sched, bin, nmax, ctas, num_sms, s);
  if constexpr (sizeof(T) == 8) {
    GS_SHAPE(64, true) GS_SHAPE(64, false) GS_SHAPE(96, true) GS_SHAPE(96, false)
    GS_SHAPE(128, true) GS_SHAPE(128, false) GS_SHAPE(160, true) GS_SHAPE(160, false)
    GS_SHAPE(192, true) GS_SHAPE(192, false) GS_SHAPE(256, true) GS_SHAPE(256, false)
  } else if constexpr (std::is_same_v<W, float>) {
    GS_SHAPE(64, true) GS_SHAPE(64, false) GS_SHAPE(96, true) GS_SHAPE(96, false)
    GS_SHAPE(128, true) GS_SHAPE(128, false) GS_SHAPE(192, true) GS_SHAPE(192, false)
    GS_SHAPE(256, true) GS_SHAPE(256, false)
  } else {
    GS_SHAPE(64, true) GS_SHAPE(128, false)
  }
#undef GS_SHAPE
  return cudaErrorInvalidValue;
}

template <class T, class W>
cudaError_t launch_all_bins(const RealBatchT<T, W>& bt, const int* order, int* sched, int num_sms,
                            cudaStream_t* streams, int nstreams, const BinTuning& t) {
  // largest bin first: it carries most of the work
  for (int i = 0; i < kNumBins; ++i) {
    const int bin = kNumBins - 1 - i;
    cudaError_t e = launch_shape(bt, order, sched, bin, t.bounds[bin], t.nt[bin], t.hsmem[bin], t.ctas[bin], num_sms,
                                 streams[i % nstreams]);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

size_t real_bin_smem_bytes(int nmax, int hsmem) { return sizeof(double) * bin_smem_elems(nmax, hsmem != 0); }
size_t real32_bin_smem_bytes(int nmax, int hsmem) { return sizeof(float) * bin_smem_elems(nmax, hsmem != 0); }

template <class T, class W>
cudaError_t launch_schur_batched_real(const RealBatchT<T, W>& bt, const int* order, int* sched, int num_sms,
                                      cudaStream_t* streams, int nstreams) {
  return launch_all_bins(bt, order, sched, num_sms, streams, nstreams, default_tuning_real());
}
template cudaError_t launch_schur_batched_real<double, double>(const RealBatchT<double, double>&, const int*, int*, int,
                                                               cudaStream_t*, int);
template cudaError_t launch_schur_batched_real<float, double>(const RealBatchT<float, double>&, const int*, int*, int,
                                                              cudaStream_t*, int);
template cudaError_t launch_schur_batched_real<float, float>(const RealBatchT<float, float>&, const int*, int*, int,
                                                             cudaStream_t*, int);

template <class T, class W>
cudaError_t launch_schur_real_one(const RealBatchT<T, W>& bt, int m, const int* order, int* sched, cudaStream_t s) {
  const BinTuning t = default_tuning_real();
  const int bin = default_bin_of(m);
  return launch_shape(bt, order, sched, bin, t.bounds[bin], t.nt[bin], t.hsmem[bin], 1, 1, s);
}
template cudaError_t launch_schur_real_one<double, double>(const RealBatchT<double, double>&, int, const int*, int*,
                                                           cudaStream_t);
template cudaError_t launch_schur_real_one<float, double>(const RealBatchT<float, double>&, int, const int*, int*,
                                                          cudaStream_t);

cudaError_t launch_schur_batched_real_tuned(const RealBatchT<double, double>& bt, const int* order, int* sched,
                                            int num_sms, cudaStream_t* streams, int nstreams, const BinTuning& tun) {
  return launch_all_bins(bt, order, sched, num_sms, streams, nstreams, tun);
}

cudaError_t launch_schur_batched_real32_tuned(const RealBatchT<float, float>& bt, const int* order, int* sched,
                                              int num_sms, cudaStream_t* streams, int nstreams, const BinTuning& tun) {
  return launch_all_bins(bt, order, sched, num_sms, streams, nstreams, tun);
}

}  // namespace gsk
