// Batched complex Schur decomposition, one CTA per matrix (n <= 128), FP64.
//
// Per matrix (GenericSchur.jl:350-372 driver):
//   1. load + _scale! (util.jl:14-29);
//   2. complex Householder Hessenberg reduction (hessenberg.jl:3-17; reflector
//      householder.jl:56-102, which also makes the last subdiagonal real);
//   3. Q formation into Z (hessenberg.jl:150-166), row-owner threads;
//   4. single-shift complex QR of gschur!(H::Hessenberg{Complex}, Z)
//      (GenericSchur.jl:194-335) with singleShiftQR! (374-504): Ahues-Tisseur
//      deflation, Wilkinson / exceptional shifts, 2-element reflector chase, the
//      phase fix-ups that keep the subdiagonal real;
//   5. T = triu(H), w = diag(T), scaling undone.
// A complex 128x128 matrix does not fit in shared memory, so the two larger bins
// reduce to Hessenberg form in the (L2-resident) output buffer and run the QR
// phase on a packed upper-Hessenberg copy in shared memory; the two smaller bins
// keep the whole matrix in shared memory throughout.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

struct ZRefl {
  double2 t1, v2;
  double t2;
};

struct CtlC {
  double2 v[2];
  ZRefl r[2];
  double2 shift;
  double2 ph;   // phase factor t of the start-row fix-up
  double2 tail; // phase factor of the tail fix-up
  int split;
  int mx;
  int phase_on, tail_on;
};

// Column offset in the packed layout of the QR phase: column j (1-based) holds
// rows 1..j+2 contiguously -- the upper Hessenberg part plus the row of the
// single-shift bulge, H[k+1, k-1].
__host__ __device__ __forceinline__ int pk_off(int j) { return ((j - 1) * (j + 4)) >> 1; }

template <bool PACKED>
struct HAcc {
  double2* p;
  int ld;
  __device__ __forceinline__ double2& operator()(int i, int j) const {
    if constexpr (PACKED) return p[pk_off(j) + i - 1];
    else return p[(i - 1) + (j - 1) * ld];
  }
};

// Hessenberg reduction on an n x n complex matrix at A (shared or global), ld.
template <int NT>
__device__ void hessenberg_cplx(int n, double2* A, int ld, double2* tau, double* red) {
  const int tid = threadIdx.x;
  const double sfmin = kFmin / kEps;
#define AA(i, j) A[((i) - 1) + ((j) - 1) * ld]
  for (int i = 1; i <= n - 1; ++i) {
    const int m = n - i;
    double2* col = &AA(i + 1, i);
    double lmax = 0.0;
    for (int r = 1 + tid; r < m; r += NT) lmax = fmax(lmax, fmax(fabs(col[r].x), fabs(col[r].y)));
    const double big = block_max<NT>(lmax, red);
    const double2 alpha0 = col[0];
    double2 tau_i = make_double2(0.0, 0.0);
    bool trivial = (big == 0.0 && alpha0.y == 0.0);
    if (!trivial) {
      double xnorm = 0.0;
      if (big != 0.0) {
        const bool safe = (big < 1.0e150 && big > 1.0e-150);
        const double sc = safe ? 1.0 : 1.0 / big;
        double ls = 0.0;
        for (int r = 1 + tid; r < m; r += NT) {
          const double a = col[r].x * sc, b = col[r].y * sc;
          ls = fma(a, a, fma(b, b, ls));
        }
        const double ssq = block_sum<NT>(ls, red);
        xnorm = safe ? sqrt(ssq) : big * sqrt(ssq);
      }
      double ar = alpha0.x, ai = alpha0.y;
      // hypot3(ar, ai, xnorm) (util.jl:562-570)
      auto hyp3 = [](double x, double y, double z) {
        const double w = fmax(fabs(x), fmax(fabs(y), fabs(z)));
        if (w == 0.0) return 0.0;
        const double rw = 1.0 / w;
        const double a = x * rw, b = y * rw, c = z * rw;
        return w * sqrt(fma(a, a, fma(b, b, c * c)));
      };
      double beta = -copysign(hyp3(ar, ai, xnorm), ar);
      int kount = 0;
      if (fabs(beta) < sfmin) {
        const double rsfmin = 1.0 / sfmin;
        double bb = beta;
        do { ++kount; bb *= rsfmin; ar *= rsfmin; ai *= rsfmin; } while (fabs(bb) < sfmin && kount < 20);
        __syncthreads();
        for (int r = 1 + tid; r < m; r += NT) {
          double2 t = col[r];
          for (int q = 0; q < kount; ++q) t = zscal(t, rsfmin);
          col[r] = t;
        }
        __syncthreads();
        double lm2 = 0.0;
        for (int r = 1 + tid; r < m; r += NT) lm2 = fmax(lm2, fmax(fabs(col[r].x), fabs(col[r].y)));
        const double big2 = block_max<NT>(lm2, red);
        const double sc2 = big2 > 0.0 ? 1.0 / big2 : 0.0;
        double ls2 = 0.0;
        for (int r = 1 + tid; r < m; r += NT) {
          const double a = col[r].x * sc2, b = col[r].y * sc2;
          ls2 = fma(a, a, fma(b, b, ls2));
        }
        const double ssq2 = block_sum<NT>(ls2, red);
        xnorm = big2 * sqrt(ssq2);
        beta = -copysign(hyp3(ar, ai, xnorm), ar);
      }
      tau_i = make_double2((beta - ar) / beta, -ai / beta);
      const double2 t = zdiv(make_double2(1.0, 0.0), make_double2(ar - beta, ai));
      for (int r = 1 + tid; r < m; r += NT) col[r] = zmul(col[r], t);
      for (int q = 0; q < kount; ++q) beta *= sfmin;
      __syncthreads();
      if (tid == 0) col[0] = make_double2(beta, 0.0);
    }
    if (tid == 0) tau[i - 1] = tau_i;
    __syncthreads();
    if (trivial) continue;
    // lmul!(H', A[i+1:n, i+1:n]) with conj(tau)
    for (int j = i + 1 + tid; j <= n; j += NT) {
      double2* hj = &AA(i + 1, j);
      double2 va = hj[0];
      for (int r = 1; r < m; ++r) va = zfmac(col[r], hj[r], va);
      va = zmul(zconj(tau_i), va);
      hj[0] = zsub(hj[0], va);
      for (int r = 1; r < m; ++r) hj[r] = zfms(va, col[r], hj[r]);
    }
    __syncthreads();
    // rmul!(A[:, i+1:n], H): x = A1 v + a1; a1 -= tau x; A1 -= tau x v^H
    for (int r = tid; r < n; r += NT) {
      double2* hr = &A[r + i * ld];
      double2 x = hr[0];
      for (int q = 1; q < m; ++q) x = zfma(hr[q * ld], col[q], x);
      x = zmul(tau_i, x);
      hr[0] = zsub(hr[0], x);
      for (int q = 1; q < m; ++q) hr[q * ld] = zfms(x, zconj(col[q]), hr[q * ld]);
    }
    __syncthreads();
  }
#undef AA
}

// nmax: the largest order the launch sized its buffers for (the bin's maximum, or the
// single large matrix's order).  An order outside [0, nmax] read from device memory gets
// ST_BADARG before anything is read or written.
template <int NT, bool HSMEM>
__device__ void solve_cplx(const CplxBatch& bt, int b, int nmax, double2* smem, CtlC& c) {
  constexpr bool PACKED = !HSMEM;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int n = bt.ns[b];
  if (n <= 0 || n > nmax) {
    if (tid == 0) bt.status[b] = (n == 0) ? ST_OK : ST_BADARG;
    return;
  }
  double2* __restrict__ Ag = bt.A + bt.offs[b];
  double2* __restrict__ Zg = bt.wantz ? bt.Z + bt.offs[b] : nullptr;
  double2* __restrict__ wg = bt.w + bt.woffs[b];
  const int ldh = HSMEM ? (n | 1) : n;
  const int hsize = HSMEM ? n * ldh : pk_off(n + 1);
  // packed H of the QR phase (shared memory)
  double2* Hs = smem;
  double2* tau = Hs + hsize;  // n
  double2* lg = tau + n;            // 3 per chase step: t1, v2, (t2, 0)
  double* red = (double*)(lg + 3 * n);
  double2* A = HSMEM ? Hs : Ag;     // where the Hessenberg reduction runs
  const int lda = HSMEM ? ldh : n;

  // ---- 1. load and scale ---------------------------------------------------------
  double amax = 0.0;
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    const double2 a = Ag[idx];
    if (HSMEM) A[i + j * lda] = a;
    const double aa = hypot(a.x, a.y);
    amax = (aa > amax || aa != aa) ? aa : amax;
  }
  amax = block_max<NT>(amax, red);
  __syncthreads();
  const double smlnum = sqrt(kSafemin) / kEps;
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
        A[i + j * lda] = zscal(A[i + j * lda], mul[f]);
      }
    __syncthreads();
  }

  // ---- 2. Hessenberg ---------------------------------------------------------------
  hessenberg_cplx<NT>(n, A, lda, tau, red);

  // ---- 3. Q formation (row-owner threads) ---------------------------------------------
  if (Zg) {
    for (int r = tid; r < n; r += NT)
      for (int j = 0; j < n; ++j) Zg[r + j * n] = make_double2(r == j ? 1.0 : 0.0, 0.0);
    for (int i = 1; i <= n - 1; ++i) {
      const double2 t = tau[i - 1];
      if (t.x == 0.0 && t.y == 0.0) continue;
      const int m = n - i;
      const double2* col = &A[i + (i - 1) * lda];
      for (int r = tid; r < n; r += NT) {
        double2* zr = Zg + r + (long long)i * n;
        double2 s = zr[0];
        for (int q = 1; q < m; ++q) s = zfma(zr[q * n], col[q], s);
        s = zmul(s, t);
        zr[0] = zsub(zr[0], s);
        for (int q = 1; q < m; ++q) zr[q * n] = zfms(s, zconj(col[q]), zr[q * n]);
      }
    }
  }
  __syncthreads();

  // ---- 4. QR --------------------------------------------------------------------------
  // move the Hessenberg part into the layout of the QR phase
  if (!HSMEM) {
    for (int j = 1; j <= n; ++j)
      for (int i = 1 + tid; i <= j + 2; i += NT)
        Hs[pk_off(j) + i - 1] = (i <= min(j + 1, n)) ? Ag[(i - 1) + (j - 1) * n] : make_double2(0.0, 0.0);
  } else {
    for (int idx = tid; idx < n * n; idx += NT) {
      const int i = idx % n, j = idx / n;
      if (i > j + 1) Hs[i + j * ldh] = make_double2(0.0, 0.0);
    }
  }
  __syncthreads();
  const HAcc<PACKED> H{Hs, ldh};
  const double ulp = kEps;
  const double smallnum = kSafemin * ((double)n / ulp);
  const long long maxiter = bt.maxiter_abs > 0 ? bt.maxiter_abs : (long long)bt.maxiter_mult * n;
  const long long maxinner = bt.maxinner_abs > 0 ? bt.maxinner_abs : (long long)bt.maxinner_mult * n;
  long long it = 0;
  int status = ST_OK;
  int iend = n;
  while (iend >= 1 && status == ST_OK) {
    int istart = 1;
    for (long long its = 0; its <= maxinner; ++its) {
      ++it;
      if (it > maxiter) { status = ST_UNCONVERGED; break; }
      // deflation scan (GenericSchur.jl:240-286): largest k in [istart, iend-1] that splits
      if (tid == 0) c.split = 0;
      __syncthreads();
      for (int k = istart + tid; k <= iend - 1; k += NT) {
        bool split = false;
        const double2 sd = H(k + 1, k);
        if (zabs1(sd) <= smallnum) {
          split = true;
        } else {
          const double2 hkk = H(k, k), hk1 = H(k + 1, k + 1);
          double tst = zabs1(hkk) + zabs1(hk1);
          if (tst == 0.0) {
            if (k - 1 >= 1) tst += fabs(H(k, k - 1).x);
            if (k + 2 <= n) tst += fabs(H(k + 2, k + 1).x);
          }
          if (fabs(sd.x) <= ulp * tst) {
            const double2 up = H(k, k + 1);
            const double ab = fmax(zabs1(sd), zabs1(up)), ba = fmin(zabs1(sd), zabs1(up));
            const double2 df = zsub(hkk, hk1);
            const double aa = fmax(zabs1(hk1), zabs1(df)), bb = fmin(zabs1(hk1), zabs1(df));
            const double s = aa + ab;
            if (ba * (ab / s) <= fmax(smallnum, ulp * (bb * (aa / s)))) split = true;
          }
        }
        if (split) atomicMax(&c.split, k);
      }
      __syncthreads();
      if (c.split > 0) istart = c.split + 1;
      if (istart > 1 && tid == 0) H(istart, istart - 1) = make_double2(0.0, 0.0);
      if (istart >= iend) { iend -= 1; break; }
      __syncthreads();
      // shift (GenericSchur.jl:302-325)
      if (tid == 0) {
        double2 t;
        if (its % 30 == 10) {
          const double s = 0.75 * fabs(H(istart + 1, istart).x);
          t = zadd(make_double2(s, 0.0), H(istart, istart));
        } else if (its % 30 == 20) {
          const double s = 0.75 * fabs(H(iend, iend - 1).x);
          t = zadd(make_double2(s, 0.0), H(iend, iend));
        } else {
          t = H(iend, iend);
          const double2 u = zmul(zsqrt(H(iend - 1, iend)), zsqrt(H(iend, iend - 1)));
          double s = zabs1(u);
          if (s != 0.0) {
            const double2 x = zscal(zsub(H(iend - 1, iend - 1), t), 0.5);
            const double sx = zabs1(x);
            s = fmax(s, zabs1(x));
            const double2 xs = zscal(x, 1.0 / s), us = zscal(u, 1.0 / s);
            double2 y = zscal(zsqrt(zadd(zmul(xs, xs), zmul(us, us))), s);
            if (sx > 0.0) {
              const double2 xn = zscal(x, 1.0 / sx);
              if (xn.x * y.x + xn.y * y.y < 0.0) y = zneg(y);
            }
            t = zsub(t, zmul(u, zdiv(u, zadd(x, y))));
          }
        }
        c.shift = t;
        c.mx = istart;
      }
      __syncthreads();
      // start row (GenericSchur.jl:390-407): largest mm with a negligible product
      {
        const double2 shift = c.shift;
        for (int mm = istart + 1 + tid; mm <= iend - 1; mm += NT) {
          const double2 h11 = H(mm, mm), h22 = H(mm + 1, mm + 1);
          double2 h11s = zsub(h11, shift);
          double h21 = H(mm + 1, mm).x;
          const double s = zabs1(h11s) + fabs(h21);
          h11s = zscal(h11s, 1.0 / s);
          h21 /= s;
          const double h10 = H(mm, mm - 1).x;
          if (fabs(h10) * fabs(h21) <= ulp * (zabs1(h11s) * (zabs1(h11) + zabs1(h22)))) atomicMax(&c.mx, mm);
        }
      }
      __syncthreads();
      const int k0 = c.mx;
      if (tid == 0) {
        const double2 h11 = H(k0, k0);
        double2 h11s = zsub(h11, c.shift);
        double h21 = H(k0 + 1, k0).x;
        const double s = zabs1(h11s) + fabs(h21);
        c.v[0] = zdiv(h11s, make_double2(s, 0.0));
        c.v[1] = make_double2(h21 / s, 0.0);
        c.phase_on = 0;
        c.ph = make_double2(1.0, 0.0);
      }
      // chase (GenericSchur.jl:426-484).  The first step runs on its own (its phase
      // fix-up changes the next reflector's inputs); after it, one barrier per step:
      // warp 0 updates the 3x2 near block and computes the next reflector while the
      // other warps update the far columns (k+2..n) and far rows (1..k-1).
      if (tid == 0) {
        double2 a = c.v[0], x1 = c.v[1];
        const double2 t1 = zreflector2_fast(a, x1);
        c.r[0].t1 = t1; c.r[0].v2 = x1; c.r[0].t2 = zmul(t1, x1).x;
        double2* l = lg + 3 * (k0 - 1);
        l[0] = t1; l[1] = x1; l[2] = make_double2(c.r[0].t2, 0.0);
      }
      __syncthreads();
      {
        const int k = k0;
        const double2 t1 = c.r[0].t1, v2 = c.r[0].v2;
        const double t2 = c.r[0].t2;
        for (int j = k + tid; j <= n; j += NT) {
          const double2 h0 = H(k, j), h1 = H(k + 1, j);
          const double2 ss = zadd(zmul(zconj(t1), h0), zscal(h1, t2));
          H(k, j) = zsub(h0, ss);
          H(k + 1, j) = zfms(ss, v2, h1);
        }
        __syncthreads();
        const int rl = min(k + 2, iend);
        for (int r = 1 + tid; r <= rl; r += NT) {
          const double2 h0 = H(r, k), h1 = H(r, k + 1);
          const double2 ss = zadd(zmul(t1, h0), zscal(h1, t2));
          H(r, k) = zsub(h0, ss);
          H(r, k + 1) = zfms(ss, zconj(v2), h1);
        }
        if (k0 > istart) {
          // phase fix-up keeping H[k0+1, k0] real (GenericSchur.jl:461-482)
          __syncthreads();
          if (tid == 0) {
            double2 t = zsub(make_double2(1.0, 0.0), t1);
            t = zscal(t, 1.0 / hypot(t.x, t.y));
            c.ph = t;
            c.phase_on = 1;
            H(k0 + 1, k0) = zmul(H(k0 + 1, k0), zconj(t));
            if (k0 + 2 <= iend) H(k0 + 2, k0 + 1) = zmul(H(k0 + 2, k0 + 1), t);
          }
          __syncthreads();
          const double2 t = c.ph;
          for (int col = k0 + 1 + tid; col <= n; col += NT)
            for (int j = k0; j <= min(iend, col - 1); ++j)
              if (j != k0 + 1) H(j, col) = zmul(H(j, col), t);
          __syncthreads();
          for (int j = k0 + tid; j <= iend; j += NT)
            if (j != k0 + 1)
              for (int r = 1; r <= j - 1; ++r) H(r, j) = zmul(H(r, j), zconj(t));
        }
        __syncthreads();
        if (tid == 0 && k0 + 1 <= iend - 1) {
          const int kk = k0 + 1;
          double2 a = H(kk, kk - 1), x1 = H(kk + 1, kk - 1);
          const double2 tn = zreflector2_fast(a, x1);
          H(kk, kk - 1) = a;
          H(kk + 1, kk - 1) = make_double2(0.0, 0.0);
          c.r[1].t1 = tn; c.r[1].v2 = x1; c.r[1].t2 = zmul(tn, x1).x;
          double2* l = lg + 3 * (kk - 1);
          l[0] = tn; l[1] = x1; l[2] = make_double2(c.r[1].t2, 0.0);
        }
        __syncthreads();
      }
      {
        int cur = 1;
        for (int k = k0 + 1; k <= iend - 1; ++k) {
          const ZRefl r = c.r[cur];
          if (warp == 0) {
            if (lane < 2) {  // left on columns k, k+1 (rows k, k+1)
              const int j = k + lane;
              const double2 h0 = H(k, j), h1 = H(k + 1, j);
              const double2 ss = zadd(zmul(zconj(r.t1), h0), zscal(h1, r.t2));
              H(k, j) = zsub(h0, ss);
              H(k + 1, j) = zfms(ss, r.v2, h1);
            }
            __syncwarp();
            if (lane < 3 && k + lane <= min(k + 2, iend)) {  // right on rows k..k+2 (columns k, k+1)
              const int rr = k + lane;
              const double2 h0 = H(rr, k), h1 = H(rr, k + 1);
              const double2 ss = zadd(zmul(r.t1, h0), zscal(h1, r.t2));
              H(rr, k) = zsub(h0, ss);
              H(rr, k + 1) = zfms(ss, zconj(r.v2), h1);
            }
            __syncwarp();
            if (lane == 0 && k + 1 <= iend - 1) {
              const int kk = k + 1;
              double2 a = H(kk, kk - 1), x1 = H(kk + 1, kk - 1);
              const double2 tn = zreflector2_fast(a, x1);
              H(kk, kk - 1) = a;
              H(kk + 1, kk - 1) = make_double2(0.0, 0.0);
              ZRefl& o = c.r[cur ^ 1];
              o.t1 = tn; o.v2 = x1; o.t2 = zmul(tn, x1).x;
              double2* l = lg + 3 * (kk - 1);
              l[0] = tn; l[1] = x1; l[2] = make_double2(o.t2, 0.0);
            }
          } else {
            const int ft = tid - 32;
            constexpr int NF = NT - 32;
            for (int j = k + 2 + ft; j <= n; j += NF) {
              const double2 h0 = H(k, j), h1 = H(k + 1, j);
              const double2 ss = zadd(zmul(zconj(r.t1), h0), zscal(h1, r.t2));
              H(k, j) = zsub(h0, ss);
              H(k + 1, j) = zfms(ss, r.v2, h1);
            }
            for (int rr = 1 + ft; rr <= k - 1; rr += NF) {
              const double2 h0 = H(rr, k), h1 = H(rr, k + 1);
              const double2 ss = zadd(zmul(r.t1, h0), zscal(h1, r.t2));
              H(rr, k) = zsub(h0, ss);
              H(rr, k + 1) = zfms(ss, zconj(r.v2), h1);
            }
          }
          __syncthreads();
          cur ^= 1;
        }
      }
      __syncthreads();
      // tail: keep H[iend, iend-1] real (GenericSchur.jl:486-500)
      if (tid == 0) {
        double2 t = H(iend, iend - 1);
        c.tail_on = 0;
        if (t.y != 0.0) {
          const double rt = hypot(t.x, t.y);
          H(iend, iend - 1) = make_double2(rt, 0.0);
          c.tail = zscal(t, 1.0 / rt);
          c.tail_on = 1;
        }
      }
      __syncthreads();
      if (c.tail_on) {
        const double2 t = c.tail;
        for (int col = iend + 1 + tid; col <= n; col += NT) H(iend, col) = zmul(H(iend, col), zconj(t));
        for (int r = 1 + tid; r <= iend - 1; r += NT) H(r, iend) = zmul(H(r, iend), t);
      }
      // Z rows: the sweep's reflectors, the start phase and the tail phase, in order
      if (Zg) {
        const bool ph = c.phase_on;
        const double2 pt = zconj(c.ph);
        const bool tl = c.tail_on;
        const double2 tt = c.tail;
        for (int r = tid; r < n; r += NT) {
          double2* zr = Zg + r;
          double2 z0 = zr[(long long)(k0 - 1) * n], z1 = zr[(long long)k0 * n];
          for (int k = k0; k <= iend - 1; ++k) {
            const double2* l = lg + 3 * (k - 1);
            const double2 t1 = l[0], v2 = l[1];
            const double t2 = l[2].x;
            const double2 ss = zadd(zmul(t1, z0), zscal(z1, t2));
            z0 = zsub(z0, ss);
            z1 = zfms(ss, zconj(v2), z1);
            if (k == k0 && ph) z0 = zmul(z0, pt);  // column k0 is in the phased set
            if (k == iend - 1) {
              if (tl) z1 = zmul(z1, tt);
              zr[(long long)(k - 1) * n] = z0;
              zr[(long long)k * n] = z1;
            } else {
              zr[(long long)(k - 1) * n] = z0;
              z0 = z1;
              z1 = zr[(long long)(k + 1) * n];
              if (ph && k + 2 <= iend) z1 = zmul(z1, pt);  // columns k0+2..iend are phased
            }
          }
        }
      }
      __syncthreads();
    }
    __syncthreads();
  }
  __syncthreads();

  // ---- 5. write back --------------------------------------------------------------
  double mul[8];
  int nf = 0;
  if (scaled) nf = safescale_factors(cscale, amax, mul);
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    double2 v = (i > j) ? make_double2(0.0, 0.0) : H(i + 1, j + 1);
    for (int f = 0; f < nf; ++f) v = zscal(v, mul[f]);
    Ag[idx] = v;
    if (i == j) wg[i] = v;
  }
  if (tid == 0) bt.status[b] = status;
  __syncthreads();
}

template <int NT, bool HSMEM>
__global__ void __launch_bounds__(NT) k_schur_cplx(CplxBatch bt, const int* __restrict__ order,
                                                   int* __restrict__ sched, int bin, int nmax) {
  extern __shared__ double2 smemz[];
  __shared__ CtlC c;
  __shared__ int s_job;
  const int start = sched[3 * bin], end = sched[3 * bin + 1];
  for (;;) {
    if (threadIdx.x == 0) s_job = start + atomicAdd(&sched[3 * bin + 2], 1);
    __syncthreads();
    const int job = s_job;
    __syncthreads();
    if (job >= end) break;
    solve_cplx<NT, HSMEM>(bt, order[job], nmax, smemz, c);
  }
}

size_t cbin_smem_bytes(int nmax, bool hsmem) {
  const size_t hsize = hsmem ? (size_t)nmax * (nmax | 1) : (size_t)pk_off(nmax + 1);
  return sizeof(double2) * (hsize + 4 * (size_t)nmax) + 32 * sizeof(double) + 64;
}

template <int NT, bool HSMEM>
cudaError_t launch_bin_c(const CplxBatch& bt, const int* order, int* sched, int bin, int nmax, int ctas, int num_sms,
                         cudaStream_t s) {
  const size_t smem = cbin_smem_bytes(nmax, HSMEM);
  cudaError_t e = cudaFuncSetAttribute(k_schur_cplx<NT, HSMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_schur_cplx<NT, HSMEM>, NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (ctas > 0 && per_sm > ctas) per_sm = ctas;
  k_schur_cplx<NT, HSMEM><<<num_sms * per_sm, NT, smem, s>>>(bt, order, sched, bin, nmax);
  return cudaGetLastError();
}

// One bin with the requested shape (every shape of kTuneThreads, with and without the
// shared-memory Hessenberg phase).
cudaError_t launch_shape_c(const CplxBatch& bt, const int* order, int* sched, int bin, int nmax, int nt, int hsmem,
                           int ctas, int num_sms, cudaStream_t s) {
#define GS_SHAPE(NTV, HS) \
  if (nt == NTV && (hsmem != 0) == HS) return launch_bin_c<NTV, HS>(bt, order, sched, bin, nmax, ctas, num_sms, s);
  GS_SHAPE(64, true) GS_SHAPE(64, false) GS_SHAPE(96, true) GS_SHAPE(96, false)
  GS_SHAPE(128, true) GS_SHAPE(128, false) GS_SHAPE(160, true) GS_SHAPE(160, false)
  GS_SHAPE(192, true) GS_SHAPE(192, false) GS_SHAPE(256, true) GS_SHAPE(256, false)
#undef GS_SHAPE
  return cudaErrorInvalidValue;
}

}  // namespace


cudaError_t launch_schur_batched_cplx_tuned(const CplxBatch& bt, const int* order, int* sched, int num_sms,
                                            cudaStream_t* streams, int nstreams, const BinTuning& t) {
  // largest bin first: it carries most of the work
  for (int i = 0; i < kNumBins; ++i) {
    const int bin = kNumBins - 1 - i;
    cudaError_t e = launch_shape_c(bt, order, sched, bin, t.bounds[bin], t.nt[bin], t.hsmem[bin], t.ctas[bin],
                                   num_sms, streams[i % nstreams]);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_schur_batched_cplx(const CplxBatch& bt, const int* order, int* sched, int num_sms,
                                      cudaStream_t* streams, int nstreams) {
  return launch_schur_batched_cplx_tuned(bt, order, sched, num_sms, streams, nstreams, default_tuning_cplx());
}

size_t cplx_bin_smem_bytes(int nmax, int hsmem) { return cbin_smem_bytes(nmax, hsmem != 0); }

cudaError_t launch_schur_cplx_one(const CplxBatch& bt, int m, const int* order, int* sched, cudaStream_t s) {
  const BinTuning t = default_tuning_cplx();
  const int bin = default_bin_of(m);
  return launch_shape_c(bt, order, sched, bin, t.bounds[bin], t.nt[bin], t.hsmem[bin], 1, 1, s);
}

}  // namespace gsk
