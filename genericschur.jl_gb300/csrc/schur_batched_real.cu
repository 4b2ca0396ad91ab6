// Batched real Schur decomposition, one CTA per matrix (n <= 128), FP64.
//
// Each CTA pulls matrix indices from its size bin's work queue (a ticket counter
// in global memory) and runs, for one matrix:
//   1. load + _scale! (util.jl:14-29), the matrix held in shared memory with an
//      odd leading dimension so that row and column sweeps are bank-conflict free;
//   2. Householder Hessenberg reduction (hessenberg.jl:3-17), reflector math as in
//      householder.jl:12-54, lmul!/rmul! as householder.jl:140-172;
//   3. Q formation (hessenberg.jl:150-166) straight into the Z output, each thread
//      owning whole rows of Z so that Z never needs a barrier;
//   4. the real double-shift Francis iteration of gschur!(H::Hessenberg{<:Real}, Z)
//      (GenericSchur.jl:513-699) with doubleShiftQR! (837-952) and _gs2x2! (716-803).
//      The deflation scan and the start-row search run one candidate per thread;
//      the bulge chase updates H in shared memory; the sweep's reflectors are
//      logged and applied to Z rows afterwards in one streaming pass;
//   5. T, eigenvalues and status written back, undoing the scaling.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

struct Ctl {
  double v[3];          // start vector of the sweep
  double t1, t2, t3, v2, v3;  // current reflector
  double s[4];          // shifts r1r, r1i, r2r, r2i
  double g[2];          // Givens cs, sn of a 2x2 deflation
  int split;
  int mx;
};

// 1-based accessor into the shared copy of H.
#define HH(i, j) H[((i) - 1) + ((j) - 1) * ldh]

template <int NT>
__device__ void solve_real(const RealBatch& bt, int b, double* smem, Ctl& c) {
  const int tid = threadIdx.x;
  const int n = bt.ns[b];
  if (n <= 0) {
    if (tid == 0) bt.status[b] = ST_OK;
    return;
  }
  const int ldh = n | 1;
  double* H = smem;
  double* tau = H + n * ldh;  // n-1 reflector scalars
  double* lg = tau + n;       // 5 per chase step: t1, t2, t3, v2, v3
  double* red = lg + 5 * n;   // reduction scratch (32)
  double* __restrict__ Ag = bt.A + bt.offs[b];
  double* __restrict__ Zg = bt.wantz ? bt.Z + bt.offs[b] : nullptr;
  double* __restrict__ wr = bt.wr + bt.woffs[b];
  double* __restrict__ wi = bt.wi + bt.woffs[b];

  // ---- 1. load and scale --------------------------------------------------
  double amax = 0.0;
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    const double a = Ag[idx];
    H[i + j * ldh] = a;
    const double aa = fabs(a);
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
        H[i + j * ldh] *= mul[f];
      }
    __syncthreads();
  }

  // ---- 2. Hessenberg reduction ------------------------------------------------
  const double sfmin = 2.0 * kFmin / kEps;
  for (int i = 1; i <= n - 2; ++i) {
    const int m = n - i;                 // reflector length: rows i+1..n
    double* col = &HH(i + 1, i);         // col[0] = alpha, col[1..m-1] = x
    double lmax = 0.0;
    for (int r = 1 + tid; r < m; r += NT) lmax = fmax(lmax, fabs(col[r]));
    const double big = block_max<NT>(lmax, red);
    double tau_i = 0.0;
    if (big != 0.0) {
      const bool safe = (big < 1.0e150 && big > 1.0e-150);
      const double sc = safe ? 1.0 : 1.0 / big;
      double ls = 0.0;
      for (int r = 1 + tid; r < m; r += NT) { const double t = col[r] * sc; ls = fma(t, t, ls); }
      const double ssq = block_sum<NT>(ls, red);
      double xnorm = safe ? sqrt(ssq) : big * sqrt(ssq);
      double alpha = col[0];
      double beta = -copysign(hypot(alpha, xnorm), alpha);
      int kount = 0;
      if (fabs(beta) < sfmin) {
        // underflow guard (householder.jl:25-42): rescale x, alpha and beta
        const double rsfmin = 1.0 / sfmin;
        double bb = beta;
        do { ++kount; bb *= rsfmin; alpha *= rsfmin; } while (fabs(bb) < sfmin && kount < 20);
        __syncthreads();
        for (int r = 1 + tid; r < m; r += NT) {
          double t = col[r];
          for (int q = 0; q < kount; ++q) t *= rsfmin;
          col[r] = t;
        }
        __syncthreads();
        double lm2 = 0.0;
        for (int r = 1 + tid; r < m; r += NT) lm2 = fmax(lm2, fabs(col[r]));
        const double big2 = block_max<NT>(lm2, red);
        const double sc2 = (big2 > 0.0) ? 1.0 / big2 : 0.0;
        double ls2 = 0.0;
        for (int r = 1 + tid; r < m; r += NT) { const double t = col[r] * sc2; ls2 = fma(t, t, ls2); }
        const double ssq2 = block_sum<NT>(ls2, red);
        xnorm = big2 * sqrt(ssq2);
        beta = -copysign(hypot(alpha, xnorm), alpha);
      }
      tau_i = (beta - alpha) / beta;
      const double t = 1.0 / (alpha - beta);
      for (int r = 1 + tid; r < m; r += NT) col[r] *= t;
      for (int q = 0; q < kount; ++q) beta *= sfmin;
      __syncthreads();
      if (tid == 0) col[0] = beta;
    }
    if (tid == 0) tau[i - 1] = tau_i;
    __syncthreads();
    if (tau_i == 0.0) continue;
    // lmul!(H', A[i+1:n, i+1:n]): one column per thread
    for (int j = i + 1 + tid; j <= n; j += NT) {
      double* hj = &HH(i + 1, j);
      double va0 = hj[0], va1 = 0.0;
      int r = 1;
      for (; r + 1 < m; r += 2) { va0 = fma(col[r], hj[r], va0); va1 = fma(col[r + 1], hj[r + 1], va1); }
      if (r < m) va0 = fma(col[r], hj[r], va0);
      const double va = (va0 + va1) * tau_i;
      hj[0] -= va;
      for (r = 1; r < m; ++r) hj[r] = fma(-va, col[r], hj[r]);
    }
    __syncthreads();
    // rmul!(A[:, i+1:n], H): one row per thread
    for (int r = tid; r < n; r += NT) {
      double* hr = &H[r + i * ldh];  // row r+1, column i+1
      double x0 = hr[0], x1 = 0.0;
      int q = 1;
      for (; q + 1 < m; q += 2) { x0 = fma(hr[q * ldh], col[q], x0); x1 = fma(hr[(q + 1) * ldh], col[q + 1], x1); }
      if (q < m) x0 = fma(hr[q * ldh], col[q], x0);
      const double x = (x0 + x1) * tau_i;
      hr[0] -= x;
      for (q = 1; q < m; ++q) hr[q * ldh] = fma(-x, col[q], hr[q * ldh]);
    }
    __syncthreads();
  }

  // ---- 3. Q formation into Z (row-owner threads, no barriers) ------------------
  if (Zg) {
    for (int r = tid; r < n; r += NT)
      for (int j = 0; j < n; ++j) Zg[r + j * n] = (r == j) ? 1.0 : 0.0;
    for (int i = 1; i <= n - 2; ++i) {
      const double t = tau[i - 1];
      if (t == 0.0) continue;
      const int m = n - i;
      const double* col = &HH(i + 1, i);
      for (int r = tid; r < n; r += NT) {
        double* zr = Zg + r + (long long)i * n;  // Z[r+1, i+1]
        double s0 = zr[0], s1 = 0.0;
        int q = 1;
        for (; q + 1 < m; q += 2) { s0 = fma(zr[q * n], col[q], s0); s1 = fma(zr[(q + 1) * n], col[q + 1], s1); }
        if (q < m) s0 = fma(zr[q * n], col[q], s0);
        const double s = (s0 + s1) * t;
        zr[0] -= s;
        for (q = 1; q < m; ++q) zr[q * n] = fma(-s, col[q], zr[q * n]);
      }
    }
  }
  __syncthreads();

  // ---- 4. Francis double-shift QR ------------------------------------------------
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    if (i > j + 1) H[i + j * ldh] = 0.0;  // triu!(HH, -1)
  }
  __syncthreads();
  const double eps = kEps;
  const double smallnum = kFmin * ((double)n / eps);
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
        const double hk = HH(k, k - 1);
        if (fabs(hk) < smallnum) {
          split = true;
        } else {
          const double hkk = HH(k, k), hkm1 = HH(k - 1, k - 1);
          double t = fabs(hkm1) + fabs(hkk);
          if (t == 0.0) {
            if (k > 2) t += fabs(HH(k - 1, k - 2));
            if (k + 1 <= n) t += fabs(HH(k + 1, k));
          }
          const double ahkkm1 = fabs(hk);
          if (ahkkm1 <= t * eps) {
            const double ahkm1k = fabs(HH(k - 1, k));
            const double ab = fmax(ahkkm1, ahkm1k), ba = fmin(ahkkm1, ahkm1k);
            const double aa = fmax(fabs(hkk), fabs(hkm1 - hkk)), bb = fmin(fabs(hkk), fabs(hkm1 - hkk));
            const double s = aa + bb;
            if (ba * (ab / s) <= fmax(smallnum, eps * (bb * (aa / s)))) split = true;
          }
        }
        if (split) atomicMax(&c.split, k);
      }
      __syncthreads();
      istart = (c.split > 0) ? c.split : 1;
      if (istart > 1 && tid == 0) HH(istart, istart - 1) = 0.0;
      if (istart >= iend - 1) { deflate = true; break; }
      ++iterqr;
      __syncthreads();
      // shifts (GenericSchur.jl:614-665)
      if (tid == 0) {
        double h11, h12, h21, h22;
        if (iterqr == 10) {
          const double s = fabs(HH(istart + 1, istart)) + fabs(HH(istart + 2, istart + 1));
          h11 = 0.75 * s + HH(istart, istart); h12 = -0.4375 * s; h21 = s; h22 = h11;
        } else if (iterqr == 20) {
          const double s = fabs(HH(iend, iend - 1)) + fabs(HH(iend - 1, iend - 2));
          h11 = 0.75 * s + HH(iend, iend); h12 = -0.4375 * s; h21 = s; h22 = h11;
        } else {
          h11 = HH(iend - 1, iend - 1); h21 = HH(iend, iend - 1);
          h12 = HH(iend - 1, iend); h22 = HH(iend, iend);
        }
        const double s = fabs(h11) + fabs(h12) + fabs(h21) + fabs(h22);
        double r1r, r2r, r1i, r2i;
        if (s == 0.0) {
          r1r = r2r = r1i = r2i = 0.0;
        } else {
          h11 /= s; h12 /= s; h21 /= s; h22 /= s;
          const double tr = (h11 + h22) / 2.0;
          const double d = (h11 - tr) * (h22 - tr) - h12 * h21;
          const double rtd = sqrt(fabs(d));
          if (d >= 0.0) {
            r1r = tr * s; r2r = r1r; r1i = rtd * s; r2i = -r1i;
          } else {
            r1r = tr + rtd; r2r = tr - rtd;
            if (fabs(r1r - h22) <= fabs(r2r - h22)) { r1r *= s; r2r = r1r; }
            else { r2r *= s; r1r = r2r; }
            r1i = r2i = 0.0;
          }
        }
        c.s[0] = r1r; c.s[1] = r1i; c.s[2] = r2r; c.s[3] = r2i;
        c.mx = istart;
      }
      __syncthreads();
      // start row (GenericSchur.jl:850-872): largest m with two small subdiagonals
      {
        const double r1r = c.s[0], r1i = c.s[1], r2r = c.s[2], r2i = c.s[3];
        for (int m = istart + 1 + tid; m <= iend - 2; m += NT) {
          double h21s = HH(m + 1, m);
          double s = fabs(HH(m, m) - r2r) + fabs(r2i) + fabs(h21s);
          h21s /= s;
          double v0 = h21s * HH(m, m + 1) + (HH(m, m) - r1r) * ((HH(m, m) - r2r) / s) - r1i * (r2i / s);
          double v1 = h21s * (HH(m, m) + HH(m + 1, m + 1) - r1r - r2r);
          double v2 = h21s * HH(m + 2, m + 1);
          s = fabs(v0) + fabs(v1) + fabs(v2);
          v0 /= s; v1 /= s; v2 /= s;
          if (fabs(HH(m, m - 1)) * (fabs(v1) + fabs(v2)) <=
              eps * fabs(v0) * (fabs(HH(m - 1, m - 1)) + fabs(HH(m, m)) + fabs(HH(m + 1, m + 1))))
            atomicMax(&c.mx, m);
        }
      }
      __syncthreads();
      const int mx = c.mx;
      if (tid == 0) {
        const double r1r = c.s[0], r1i = c.s[1], r2r = c.s[2], r2i = c.s[3];
        const int m = mx;
        double h21s = HH(m + 1, m);
        double s = fabs(HH(m, m) - r2r) + fabs(r2i) + fabs(h21s);
        h21s /= s;
        double v0 = h21s * HH(m, m + 1) + (HH(m, m) - r1r) * ((HH(m, m) - r2r) / s) - r1i * (r2i / s);
        double v1 = h21s * (HH(m, m) + HH(m + 1, m + 1) - r1r - r2r);
        double v2 = h21s * HH(m + 2, m + 1);
        s = fabs(v0) + fabs(v1) + fabs(v2);
        c.v[0] = v0 / s; c.v[1] = v1 / s; c.v[2] = v2 / s;
      }
      // bulge chase (GenericSchur.jl:877-949)
      for (int k = mx; k <= iend - 1; ++k) {
        const int nr = min(3, iend - k + 1);
        __syncthreads();
        if (tid == 0) {
          double a, x1, x2 = 0.0;
          if (k > mx) {
            a = HH(k, k - 1); x1 = HH(k + 1, k - 1);
            if (nr == 3) x2 = HH(k + 2, k - 1);
          } else {
            a = c.v[0]; x1 = c.v[1]; x2 = (nr == 3) ? c.v[2] : 0.0;
          }
          const double t1 = reflector_small(a, x1, x2, nr);
          if (k > mx) {
            HH(k, k - 1) = a;
            HH(k + 1, k - 1) = 0.0;
            if (k < iend - 1) HH(k + 2, k - 1) = 0.0;
          } else if (mx > istart) {
            HH(k, k - 1) *= (1.0 - t1);
          }
          c.t1 = t1; c.v2 = x1; c.v3 = x2; c.t2 = t1 * x1; c.t3 = t1 * x2;
          double* l = lg + 5 * (k - 1);
          l[0] = t1; l[1] = t1 * x1; l[2] = t1 * x2; l[3] = x1; l[4] = x2;
        }
        __syncthreads();
        const double t1 = c.t1, t2 = c.t2, t3 = c.t3, v2 = c.v2, v3 = c.v3;
        if (nr == 3) {
          for (int j = k + tid; j <= n; j += NT) {
            double* hj = &HH(k, j);
            const double ss = fma(v3, hj[2], fma(v2, hj[1], hj[0]));
            hj[0] = fma(-ss, t1, hj[0]);
            hj[1] = fma(-ss, t2, hj[1]);
            hj[2] = fma(-ss, t3, hj[2]);
          }
          __syncthreads();
          const int rl = min(k + 3, iend);
          for (int r = 1 + tid; r <= rl; r += NT) {
            double* hr = &HH(r, k);
            const double ss = fma(v3, hr[2 * ldh], fma(v2, hr[ldh], hr[0]));
            hr[0] = fma(-ss, t1, hr[0]);
            hr[ldh] = fma(-ss, t2, hr[ldh]);
            hr[2 * ldh] = fma(-ss, t3, hr[2 * ldh]);
          }
        } else {
          for (int j = k + tid; j <= n; j += NT) {
            double* hj = &HH(k, j);
            const double ss = fma(v2, hj[1], hj[0]);
            hj[0] = fma(-ss, t1, hj[0]);
            hj[1] = fma(-ss, t2, hj[1]);
          }
          __syncthreads();
          for (int r = 1 + tid; r <= iend; r += NT) {
            double* hr = &HH(r, k);
            const double ss = fma(v2, hr[ldh], hr[0]);
            hr[0] = fma(-ss, t1, hr[0]);
            hr[ldh] = fma(-ss, t2, hr[ldh]);
          }
        }
      }
      __syncthreads();
      // apply the sweep's reflectors to the Z rows each thread owns
      if (Zg) {
        for (int r = tid; r < n; r += NT) {
          double* zr = Zg + r;
          double z0 = zr[(long long)(mx - 1) * n], z1 = zr[(long long)mx * n];
          for (int k = mx; k <= iend - 1; ++k) {
            const double* l = lg + 5 * (k - 1);
            if (k <= iend - 2) {
              const double z2 = zr[(long long)(k + 1) * n];
              const double ss = fma(l[4], z2, fma(l[3], z1, z0));
              zr[(long long)(k - 1) * n] = fma(-ss, l[0], z0);
              z0 = fma(-ss, l[1], z1);
              z1 = fma(-ss, l[2], z2);
            } else {
              const double ss = fma(l[3], z1, z0);
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
      if (tid == 0) { wr[iend - 1] = HH(iend, iend); wi[iend - 1] = 0.0; }
    } else if (deflate && istart + 1 == iend) {
      const int p = iend - 1, q = iend;
      if (tid == 0) {
        double a = HH(p, p), bq = HH(p, q), cc = HH(q, p), d = HH(q, q), cs, sn, w1r, w1i, w2r, w2i;
        gs2x2(a, bq, cc, d, cs, sn, w1r, w1i, w2r, w2i);
        wr[q - 1] = w2r; wi[q - 1] = w2i; wr[p - 1] = w1r; wi[p - 1] = w1i;
        c.g[0] = cs; c.g[1] = sn;
        c.v[0] = a; c.v[1] = bq; c.v[2] = cc; c.s[0] = d;
      }
      __syncthreads();
      const double cs = c.g[0], sn = c.g[1];
      for (int j = q + 1 + tid; j <= n; j += NT) {  // lmul!(G, HH[:, istart:n]) beyond the block
        const double a1 = HH(p, j), a2 = HH(q, j);
        HH(p, j) = cs * a1 + sn * a2;
        HH(q, j) = -sn * a1 + cs * a2;
      }
      for (int r = 1 + tid; r <= p - 1; r += NT) {  // rmul!(HH[1:iend, :], G') above the block
        const double a1 = HH(r, p), a2 = HH(r, q);
        HH(r, p) = cs * a1 + sn * a2;
        HH(r, q) = -sn * a1 + cs * a2;
      }
      if (Zg)
        for (int r = tid; r < n; r += NT) {
          double* zp = Zg + r + (long long)(p - 1) * n;
          const double a1 = zp[0], a2 = zp[n];
          zp[0] = cs * a1 + sn * a2;
          zp[n] = -sn * a1 + cs * a2;
        }
      if (tid == 0) {
        HH(p, p) = c.v[0]; HH(p, q) = c.v[1]; HH(q, p) = c.v[2]; HH(q, q) = c.s[0];
        if (iend > 2) HH(iend - 1, iend - 2) = 0.0;
      }
    }
    iend = istart - 1;
    __syncthreads();
  }
  __syncthreads();

  // ---- 5. write back -----------------------------------------------------------
  double mul[8];
  int nf = 0;
  if (scaled) nf = safescale_factors(cscale, amax, mul);
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    double v = (i > j + 1) ? 0.0 : H[i + j * ldh];
    for (int f = 0; f < nf; ++f) v *= mul[f];
    Ag[idx] = v;
  }
  if (scaled)
    for (int i = tid; i < n; i += NT) {
      double a = wr[i], bq = wi[i];
      for (int f = 0; f < nf; ++f) { a *= mul[f]; bq *= mul[f]; }
      wr[i] = a; wi[i] = bq;
    }
  if (tid == 0) bt.status[b] = status;
  __syncthreads();
}
#undef HH

template <int NT>
__global__ void __launch_bounds__(NT) k_schur_real(RealBatch bt, const int* __restrict__ order,
                                                   int* __restrict__ sched, int bin) {
  extern __shared__ double smem[];
  __shared__ Ctl c;
  __shared__ int s_job;
  const int start = sched[3 * bin], end = sched[3 * bin + 1];
  for (;;) {
    if (threadIdx.x == 0) s_job = start + atomicAdd(&sched[3 * bin + 2], 1);
    __syncthreads();
    const int job = s_job;
    __syncthreads();
    if (job >= end) break;
    solve_real<NT>(bt, order[job], smem, c);
  }
}

template <int NT>
cudaError_t launch_bin(const RealBatch& bt, const int* order, int* sched, int bin, int num_sms,
                       cudaStream_t s) {
  const int nmax = bin_max(bin);
  const size_t smem = sizeof(double) * ((size_t)nmax * (nmax | 1) + 6 * nmax + 32);
  cudaError_t e = cudaFuncSetAttribute(k_schur_real<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_schur_real<NT>, NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const int grid = num_sms * per_sm;
  k_schur_real<NT><<<grid, NT, smem, s>>>(bt, order, sched, bin);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_schur_batched_real(const RealBatch& bt, const int* order, int* sched, int num_sms,
                                      cudaStream_t* streams, int nstreams) {
  cudaError_t e;
  // largest bin first: it carries most of the work
  if ((e = launch_bin<128>(bt, order, sched, 3, num_sms, streams[0 % nstreams])) != cudaSuccess) return e;
  if ((e = launch_bin<128>(bt, order, sched, 2, num_sms, streams[1 % nstreams])) != cudaSuccess) return e;
  if ((e = launch_bin<64>(bt, order, sched, 1, num_sms, streams[2 % nstreams])) != cudaSuccess) return e;
  if ((e = launch_bin<32>(bt, order, sched, 0, num_sms, streams[3 % nstreams])) != cudaSuccess) return e;
  return cudaSuccess;
}

}  // namespace gsk
