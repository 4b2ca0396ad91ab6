// Generalized Schur decomposition of real pencils: ggschur!(A::Real, B) (rgeneralized.jl:
// 10-66) with qr!(B), the Hessenberg-triangular reduction _hessenberg! (generalized.jl:
// 84-113) and the real QZ iteration _gqz! (rgeneralized.jl:68-808, LAPACK dhgeqz: single
// real shifts, Francis double shifts, 2 x 2 blocks of complex eigenvalues standardised with
// _gsvd_2x2 / dlasv2 and evaluated with _ggs_2x2 / dlag2).  S = Q^T A Z is quasi-triangular,
// T = Q^T B Z upper triangular with a non-negative diagonal.
//
// One CTA per pencil (a ragged batch or a batch of one), the matrices in global memory
// (L2-resident at the orders this path serves).  Every thread runs the reference's scalar
// control flow on the same data -- shift, Givens and reflector computations, deflation
// tests -- so all threads take the same branches; thread 0 alone writes scalar entries
// (between barriers), and the row / column updates of H, B, Q, Z are split over the CTA.
#include <algorithm>

#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kQrT = 128;

#define HH(i, j) H[((i) - 1) + (size_t)((j) - 1) * n]
#define BB(i, j) B[((i) - 1) + (size_t)((j) - 1) * n]
#define SYNC() __syncthreads()

// Julia's Givens(i1, i2, c, s) on the CTA: lmul! rows (columns j0..j1), rmul!(M, G) and
// rmul!(M, G') columns (rows r0..r1).  Callers synchronise afterwards.
__device__ void crows(double* M, int n, int i1, int i2, double c, double s, int j0, int j1) {
  for (int j = j0 + (int)threadIdx.x; j <= j1; j += kQrT) {
    double* p1 = M + (i1 - 1) + (size_t)(j - 1) * n;
    double* p2 = M + (i2 - 1) + (size_t)(j - 1) * n;
    const double x = *p1, y = *p2;
    *p1 = c * x + s * y;
    *p2 = c * y - s * x;
  }
}
__device__ void ccols(double* M, int n, int i1, int i2, double c, double s, int r0, int r1) {
  double* c1 = M + (size_t)(i1 - 1) * n;
  double* c2 = M + (size_t)(i2 - 1) * n;
  for (int r = r0 - 1 + (int)threadIdx.x; r <= r1 - 1; r += kQrT) {
    const double x = c1[r], y = c2[r];
    c1[r] = x * c - y * s;
    c2[r] = x * s + y * c;
  }
}
__device__ void ccols_adj(double* M, int n, int i1, int i2, double c, double s, int r0, int r1) {
  double* c1 = M + (size_t)(i1 - 1) * n;
  double* c2 = M + (size_t)(i2 - 1) * n;
  for (int r = r0 - 1 + (int)threadIdx.x; r <= r1 - 1; r += kQrT) {
    const double x = c1[r], y = c2[r];
    c1[r] = x * c + y * s;
    c2[r] = y * c - x * s;
  }
}
__device__ void cnegcol(double* M, int n, int col, int r0, int r1) {
  double* p = M + (size_t)(col - 1) * n;
  for (int r = r0 - 1 + (int)threadIdx.x; r <= r1 - 1; r += kQrT) p[r] = -p[r];
}

// Base.hypot(x, y, z): the largest modulus times the norm of the scaled triple.
__device__ __forceinline__ double bhypot3(double x, double y, double z) {
  const double m = fmax(fmax(fabs(x), fabs(y)), fabs(z));
  if (m != m) return (isinf(x) || isinf(y) || isinf(z)) ? __longlong_as_double(0x7ff0000000000000LL) : m;
  if (m == 0.0 || isinf(m)) return m;
  const double a = x / m, b = y / m, c = z / m;
  return m * sqrt(a * a + b * b + c * c);
}

// _reflector! of a 3-vector in registers (householder.jl:12-54), the reference's
// _norm2 semantics for the tail.
__device__ double refl3(double& a, double& x1, double& x2) {
  const double m = fmax(fabs(x1), fabs(x2));
  double xnorm = 0.0;
  if (m > 0.0) {
    if (isfinite(m)) {
      const double p = x1 / m, q = x2 / m;
      xnorm = m * sqrt(p * p + q * q);
    } else {
      xnorm = m;
    }
  }
  if (xnorm == 0.0) return 0.0;
  const double sfmin = 2.0 * Prec<double>::fmin / Prec<double>::eps;
  double alpha = a;
  double beta = -copysign(hypot(alpha, xnorm), alpha);
  int kount = 0;
  if (fabs(beta) < sfmin) {
    const double rs = 1.0 / sfmin;
    bool smallb = true;
    while (smallb) {
      ++kount;
      x1 *= rs;
      x2 *= rs;
      beta *= rs;
      alpha *= rs;
      smallb = fabs(beta) < sfmin && kount < 20;
    }
    const double m2 = fmax(fabs(x1), fabs(x2));
    const double p = x1 / m2, q = x2 / m2;
    xnorm = m2 * sqrt(p * p + q * q);
    beta = -copysign(hypot(alpha, xnorm), alpha);
  }
  const double tau = (beta - alpha) / beta;
  const double t = 1.0 / (alpha - beta);
  x1 *= t;
  x2 *= t;
  for (int k = 0; k < kount; ++k) beta *= sfmin;
  a = beta;
  return tau;
}

// dlag2 (rgeneralized.jl:810-948) on the 2 x 2 pencil at (i, i) of H, B.
__device__ void ggs2x2(const double* H, const double* B, int n, int i, double safmin, double& scale1, double& scale2,
                       double& wr1, double& wr2, double& wi) {
  const double rtmin = sqrt(safmin), rtmax = 1.0 / rtmin, safmax = 1.0 / safmin;
  const double fuzzy1 = 1.0 + sqrt(sqrt(Prec<double>::eps)) / 10.0;
  const double A11 = HH(i, i), A21 = HH(i + 1, i), A12 = HH(i, i + 1), A22 = HH(i + 1, i + 1);
  const double anorm = fmax(fmax(fabs(A11) + fabs(A21), fabs(A12) + fabs(A22)), safmin);
  const double ascale = 1.0 / anorm;
  const double a11 = ascale * A11, a12 = ascale * A12, a21 = ascale * A21, a22 = ascale * A22;
  double b11 = BB(i, i), b12 = BB(i, i + 1), b22 = BB(i + 1, i + 1);
  const double bmin = rtmin * fmax(fmax(fabs(b11), fabs(b12)), fmax(fabs(b22), rtmin));
  if (fabs(b11) < bmin) b11 = b11 < 0.0 ? -bmin : bmin;
  if (fabs(b22) < bmin) b22 = b22 < 0.0 ? -bmin : bmin;
  const double bnorm = fmax(fmax(fabs(b11), fabs(b12) + fabs(b22)), safmin);
  const double bsize = fmax(fabs(b11), fabs(b22));
  const double bscale = 1.0 / bsize;
  b11 *= bscale;
  b12 *= bscale;
  b22 *= bscale;
  const double binv11 = 1.0 / b11, binv22 = 1.0 / b22;
  const double s1 = a11 * binv11, s2 = a22 * binv22;
  double as12, ss, abi22, pp, shift;
  if (fabs(s1) <= fabs(s2)) {
    as12 = a12 - s1 * b12;
    const double as22 = a22 - s1 * b22;
    ss = a21 * (binv11 * binv22);
    abi22 = as22 * binv22 - ss * b12;
    pp = abi22 / 2.0;
    shift = s1;
  } else {
    as12 = a12 - s2 * b12;
    const double as11 = a11 - s2 * b11;
    ss = a21 * (binv11 * binv22);
    abi22 = -ss * b12;
    pp = (as11 * binv11 + abi22) / 2.0;
    shift = s2;
  }
  const double qq = ss * as12;
  double discr, r;
  if (fabs(pp * rtmin) >= 1.0) {
    discr = (rtmin * pp) * (rtmin * pp) + qq * safmin;
    r = sqrt(fabs(discr)) * rtmax;
  } else if (pp * pp + fabs(qq) <= safmin) {
    discr = (rtmax * pp) * (rtmax * pp) + qq * safmax;
    r = sqrt(fabs(discr)) * rtmin;
  } else {
    discr = pp * pp + qq;
    r = sqrt(fabs(discr));
  }
  if (discr >= 0.0 || r == 0.0) {
    const double sm = pp + (pp < 0.0 ? -r : r);
    const double df = pp - (pp < 0.0 ? -r : r);
    const double wbig = shift + sm;
    double wsmall = shift + df;
    if (fabs(wbig) / 2.0 > fmax(fabs(wsmall), safmin)) {
      const double wdet = (a11 * a22 - a12 * a21) * (binv11 * binv22);
      wsmall = wdet / wbig;
    }
    if (pp > abi22) {
      wr1 = fmin(wbig, wsmall);
      wr2 = fmax(wbig, wsmall);
    } else {
      wr2 = fmin(wbig, wsmall);
      wr1 = fmax(wbig, wsmall);
    }
    wi = 0.0;
  } else {
    wr1 = shift + pp;
    wr2 = wr1;
    wi = r;
  }
  const double c1 = bsize * (safmin * fmax(1.0, ascale));
  const double c2 = safmin * fmax(1.0, bnorm);
  const double c3 = bsize * safmin;
  const double c4 = (ascale <= 1.0 && bsize <= 1.0) ? fmin(1.0, (ascale / safmin) * bsize) : 1.0;
  const double c5 = (ascale <= 1.0 || bsize <= 1.0) ? fmin(1.0, ascale * bsize) : 1.0;
  scale1 = 1.0;
  scale2 = 1.0;
  const double wabs = fabs(wr1) + fabs(wi);
  double wsize = fmax(fmax(safmin, c1), fmax(fuzzy1 * (wabs * c2 + c3), fmin(c4, fmax(wabs, c5) / 2.0)));
  if (wsize != 1.0) {
    const double wscale = 1.0 / wsize;
    if (wsize > 1.0) scale1 = (fmax(ascale, bsize) * wscale) * fmin(ascale, bsize);
    else scale1 = (fmin(ascale, bsize) * wscale) * fmax(ascale, bsize);
    wr1 *= wscale;
    if (wi != 0.0) {
      wi *= wscale;
      wr2 = wr1;
      scale2 = scale1;
    }
  } else {
    scale1 = ascale * bsize;
    scale2 = scale1;
  }
  if (wi == 0.0) {
    wsize = fmax(fmax(safmin, c1), fmax(fuzzy1 * (fabs(wr2) * c2 + c3), fmin(c4, fmax(fabs(wr2), c5) / 2.0)));
    if (wsize != 1.0) {
      const double wscale = 1.0 / wsize;
      if (wsize > 1.0) scale2 = (fmax(ascale, bsize) * wscale) * fmin(ascale, bsize);
      else scale2 = (fmin(ascale, bsize) * wscale) * fmax(ascale, bsize);
      wr2 *= wscale;
    } else {
      scale2 = ascale * bsize;
    }
  }
}

// dlasv2 (rgeneralized.jl:950-1038) of [f g; 0 h].
__device__ void gsvd2x2(double f0, double g0, double h0, double& ssmin, double& ssmax, double& snr, double& csr,
                        double& snl, double& csl) {
  double ft = f0, gt = g0, ht = h0, fa = fabs(ft), ha = fabs(ht);
  int pmax = 1;
  const bool swap = ha > fa;
  if (swap) {
    pmax = 3;
    double t = ft; ft = ht; ht = t;
    t = fa; fa = ha; ha = t;
  }
  const double ga = fabs(gt);
  double clt, crt, slt, srt;
  if (ga == 0.0) {
    ssmin = ha; ssmax = fa; clt = 1.0; crt = 1.0; slt = 0.0; srt = 0.0;
  } else {
    bool ga_small = true;
    if (ga > fa) {
      pmax = 2;
      if ((fa / ga) < Prec<double>::eps) {
        ga_small = false;
        ssmax = ga;
        ssmin = (ha > 1.0) ? (fa / (ga / ha)) : ((fa / ha) * ha);
        clt = 1.0;
        slt = ht / gt;
        srt = 1.0;
        crt = ft / gt;
      }
    }
    if (ga_small) {
      const double d = fa - ha;
      double l = (d == fa) ? 1.0 : (d / fa);
      const double m = gt / ft;
      double t = 2.0 - l;
      const double mm = m * m, tt = t * t;
      const double s = sqrt(tt + mm);
      const double r = (l == 0.0) ? fabs(m) : sqrt(l * l + mm);
      const double a = (s + r) / 2.0;
      ssmin = ha / a;
      ssmax = fa * a;
      if (mm == 0.0) {
        if (l == 0.0) t = copysign(2.0, ft) * copysign(1.0, gt);
        else t = gt / copysign(d, ft) + m / t;
      } else {
        t = (m / (s + t) + m / (r + l)) * (1.0 + a);
      }
      l = sqrt(t * t + 4.0);
      crt = 2.0 / l;
      srt = t / l;
      clt = (crt + srt * m) / a;
      slt = (ht / ft) * srt / a;
    }
  }
  if (swap) { csl = srt; snl = crt; csr = slt; snr = clt; }
  else { csl = clt; snl = slt; csr = crt; snr = srt; }
  double tsgn;
  if (pmax == 1) tsgn = copysign(1.0, csr) * copysign(1.0, csl) * copysign(1.0, f0);
  else if (pmax == 2) tsgn = copysign(1.0, snr) * copysign(1.0, csl) * copysign(1.0, g0);
  else tsgn = copysign(1.0, snr) * copysign(1.0, snl) * copysign(1.0, h0);
  ssmax = copysign(ssmax, tsgn);
  ssmin = copysign(ssmin, tsgn * copysign(1.0, f0) * copysign(1.0, h0));
}

// 2-norm of all n x n entries (Frobenius) without overflow.
__device__ double cta_fro_real(const double* M, int n, double* red) {
  return cta_norm2<double, kQrT>(M, n * n, red);
}

// _gqz! (rgeneralized.jl:68-808), ilo = 1, ihi = n, wantSchur; returns 0 or 1.
__device__ int gqz_real(double* H, double* B, double* Q, double* Z, int n, double2* alpha, double* beta,
                        long long maxiter, double* red) {
  const int tid = threadIdx.x;
  const int ilo = 1;
  const double ulp = Prec<double>::eps, safmin = Prec<double>::fmin, safmax = 1.0 / safmin, safety = 100.0;
  const double anorm = cta_fro_real(H, n, red), bnorm = cta_fro_real(B, n, red);
  const double atol = fmax(safmin, ulp * anorm), btol = fmax(safmin, ulp * bnorm);
  const double ascale = 1.0 / fmax(safmin, anorm), bscale = 1.0 / fmax(safmin, bnorm);
  int ifirst = ilo, ilast = n;
  const int ifirstm = 1, ilastm = n;
  int shiftcount = 0;
  double eshift = 0.0;
  enum { UNKNOWN, NONE, NORMAL, INF };
  for (long long it = 1; it <= maxiter; ++it) {
    SYNC();
    int br = UNKNOWN;
    if (ilast == ilo) {
      br = NORMAL;
    } else if (fabs(HH(ilast, ilast - 1)) < fmax(safmin, ulp * (fabs(HH(ilast, ilast)) + fabs(HH(ilast - 1, ilast - 1))))) {
      SYNC();
      if (tid == 0) HH(ilast, ilast - 1) = 0.0;
      SYNC();
      br = NORMAL;
    }
    if (br == UNKNOWN) {
      if (fabs(BB(ilast, ilast)) <= btol) {
        SYNC();
        if (tid == 0) BB(ilast, ilast) = 0.0;
        SYNC();
        br = INF;
      } else {
        for (int j = ilast - 1; j >= ilo; --j) {
          bool h0 = false;
          if (j == ilo) {
            h0 = true;
          } else if (fabs(HH(j, j - 1)) <= atol) {
            SYNC();
            if (tid == 0) HH(j, j - 1) = 0.0;
            SYNC();
            h0 = true;
          }
          if (fabs(BB(j, j)) < btol) {
            SYNC();
            if (tid == 0) BB(j, j) = 0.0;
            SYNC();
            bool have2 = false;
            if (!h0) {
              double t = fabs(HH(j, j - 1)), t2 = fabs(HH(j, j));
              const double tr = fmax(t, t2);
              if (tr < 1.0 && tr != 0.0) { t = t / tr; t2 = t2 / tr; }
              have2 = (t * (ascale * fabs(HH(j + 1, j))) <= t2 * (ascale * atol));
            }
            if (h0 || have2) {
              for (int jch = j; jch <= ilast - 1; ++jch) {
                double c, s, r;
                givens_alg(HH(jch, jch), HH(jch + 1, jch), c, s, r);
                SYNC();
                if (tid == 0) { HH(jch, jch) = r; HH(jch + 1, jch) = 0.0; }
                crows(H, n, jch, jch + 1, c, s, jch + 1, ilastm);
                crows(B, n, jch, jch + 1, c, s, jch + 1, ilastm);
                if (Q) ccols_adj(Q, n, jch, jch + 1, c, s, 1, n);
                SYNC();
                if (have2) {
                  if (tid == 0) HH(jch, jch - 1) *= c;
                  SYNC();
                }
                have2 = false;
                if (fabs(BB(jch + 1, jch + 1)) > btol) {
                  if (jch + 1 >= ilast) br = NORMAL;
                  else { ifirst = jch + 1; br = NONE; }
                  break;
                }
                SYNC();
                if (tid == 0) BB(jch + 1, jch + 1) = 0.0;
                SYNC();
              }
              if (br == UNKNOWN) br = INF;
              break;
            } else {
              for (int jch = j; jch <= ilast - 1; ++jch) {
                double c, s, r;
                givens_alg(BB(jch, jch + 1), BB(jch + 1, jch + 1), c, s, r);
                SYNC();
                if (tid == 0) { BB(jch, jch + 1) = r; BB(jch + 1, jch + 1) = 0.0; }
                if (jch < ilastm - 1) crows(B, n, jch, jch + 1, c, s, jch + 2, ilastm);
                crows(H, n, jch, jch + 1, c, s, jch - 1, ilastm);
                if (Q) ccols_adj(Q, n, jch, jch + 1, c, s, 1, n);
                SYNC();
                givens_alg(HH(jch + 1, jch), HH(jch + 1, jch - 1), c, s, r);
                SYNC();
                if (tid == 0) { HH(jch + 1, jch) = r; HH(jch + 1, jch - 1) = 0.0; }
                SYNC();
                ccols_adj(H, n, jch, jch - 1, c, s, ifirstm, jch);
                ccols_adj(B, n, jch, jch - 1, c, s, ifirstm, jch - 1);
                if (Z) ccols_adj(Z, n, jch, jch - 1, c, s, 1, n);
                SYNC();
              }
              br = INF;
              break;
            }
          } else if (h0) {
            ifirst = j;
            br = NONE;
            break;
          }
        }
      }
      if (br == INF) {
        double c, s, r;
        givens_alg(HH(ilast, ilast), HH(ilast, ilast - 1), c, s, r);
        SYNC();
        if (tid == 0) { HH(ilast, ilast) = r; HH(ilast, ilast - 1) = 0.0; }
        SYNC();
        ccols_adj(H, n, ilast, ilast - 1, c, s, ifirstm, ilast - 1);
        ccols_adj(B, n, ilast, ilast - 1, c, s, ifirstm, ilast - 1);
        if (Z) ccols_adj(Z, n, ilast, ilast - 1, c, s, 1, n);
        SYNC();
        br = NORMAL;
      }
    }
    if (br == NORMAL) {
      if (BB(ilast, ilast) < 0.0) {
        SYNC();
        cnegcol(H, n, ilast, ifirstm, ilast);
        cnegcol(B, n, ilast, ifirstm, ilast);
        if (Z) cnegcol(Z, n, ilast, 1, n);
        SYNC();
      }
      if (tid == 0) {
        alpha[ilast - 1] = make_double2(HH(ilast, ilast), 0.0);
        beta[ilast - 1] = BB(ilast, ilast);
      }
      ilast -= 1;
      if (ilast < ilo) break;
      shiftcount = 0;
      eshift = 0.0;
      continue;
    }
    // ---- QZ step on ifirst..ilast
    ++shiftcount;
    double s1, s2, wr, wr2, wi;
    if (shiftcount % 10 != 0) {
      ggs2x2(H, B, n, ilast - 1, safmin * safety, s1, s2, wr, wr2, wi);
      if (fabs((wr / s1) * BB(ilast, ilast) - HH(ilast, ilast)) > fabs((wr2 / s2) * BB(ilast, ilast) - HH(ilast, ilast))) {
        double t = wr; wr = wr2; wr2 = t;
        t = s1; s1 = s2; s2 = t;
      }
    } else {
      if ((double)maxiter * safmin * fabs(HH(ilast, ilast - 1)) < fabs(BB(ilast - 1, ilast - 1)))
        eshift = HH(ilast, ilast - 1) / BB(ilast - 1, ilast - 1);
      else
        eshift += 1.0 / (safmin * (double)maxiter);
      s1 = 1.0;
      wr = eshift;
      wi = 0.0;
    }
    if (wi == 0.0) {
      // single real shift
      double t = fmin(ascale, 1.0) * (safmax / 2.0);
      double scale = s1 > t ? t / s1 : 1.0;
      t = fmin(bscale, 1.0) * (safmax / 2.0);
      if (fabs(wr) > t) scale = fmin(scale, t / fabs(wr));
      s1 *= scale;
      wr *= scale;
      int istart = -1;
      bool gotit = false;
      for (int j = ilast - 1; j >= ifirst + 1; --j) {
        istart = j;
        double t1 = fabs(s1 * HH(j, j - 1));
        double t2 = fabs(s1 * HH(j, j) - wr * BB(j, j));
        const double tr = fmax(t1, t2);
        if (tr < 1.0 && tr != 0.0) { t1 /= tr; t2 /= tr; }
        if (fabs((ascale * HH(j + 1, j)) * t1) <= ascale * atol * t2) { gotit = true; break; }
      }
      if (!gotit) istart = ifirst;
      const double f1 = s1 * HH(istart, istart) - wr * BB(istart, istart);
      const double g2 = s1 * HH(istart + 1, istart);
      double c, s, t3;
      givens_alg(f1, g2, c, s, t3);
      for (int j = istart; j <= ilast - 1; ++j) {
        if (j > istart) {
          double r;
          givens_alg(HH(j, j - 1), HH(j + 1, j - 1), c, s, r);
          SYNC();
          if (tid == 0) { HH(j, j - 1) = r; HH(j + 1, j - 1) = 0.0; }
        }
        SYNC();
        crows(H, n, j, j + 1, c, s, j, ilastm);
        crows(B, n, j, j + 1, c, s, j, ilastm);
        if (Q) ccols_adj(Q, n, j, j + 1, c, s, 1, n);
        SYNC();
        double r;
        givens_alg(BB(j + 1, j + 1), BB(j + 1, j), c, s, r);
        SYNC();
        if (tid == 0) { BB(j + 1, j + 1) = r; BB(j + 1, j) = 0.0; }
        SYNC();
        ccols(H, n, j, j + 1, c, s, ifirstm, min(j + 2, ilast));
        ccols(B, n, j, j + 1, c, s, ifirstm, j);
        if (Z) ccols(Z, n, j, j + 1, c, s, 1, n);
        SYNC();
      }
    } else if (ilast == ifirst + 1) {
      // 2 x 2 block with complex eigenvalues: diagonalise the B block, then alpha, beta
      double b22, b11, sr, cr, sl, cl;
      gsvd2x2(BB(ifirst, ifirst), BB(ifirst, ilast), BB(ilast, ilast), b22, b11, sr, cr, sl, cl);
      if (b11 < 0.0) { cr = -cr; sr = -sr; b11 = -b11; b22 = -b22; }
      SYNC();
      crows(H, n, ifirst, ilast, cl, sl, ifirst, ilastm);
      SYNC();
      ccols_adj(H, n, ifirst, ilast, cr, sr, ifirstm, ilast);
      if (ilast < ilastm) crows(B, n, ifirst, ilast, cl, sl, ilast + 1, ilastm);
      if (ifirstm < ifirst) ccols_adj(B, n, ifirst, ilast, cr, sr, ifirstm, ifirst - 1);
      if (Q) ccols_adj(Q, n, ifirst, ilast, cl, sl, 1, n);
      if (Z) ccols_adj(Z, n, ifirst, ilast, cr, sr, 1, n);
      SYNC();
      if (tid == 0) {
        BB(ilast - 1, ilast - 1) = b11;
        BB(ilast - 1, ilast) = 0.0;
        BB(ilast, ilast - 1) = 0.0;
        BB(ilast, ilast) = b22;
      }
      SYNC();
      if (b22 < 0.0) {
        cnegcol(H, n, ilast, ifirstm, ilast);
        cnegcol(B, n, ilast, ifirstm, ilast);
        if (Z) cnegcol(Z, n, ilast, 1, n);
        SYNC();
        b22 = -b22;
      }
      double d2, d3;
      ggs2x2(H, B, n, ilast - 1, safmin * safety, s1, d2, wr, d3, wi);
      if (wi == 0.0) continue;  // back to a single shift
      const double s1inv = 1.0 / s1;
      const double a11 = HH(ilast - 1, ilast - 1), a21 = HH(ilast, ilast - 1), a12 = HH(ilast - 1, ilast),
                   a22 = HH(ilast, ilast);
      const double c11r = s1 * a11 - wr * b11, c11i = -wi * b11, c12 = s1 * a12, c21 = s1 * a21;
      const double c22r = s1 * a22 - wr * b22, c22i = -wi * b22;
      double cz, szr, szi;
      if (fabs(c11r) + fabs(c11i) + fabs(c12) > fabs(c21) + fabs(c22r) + fabs(c22i)) {
        const double t1 = bhypot3(c12, c11r, c11i);
        cz = c12 / t1;
        szr = -c11r / t1;
        szi = -c11i / t1;
      } else {
        cz = hypot(c22r, c22i);
        if (cz <= safmin) { cz = 0.0; szr = 1.0; szi = 0.0; }
        else {
          const double tr = c22r / cz, ti = c22i / cz;
          const double t1 = hypot(cz, c21);
          cz /= t1;
          szr = -c21 * tr / t1;
          szi = c21 * ti / t1;
        }
      }
      const double an = fabs(a11) + fabs(a12) + fabs(a21) + fabs(a22);
      const double bn = fabs(b11) + fabs(b22);
      const double wabs = fabs(wr) + fabs(wi);
      double cq, sqr, sqi;
      if (s1 * an > wabs * bn) {
        cq = cz * b11;
        sqr = szr * b22;
        sqi = -szi * b22;
      } else {
        const double a1r = cz * a11 + szr * a12, a1i = szi * a12;
        const double a2r = cz * a21 + szr * a22, a2i = szi * a22;
        cq = hypot(a1r, a1i);
        if (cq <= safmin) { cq = 0.0; sqr = 1.0; sqi = 0.0; }
        else {
          const double tr = a1r / cq, ti = a1i / cq;
          sqr = tr * a2r + ti * a2i;
          sqi = ti * a2r - tr * a2i;
        }
      }
      const double t1 = bhypot3(cq, sqr, sqi);
      cq /= t1;
      sqr /= t1;
      sqi /= t1;
      const double tr = sqr * szr - sqi * szi, ti = sqr * szi + sqi * szr;
      const double b1r = cq * cz * b11 + tr * b22, b1i = ti * b22;
      const double b1a = hypot(b1r, b1i);
      const double b2r = cq * cz * b22 + tr * b11, b2i = -ti * b11;
      const double b2a = hypot(b2r, b2i);
      if (tid == 0) {
        beta[ilast - 2] = b1a;
        beta[ilast - 1] = b2a;
        alpha[ilast - 2] = make_double2((wr * b1a) * s1inv, (wi * b1a) * s1inv);
        alpha[ilast - 1] = make_double2((wr * b2a) * s1inv, (-wi * b2a) * s1inv);
      }
      ilast = ifirst - 1;
      if (ilast < ilo) break;
      shiftcount = 0;
      eshift = 0.0;
    } else {
      // Francis implicit double shift (block of order >= 3)
      const double ad11 = (ascale * HH(ilast - 1, ilast - 1)) / (bscale * BB(ilast - 1, ilast - 1));
      const double ad21 = (ascale * HH(ilast, ilast - 1)) / (bscale * BB(ilast - 1, ilast - 1));
      const double ad12 = (ascale * HH(ilast - 1, ilast)) / (bscale * BB(ilast, ilast));
      const double ad22 = (ascale * HH(ilast, ilast)) / (bscale * BB(ilast, ilast));
      const double u12 = BB(ilast - 1, ilast) / BB(ilast, ilast);
      const double ad11l = (ascale * HH(ifirst, ifirst)) / (bscale * BB(ifirst, ifirst));
      const double ad21l = (ascale * HH(ifirst + 1, ifirst)) / (bscale * BB(ifirst, ifirst));
      const double ad12l = (ascale * HH(ifirst, ifirst + 1)) / (bscale * BB(ifirst + 1, ifirst + 1));
      const double ad22l = (ascale * HH(ifirst + 1, ifirst + 1)) / (bscale * BB(ifirst + 1, ifirst + 1));
      const double ad32l = (ascale * HH(ifirst + 2, ifirst + 1)) / (bscale * BB(ifirst + 1, ifirst + 1));
      const double u12l = BB(ifirst, ifirst + 1) / BB(ifirst + 1, ifirst + 1);
      double v0 = ((ad11 - ad11l) * (ad22 - ad11l) - ad12 * ad21 + ad21 * u12 * ad11l + (ad12l - ad11l * u12l) * ad21l);
      double v1 = (((ad22l - ad11l) - ad21l * u12l - (ad11 - ad11l) - (ad22 - ad11l) + ad21 * u12)) * ad21l;
      double v2 = ad32l * ad21l;
      const int istart = ifirst;
      double tau = refl3(v0, v1, v2);
      for (int j = istart; j <= ilast - 2; ++j) {
        if (j > istart) {
          v0 = HH(j, j - 1);
          v1 = HH(j + 1, j - 1);
          v2 = HH(j + 2, j - 1);
          tau = refl3(v0, v1, v2);
          SYNC();
          if (tid == 0) { HH(j, j - 1) = v0; HH(j + 1, j - 1) = 0.0; HH(j + 2, j - 1) = 0.0; }
        }
        SYNC();
        {
          const double t2 = tau * v1, t3 = tau * v2;
          for (int jc = j + tid; jc <= ilastm; jc += kQrT) {
            double t1 = HH(j, jc) + v1 * HH(j + 1, jc) + v2 * HH(j + 2, jc);
            HH(j, jc) -= t1 * tau;
            HH(j + 1, jc) -= t1 * t2;
            HH(j + 2, jc) -= t1 * t3;
            t1 = BB(j, jc) + v1 * BB(j + 1, jc) + v2 * BB(j + 2, jc);
            BB(j, jc) -= t1 * tau;
            BB(j + 1, jc) -= t1 * t2;
            BB(j + 2, jc) -= t1 * t3;
          }
          if (Q)
            for (int jr = 1 + tid; jr <= n; jr += kQrT) {
              double* qr = Q + (jr - 1);
              const double t1 = qr[(size_t)(j - 1) * n] + v1 * qr[(size_t)j * n] + v2 * qr[(size_t)(j + 1) * n];
              qr[(size_t)(j - 1) * n] -= t1 * tau;
              qr[(size_t)j * n] -= t1 * t2;
              qr[(size_t)(j + 1) * n] -= t1 * t3;
            }
        }
        SYNC();
        // zero the j-th column of B: 2 x 2 solve with pivoting
        bool pivot = false;
        double scale, u1, u2;
        {
          double t1 = fmax(fabs(BB(j + 1, j + 1)), fabs(BB(j + 1, j + 2)));
          const double tt2 = fmax(fabs(BB(j + 2, j + 1)), fabs(BB(j + 2, j + 2)));
          if (fmax(t1, tt2) < safmin) {
            scale = 0.0; u1 = 1.0; u2 = 0.0;
          } else {
            double w11, w21, w12, w22;
            if (t1 >= tt2) {
              w11 = BB(j + 1, j + 1); w21 = BB(j + 2, j + 1); w12 = BB(j + 1, j + 2); w22 = BB(j + 2, j + 2);
              u1 = BB(j + 1, j); u2 = BB(j + 2, j);
            } else {
              w21 = BB(j + 1, j + 1); w11 = BB(j + 2, j + 1); w22 = BB(j + 1, j + 2); w12 = BB(j + 2, j + 2);
              u2 = BB(j + 1, j); u1 = BB(j + 2, j);
            }
            if (fabs(w12) > fabs(w11)) {
              pivot = true;
              double t = w11; w11 = w12; w12 = t;
              t = w21; w21 = w22; w22 = t;
            }
            t1 = w21 / w11;
            u2 -= t1 * u1;
            w22 -= t1 * w12;
            scale = 1.0;
            if (fabs(w22) < safmin) {
              scale = 0.0;
            } else {
              if (fabs(w22) < fabs(u2)) scale = fabs(w22 / u2);
              if (fabs(w11) < fabs(u1)) scale = fmin(scale, fabs(w11 / u1));
              u2 = (scale * u2) / w22;
              u1 = (scale * u1 - w12 * u2) / w11;
            }
          }
        }
        if (pivot) { const double t = u1; u1 = u2; u2 = t; }
        {
          const double t1 = bhypot3(scale, u1, u2);
          tau = 1.0 + scale / t1;
          const double vs = -1.0 / (scale + t1);
          v1 = vs * u1;
          v2 = vs * u2;
        }
        {
          const double t2 = tau * v1, t3 = tau * v2;
          const int rh = min(j + 3, ilast);
          for (int jr = ifirstm + tid; jr <= rh; jr += kQrT) {
            const double t1 = HH(jr, j) + v1 * HH(jr, j + 1) + v2 * HH(jr, j + 2);
            HH(jr, j) -= t1 * tau;
            HH(jr, j + 1) -= t2 * t1;
            HH(jr, j + 2) -= t3 * t1;
          }
          for (int jr = ifirstm + tid; jr <= j + 2; jr += kQrT) {
            const double t1 = BB(jr, j) + v1 * BB(jr, j + 1) + v2 * BB(jr, j + 2);
            BB(jr, j) -= t1 * tau;
            BB(jr, j + 1) -= t2 * t1;
            BB(jr, j + 2) -= t3 * t1;
          }
          if (Z)
            for (int jr = 1 + tid; jr <= n; jr += kQrT) {
              double* zr = Z + (jr - 1);
              const double t1 = zr[(size_t)(j - 1) * n] + v1 * zr[(size_t)j * n] + v2 * zr[(size_t)(j + 1) * n];
              zr[(size_t)(j - 1) * n] -= t1 * tau;
              zr[(size_t)j * n] -= t2 * t1;
              zr[(size_t)(j + 1) * n] -= t3 * t1;
            }
        }
        SYNC();
        if (tid == 0) { BB(j + 1, j) = 0.0; BB(j + 2, j) = 0.0; }
        SYNC();
      }
      // the last two rotations
      const int j = ilast - 1;
      double c, s, r;
      givens_alg(HH(j, j - 1), HH(j + 1, j - 1), c, s, r);
      SYNC();
      if (tid == 0) { HH(j, j - 1) = r; HH(j + 1, j - 1) = 0.0; }
      crows(H, n, j, j + 1, c, s, j, ilastm);
      crows(B, n, j, j + 1, c, s, j, ilastm);
      if (Q) ccols_adj(Q, n, j, j + 1, c, s, 1, n);
      SYNC();
      givens_alg(BB(j + 1, j + 1), BB(j + 1, j), c, s, r);
      SYNC();
      if (tid == 0) { BB(j + 1, j + 1) = r; BB(j + 1, j) = 0.0; }
      SYNC();
      ccols_adj(H, n, j + 1, j, c, s, ifirstm, ilast);
      ccols_adj(B, n, j + 1, j, c, s, ifirstm, ilast - 1);
      if (Z) ccols_adj(Z, n, j + 1, j, c, s, 1, n);
      SYNC();
    }
    if (it >= maxiter) return 1;
  }
  return 0;
}

// Largest |a_ij|, NaN-propagating.
__device__ double cta_maxabs_real(const double* M, int n, double* red) {
  double v = 0.0;
  for (size_t e = threadIdx.x; e < (size_t)n * n; e += kQrT) {
    const double a = fabs(M[e]);
    if (a > v || a != a) v = a;
  }
  return block_max<kQrT>(v, red);
}

__device__ void cta_safescale_real(double* M, size_t len, double cfrom, double cto) {
  double mul[8];
  const int k = safescale_factors(cfrom, cto, mul);
  for (size_t e = threadIdx.x; e < len; e += kQrT) {
    double v = M[e];
    for (int q = 0; q < k; ++q) v *= mul[q];
    M[e] = v;
  }
  __syncthreads();
}

// _scale! (util.jl:14-29)
__device__ bool cta_scale_real(double* M, int n, double* red, double& cscale, double& anrm) {
  const double smlnum = sqrt(Prec<double>::fmin) / Prec<double>::eps, bignum = 1.0 / smlnum;
  anrm = cta_maxabs_real(M, n, red);
  cscale = 1.0;
  bool sc = false;
  if (anrm > 0.0 && anrm < smlnum) { sc = true; cscale = smlnum; }
  else if (anrm > bignum) { sc = true; cscale = bignum; }
  if (sc) cta_safescale_real(M, (size_t)n * n, anrm, cscale);
  return sc;
}

__global__ void __launch_bounds__(kQrT) k_ggschur_real(QzrBatch bt) {
  __shared__ double red[kQrT / 32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int b = blockIdx.x; b < bt.count; b += gridDim.x) {
    const int n = bt.ns ? bt.ns[b] : bt.n1;
    const long long off = bt.ns ? bt.offs[b] : 0, woff = bt.ns ? bt.woffs[b] : 0;
    double* A = bt.A + off;
    double* B = bt.B + off;
    double* Q = bt.Q ? bt.Q + off : nullptr;
    double* Z = bt.Z ? bt.Z + off : nullptr;
    double2* alpha = bt.alpha + woff;
    double* beta = bt.beta + woff;
    if (n == 0) {
      if (tid == 0 && bt.status) bt.status[b] = 0;
      continue;
    }
    double cscale = 1.0, anrm = 1.0, cscaleb = 1.0, bnrm = 1.0;
    bool scA = false, scB = false;
    if (bt.scale) {
      scA = cta_scale_real(A, n, red, cscale, anrm);
      scB = cta_scale_real(B, n, red, cscaleb, bnrm);
    }
    // qr!(B), A <- Q^T A; tau in beta (scratch until the iteration)
    for (int j = 1; j <= n; ++j) {
      const int len = n - j + 1;
      double* v = B + (j - 1) + (size_t)(j - 1) * n;
      const double t = cta_reflector<kQrT>(v, len, red);
      if (tid == 0) beta[j - 1] = t;
      __syncthreads();
      if (t != 0.0) {
        for (int col = wid; col < (n - j) + n; col += kQrT / 32) {
          double* x = col < n - j ? B + (j - 1) + (size_t)(j + col) * n : A + (j - 1) + (size_t)(col - (n - j)) * n;
          double sacc = 0.0;
          for (int r = lane; r < len; r += 32) sacc = fma(r == 0 ? 1.0 : v[r], x[r], sacc);
          for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
          const double ts = t * sacc;
          for (int r = lane; r < len; r += 32) x[r] = fma(-ts, r == 0 ? 1.0 : v[r], x[r]);
        }
      }
      __syncthreads();
    }
    if (Q) {
      for (size_t e = tid; e < (size_t)n * n; e += kQrT) Q[e] = ((e % n) == (e / n)) ? 1.0 : 0.0;
      __syncthreads();
      for (int j = n; j >= 1; --j) {
        const double t = beta[j - 1];
        const int len = n - j + 1;
        const double* v = B + (j - 1) + (size_t)(j - 1) * n;
        if (t != 0.0) {
          for (int col = j + wid; col <= n; col += kQrT / 32) {
            double* x = Q + (j - 1) + (size_t)(col - 1) * n;
            double sacc = 0.0;
            for (int r = lane; r < len; r += 32) sacc = fma(r == 0 ? 1.0 : v[r], x[r], sacc);
            for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
            const double ts = t * sacc;
            for (int r = lane; r < len; r += 32) x[r] = fma(-ts, r == 0 ? 1.0 : v[r], x[r]);
          }
        }
        __syncthreads();
      }
    }
    for (size_t e = tid; e < (size_t)n * n; e += kQrT) {
      if ((e % n) > (e / n)) B[e] = 0.0;
      if (Z) Z[e] = ((e % n) == (e / n)) ? 1.0 : 0.0;
    }
    __syncthreads();
    // _hessenberg!(A, B, Q, Z) (generalized.jl:84-113)
    for (int jc = 1; jc <= n - 2; ++jc)
      for (int jr = n; jr >= jc + 2; --jr) {
        double c, s, r;
        {
          const double* H = A;
          givens_alg(HH(jr - 1, jc), HH(jr, jc), c, s, r);
        }
        __syncthreads();
        crows(A, n, jr - 1, jr, c, s, 1, n);
        crows(B, n, jr - 1, jr, c, s, 1, n);
        if (Q) ccols_adj(Q, n, jr - 1, jr, c, s, 1, n);
        __syncthreads();
        givens_alg(BB(jr, jr), BB(jr, jr - 1), c, s, r);
        __syncthreads();
        ccols_adj(A, n, jr, jr - 1, c, s, 1, n);
        ccols_adj(B, n, jr, jr - 1, c, s, 1, n);
        if (Z) ccols_adj(Z, n, jr, jr - 1, c, s, 1, n);
        __syncthreads();
      }
    for (size_t e = tid; e < (size_t)n * n; e += kQrT) {
      const int i = (int)(e % n), j = (int)(e / n);
      if (i > j + 1) A[e] = 0.0;
      if (i > j) B[e] = 0.0;
    }
    __syncthreads();
    const int st = gqz_real(A, B, Q, Z, n, alpha, beta, 100LL * n, red);
    __syncthreads();
    if (scA) {
      cta_safescale_real(A, (size_t)n * n, cscale, anrm);
      cta_safescale_real(reinterpret_cast<double*>(alpha), 2 * (size_t)n, cscale, anrm);
    }
    if (scB) {
      cta_safescale_real(B, (size_t)n * n, cscaleb, bnrm);
      cta_safescale_real(beta, (size_t)n, cscaleb, bnrm);
    }
    if (tid == 0 && bt.status) bt.status[b] = st;
    __syncthreads();
  }
}

#undef HH
#undef BB
#undef SYNC

// ---- reordering of real generalized Schur forms (rordschur.jl:542-1178) -----------------
// gordschur!(S, T, Q, Z, select) for a real pair in one CTA.  Thread 0 plans each swap of
// adjacent blocks on copies of the (at most 4 x 4) diagonal blocks -- the Kronecker form
// of the generalized Sylvester equation by _safe_lu_solve!, the QR and RQ factorizations
// (LAPACK's reflector convention), the weak and strong stability tests and the
// standardization of the new 2 x 2 blocks (_gqz_2x2!) -- and the CTA applies the accepted
// transformation to the rest of S, T and to Q, Z.  Kept from the reference: `nbold == 3`
// in _trexchange! (a block that splits stays nbold = 2), t2 from A in _gqz_2x2!, and its
// singular-B1 branch rotating columns.

// _safe_lu_solve! (util.jl:603-690) of a real nn x nn system (nn <= 8), in place on b
__device__ double safe_lu_real(int nn, double* a, double* b) {
#define LA(i, j) a[((i) - 1) + ((j) - 1) * nn]
  const double eps = Prec<double>::eps, smallnum = Prec<double>::fmin / eps;
  double smin = 0.0;
  for (int e = 0; e < nn * nn; ++e) smin = fmax(smin, fabs(a[e]));
  smin = fmax(eps * smin, smallnum);
  int jpiv[8];
  for (int i = 1; i <= nn - 1; ++i) {
    double xmax = 0.0;
    int ipsv = i, jpsv = i;
    for (int ip = i; ip <= nn; ++ip)
      for (int jp = i; jp <= nn; ++jp)
        if (fabs(LA(ip, jp)) >= xmax) { xmax = fabs(LA(ip, jp)); ipsv = ip; jpsv = jp; }
    if (ipsv != i) {
      for (int j = 1; j <= nn; ++j) { const double t = LA(ipsv, j); LA(ipsv, j) = LA(i, j); LA(i, j) = t; }
      const double t = b[i - 1]; b[i - 1] = b[ipsv - 1]; b[ipsv - 1] = t;
    }
    if (jpsv != i)
      for (int j = 1; j <= nn; ++j) { const double t = LA(j, jpsv); LA(j, jpsv) = LA(j, i); LA(j, i) = t; }
    jpiv[i - 1] = jpsv;
    if (fabs(LA(i, i)) < smin) LA(i, i) = smin;
    for (int j = i + 1; j <= nn; ++j) {
      LA(j, i) = LA(j, i) / LA(i, i);
      b[j - 1] -= LA(j, i) * b[i - 1];
      for (int k = i + 1; k <= nn; ++k) LA(j, k) -= LA(j, i) * LA(i, k);
    }
  }
  if (fabs(LA(nn, nn)) < smin) LA(nn, nn) = smin;
  jpiv[nn - 1] = nn;
  double scale = 1.0;
  const double aa = 8.0 * smallnum;
  bool needscl = false;
  for (int i = 1; i <= nn; ++i)
    if (aa * fabs(b[i - 1]) > fabs(LA(i, i))) { needscl = true; break; }
  if (needscl) {
    double bmax = 0.0;
    for (int i = 0; i < nn; ++i) bmax = fmax(bmax, fabs(b[i]));
    scale = (1.0 / 8.0) / bmax;
    for (int i = 0; i < nn; ++i) b[i] *= scale;
  }
  for (int i = 1; i <= nn; ++i) {
    const int k = nn + 1 - i;
    const double t = 1.0 / LA(k, k);
    b[k - 1] *= t;
    for (int j = k + 1; j <= nn; ++j) b[k - 1] -= (t * LA(k, j)) * b[j - 1];
  }
  for (int i = 1; i <= nn - 1; ++i) {
    const int jj = jpiv[nn - i - 1];
    if (jj != nn - i) { const double t = b[nn - i - 1]; b[nn - i - 1] = b[jj - 1]; b[jj - 1] = t; }
  }
  return scale;
#undef LA
}

// _safe_fnorm of a rows x cols block (columns in order, scale starting at 1)
__device__ double safe_fnorm_blk(const double* m, int ld, int rows, int cols) {
  double scale = 1.0, sumsq = 0.0;
  for (int j = 0; j < cols; ++j)
    for (int i = 0; i < rows; ++i) {
      const double t1 = fabs(m[i + j * ld]);
      if (t1 > 0.0 || t1 != t1) {
        if (scale < t1) { sumsq = 1.0 + sumsq * (scale / t1) * (scale / t1); scale = t1; }
        else sumsq += (t1 / scale) * (t1 / scale);
      }
    }
  return scale * sqrt(sumsq);
}

// dlarfg on alpha and x (n - 1 entries, stride inc); returns tau
__device__ double larfg_d(int n, double* alpha, double* x, int inc) {
  if (n <= 1) return 0.0;
  auto nrm2 = [&]() {
    double sc = 0.0, sq = 1.0;
    for (int i = 0; i < n - 1; ++i) {
      const double a = fabs(x[i * inc]);
      if (a > 0.0) {
        if (sc < a) { sq = 1.0 + sq * (sc / a) * (sc / a); sc = a; }
        else sq += (a / sc) * (a / sc);
      }
    }
    return sc * sqrt(sq);
  };
  double xnorm = nrm2();
  if (xnorm == 0.0) return 0.0;
  double beta = -copysign(hypot(*alpha, xnorm), *alpha);
  const double sfmin = Prec<double>::fmin / Prec<double>::eps;
  int knt = 0;
  if (fabs(beta) < sfmin) {
    const double rsfmn = 1.0 / sfmin;
    do {
      ++knt;
      for (int i = 0; i < n - 1; ++i) x[i * inc] *= rsfmn;
      beta *= rsfmn;
      *alpha *= rsfmn;
    } while (fabs(beta) < sfmin && knt < 20);
    xnorm = nrm2();
    beta = -copysign(hypot(*alpha, xnorm), *alpha);
  }
  const double tau = (beta - *alpha) / beta;
  const double sc = 1.0 / (*alpha - beta);
  for (int i = 0; i < n - 1; ++i) x[i * inc] *= sc;
  for (int j = 0; j < knt; ++j) beta *= sfmin;
  *alpha = beta;
  return tau;
}

// QR of a (m x k, ld m): R in the upper triangle, the full Q (m x m) in q
__device__ void house_qr_d(int m, int k, double* a, double* q) {
#define A_(i, j) a[((i) - 1) + ((j) - 1) * m]
  double tau[4];
  for (int i = 1; i <= k; ++i) {
    tau[i - 1] = larfg_d(m - i + 1, &A_(i, i), i < m ? &A_(i + 1, i) : &A_(i, i), 1);
    if (i < k && tau[i - 1] != 0.0) {
      const double aii = A_(i, i);
      A_(i, i) = 1.0;
      for (int j = i + 1; j <= k; ++j) {
        double t = 0.0;
        for (int r = i; r <= m; ++r) t += A_(r, i) * A_(r, j);
        for (int r = i; r <= m; ++r) A_(r, j) -= tau[i - 1] * A_(r, i) * t;
      }
      A_(i, i) = aii;
    }
  }
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) q[i + j * m] = i == j ? 1.0 : 0.0;
  for (int i = k; i >= 1; --i) {
    if (tau[i - 1] == 0.0) continue;
    for (int j = 1; j <= m; ++j) {
      double t = q[(i - 1) + (j - 1) * m];
      for (int r = i + 1; r <= m; ++r) t += A_(r, i) * q[(r - 1) + (j - 1) * m];
      t *= tau[i - 1];
      q[(i - 1) + (j - 1) * m] -= t;
      for (int r = i + 1; r <= m; ++r) q[(r - 1) + (j - 1) * m] -= A_(r, i) * t;
    }
  }
  for (int j = 1; j <= k; ++j)
    for (int i = j + 1; i <= m; ++i) A_(i, j) = 0.0;
#undef A_
}

// RQ of a (mr x n, ld mr, mr <= n): a = R Q, the full Q (n x n) = H(1) ... H(k) in q
__device__ void house_rq_d(int mr, int n, double* a, double* q) {
#define A_(i, j) a[((i) - 1) + ((j) - 1) * mr]
  const int k = mr < n ? mr : n;
  double tau[4];
  for (int i = k; i >= 1; --i) {
    const int row = mr - k + i, col = n - k + i;
    tau[i - 1] = larfg_d(col, &A_(row, col), &A_(row, 1), mr);
    if (tau[i - 1] != 0.0 && row > 1) {
      const double aii = A_(row, col);
      A_(row, col) = 1.0;
      for (int r = 1; r <= row - 1; ++r) {
        double t = 0.0;
        for (int c = 1; c <= col; ++c) t += A_(r, c) * A_(row, c);
        for (int c = 1; c <= col; ++c) A_(r, c) -= tau[i - 1] * t * A_(row, c);
      }
      A_(row, col) = aii;
    }
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) q[i + j * n] = i == j ? 1.0 : 0.0;
  for (int i = k; i >= 1; --i) {
    const int row = mr - k + i, col = n - k + i;
    if (tau[i - 1] == 0.0) continue;
    for (int j = 1; j <= n; ++j) {
      double t = q[(col - 1) + (j - 1) * n];
      for (int c = 1; c <= col - 1; ++c) t += A_(row, c) * q[(c - 1) + (j - 1) * n];
      t *= tau[i - 1];
      q[(col - 1) + (j - 1) * n] -= t;
      for (int c = 1; c <= col - 1; ++c) q[(c - 1) + (j - 1) * n] -= A_(row, c) * t;
    }
  }
  for (int i = 1; i <= mr; ++i)
    for (int j = 1; j <= n; ++j)
      if (j < n - mr + i) A_(i, j) = 0.0;
#undef A_
}

// C = op(A) op(B), all m x m (m <= 4)
__device__ void mm_d(int m, const double* A, bool ta, const double* B, bool tb, double* C) {
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) {
      double t = 0.0;
      for (int l = 0; l < m; ++l) t += (ta ? A[l + i * m] : A[i + l * m]) * (tb ? B[j + l * m] : B[l + j * m]);
      C[i + j * m] = t;
    }
}

// thread-local Julia Givens on a small matrix (ld): lmul!(G) rows, rmul!(., G) and
// rmul!(., G') columns, over the given range
__device__ void lrows(double* M, int ld, int i1, int i2, double c, double s, int j0, int j1) {
  for (int j = j0; j <= j1; ++j) {
    double* p1 = M + (i1 - 1) + (j - 1) * ld;
    double* p2 = M + (i2 - 1) + (j - 1) * ld;
    const double x = *p1, y = *p2;
    *p1 = c * x + s * y;
    *p2 = c * y - s * x;
  }
}
__device__ void lcols(double* M, int ld, int i1, int i2, double c, double s, int r0, int r1) {
  for (int r = r0; r <= r1; ++r) {
    double* p1 = M + (r - 1) + (i1 - 1) * ld;
    double* p2 = M + (r - 1) + (i2 - 1) * ld;
    const double x = *p1, y = *p2;
    *p1 = x * c - y * s;
    *p2 = x * s + y * c;
  }
}
__device__ void lcols_adj(double* M, int ld, int i1, int i2, double c, double s, int r0, int r1) {
  for (int r = r0; r <= r1; ++r) {
    double* p1 = M + (r - 1) + (i1 - 1) * ld;
    double* p2 = M + (r - 1) + (i2 - 1) * ld;
    const double x = *p1, y = *p2;
    *p1 = x * c + y * s;
    *p2 = y * c - x * s;
  }
}

// _gqz_2x2!(A, B) on the 2 x 2 blocks at a, b (ld)
__device__ void gqz_2x2_d(double* a, double* b, int ld, double& csl, double& snl, double& csr, double& snr) {
#define GA(i, j) a[((i) - 1) + ((j) - 1) * ld]
#define GB(i, j) b[((i) - 1) + ((j) - 1) * ld]
  const double safmin = Prec<double>::fmin, ulp = Prec<double>::eps;
  const double anorm = fmax(fmax(fabs(GA(1, 1)) + fabs(GA(2, 1)), fabs(GA(1, 2)) + fabs(GA(2, 2))), safmin);
  const double ascale = 1.0 / anorm;
  for (int j = 1; j <= 2; ++j) for (int i = 1; i <= 2; ++i) GA(i, j) *= ascale;
  const double bnorm = fmax(fmax(fabs(GB(1, 1)), fabs(GB(1, 2)) + fabs(GB(2, 2))), safmin);
  const double bscale = 1.0 / bnorm;
  for (int j = 1; j <= 2; ++j) for (int i = 1; i <= 2; ++i) GB(i, j) *= bscale;
  double rr;
  if (fabs(GA(2, 1)) < ulp) {
    csl = 1.0; snl = 0.0; csr = 1.0; snr = 0.0;
    GA(2, 1) = 0.0;
    GB(2, 1) = 0.0;
  } else if (fabs(GB(1, 1)) < ulp) {
    givens_alg(GA(1, 1), GA(2, 1), csl, snl, rr);
    csr = 1.0; snr = 0.0;
    lcols(a, ld, 1, 2, csl, snl, 1, 2);
    lcols(b, ld, 1, 2, csl, snl, 1, 2);
    GA(2, 1) = 0.0;
    GB(1, 1) = 0.0;
    GB(2, 1) = 0.0;
  } else if (fabs(GB(2, 2)) < ulp) {
    givens_alg(GA(2, 2), GA(2, 1), csr, snr, rr);
    lrows(a, ld, 1, 2, csr, -snr, 1, 2);
    lrows(b, ld, 1, 2, csr, -snr, 1, 2);
    csl = 1.0; snl = 0.0;
    GA(2, 1) = 0.0;
    GB(2, 1) = 0.0;
    GB(2, 2) = 0.0;
  } else {
    double scale1, scale2, wr1, wr2, wi;
    ggs2x2(a, b, ld, 1, safmin, scale1, scale2, wr1, wr2, wi);
    if (wi == 0.0) {
      const double h1 = scale1 * GA(1, 1) - wr1 * GB(1, 1);
      const double h2 = scale1 * GA(1, 2) - wr1 * GB(1, 2);
      const double h3 = scale1 * GA(2, 2) - wr1 * GB(2, 2);
      const double rr2 = hypot(h2, h1), qq = hypot(scale1 * GA(2, 1), h3);
      if (rr2 > qq) givens_alg(h2, h1, csr, snr, rr);
      else givens_alg(h3, scale1 * GA(2, 1), csr, snr, rr);
      lcols(a, ld, 1, 2, csr, snr, 1, 2);
      lcols(b, ld, 1, 2, csr, snr, 1, 2);
      snr = -snr;
      const double t1 = fmax(fabs(GA(1, 1)) + fabs(GA(1, 2)), fabs(GA(2, 1)) + fabs(GA(2, 2)));
      const double t2 = t1;
      if (scale1 * t1 >= fabs(wr1) * t2) givens_alg(GB(1, 1), GB(2, 1), csl, snl, rr);
      else givens_alg(GA(1, 1), GA(2, 1), csl, snl, rr);
      lrows(a, ld, 1, 2, csl, snl, 1, 2);
      lrows(b, ld, 1, 2, csl, snl, 1, 2);
      GA(2, 1) = 0.0;
      GB(2, 1) = 0.0;
    } else {
      double ssmin, ssmax;
      gsvd2x2(GB(1, 1), GB(1, 2), GB(2, 2), ssmin, ssmax, snr, csr, snl, csl);
      lcols_adj(a, ld, 1, 2, csr, snr, 1, 2);
      lcols_adj(b, ld, 1, 2, csr, snr, 1, 2);
      lrows(a, ld, 1, 2, csl, snl, 1, 2);
      lrows(b, ld, 1, 2, csl, snl, 1, 2);
      GB(2, 1) = 0.0;
      GB(1, 2) = 0.0;
    }
  }
  for (int j = 1; j <= 2; ++j) for (int i = 1; i <= 2; ++i) GA(i, j) *= anorm;
  for (int j = 1; j <= 2; ++j) for (int i = 1; i <= 2; ++i) GB(i, j) *= bnorm;
#undef GA
#undef GB
}

// The plan of one swap, written by thread 0: for 1 x 1 pairs the four rotation
// coefficients; otherwise the new m x m blocks of A and B and the transforms qf, zf.
struct RordPlan {
  int ok, m;
  double cz, sz, cq, sq;
  double SA[16], SB[16], qf[16], zf[16];
};

// _rtrexch2! (1096-1178): the rotations and the stability tests, on copies
__device__ void plan_rtrexch2(const double* A, const double* B, int n, int j1, RordPlan& P) {
  double S[4] = {A[(j1 - 1) + (size_t)(j1 - 1) * n], A[j1 + (size_t)(j1 - 1) * n], A[(j1 - 1) + (size_t)j1 * n],
                 A[j1 + (size_t)j1 * n]};
  double T[4] = {B[(j1 - 1) + (size_t)(j1 - 1) * n], B[j1 + (size_t)(j1 - 1) * n], B[(j1 - 1) + (size_t)j1 * n],
                 B[j1 + (size_t)j1 * n]};
  const double S0[4] = {S[0], S[1], S[2], S[3]}, T0[4] = {T[0], T[1], T[2], T[3]};
  const double smlnum = Prec<double>::fmin / Prec<double>::eps;
  double W[8] = {S[0], S[1], S[2], S[3], T[0], T[1], T[2], T[3]};
  double sa = safe_fnorm_blk(W, 8, 8, 1);
  const double thresh = fmax(20.0 * Prec<double>::eps * sa, smlnum);
  const double f = S[3] * T[0] - T[3] * S[0];
  const double g = S[3] * T[2] - T[3] * S[2];
  sa = fabs(S[3]) * fabs(T[0]);
  const double sb = fabs(S[0]) * fabs(T[3]);
  double cz, sz, rr;
  givens_alg(f, g, cz, sz, rr);
  { const double t = sz; sz = cz; cz = t; }
  lcols_adj(S, 2, 1, 2, cz, -sz, 1, 2);
  lcols_adj(T, 2, 1, 2, cz, -sz, 1, 2);
  const double fq = sa >= sb ? S[0] : T[0], gq = sa >= sb ? S[1] : T[1];
  double cq, sq;
  if (sz != 0.0 && fq == 0.0 && gq == 0.0) { cq = 0.0; sq = 1.0; }
  else givens_alg(fq, gq, cq, sq, rr);
  lrows(S, 2, 1, 2, cq, sq, 1, 2);
  lrows(T, 2, 1, 2, cq, sq, 1, 2);
  P.cz = cz; P.sz = sz; P.cq = cq; P.sq = sq; P.m = 2;
  const double ws = fabs(S[1]) + fabs(T[1]);
  if (!(ws <= thresh)) { P.ok = 0; return; }
  double Ss[4] = {S[0], S[1], S[2], S[3]}, Ts[4] = {T[0], T[1], T[2], T[3]};
  lcols_adj(Ss, 2, 1, 2, cz, sz, 1, 2);
  lcols_adj(Ts, 2, 1, 2, cz, sz, 1, 2);
  lrows(Ss, 2, 1, 2, cq, -sq, 1, 2);
  lrows(Ts, 2, 1, 2, cq, -sq, 1, 2);
  for (int e = 0; e < 4; ++e) { W[e] = Ss[e] - S0[e]; W[4 + e] = Ts[e] - T0[e]; }
  const double ss = safe_fnorm_blk(W, 8, 8, 1);
  P.ok = ss <= thresh ? 1 : 0;
}

// _swap1or2! (768-962) with at least one 2 x 2 block: the new blocks and transforms
__device__ void plan_swap2(const double* A, const double* B, int n, int j1, int n1, int n2, RordPlan& P) {
  const int m = n1 + n2;
  P.m = m;
  double S[16], T[16];
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) {
      S[i + j * m] = A[(j1 - 1 + i) + (size_t)(j1 - 1 + j) * n];
      T[i + j * m] = B[(j1 - 1 + i) + (size_t)(j1 - 1 + j) * n];
    }
  const double eps = Prec<double>::eps, smallnum = Prec<double>::fmin / eps;
  double dnorm = 0.0, tnorm = 0.0;
  for (int e = 0; e < m * m; ++e) { dnorm = fmax(dnorm, fabs(S[e])); tnorm = fmax(tnorm, fabs(T[e])); }
  const double thresh = fmax(20.0 * eps * dnorm, smallnum), threshb = fmax(20.0 * eps * tnorm, smallnum);
  // _syl1or2: the Kronecker system for [vec R; vec L]
  const int nn = n1 * n2, kd = 2 * nn;
  double K[64], rl[8];
  for (int e = 0; e < kd * kd; ++e) K[e] = 0.0;
  for (int q = 0; q < n2; ++q)
    for (int p = 0; p < n1; ++p) {
      const int row = p + q * n1;
      for (int pp = 0; pp < n1; ++pp) {
        K[row + (pp + q * n1) * kd] = S[p + pp * m];
        K[(nn + row) + (pp + q * n1) * kd] = T[p + pp * m];
      }
      for (int qq = 0; qq < n2; ++qq) {
        K[row + (nn + p + qq * n1) * kd] = -S[(n1 + qq) + (n1 + q) * m];
        K[(nn + row) + (nn + p + qq * n1) * kd] = -T[(n1 + qq) + (n1 + q) * m];
      }
      rl[row] = S[p + (n1 + q) * m];
      rl[nn + row] = T[p + (n1 + q) * m];
    }
  const double scale = safe_lu_real(kd, K, rl);
  double LI[8], IR[8], qli[16], zir[16];
  for (int j = 0; j < n2; ++j) {
    for (int i = 0; i < n1; ++i) LI[i + j * m] = -rl[nn + i + j * n1];
    for (int i = 0; i < n2; ++i) LI[n1 + i + j * m] = i == j ? scale : 0.0;
  }
  for (int i = 0; i < n1; ++i) {
    for (int j = 0; j < n1; ++j) IR[i + j * n1] = i == j ? scale : 0.0;
    for (int j = 0; j < n2; ++j) IR[i + (n1 + j) * n1] = rl[i + j * n1];
  }
  house_qr_d(m, n2, LI, qli);
  house_rq_d(n1, m, IR, zir);
  double tmp[16], s1[16], t1[16];
  mm_d(m, qli, true, S, false, tmp);
  mm_d(m, tmp, false, zir, true, s1);
  mm_d(m, qli, true, T, false, tmp);
  mm_d(m, tmp, false, zir, true, t1);
  double t2a[16], zt1a[16], s2a[16], z2a[16], t2b[16], qt1b[16], s2b[16], q2b[16];
  for (int e = 0; e < m * m; ++e) { t2a[e] = t1[e]; t2b[e] = t1[e]; }
  house_rq_d(m, m, t2a, zt1a);
  mm_d(m, s1, false, zt1a, true, s2a);
  mm_d(m, zt1a, false, zir, false, z2a);
  const double brq = safe_fnorm_blk(s2a + n2, m, m - n2, n2);
  house_qr_d(m, m, t2b, qt1b);
  mm_d(m, qt1b, true, s1, false, s2b);
  mm_d(m, qli, false, qt1b, false, q2b);
  const double bqr = safe_fnorm_blk(s2b + n2, m, m - n2, n2);
  if (!(fmin(bqr, brq) <= thresh) || bqr != bqr || brq != brq) { P.ok = 0; return; }
  const bool useb = bqr <= brq;
  double* snew = useb ? s2b : s2a;
  double* tnew = useb ? t2b : t2a;
  const double* znew = useb ? zir : z2a;
  const double* qnew = useb ? q2b : qli;
  {
    double r1[16], r2[16];
    mm_d(m, qnew, false, snew, false, r1);
    mm_d(m, r1, false, znew, false, r2);
    for (int e = 0; e < m * m; ++e) r2[e] = S[e] - r2[e];
    const double resa = safe_fnorm_blk(r2, m, m, m);
    mm_d(m, qnew, false, tnew, false, r1);
    mm_d(m, r1, false, znew, false, r2);
    for (int e = 0; e < m * m; ++e) r2[e] = T[e] - r2[e];
    const double resb = safe_fnorm_blk(r2, m, m, m);
    if (!(resa <= thresh && resb <= threshb)) { P.ok = 0; return; }
  }
  for (int j = 0; j < n2; ++j)
    for (int i = n2; i < m; ++i) snew[i + j * m] = 0.0;
  double qtmp[16], ztmp[16];
  for (int e = 0; e < m * m; ++e) { qtmp[e] = 0.0; ztmp[e] = 0.0; }
  double csl, snl, csr, snr;
  if (n2 > 1) {
    gqz_2x2_d(snew, tnew, m, csl, snl, csr, snr);
    qtmp[0] = csl; qtmp[1] = snl; qtmp[m] = -snl; qtmp[m + 1] = csl;
    ztmp[0] = csr; ztmp[1] = snr; ztmp[m] = -snr; ztmp[m + 1] = csr;
  } else {
    ztmp[0] = 1.0;
    qtmp[0] = 1.0;
  }
  if (n1 > 1) {
    const int o = n2 + n2 * m;  // (j3, j3) within the block
    gqz_2x2_d(snew + o, tnew + o, m, csl, snl, csr, snr);
    qtmp[(m - 2) + (m - 2) * m] = csl; qtmp[(m - 1) + (m - 2) * m] = snl;
    qtmp[(m - 2) + (m - 1) * m] = -snl; qtmp[(m - 1) + (m - 1) * m] = csl;
    ztmp[(m - 2) + (m - 2) * m] = csr; ztmp[(m - 1) + (m - 2) * m] = snr;
    ztmp[(m - 2) + (m - 1) * m] = -snr; ztmp[(m - 1) + (m - 1) * m] = csr;
  } else {
    qtmp[(m - 1) + (m - 1) * m] = 1.0;
    ztmp[(m - 1) + (m - 1) * m] = 1.0;
  }
  // the off-diagonal block: qtmp[1:n2,1:n2]' X ztmp[n2+1:m, n2+1:m]
  for (int w = 0; w < 2; ++w) {
    double* M = w == 0 ? snew : tnew;
    double X[4], ab[4];
    for (int j = 0; j < n1; ++j) for (int i = 0; i < n2; ++i) X[i + j * n2] = M[i + (n2 + j) * m];
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n2; ++i) {
        double t = 0.0;
        for (int l = 0; l < n2; ++l) t += qtmp[l + i * m] * X[l + j * n2];
        ab[i + j * n2] = t;
      }
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n2; ++i) {
        double t = 0.0;
        for (int l = 0; l < n1; ++l) t += ab[i + l * n2] * ztmp[(n2 + l) + (n2 + j) * m];
        M[i + (n2 + j) * m] = t;
      }
  }
  mm_d(m, qnew, false, qtmp, false, P.qf);
  mm_d(m, znew, true, ztmp, false, P.zf);
  for (int e = 0; e < m * m; ++e) { P.SA[e] = snew[e]; P.SB[e] = tnew[e]; }
  P.ok = 1;
}

// _swap1or2!(A, B, Q, Z, j1, n1, n2) on the CTA
__device__ bool cta_swap1or2(double* A, double* B, double* Q, double* Z, int n, int j1, int n1, int n2, RordPlan& P) {
  if (j1 + n1 > n) return true;
  const int tid = threadIdx.x;
  __syncthreads();
  if (tid == 0) {
    if (n1 == 1 && n2 == 1) plan_rtrexch2(A, B, n, j1, P);
    else plan_swap2(A, B, n, j1, n1, n2, P);
  }
  __syncthreads();
  if (!P.ok) return false;
  if (n1 == 1 && n2 == 1) {
    const double cz = P.cz, sz = P.sz, cq = P.cq, sq = P.sq;
    ccols_adj(A, n, j1, j1 + 1, cz, -sz, 1, n);
    ccols_adj(B, n, j1, j1 + 1, cz, -sz, 1, n);
    __syncthreads();
    crows(A, n, j1, j1 + 1, cq, sq, 1, n);
    crows(B, n, j1, j1 + 1, cq, sq, 1, n);
    __syncthreads();
    if (tid == 0) {
      A[j1 + (size_t)(j1 - 1) * n] = 0.0;
      B[j1 + (size_t)(j1 - 1) * n] = 0.0;
    }
    if (Z) ccols_adj(Z, n, j1, j1 + 1, cz, -sz, 1, n);
    if (Q) ccols_adj(Q, n, j1, j1 + 1, cq, sq, 1, n);
    __syncthreads();
    return true;
  }
  const int m = P.m, je = j1 + m - 1;
  for (int e = tid; e < m * m; e += kQrT) {
    const int i = e % m, j = e / m;
    A[(j1 - 1 + i) + (size_t)(j1 - 1 + j) * n] = P.SA[e];
    B[(j1 - 1 + i) + (size_t)(j1 - 1 + j) * n] = P.SB[e];
  }
  // Q[:, j1:je] qf, Z[:, j1:je] zf, A[1:j1-1, j1:je] zf (and B)
  for (int r = tid; r < n; r += kQrT) {
    double v[4];
    if (Q) {
      for (int j = 0; j < m; ++j) v[j] = Q[r + (size_t)(j1 - 1 + j) * n];
      for (int j = 0; j < m; ++j) {
        double t = 0.0;
        for (int l = 0; l < m; ++l) t += v[l] * P.qf[l + j * m];
        Q[r + (size_t)(j1 - 1 + j) * n] = t;
      }
    }
    if (Z) {
      for (int j = 0; j < m; ++j) v[j] = Z[r + (size_t)(j1 - 1 + j) * n];
      for (int j = 0; j < m; ++j) {
        double t = 0.0;
        for (int l = 0; l < m; ++l) t += v[l] * P.zf[l + j * m];
        Z[r + (size_t)(j1 - 1 + j) * n] = t;
      }
    }
    if (r < j1 - 1)
      for (int w = 0; w < 2; ++w) {
        double* M = w == 0 ? A : B;
        for (int j = 0; j < m; ++j) v[j] = M[r + (size_t)(j1 - 1 + j) * n];
        for (int j = 0; j < m; ++j) {
          double t = 0.0;
          for (int l = 0; l < m; ++l) t += v[l] * P.zf[l + j * m];
          M[r + (size_t)(j1 - 1 + j) * n] = t;
        }
      }
  }
  // A[j1:je, je+1:n] = qf' A[j1:je, je+1:n] (and B)
  for (int c = je + 1 + tid; c <= n; c += kQrT)
    for (int w = 0; w < 2; ++w) {
      double* M = w == 0 ? A : B;
      double v[4];
      for (int i = 0; i < m; ++i) v[i] = M[(j1 - 1 + i) + (size_t)(c - 1) * n];
      for (int i = 0; i < m; ++i) {
        double t = 0.0;
        for (int l = 0; l < m; ++l) t += P.qf[l + i * m] * v[l];
        M[(j1 - 1 + i) + (size_t)(c - 1) * n] = t;
      }
    }
  __syncthreads();
  return true;
}

__global__ void __launch_bounds__(kQrT) k_ggordschur_real(double* S, double* T, double* Q, double* Z, int n,
                                                          const int* __restrict__ select, int scale, double2* alpha,
                                                          double* beta, int* status) {
  __shared__ double red[kQrT / 32];
  __shared__ RordPlan P;
  const int tid = threadIdx.x;
  double cscale = 1.0, anrm = 1.0, cscaleb = 1.0, bnrm = 1.0;
  bool scA = false, scB = false;
  if (scale) {
    scA = cta_scale_real(S, n, red, cscale, anrm);
    scB = cta_scale_real(T, n, red, cscaleb, bnrm);
  }
  __syncthreads();
#define SM(i, j) S[((i) - 1) + (size_t)((j) - 1) * n]
#define TM(i, j) T[((i) - 1) + (size_t)((j) - 1) * n]
  int st = 0, ks = 0;
  bool inpair = false;
  for (int k = 1; k <= n && !st; ++k) {
    if (inpair) { inpair = false; continue; }
    __syncthreads();
    bool doswap = select[k - 1] != 0;
    if (k < n && SM(k + 1, k) != 0.0) {
      inpair = true;
      doswap = doswap || select[k] != 0;
    }
    if (!doswap) continue;
    ks += 1;
    if (k != ks) {
      // _trexchange!(S, T, Q, Z, k, ks), the move-up branch
      int iold = k, inew = ks;
      if (iold > 1 && SM(iold, iold - 1) != 0.0) iold -= 1;
      const int nbold = (iold < n && SM(iold + 1, iold) != 0.0) ? 2 : 1;
      if (inew > 1 && SM(inew, inew - 1) != 0.0) inew -= 1;
      int ihere = iold;
      bool ok = iold >= inew;
      while (ok && ihere > inew) {
        __syncthreads();
        const int nbnext = (ihere >= 3 && SM(ihere - 1, ihere - 2) != 0.0) ? 2 : 1;
        ok = cta_swap1or2(S, T, Q, Z, n, ihere - nbnext, nbnext, nbold, P);
        if (ok) ihere -= nbnext;
      }
      if (!ok) { st = 1 + k; break; }
      ks = ihere;
    }
    if (inpair) ks += 1;
  }
  __syncthreads();
  if (!st) {
    if (scA) cta_safescale_real(S, (size_t)n * n, cscale, anrm);
    if (scB) cta_safescale_real(T, (size_t)n * n, cscaleb, bnrm);
    __syncthreads();
    inpair = false;
    for (int k = 1; k <= n; ++k) {
      if (inpair) { inpair = false; continue; }
      __syncthreads();
      if (k < n && SM(k + 1, k) != 0.0) inpair = true;
      if (inpair) {
        if (tid == 0) {
          double b1, b2, ar1, ar2, ai;
          ggs2x2(&SM(k, k), &TM(k, k), n, 1, Prec<double>::fmin, b1, b2, ar1, ar2, ai);
          alpha[k - 1] = make_double2(ar1, ai);
          alpha[k] = make_double2(ar2, -ai);
          beta[k - 1] = b1;
          beta[k] = b2;
        }
      } else {
        if (copysign(1.0, TM(k, k)) < 0.0) {
          __syncthreads();
          for (int j = 1 + tid; j <= n; j += kQrT) { SM(k, j) = -SM(k, j); TM(k, j) = -TM(k, j); }
          if (Q) cnegcol(Q, n, k, 1, n);
          __syncthreads();
        }
        if (tid == 0) {
          alpha[k - 1] = make_double2(SM(k, k), 0.0);
          beta[k - 1] = TM(k, k);
        }
      }
    }
  }
#undef SM
#undef TM
  if (tid == 0) *status = st;
}

}  // namespace

cudaError_t launch_ggordschur_real(int n, double* S, double* T, double* Q, double* Z, const int* select, int scale,
                                   double2* alpha, double* beta, int* status, cudaStream_t s) {
  k_ggordschur_real<<<1, kQrT, 0, s>>>(S, T, Q, Z, n, select, scale, alpha, beta, status);
  return cudaGetLastError();
}

cudaError_t launch_ggschur_real(const QzrBatch& bt, int num_sms, cudaStream_t s) {
  if (bt.count <= 0) return cudaSuccess;
  const int grid = std::min(bt.count, 8 * num_sms);
  k_ggschur_real<<<grid, kQrT, 0, s>>>(bt);
  return cudaGetLastError();
}

}  // namespace gsk
