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

}  // namespace

cudaError_t launch_ggschur_real(const QzrBatch& bt, int num_sms, cudaStream_t s) {
  if (bt.count <= 0) return cudaSuccess;
  const int grid = std::min(bt.count, 8 * num_sms);
  k_ggschur_real<<<grid, kQrT, 0, s>>>(bt);
  return cudaGetLastError();
}

}  // namespace gsk
