// Generalized Schur decomposition of complex pencils: ggschur!(A, B) (generalized.jl:21-80)
// with qr!(B), the Hessenberg-triangular reduction _hessenberg! (82-113, zgghrd) and the
// single-shift QZ iteration _gqz! (125-487, zhgeqz).  One CTA per pencil (a ragged batch,
// or a batch of one), the four matrices in global memory (L2-resident for the orders this
// path serves).  The control flow of the reference runs warp-uniform: every scalar
// decision and every Givens rotation is computed by thread 0 and published through
// shared memory; the rotations are applied to rows / columns by all threads between
// barriers.  Row rotations read strided (column-major storage), column rotations
// coalesced.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kQzT = 128;

__device__ __forceinline__ double cabs1max(double2 z) { return fmax(fabs(z.x), fabs(z.y)); }
__device__ __forceinline__ double2 zmulr(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ bool zis0(double2 a) { return a.x == 0.0 && a.y == 0.0; }

// LinearAlgebra.givensAlgorithm(f::Complex, g::Complex) (LAPACK 3.x zlartg): c real,
// [c s; -conj(s) c] [f; g] = [r; 0].
__device__ void zgivens(double2 f, double2 g, double& cs, double2& sn, double2& r) {
  const double mn2 = 0x1p-485, mx2 = 0x1p485;
  const double safmin = Prec<double>::fmin;
  double2 fs = f, gs = g;
  double scale = fmax(cabs1max(f), cabs1max(g));
  int count = 0;
  if (scale >= mx2) {
    do { ++count; fs = zmulr(fs, mn2); gs = zmulr(gs, mn2); scale *= mn2; } while (!(scale < mx2 || count >= 20));
  } else if (scale <= mn2) {
    if (zis0(g)) { cs = 1.0; sn = make_double2(0.0, 0.0); r = f; return; }
    do { --count; fs = zmulr(fs, mx2); gs = zmulr(gs, mx2); scale *= mx2; } while (!(scale > mn2) && count > -80);
  }
  const double f2 = fs.x * fs.x + fs.y * fs.y, g2 = gs.x * gs.x + gs.y * gs.y;
  if (f2 <= fmax(g2, 1.0) * safmin) {
    if (zis0(f)) {
      cs = 0.0;
      r = make_double2(hypot(g.x, g.y), 0.0);
      const double d = hypot(gs.x, gs.y);
      sn = make_double2(gs.x / d, -gs.y / d);
      return;
    }
    const double f2s = hypot(fs.x, fs.y), g2s = sqrt(g2);
    cs = f2s / g2s;
    double2 ff;
    if (cabs1max(f) > 1.0) {
      const double d = hypot(f.x, f.y);
      ff = make_double2(f.x / d, f.y / d);
    } else {
      const double dr = mx2 * f.x, di = mx2 * f.y, d = hypot(dr, di);
      ff = make_double2(dr / d, di / d);
    }
    sn = zmul(ff, make_double2(gs.x / g2s, -gs.y / g2s));
    r = zadd(zmulr(f, cs), zmul(sn, g));
    return;
  }
  const double f2s = sqrt(1.0 + g2 / f2);
  double2 rr = make_double2(f2s * fs.x, f2s * fs.y);
  cs = 1.0 / f2s;
  const double d = f2 + g2;
  sn = zmul(make_double2(rr.x / d, rr.y / d), zconj(gs));
  if (count > 0) for (int i = 0; i < count; ++i) rr = zmulr(rr, mx2);
  else for (int i = 0; i < -count; ++i) rr = zmulr(rr, mn2);
  r = rr;
}

struct QzMats {
  double2* A;  // H (the S factor on return)
  double2* B;  // T
  double2* Q;  // null when not wanted
  double2* Z;
  int n;
};
#define QA(i, j) m.A[((i) - 1) + (size_t)((j) - 1) * m.n]
#define QB(i, j) m.B[((i) - 1) + (size_t)((j) - 1) * m.n]

// lmul!(G, M) on rows i1, i2, columns j0..j1 (1-based): [x; y] <- [c x + s y; c y - conj(s) x]
__device__ __forceinline__ void rot_rows(double2* M, int n, int i1, int i2, double c, double2 s, int j0, int j1) {
  for (int j = j0 + (int)threadIdx.x; j <= j1; j += kQzT) {
    double2* p1 = M + (i1 - 1) + (size_t)(j - 1) * n;
    double2* p2 = M + (i2 - 1) + (size_t)(j - 1) * n;
    const double2 x = *p1, y = *p2;
    *p1 = zfma(s, y, zmulr(x, c));
    *p2 = zsub(zmulr(y, c), zmul(zconj(s), x));
  }
}
// rmul!(M, G) on columns i1, i2, rows r0..r1: [a1 a2] <- [c a1 - conj(s) a2, s a1 + c a2]
__device__ __forceinline__ void rot_cols(double2* M, int n, int i1, int i2, double c, double2 s, int r0, int r1) {
  for (int r = r0 + (int)threadIdx.x; r <= r1; r += kQzT) {
    double2* p1 = M + (r - 1) + (size_t)(i1 - 1) * n;
    double2* p2 = M + (r - 1) + (size_t)(i2 - 1) * n;
    const double2 x = *p1, y = *p2;
    *p1 = zsub(zmulr(x, c), zmul(y, zconj(s)));
    *p2 = zfma(x, s, zmulr(y, c));
  }
}
// rmul!(M, G') on columns i1, i2, rows r0..r1: [a1 a2] <- [c a1 + conj(s) a2, c a2 - s a1]
__device__ __forceinline__ void rot_cols_adj(double2* M, int n, int i1, int i2, double c, double2 s, int r0, int r1) {
  for (int r = r0 + (int)threadIdx.x; r <= r1; r += kQzT) {
    double2* p1 = M + (r - 1) + (size_t)(i1 - 1) * n;
    double2* p2 = M + (r - 1) + (size_t)(i2 - 1) * n;
    const double2 x = *p1, y = *p2;
    *p1 = zfma(zconj(s), y, zmulr(x, c));
    *p2 = zsub(zmulr(y, c), zmul(s, x));
  }
}

// Largest modulus of an n x n matrix (norm(M, Inf) of a matrix), NaN-propagating.
__device__ double cta_maxabs(const double2* M, int n, double* red) {
  double v = 0.0;
  for (size_t e = threadIdx.x; e < (size_t)n * n; e += kQzT) {
    const double a = hypot(M[e].x, M[e].y);
    if (a > v || a != a) v = a;
  }
  return block_max<kQzT>(v, red);
}

// safescale!(M, cfrom, cto) (util.jl:41-80) on all n x n entries.
__device__ void cta_safescale(double2* M, int n, double cfrom, double cto) {
  double mul[8];
  const int k = safescale_factors(cfrom, cto, mul);
  for (size_t e = threadIdx.x; e < (size_t)n * n; e += kQzT) {
    double2 v = M[e];
    for (int q = 0; q < k; ++q) v = zmulr(v, mul[q]);
    M[e] = v;
  }
  __syncthreads();
}

// _scale! (util.jl:14-29): returns whether M was scaled; cscale / anrm as the reference.
__device__ bool cta_scale(double2* M, int n, double* red, double& cscale, double& anrm) {
  const double smlnum = sqrt(Prec<double>::fmin) / Prec<double>::eps, bignum = 1.0 / smlnum;
  anrm = cta_maxabs(M, n, red);
  cscale = 1.0;
  bool sc = false;
  if (anrm > 0.0 && anrm < smlnum) { sc = true; cscale = smlnum; }
  else if (anrm > bignum) { sc = true; cscale = bignum; }
  if (sc) cta_safescale(M, n, anrm, cscale);
  return sc;
}

// Frobenius norm of an n x n matrix without overflow.
__device__ double cta_fro(const double2* M, int n, double* red) {
  double mx = 0.0;
  for (size_t e = threadIdx.x; e < (size_t)n * n; e += kQzT) mx = fmax(mx, fmax(fabs(M[e].x), fabs(M[e].y)));
  mx = block_max<kQzT>(mx, red);
  if (!(mx > 0.0) || !isfinite(mx)) return mx;
  const double inv = 1.0 / mx;
  double ss = 0.0;
  for (size_t e = threadIdx.x; e < (size_t)n * n; e += kQzT) {
    const double a = M[e].x * inv, b = M[e].y * inv;
    ss = fma(a, a, fma(b, b, ss));
  }
  ss = block_sum<kQzT>(ss, red);
  return mx * sqrt(ss);
}

struct QzShared {
  double c;
  double2 s;
  int br, j, t1a, ifirst, ilast, brk, done, status, istart, shiftcount;
  double2 eshift, signbc;
  double absb;
  long long niter;
};

enum { BR_UNKNOWN = 0, BR_NONE = 1, BR_NORMAL = 2, BR_INF = 3, BR_CHASE_H = 4, BR_CHASE_B = 5 };

// _gqz! with ilo = 1, ihi = n, wantSchur.  Returns 0 or 1 (iteration limit).
__device__ int qz_iterate(const QzMats& m, double2* alpha, double2* beta, long long maxiter, double* red,
                          QzShared& sh) {
  const int n = m.n, tid = threadIdx.x;
  const int ilo = 1;
  const double ulp = Prec<double>::eps, safmin = Prec<double>::fmin;
  const double anorm = cta_fro(m.A, n, red), bnorm = cta_fro(m.B, n, red);
  const double atol = fmax(safmin, ulp * anorm), btol = fmax(safmin, ulp * bnorm);
  const double ascale = 1.0 / fmax(safmin, anorm), bscale = 1.0 / fmax(safmin, bnorm);
  if (tid == 0) {
    sh.ifirst = ilo; sh.ilast = n; sh.shiftcount = 0; sh.eshift = make_double2(0.0, 0.0);
    sh.niter = 0; sh.done = 0; sh.status = 0;
  }
  for (;;) {
    __syncthreads();  // every thread has read the previous iteration's shared state
    // ---- deflation checks (thread 0) ----
    if (tid == 0) {
      int br = BR_UNKNOWN;
      const int ilast = sh.ilast;
      if (++sh.niter > maxiter) { sh.status = 1; sh.done = 1; }
      else if (ilast == ilo) br = BR_NORMAL;
      else if (zabs1(QA(ilast, ilast - 1)) < fmax(safmin, ulp * (zabs1(QA(ilast, ilast)) + zabs1(QA(ilast - 1, ilast - 1))))) {
        QA(ilast, ilast - 1) = make_double2(0.0, 0.0);
        br = BR_NORMAL;
      }
      if (!sh.done && br == BR_UNKNOWN) {
        if (zabs(QB(ilast, ilast)) <= btol) {
          QB(ilast, ilast) = make_double2(0.0, 0.0);
          br = BR_INF;
        } else {
          for (int j = ilast - 1; j >= ilo; --j) {
            bool t1 = false;
            if (j == ilo) t1 = true;
            else if (zabs1(QA(j, j - 1)) <= fmax(safmin, ulp * (zabs1(QA(j, j)) + zabs1(QA(j - 1, j - 1))))) {
              QA(j, j - 1) = make_double2(0.0, 0.0);
              t1 = true;
            }
            const bool t2 = zabs(QB(j, j)) < btol;
            if (t2) {
              QB(j, j) = make_double2(0.0, 0.0);
              const bool t1a = !t1 && (zabs1(QA(j, j - 1)) * (ascale * zabs1(QA(j + 1, j))) <= zabs1(QA(j, j)) * (ascale * atol));
              sh.j = j;
              sh.t1a = t1a ? 1 : 0;
              br = (t1 || t1a) ? BR_CHASE_H : BR_CHASE_B;
              break;
            } else if (t1) {
              sh.ifirst = j;
              br = BR_NONE;
              break;
            }
          }
        }
      }
      sh.br = br;
    }
    __syncthreads();
    if (sh.done) break;
    int br = sh.br;
    const int ilast = sh.ilast;
    if (br == BR_CHASE_H) {
      // split a 1x1 block off the top of the singular part (generalized.jl:214-247)
      int res = BR_UNKNOWN;
      for (int jch = sh.j; jch <= ilast - 1; ++jch) {
        if (tid == 0) {
          double c;
          double2 s, r;
          zgivens(QA(jch, jch), QA(jch + 1, jch), c, s, r);
          QA(jch, jch) = r;
          QA(jch + 1, jch) = make_double2(0.0, 0.0);
          sh.c = c; sh.s = s;
        }
        __syncthreads();
        const double c = sh.c;
        const double2 s = sh.s;
        rot_rows(m.A, n, jch, jch + 1, c, s, jch + 1, n);
        rot_rows(m.B, n, jch, jch + 1, c, s, jch + 1, n);
        if (m.Q) rot_cols_adj(m.Q, n, jch, jch + 1, c, s, 1, n);
        __syncthreads();
        if (tid == 0) {
          if (sh.t1a) QA(jch, jch - 1) = zmulr(QA(jch, jch - 1), c);
          sh.t1a = 0;
          sh.brk = 0;
          if (zabs1(QB(jch + 1, jch + 1)) > btol) {
            if (jch + 1 >= ilast) sh.brk = BR_NORMAL;
            else { sh.ifirst = jch + 1; sh.brk = BR_NONE; }
          } else {
            QB(jch + 1, jch + 1) = make_double2(0.0, 0.0);
          }
        }
        __syncthreads();
        if (sh.brk) { res = sh.brk; break; }
      }
      br = res == BR_UNKNOWN ? BR_INF : res;
    } else if (br == BR_CHASE_B) {
      // chase the zero of B down to B[ilast, ilast] (generalized.jl:248-275)
      for (int jch = sh.j; jch <= ilast - 1; ++jch) {
        if (tid == 0) {
          double c;
          double2 s, r;
          zgivens(QB(jch, jch + 1), QB(jch + 1, jch + 1), c, s, r);
          QB(jch, jch + 1) = r;
          QB(jch + 1, jch + 1) = make_double2(0.0, 0.0);
          sh.c = c; sh.s = s;
        }
        __syncthreads();
        {
          const double c = sh.c;
          const double2 s = sh.s;
          if (jch < n - 1) rot_rows(m.B, n, jch, jch + 1, c, s, jch + 2, n);
          rot_rows(m.A, n, jch, jch + 1, c, s, jch - 1, n);
          if (m.Q) rot_cols_adj(m.Q, n, jch, jch + 1, c, s, 1, n);
        }
        __syncthreads();
        if (tid == 0) {
          double c;
          double2 s, r;
          zgivens(zconj(QA(jch + 1, jch)), zconj(QA(jch + 1, jch - 1)), c, s, r);
          QA(jch + 1, jch) = zconj(r);
          QA(jch + 1, jch - 1) = make_double2(0.0, 0.0);
          sh.c = c; sh.s = s;
        }
        __syncthreads();
        {
          const double c = sh.c;
          const double2 s = sh.s;
          rot_cols_adj(m.A, n, jch, jch - 1, c, s, 1, jch);
          rot_cols_adj(m.B, n, jch, jch - 1, c, s, 1, jch + 1);
          if (m.Z) rot_cols_adj(m.Z, n, jch, jch - 1, c, s, 1, n);
        }
        __syncthreads();
      }
      br = BR_INF;
    }
    if (br == BR_INF) {
      // B[ilast, ilast] == 0: clear H[ilast, ilast-1] (generalized.jl:284-294)
      if (tid == 0) {
        double c;
        double2 s, r;
        zgivens(zconj(QA(ilast, ilast)), zconj(QA(ilast, ilast - 1)), c, s, r);
        QA(ilast, ilast) = zconj(r);
        QA(ilast, ilast - 1) = make_double2(0.0, 0.0);
        sh.c = c; sh.s = s;
      }
      __syncthreads();
      const double c = sh.c;
      const double2 s = sh.s;
      rot_cols_adj(m.A, n, ilast, ilast - 1, c, s, 1, ilast - 1);
      rot_cols_adj(m.B, n, ilast, ilast - 1, c, s, 1, ilast - 1);
      if (m.Z) rot_cols_adj(m.Z, n, ilast, ilast - 1, c, s, 1, n);
      __syncthreads();
      br = BR_NORMAL;
    }
    if (br == BR_NORMAL) {
      // standardize B[ilast, ilast] real >= 0; record alpha, beta (generalized.jl:296-330)
      if (tid == 0) {
        const double absb = zabs(QB(ilast, ilast));
        sh.absb = absb;
        if (absb > safmin) {
          const double2 bl = QB(ilast, ilast);
          sh.signbc = zconj(make_double2(bl.x / absb, bl.y / absb));
        }
      }
      __syncthreads();
      if (sh.absb > safmin) {
        const double2 sg = sh.signbc;
        for (int i = 1 + tid; i <= ilast - 1; i += kQzT) QB(i, ilast) = zmul(QB(i, ilast), sg);
        for (int i = 1 + tid; i <= ilast; i += kQzT) QA(i, ilast) = zmul(QA(i, ilast), sg);
        if (m.Z)
          for (int i = tid; i < n; i += kQzT) {
            double2* z = m.Z + i + (size_t)(ilast - 1) * n;
            *z = zmul(*z, sg);
          }
      }
      __syncthreads();
      if (tid == 0) {
        if (sh.absb > safmin) QB(ilast, ilast) = make_double2(sh.absb, 0.0);
        else QB(ilast, ilast) = make_double2(0.0, 0.0);
        alpha[ilast - 1] = QA(ilast, ilast);
        beta[ilast - 1] = QB(ilast, ilast);
        sh.ilast = ilast - 1;
        if (sh.ilast < ilo) sh.done = 1;
        sh.shiftcount = 0;
        sh.eshift = make_double2(0.0, 0.0);
      }
      __syncthreads();
      if (sh.done) break;
      continue;
    }
    // ---- QZ step on ifirst:ilast (generalized.jl:339-449) ----
    if (tid == 0) {
      const int ifirst = sh.ifirst;
      sh.shiftcount += 1;
      double2 shift;
      if (sh.shiftcount % 10 != 0) {
        const double2 b11 = zmulr(QB(ilast - 1, ilast - 1), bscale);
        const double2 b22 = zmulr(QB(ilast, ilast), bscale);
        const double2 u12 = zdiv(zmulr(QB(ilast - 1, ilast), bscale), b22);
        const double2 ad11 = zdiv(zmulr(QA(ilast - 1, ilast - 1), ascale), b11);
        const double2 ad21 = zdiv(zmulr(QA(ilast, ilast - 1), ascale), b11);
        const double2 ad12 = zdiv(zmulr(QA(ilast - 1, ilast), ascale), b22);
        const double2 ad22 = zdiv(zmulr(QA(ilast, ilast), ascale), b22);
        const double2 abi22 = zsub(ad22, zmul(u12, ad21));
        const double2 abi12 = zsub(ad12, zmul(u12, ad11));
        shift = abi22;
        const double2 t = zmul(zsqrt(abi12), zsqrt(ad21));
        double t1 = zabs1(t);
        if (!zis0(t)) {
          const double2 x = zmulr(zsub(ad11, shift), 0.5);
          const double t2 = zabs1(x);
          t1 = fmax(t1, t2);
          const double2 xt = make_double2(x.x / t1, x.y / t1), tt = make_double2(t.x / t1, t.y / t1);
          double2 y = zmulr(zsqrt(zadd(zmul(xt, xt), zmul(tt, tt))), t1);
          if (t2 > 0.0) {
            const double2 xs = make_double2(x.x / t2, x.y / t2);
            if (xs.x * y.x + xs.y * y.y < 0.0) y = make_double2(-y.x, -y.y);
          }
          shift = zsub(shift, zmul(t, zdiv(t, zadd(x, y))));
        }
      } else {
        if (sh.shiftcount % 20 == 0 && bscale * zabs1(QB(ilast, ilast)) > safmin)
          sh.eshift = zadd(sh.eshift, zdiv(zmulr(QA(ilast, ilast), ascale), zmulr(QB(ilast, ilast), bscale)));
        else
          sh.eshift = zadd(sh.eshift, zdiv(zmulr(QA(ilast, ilast - 1), ascale), zmulr(QB(ilast - 1, ilast - 1), bscale)));
        shift = sh.eshift;
      }
      double2 f1 = make_double2(1.0, 0.0);
      int istart = -1;
      bool gotit = false;
      for (int j = ilast - 1; j >= ifirst + 1; --j) {
        istart = j;
        f1 = zsub(zmulr(QA(j, j), ascale), zmul(shift, zmulr(QB(j, j), bscale)));
        double t1 = zabs1(f1);
        double t2 = ascale * zabs1(QA(j + 1, j));
        const double tr = fmax(t1, t2);
        if (tr < 1.0 && tr != 0.0) { t1 /= tr; t2 /= tr; }
        if (zabs1(QA(j, j - 1)) * t2 <= t1 * atol) { gotit = true; break; }
      }
      if (!gotit) {
        istart = ifirst;
        f1 = zsub(zmulr(QA(ifirst, ifirst), ascale), zmul(shift, zmulr(QB(ifirst, ifirst), bscale)));
      }
      const double2 g2 = zmulr(QA(istart + 1, istart), ascale);
      double c;
      double2 s, r;
      zgivens(f1, g2, c, s, r);
      sh.c = c; sh.s = s;
      sh.istart = istart;
    }
    __syncthreads();
    const int istart = sh.istart;
    for (int j = istart; j <= ilast - 1; ++j) {
      if (j > istart) {
        if (tid == 0) {
          double c;
          double2 s, r;
          zgivens(QA(j, j - 1), QA(j + 1, j - 1), c, s, r);
          QA(j, j - 1) = r;
          QA(j + 1, j - 1) = make_double2(0.0, 0.0);
          sh.c = c; sh.s = s;
        }
        __syncthreads();
      }
      {
        const double c = sh.c;
        const double2 s = sh.s;
        rot_rows(m.A, n, j, j + 1, c, s, j, n);
        rot_rows(m.B, n, j, j + 1, c, s, j, n);
        if (m.Q) rot_cols_adj(m.Q, n, j, j + 1, c, s, 1, n);
      }
      __syncthreads();
      if (tid == 0) {
        double c;
        double2 s, r;
        zgivens(QB(j + 1, j + 1), QB(j + 1, j), c, s, r);
        QB(j + 1, j + 1) = r;
        QB(j + 1, j) = make_double2(0.0, 0.0);
        sh.c = c; sh.s = s;
      }
      __syncthreads();
      {
        const double c = sh.c;
        const double2 s = sh.s;
        rot_cols(m.A, n, j, j + 1, c, s, 1, min(j + 2, ilast));
        rot_cols(m.B, n, j, j + 1, c, s, 1, j);
        if (m.Z) rot_cols(m.Z, n, j, j + 1, c, s, 1, n);
      }
      __syncthreads();
    }
  }
  return sh.status;
}

__global__ void __launch_bounds__(kQzT) k_ggschur(QzBatch bt) {
  __shared__ double red[kQzT / 32];
  __shared__ QzShared sh;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int b = blockIdx.x; b < bt.count; b += gridDim.x) {
    const int n = bt.ns ? bt.ns[b] : bt.n1;
    const long long off = bt.ns ? bt.offs[b] : 0, woff = bt.ns ? bt.woffs[b] : 0;
    QzMats m{bt.A + off, bt.B + off, bt.Q ? bt.Q + off : nullptr, bt.Z ? bt.Z + off : nullptr, n};
    double2* alpha = bt.alpha + woff;
    double2* beta = bt.beta + woff;
    if (n == 0) {
      if (tid == 0 && bt.status) bt.status[b] = 0;
      continue;
    }
    // _scale! both (generalized.jl:35-44)
    double cscale = 1.0, anrm = 1.0, cscaleb = 1.0, bnrm = 1.0;
    bool scA = false, scB = false;
    if (bt.scale) {
      scA = cta_scale(m.A, n, red, cscale, anrm);
      scB = cta_scale(m.B, n, red, cscaleb, bnrm);
    }
    // qr!(B), A <- Q^H A (Householder, real R diagonal); tau in alpha (scratch)
    for (int j = 1; j <= n; ++j) {
      const int len = n - j + 1;
      double2* v = m.B + (j - 1) + (size_t)(j - 1) * n;
      const double2 t = cta_reflector<kQzT>(v, len, red);
      if (tid == 0) alpha[j - 1] = t;
      __syncthreads();
      if (!zis0(t)) {
        const double2 ct = zconj(t);
        // columns j+1..n of B and 1..n of A: x <- x - conj(t) v (v^H x), warp per column
        for (int col = wid; col < (n - j) + n; col += kQzT / 32) {
          double2* x = col < n - j ? m.B + (j - 1) + (size_t)(j + col) * n : m.A + (j - 1) + (size_t)(col - (n - j)) * n;
          double2 sacc = make_double2(0.0, 0.0);
          for (int r = lane; r < len; r += 32) sacc = zfmac(r == 0 ? make_double2(1.0, 0.0) : v[r], x[r], sacc);
          for (int o = 16; o > 0; o >>= 1)
            sacc = zadd(sacc, make_double2(__shfl_xor_sync(0xffffffffu, sacc.x, o), __shfl_xor_sync(0xffffffffu, sacc.y, o)));
          const double2 ts = zmul(ct, sacc);
          for (int r = lane; r < len; r += 32) x[r] = zsub(x[r], zmul(ts, r == 0 ? make_double2(1.0, 0.0) : v[r]));
        }
      }
      __syncthreads();
    }
    // Q = H_1 ... H_n (backwards into the identity), warp per column
    if (m.Q) {
      for (size_t e = tid; e < (size_t)n * n; e += kQzT)
        m.Q[e] = make_double2((e % n) == (e / n) ? 1.0 : 0.0, 0.0);
      __syncthreads();
      for (int j = n; j >= 1; --j) {
        const double2 t = alpha[j - 1];
        const int len = n - j + 1;
        const double2* v = m.B + (j - 1) + (size_t)(j - 1) * n;
        if (!zis0(t)) {
          for (int col = j + wid; col <= n; col += kQzT / 32) {
            double2* x = m.Q + (j - 1) + (size_t)(col - 1) * n;
            double2 sacc = make_double2(0.0, 0.0);
            for (int r = lane; r < len; r += 32) sacc = zfmac(r == 0 ? make_double2(1.0, 0.0) : v[r], x[r], sacc);
            for (int o = 16; o > 0; o >>= 1)
              sacc = zadd(sacc, make_double2(__shfl_xor_sync(0xffffffffu, sacc.x, o), __shfl_xor_sync(0xffffffffu, sacc.y, o)));
            const double2 ts = zmul(t, sacc);
            for (int r = lane; r < len; r += 32) x[r] = zsub(x[r], zmul(ts, r == 0 ? make_double2(1.0, 0.0) : v[r]));
          }
        }
        __syncthreads();
      }
    }
    // R = triu(B); Z = I
    for (size_t e = tid; e < (size_t)n * n; e += kQzT) {
      if ((e % n) > (e / n)) m.B[e] = make_double2(0.0, 0.0);
      if (m.Z) m.Z[e] = make_double2((e % n) == (e / n) ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    // _hessenberg!(A, B, Q, Z) (zgghrd): rows jr-1, jr null A[jr, jc]; columns jr, jr-1
    // null B[jr, jr-1]
    for (int jc = 1; jc <= n - 2; ++jc)
      for (int jr = n; jr >= jc + 2; --jr) {
        if (tid == 0) {
          double c;
          double2 s, r;
          zgivens(QA(jr - 1, jc), QA(jr, jc), c, s, r);
          sh.c = c; sh.s = s;
        }
        __syncthreads();
        {
          const double c = sh.c;
          const double2 s = sh.s;
          rot_rows(m.A, n, jr - 1, jr, c, s, 1, n);
          rot_rows(m.B, n, jr - 1, jr, c, s, 1, n);
          if (m.Q) rot_cols_adj(m.Q, n, jr - 1, jr, c, s, 1, n);
        }
        __syncthreads();
        if (tid == 0) {
          double c;
          double2 s, r;
          zgivens(zconj(QB(jr, jr)), zconj(QB(jr, jr - 1)), c, s, r);
          sh.c = c; sh.s = s;
        }
        __syncthreads();
        {
          const double c = sh.c;
          const double2 s = sh.s;
          rot_cols_adj(m.A, n, jr, jr - 1, c, s, 1, n);
          rot_cols_adj(m.B, n, jr, jr - 1, c, s, 1, n);
          if (m.Z) rot_cols_adj(m.Z, n, jr, jr - 1, c, s, 1, n);
        }
        __syncthreads();
      }
    for (size_t e = tid; e < (size_t)n * n; e += kQzT) {
      const int i = (int)(e % n), j = (int)(e / n);
      if (i > j + 1) m.A[e] = make_double2(0.0, 0.0);
      if (i > j) m.B[e] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    const int st = qz_iterate(m, alpha, beta, 100LL * n, red, sh);
    __syncthreads();
    if (scA) {
      cta_safescale(m.A, n, cscale, anrm);
      for (int i = tid; i < n; i += kQzT) alpha[i] = m.A[i + (size_t)i * n];
    }
    if (scB) {
      cta_safescale(m.B, n, cscaleb, bnrm);
      for (int i = tid; i < n; i += kQzT) beta[i] = m.B[i + (size_t)i * n];
    }
    if (tid == 0 && bt.status) bt.status[b] = st;
    __syncthreads();
  }
}

// ---- gordschur!(S, T, Q, Z, select) for a complex generalized Schur form (ordschur.jl:
// 147-305): selected eigenvalues move to the top in their order by adjacent swaps
// (_trexch2!, ztgex2 with the weak and strong stability tests).  One CTA: every thread
// computes the swap's 2 x 2 rotations from the same entries (identical decisions), the
// rotations of rows and columns of S, T, Q, Z are split over the CTA.

// _safe_fnorm of 8 complex numbers (util.jl:83-94, _ssq 466-505: the scale starts at 1).
__device__ double safe_fnorm8(const double2* w) {
  double scale = 1.0, sumsq = 0.0;
  for (int i = 0; i < 8; ++i) {
    const double parts[2] = {fabs(w[i].x), fabs(w[i].y)};
    for (int q = 0; q < 2; ++q) {
      const double t1 = parts[q];
      if (t1 > 0.0 || t1 != t1) {
        if (scale < t1) { const double r = scale / t1; sumsq = 1.0 + sumsq * r * r; scale = t1; }
        else { const double r = t1 / scale; sumsq += r * r; }
      }
    }
  }
  return scale * sqrt(sumsq);
}

// rmul!(M2x2, Givens(1, 2, c, s)) / lmul!(Givens(1, 2, c, s), M2x2) on a column-major 2 x 2
__device__ __forceinline__ void rz2(double2* M, double c, double2 sv) {
  for (int r = 0; r < 2; ++r) {
    const double2 m1 = M[r], m2 = M[r + 2];
    M[r] = zsub(zmulr(m1, c), zmul(m2, zconj(sv)));
    M[r + 2] = zadd(zmul(m1, sv), zmulr(m2, c));
  }
}
__device__ __forceinline__ void lq2(double2* M, double c, double2 sv) {
  for (int k = 0; k < 2; ++k) {
    const double2 m1 = M[2 * k], m2 = M[2 * k + 1];
    M[2 * k] = zadd(zmulr(m1, c), zmul(sv, m2));
    M[2 * k + 1] = zsub(zmulr(m2, c), zmul(zconj(sv), m1));
  }
}

// One adjacent swap at j1 (1-based); false if a stability test rejects it.  All threads
// call it; the caller synchronises before (entries read) and it synchronises after.
__device__ bool trexch2_cplx(const QzMats& m, int j1) {
  const int n = m.n, tid = threadIdx.x;
  double2 S[4] = {QA(j1, j1), QA(j1 + 1, j1), QA(j1, j1 + 1), QA(j1 + 1, j1 + 1)};
  double2 T[4] = {QB(j1, j1), QB(j1 + 1, j1), QB(j1, j1 + 1), QB(j1 + 1, j1 + 1)};
  const double2 orig[8] = {S[0], S[1], S[2], S[3], T[0], T[1], T[2], T[3]};
  const double eps = Prec<double>::eps;
  const double smlnum = Prec<double>::fmin / eps;
  double sa = safe_fnorm8(orig);
  const double thresh = fmax(20.0 * eps * sa, smlnum);
  const double2 f = zsub(zmul(S[3], T[0]), zmul(T[3], S[0]));
  const double2 g = zsub(zmul(S[3], T[2]), zmul(T[3], S[2]));
  sa = zabs(S[3]) * zabs(T[0]);
  const double sb = zabs(S[0]) * zabs(T[3]);
  double cz;
  double2 sz, r;
  if (zis0(f) && zis0(g)) { cz = 0.0; sz = make_double2(1.0, 0.0); }
  else zgivens(g, f, cz, sz, r);
  rz2(S, cz, sz);
  rz2(T, cz, sz);
  double2 fq, gq;
  if (sa >= sb) { fq = S[0]; gq = S[1]; } else { fq = T[0]; gq = T[1]; }
  double cq;
  double2 sq;
  if (!zis0(sz) && zis0(fq) && zis0(gq)) { cq = 0.0; sq = make_double2(1.0, 0.0); }
  else zgivens(fq, gq, cq, sq, r);
  lq2(S, cq, sq);
  lq2(T, cq, sq);
  const double ws = zabs(S[1]) + zabs(T[1]);
  if (!(ws <= thresh)) return false;
  double2 Ss[4] = {S[0], S[1], S[2], S[3]}, Ts[4] = {T[0], T[1], T[2], T[3]};
  rz2(Ss, cz, zneg(sz));
  rz2(Ts, cz, zneg(sz));
  lq2(Ss, cq, zneg(sq));
  lq2(Ts, cq, zneg(sq));
  double2 W[8];
  for (int k = 0; k < 4; ++k) { W[k] = zsub(Ss[k], orig[k]); W[4 + k] = zsub(Ts[k], orig[4 + k]); }
  if (!(safe_fnorm8(W) <= thresh)) return false;
  __syncthreads();
  // columns j1, j1+1 of A, B, Z (rmul! by Gz') and of Q (rmul! by Gq'), all rows
  for (int i = tid; i < 4 * n; i += kQzT) {
    const int which = i / n, rr = i % n;
    double2* M = which == 0 ? m.A : which == 1 ? m.B : which == 2 ? m.Z : m.Q;
    if (!M) continue;
    double2* c1 = M + rr + (size_t)(j1 - 1) * n;
    double2* c2 = M + rr + (size_t)j1 * n;
    const double2 m1 = *c1, m2 = *c2;
    if (which < 3) {
      *c1 = zsub(zmulr(m1, cz), zmul(m2, zconj(sz)));
      *c2 = zadd(zmul(m1, sz), zmulr(m2, cz));
    } else {
      *c1 = zadd(zmulr(m1, cq), zmul(m2, zconj(sq)));
      *c2 = zsub(zmulr(m2, cq), zmul(m1, sq));
    }
  }
  __syncthreads();
  // rows j1, j1+1 of A and B (lmul! by Gq), all columns
  for (int i = tid; i < 2 * n; i += kQzT) {
    double2* M = i < n ? m.A : m.B;
    const int cc = i % n;
    double2* r1 = M + (j1 - 1) + (size_t)cc * n;
    double2* r2 = M + j1 + (size_t)cc * n;
    const double2 m1 = *r1, m2 = *r2;
    *r1 = zadd(zmulr(m1, cq), zmul(sq, m2));
    *r2 = zsub(zmulr(m2, cq), zmul(zconj(sq), m1));
  }
  __syncthreads();
  if (tid == 0) {
    QA(j1 + 1, j1) = make_double2(0.0, 0.0);
    QB(j1 + 1, j1) = make_double2(0.0, 0.0);
  }
  __syncthreads();
  return true;
}

__global__ void __launch_bounds__(kQzT) k_ggordschur_cplx(QzMats m, const int* __restrict__ select, int scale,
                                                          double2* alpha, double2* beta, int* status) {
  __shared__ double red[kQzT / 32];
  const int n = m.n, tid = threadIdx.x;
  double cscale = 1.0, anrm = 1.0, cscaleb = 1.0, bnrm = 1.0;
  bool scA = false, scB = false;
  if (scale) {
    scA = cta_scale(m.A, n, red, cscale, anrm);
    scB = cta_scale(m.B, n, red, cscaleb, bnrm);
  }
  __syncthreads();
  int st = 0;
  int ks = 0;
  for (int k = 1; k <= n && !st; ++k) {
    if (!select[k - 1]) continue;
    ks += 1;
    if (k != ks)
      for (int icur = k - 1; icur >= ks; --icur) {
        __syncthreads();
        if (!trexch2_cplx(m, icur)) { st = 1 + icur; break; }
      }
  }
  __syncthreads();
  if (scA) cta_safescale(m.A, n, cscale, anrm);
  if (scB) cta_safescale(m.B, n, cscaleb, bnrm);
  for (size_t e = tid; e < (size_t)n * n; e += kQzT) {
    const int i = (int)(e % n), j = (int)(e / n);
    if (i > j) { m.A[e] = make_double2(0.0, 0.0); m.B[e] = make_double2(0.0, 0.0); }
  }
  __syncthreads();
  for (int i = tid; i < n; i += kQzT) {
    alpha[i] = m.A[i + (size_t)i * n];
    beta[i] = m.B[i + (size_t)i * n];
  }
  if (tid == 0) *status = st;
}

#undef QA
#undef QB

}  // namespace

cudaError_t launch_ggordschur_cplx(int n, double2* S, double2* T, double2* Q, double2* Z, const int* select, int scale,
                                   double2* alpha, double2* beta, int* status, cudaStream_t s) {
  QzMats m{S, T, Q, Z, n};
  k_ggordschur_cplx<<<1, kQzT, 0, s>>>(m, select, scale, alpha, beta, status);
  return cudaGetLastError();
}

cudaError_t launch_ggschur(const QzBatch& bt, int num_sms, cudaStream_t s) {
  if (bt.count <= 0) return cudaSuccess;
  const int grid = std::min(bt.count, 8 * num_sms);
  k_ggschur<<<grid, kQzT, 0, s>>>(bt);
  return cudaGetLastError();
}

}  // namespace gsk
