// Eigenvectors of a real generalized Schur pair (S quasi-triangular, P upper triangular):
// the reference's dtgevc restatements in complex arithmetic, _geigvecs (right,
// vectors.jl:1040-1283) and _gleigvecs (left, vectors.jl:1285-1513), with _xsolve
// (util.jl:698-751) on the 1 x 1 and 2 x 2 diagonal blocks and _ggs_2x2 (dlag2) for the
// coefficients of a complex pair.  A complex pair's second column is the conjugate of the
// first, as in the reference.
//
// One thread per real eigenvalue or complex pair (the other row of a pair idles), CTAs over
// blocks of 64 eigenvalues.  All threads of a CTA walk the diagonal blocks in the same order
// (block boundaries come from S alone, so they agree), reading S and P as broadcasts; a
// thread whose eigenvector does not involve a block is masked.  Partial solutions live in
// a scratch array with one row per index (coalesced).
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kRgT = 64;
constexpr double kSafety = 100.0;

#define SS(i, j) S[((i) - 1) + (size_t)((j) - 1) * n]
#define PP(i, j) P[((i) - 1) + (size_t)((j) - 1) * n]
#define XX(i) X[(size_t)((i) - 1) * n + col]

__global__ void k_rg_norms(int n, const double* __restrict__ S, const double* __restrict__ P, double* __restrict__ sn,
                           double* __restrict__ pn, unsigned long long* __restrict__ ab) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > n) return;
  double s = 0.0, p = 0.0;
  for (int i = 1; i <= j - 1; ++i) {
    s += fabs(SS(i, j));
    p += fabs(PP(i, j));
  }
  sn[j - 1] = s;
  pn[j - 1] = p;
  const double a = (j == 1) ? fabs(SS(1, 1)) : s + fabs(SS(j, j));
  const double b = (j == 1) ? fabs(PP(1, 1)) : p + fabs(PP(j, j));
  atomicMax(ab, (unsigned long long)__double_as_longlong(a));
  atomicMax(ab + 1, (unsigned long long)__double_as_longlong(b));
}

// dlag2 (rgeneralized.jl:810-948) on the 2 x 2 pencil at (i, i); only scale1, wr1, wi.
__device__ void rg_ggs2x2(const double* S, const double* P, int n, int i, double safmin, double& scale1, double& wr1,
                          double& wi) {
  const double rtmin = sqrt(safmin), rtmax = 1.0 / rtmin, safmax = 1.0 / safmin;
  const double fuzzy1 = 1.0 + sqrt(sqrt(kEps)) / 10.0;
  const double A11 = SS(i, i), A21 = SS(i + 1, i), A12 = SS(i, i + 1), A22 = SS(i + 1, i + 1);
  const double anorm = fmax(fmax(fabs(A11) + fabs(A21), fabs(A12) + fabs(A22)), safmin);
  const double ascale = 1.0 / anorm;
  const double a11 = ascale * A11, a12 = ascale * A12, a21 = ascale * A21, a22 = ascale * A22;
  double b11 = PP(i, i), b12 = PP(i, i + 1), b22 = PP(i + 1, i + 1);
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
    wr1 = (pp > abi22) ? fmin(wbig, wsmall) : fmax(wbig, wsmall);
    wi = 0.0;
  } else {
    wr1 = shift + pp;
    wi = r;
  }
  const double c1 = bsize * (safmin * fmax(1.0, ascale));
  const double c2 = safmin * fmax(1.0, bnorm);
  const double c3 = bsize * safmin;
  const double c4 = (ascale <= 1.0 && bsize <= 1.0) ? fmin(1.0, (ascale / safmin) * bsize) : 1.0;
  const double c5 = (ascale <= 1.0 || bsize <= 1.0) ? fmin(1.0, ascale * bsize) : 1.0;
  const double wabs = fabs(wr1) + fabs(wi);
  const double wsize = fmax(fmax(safmin, c1), fmax(fuzzy1 * (wabs * c2 + c3), fmin(c4, fmax(wabs, c5) / 2.0)));
  if (wsize != 1.0) {
    const double wscale = 1.0 / wsize;
    if (wsize > 1.0) scale1 = (fmax(ascale, bsize) * wscale) * fmin(ascale, bsize);
    else scale1 = (fmin(ascale, bsize) * wscale) * fmax(ascale, bsize);
    wr1 *= wscale;
    if (wi != 0.0) wi *= wscale;
  } else {
    scale1 = ascale * bsize;
  }
}

// 2-norm of two complex numbers without overflow.
__device__ __forceinline__ double znorm2(double2 a, double2 b) {
  const double m = fmax(fmax(fabs(a.x), fabs(a.y)), fmax(fabs(b.x), fabs(b.y)));
  if (!(m > 0.0) || !isfinite(m)) return m;
  const double p = a.x / m, q = a.y / m, r = b.x / m, s = b.y / m;
  return m * sqrt(p * p + q * q + r * r + s * s);
}

// _safe_lu_solve! (util.jl:603-690) of a complex 2 x 2 system m (column-major), in place on b.
__device__ double safe_lu2(double2 m[4], double2 b[2]) {
  const double smallnum = Prec<double>::fmin / kEps;
  double smin = 0.0;
  for (int e = 0; e < 4; ++e) smin = fmax(smin, zabs(m[e]));
  smin = fmax(kEps * smin, smallnum);
  // complete pivoting for i = 1
  double xmax = 0.0;
  int ipsv = 1, jpsv = 1;
  for (int ip = 1; ip <= 2; ++ip)
    for (int jp = 1; jp <= 2; ++jp) {
      const double v = zabs(m[(ip - 1) + (jp - 1) * 2]);
      if (v >= xmax) { xmax = v; ipsv = ip; jpsv = jp; }
    }
  if (ipsv != 1) {
    for (int j = 0; j < 2; ++j) { const double2 t = m[1 + j * 2]; m[1 + j * 2] = m[0 + j * 2]; m[0 + j * 2] = t; }
    const double2 t = b[0]; b[0] = b[1]; b[1] = t;
  }
  if (jpsv != 1)
    for (int i = 0; i < 2; ++i) { const double2 t = m[i + 2]; m[i + 2] = m[i]; m[i] = t; }
  if (zabs(m[0]) < smin) m[0] = make_double2(smin, 0.0);
  m[1] = zdiv(m[1], m[0]);
  b[1] = zsub(b[1], zmul(m[1], b[0]));
  m[3] = zsub(m[3], zmul(m[1], m[2]));
  if (zabs(m[3]) < smin) m[3] = make_double2(smin, 0.0);
  double scale = 1.0;
  const double aa = 8.0 * smallnum;
  if (aa * zabs(b[0]) > zabs(m[0]) || aa * zabs(b[1]) > zabs(m[3])) {
    const double bmax = fmax(zabs(b[0]), zabs(b[1]));
    scale = (1.0 / 8.0) / bmax;
    b[0] = zscal(b[0], scale);
    b[1] = zscal(b[1], scale);
  }
  // back substitution, k = 2 then 1
  {
    const double2 t = zdiv(make_double2(1.0, 0.0), m[3]);
    b[1] = zmul(b[1], t);
  }
  {
    const double2 t = zdiv(make_double2(1.0, 0.0), m[0]);
    b[0] = zmul(b[0], t);
    b[0] = zsub(b[0], zmul(zmul(t, m[2]), b[1]));
  }
  if (jpsv != 1) { const double2 t = b[0]; b[0] = b[1]; b[1] = t; }
  return scale;
}

// _xsolve(a, A, d, b, B, smin) (util.jl:698-751) for na = 1, 2; A column-major na x na.
__device__ double xsolve_gen(double a, const double* A, int na, const double* d, double2 b, double2 B[2], double smin,
                             double& xnorm) {
  double s = 1.0;
  const double small = 2.0 * kSafemin;
  const double bignum = s / small;
  smin = fmax(smin, small);
  if (na == 1) {
    double csr = a * A[0] - b.x * d[0];
    double csi = -b.y * d[0];
    double cnorm = fabs(csr) + fabs(csi);
    if (cnorm < smin) { csr = smin; csi = 0.0; cnorm = smin; }
    const double bnorm = zabs1(B[0]);
    if (cnorm < 1.0 && bnorm > 1.0 && bnorm > bignum * cnorm) s = 1.0 / bnorm;
    const double2 x = zdiv(zscal(B[0], s), make_double2(csr, csi));
    xnorm = zabs1(x);
    B[0] = x;
    return s;
  }
  double2 m[4];
  double cmax = 0.0;
  for (int j = 1; j <= 2; ++j)
    for (int i = 1; i <= 2; ++i) {
      double2 z = make_double2(a * A[(i - 1) + (j - 1) * 2], 0.0);
      if (i == j) z = zsub(z, zscal(b, d[i - 1]));
      m[(i - 1) + (j - 1) * 2] = z;
      cmax = fmax(cmax, zabs1(z));
    }
  if (cmax < smin) {
    const double bnorm = fmax(zabs1(B[0]), zabs1(B[1]));
    if (smin < 1.0 && bnorm > 1.0 && bnorm > bignum * smin) s = 1.0 / bnorm;
    const double t1 = s / smin;
    B[0] = zscal(B[0], t1);
    B[1] = zscal(B[1], t1);
  } else {
    s = safe_lu2(m, B);
  }
  xnorm = znorm2(B[0], B[1]);
  return s;
}

struct RgCoef {
  double a, br, bi, aa, ba, xmax;
  int role;  // 0 idle (other row of a pair), 1 real eigenvalue, 2 complex pair, 3 singular
};

// vectors.jl:1097-1139 (real) and 1147-1183 (pair); right = pair rows (k-1, k), left = (k, k+1).
__device__ RgCoef rg_setup(const double* S, const double* P, int n, int k, double Anorm, double Bnorm, bool left) {
  const double ulp = kEps, safmin = kSafemin;
  const double smallnum = safmin * ((double)n / ulp);
  const double bigx = 1.0 / smallnum;
  const double ascale = 1.0 / fmax(Anorm, safmin), bscale = 1.0 / fmax(Bnorm, safmin);
  RgCoef c;
  c.a = c.br = c.bi = c.aa = c.ba = 0.0;
  c.xmax = 1.0;
  const bool pair_here = left ? (k < n && SS(k + 1, k) != 0.0) : (k > 1 && SS(k, k - 1) != 0.0);
  const bool other_row = left ? (k > 1 && SS(k, k - 1) != 0.0) : (k < n && SS(k + 1, k) != 0.0);
  if (other_row && !pair_here) { c.role = 0; return c; }
  if (!pair_here) {
    if (fabs(SS(k, k)) <= safmin && fabs(PP(k, k)) <= safmin) { c.role = 3; return c; }
    const double skk = SS(k, k), pkk = PP(k, k);
    const double t = 1.0 / fmax(fmax(fabs(skk) * ascale, fabs(pkk) * bscale), safmin);
    const double sar = (t * skk) * ascale, sb = (t * pkk) * bscale;
    double a = sb * ascale, br = sar * bscale;
    const bool lsa = fabs(sb) >= safmin && fabs(a) < smallnum;
    const bool lsb = fabs(sar) >= safmin && fabs(br) < smallnum;
    double s = 1.0;
    if (lsa) s = (smallnum / fabs(sb)) * fmin(Anorm, bigx);
    if (lsb) s = fmax(s, (smallnum / fabs(sar)) * fmin(Bnorm, bigx));
    if (lsa || lsb) {
      s = fmin(s, 1.0 / (safmin * fmax(fmax(1.0, fabs(a)), fabs(br))));
      a = lsa ? ascale * (s * sb) : a * s;
      br = lsb ? bscale * (s * sar) : br * s;
    }
    c.a = a; c.br = br; c.bi = 0.0;
    c.aa = fabs(a); c.ba = fabs(br);
    c.role = 1;
    return c;
  }
  double s1, wr1, wi;
  rg_ggs2x2(S, P, n, left ? k : k - 1, safmin * kSafety, s1, wr1, wi);
  double a = s1, br = wr1, bi = left ? -wi : wi;
  {
    const double aa = fabs(a), ba = fabs(br) + fabs(bi);
    double scale = 1.0;
    if (aa * ulp < safmin && aa >= safmin) scale = (safmin / ulp) / aa;
    if (ba * ulp < safmin && ba >= safmin) scale = fmax(scale, (safmin / ulp) / ba);
    if (safmin * aa > ascale) scale = ascale / (safmin * aa);
    if (safmin * ba > bscale) scale = fmin(scale, bscale / (safmin * ba));
    if (scale != 1.0) { a *= scale; br *= scale; bi *= scale; }
  }
  c.a = a; c.br = br; c.bi = bi;
  c.aa = fabs(a); c.ba = fabs(br) + fabs(bi);
  c.role = 2;
  return c;
}

__global__ void __launch_bounds__(kRgT) k_rgevc_right(int n, const double* __restrict__ S, const double* __restrict__ P,
                                                     const double* __restrict__ sn, const double* __restrict__ pn,
                                                     const unsigned long long* __restrict__ ab,
                                                     double2* __restrict__ X, double* __restrict__ xm,
                                                     int* __restrict__ role) {
  const int col = blockIdx.x * kRgT + threadIdx.x;
  const int je = col + 1;
  const bool live_t = col < n;
  const double Anorm = __longlong_as_double((long long)ab[0]), Bnorm = __longlong_as_double((long long)ab[1]);
  const double ulp = kEps, safmin = kSafemin;
  const double bignum = 1.0 / ((double)n * safmin);
  RgCoef c;
  c.role = 0;
  c.a = c.br = c.bi = c.aa = c.ba = 0.0;
  c.xmax = 1.0;
  if (live_t) c = rg_setup(S, P, n, je, Anorm, Bnorm, false);
  if (live_t) role[col] = c.role;
  const bool act = live_t && (c.role == 1 || c.role == 2);
  const int nw = c.role == 2 ? 2 : 1;
  const double2 bc = make_double2(c.br, c.bi);
  double xmax = 1.0;
  if (act) {
    for (int i = 1; i <= n; ++i) XX(i) = make_double2(0.0, 0.0);
    if (c.role == 1) {
      XX(je) = make_double2(1.0, 0.0);
      for (int jr = 1; jr <= je - 1; ++jr) XX(jr) = make_double2(c.br * PP(jr, je) - c.a * SS(jr, je), 0.0);
    } else {
      double t1 = c.a * SS(je, je - 1);
      const double t2r = c.a * SS(je, je) - c.br * PP(je, je), t2i = -c.bi * PP(je, je);
      double2 vj, vjm;
      if (fabs(t1) > fabs(t2r) + fabs(t2i)) {
        vj = make_double2(1.0, 0.0);
        vjm = zdiv(make_double2(-t2r, -t2i), make_double2(t1, 0.0));
      } else {
        vjm = make_double2(1.0, 0.0);
        t1 = c.a * SS(je - 1, je);
        vj = make_double2((c.br * PP(je - 1, je - 1) - c.a * SS(je - 1, je - 1)) / t1, c.bi * PP(je - 1, je - 1) / t1);
      }
      XX(je) = vj;
      XX(je - 1) = vjm;
      xmax = fmax(zabs1(vj), zabs1(vjm));
      const double2 ca = zscal(vjm, c.a), cb = zmul(bc, vjm), c2a = zscal(vj, c.a), c2b = zmul(bc, vj);
      for (int jr = 1; jr <= je - 2; ++jr) {
        double2 v = zscal(ca, -SS(jr, je - 1));
        v = zadd(v, zscal(cb, PP(jr, je - 1)));
        v = zsub(v, zscal(c2a, SS(jr, je)));
        v = zadd(v, zscal(c2b, PP(jr, je)));
        XX(jr) = v;
      }
    }
  }
  const double dmin = fmax(fmax(ulp * c.aa * Anorm, ulp * c.ba * Bnorm), safmin);
  const int j0 = je - nw;  // the thread's first block ends at row j0
  // lockstep over the diagonal blocks from the CTA's largest starting row down
  int jb = min(n, (int)(blockIdx.x + 1) * kRgT) - 1;
  while (jb >= 1) {
    const bool two = jb > 1 && SS(jb, jb - 1) != 0.0;
    const int na = two ? 2 : 1;
    const int jt = jb - na + 1;  // top row of the block
    const bool on = act && jb <= j0;
    double t1 = 0.0;
    double2 x[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    if (on) {
      double blk[4], dg[2];
      for (int q = 0; q < na; ++q) {
        dg[q] = PP(jt + q, jt + q);
        for (int p = 0; p < na; ++p) blk[p + q * na] = SS(jt + p, jt + q);
      }
      x[0] = XX(jt);
      if (na == 2) x[1] = XX(jt + 1);
      const double scale = xsolve_gen(c.a, blk, na, dg, bc, x, dmin, t1);
      // the reference's _xsolve overwrites a view of v, so the rescaling of v[1:je] that
      // follows also applies to the new solution entries (vectors.jl:1229-1236)
      XX(jt) = x[0];
      if (na == 2) XX(jt + 1) = x[1];
      if (scale < 1.0)
        for (int r = 1; r <= je; ++r) XX(r) = zscal(XX(r), scale);
      xmax = fmax(scale * xmax, t1);
      if (jt > 1) {
        const double xscale = 1.0 / fmax(1.0, xmax);
        t1 = fmax(t1, c.aa * sn[jt - 1] + c.ba * pn[jt - 1]);
        if (na == 2) t1 = fmax(t1, c.aa * sn[jt] + c.ba * pn[jt]);
        t1 = fmax(fmax(t1, c.aa), c.ba);
        if (t1 > bignum * xscale) {
          for (int r = 1; r <= je; ++r) XX(r) = zscal(XX(r), xscale);
          xmax *= xscale;
        }
      }
      x[0] = XX(jt);
      if (na == 2) x[1] = XX(jt + 1);
    }
    if (jt > 1) {
      for (int ja = 0; ja < na; ++ja) {
        double2 ca = make_double2(0.0, 0.0), cb = ca;
        if (on) {
          ca = zscal(x[ja], c.a);
          cb = zmul(bc, x[ja]);
        }
        for (int i = 1; i <= jt - 1; ++i) {
          const double s = SS(i, jt + ja), p = PP(i, jt + ja);
          if (on) XX(i) = zadd(zsub(XX(i), zscal(ca, s)), zscal(cb, p));
        }
      }
    }
    jb = jt - 1;
  }
  if (live_t) xm[col] = xmax;
}

__global__ void __launch_bounds__(kRgT) k_rgevc_left(int n, const double* __restrict__ S, const double* __restrict__ P,
                                                    const double* __restrict__ sn, const double* __restrict__ pn,
                                                    const unsigned long long* __restrict__ ab,
                                                    double2* __restrict__ X, double* __restrict__ xm,
                                                    int* __restrict__ role) {
  const int col = blockIdx.x * kRgT + threadIdx.x;
  const int je = col + 1;
  const bool live_t = col < n;
  const double Anorm = __longlong_as_double((long long)ab[0]), Bnorm = __longlong_as_double((long long)ab[1]);
  const double ulp = kEps, safmin = kSafemin;
  const double bignum = 1.0 / ((double)n * safmin);
  RgCoef c;
  c.role = 0;
  c.a = c.br = c.bi = c.aa = c.ba = 0.0;
  c.xmax = 1.0;
  if (live_t) c = rg_setup(S, P, n, je, Anorm, Bnorm, true);
  if (live_t) role[col] = c.role;
  const bool act = live_t && (c.role == 1 || c.role == 2);
  const int nw = c.role == 2 ? 2 : 1;
  const double2 bc = make_double2(c.br, c.bi);
  double xmax = 1.0;
  if (act) {
    for (int i = 1; i <= n; ++i) XX(i) = make_double2(0.0, 0.0);
    if (c.role == 1) {
      XX(je) = make_double2(1.0, 0.0);
    } else {
      double t1 = c.a * SS(je + 1, je);
      const double t2r = c.a * SS(je, je) - c.br * PP(je, je), t2i = -c.bi * PP(je, je);
      double2 v0, v1;
      if (fabs(t1) > fabs(t2r) + fabs(t2i)) {
        v0 = make_double2(1.0, 0.0);
        v1 = zdiv(make_double2(-t2r, -t2i), make_double2(t1, 0.0));
      } else {
        v1 = make_double2(1.0, 0.0);
        t1 = c.a * SS(je, je + 1);
        v0 = make_double2((c.br * PP(je + 1, je + 1) - c.a * SS(je + 1, je + 1)) / t1, c.bi * PP(je + 1, je + 1) / t1);
      }
      XX(je) = v0;
      XX(je + 1) = v1;
      xmax = fmax(zabs1(v0), zabs1(v1));
    }
  }
  const double dmin = fmax(fmax(ulp * c.aa * Anorm, ulp * c.ba * Bnorm), safmin);
  const int j0 = je + nw;  // the thread's first block starts at row j0
  const int kmin = blockIdx.x * kRgT + 1;  // smallest je of the CTA
  int jb = kmin + 1;
  while (jb <= n) {
    const bool two = jb < n && SS(jb + 1, jb) != 0.0;
    const int na = two ? 2 : 1;
    const bool on = act && jb >= j0;
    if (on) {
      const double xscale = 1.0 / fmax(1.0, xmax);
      double t1 = fmax(fmax(sn[jb - 1], pn[jb - 1]), c.aa * sn[jb - 1] + c.ba * sn[jb - 1]);
      if (na == 2) t1 = fmax(fmax(t1, sn[jb]), fmax(pn[jb], c.aa * sn[jb] + c.ba * sn[jb]));
      if (t1 > bignum * xscale) {
        for (int r = je; r <= jb - 1; ++r) XX(r) = zscal(XX(r), xscale);
        xmax *= xscale;
      }
    }
    double2 sS[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)}, sP[2] = {sS[0], sS[0]};
    for (int jr = kmin; jr <= jb - 1; ++jr) {
      const double s0 = SS(jr, jb), p0 = PP(jr, jb);
      const double s1 = na == 2 ? SS(jr, jb + 1) : 0.0, p1 = na == 2 ? PP(jr, jb + 1) : 0.0;
      if (on && jr >= je) {
        const double2 v = XX(jr);
        sS[0] = zadd(sS[0], zscal(v, s0));
        sP[0] = zadd(sP[0], zscal(v, p0));
        if (na == 2) {
          sS[1] = zadd(sS[1], zscal(v, s1));
          sP[1] = zadd(sP[1], zscal(v, p1));
        }
      }
    }
    if (on) {
      double2 y[2];
      for (int q = 0; q < na; ++q) y[q] = zadd(zscal(sS[q], -c.a), zmul(bc, sP[q]));
      if (na == 1) y[1] = make_double2(0.0, 0.0);
      double blk[4], dg[2];
      for (int q = 0; q < na; ++q) {
        dg[q] = PP(jb + q, jb + q);
        for (int p = 0; p < na; ++p) blk[p + q * na] = SS(jb + q, jb + p);  // transposed block
      }
      double t1;
      const double scale = xsolve_gen(c.a, blk, na, dg, bc, y, dmin, t1);
      XX(jb) = y[0];
      if (na == 2) XX(jb + 1) = y[1];
      if (scale < 1.0) {
        for (int r = je; r <= jb - 1; ++r) XX(r) = zscal(XX(r), scale);
        xmax *= scale;
      }
      xmax = fmax(xmax, t1);
    }
    jb += na;
  }
  if (live_t) xm[col] = xmax;
}

// Back-transform by M (real, or none), scaling, unit vectors of singular pencils and the
// conjugate column of a pair.  Right: the vector of thread col goes to column col (real) or
// col - 1 (pair, conjugate to col); left: col (real) or col (pair, conjugate to col + 1).
__global__ void __launch_bounds__(kRgT) k_rgevc_back(int n, const double2* __restrict__ X, const double* __restrict__ M,
                                                    const double* __restrict__ xm, const int* __restrict__ role,
                                                    int left, double2* __restrict__ V) {
  const int col = blockIdx.x * kRgT + threadIdx.x;
  const bool live_t = col < n;
  const int k = col + 1;
  const int rl = live_t ? role[col] : 0;
  const bool act = rl == 1 || rl == 2;
  const int nw = rl == 2 ? 2 : 1;
  const int out = (left || rl != 2) ? col : col - 1;  // 0-based output column
  const double safmin = kSafemin;
  const int lo = left ? k : 1, hi = left ? n : k;  // X's nonzero rows
  const int r0 = M ? 1 : lo, r1 = M ? n : hi;
  const int klo = blockIdx.x * kRgT + 1, khi = min(n, (int)(blockIdx.x + 1) * kRgT);
  double xmax = left ? 0.0 : (act ? xm[col] : 0.0);
  if (M) {
    const int qlo = left ? klo : 1, qhi = left ? n : khi;
    for (int r = 1; r <= n; ++r) {
      double2 acc = make_double2(0.0, 0.0);
      for (int q = qlo; q <= qhi; ++q) {
        const double m = M[(r - 1) + (size_t)(q - 1) * n];
        if (act && q >= lo && q <= hi) acc = zadd(acc, zscal(X[(size_t)(q - 1) * n + col], m));
      }
      if (act) {
        V[(r - 1) + (size_t)out * n] = acc;
        xmax = fmax(xmax, zabs1(acc));
      }
    }
  } else if (act) {
    for (int r = 1; r <= n; ++r) {
      const double2 x = (r >= lo && r <= hi) ? X[(size_t)(r - 1) * n + col] : make_double2(0.0, 0.0);
      V[(r - 1) + (size_t)out * n] = x;
      if (r >= lo && r <= hi) xmax = fmax(xmax, zabs1(x));
    }
  }
  if (!live_t) return;
  if (rl == 3) {
    double2* vc = V + (size_t)col * n;
    for (int r = 1; r <= n; ++r) vc[r - 1] = make_double2(r == k ? 1.0 : 0.0, 0.0);
    return;
  }
  if (!act) return;
  double2* vc = V + (size_t)out * n;
  if (xmax > safmin) {
    const double t = 1.0 / xmax;
    for (int r = r0; r <= r1; ++r) vc[r - 1] = zscal(vc[r - 1], t);
  }
  if (nw == 2) {
    double2* v2 = V + (size_t)(out + 1) * n;
    for (int r = 1; r <= n; ++r) v2[r - 1] = zconj(vc[r - 1]);
  }
}

#undef SS
#undef PP
#undef XX

}  // namespace

size_t rgevc_ws_bytes(int n) {
  return (size_t)n * n * sizeof(double2) + 3 * (size_t)n * sizeof(double) + (size_t)n * sizeof(int) + 1024;
}

cudaError_t launch_rgevc(int n, const double* S, const double* P, const double* M, int left, double2* V, void* ws,
                         cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  char* w = static_cast<char*>(ws);
  double2* X = reinterpret_cast<double2*>(w);
  w += (size_t)n * n * sizeof(double2);
  double* sn = reinterpret_cast<double*>(w);
  double* pn = sn + n;
  double* xm = pn + n;
  w += 3 * (size_t)n * sizeof(double);
  int* role = reinterpret_cast<int*>(w);
  w += (size_t)n * sizeof(int);
  w = reinterpret_cast<char*>(((uintptr_t)w + 15) & ~uintptr_t(15));
  unsigned long long* ab = reinterpret_cast<unsigned long long*>(w);
  cudaError_t e = cudaMemsetAsync(ab, 0, 2 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  // V starts at zero: a pair's idle row writes nothing and singular columns are set below
  e = cudaMemsetAsync(V, 0, (size_t)n * n * sizeof(double2), s);
  if (e != cudaSuccess) return e;
  k_rg_norms<<<(n + 127) / 128, 128, 0, s>>>(n, S, P, sn, pn, ab);
  const int g = (n + kRgT - 1) / kRgT;
  if (left) k_rgevc_left<<<g, kRgT, 0, s>>>(n, S, P, sn, pn, ab, X, xm, role);
  else k_rgevc_right<<<g, kRgT, 0, s>>>(n, S, P, sn, pn, ab, X, xm, role);
  k_rgevc_back<<<g, kRgT, 0, s>>>(n, X, M, xm, role, left, V);
  return cudaGetLastError();
}

}  // namespace gsk
