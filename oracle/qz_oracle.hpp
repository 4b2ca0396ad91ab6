// CPU oracle of the generalized Schur decomposition of a complex pencil (TEST
// INFRASTRUCTURE ONLY; the shipped library never links this): a restatement of
//   ggschur!(A, B; wantQ, wantZ, scale)   src/generalized.jl:21-80
//   _hessenberg!(A, B, Q, Z)              src/generalized.jl:82-113 (from LAPACK's zgghrd)
//   _gqz!(H, B, Q, Z, wantSchur)          src/generalized.jl:125-487 (from LAPACK's zhgeqz)
// with qr!(B) as Householder QR with the reference's _reflector! (xLARFG conventions,
// real R diagonal) and LinearAlgebra's complex givensAlgorithm (LAPACK 3.x zlartg with its
// safmn2 / safmx2 rescaling).  1-based index macros; column-major.
#pragma once
#include <vector>
#include "gschur_oracle.hpp"

namespace orc {

template <class R> inline R cabs1max(cx<R> z) { return m_max(m_abs(z.re), m_abs(z.im)); }

// LinearAlgebra.givensAlgorithm(f::Complex, g::Complex) (LAPACK 3.x zlartg).
template <class R> void zgivens_alg(cx<R> f, cx<R> g, R* cs, cx<R>* sn, cx<R>* r) {
  R mn2 = R(1);
  for (int k = 0; k < 485; ++k) mn2 *= R(0.5);
  const R mx2 = R(1) / mn2;
  const R safmin = lim<R>::fmin();
  cx<R> fs = f, gs = g;
  R scale = m_max(cabs1max(f), cabs1max(g));
  int count = 0;
  if (scale >= mx2) {
    do {
      ++count;
      fs = fs * mn2;
      gs = gs * mn2;
      scale *= mn2;
    } while (!(scale < mx2 || count >= 20));
  } else if (scale <= mn2) {
    if (g == cx<R>(0)) { *cs = R(1); *sn = cx<R>(0); *r = f; return; }
    do {
      --count;
      fs = fs * mx2;
      gs = gs * mx2;
      scale *= mx2;
    } while (!(scale > mn2));
  }
  const R f2 = abs2(fs), g2 = abs2(gs);
  if (f2 <= m_max(g2, R(1)) * safmin) {
    if (f == cx<R>(0)) {
      *cs = R(0);
      *r = cx<R>(m_hypot(g.re, g.im));
      const R d = m_hypot(gs.re, gs.im);
      *sn = cx<R>(gs.re / d, -gs.im / d);
      return;
    }
    const R f2s = m_hypot(fs.re, fs.im);
    const R g2s = m_sqrt(g2);
    const R c = f2s / g2s;
    cx<R> ff;
    if (cabs1max(f) > R(1)) {
      const R d = m_hypot(f.re, f.im);
      ff = cx<R>(f.re / d, f.im / d);
    } else {
      const R dr = mx2 * f.re, di = mx2 * f.im;
      const R d = m_hypot(dr, di);
      ff = cx<R>(dr / d, di / d);
    }
    const cx<R> s = ff * cx<R>(gs.re / g2s, -gs.im / g2s);
    *cs = c;
    *sn = s;
    *r = f * c + s * g;
    return;
  }
  const R f2s = m_sqrt(R(1) + g2 / f2);
  cx<R> rr(f2s * fs.re, f2s * fs.im);
  const R c = R(1) / f2s;
  const R d = f2 + g2;
  cx<R> s(rr.re / d, rr.im / d);
  s = s * conj(gs);
  if (count > 0) for (int i = 0; i < count; ++i) rr = rr * mx2;
  else if (count < 0) for (int i = 0; i < -count; ++i) rr = rr * mn2;
  *cs = c;
  *sn = s;
  *r = rr;
}

// Givens G = [c s; -conj(s) c] on rows i1, i2 of M, columns j0..j1 (lmul!(G, M)).
template <class R> inline void g_rows(cx<R>* m, int ld, int i1, int i2, R c, cx<R> s, int j0, int j1) {
  for (int j = j0; j <= j1; ++j) {
    cx<R>& a1 = m[(i1 - 1) + (long long)(j - 1) * ld];
    cx<R>& a2 = m[(i2 - 1) + (long long)(j - 1) * ld];
    const cx<R> x = a1, y = a2;
    a1 = x * c + s * y;
    a2 = y * c - conj(s) * x;
  }
}
// rmul!(M, G) on columns i1, i2, rows r0..r1: [a1 a2] <- [c a1 - conj(s) a2, s a1 + c a2]
template <class R> inline void g_cols(cx<R>* m, int ld, int i1, int i2, R c, cx<R> s, int r0, int r1) {
  for (int r = r0; r <= r1; ++r) {
    cx<R>& a1 = m[(r - 1) + (long long)(i1 - 1) * ld];
    cx<R>& a2 = m[(r - 1) + (long long)(i2 - 1) * ld];
    const cx<R> x = a1, y = a2;
    a1 = x * c - y * conj(s);
    a2 = x * s + y * c;
  }
}
// rmul!(M, G') on columns i1, i2, rows r0..r1: [a1 a2] <- [c a1 + conj(s) a2, -s a1 + c a2]
template <class R> inline void g_cols_adj(cx<R>* m, int ld, int i1, int i2, R c, cx<R> s, int r0, int r1) {
  for (int r = r0; r <= r1; ++r) {
    cx<R>& a1 = m[(r - 1) + (long long)(i1 - 1) * ld];
    cx<R>& a2 = m[(r - 1) + (long long)(i2 - 1) * ld];
    const cx<R> x = a1, y = a2;
    a1 = x * c + conj(s) * y;
    a2 = y * c - s * x;
  }
}

template <class R> R fro_norm_block(const cx<R>* m, int ld, int lo, int hi) {
  R scale = 0, ssq = 1;
  for (int j = lo; j <= hi; ++j)
    for (int i = lo; i <= hi; ++i) {
      const cx<R> z = m[(i - 1) + (long long)(j - 1) * ld];
      const R parts[2] = {m_abs(z.re), m_abs(z.im)};
      for (R a : parts) {
        if (a == R(0)) continue;
        if (scale < a) { ssq = R(1) + ssq * (scale / a) * (scale / a); scale = a; }
        else ssq += (a / scale) * (a / scale);
      }
    }
  return scale * m_sqrt(ssq);
}

// _gqz! (generalized.jl:125-487) on H (Hessenberg) and B (upper triangular), ilo = 1,
// ihi = n, wantSchur = true.  Returns 0, or 1 when the iteration limit is reached.
template <class R>
int gqz_cplx(int n, cx<R>* h, int ldh, cx<R>* b, int ldb, cx<R>* q, int ldq, cx<R>* z, int ldz, cx<R>* alpha,
             cx<R>* beta, long long maxiter) {
  typedef cx<R> C;
#define H(i, j) h[((i) - 1) + (long long)((j) - 1) * ldh]
#define B(i, j) b[((i) - 1) + (long long)((j) - 1) * ldb]
  const bool wantQ = q != nullptr, wantZ = z != nullptr;
  const int ilo = 1, ihi = n;
  const R ulp = lim<R>::eps(), safmin = safemin<R>();
  const R anorm = fro_norm_block(h, ldh, ilo, ihi), bnorm = fro_norm_block(b, ldb, ilo, ihi);
  const R atol = m_max(safmin, ulp * anorm), btol = m_max(safmin, ulp * bnorm);
  const R ascale = R(1) / m_max(safmin, anorm), bscale = R(1) / m_max(safmin, bnorm);
  const R half = R(0.5);
  int ifirst = ilo, ilast = ihi;
  const int ifirstm = 1, ilastm = n;
  int shiftcount = 0;
  C eshift(0);
  long long niter = 0;
  enum { UNKNOWN, NONE, NORMAL, INF };
  while (true) {
    if (++niter > maxiter) return 1;
    int br = UNKNOWN;
    if (ilast == ilo) {
      br = NORMAL;
    } else if (abs1(H(ilast, ilast - 1)) < m_max(safmin, ulp * (abs1(H(ilast, ilast)) + abs1(H(ilast - 1, ilast - 1))))) {
      H(ilast, ilast - 1) = C(0);
      br = NORMAL;
    }
    if (br == UNKNOWN) {
      if (cabs(B(ilast, ilast)) <= btol) {
        B(ilast, ilast) = C(0);
        br = INF;
      } else {
        for (int j = ilast - 1; j >= ilo; --j) {
          bool t1 = false;
          if (j == ilo) {
            t1 = true;
          } else if (abs1(H(j, j - 1)) <= m_max(safmin, ulp * (abs1(H(j, j)) + abs1(H(j - 1, j - 1))))) {
            H(j, j - 1) = C(0);
            t1 = true;
          }
          const bool t2 = cabs(B(j, j)) < btol;
          if (t2) {
            B(j, j) = C(0);
            bool t1a = !t1 && (abs1(H(j, j - 1)) * (ascale * abs1(H(j + 1, j))) <= abs1(H(j, j)) * (ascale * atol));
            if (t1 || t1a) {
              for (int jch = j; jch <= ilast - 1; ++jch) {
                R c;
                C s, r;
                zgivens_alg(H(jch, jch), H(jch + 1, jch), &c, &s, &r);
                H(jch, jch) = r;
                H(jch + 1, jch) = C(0);
                g_rows(h, ldh, jch, jch + 1, c, s, jch + 1, ilastm);
                g_rows(b, ldb, jch, jch + 1, c, s, jch + 1, ilastm);
                if (wantQ) g_cols_adj(q, ldq, jch, jch + 1, c, s, 1, n);
                if (t1a) H(jch, jch - 1) = H(jch, jch - 1) * c;
                t1a = false;
                if (abs1(B(jch + 1, jch + 1)) > btol) {
                  if (jch + 1 >= ilast) br = NORMAL;
                  else { ifirst = jch + 1; br = NONE; }
                  break;
                }
                B(jch + 1, jch + 1) = C(0);
              }
              if (br == UNKNOWN) br = INF;
              break;
            } else {
              for (int jch = j; jch <= ilast - 1; ++jch) {
                R c;
                C s, r;
                zgivens_alg(B(jch, jch + 1), B(jch + 1, jch + 1), &c, &s, &r);
                B(jch, jch + 1) = r;
                B(jch + 1, jch + 1) = C(0);
                if (jch < ilastm - 1) g_rows(b, ldb, jch, jch + 1, c, s, jch + 2, ilastm);
                g_rows(h, ldh, jch, jch + 1, c, s, jch - 1, ilastm);
                if (wantQ) g_cols_adj(q, ldq, jch, jch + 1, c, s, 1, n);
                zgivens_alg(conj(H(jch + 1, jch)), conj(H(jch + 1, jch - 1)), &c, &s, &r);
                H(jch + 1, jch) = conj(r);
                H(jch + 1, jch - 1) = C(0);
                // G = Givens(jch, jch-1, c, s): rmul!(M, G') on columns jch, jch-1
                g_cols_adj(h, ldh, jch, jch - 1, c, s, ifirstm, jch);
                g_cols_adj(b, ldb, jch, jch - 1, c, s, ifirstm, jch + 1);
                if (wantZ) g_cols_adj(z, ldz, jch, jch - 1, c, s, 1, n);
              }
              br = INF;
              break;
            }
          } else if (t1) {
            ifirst = j;
            br = NONE;
            break;
          }
        }
      }
      if (br == INF) {
        R c;
        C s, r;
        zgivens_alg(conj(H(ilast, ilast)), conj(H(ilast, ilast - 1)), &c, &s, &r);
        H(ilast, ilast) = conj(r);
        H(ilast, ilast - 1) = C(0);
        g_cols_adj(h, ldh, ilast, ilast - 1, c, s, ifirstm, ilast - 1);
        g_cols_adj(b, ldb, ilast, ilast - 1, c, s, ifirstm, ilast - 1);
        if (wantZ) g_cols_adj(z, ldz, ilast, ilast - 1, c, s, 1, n);
        br = NORMAL;
      }
    }
    if (br == NORMAL) {
      const R absb = cabs(B(ilast, ilast));
      if (absb > safmin) {
        const C signbc = conj(B(ilast, ilast) / absb);
        B(ilast, ilast) = C(absb);
        for (int i = ifirstm; i <= ilast - 1; ++i) B(i, ilast) = B(i, ilast) * signbc;
        for (int i = ifirstm; i <= ilast; ++i) H(i, ilast) = H(i, ilast) * signbc;
        if (wantZ)
          for (int i = 1; i <= n; ++i) z[(i - 1) + (long long)(ilast - 1) * ldz] = z[(i - 1) + (long long)(ilast - 1) * ldz] * signbc;
      } else {
        B(ilast, ilast) = C(0);
      }
      alpha[ilast - 1] = H(ilast, ilast);
      beta[ilast - 1] = B(ilast, ilast);
      ilast -= 1;
      if (ilast < ilo) break;
      shiftcount = 0;
      eshift = C(0);
      continue;
    }
    // QZ step on ifirst:ilast
    shiftcount += 1;
    C shift;
    if (shiftcount % 10 != 0) {
      const C b11 = B(ilast - 1, ilast - 1) * bscale;
      const C b22 = B(ilast, ilast) * bscale;
      const C u12 = (B(ilast - 1, ilast) * bscale) / b22;
      const C ad11 = (H(ilast - 1, ilast - 1) * ascale) / b11;
      const C ad21 = (H(ilast, ilast - 1) * ascale) / b11;
      const C ad12 = (H(ilast - 1, ilast) * ascale) / b22;
      const C ad22 = (H(ilast, ilast) * ascale) / b22;
      const C abi22 = ad22 - u12 * ad21;
      const C abi12 = ad12 - u12 * ad11;
      shift = abi22;
      const C t = csqrt(abi12) * csqrt(ad21);
      R t1 = abs1(t);
      if (!(t == C(0))) {
        const C x = (ad11 - shift) * half;
        const R t2 = abs1(x);
        t1 = m_max(t1, t2);
        const C xt = x / t1, tt = t / t1;
        C y = csqrt(xt * xt + tt * tt) * t1;
        if (t2 > R(0)) {
          const C xs = x / t2;
          if (xs.re * y.re + xs.im * y.im < R(0)) y = -y;
        }
        shift = shift - t * (t / (x + y));
      }
    } else {
      if (shiftcount % 20 == 0 && bscale * abs1(B(ilast, ilast)) > safmin)
        eshift += (H(ilast, ilast) * ascale) / (B(ilast, ilast) * bscale);
      else
        eshift += (H(ilast, ilast - 1) * ascale) / (B(ilast - 1, ilast - 1) * bscale);
      shift = eshift;
    }
    C f1(1);
    int istart = -1;
    bool gotit = false;
    for (int j = ilast - 1; j >= ifirst + 1; --j) {
      istart = j;
      f1 = H(j, j) * ascale - shift * (B(j, j) * bscale);
      R t1 = abs1(f1);
      R t2 = ascale * abs1(H(j + 1, j));
      const R tr = m_max(t1, t2);
      if (tr < R(1) && tr != R(0)) { t1 /= tr; t2 /= tr; }
      if (abs1(H(j, j - 1)) * t2 <= t1 * atol) { gotit = true; break; }
    }
    if (!gotit) {
      istart = ifirst;
      f1 = H(ifirst, ifirst) * ascale - shift * (B(ifirst, ifirst) * bscale);
    }
    const C g2 = H(istart + 1, istart) * ascale;
    R c;
    C s, r;
    zgivens_alg(f1, g2, &c, &s, &r);
    for (int j = istart; j <= ilast - 1; ++j) {
      if (j > istart) {
        zgivens_alg(H(j, j - 1), H(j + 1, j - 1), &c, &s, &r);
        H(j, j - 1) = r;
        H(j + 1, j - 1) = C(0);
      }
      g_rows(h, ldh, j, j + 1, c, s, j, ilastm);
      g_rows(b, ldb, j, j + 1, c, s, j, ilastm);
      if (wantQ) g_cols_adj(q, ldq, j, j + 1, c, s, 1, n);
      zgivens_alg(B(j + 1, j + 1), B(j + 1, j), &c, &s, &r);
      B(j + 1, j + 1) = r;
      B(j + 1, j) = C(0);
      g_cols(h, ldh, j, j + 1, c, s, ifirstm, m_min(j + 2, ilast));
      g_cols(b, ldb, j, j + 1, c, s, ifirstm, j);
      if (wantZ) g_cols(z, ldz, j, j + 1, c, s, 1, n);
    }
  }
  return 0;
#undef H
#undef B
}

// ggschur!(A, B; wantQ, wantZ, scale) for complex A, B (generalized.jl:21-80 with
// _hessenberg! 82-113).  A <- S, B <- T; Q, Z n x n (wanted when non-null).
template <class R>
int ggschur_cplx(int n, cx<R>* a, int lda, cx<R>* b, int ldb, cx<R>* q, cx<R>* z, cx<R>* alpha, cx<R>* beta,
                 bool scale, long long maxiter) {
  typedef cx<R> C;
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * lda]
#define B_(i, j) b[((i) - 1) + (long long)((j) - 1) * ldb]
  R cscale = 1, anrm = 1, cscaleb = 1, bnrm = 1;
  bool scaleA = false, scaleB = false;
  if (scale) {
    scaleA = scale_matrix<R, C>(n, a, lda, &cscale, &anrm);
    scaleB = scale_matrix<R, C>(n, b, ldb, &cscaleb, &bnrm);
  }
  // qr!(B); A <- Q' A; Q = Matrix(Q)
  std::vector<C> tau(n > 0 ? n : 1);
  for (int j = 1; j <= n; ++j) {
    const int m = n - j + 1;
    const C t = reflector(&B_(j, j), m);
    tau[j - 1] = t;
    // apply H^H = I - conj(t) v v^H (v = [1; B[j+1:n, j]]) to B[j:n, j+1:n] and A[j:n, :]
    auto apply = [&](C* m0, int ld, int c0, int c1) {
      for (int col = c0; col <= c1; ++col) {
        C* x = m0 + (j - 1) + (long long)(col - 1) * ld;
        C s = x[0];
        for (int r = 1; r < m; ++r) s += conj(B_(j + r, j)) * x[r];
        s = conj(t) * s;
        x[0] -= s;
        for (int r = 1; r < m; ++r) x[r] -= s * B_(j + r, j);
      }
    };
    apply(b, ldb, j + 1, n);
    apply(a, lda, 1, n);
  }
  if (q) {
    // Q = H_1 H_2 ... H_n applied backwards to the identity
    for (int jj = 1; jj <= n; ++jj)
      for (int ii = 1; ii <= n; ++ii) q[(ii - 1) + (long long)(jj - 1) * n] = C(ii == jj ? 1 : 0);
    for (int j = n; j >= 1; --j) {
      const int m = n - j + 1;
      const C t = tau[j - 1];
      for (int col = j; col <= n; ++col) {
        C* x = q + (j - 1) + (long long)(col - 1) * n;
        C s = x[0];
        for (int r = 1; r < m; ++r) s += conj(B_(j + r, j)) * x[r];
        s = t * s;
        x[0] -= s;
        for (int r = 1; r < m; ++r) x[r] -= s * B_(j + r, j);
      }
    }
  }
  // R = triu(B)
  for (int jj = 1; jj <= n; ++jj)
    for (int ii = jj + 1; ii <= n; ++ii) B_(ii, jj) = C(0);
  if (z)
    for (int jj = 1; jj <= n; ++jj)
      for (int ii = 1; ii <= n; ++ii) z[(ii - 1) + (long long)(jj - 1) * n] = C(ii == jj ? 1 : 0);
  // _hessenberg!(A, B, Q, Z) (zgghrd)
  for (int jc = 1; jc <= n - 2; ++jc)
    for (int jr = n; jr >= jc + 2; --jr) {
      R c;
      C s, r;
      zgivens_alg(A_(jr - 1, jc), A_(jr, jc), &c, &s, &r);
      g_rows(a, lda, jr - 1, jr, c, s, 1, n);
      g_rows(b, ldb, jr - 1, jr, c, s, 1, n);
      if (q) g_cols_adj(q, n, jr - 1, jr, c, s, 1, n);
      zgivens_alg(conj(B_(jr, jr)), conj(B_(jr, jr - 1)), &c, &s, &r);
      g_cols_adj(a, lda, jr, jr - 1, c, s, 1, n);
      g_cols_adj(b, ldb, jr, jr - 1, c, s, 1, n);
      if (z) g_cols_adj(z, n, jr, jr - 1, c, s, 1, n);
    }
  for (int jj = 1; jj <= n; ++jj)
    for (int ii = 1; ii <= n; ++ii) {
      if (ii > jj + 1) A_(ii, jj) = C(0);
      if (ii > jj) B_(ii, jj) = C(0);
    }
  const int st = gqz_cplx<R>(n, a, lda, b, ldb, q, n, z, n, alpha, beta, maxiter);
  if (scaleA) {
    for (int jj = 1; jj <= n; ++jj) safescale<R, C>(a + (long long)(jj - 1) * lda, n, cscale, anrm);
    for (int i = 1; i <= n; ++i) alpha[i - 1] = A_(i, i);
  }
  if (scaleB) {
    for (int jj = 1; jj <= n; ++jj) safescale<R, C>(b + (long long)(jj - 1) * ldb, n, cscaleb, bnrm);
    for (int i = 1; i <= n; ++i) beta[i - 1] = B_(i, i);
  }
  return st;
#undef A_
#undef B_
}


// ---------------------------------------------------------------------------
// Eigenvectors of a complex generalized Schur pair (S, P upper triangular):
//   right  _geigvecs(S, P[, Z])   src/vectors.jl:723-842
//   left   _gleigvecs(S, P[, Q])  src/vectors.jl:845-1038
// Column idx of V is the eigenvector of (S[idx,idx], P[idx,idx]), back-transformed by
// X (Z for right, Q for left) when X is non-null, scaled so that max |re|+|im| = 1.
// Column-major, leading dimension n.  Same operation order as the reference.
// ---------------------------------------------------------------------------
template <class R>
R gg_safemin() {
  // safemin(T) (util.jl:5-12): floatmin unless 1/floatmax is larger
  R sfmin = std::numeric_limits<R>::min();
  R small = R(1) / std::numeric_limits<R>::max();
  if (small >= sfmin) sfmin = small * (R(1) + std::numeric_limits<R>::epsilon());
  return sfmin;
}

template <class R>
void gg_norms(int n, const cx<R>* S, const cx<R>* P, std::vector<R>& sn, std::vector<R>& pn, R* anorm, R* bnorm) {
  sn.assign(n, R(0));
  pn.assign(n, R(0));
  R an = abs1(S[0]), bn = abs1(P[0]);
  for (int j = 2; j <= n; ++j) {
    for (int i = 1; i <= j - 1; ++i) {
      sn[j - 1] += abs1(S[(i - 1) + (size_t)(j - 1) * n]);
      pn[j - 1] += abs1(P[(i - 1) + (size_t)(j - 1) * n]);
    }
    an = m_max(an, sn[j - 1] + abs1(S[(j - 1) + (size_t)(j - 1) * n]));
    bn = m_max(bn, pn[j - 1] + abs1(P[(j - 1) + (size_t)(j - 1) * n]));
  }
  *anorm = an;
  *bnorm = bn;
}

// coefficients a (real), b (complex) of (a S - b P) for diagonal entry k (1-based),
// vectors.jl:775-812 / 930-967; returns false for the singular pencil case
template <class R>
bool gg_coeffs(int n, const cx<R>* S, const cx<R>* P, int k, R anorm, R bnorm, R ascale, R bscale, R* acoeff,
               cx<R>* bcoeff) {
  const R ulp = std::numeric_limits<R>::epsilon();
  const R safmin = gg_safemin<R>();
  const R smallnum = safmin * (R(n) / ulp);
  const R bigx = R(1) / smallnum;
  const cx<R> skk = S[(k - 1) + (size_t)(k - 1) * n];
  const R pkk = P[(k - 1) + (size_t)(k - 1) * n].re;
  if (abs1(skk) <= safmin && m_abs(pkk) <= safmin) return false;
  const R t = R(1) / m_max(m_max(abs1(skk) * ascale, m_abs(pkk) * bscale), safmin);
  const cx<R> salpha = (t * skk) * ascale;
  const R sbeta = (t * pkk) * bscale;
  R ac = sbeta * ascale;
  cx<R> bc = salpha * bscale;
  const bool lsa = m_abs(sbeta) >= safmin && m_abs(ac) < smallnum;
  const bool lsb = abs1(salpha) >= safmin && abs1(bc) < smallnum;
  R s = R(1);
  if (lsa) s = (smallnum / m_abs(sbeta)) * m_min(anorm, bigx);
  if (lsb) s = m_max(s, (smallnum / abs1(salpha)) * m_min(bnorm, bigx));
  if (lsa || lsb) {
    s = m_min(s, R(1) / (safmin * m_max(m_max(R(1), m_abs(ac)), abs1(bc))));
    if (lsa) ac = ascale * (s * sbeta);
    else ac = ac * s;
    if (lsb) bc = bscale * (s * salpha);
    else bc = bc * s;
  }
  *acoeff = ac;
  *bcoeff = bc;
  return true;
}

template <class R>
void ggevc_right(int n, const cx<R>* S, const cx<R>* P, const cx<R>* Z, cx<R>* V) {
  const R ulp = std::numeric_limits<R>::epsilon();
  const R safmin = gg_safemin<R>();
  const R bignum = R(1) / (R(n) * safmin);
  std::vector<R> sn, pn;
  R anorm, bnorm;
  gg_norms(n, S, P, sn, pn, &anorm, &bnorm);
  const R ascale = R(1) / m_max(anorm, safmin), bscale = R(1) / m_max(bnorm, safmin);
  std::vector<cx<R>> v(n), v2(n);
#define SS(i, j) S[((i) - 1) + (size_t)((j) - 1) * n]
#define PP(i, j) P[((i) - 1) + (size_t)((j) - 1) * n]
  for (int ki = n; ki >= 1; --ki) {
    const int idx = ki;
    cx<R>* col = V + (size_t)(idx - 1) * n;
    R acoeff;
    cx<R> bcoeff;
    if (!gg_coeffs(n, S, P, ki, anorm, bnorm, ascale, bscale, &acoeff, &bcoeff)) {
      for (int r = 0; r < n; ++r) col[r] = cx<R>(R(0));
      col[idx - 1] = cx<R>(R(1));
      continue;
    }
    const R aca = m_abs(acoeff), acb = abs1(bcoeff);
    for (int r = 0; r < n; ++r) v[r] = cx<R>(R(0));
    const R dmin = m_max(m_max(ulp * aca * anorm, ulp * acb * bnorm), safmin);
    for (int i = 1; i <= ki - 1; ++i) v[i - 1] = acoeff * SS(i, ki) - bcoeff * PP(i, ki);
    v[ki - 1] = cx<R>(R(1));
    for (int j = ki - 1; j >= 1; --j) {
      cx<R> d = acoeff * SS(j, j) - bcoeff * PP(j, j);
      if (abs1(d) <= dmin) d = cx<R>(dmin);
      if (abs1(d) < R(1)) {
        if (abs1(v[j - 1]) >= bignum * abs1(d)) {
          const R t = R(1) / abs1(v[j - 1]);
          for (int r = 0; r < ki; ++r) v[r] = v[r] * t;
        }
      }
      v[j - 1] = -v[j - 1] / d;
      if (j > 1) {
        if (abs1(v[j - 1]) > R(1)) {
          const R t = R(1) / abs1(v[j - 1]);
          if (aca * sn[j - 1] + acb * pn[j - 1] >= bignum * t)
            for (int r = 0; r < ki; ++r) v[r] = v[r] * t;
        }
        const cx<R> ca = acoeff * v[j - 1];
        const cx<R> cb = bcoeff * v[j - 1];
        for (int i = 1; i <= j - 1; ++i) v[i - 1] = v[i - 1] + (ca * SS(i, j) - cb * PP(i, j));
      }
    }
    int iend;
    const cx<R>* src = v.data();
    if (Z) {
      for (int r = 0; r < n; ++r) {
        cx<R> s(R(0));
        for (int k = 0; k < n; ++k) s += Z[r + (size_t)k * n] * v[k];
        v2[r] = s;
      }
      src = v2.data();
      iend = n;
    } else {
      iend = ki;
    }
    R xmax = R(0);
    for (int jr = 1; jr <= iend; ++jr) xmax = m_max(xmax, abs1(src[jr - 1]));
    if (xmax > safmin) {
      const R t = R(1) / xmax;
      for (int jr = 1; jr <= iend; ++jr) col[jr - 1] = t * src[jr - 1];
    } else {
      iend = 0;
    }
    for (int jr = iend + 1; jr <= n; ++jr) col[jr - 1] = cx<R>(R(0));
  }
#undef SS
#undef PP
}

template <class R>
void ggevc_left(int n, const cx<R>* S, const cx<R>* P, const cx<R>* Q, cx<R>* V) {
  const R ulp = std::numeric_limits<R>::epsilon();
  const R safmin = gg_safemin<R>();
  const R bignum = R(1) / (R(n) * safmin);
  std::vector<R> sn, pn;
  R anorm, bnorm;
  gg_norms(n, S, P, sn, pn, &anorm, &bnorm);
  const R ascale = R(1) / m_max(anorm, safmin), bscale = R(1) / m_max(bnorm, safmin);
  std::vector<cx<R>> v(n), v2(n);
#define SS(i, j) S[((i) - 1) + (size_t)((j) - 1) * n]
#define PP(i, j) P[((i) - 1) + (size_t)((j) - 1) * n]
  for (int je = 1; je <= n; ++je) {
    const int idx = je;
    cx<R>* col = V + (size_t)(idx - 1) * n;
    R acoeff;
    cx<R> bcoeff;
    if (!gg_coeffs(n, S, P, je, anorm, bnorm, ascale, bscale, &acoeff, &bcoeff)) {
      for (int r = 0; r < n; ++r) col[r] = cx<R>(R(0));
      col[idx - 1] = cx<R>(R(1));
      continue;
    }
    const R aca = m_abs(acoeff), acb = abs1(bcoeff);
    R xmax = R(1);
    for (int r = 0; r < n; ++r) v[r] = cx<R>(R(0));
    const R dmin = m_max(m_max(ulp * aca * anorm, ulp * acb * bnorm), safmin);
    v[je - 1] = cx<R>(R(1));
    for (int j = je + 1; j <= n; ++j) {
      R t = R(1) / xmax;
      if (aca * sn[j - 1] + acb * pn[j - 1] > bignum * t) {
        for (int r = je; r <= j - 1; ++r) v[r - 1] = v[r - 1] * t;
        xmax = R(1);
      }
      cx<R> suma(R(0)), sumb(R(0));
      for (int jr = je; jr <= j - 1; ++jr) {
        suma += conj(SS(jr, j)) * v[jr - 1];
        sumb += conj(PP(jr, j)) * v[jr - 1];
      }
      cx<R> sumx = acoeff * suma - conj(bcoeff) * sumb;
      cx<R> d = conj(acoeff * SS(j, j) - bcoeff * PP(j, j));
      if (abs1(d) <= dmin) d = cx<R>(dmin);
      if (abs1(d) < R(1)) {
        if (abs1(sumx) >= bignum * abs1(d)) {
          t = R(1) / abs1(sumx);
          for (int r = je; r <= j - 1; ++r) v[r - 1] = v[r - 1] * t;
          xmax *= t;
          sumx = sumx * t;
        }
      }
      v[j - 1] = -sumx / d;
      xmax = m_max(xmax, abs1(v[j - 1]));
    }
    int ibegin;
    const cx<R>* src = v.data();
    if (Q) {
      for (int r = 0; r < n; ++r) {
        cx<R> s(R(0));
        for (int k = 0; k < n; ++k) s += Q[r + (size_t)k * n] * v[k];
        v2[r] = s;
      }
      src = v2.data();
      ibegin = 1;
    } else {
      ibegin = je;
    }
    xmax = R(0);
    for (int jr = ibegin; jr <= n; ++jr) xmax = m_max(xmax, abs1(src[jr - 1]));
    if (xmax > safmin) {
      const R t = R(1) / xmax;
      for (int jr = ibegin; jr <= n; ++jr) col[jr - 1] = t * src[jr - 1];
    } else {
      ibegin = n + 1;
    }
    for (int jr = 1; jr <= ibegin - 1; ++jr) col[jr - 1] = cx<R>(R(0));
  }
#undef SS
#undef PP
}
}  // namespace orc
