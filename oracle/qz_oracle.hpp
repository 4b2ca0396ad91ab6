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
#include "hermitian_oracle.hpp"
#include "eigvecs_oracle.hpp"

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

// ---------------------------------------------------------------------------
// Real pencils: ggschur!(A::Real, B) (src/rgeneralized.jl:10-66) with the real
// _hessenberg! (src/generalized.jl:84-113), _gqz! (dhgeqz, src/rgeneralized.jl:68-808),
// _ggs_2x2 (dlag2, 810-948) and _gsvd_2x2 (dlasv2, 950-1038).
// Julia's Givens(i1, i2, c, s): lmul! [x; y] <- [c x + s y; c y - s x]; rmul!(M, G)
// [a1 a2] <- [c a1 - s a2, s a1 + c a2]; rmul!(M, G') [a1 a2] <- [c a1 + s a2, c a2 - s a1].
// givens(f, g, i1, i2) with i1 > i2 swaps the indices and negates s, which equals applying
// the rotation with the indices in the given order (done below).
// ---------------------------------------------------------------------------
// Base.hypot(x, y, z) of Julia: the largest modulus times the 2-norm of the scaled triple.
template <class R> inline R base_hypot3(R x, R y, R z) {
  const R m = m_max(m_max(m_abs(x), m_abs(y)), m_abs(z));
  if (m != m) return (m_abs(x) == std::numeric_limits<R>::infinity() || m_abs(y) == std::numeric_limits<R>::infinity() ||
                      m_abs(z) == std::numeric_limits<R>::infinity()) ? std::numeric_limits<R>::infinity() : m;
  if (m == R(0) || m == std::numeric_limits<R>::infinity()) return m;
  const R a = x / m, b = y / m, c = z / m;
  return m * m_sqrt(a * a + b * b + c * c);
}
template <class R> inline void gr_rows(R* m, int ld, int i1, int i2, R c, R s, int j0, int j1) {
  for (int j = j0; j <= j1; ++j) {
    R& a1 = m[(i1 - 1) + (long long)(j - 1) * ld];
    R& a2 = m[(i2 - 1) + (long long)(j - 1) * ld];
    const R x = a1, y = a2;
    a1 = c * x + s * y;
    a2 = c * y - s * x;
  }
}
template <class R> inline void gr_cols(R* m, int ld, int i1, int i2, R c, R s, int r0, int r1) {
  for (int r = r0; r <= r1; ++r) {
    R& a1 = m[(r - 1) + (long long)(i1 - 1) * ld];
    R& a2 = m[(r - 1) + (long long)(i2 - 1) * ld];
    const R x = a1, y = a2;
    a1 = x * c - y * s;
    a2 = x * s + y * c;
  }
}
template <class R> inline void gr_cols_adj(R* m, int ld, int i1, int i2, R c, R s, int r0, int r1) {
  for (int r = r0; r <= r1; ++r) {
    R& a1 = m[(r - 1) + (long long)(i1 - 1) * ld];
    R& a2 = m[(r - 1) + (long long)(i2 - 1) * ld];
    const R x = a1, y = a2;
    a1 = x * c + y * s;
    a2 = y * c - x * s;
  }
}

template <class R> R fro_norm_real(const R* m, int ld, int n) {
  R scale = 0, ssq = 1;
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= n; ++i) {
      const R a = m_abs(m[(i - 1) + (long long)(j - 1) * ld]);
      if (a == R(0)) continue;
      if (scale < a) { ssq = R(1) + ssq * (scale / a) * (scale / a); scale = a; }
      else ssq += (a / scale) * (a / scale);
    }
  return scale * m_sqrt(ssq);
}

// dlag2: eigenvalues (wr1 + i wi)/scale1, (wr2 - i wi)/scale2 of the 2 x 2 pencil (A, B), B
// upper triangular; a, b column-major 2 x 2 (ld 2 views passed as pointers + ld).
template <class R>
void ggs_2x2(const R* a, int lda, const R* b, int ldb, R safmin, R* scale1o, R* scale2o, R* wr1o, R* wr2o, R* wio) {
  const R rtmin = m_sqrt(safmin), rtmax = R(1) / rtmin, safmax = R(1) / safmin;
  const R fuzzy1 = R(1) + m_sqrt(m_sqrt(std::numeric_limits<R>::epsilon())) / R(10);
#define GA(i, j) a[((i) - 1) + ((j) - 1) * lda]
#define GB(i, j) b[((i) - 1) + ((j) - 1) * ldb]
  const R anorm = m_max(m_max(m_abs(GA(1, 1)) + m_abs(GA(2, 1)), m_abs(GA(1, 2)) + m_abs(GA(2, 2))), safmin);
  const R ascale = R(1) / anorm;
  const R a11 = ascale * GA(1, 1), a12 = ascale * GA(1, 2), a21 = ascale * GA(2, 1), a22 = ascale * GA(2, 2);
  R b11 = GB(1, 1), b12 = GB(1, 2), b22 = GB(2, 2);
  const R bmin = rtmin * m_max(m_max(m_abs(b11), m_abs(b12)), m_max(m_abs(b22), rtmin));
  if (m_abs(b11) < bmin) b11 = b11 < R(0) ? -bmin : bmin;
  if (m_abs(b22) < bmin) b22 = b22 < R(0) ? -bmin : bmin;
  const R bnorm = m_max(m_max(m_abs(b11), m_abs(b12) + m_abs(b22)), safmin);
  const R bsize = m_max(m_abs(b11), m_abs(b22));
  const R bscale = R(1) / bsize;
  b11 *= bscale;
  b12 *= bscale;
  b22 *= bscale;
  const R binv11 = R(1) / b11, binv22 = R(1) / b22;
  const R s1 = a11 * binv11, s2 = a22 * binv22;
  R as12, ss, abi22, pp, shift;
  if (m_abs(s1) <= m_abs(s2)) {
    as12 = a12 - s1 * b12;
    const R as22 = a22 - s1 * b22;
    ss = a21 * (binv11 * binv22);
    abi22 = as22 * binv22 - ss * b12;
    pp = abi22 / R(2);
    shift = s1;
  } else {
    as12 = a12 - s2 * b12;
    const R as11 = a11 - s2 * b11;
    ss = a21 * (binv11 * binv22);
    abi22 = -ss * b12;
    pp = (as11 * binv11 + abi22) / R(2);
    shift = s2;
  }
  const R qq = ss * as12;
  R discr, r;
  if (m_abs(pp * rtmin) >= R(1)) {
    discr = (rtmin * pp) * (rtmin * pp) + qq * safmin;
    r = m_sqrt(m_abs(discr)) * rtmax;
  } else if (pp * pp + m_abs(qq) <= safmin) {
    discr = (rtmax * pp) * (rtmax * pp) + qq * safmax;
    r = m_sqrt(m_abs(discr)) * rtmin;
  } else {
    discr = pp * pp + qq;
    r = m_sqrt(m_abs(discr));
  }
  R wr1, wr2, wi;
  if (discr >= R(0) || r == R(0)) {
    const R sm = pp + (pp < R(0) ? -r : r);
    const R df = pp - (pp < R(0) ? -r : r);
    const R wbig = shift + sm;
    R wsmall = shift + df;
    if (m_abs(wbig) / R(2) > m_max(m_abs(wsmall), safmin)) {
      const R wdet = (a11 * a22 - a12 * a21) * (binv11 * binv22);
      wsmall = wdet / wbig;
    }
    if (pp > abi22) {
      wr1 = m_min(wbig, wsmall);
      wr2 = m_max(wbig, wsmall);
    } else {
      wr2 = m_min(wbig, wsmall);
      wr1 = m_max(wbig, wsmall);
    }
    wi = R(0);
  } else {
    wr1 = shift + pp;
    wr2 = wr1;
    wi = r;
  }
  const R c1 = bsize * (safmin * m_max(R(1), ascale));
  const R c2 = safmin * m_max(R(1), bnorm);
  const R c3 = bsize * safmin;
  const R c4 = (ascale <= R(1) && bsize <= R(1)) ? m_min(R(1), (ascale / safmin) * bsize) : R(1);
  const R c5 = (ascale <= R(1) || bsize <= R(1)) ? m_min(R(1), ascale * bsize) : R(1);
  R scale1 = R(1), scale2 = R(1);
  const R wabs = m_abs(wr1) + m_abs(wi);
  R wsize = m_max(m_max(safmin, c1), m_max(fuzzy1 * (wabs * c2 + c3), m_min(c4, m_max(wabs, c5) / R(2))));
  if (wsize != R(1)) {
    const R wscale = R(1) / wsize;
    if (wsize > R(1)) scale1 = (m_max(ascale, bsize) * wscale) * m_min(ascale, bsize);
    else scale1 = (m_min(ascale, bsize) * wscale) * m_max(ascale, bsize);
    wr1 *= wscale;
    if (wi != R(0)) {
      wi *= wscale;
      wr2 = wr1;
      scale2 = scale1;
    }
  } else {
    scale1 = ascale * bsize;
    scale2 = scale1;
  }
  if (wi == R(0)) {
    wsize = m_max(m_max(safmin, c1), m_max(fuzzy1 * (m_abs(wr2) * c2 + c3), m_min(c4, m_max(m_abs(wr2), c5) / R(2))));
    if (wsize != R(1)) {
      const R wscale = R(1) / wsize;
      if (wsize > R(1)) scale2 = (m_max(ascale, bsize) * wscale) * m_min(ascale, bsize);
      else scale2 = (m_min(ascale, bsize) * wscale) * m_max(ascale, bsize);
      wr2 *= wscale;
    } else {
      scale2 = ascale * bsize;
    }
  }
  *scale1o = scale1; *scale2o = scale2; *wr1o = wr1; *wr2o = wr2; *wio = wi;
#undef GA
#undef GB
}

// dlasv2 on the upper triangular 2 x 2 [f g; 0 h]: returns ssmin, ssmax, snr, csr, snl, csl.
template <class R>
void gsvd_2x2(R f0, R g0, R h0, R* ssmino, R* ssmaxo, R* snro, R* csro, R* snlo, R* cslo) {
  R ft = f0, gt = g0, ht = h0;
  R fa = m_abs(ft), ha = m_abs(ht);
  int pmax = 1;
  const bool swap = ha > fa;
  if (swap) {
    pmax = 3;
    R t = ft; ft = ht; ht = t;
    t = fa; fa = ha; ha = t;
  }
  const R ga = m_abs(gt);
  R ssmin, ssmax, clt, crt, slt, srt;
  if (ga == R(0)) {
    ssmin = ha; ssmax = fa; clt = R(1); crt = R(1); slt = R(0); srt = R(0);
  } else {
    bool ga_small = true;
    if (ga > fa) {
      pmax = 2;
      if ((fa / ga) < std::numeric_limits<R>::epsilon()) {
        ga_small = false;
        ssmax = ga;
        ssmin = (ha > R(1)) ? (fa / (ga / ha)) : ((fa / ha) * ha);
        clt = R(1);
        slt = ht / gt;
        srt = R(1);
        crt = ft / gt;
      }
    }
    if (ga_small) {
      const R d = fa - ha;
      R l = (d == fa) ? R(1) : (d / fa);
      const R m = gt / ft;
      R t = R(2) - l;
      const R mm = m * m, tt = t * t;
      const R s = m_sqrt(tt + mm);
      const R r = (l == R(0)) ? m_abs(m) : m_sqrt(l * l + mm);
      const R a = (s + r) / R(2);
      ssmin = ha / a;
      ssmax = fa * a;
      if (mm == R(0)) {
        if (l == R(0)) t = m_copysign(R(2), ft) * m_copysign(R(1), gt);
        else t = gt / m_copysign(d, ft) + m / t;
      } else {
        t = (m / (s + t) + m / (r + l)) * (R(1) + a);
      }
      l = m_sqrt(t * t + R(4));
      crt = R(2) / l;
      srt = t / l;
      clt = (crt + srt * m) / a;
      slt = (ht / ft) * srt / a;
    }
  }
  R csl, snl, csr, snr;
  if (swap) { csl = srt; snl = crt; csr = slt; snr = clt; }
  else { csl = clt; snl = slt; csr = crt; snr = srt; }
  R tsgn;
  if (pmax == 1) tsgn = m_copysign(R(1), csr) * m_copysign(R(1), csl) * m_copysign(R(1), f0);
  else if (pmax == 2) tsgn = m_copysign(R(1), snr) * m_copysign(R(1), csl) * m_copysign(R(1), g0);
  else tsgn = m_copysign(R(1), snr) * m_copysign(R(1), snl) * m_copysign(R(1), h0);
  ssmax = m_copysign(ssmax, tsgn);
  ssmin = m_copysign(ssmin, tsgn * m_copysign(R(1), f0) * m_copysign(R(1), h0));
  *ssmino = ssmin; *ssmaxo = ssmax; *snro = snr; *csro = csr; *snlo = snl; *cslo = csl;
}

// _gqz! for real H, B (src/rgeneralized.jl:68-808), ilo = 1, ihi = n, wantSchur = true.
// alphar/alphai/beta: the generalized eigenvalues (alpha complex, beta real).
// Returns 0, or 1 at the iteration limit.
template <class R>
int gqz_real(int n, R* h, int ldh, R* b, int ldb, R* q, int ldq, R* z, int ldz, R* alr, R* ali, R* be,
             long long maxiter) {
#define H_(i, j) h[((i) - 1) + (long long)((j) - 1) * ldh]
#define B_(i, j) b[((i) - 1) + (long long)((j) - 1) * ldb]
  const int ilo = 1, ihi = n;
  const R ulp = std::numeric_limits<R>::epsilon();
  const R safmin = std::numeric_limits<R>::min();
  const R safmax = R(1) / safmin;
  const R safety = R(100);
  const R anorm = fro_norm_real(h, ldh, n), bnorm = fro_norm_real(b, ldb, n);
  const R atol = m_max(safmin, ulp * anorm), btol = m_max(safmin, ulp * bnorm);
  const R ascale = R(1) / m_max(safmin, anorm), bscale = R(1) / m_max(safmin, bnorm);
  int ifirst = ilo, ilast = ihi;
  const int ifirstm = 1, ilastm = n;
  int shiftcount = 0;
  R eshift = R(0);
  R v[3] = {0, 0, 0};
  enum { UNKNOWN, NONE, NORMAL, INF };
  for (long long it = 1; it <= maxiter; ++it) {
    int br = UNKNOWN;
    if (ilast == ilo) br = NORMAL;
    else if (m_abs(H_(ilast, ilast - 1)) < m_max(safmin, ulp * (m_abs(H_(ilast, ilast)) + m_abs(H_(ilast - 1, ilast - 1))))) {
      H_(ilast, ilast - 1) = R(0);
      br = NORMAL;
    }
    if (br == UNKNOWN) {
      if (m_abs(B_(ilast, ilast)) <= btol) {
        B_(ilast, ilast) = R(0);
        br = INF;
      } else {
        for (int j = ilast - 1; j >= ilo; --j) {
          bool have_H_0sd = false;
          if (j == ilo) have_H_0sd = true;
          else if (m_abs(H_(j, j - 1)) <= atol) {
            H_(j, j - 1) = R(0);
            have_H_0sd = true;
          }
          if (m_abs(B_(j, j)) < btol) {
            B_(j, j) = R(0);
            bool have2 = false;
            if (!have_H_0sd) {
              R t = m_abs(H_(j, j - 1)), t2 = m_abs(H_(j, j));
              const R tr = m_max(t, t2);
              if (tr < R(1) && tr != R(0)) { t = t / tr; t2 = t2 / tr; }
              have2 = (t * (ascale * m_abs(H_(j + 1, j))) <= t2 * (ascale * atol));
            }
            if (have_H_0sd || have2) {
              for (int jch = j; jch <= ilast - 1; ++jch) {
                R c, s, r;
                givens_alg(H_(jch, jch), H_(jch + 1, jch), &c, &s, &r);
                H_(jch, jch) = r;
                H_(jch + 1, jch) = R(0);
                gr_rows(h, ldh, jch, jch + 1, c, s, jch + 1, ilastm);
                gr_rows(b, ldb, jch, jch + 1, c, s, jch + 1, ilastm);
                if (q) gr_cols_adj(q, ldq, jch, jch + 1, c, s, 1, n);
                if (have2) H_(jch, jch - 1) *= c;
                have2 = false;
                if (m_abs(B_(jch + 1, jch + 1)) > btol) {
                  if (jch + 1 >= ilast) br = NORMAL;
                  else { ifirst = jch + 1; br = NONE; }
                  break;
                }
                B_(jch + 1, jch + 1) = R(0);
              }
              if (br == UNKNOWN) br = INF;
              break;
            } else {
              for (int jch = j; jch <= ilast - 1; ++jch) {
                R c, s, r;
                givens_alg(B_(jch, jch + 1), B_(jch + 1, jch + 1), &c, &s, &r);
                B_(jch, jch + 1) = r;
                B_(jch + 1, jch + 1) = R(0);
                if (jch < ilastm - 1) gr_rows(b, ldb, jch, jch + 1, c, s, jch + 2, ilastm);
                gr_rows(h, ldh, jch, jch + 1, c, s, jch - 1, ilastm);
                if (q) gr_cols_adj(q, ldq, jch, jch + 1, c, s, 1, n);
                givens_alg(H_(jch + 1, jch), H_(jch + 1, jch - 1), &c, &s, &r);
                H_(jch + 1, jch) = r;
                H_(jch + 1, jch - 1) = R(0);
                gr_cols_adj(h, ldh, jch, jch - 1, c, s, ifirstm, jch);
                gr_cols_adj(b, ldb, jch, jch - 1, c, s, ifirstm, jch - 1);
                if (z) gr_cols_adj(z, ldz, jch, jch - 1, c, s, 1, n);
              }
              br = INF;
              break;
            }
          } else if (have_H_0sd) {
            ifirst = j;
            br = NONE;
            break;
          }
        }
      }
      if (br == INF) {
        R c, s, r;
        givens_alg(H_(ilast, ilast), H_(ilast, ilast - 1), &c, &s, &r);
        H_(ilast, ilast) = r;
        H_(ilast, ilast - 1) = R(0);
        gr_cols_adj(h, ldh, ilast, ilast - 1, c, s, ifirstm, ilast - 1);
        gr_cols_adj(b, ldb, ilast, ilast - 1, c, s, ifirstm, ilast - 1);
        if (z) gr_cols_adj(z, ldz, ilast, ilast - 1, c, s, 1, n);
        br = NORMAL;
      }
    }
    if (br == NORMAL) {
      if (B_(ilast, ilast) < R(0)) {
        for (int i = ifirstm; i <= ilast; ++i) { H_(i, ilast) = -H_(i, ilast); B_(i, ilast) = -B_(i, ilast); }
        if (z) for (int i = 1; i <= n; ++i) z[(i - 1) + (long long)(ilast - 1) * ldz] *= R(-1);
      }
      alr[ilast - 1] = H_(ilast, ilast);
      ali[ilast - 1] = R(0);
      be[ilast - 1] = B_(ilast, ilast);
      ilast -= 1;
      if (ilast < ilo) break;
      shiftcount = 0;
      eshift = R(0);
      continue;
    }
    // QZ step on ifirst..ilast
    ++shiftcount;
    R s1, s2, wr, wr2, wi;
    if (shiftcount % 10 != 0) {
      ggs_2x2(&H_(ilast - 1, ilast - 1), ldh, &B_(ilast - 1, ilast - 1), ldb, safmin * safety, &s1, &s2, &wr, &wr2, &wi);
      if (m_abs((wr / s1) * B_(ilast, ilast) - H_(ilast, ilast)) > m_abs((wr2 / s2) * B_(ilast, ilast) - H_(ilast, ilast))) {
        R t = wr; wr = wr2; wr2 = t;
        t = s1; s1 = s2; s2 = t;
      }
    } else {
      if (R(maxiter) * safmin * m_abs(H_(ilast, ilast - 1)) < m_abs(B_(ilast - 1, ilast - 1)))
        eshift = H_(ilast, ilast - 1) / B_(ilast - 1, ilast - 1);
      else
        eshift += R(1) / (safmin * R(maxiter));
      s1 = R(1);
      wr = eshift;
      wi = R(0);
    }
    if (wi == R(0)) {
      R t = m_min(ascale, R(1)) * (safmax / R(2));
      R scale = s1 > t ? t / s1 : R(1);
      t = m_min(bscale, R(1)) * (safmax / R(2));
      if (m_abs(wr) > t) scale = m_min(scale, t / m_abs(wr));
      s1 *= scale;
      wr *= scale;
      int istart = -1;
      bool gotit = false;
      for (int j = ilast - 1; j >= ifirst + 1; --j) {
        istart = j;
        R t1 = m_abs(s1 * H_(j, j - 1));
        R t2 = m_abs(s1 * H_(j, j) - wr * B_(j, j));
        const R tr = m_max(t1, t2);
        if (tr < R(1) && tr != R(0)) { t1 /= tr; t2 /= tr; }
        if (m_abs((ascale * H_(j + 1, j)) * t1) <= ascale * atol * t2) { gotit = true; break; }
      }
      if (!gotit) istart = ifirst;
      const R f1 = s1 * H_(istart, istart) - wr * B_(istart, istart);
      const R g2 = s1 * H_(istart + 1, istart);
      R c, s, t3;
      givens_alg(f1, g2, &c, &s, &t3);
      for (int j = istart; j <= ilast - 1; ++j) {
        if (j > istart) {
          R r;
          givens_alg(H_(j, j - 1), H_(j + 1, j - 1), &c, &s, &r);
          H_(j, j - 1) = r;
          H_(j + 1, j - 1) = R(0);
        }
        gr_rows(h, ldh, j, j + 1, c, s, j, ilastm);
        gr_rows(b, ldb, j, j + 1, c, s, j, ilastm);
        if (q) gr_cols_adj(q, ldq, j, j + 1, c, s, 1, n);
        R r;
        givens_alg(B_(j + 1, j + 1), B_(j + 1, j), &c, &s, &r);
        B_(j + 1, j + 1) = r;
        B_(j + 1, j) = R(0);
        gr_cols(h, ldh, j, j + 1, c, s, ifirstm, m_min(j + 2, ilast));
        gr_cols(b, ldb, j, j + 1, c, s, ifirstm, j);
        if (z) gr_cols(z, ldz, j, j + 1, c, s, 1, n);
      }
    } else if (ilast == ifirst + 1) {
      // 2 x 2 block with complex eigenvalues: diagonalise B, then alpha, beta
      R b22, b11, sr, cr, sl, cl;
      gsvd_2x2(B_(ifirst, ifirst), B_(ifirst, ilast), B_(ilast, ilast), &b22, &b11, &sr, &cr, &sl, &cl);
      if (b11 < R(0)) { cr = -cr; sr = -sr; b11 = -b11; b22 = -b22; }
      gr_rows(h, ldh, ifirst, ilast, cl, sl, ifirst, ilastm);
      gr_cols_adj(h, ldh, ifirst, ilast, cr, sr, ifirstm, ilast);
      if (ilast < ilastm) gr_rows(b, ldb, ifirst, ilast, cl, sl, ilast + 1, ilastm);
      if (ifirstm < ifirst) gr_cols_adj(b, ldb, ifirst, ilast, cr, sr, ifirstm, ifirst - 1);
      if (q) gr_cols_adj(q, ldq, ifirst, ilast, cl, sl, 1, n);
      if (z) gr_cols_adj(z, ldz, ifirst, ilast, cr, sr, 1, n);
      B_(ilast - 1, ilast - 1) = b11;
      B_(ilast - 1, ilast) = R(0);
      B_(ilast, ilast - 1) = R(0);
      B_(ilast, ilast) = b22;
      if (b22 < R(0)) {
        for (int i = ifirstm; i <= ilast; ++i) { H_(i, ilast) = -H_(i, ilast); B_(i, ilast) = -B_(i, ilast); }
        if (z) for (int i = 1; i <= n; ++i) z[(i - 1) + (long long)(ilast - 1) * ldz] *= R(-1);
        b22 = -b22;
      }
      R d2, d3;
      ggs_2x2(&H_(ilast - 1, ilast - 1), ldh, &B_(ilast - 1, ilast - 1), ldb, safmin * safety, &s1, &d2, &wr, &d3, &wi);
      if (wi == R(0)) continue;  // back to a single shift
      const R s1inv = R(1) / s1;
      const R a11 = H_(ilast - 1, ilast - 1), a21 = H_(ilast, ilast - 1), a12 = H_(ilast - 1, ilast), a22 = H_(ilast, ilast);
      const R c11r = s1 * a11 - wr * b11, c11i = -wi * b11, c12 = s1 * a12, c21 = s1 * a21;
      const R c22r = s1 * a22 - wr * b22, c22i = -wi * b22;
      R cz, szr, szi;
      if (m_abs(c11r) + m_abs(c11i) + m_abs(c12) > m_abs(c21) + m_abs(c22r) + m_abs(c22i)) {
        const R t1 = base_hypot3(c12, c11r, c11i);
        cz = c12 / t1;
        szr = -c11r / t1;
        szi = -c11i / t1;
      } else {
        cz = m_hypot(c22r, c22i);
        if (cz <= safmin) { cz = R(0); szr = R(1); szi = R(0); }
        else {
          const R tr = c22r / cz, ti = c22i / cz;
          const R t1 = m_hypot(cz, c21);
          cz /= t1;
          szr = -c21 * tr / t1;
          szi = c21 * ti / t1;
        }
      }
      const R an = m_abs(a11) + m_abs(a12) + m_abs(a21) + m_abs(a22);
      const R bn = m_abs(b11) + m_abs(b22);
      const R wabs = m_abs(wr) + m_abs(wi);
      R cq, sqr, sqi;
      if (s1 * an > wabs * bn) {
        cq = cz * b11;
        sqr = szr * b22;
        sqi = -szi * b22;
      } else {
        const R a1r = cz * a11 + szr * a12, a1i = szi * a12;
        const R a2r = cz * a21 + szr * a22, a2i = szi * a22;
        cq = m_hypot(a1r, a1i);
        if (cq <= safmin) { cq = R(0); sqr = R(1); sqi = R(0); }
        else {
          const R tr = a1r / cq, ti = a1i / cq;
          sqr = tr * a2r + ti * a2i;
          sqi = ti * a2r - tr * a2i;
        }
      }
      const R t1 = base_hypot3(cq, sqr, sqi);
      cq /= t1;
      sqr /= t1;
      sqi /= t1;
      const R tr = sqr * szr - sqi * szi, ti = sqr * szi + sqi * szr;
      const R b1r = cq * cz * b11 + tr * b22, b1i = ti * b22;
      const R b1a = m_hypot(b1r, b1i);
      const R b2r = cq * cz * b22 + tr * b11, b2i = -ti * b11;
      const R b2a = m_hypot(b2r, b2i);
      be[ilast - 2] = b1a;
      be[ilast - 1] = b2a;
      alr[ilast - 2] = (wr * b1a) * s1inv;
      ali[ilast - 2] = (wi * b1a) * s1inv;
      alr[ilast - 1] = (wr * b2a) * s1inv;
      ali[ilast - 1] = (-wi * b2a) * s1inv;
      ilast = ifirst - 1;
      if (ilast < ilo) break;
      shiftcount = 0;
      eshift = R(0);
    } else {
      // Francis implicit double shift on a block of order >= 3
      const R ad11 = (ascale * H_(ilast - 1, ilast - 1)) / (bscale * B_(ilast - 1, ilast - 1));
      const R ad21 = (ascale * H_(ilast, ilast - 1)) / (bscale * B_(ilast - 1, ilast - 1));
      const R ad12 = (ascale * H_(ilast - 1, ilast)) / (bscale * B_(ilast, ilast));
      const R ad22 = (ascale * H_(ilast, ilast)) / (bscale * B_(ilast, ilast));
      const R u12 = B_(ilast - 1, ilast) / B_(ilast, ilast);
      const R ad11l = (ascale * H_(ifirst, ifirst)) / (bscale * B_(ifirst, ifirst));
      const R ad21l = (ascale * H_(ifirst + 1, ifirst)) / (bscale * B_(ifirst, ifirst));
      const R ad12l = (ascale * H_(ifirst, ifirst + 1)) / (bscale * B_(ifirst + 1, ifirst + 1));
      const R ad22l = (ascale * H_(ifirst + 1, ifirst + 1)) / (bscale * B_(ifirst + 1, ifirst + 1));
      const R ad32l = (ascale * H_(ifirst + 2, ifirst + 1)) / (bscale * B_(ifirst + 1, ifirst + 1));
      const R u12l = B_(ifirst, ifirst + 1) / B_(ifirst + 1, ifirst + 1);
      v[0] = ((ad11 - ad11l) * (ad22 - ad11l) - ad12 * ad21 + ad21 * u12 * ad11l + (ad12l - ad11l * u12l) * ad21l);
      v[1] = (((ad22l - ad11l) - ad21l * u12l - (ad11 - ad11l) - (ad22 - ad11l) + ad21 * u12)) * ad21l;
      v[2] = ad32l * ad21l;
      const int istart = ifirst;
      R tau = reflector_real(v, 3);
      v[0] = R(1);
      for (int j = istart; j <= ilast - 2; ++j) {
        if (j > istart) {
          v[0] = H_(j, j - 1); v[1] = H_(j + 1, j - 1); v[2] = H_(j + 2, j - 1);
          tau = reflector_real(v, 3);
          H_(j, j - 1) = v[0];
          v[0] = R(1);
          H_(j + 1, j - 1) = R(0);
          H_(j + 2, j - 1) = R(0);
        }
        R t2 = tau * v[1], t3 = tau * v[2];
        for (int jc = j; jc <= ilastm; ++jc) {
          R t1 = H_(j, jc) + v[1] * H_(j + 1, jc) + v[2] * H_(j + 2, jc);
          H_(j, jc) -= t1 * tau;
          H_(j + 1, jc) -= t1 * t2;
          H_(j + 2, jc) -= t1 * t3;
          t1 = B_(j, jc) + v[1] * B_(j + 1, jc) + v[2] * B_(j + 2, jc);
          B_(j, jc) -= t1 * tau;
          B_(j + 1, jc) -= t1 * t2;
          B_(j + 2, jc) -= t1 * t3;
        }
        if (q)
          for (int jr = 1; jr <= n; ++jr) {
            R* qr = q + (jr - 1);
            const R t1 = qr[(long long)(j - 1) * ldq] + v[1] * qr[(long long)j * ldq] + v[2] * qr[(long long)(j + 1) * ldq];
            qr[(long long)(j - 1) * ldq] -= t1 * tau;
            qr[(long long)j * ldq] -= t1 * t2;
            qr[(long long)(j + 1) * ldq] -= t1 * t3;
          }
        // zero the j-th column of B: 2 x 2 solve with pivoting
        bool pivot = false;
        R scale, u1, u2;
        {
          R t1 = m_max(m_abs(B_(j + 1, j + 1)), m_abs(B_(j + 1, j + 2)));
          R tt2 = m_max(m_abs(B_(j + 2, j + 1)), m_abs(B_(j + 2, j + 2)));
          if (m_max(t1, tt2) < safmin) {
            scale = R(0); u1 = R(1); u2 = R(0);
          } else {
            R w11, w21, w12, w22;
            if (t1 >= tt2) {
              w11 = B_(j + 1, j + 1); w21 = B_(j + 2, j + 1); w12 = B_(j + 1, j + 2); w22 = B_(j + 2, j + 2);
              u1 = B_(j + 1, j); u2 = B_(j + 2, j);
            } else {
              w21 = B_(j + 1, j + 1); w11 = B_(j + 2, j + 1); w22 = B_(j + 1, j + 2); w12 = B_(j + 2, j + 2);
              u2 = B_(j + 1, j); u1 = B_(j + 2, j);
            }
            if (m_abs(w12) > m_abs(w11)) {
              pivot = true;
              R t = w11; w11 = w12; w12 = t;
              t = w21; w21 = w22; w22 = t;
            }
            t1 = w21 / w11;
            u2 -= t1 * u1;
            w22 -= t1 * w12;
            scale = R(1);
            if (m_abs(w22) < safmin) {
              scale = R(0);
            } else {
              if (m_abs(w22) < m_abs(u2)) scale = m_abs(w22 / u2);
              if (m_abs(w11) < m_abs(u1)) scale = m_min(scale, m_abs(w11 / u1));
              u2 = (scale * u2) / w22;
              u1 = (scale * u1 - w12 * u2) / w11;
            }
          }
        }
        if (pivot) { R t = u1; u1 = u2; u2 = t; }
        {
          const R t1 = base_hypot3(scale, u1, u2);
          tau = R(1) + scale / t1;
          const R vs = -R(1) / (scale + t1);
          v[0] = R(1);
          v[1] = vs * u1;
          v[2] = vs * u2;
        }
        t2 = tau * v[1];
        t3 = tau * v[2];
        for (int jr = ifirstm; jr <= m_min(j + 3, ilast); ++jr) {
          const R t1 = H_(jr, j) + v[1] * H_(jr, j + 1) + v[2] * H_(jr, j + 2);
          H_(jr, j) -= t1 * tau;
          H_(jr, j + 1) -= t2 * t1;
          H_(jr, j + 2) -= t3 * t1;
        }
        for (int jr = ifirstm; jr <= j + 2; ++jr) {
          const R t1 = B_(jr, j) + v[1] * B_(jr, j + 1) + v[2] * B_(jr, j + 2);
          B_(jr, j) -= t1 * tau;
          B_(jr, j + 1) -= t2 * t1;
          B_(jr, j + 2) -= t3 * t1;
        }
        if (z)
          for (int jr = 1; jr <= n; ++jr) {
            R* zr = z + (jr - 1);
            const R t1 = zr[(long long)(j - 1) * ldz] + v[1] * zr[(long long)j * ldz] + v[2] * zr[(long long)(j + 1) * ldz];
            zr[(long long)(j - 1) * ldz] -= t1 * tau;
            zr[(long long)j * ldz] -= t2 * t1;
            zr[(long long)(j + 1) * ldz] -= t3 * t1;
          }
        B_(j + 1, j) = R(0);
        B_(j + 2, j) = R(0);
      }
      // last two rotations
      const int j = ilast - 1;
      R c, s, r;
      givens_alg(H_(j, j - 1), H_(j + 1, j - 1), &c, &s, &r);
      H_(j, j - 1) = r;
      H_(j + 1, j - 1) = R(0);
      gr_rows(h, ldh, j, j + 1, c, s, j, ilastm);
      gr_rows(b, ldb, j, j + 1, c, s, j, ilastm);
      if (q) gr_cols_adj(q, ldq, j, j + 1, c, s, 1, n);
      givens_alg(B_(j + 1, j + 1), B_(j + 1, j), &c, &s, &r);
      B_(j + 1, j + 1) = r;
      B_(j + 1, j) = R(0);
      gr_cols_adj(h, ldh, j + 1, j, c, s, ifirstm, ilast);
      gr_cols_adj(b, ldb, j + 1, j, c, s, ifirstm, ilast - 1);
      if (z) gr_cols_adj(z, ldz, j + 1, j, c, s, 1, n);
    }
    if (it >= maxiter) return 1;
  }
  return 0;
#undef H_
#undef B_
}

// ggschur!(A, B) for real A, B (src/rgeneralized.jl:10-66).  A <- S (quasi-triangular), B <- T,
// Q, Z (n x n, wanted when non-null); alphar + i alphai, beta the eigenvalues alpha ./ beta.
template <class R>
int ggschur_real(int n, R* a, int lda, R* b, int ldb, R* q, R* z, R* alr, R* ali, R* be, bool scale,
                 long long maxiter) {
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * lda]
#define B_(i, j) b[((i) - 1) + (long long)((j) - 1) * ldb]
  R cscale = 1, anrm = 1, cscaleb = 1, bnrm = 1;
  bool scaleA = false, scaleB = false;
  if (scale) {
    scaleA = scale_matrix<R, R>(n, a, lda, &cscale, &anrm);
    scaleB = scale_matrix<R, R>(n, b, ldb, &cscaleb, &bnrm);
  }
  // qr!(B); A <- Q' A; Q = Matrix(Q)
  std::vector<R> tau(n > 0 ? n : 1);
  for (int j = 1; j <= n; ++j) {
    const int m = n - j + 1;
    const R t = reflector_real(&B_(j, j), m);
    tau[j - 1] = t;
    auto apply = [&](R* m0, int ld, int c0, int c1) {
      for (int col = c0; col <= c1; ++col) {
        R* x = m0 + (j - 1) + (long long)(col - 1) * ld;
        R s = x[0];
        for (int r = 1; r < m; ++r) s += B_(j + r, j) * x[r];
        s = t * s;
        x[0] -= s;
        for (int r = 1; r < m; ++r) x[r] -= s * B_(j + r, j);
      }
    };
    apply(b, ldb, j + 1, n);
    apply(a, lda, 1, n);
  }
  if (q) {
    for (int jj = 1; jj <= n; ++jj)
      for (int ii = 1; ii <= n; ++ii) q[(ii - 1) + (long long)(jj - 1) * n] = R(ii == jj ? 1 : 0);
    for (int j = n; j >= 1; --j) {
      const int m = n - j + 1;
      const R t = tau[j - 1];
      for (int col = j; col <= n; ++col) {
        R* x = q + (j - 1) + (long long)(col - 1) * n;
        R s = x[0];
        for (int r = 1; r < m; ++r) s += B_(j + r, j) * x[r];
        s = t * s;
        x[0] -= s;
        for (int r = 1; r < m; ++r) x[r] -= s * B_(j + r, j);
      }
    }
  }
  for (int jj = 1; jj <= n; ++jj)
    for (int ii = jj + 1; ii <= n; ++ii) B_(ii, jj) = R(0);
  if (z)
    for (int jj = 1; jj <= n; ++jj)
      for (int ii = 1; ii <= n; ++ii) z[(ii - 1) + (long long)(jj - 1) * n] = R(ii == jj ? 1 : 0);
  // _hessenberg!(A, B, Q, Z) (src/generalized.jl:84-113)
  for (int jc = 1; jc <= n - 2; ++jc)
    for (int jr = n; jr >= jc + 2; --jr) {
      R c, s, r;
      givens_alg(A_(jr - 1, jc), A_(jr, jc), &c, &s, &r);
      gr_rows(a, lda, jr - 1, jr, c, s, 1, n);
      gr_rows(b, ldb, jr - 1, jr, c, s, 1, n);
      if (q) gr_cols_adj(q, n, jr - 1, jr, c, s, 1, n);
      givens_alg(B_(jr, jr), B_(jr, jr - 1), &c, &s, &r);
      gr_cols_adj(a, lda, jr, jr - 1, c, s, 1, n);
      gr_cols_adj(b, ldb, jr, jr - 1, c, s, 1, n);
      if (z) gr_cols_adj(z, n, jr, jr - 1, c, s, 1, n);
    }
  for (int jj = 1; jj <= n; ++jj)
    for (int ii = 1; ii <= n; ++ii) {
      if (ii > jj + 1) A_(ii, jj) = R(0);
      if (ii > jj) B_(ii, jj) = R(0);
    }
  const int st = gqz_real<R>(n, a, lda, b, ldb, q, n, z, n, alr, ali, be, maxiter);
  if (scaleA) {
    for (int jj = 1; jj <= n; ++jj) safescale<R, R>(a + (long long)(jj - 1) * lda, n, cscale, anrm);
    safescale<R, R>(alr, n, cscale, anrm);
    safescale<R, R>(ali, n, cscale, anrm);
  }
  if (scaleB) {
    for (int jj = 1; jj <= n; ++jj) safescale<R, R>(b + (long long)(jj - 1) * ldb, n, cscaleb, bnrm);
    safescale<R, R>(be, n, cscaleb, bnrm);
  }
  return st;
#undef A_
#undef B_
}


// ---------------------------------------------------------------------------
// Eigenvectors of a real generalized Schur pair (S quasi-triangular, P upper triangular),
// the reference's dtgevc restatements in complex arithmetic:
//   right _geigvecs(S, P[, Z])   src/vectors.jl:1040-1283
//   left  _gleigvecs(S, P[, Q])  src/vectors.jl:1285-1513
// with _xsolve (src/util.jl:698-751) for the 1 x 1 / 2 x 2 diagonal blocks.
// ---------------------------------------------------------------------------

// _xsolve(a, A, d, b, B, smin): (a A - b D) X = s B, A na x na real (column-major, ld na),
// D = diag(d), b complex; B overwritten with X; returns s.
template <class R>
R xsolve_gen(R a, const R* A, int na, const R* d, cx<R> b, cx<R>* B, R smin, R* xnorm, bool* perturbed) {
  typedef cx<R> C;
  R s = 1;
  const R small = R(2) * safemin<R>();
  const R bignum = s / small;
  smin = m_max(smin, small);
  *perturbed = false;
  if (na == 1) {
    R csr = a * A[0] - b.re * d[0];
    R csi = -b.im * d[0];
    R cnorm = m_abs(csr) + m_abs(csi);
    if (cnorm < smin) { *perturbed = true; csr = smin; csi = 0; cnorm = smin; }
    const R bnorm = abs1(B[0]);
    if (cnorm < R(1) && bnorm > R(1) && bnorm > bignum * cnorm) s = R(1) / bnorm;
    const C x = (B[0] * s) / C(csr, csi);
    *xnorm = abs1(x);
    B[0] = x;
    return s;
  }
  R cmax = 0;
  C m[4];
  for (int j = 1; j <= na; ++j)
    for (int i = 1; i <= na; ++i) {
      C zz = C(a * A[(i - 1) + (j - 1) * na]);
      if (i == j) zz -= b * d[i - 1];
      m[(i - 1) + (j - 1) * na] = zz;
      cmax = m_max(cmax, abs1(zz));
    }
  if (cmax < smin) {
    *perturbed = true;
    R bnorm = 0;
    for (int i = 0; i < na; ++i) bnorm = m_max(bnorm, abs1(B[i]));
    if (smin < R(1) && bnorm > R(1) && bnorm > bignum * smin) s = R(1) / bnorm;
    const R t1 = s / smin;
    for (int i = 0; i < na; ++i) B[i] *= t1;
  } else {
    bool pert2 = false;
    s = safe_lu_solve<R>(na, m, B, &pert2);
  }
  *xnorm = norm2_cplx(B, na);
  return s;
}

// scaled coefficients of a real eigenvalue k (vectors.jl:1097-1139 / 1336-1378)
template <class R>
void rg_coeffs_real(const R* S, const R* P, int n, int k, R Anorm, R Bnorm, R ascale, R bscale, R* ao, R* bro) {
  const R ulp = std::numeric_limits<R>::epsilon();
  const R safmin = safemin<R>();
  const R smallnum = safmin * (R(n) / ulp);
  const R bigx = R(1) / smallnum;
  const R skk = S[(k - 1) + (long long)(k - 1) * n], pkk = P[(k - 1) + (long long)(k - 1) * n];
  const R t = R(1) / m_max(m_max(m_abs(skk) * ascale, m_abs(pkk) * bscale), safmin);
  const R sar = (t * skk) * ascale;
  const R sb = (t * pkk) * bscale;
  R a = sb * ascale, br = sar * bscale;
  const bool lsa = m_abs(sb) >= safmin && m_abs(a) < smallnum;
  const bool lsb = m_abs(sar) >= safmin && m_abs(br) < smallnum;
  R s = R(1);
  if (lsa) s = (smallnum / m_abs(sb)) * m_min(Anorm, bigx);
  if (lsb) s = m_max(s, (smallnum / m_abs(sar)) * m_min(Bnorm, bigx));
  if (lsa || lsb) {
    s = m_min(s, R(1) / (safmin * m_max(m_max(R(1), m_abs(a)), m_abs(br))));
    a = lsa ? ascale * (s * sb) : a * s;
    br = lsb ? bscale * (s * sar) : br * s;
  }
  *ao = a;
  *bro = br;
}

// scaling of a complex pair's (a, br, bi) (vectors.jl:1163-1183 / 1401-1421)
template <class R>
void rg_scale_pair(R* a, R* br, R* bi, R ascale, R bscale) {
  const R ulp = std::numeric_limits<R>::epsilon();
  const R safmin = safemin<R>();
  const R aa = m_abs(*a), ba = m_abs(*br) + m_abs(*bi);
  R scale = R(1);
  if (aa * ulp < safmin && aa >= safmin) scale = (safmin / ulp) / aa;
  if (ba * ulp < safmin && ba >= safmin) scale = m_max(scale, (safmin / ulp) / ba);
  if (safmin * aa > ascale) scale = ascale / (safmin * aa);
  if (safmin * ba > bscale) scale = m_min(scale, bscale / (safmin * ba));
  if (scale != R(1)) { *a *= scale; *br *= scale; *bi *= scale; }
}

template <class R>
void rg_norms(int n, const R* S, const R* P, std::vector<R>& sn, std::vector<R>& pn, R* An, R* Bn) {
  sn.assign(n, R(0));
  pn.assign(n, R(0));
  R a = m_abs(S[0]), b = m_abs(P[0]);
  for (int j = 2; j <= n; ++j) {
    for (int i = 1; i <= j - 1; ++i) {
      sn[j - 1] += m_abs(S[(i - 1) + (long long)(j - 1) * n]);
      pn[j - 1] += m_abs(P[(i - 1) + (long long)(j - 1) * n]);
    }
    a = m_max(a, sn[j - 1] + m_abs(S[(j - 1) + (long long)(j - 1) * n]));
    b = m_max(b, pn[j - 1] + m_abs(P[(j - 1) + (long long)(j - 1) * n]));
  }
  *An = a;
  *Bn = b;
}

template <class R>
void rgevc_right(int n, const R* S, const R* P, const R* Z, cx<R>* V) {
  typedef cx<R> C;
  const R ulp = std::numeric_limits<R>::epsilon();
  const R safmin = safemin<R>();
  const R bignum = R(1) / (R(n) * safmin);
  const R safety = R(100);
  std::vector<R> sn, pn;
  R Anorm, Bnorm;
  rg_norms(n, S, P, sn, pn, &Anorm, &Bnorm);
  const R ascale = R(1) / m_max(Anorm, safmin), bscale = R(1) / m_max(Bnorm, safmin);
  std::vector<C> v(n);
#define SS(i, j) S[((i) - 1) + (long long)((j) - 1) * n]
#define PP(i, j) P[((i) - 1) + (long long)((j) - 1) * n]
  int idx = n + 1;
  bool inpair = false;
  for (int je = n; je >= 1; --je) {
    if (inpair) { inpair = false; continue; }
    int nw = 1;
    if (je > 1 && SS(je, je - 1) != R(0)) { inpair = true; nw = 2; }
    R a, br, bi, aa, ba, xmax;
    if (!inpair) {
      if (m_abs(SS(je, je)) <= safmin && m_abs(PP(je, je)) <= safmin) {
        idx -= 1;
        cx<R>* col = V + (long long)(idx - 1) * n;
        for (int r = 0; r < n; ++r) col[r] = C(R(0));
        col[idx - 1] = C(R(1));
        continue;
      }
      rg_coeffs_real(S, P, n, je, Anorm, Bnorm, ascale, bscale, &a, &br);
      bi = R(0);
      aa = m_abs(a);
      ba = m_abs(br);
      for (int r = 0; r < n; ++r) v[r] = C(R(0));
      v[je - 1] = C(R(1));
      xmax = R(1);
      for (int jr = 1; jr <= je - 1; ++jr) v[jr - 1] = C(br * PP(jr, je) - a * SS(jr, je));
    } else {
      R s1, s2, wr1, wr2, wi;
      ggs_2x2(&SS(je - 1, je - 1), n, &PP(je - 1, je - 1), n, safmin * safety, &s1, &s2, &wr1, &wr2, &wi);
      a = s1;
      br = wr1;
      bi = wi;
      rg_scale_pair(&a, &br, &bi, ascale, bscale);
      aa = m_abs(a);
      ba = m_abs(br) + m_abs(bi);
      for (int r = 0; r < n; ++r) v[r] = C(R(0));
      R t1 = a * SS(je, je - 1);
      const R t2r = a * SS(je, je) - br * PP(je, je), t2i = -bi * PP(je, je);
      if (m_abs(t1) > m_abs(t2r) + m_abs(t2i)) {
        v[je - 1] = C(R(1));
        v[je - 2] = -(C(t2r, t2i)) / C(t1);
      } else {
        v[je - 2] = C(R(1));
        t1 = a * SS(je - 1, je);
        v[je - 1] = C((br * PP(je - 1, je - 1) - a * SS(je - 1, je - 1)) / t1, bi * PP(je - 1, je - 1) / t1);
      }
      xmax = m_max(abs1(v[je - 1]), abs1(v[je - 2]));
      const C bc(br, bi);
      const C ca = a * v[je - 2], cb = bc * v[je - 2], c2a = a * v[je - 1], c2b = bc * v[je - 1];
      for (int jr = 1; jr <= je - 2; ++jr)
        v[jr - 1] = -ca * SS(jr, je - 1) + cb * PP(jr, je - 1) - c2a * SS(jr, je) + c2b * PP(jr, je);
    }
    const R dmin = m_max(m_max(ulp * aa * Anorm, ulp * ba * Bnorm), safmin);
    const C bc(br, bi);
    bool in2x2 = false;
    for (int j = je - nw; j >= 1; --j) {
      if (!in2x2 && j > 1 && SS(j, j - 1) != R(0)) { in2x2 = true; continue; }
      const int na = in2x2 ? 2 : 1;
      R dg[2] = {PP(j, j), na == 2 ? PP(j + 1, j + 1) : R(0)};
      R blk[4];
      for (int q = 0; q < na; ++q)
        for (int p = 0; p < na; ++p) blk[p + q * na] = SS(j + p, j + q);
      C x[2] = {v[j - 1], na == 2 ? v[j] : C(R(0))};
      R t1;
      bool pert;
      const R scale = xsolve_gen<R>(a, blk, na, dg, bc, x, dmin, &t1, &pert);
      // _xsolve overwrites its right-hand side, a view of v (vectors.jl:1229-1236), so the
      // rescaling of v[1:je] that follows also applies to the new solution entries
      for (int q = 0; q < na; ++q) v[j - 1 + q] = x[q];
      if (scale < R(1))
        for (int r = 0; r < je; ++r) v[r] = scale * v[r];
      xmax = m_max(scale * xmax, t1);
      if (j > 1) {
        const R xscale = R(1) / m_max(R(1), xmax);
        t1 = m_max(t1, aa * sn[j - 1] + ba * pn[j - 1]);
        if (in2x2) t1 = m_max(t1, aa * sn[j] + ba * pn[j]);
        t1 = m_max(m_max(t1, aa), ba);
        if (t1 > bignum * xscale) {
          for (int r = 0; r < je; ++r) v[r] = xscale * v[r];
          xmax *= xscale;
        }
        for (int ja = 1; ja <= na; ++ja) {
          const C ca = a * v[j + ja - 2], cb = bc * v[j + ja - 2];
          for (int i = 1; i <= j - 1; ++i) v[i - 1] = v[i - 1] - ca * SS(i, j + ja - 1) + cb * PP(i, j + ja - 1);
        }
      }
      in2x2 = false;
    }
    idx -= nw;
    cx<R>* col = V + (long long)(idx - 1) * n;
    int iend;
    if (Z) {
      for (int r = 0; r < n; ++r) {
        C acc(R(0));
        for (int k = 0; k < n; ++k) acc += Z[r + (long long)k * n] * v[k];
        col[r] = acc;
      }
      iend = n;
    } else {
      for (int r = 0; r < n; ++r) col[r] = v[r];
      iend = je;
    }
    for (int jr = 1; jr <= iend; ++jr) xmax = m_max(xmax, abs1(col[jr - 1]));
    if (xmax > safmin) {
      const R xs = R(1) / xmax;
      for (int jr = 1; jr <= iend; ++jr) col[jr - 1] = xs * col[jr - 1];
    }
    if (inpair) {
      cx<R>* col2 = V + (long long)idx * n;
      for (int r = 0; r < n; ++r) col2[r] = conj(col[r]);
    }
  }
#undef SS
#undef PP
}

template <class R>
void rgevc_left(int n, const R* S, const R* P, const R* Q, cx<R>* V) {
  typedef cx<R> C;
  const R ulp = std::numeric_limits<R>::epsilon();
  const R safmin = safemin<R>();
  const R bignum = R(1) / (R(n) * safmin);
  const R safety = R(100);
  std::vector<R> sn, pn;
  R Anorm, Bnorm;
  rg_norms(n, S, P, sn, pn, &Anorm, &Bnorm);
  const R ascale = R(1) / m_max(Anorm, safmin), bscale = R(1) / m_max(Bnorm, safmin);
  std::vector<C> v(n);
#define SS(i, j) S[((i) - 1) + (long long)((j) - 1) * n]
#define PP(i, j) P[((i) - 1) + (long long)((j) - 1) * n]
  int idx = 0;
  bool inpair = false;
  for (int je = 1; je <= n; ++je) {
    if (inpair) { inpair = false; continue; }
    int nw = 1;
    if (je < n && SS(je + 1, je) != R(0)) { inpair = true; nw = 2; }
    R a, br, bi, aa, ba, xmax;
    if (!inpair) {
      if (m_abs(SS(je, je)) <= safmin && m_abs(PP(je, je)) <= safmin) {
        idx += 1;
        cx<R>* col = V + (long long)(idx - 1) * n;
        for (int r = 0; r < n; ++r) col[r] = C(R(0));
        col[idx - 1] = C(R(1));
        continue;
      }
      rg_coeffs_real(S, P, n, je, Anorm, Bnorm, ascale, bscale, &a, &br);
      bi = R(0);
      aa = m_abs(a);
      ba = m_abs(br);
      for (int r = 0; r < n; ++r) v[r] = C(R(0));
      v[je - 1] = C(R(1));
      xmax = R(1);
    } else {
      R s1, s2, wr1, wr2, wi;
      ggs_2x2(&SS(je, je), n, &PP(je, je), n, safmin * safety, &s1, &s2, &wr1, &wr2, &wi);
      a = s1;
      br = wr1;
      bi = -wi;
      rg_scale_pair(&a, &br, &bi, ascale, bscale);
      aa = m_abs(a);
      ba = m_abs(br) + m_abs(bi);
      for (int r = 0; r < n; ++r) v[r] = C(R(0));
      R t1 = a * SS(je + 1, je);
      const R t2r = a * SS(je, je) - br * PP(je, je), t2i = -bi * PP(je, je);
      if (m_abs(t1) > m_abs(t2r) + m_abs(t2i)) {
        v[je - 1] = C(R(1));
        v[je] = -(C(t2r, t2i)) / C(t1);
      } else {
        v[je] = C(R(1));
        t1 = a * SS(je, je + 1);
        v[je - 1] = C((br * PP(je + 1, je + 1) - a * SS(je + 1, je + 1)) / t1, bi * PP(je + 1, je + 1) / t1);
      }
      xmax = m_max(abs1(v[je - 1]), abs1(v[je]));
    }
    const R dmin = m_max(m_max(ulp * aa * Anorm, ulp * ba * Bnorm), safmin);
    const C bc(br, bi);
    bool in2x2 = false;
    for (int j = je + nw; j <= n; ++j) {
      if (in2x2) { in2x2 = false; continue; }
      int na = 1;
      if (j < n && SS(j + 1, j) != R(0)) { in2x2 = true; na = 2; }
      R dg[2] = {PP(j, j), na == 2 ? PP(j + 1, j + 1) : R(0)};
      const R xscale = R(1) / m_max(R(1), xmax);
      R t1 = m_max(m_max(sn[j - 1], pn[j - 1]), aa * sn[j - 1] + ba * sn[j - 1]);
      if (in2x2) t1 = m_max(m_max(t1, sn[j]), m_max(pn[j], aa * sn[j] + ba * sn[j]));
      if (t1 > bignum * xscale) {
        for (int r = je; r <= j - 1; ++r) v[r - 1] = v[r - 1] * xscale;
        xmax *= xscale;
      }
      C sumS[2] = {C(R(0)), C(R(0))}, sumP[2] = {C(R(0)), C(R(0))};
      const int jx = j + na - 1;
      for (int jr = je; jr <= j - 1; ++jr)
        for (int q = 0; q <= jx - j; ++q) {
          sumS[q] = sumS[q] + SS(jr, j + q) * v[jr - 1];
          sumP[q] = sumP[q] + PP(jr, j + q) * v[jr - 1];
        }
      C y[2];
      for (int q = 0; q < na; ++q) y[q] = -a * sumS[q] + bc * sumP[q];
      // the block of S', i.e. the transposed block of S
      R blk[4];
      for (int q = 0; q < na; ++q)
        for (int p = 0; p < na; ++p) blk[p + q * na] = SS(j + q, j + p);
      bool pert;
      const R scale = xsolve_gen<R>(a, blk, na, dg, bc, y, dmin, &t1, &pert);
      for (int q = 0; q < na; ++q) v[j - 1 + q] = y[q];
      if (scale < R(1)) {
        for (int r = je; r <= j - 1; ++r) v[r - 1] = scale * v[r - 1];
        xmax *= scale;
      }
      xmax = m_max(xmax, t1);
    }
    idx += 1;
    cx<R>* col = V + (long long)(idx - 1) * n;
    int ibegin;
    if (Q) {
      for (int r = 0; r < n; ++r) {
        C acc(R(0));
        for (int k = 0; k < n; ++k) acc += Q[r + (long long)k * n] * v[k];
        col[r] = acc;
      }
      ibegin = 1;
    } else {
      for (int r = 0; r < n; ++r) col[r] = v[r];
      ibegin = je;
    }
    xmax = R(0);
    for (int jr = ibegin; jr <= n; ++jr) xmax = m_max(xmax, abs1(col[jr - 1]));
    if (xmax > safmin) {
      const R xs = R(1) / xmax;
      for (int jr = ibegin; jr <= n; ++jr) col[jr - 1] = xs * col[jr - 1];
    }
    if (inpair) {
      cx<R>* col2 = V + (long long)idx * n;
      for (int r = 0; r < n; ++r) col2[r] = conj(col[r]);
    }
    idx += nw - 1;
  }
#undef SS
#undef PP
}


// ---------------------------------------------------------------------------
// Reordering a complex generalized Schur form: gordschur!(S, T, Q, Z, select)
// (src/ordschur.jl:147-305): _trexchange! by adjacent swaps _trexch2! (ztgex2 with the
// weak and strong stability tests).  Returns 0, or 1 + (1-based j1) of a rejected swap
// (the reference's IllConditionException).
// ---------------------------------------------------------------------------
// _safe_fnorm(vec(W)) (util.jl:83-94 with _ssq 466-505): real and imaginary parts, the
// running scale starting at 1.
template <class R> R safe_fnorm_c(const cx<R>* w, int cnt) {
  R scale = R(1), sumsq = R(0);
  for (int i = 0; i < cnt; ++i) {
    const R parts[2] = {m_abs(w[i].re), m_abs(w[i].im)};
    for (R t1 : parts) {
      if (t1 > R(0) || t1 != t1) {
        if (scale < t1) { sumsq = R(1) + sumsq * (scale / t1) * (scale / t1); scale = t1; }
        else sumsq += (t1 / scale) * (t1 / scale);
      }
    }
  }
  return scale * m_sqrt(sumsq);
}

template <class R>
bool trexch2_cplx(int n, cx<R>* A, cx<R>* B, cx<R>* Q, cx<R>* Z, int j1) {
  typedef cx<R> C;
#define A_(i, j) A[((i) - 1) + (long long)((j) - 1) * n]
#define B_(i, j) B[((i) - 1) + (long long)((j) - 1) * n]
  C S[4] = {A_(j1, j1), A_(j1 + 1, j1), A_(j1, j1 + 1), A_(j1 + 1, j1 + 1)};  // column-major 2 x 2
  C T[4] = {B_(j1, j1), B_(j1 + 1, j1), B_(j1, j1 + 1), B_(j1 + 1, j1 + 1)};
  const R eps = std::numeric_limits<R>::epsilon();
  const R smlnum = safemin<R>() / eps;
  C W[8] = {S[0], S[1], S[2], S[3], T[0], T[1], T[2], T[3]};
  R sa = safe_fnorm_c(W, 8);
  const R thresh = m_max(R(20) * eps * sa, smlnum);
  const C f = S[3] * T[0] - T[3] * S[0];
  const C g = S[3] * T[2] - T[3] * S[2];
  sa = cabs(S[3]) * cabs(T[0]);
  const R sb = cabs(S[0]) * cabs(T[3]);
  R cz;
  C sz;
  if (f == C(R(0)) && g == C(R(0))) { cz = R(0); sz = C(R(1)); }
  else { C r; zgivens_alg(g, f, &cz, &sz, &r); }
  // rmul!(M, Givens(1, 2, cz, sz)): [m1 m2] <- [m1 cz - m2 conj(sz), m1 sz + m2 cz]
  auto rz = [&](C* M, R c, C sv) {
    for (int r = 0; r < 2; ++r) {
      const C m1 = M[r], m2 = M[r + 2];
      M[r] = m1 * c - m2 * conj(sv);
      M[r + 2] = m1 * sv + m2 * c;
    }
  };
  // lmul!(Givens(1, 2, c, s), M): [m1; m2] <- [c m1 + s m2; -conj(s) m1 + c m2]
  auto lq = [&](C* M, R c, C sv) {
    for (int k = 0; k < 2; ++k) {
      const C m1 = M[2 * k], m2 = M[2 * k + 1];
      M[2 * k] = m1 * c + sv * m2;
      M[2 * k + 1] = m2 * c - conj(sv) * m1;
    }
  };
  rz(S, cz, sz);
  rz(T, cz, sz);
  C fq, gq;
  if (sa >= sb) { fq = S[0]; gq = S[1]; } else { fq = T[0]; gq = T[1]; }
  R cq;
  C sq;
  if (sz != C(R(0)) && fq == C(R(0)) && gq == C(R(0))) { cq = R(0); sq = C(R(1)); }
  else { C r; zgivens_alg(fq, gq, &cq, &sq, &r); }
  lq(S, cq, sq);
  lq(T, cq, sq);
  const R ws = cabs(S[1]) + cabs(T[1]);
  if (!(ws <= thresh)) return false;
  // strong test: undo the rotations on copies and compare with the original block
  C Ss[4] = {S[0], S[1], S[2], S[3]}, Ts[4] = {T[0], T[1], T[2], T[3]};
  rz(Ss, cz, -sz);
  rz(Ts, cz, -sz);
  lq(Ss, cq, -sq);
  lq(Ts, cq, -sq);
  const C orig[8] = {A_(j1, j1), A_(j1 + 1, j1), A_(j1, j1 + 1), A_(j1 + 1, j1 + 1),
                     B_(j1, j1), B_(j1 + 1, j1), B_(j1, j1 + 1), B_(j1 + 1, j1 + 1)};
  for (int k = 0; k < 4; ++k) { W[k] = Ss[k] - orig[k]; W[4 + k] = Ts[k] - orig[4 + k]; }
  const R ss = safe_fnorm_c(W, 8);
  if (!(ss <= thresh)) return false;
  // apply: rmul!(A, Gz'), rmul!(B, Gz') on all rows; lmul!(Gq, A), lmul!(Gq, B) on all columns
  for (int r = 1; r <= n; ++r) {
    C m1 = A_(r, j1), m2 = A_(r, j1 + 1);
    A_(r, j1) = m1 * cz - m2 * conj(sz);
    A_(r, j1 + 1) = m1 * sz + m2 * cz;
    m1 = B_(r, j1); m2 = B_(r, j1 + 1);
    B_(r, j1) = m1 * cz - m2 * conj(sz);
    B_(r, j1 + 1) = m1 * sz + m2 * cz;
  }
  for (int c = 1; c <= n; ++c) {
    C m1 = A_(j1, c), m2 = A_(j1 + 1, c);
    A_(j1, c) = m1 * cq + sq * m2;
    A_(j1 + 1, c) = m2 * cq - conj(sq) * m1;
    m1 = B_(j1, c); m2 = B_(j1 + 1, c);
    B_(j1, c) = m1 * cq + sq * m2;
    B_(j1 + 1, c) = m2 * cq - conj(sq) * m1;
  }
  A_(j1 + 1, j1) = C(R(0));
  B_(j1 + 1, j1) = C(R(0));
  // rmul!(Z, Gz') and rmul!(Q, Gq')
  for (int r = 0; r < n; ++r) {
    C* z1 = Z + r + (long long)(j1 - 1) * n;
    C* z2 = Z + r + (long long)j1 * n;
    C m1 = *z1, m2 = *z2;
    *z1 = m1 * cz - m2 * conj(sz);
    *z2 = m1 * sz + m2 * cz;
    C* q1 = Q + r + (long long)(j1 - 1) * n;
    C* q2 = Q + r + (long long)j1 * n;
    m1 = *q1; m2 = *q2;
    *q1 = m1 * cq + m2 * conj(sq);
    *q2 = m2 * cq - m1 * sq;
  }
  return true;
#undef A_
#undef B_
}

template <class R>
int gordschur_cplx(int n, cx<R>* S, cx<R>* T, cx<R>* Q, cx<R>* Z, const int* select, bool scale, cx<R>* alpha,
                   cx<R>* beta) {
  R cscale = 1, anrm = 1, cscaleb = 1, bnrm = 1;
  bool scA = false, scB = false;
  if (scale) {
    scA = scale_matrix<R, cx<R>>(n, S, n, &cscale, &anrm);
    scB = scale_matrix<R, cx<R>>(n, T, n, &cscaleb, &bnrm);
  }
  int status = 0;
  int ks = 0;
  for (int k = 1; k <= n && !status; ++k) {
    if (!select[k - 1]) continue;
    ks += 1;
    if (k != ks)
      for (int icur = k - 1; icur >= ks; --icur)
        if (!trexch2_cplx<R>(n, S, T, Q, Z, icur)) { status = 1 + icur; break; }
  }
  if (scA) for (int j = 0; j < n; ++j) safescale<R, cx<R>>(S + (long long)j * n, n, cscale, anrm);
  if (scB) for (int j = 0; j < n; ++j) safescale<R, cx<R>>(T + (long long)j * n, n, cscaleb, bnrm);
  for (int j = 0; j < n; ++j)
    for (int i = j + 1; i < n; ++i) {
      S[i + (long long)j * n] = cx<R>(R(0));
      T[i + (long long)j * n] = cx<R>(R(0));
    }
  for (int i = 0; i < n; ++i) {
    alpha[i] = S[i + (long long)i * n];
    beta[i] = T[i + (long long)i * n];
  }
  return status;
}

// ---------------------------------------------------------------------------
// Reordering of real generalized Schur forms: gordschur!(S, T, Q, Z, select) for real
// pencils (rordschur.jl:542-627), _trexchange! (629-766, its move-up branch: gordschur!
// only moves blocks up), _swap1or2! (768-962), _gqz_2x2! (964-1063), _syl1or2 (1071-1091),
// _rtrexch2! (1096-1178).  Kept from the reference: `nbold == 3` (a comparison, so a 2 x 2
// block that splits keeps nbold = 2, 717-721), t2 computed from A as t1 is in _gqz_2x2!
// (1023-1024), the singular-B1 branch rotating columns (991-993).  The QR and RQ
// factorizations (LinearAlgebra.qr / MatrixFactorizations.rq, LAPACK geqrt / gerqf for
// Float64) are restated with LAPACK's reflector convention (dlarfg) and formed explicitly.
// ---------------------------------------------------------------------------
// _safe_fnorm of a rows x cols block (columns in order; util.jl:83-94 with _ssq 466-505)
template <class R> R safe_fnorm_r(const R* m, int ld, int rows, int cols) {
  R scale = R(1), sumsq = R(0);
  for (int j = 0; j < cols; ++j)
    for (int i = 0; i < rows; ++i) {
      const R t1 = m_abs(m[i + (long long)j * ld]);
      if (t1 > R(0) || t1 != t1) {
        if (scale < t1) { sumsq = R(1) + sumsq * (scale / t1) * (scale / t1); scale = t1; }
        else sumsq += (t1 / scale) * (t1 / scale);
      }
    }
  return scale * m_sqrt(sumsq);
}

// dlarfg: H (I - tau v v', v = [1; x]) with H [alpha; x] = [beta; 0]; x has n - 1 entries
// at stride inc; alpha becomes beta, x becomes v's tail; returns tau.
template <class R> R larfg_r(int n, R* alpha, R* x, int inc) {
  if (n <= 1) return R(0);
  auto nrm2 = [&]() {
    R sc = R(0), sq = R(1);
    for (int i = 0; i < n - 1; ++i) {
      const R a = m_abs(x[i * inc]);
      if (a > R(0)) {
        if (sc < a) { sq = R(1) + sq * (sc / a) * (sc / a); sc = a; }
        else sq += (a / sc) * (a / sc);
      }
    }
    return sc * m_sqrt(sq);
  };
  R xnorm = nrm2();
  if (xnorm == R(0)) return R(0);
  R beta = -m_copysign(m_hypot(*alpha, xnorm), *alpha);
  const R sfmin = lim<R>::fmin() / lim<R>::eps();
  int knt = 0;
  if (m_abs(beta) < sfmin) {
    const R rsfmn = R(1) / sfmin;
    do {
      ++knt;
      for (int i = 0; i < n - 1; ++i) x[i * inc] *= rsfmn;
      beta *= rsfmn;
      *alpha *= rsfmn;
    } while (m_abs(beta) < sfmin && knt < 20);
    xnorm = nrm2();
    beta = -m_copysign(m_hypot(*alpha, xnorm), *alpha);
  }
  const R tau = (beta - *alpha) / beta;
  const R sc = R(1) / (*alpha - beta);
  for (int i = 0; i < n - 1; ++i) x[i * inc] *= sc;
  for (int j = 0; j < knt; ++j) beta *= sfmin;
  *alpha = beta;
  return tau;
}

// QR of the m x k matrix a (ld m, k <= m): R in the upper triangle, Q (m x m) formed
template <class R> void house_qr_r(int m, int k, R* a, R* q) {
  std::vector<R> tau(k), w(m);
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * m]
  for (int i = 1; i <= k; ++i) {
    tau[i - 1] = larfg_r<R>(m - i + 1, &A_(i, i), i < m ? &A_(i + 1, i) : &A_(i, i), 1);
    if (i < k && tau[i - 1] != R(0)) {
      const R aii = A_(i, i);
      A_(i, i) = R(1);
      for (int j = i + 1; j <= k; ++j) {
        R t = R(0);
        for (int r = i; r <= m; ++r) t += A_(r, i) * A_(r, j);
        for (int r = i; r <= m; ++r) A_(r, j) -= tau[i - 1] * A_(r, i) * t;
      }
      A_(i, i) = aii;
    }
  }
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) q[i + (long long)j * m] = i == j ? R(1) : R(0);
  for (int i = k; i >= 1; --i) {
    if (tau[i - 1] == R(0)) continue;
    for (int j = 1; j <= m; ++j) {
      R t = q[(i - 1) + (long long)(j - 1) * m];
      for (int r = i + 1; r <= m; ++r) t += A_(r, i) * q[(r - 1) + (long long)(j - 1) * m];
      t *= tau[i - 1];
      q[(i - 1) + (long long)(j - 1) * m] -= t;
      for (int r = i + 1; r <= m; ++r) q[(r - 1) + (long long)(j - 1) * m] -= A_(r, i) * t;
    }
  }
  for (int j = 1; j <= k; ++j)
    for (int i = j + 1; i <= m; ++i) A_(i, j) = R(0);
#undef A_
}

// RQ of the mr x n matrix a (ld mr, mr <= n): a = R Q, R (mr x n) upper trapezoidal in the
// last mr columns, Q (n x n) = H(1) ... H(k) formed
template <class R> void house_rq_r(int mr, int n, R* a, R* q) {
  const int k = mr < n ? mr : n;
  std::vector<R> tau(k);
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * mr]
  for (int i = k; i >= 1; --i) {
    const int row = mr - k + i, col = n - k + i;
    tau[i - 1] = larfg_r<R>(col, &A_(row, col), &A_(row, 1), mr);
    if (tau[i - 1] != R(0) && row > 1) {
      const R aii = A_(row, col);
      A_(row, col) = R(1);
      for (int r = 1; r <= row - 1; ++r) {
        R t = R(0);
        for (int c = 1; c <= col; ++c) t += A_(r, c) * A_(row, c);
        for (int c = 1; c <= col; ++c) A_(r, c) -= tau[i - 1] * t * A_(row, c);
      }
      A_(row, col) = aii;
    }
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) q[i + (long long)j * n] = i == j ? R(1) : R(0);
  for (int i = k; i >= 1; --i) {
    const int row = mr - k + i, col = n - k + i;
    if (tau[i - 1] == R(0)) continue;
    // Q = H(i) Q; v = [A(row, 1:col-1); 1]
    for (int j = 1; j <= n; ++j) {
      R t = q[(col - 1) + (long long)(j - 1) * n];
      for (int c = 1; c <= col - 1; ++c) t += A_(row, c) * q[(c - 1) + (long long)(j - 1) * n];
      t *= tau[i - 1];
      q[(col - 1) + (long long)(j - 1) * n] -= t;
      for (int c = 1; c <= col - 1; ++c) q[(c - 1) + (long long)(j - 1) * n] -= A_(row, c) * t;
    }
  }
  // R: zero what lies left of the trapezoid's diagonal
  for (int i = 1; i <= mr; ++i)
    for (int j = 1; j <= n; ++j)
      if (j < n - mr + i) A_(i, j) = R(0);
#undef A_
}

// small dense products (column-major): C = op(A) op(B)
template <class R> void mm_r(int m, int nn, int kk, const R* A, bool ta, const R* B, bool tb, R* C) {
  for (int j = 0; j < nn; ++j)
    for (int i = 0; i < m; ++i) {
      R t = R(0);
      for (int l = 0; l < kk; ++l) {
        const R a = ta ? A[l + (long long)i * kk] : A[i + (long long)l * m];
        const R b = tb ? B[j + (long long)l * nn] : B[l + (long long)j * kk];
        t += a * b;
      }
      C[i + (long long)j * m] = t;
    }
}

// _gqz_2x2!(A, B) on the 2 x 2 blocks at a, b (ld): standardizes in place, returns the
// rotations (csl, snl, csr, snr)
template <class R> void gqz_2x2_r(R* a, R* b, int ld, R* cslo, R* snlo, R* csro, R* snro) {
#define GA(i, j) a[((i) - 1) + (long long)((j) - 1) * ld]
#define GB(i, j) b[((i) - 1) + (long long)((j) - 1) * ld]
  const R safmin = lim<R>::fmin(), ulp = lim<R>::eps();
  const R anorm = m_max(m_max(m_abs(GA(1, 1)) + m_abs(GA(2, 1)), m_abs(GA(1, 2)) + m_abs(GA(2, 2))), safmin);
  const R ascale = R(1) / anorm;
  for (int j = 1; j <= 2; ++j) for (int i = 1; i <= 2; ++i) GA(i, j) *= ascale;
  const R bnorm = m_max(m_max(m_abs(GB(1, 1)), m_abs(GB(1, 2)) + m_abs(GB(2, 2))), safmin);
  const R bscale = R(1) / bnorm;
  for (int j = 1; j <= 2; ++j) for (int i = 1; i <= 2; ++i) GB(i, j) *= bscale;
  R csl, snl, csr, snr, rr;
  if (m_abs(GA(2, 1)) < ulp) {
    csl = 1; snl = 0; csr = 1; snr = 0;
    GA(2, 1) = 0;
    GB(2, 1) = 0;
  } else if (m_abs(GB(1, 1)) < ulp) {
    givens_alg<R>(GA(1, 1), GA(2, 1), &csl, &snl, &rr);
    csr = 1; snr = 0;
    gr_cols<R>(a, ld, 1, 2, csl, snl, 1, 2);
    gr_cols<R>(b, ld, 1, 2, csl, snl, 1, 2);
    GA(2, 1) = 0;
    GB(1, 1) = 0;
    GB(2, 1) = 0;
  } else if (m_abs(GB(2, 2)) < ulp) {
    givens_alg<R>(GA(2, 2), GA(2, 1), &csr, &snr, &rr);
    gr_rows<R>(a, ld, 1, 2, csr, -snr, 1, 2);
    gr_rows<R>(b, ld, 1, 2, csr, -snr, 1, 2);
    csl = 1; snl = 0;
    GA(2, 1) = 0;
    GB(2, 1) = 0;
    GB(2, 2) = 0;
  } else {
    R scale1, scale2, wr1, wr2, wi;
    ggs_2x2<R>(a, ld, b, ld, safmin, &scale1, &scale2, &wr1, &wr2, &wi);
    if (wi == R(0)) {
      const R h1 = scale1 * GA(1, 1) - wr1 * GB(1, 1);
      const R h2 = scale1 * GA(1, 2) - wr1 * GB(1, 2);
      const R h3 = scale1 * GA(2, 2) - wr1 * GB(2, 2);
      const R rr2 = m_hypot(h2, h1);
      const R qq = m_hypot(scale1 * GA(2, 1), h3);
      if (rr2 > qq) givens_alg<R>(h2, h1, &csr, &snr, &rr);
      else givens_alg<R>(h3, scale1 * GA(2, 1), &csr, &snr, &rr);
      gr_cols<R>(a, ld, 1, 2, csr, snr, 1, 2);
      gr_cols<R>(b, ld, 1, 2, csr, snr, 1, 2);
      snr = -snr;
      const R t1 = m_max(m_abs(GA(1, 1)) + m_abs(GA(1, 2)), m_abs(GA(2, 1)) + m_abs(GA(2, 2)));
      const R t2 = m_max(m_abs(GA(1, 1)) + m_abs(GA(1, 2)), m_abs(GA(2, 1)) + m_abs(GA(2, 2)));
      if (scale1 * t1 >= m_abs(wr1) * t2) givens_alg<R>(GB(1, 1), GB(2, 1), &csl, &snl, &rr);
      else givens_alg<R>(GA(1, 1), GA(2, 1), &csl, &snl, &rr);
      gr_rows<R>(a, ld, 1, 2, csl, snl, 1, 2);
      gr_rows<R>(b, ld, 1, 2, csl, snl, 1, 2);
      GA(2, 1) = 0;
      GB(2, 1) = 0;
    } else {
      R ssmin, ssmax;
      gsvd_2x2<R>(GB(1, 1), GB(1, 2), GB(2, 2), &ssmin, &ssmax, &snr, &csr, &snl, &csl);
      gr_cols_adj<R>(a, ld, 1, 2, csr, snr, 1, 2);
      gr_cols_adj<R>(b, ld, 1, 2, csr, snr, 1, 2);
      gr_rows<R>(a, ld, 1, 2, csl, snl, 1, 2);
      gr_rows<R>(b, ld, 1, 2, csl, snl, 1, 2);
      GB(2, 1) = 0;
      GB(1, 2) = 0;
    }
  }
  for (int j = 1; j <= 2; ++j) for (int i = 1; i <= 2; ++i) GA(i, j) *= anorm;
  for (int j = 1; j <= 2; ++j) for (int i = 1; i <= 2; ++i) GB(i, j) *= bnorm;
  *cslo = csl; *snlo = snl; *csro = csr; *snro = snr;
#undef GA
#undef GB
}

// _rtrexch2!(A, B, Q, Z, j1): swap two 1 x 1 blocks of a real pair
template <class R> bool rtrexch2_r(int n, R* A, R* B, R* Q, R* Z, int j1) {
#define AM(i, j) A[((i) - 1) + (long long)((j) - 1) * n]
#define BM(i, j) B[((i) - 1) + (long long)((j) - 1) * n]
  R S[4] = {AM(j1, j1), AM(j1 + 1, j1), AM(j1, j1 + 1), AM(j1 + 1, j1 + 1)};
  R T[4] = {BM(j1, j1), BM(j1 + 1, j1), BM(j1, j1 + 1), BM(j1 + 1, j1 + 1)};
  const R S0[4] = {S[0], S[1], S[2], S[3]}, T0[4] = {T[0], T[1], T[2], T[3]};
  const R smlnum = safemin<R>() / lim<R>::eps();
  R W[8] = {S[0], S[1], S[2], S[3], T[0], T[1], T[2], T[3]};
  R sa = safe_fnorm_r<R>(W, 8, 8, 1);
  const R thresh = m_max(R(20) * lim<R>::eps() * sa, smlnum);
  const R f = S[3] * T[0] - T[3] * S[0];
  const R g = S[3] * T[2] - T[3] * S[2];
  sa = m_abs(S[3]) * m_abs(T[0]);
  const R sb = m_abs(S[0]) * m_abs(T[3]);
  R cz, sz, rr;
  givens_alg<R>(f, g, &cz, &sz, &rr);
  { const R t = sz; sz = cz; cz = t; }
  gr_cols_adj<R>(S, 2, 1, 2, cz, -sz, 1, 2);
  gr_cols_adj<R>(T, 2, 1, 2, cz, -sz, 1, 2);
  const R fq = sa >= sb ? S[0] : T[0], gq = sa >= sb ? S[1] : T[1];
  R cq, sq;
  if (sz != R(0) && fq == R(0) && gq == R(0)) { cq = 0; sq = 1; }
  else givens_alg<R>(fq, gq, &cq, &sq, &rr);
  gr_rows<R>(S, 2, 1, 2, cq, sq, 1, 2);
  gr_rows<R>(T, 2, 1, 2, cq, sq, 1, 2);
  const R ws = m_abs(S[1]) + m_abs(T[1]);
  if (!(ws <= thresh)) return false;
  R Ss[4] = {S[0], S[1], S[2], S[3]}, Ts[4] = {T[0], T[1], T[2], T[3]};
  gr_cols_adj<R>(Ss, 2, 1, 2, cz, sz, 1, 2);
  gr_cols_adj<R>(Ts, 2, 1, 2, cz, sz, 1, 2);
  gr_rows<R>(Ss, 2, 1, 2, cq, -sq, 1, 2);
  gr_rows<R>(Ts, 2, 1, 2, cq, -sq, 1, 2);
  for (int e = 0; e < 4; ++e) { W[e] = Ss[e] - S0[e]; W[4 + e] = Ts[e] - T0[e]; }
  const R ss = safe_fnorm_r<R>(W, 8, 8, 1);
  if (!(ss <= thresh)) return false;
  gr_cols_adj<R>(A, n, j1, j1 + 1, cz, -sz, 1, n);
  gr_cols_adj<R>(B, n, j1, j1 + 1, cz, -sz, 1, n);
  gr_rows<R>(A, n, j1, j1 + 1, cq, sq, 1, n);
  gr_rows<R>(B, n, j1, j1 + 1, cq, sq, 1, n);
  AM(j1 + 1, j1) = R(0);
  BM(j1 + 1, j1) = R(0);
  if (Z) gr_cols_adj<R>(Z, n, j1, j1 + 1, cz, -sz, 1, n);
  if (Q) gr_cols_adj<R>(Q, n, j1, j1 + 1, cq, sq, 1, n);
  return true;
#undef AM
#undef BM
}

// _swap1or2!(A, B, Q, Z, j1, n1, n2) (dtgex2)
template <class R> bool swap1or2_r(int n, R* A, R* B, R* Q, R* Z, int j1, int n1, int n2) {
  if (j1 + n1 > n) return true;
  if (n1 == 1 && n2 == 1) return rtrexch2_r<R>(n, A, B, Q, Z, j1);
#define AM(i, j) A[((i) - 1) + (long long)((j) - 1) * n]
#define BM(i, j) B[((i) - 1) + (long long)((j) - 1) * n]
  const int m = n1 + n2, je = j1 + m - 1;
  R S[16], T[16];
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) { S[i + j * m] = AM(j1 + i, j1 + j); T[i + j * m] = BM(j1 + i, j1 + j); }
  const R eps = lim<R>::eps(), smallnum = lim<R>::fmin() / eps;
  R dnorm = 0, tnorm = 0;
  for (int e = 0; e < m * m; ++e) { dnorm = m_max(dnorm, m_abs(S[e])); tnorm = m_max(tnorm, m_abs(T[e])); }
  const R thresh = m_max(R(20) * eps * dnorm, smallnum);
  const R threshb = m_max(R(20) * eps * tnorm, smallnum);
  // _syl1or2: K [vec R; vec L] = [vec S12; vec T12], K = [I(n2)(x)S11, -S22'(x)I(n1); I(n2)(x)T11, -T22'(x)I(n1)]
  const int nn = n1 * n2, kd = 2 * nn;
  std::vector<cx<R>> K((size_t)kd * kd, cx<R>(R(0))), rl(kd);
  auto Sb = [&](int i, int j) { return S[(i - 1) + (j - 1) * m]; };
  auto Tb = [&](int i, int j) { return T[(i - 1) + (j - 1) * m]; };
  for (int q = 0; q < n2; ++q)
    for (int p = 0; p < n1; ++p) {
      const int row = p + q * n1;  // (p, q) of an n1 x n2 block
      for (int pp = 0; pp < n1; ++pp) {
        K[row + (size_t)(pp + q * n1) * kd] = cx<R>(Sb(1 + p, 1 + pp));
        K[(nn + row) + (size_t)(pp + q * n1) * kd] = cx<R>(Tb(1 + p, 1 + pp));
      }
      for (int qq = 0; qq < n2; ++qq) {
        K[row + (size_t)(nn + p + qq * n1) * kd] = cx<R>(-Sb(n1 + 1 + qq, n1 + 1 + q));
        K[(nn + row) + (size_t)(nn + p + qq * n1) * kd] = cx<R>(-Tb(n1 + 1 + qq, n1 + 1 + q));
      }
      rl[row] = cx<R>(Sb(1 + p, n1 + 1 + q));
      rl[nn + row] = cx<R>(Tb(1 + p, n1 + 1 + q));
    }
  bool pert = false;
  const R scale = safe_lu_solve<R>(kd, K.data(), rl.data(), &pert);
  // LI = [-XL; scale I(n2)] (m x n2), IR = [scale I(n1) XR] (n1 x m)
  R LI[8], IR[8], qli[16], zir[16];
  for (int j = 0; j < n2; ++j) {
    for (int i = 0; i < n1; ++i) LI[i + j * m] = -rl[nn + i + j * n1].re;
    for (int i = 0; i < n2; ++i) LI[n1 + i + j * m] = i == j ? scale : R(0);
  }
  for (int i = 0; i < n1; ++i) {
    for (int j = 0; j < n1; ++j) IR[i + j * n1] = i == j ? scale : R(0);
    for (int j = 0; j < n2; ++j) IR[i + (n1 + j) * n1] = rl[i + j * n1].re;
  }
  house_qr_r<R>(m, n2, LI, qli);
  house_rq_r<R>(n1, m, IR, zir);
  R tmp[16], s1[16], t1[16];
  mm_r<R>(m, m, m, qli, true, S, false, tmp);
  mm_r<R>(m, m, m, tmp, false, zir, true, s1);
  mm_r<R>(m, m, m, qli, true, T, false, tmp);
  mm_r<R>(m, m, m, tmp, false, zir, true, t1);
  // triangularize t1 by RQ (a) and by QR (b)
  R t2a[16], zt1a[16], s2a[16], z2a[16], t2b[16], qt1b[16], s2b[16], q2b[16];
  for (int e = 0; e < m * m; ++e) { t2a[e] = t1[e]; t2b[e] = t1[e]; }
  house_rq_r<R>(m, m, t2a, zt1a);
  mm_r<R>(m, m, m, s1, false, zt1a, true, s2a);
  mm_r<R>(m, m, m, zt1a, false, zir, false, z2a);
  const R brq = safe_fnorm_r<R>(s2a + n2, m, m - n2, n2);
  house_qr_r<R>(m, m, t2b, qt1b);
  mm_r<R>(m, m, m, qt1b, true, s1, false, s2b);
  mm_r<R>(m, m, m, qli, false, qt1b, false, q2b);
  const R bqr = safe_fnorm_r<R>(s2b + n2, m, m - n2, n2);
  if (!(m_min(bqr, brq) <= thresh)) return false;
  R *snew, *tnew, *znew, *qnew;
  if (bqr <= brq) { snew = s2b; tnew = t2b; znew = zir; qnew = q2b; }
  else { snew = s2a; tnew = t2a; znew = z2a; qnew = qli; }
  {
    R r1[16], r2[16];
    mm_r<R>(m, m, m, qnew, false, snew, false, r1);
    mm_r<R>(m, m, m, r1, false, znew, false, r2);
    for (int e = 0; e < m * m; ++e) r2[e] = S[e] - r2[e];
    const R resa = safe_fnorm_r<R>(r2, m, m, m);
    mm_r<R>(m, m, m, qnew, false, tnew, false, r1);
    mm_r<R>(m, m, m, r1, false, znew, false, r2);
    for (int e = 0; e < m * m; ++e) r2[e] = T[e] - r2[e];
    const R resb = safe_fnorm_r<R>(r2, m, m, m);
    if (!(resa <= thresh && resb <= threshb)) return false;
  }
  for (int j = 0; j < n2; ++j)
    for (int i = n2; i < m; ++i) snew[i + j * m] = R(0);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) { AM(j1 + i, j1 + j) = snew[i + j * m]; BM(j1 + i, j1 + j) = tnew[i + j * m]; }
  R qtmp[16], ztmp[16];
  for (int e = 0; e < m * m; ++e) { qtmp[e] = R(0); ztmp[e] = R(0); }
  R csl, snl, csr, snr;
  if (n2 > 1) {
    gqz_2x2_r<R>(&AM(j1, j1), &BM(j1, j1), n, &csl, &snl, &csr, &snr);
    qtmp[0] = csl; qtmp[1] = snl; qtmp[m] = -snl; qtmp[m + 1] = csl;
    ztmp[0] = csr; ztmp[1] = snr; ztmp[m] = -snr; ztmp[m + 1] = csr;
  } else {
    ztmp[0] = R(1);
    qtmp[0] = R(1);
  }
  const int j3 = j1 + n2;
  if (n1 > 1) {
    gqz_2x2_r<R>(&AM(j3, j3), &BM(j3, j3), n, &csl, &snl, &csr, &snr);
    qtmp[(m - 2) + (m - 2) * m] = csl; qtmp[(m - 1) + (m - 2) * m] = snl;
    qtmp[(m - 2) + (m - 1) * m] = -snl; qtmp[(m - 1) + (m - 1) * m] = csl;
    ztmp[(m - 2) + (m - 2) * m] = csr; ztmp[(m - 1) + (m - 2) * m] = snr;
    ztmp[(m - 2) + (m - 1) * m] = -snr; ztmp[(m - 1) + (m - 1) * m] = csr;
  } else {
    qtmp[(m - 1) + (m - 1) * m] = R(1);
    ztmp[(m - 1) + (m - 1) * m] = R(1);
  }
  // the off-diagonal block of the active region: qtmp[1:n2,1:n2]' X ztmp[n2+1:m, n2+1:m]
  for (R* M : {A, B}) {
    R X[4], ab[4];
    for (int j = 0; j < n1; ++j) for (int i = 0; i < n2; ++i) X[i + j * n2] = M[(j1 - 1 + i) + (long long)(j3 - 1 + j) * n];
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n2; ++i) {
        R t = R(0);
        for (int l = 0; l < n2; ++l) t += qtmp[l + i * m] * X[l + j * n2];
        ab[i + j * n2] = t;
      }
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n2; ++i) {
        R t = R(0);
        for (int l = 0; l < n1; ++l) t += ab[i + l * n2] * ztmp[(n2 + l) + (n2 + j) * m];
        M[(j1 - 1 + i) + (long long)(j3 - 1 + j) * n] = t;
      }
  }
  R qf[16], zf[16];
  mm_r<R>(m, m, m, qnew, false, qtmp, false, qf);
  mm_r<R>(m, m, m, znew, true, ztmp, false, zf);
  auto cols_times = [&](R* M, int rows, const R* X) {  // M[1:rows, j1:je] = M[1:rows, j1:je] X
    for (int r = 1; r <= rows; ++r) {
      R v[4];
      for (int j = 0; j < m; ++j) v[j] = M[(r - 1) + (long long)(j1 - 1 + j) * n];
      for (int j = 0; j < m; ++j) {
        R t = R(0);
        for (int l = 0; l < m; ++l) t += v[l] * X[l + j * m];
        M[(r - 1) + (long long)(j1 - 1 + j) * n] = t;
      }
    }
  };
  if (Q) cols_times(Q, n, qf);
  if (Z) cols_times(Z, n, zf);
  if (je < n)
    for (R* M : {A, B})
      for (int c = je + 1; c <= n; ++c) {
        R v[4];
        for (int i = 0; i < m; ++i) v[i] = M[(j1 - 1 + i) + (long long)(c - 1) * n];
        for (int i = 0; i < m; ++i) {
          R t = R(0);
          for (int l = 0; l < m; ++l) t += qf[l + i * m] * v[l];
          M[(j1 - 1 + i) + (long long)(c - 1) * n] = t;
        }
      }
  cols_times(A, j1 - 1, zf);
  cols_times(B, j1 - 1, zf);
  return true;
#undef AM
#undef BM
}

// _trexchange!(S, T, Q, Z, iold, inew) for inew <= iold; returns ok, *inew_out the final row
template <class R> bool trexchange_r(int n, R* S, R* T, R* Q, R* Z, int iold, int inew, int* inew_out) {
#define SM(i, j) S[((i) - 1) + (long long)((j) - 1) * n]
  *inew_out = inew;
  if (n <= 1) return true;
  auto nbsize = [&](int j) { return (j < n && SM(j + 1, j) != R(0)) ? 2 : 1; };
  if (iold > 1 && SM(iold, iold - 1) != R(0)) iold -= 1;
  const int nbold = nbsize(iold);
  if (inew > 1 && SM(inew, inew - 1) != R(0)) inew -= 1;
  if (iold == inew) { *inew_out = inew; return true; }
  if (iold < inew) return false;  // the move-down branch; gordschur! only moves blocks up
  int ihere = iold;
  while (ihere > inew) {
    const int nbnext = (ihere >= 3 && SM(ihere - 1, ihere - 2) != R(0)) ? 2 : 1;
    if (!swap1or2_r<R>(n, S, T, Q, Z, ihere - nbnext, nbnext, nbold)) { *inew_out = ihere; return false; }
    ihere -= nbnext;
  }
  *inew_out = ihere;
  return true;
#undef SM
}

// gordschur!(S, T, Q, Z, select; scale) for a real pair; returns 0 or 1 + k of the block
// that could not be moved (IllConditionException(k))
template <class R>
int gordschur_real(int n, R* S, R* T, R* Q, R* Z, const int* select, bool scale, cx<R>* alpha, R* beta) {
  R cscale = 1, anrm = 1, cscaleb = 1, bnrm = 1;
  bool scA = false, scB = false;
  if (scale) {
    scA = scale_matrix<R, R>(n, S, n, &cscale, &anrm);
    scB = scale_matrix<R, R>(n, T, n, &cscaleb, &bnrm);
  }
#define SM(i, j) S[((i) - 1) + (long long)((j) - 1) * n]
#define TM(i, j) T[((i) - 1) + (long long)((j) - 1) * n]
  const R safmin = lim<R>::fmin();
  int ks = 0;
  bool inpair = false;
  for (int k = 1; k <= n; ++k) {
    if (inpair) { inpair = false; continue; }
    bool doswap = select[k - 1] != 0;
    if (k < n && SM(k + 1, k) != R(0)) {
      inpair = true;
      doswap = doswap || select[k] != 0;
    }
    if (doswap) {
      ks += 1;
      if (k != ks) {
        int kn = ks;
        if (!trexchange_r<R>(n, S, T, Q, Z, k, ks, &kn)) return 1 + k;
        ks = kn;
      }
      if (inpair) ks += 1;
    }
  }
  if (scA) for (int j = 0; j < n; ++j) safescale<R, R>(S + (long long)j * n, n, cscale, anrm);
  if (scB) for (int j = 0; j < n; ++j) safescale<R, R>(T + (long long)j * n, n, cscaleb, bnrm);
  inpair = false;
  for (int k = 1; k <= n; ++k) {
    if (inpair) { inpair = false; continue; }
    if (k < n && SM(k + 1, k) != R(0)) inpair = true;
    if (inpair) {
      R b1, b2, ar1, ar2, ai;
      ggs_2x2<R>(&SM(k, k), n, &TM(k, k), n, safmin, &b1, &b2, &ar1, &ar2, &ai);
      alpha[k - 1] = cx<R>(ar1, ai);
      alpha[k] = cx<R>(ar2, -ai);
      beta[k - 1] = b1;
      beta[k] = b2;
    } else {
      if (m_copysign(R(1), TM(k, k)) < R(0)) {
        for (int j = 1; j <= n; ++j) { SM(k, j) = -SM(k, j); TM(k, j) = -TM(k, j); }
        if (Q) for (int i = 0; i < n; ++i) Q[i + (long long)(k - 1) * n] = -Q[i + (long long)(k - 1) * n];
      }
      alpha[k - 1] = cx<R>(SM(k, k));
      beta[k - 1] = TM(k, k);
    }
  }
  return 0;
#undef SM
#undef TM
}

}  // namespace orc
