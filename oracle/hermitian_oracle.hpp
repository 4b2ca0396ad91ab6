// CPU oracle of the Hermitian / real symmetric eigen path (TEST INFRASTRUCTURE ONLY; the
// shipped library never links this): restatements of
//   _hehessenberg! (:L and :U)          src/hessenberg.jl:26-130 (from LAPACK's zhetd2),
//   _materializeQ (:L and :U)           src/hessenberg.jl:145-231,
//   _gschur!(::SymTridiagonal, QRIteration, Z) with _st_QLIter!, _st_QRIter!,
//   _st_findsplit_fwd!, _dgz_sym2x2     src/symtridiag.jl:79-427 (from LAPACK's zsteqr),
//   geigen! / geigvals!                 src/GenericSchur.jl:126-146 (sorted by eigsortby),
// and of LinearAlgebra's givensAlgorithm (LAPACK 3.x dlartg, with its safmn2 / safmx2
// rescaling loops), which the QL/QR sweeps call.  1-based index macros; column-major.
#pragma once
#include <algorithm>
#include <numeric>
#include <vector>
#include "gschur_oracle.hpp"

namespace orc {

template <class R> inline R re_part(R x) { return x; }
template <class R> inline R re_part(cx<R> x) { return x.re; }

// _hehessenberg!(Hermitian(A, :L)) (hessenberg.jl:26-58; rank2update! :L 113-130).
template <class R, class S> void he_tridiag_L(int n, S* a, int lda, S* tau, R* d, R* e) {
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * lda]
  if (n == 0) return;
  std::vector<S> w(n > 1 ? n - 1 : 1);
  A_(1, 1) = S(re_part(A_(1, 1)));
  for (int i = 1; i <= n - 1; ++i) {
    const int m = n - i;
    S* xi = &A_(i + 1, i);
    const S ti = reflector(xi, m);
    e[i - 1] = re_part(A_(i + 1, i));
    if (!(ti == S(0))) {
      xi[0] = S(1);
      // w = ti * Hermitian(A22, :L) * xi
      for (int r = 1; r <= m; ++r) {
        S s = S(0);
        for (int c = 1; c <= m; ++c) {
          S h;
          if (r == c) h = S(re_part(A_(i + r, i + c)));
          else if (r > c) h = A_(i + r, i + c);
          else h = cj(A_(i + c, i + r));
          s += h * xi[c - 1];
        }
        w[r - 1] = s * ti;
      }
      // alpha = -(ti / 2) dot(w, xi); w += alpha xi
      S dw = S(0);
      for (int r = 0; r < m; ++r) dw += cj(w[r]) * xi[r];
      const S alpha = -(ti * R(0.5)) * dw;
      for (int r = 0; r < m; ++r) w[r] = w[r] + alpha * xi[r];
      // rank2update!(A22, -1, xi, w, :L)
      for (int j = 1; j <= m; ++j) {
        if (xi[j - 1] == S(0) && w[j - 1] == S(0)) {
          A_(i + j, i + j) = S(re_part(A_(i + j, i + j)));
        } else {
          const S t1 = S(R(-1)) * cj(w[j - 1]);
          const S t2 = cj(S(R(-1)) * xi[j - 1]);
          A_(i + j, i + j) = S(re_part(A_(i + j, i + j)) + re_part(xi[j - 1] * t1 + w[j - 1] * t2));
          for (int r = j + 1; r <= m; ++r) A_(i + r, i + j) += xi[r - 1] * t1 + w[r - 1] * t2;
        }
      }
    } else {
      A_(i + 1, i + 1) = S(re_part(A_(i + 1, i + 1)));
    }
    A_(i + 1, i) = S(e[i - 1]);
    d[i - 1] = re_part(A_(i, i));
    tau[i - 1] = ti;
  }
  d[n - 1] = re_part(A_(n, n));
#undef A_
}

// _hehessenberg!(Hermitian(A, :U)) (hessenberg.jl:60-96; rank2update! :U 98-111).
template <class R, class S> void he_tridiag_U(int n, S* a, int lda, S* tau, R* d, R* e) {
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * lda]
  if (n == 0) return;
  std::vector<S> xi(n), w(n);
  A_(n, n) = S(re_part(A_(n, n)));
  for (int i = n - 1; i >= 1; --i) {
    xi[0] = A_(i, i + 1);
    for (int r = 2; r <= i; ++r) xi[r - 1] = A_(r - 1, i + 1);
    const S ti = reflector(xi.data(), i);
    e[i - 1] = re_part(xi[0]);
    for (int r = 2; r <= i; ++r) A_(r - 1, i + 1) = xi[r - 1];
    if (!(ti == S(0))) {
      A_(i, i + 1) = S(1);
      // v = A[1:i, i+1]; w = ti * Hermitian(A[1:i,1:i], :U) * v
      std::vector<S> v(i);
      for (int r = 1; r <= i; ++r) v[r - 1] = A_(r, i + 1);
      for (int r = 1; r <= i; ++r) {
        S s = S(0);
        for (int c = 1; c <= i; ++c) {
          S h;
          if (r == c) h = S(re_part(A_(r, c)));
          else if (r < c) h = A_(r, c);
          else h = cj(A_(c, r));
          s += h * v[c - 1];
        }
        w[r - 1] = s * ti;
      }
      S dw = S(0);
      for (int r = 0; r < i; ++r) dw += cj(w[r]) * v[r];
      const S alpha = -(ti * R(0.5)) * dw;
      for (int r = 0; r < i; ++r) w[r] = w[r] + alpha * v[r];
      // rank2update!(A[1:i,1:i], -1, v, w, :U)
      for (int j = 1; j <= i; ++j) {
        if (v[j - 1] == S(0) && w[j - 1] == S(0)) {
          A_(j, j) = S(re_part(A_(j, j)));
        } else {
          const S t1 = S(R(-1)) * cj(w[j - 1]);
          const S t2 = cj(S(R(-1)) * v[j - 1]);
          for (int r = 1; r <= j - 1; ++r) A_(r, j) += v[r - 1] * t1 + w[r - 1] * t2;
          A_(j, j) = S(re_part(A_(j, j)) + re_part(v[j - 1] * t1 + w[j - 1] * t2));
        }
      }
    } else {
      A_(i, i) = S(re_part(A_(i, i)));
    }
    A_(i, i + 1) = S(e[i - 1]);
    d[i] = re_part(A_(i + 1, i + 1));
    tau[i - 1] = ti;
  }
  d[0] = re_part(A_(1, 1));
#undef A_
}

// _materializeQ(H, Val(:U)) (hessenberg.jl:200-231).
template <class S> void materialize_q_U(int n, const S* f, int ldf, const S* tau, S* q, int ldq) {
#define A_(i, j) q[((i) - 1) + (long long)((j) - 1) * ldq]
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= n; ++i) A_(i, j) = f[(i - 1) + (long long)(j - 1) * ldf];
  for (int j = 1; j <= n - 1; ++j) {
    for (int i = 1; i <= j - 1; ++i) A_(i, j) = A_(i, j + 1);
    for (int i = j; i <= n; ++i) A_(i, j) = S(0);
  }
  for (int i = 1; i <= n - 1; ++i) A_(i, n) = S(0);
  A_(n, n) = S(1);
  std::vector<S> w(n > 1 ? n - 1 : 1);
  for (int i = 1; i <= n - 1; ++i) {
    A_(i, i) = S(1);
    const S ti = tau[i - 1];
    for (int j = 1; j <= i - 1; ++j) {
      S s = S(0);
      for (int k = 1; k <= i; ++k) s += cj(A_(k, j)) * A_(k, i);
      w[j - 1] = s;
    }
    for (int j = 1; j <= i - 1; ++j) {
      const S t = ti * cj(w[j - 1]);
      for (int k = 1; k <= i; ++k) A_(k, j) -= A_(k, i) * t;
    }
    for (int k = 1; k <= i - 1; ++k) A_(k, i) = A_(k, i) * (-ti);
    A_(i, i) = S(1) - ti;
    for (int k = i + 1; k <= n; ++k) A_(k, i) = S(0);
  }
#undef A_
}

// LinearAlgebra.givensAlgorithm(f, g) for AbstractFloat (LAPACK 3.x dlartg).
template <class R> void givens_alg(R f, R g, R* cs, R* sn, R* r) {
  // safmn2 = 2^floor(log2(floatmin / eps) / 2): 2^-485 for Float64, 2^-63 for Float32
  R mn2 = R(1);
  for (int k = 0; k < (std::is_same<R, float>::value ? 63 : 485); ++k) mn2 *= R(0.5);
  const R mx2 = R(1) / mn2;
  if (g == R(0)) { *cs = R(1); *sn = R(0); *r = f; return; }
  if (f == R(0)) { *cs = R(0); *sn = R(1); *r = g; return; }
  R f1 = f, g1 = g;
  R scale = m_max(m_abs(f1), m_abs(g1));
  R c, s, rr;
  if (scale >= mx2) {
    int count = 0;
    do {
      ++count;
      f1 *= mn2;
      g1 *= mn2;
      scale = m_max(m_abs(f1), m_abs(g1));
    } while (!(scale < mx2 || count >= 20));
    rr = m_sqrt(f1 * f1 + g1 * g1);
    c = f1 / rr;
    s = g1 / rr;
    for (int i = 0; i < count; ++i) rr *= mx2;
  } else if (scale <= mn2) {
    int count = 0;
    do {
      ++count;
      f1 *= mx2;
      g1 *= mx2;
      scale = m_max(m_abs(f1), m_abs(g1));
    } while (!(scale > mn2));
    rr = m_sqrt(f1 * f1 + g1 * g1);
    c = f1 / rr;
    s = g1 / rr;
    for (int i = 0; i < count; ++i) rr *= mn2;
  } else {
    rr = m_sqrt(f1 * f1 + g1 * g1);
    c = f1 / rr;
    s = g1 / rr;
  }
  if (m_abs(f) > m_abs(g) && c < R(0)) { c = -c; s = -s; rr = -rr; }
  *cs = c; *sn = s; *r = rr;
}

// _dgz_sym2x2(a, b, c, wantvec) (symtridiag.jl:370-427).
template <class R> void dgz_sym2x2(R a, R b, R c, bool wantvec, R* rt1o, R* rt2o, R* cs1o, R* sn1o) {
  const R sm = a + c, df = a - c, adf = m_abs(df), tb = R(2) * b, ab = m_abs(tb);
  R acmx, acmn;
  if (m_abs(a) > m_abs(c)) { acmx = a; acmn = c; } else { acmx = c; acmn = a; }
  const R rt = m_hypot(ab, adf);
  R rt1, rt2;
  int sgn1;
  if (sm < R(0)) {
    rt1 = (sm - rt) / R(2);
    sgn1 = -1;
    rt2 = (acmx / rt1) * acmn - (b / rt1) * b;
  } else if (sm > R(0)) {
    rt1 = (sm + rt) / R(2);
    sgn1 = 1;
    rt2 = (acmx / rt1) * acmn - (b / rt1) * b;
  } else {
    rt1 = rt / R(2);
    rt2 = -rt / R(2);
    sgn1 = 1;
  }
  R cs1 = R(0), sn1 = R(0);
  if (wantvec) {
    R cs;
    int sgn2;
    if (df > R(0)) { cs = df + rt; sgn2 = 1; } else { cs = df - rt; sgn2 = -1; }
    const R acs = m_abs(cs);
    if (acs > ab) {
      const R ct = -tb / cs;
      sn1 = R(1) / m_sqrt(R(1) + ct * ct);
      cs1 = ct * sn1;
    } else {
      if (ab == R(0)) { cs1 = R(1); sn1 = R(0); }
      else {
        const R tn = -cs / tb;
        cs1 = R(1) / m_sqrt(R(1) + tn * tn);
        sn1 = tn * cs1;
      }
    }
    if (sgn1 == sgn2) { const R tn = cs1; cs1 = -sn1; sn1 = tn; }
  }
  *rt1o = rt1; *rt2o = rt2; *cs1o = cs1; *sn1o = sn1;
}

// rmul!(Z, Givens(i, i+1, c, s)') on the nz rows of Z.
template <class R, class S> inline void rot_cols(S* z, int ldz, int nz, int i, R c, R s) {
  S* z1 = z + (long long)(i - 1) * ldz;
  S* z2 = z + (long long)i * ldz;
  for (int r = 0; r < nz; ++r) {
    const S a1 = z1[r], a2 = z2[r];
    z1[r] = a1 * c + a2 * s;
    z2[r] = a2 * c - a1 * s;
  }
}

// opnorm(SymTridiagonal(d[l:lend], e[l:lend-1]), Inf)
template <class R> R st_norm_inf(const R* d, const R* e, int l, int lend) {
  R m = 0;
  for (int i = l; i <= lend; ++i) {
    R s = m_abs(d[i - 1]);
    if (i > l) s += m_abs(e[i - 2]);
    if (i < lend) s += m_abs(e[i - 1]);
    if (s > m || s != s) m = s;
  }
  return m;
}

// _gschur!(SymTridiagonal(d, e), QRIteration(), Z) (symtridiag.jl:79-183).  Z: nz x n
// (nz = 0: eigenvalues only).  The reference's iteration counter never advances
// (symtridiag.jl:155), so it has no effective limit; maxsweeps here bounds the total
// number of QL/QR sweeps and returns 1 when reached.
template <class R, class S> int steqr(int n, R* d, R* e, S* z, int ldz, int nz, long long maxsweeps) {
#define D(i) d[(i) - 1]
#define E(i) e[(i) - 1]
  const bool wantZ = z != nullptr && nz > 0;
  const R epsT = lim<R>::eps(), eps2 = epsT * epsT;
  const R safmin = lim<R>::fmin(), safmax = R(1) / safmin;
  const R ssfmax = m_sqrt(safmax) / R(3), ssfmin = m_sqrt(safmin) / eps2;
  long long sweeps = 0;
  int l1 = 1;
  while (l1 <= n) {
    if (l1 > 1) E(l1 - 1) = R(0);
    // _st_findsplit_fwd!
    int msplit = n;
    for (int m = l1; m <= n - 1; ++m) {
      const R tst = m_abs(E(m));
      if (tst == R(0)) { msplit = m; break; }
      if (tst <= m_sqrt(m_abs(D(m))) * m_sqrt(m_abs(D(m + 1))) * epsT) { E(m) = R(0); msplit = m; break; }
    }
    int l = l1;
    const int lsave = l;
    int lend = msplit;
    const int lendsave = lend;
    l1 = msplit + 1;
    if (lend == l) continue;
    const R anorm = st_norm_inf(d, e, l, lend);
    int iscale = 0;
    if (anorm == R(0)) continue;
    if (anorm > ssfmax) {
      iscale = 1;
      safescale<R, R>(&D(l), lend - l + 1, anorm, ssfmax);
      safescale<R, R>(&E(l), lend - l, anorm, ssfmax);
    } else if (anorm < ssfmin) {
      iscale = 2;
      safescale<R, R>(&D(l), lend - l + 1, anorm, ssfmin);
      safescale<R, R>(&E(l), lend - l, anorm, ssfmin);
    }
    if (m_abs(D(lend)) < m_abs(D(l))) { lend = lsave; l = lendsave; }
    if (lend > l) {
      // _st_QLIter! (symtridiag.jl:185-266)
      while (l <= lend) {
        int ms = lend;
        for (int m = l; m <= lend - 1; ++m)
          if (E(m) * E(m) <= (eps2 * m_abs(D(m))) * m_abs(D(m + 1)) + safmin) { ms = m; break; }
        if (ms < lend) E(ms) = R(0);
        R p = D(l);
        if (ms != l) {
          if (ms == l + 1) {
            R rt1, rt2, cs, sn;
            dgz_sym2x2(D(l), E(l), D(l + 1), wantZ, &rt1, &rt2, &cs, &sn);
            if (wantZ) rot_cols<R, S>(z, ldz, nz, l, cs, sn);
            D(l) = rt1; D(l + 1) = rt2; E(l) = R(0);
            l += 2;
            if (l <= lend) continue;
            break;
          }
          if (++sweeps > maxsweeps) return 1;
          R g = (D(l + 1) - p) / (R(2) * E(l));
          R r = m_hypot(g, R(1));
          g = D(ms) - p + (E(l) / (g + m_copysign(r, g)));
          R s = 1, c = 1;
          p = 0;
          std::vector<R> cv, sv;
          for (int i = ms - 1; i >= l; --i) {
            const R f = s * E(i), b = c * E(i);
            givens_alg(g, f, &c, &s, &r);
            if (i < ms - 1) E(i + 1) = r;
            g = D(i + 1) - p;
            r = (D(i) - g) * s + R(2) * c * b;
            p = s * r;
            D(i + 1) = g + p;
            g = c * r - b;
            if (wantZ) { cv.push_back(c); sv.push_back(-s); }
          }
          if (wantZ)
            for (int i = ms - 1, q = 0; i >= l; --i, ++q) rot_cols<R, S>(z, ldz, nz, i, cv[q], sv[q]);
          D(l) -= p;
          E(l) = g;
        } else {
          D(l) = p;
          l += 1;
        }
      }
    } else {
      // _st_QRIter! (symtridiag.jl:268-346)
      while (l >= lend) {
        int ms = lend;
        for (int m = l; m >= lend + 1; --m)
          if (E(m - 1) * E(m - 1) <= (eps2 * m_abs(D(m))) * m_abs(D(m - 1)) + safmin) { ms = m; break; }
        if (ms > lend) E(ms - 1) = R(0);
        R p = D(l);
        if (ms != l) {
          if (ms == l - 1) {
            R rt1, rt2, cs, sn;
            dgz_sym2x2(D(l - 1), E(l - 1), D(l), wantZ, &rt1, &rt2, &cs, &sn);
            if (wantZ) rot_cols<R, S>(z, ldz, nz, ms, cs, sn);
            D(l - 1) = rt1; D(l) = rt2; E(l - 1) = R(0);
            l -= 2;
            if (l >= lend) continue;
            break;
          }
          if (++sweeps > maxsweeps) return 1;
          R g = (D(l - 1) - p) / (R(2) * E(l - 1));
          R r = m_hypot(g, R(1));
          g = D(ms) - p + (E(l - 1) / (g + m_copysign(r, g)));
          R s = 1, c = 1;
          p = 0;
          std::vector<R> cv, sv;
          for (int i = ms; i <= l - 1; ++i) {
            const R f = s * E(i), b = c * E(i);
            givens_alg(g, f, &c, &s, &r);
            if (i != ms) E(i - 1) = r;
            g = D(i) - p;
            r = (D(i + 1) - g) * s + R(2) * c * b;
            p = s * r;
            D(i) = g + p;
            g = c * r - b;
            if (wantZ) { cv.push_back(c); sv.push_back(s); }
          }
          if (wantZ)
            for (int i = ms, q = 0; i <= l - 1; ++i, ++q) rot_cols<R, S>(z, ldz, nz, i, cv[q], sv[q]);
          D(l) -= p;
          E(l - 1) = g;
        } else {
          D(l) = p;
          l -= 1;
        }
      }
    }
    if (iscale == 1) {
      safescale<R, R>(&D(lsave), lendsave - lsave + 1, ssfmax, anorm);
      safescale<R, R>(&E(lsave), lendsave - lsave, ssfmax, anorm);
    } else if (iscale == 2) {
      safescale<R, R>(&D(lsave), lendsave - lsave + 1, ssfmin, anorm);
      safescale<R, R>(&E(lsave), lendsave - lsave, ssfmin, anorm);
    }
  }
  return 0;
#undef D
#undef E
}

// geigen! / geigvals! (GenericSchur.jl:126-146) for Hermitian(A, uplo): w ascending
// (eigsortby, stable), V (n x n) the eigenvectors (when wantv).  A is overwritten.
template <class R, class S> int heev(int n, S* a, int lda, bool upper, bool wantv, R* w, S* v, int ldv) {
  if (n == 0) return 0;
  std::vector<S> tau(n > 1 ? n - 1 : 1);
  std::vector<R> e(n > 1 ? n - 1 : 1);
  if (upper) he_tridiag_U<R, S>(n, a, lda, tau.data(), w, e.data());
  else he_tridiag_L<R, S>(n, a, lda, tau.data(), w, e.data());
  std::vector<S> q;
  if (wantv) {
    q.assign((size_t)n * n, S(0));
    if (upper) materialize_q_U<S>(n, a, lda, tau.data(), q.data(), n);
    else materialize_q<S>(n, a, lda, tau.data(), q.data(), n);
  }
  const int st = steqr<R, S>(n, w, e.data(), wantv ? q.data() : nullptr, n, wantv ? n : 0, 30LL * n);
  std::vector<int> p(n);
  std::iota(p.begin(), p.end(), 0);
  std::stable_sort(p.begin(), p.end(), [&](int x, int y) { return w[x] < w[y]; });
  std::vector<R> ws(w, w + n);
  for (int j = 0; j < n; ++j) w[j] = ws[p[j]];
  if (wantv)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) v[i + (long long)j * ldv] = q[i + (size_t)p[j] * n];
  return st;
}

}  // namespace orc
