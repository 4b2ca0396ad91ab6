// CPU oracle of the condition estimators of a Schur form (TEST INFRASTRUCTURE ONLY; the
// shipped library never links this): restatements of
//   trsylvester! / adjtrsylvester!   (src/sylvester.jl:11-139, from LAPACK's ztrsyl),
//   norm1est!                        (src/norm1est.jl:21-74, Hager / Higham),
//   eigvalscond / subspacesep        (src/ordschur.jl:84-140, from LAPACK's ztrsen).
// The Sylvester solves read only the upper triangles of A and B, as the reference does,
// so for a real quasi-triangular T the 2x2 blocks' subdiagonal entries are ignored there
// too.  Column-major, 0-based.
#pragma once
#include <type_traits>
#include <vector>
#include "scalar.hpp"

namespace orc {

template <class S> inline S s_zero() { return S(0); }
template <class R> inline R mod_of(R x) { return m_abs(x); }
template <class R> inline R mod_of(cx<R> x) { return cabs(x); }

// Entrywise max-modulus norm (Julia's norm(A, Inf) of a matrix view).
template <class R, class S> R maxabs_block(const S* a, int lda, int rows, int cols) {
  R m = 0;
  for (int j = 0; j < cols; ++j)
    for (int i = 0; i < rows; ++i) {
      const R v = mod_of(a[i + (long long)j * lda]);
      if (v > m || v != v) m = v;
    }
  return m;
}

// trsylvester! (adj = false): A X - X B = scale C;  adjtrsylvester! (adj = true):
// A^H X - X B^H = scale C; with possign the signs of the B terms are +.  A m x m, B p x p upper triangular; C m x p overwritten by X.
// Returns scale; *perturbed set when a diagonal difference was replaced by smin.
template <class R, class S>
R trsylvester(bool adj, int m, int p, const S* A, int lda, const S* B, int ldb, S* C, int ldc, bool* perturbed,
              bool possign = false) {
#define SA(i, j) A[(i) + (long long)(j) * lda]
#define SB(i, j) B[(i) + (long long)(j) * ldb]
#define SC(i, j) C[(i) + (long long)(j) * ldc]
  R scale = 1;
  const R tiny = std::numeric_limits<R>::epsilon();
  const R small = safemin<R>() * m * p / tiny;
  const R bignum = R(1) / small;
  const R smin = m_max(small, tiny * maxabs_block<R>(A, lda, m, m) * maxabs_block<R>(B, ldb, p, p));
  bool pert = false;
  auto step = [&](int k, int l, S v, S a11) {
    R da11 = abs1(a11);
    const bool low = adj ? (da11 < smin) : (da11 <= smin);
    if (low) { a11 = S(smin); da11 = smin; pert = true; }
    R scaloc = 1;
    const R db = abs1(v);
    if (da11 < R(1) && db > R(1) && db > bignum * da11) scaloc = R(1) / db;
    const S x11 = (v * scaloc) / a11;
    if (scaloc != R(1)) {
      for (int jj = 0; jj < p; ++jj)
        for (int ii = 0; ii < m; ++ii) SC(ii, jj) = SC(ii, jj) * scaloc;
      scale *= scaloc;
    }
    SC(k, l) = x11;
  };
  if (!adj) {
    // sylvester.jl:44-71: l ascending, k descending; isgn = -1
    for (int l = 0; l < p; ++l)
      for (int k = m - 1; k >= 0; --k) {
        S suml = s_zero<S>(), sumr = s_zero<S>();
        for (int j = k + 1; j < m; ++j) suml += SA(k, j) * SC(j, l);
        for (int j = 0; j < l; ++j) sumr += SC(k, j) * SB(j, l);
        if (possign) step(k, l, SC(k, l) - (suml + sumr), SA(k, k) + SB(l, l));
        else step(k, l, SC(k, l) - (suml - sumr), SA(k, k) - SB(l, l));
      }
  } else {
    // sylvester.jl:110-136: l descending, k ascending
    for (int l = p - 1; l >= 0; --l)
      for (int k = 0; k < m; ++k) {
        S suml = s_zero<S>(), sumr = s_zero<S>();
        for (int j = 0; j < k; ++j) suml += cj(SA(j, k)) * SC(j, l);
        for (int j = l + 1; j < p; ++j) sumr += cj(SC(k, j)) * SB(l, j);
        if (possign) step(k, l, SC(k, l) - (suml + cj(sumr)), cj(SA(k, k) + SB(l, l)));
        else step(k, l, SC(k, l) - (suml - cj(sumr)), cj(SA(k, k) - SB(l, l)));
      }
  }
  if (perturbed) *perturbed = pert;
  return scale;
#undef SA
#undef SB
#undef SC
}

template <class R> inline R vnorm1(const std::vector<R>& x) {
  R s = 0;
  for (R v : x) s += m_abs(v);
  return s;
}
template <class R> inline R vnorm1(const std::vector<cx<R>>& x) {
  R s = 0;
  for (const cx<R>& v : x) s += cabs(v);
  return s;
}

// 2-norm of a vector without overflow (Julia's norm(R) of the Sylvester solution).
template <class R, class S> R vnorm2(const S* x, long long cnt) {
  R scale = 0, ssq = 1;
  for (long long i = 0; i < cnt; ++i) {
    R parts[2];
    int np;
    if constexpr (std::is_same<S, R>::value) { parts[0] = x[i]; np = 1; }
    else { parts[0] = x[i].re; parts[1] = x[i].im; np = 2; }
    for (int q = 0; q < np; ++q) {
      const R a = m_abs(parts[q]);
      if (a == R(0)) continue;
      if (scale < a) { ssq = R(1) + ssq * (scale / a) * (scale / a); scale = a; }
      else ssq += (a / scale) * (a / scale);
    }
  }
  return scale * m_sqrt(ssq);
}

// _findamax (norm1est.jl:76-99): first index of the largest |x| (via |x|^2 for complex).
template <class R> inline void findamax(const std::vector<R>& x, R* ax, int* idx) {
  R a0 = m_abs(x[0]);
  int i0 = 0;
  for (size_t i = 1; i < x.size(); ++i)
    if (m_abs(x[i]) > a0) { a0 = m_abs(x[i]); i0 = (int)i; }
  *ax = a0; *idx = i0;
}
template <class R> inline void findamax(const std::vector<cx<R>>& x, R* ax, int* idx) {
  R a0 = abs2(x[0]);
  int i0 = 0;
  for (size_t i = 1; i < x.size(); ++i)
    if (abs2(x[i]) > a0) { a0 = abs2(x[i]); i0 = (int)i; }
  *ax = m_sqrt(a0); *idx = i0;
}

template <class R> inline R unit_of(R x, R ax) { return x / ax; }
template <class R> inline cx<R> unit_of(cx<R> x, R ax) { return x / ax; }

// norm1est!(applyA!, applyAH!, y; maxiter = 5) (norm1est.jl:21-74).
template <class R, class S, class FA, class FH> R norm1est(int N, FA applyA, FH applyAH, int maxiter = 5) {
  std::vector<S> x(N, S(R(1) / R(N)));
  applyA(x);
  if (N == 1) return mod_of(x[0]);
  R gamma = vnorm1(x);
  const R tiny = safemin<R>();
  auto signs = [&]() {
    for (int i = 0; i < N; ++i) {
      const R a = mod_of(x[i]);
      x[i] = a > tiny ? unit_of(x[i], a) : S(R(1));
    }
  };
  signs();
  applyAH(x);
  R ax0;
  int j0;
  findamax(x, &ax0, &j0);
  for (int iter = 0; iter < maxiter; ++iter) {
    for (int i = 0; i < N; ++i) x[i] = S(R(0));
    x[j0] = S(R(1));
    applyA(x);
    const R old = gamma;
    gamma = vnorm1(x);
    if (gamma <= old) break;
    signs();
    applyAH(x);
    const int jlast = j0;
    findamax(x, &ax0, &j0);
    if (mod_of(x[jlast]) == ax0) break;
  }
  int isign = 1;
  for (int i = 0; i < N; ++i) {
    x[i] = S(R(isign) * (R(1) + R(i) / R(N - 1)));
    isign = -isign;
  }
  applyA(x);
  const R t = R(2) * vnorm1(x) / R(3 * N);
  return m_max(t, gamma);
}

// eigvalscond(S, nsub) (ordschur.jl:92-105) on the n x n upper (quasi-)triangular T.
template <class R, class S> R eigvalscond(int n, const S* T, int ldt, int nsub) {
  const int p = n - nsub;
  std::vector<S> Rm((size_t)nsub * p);
  for (int j = 0; j < p; ++j)
    for (int i = 0; i < nsub; ++i) Rm[i + (size_t)j * nsub] = T[i + (long long)(nsub + j) * ldt];
  const R scale = trsylvester<R, S>(false, nsub, p, T, ldt, T + nsub + (long long)nsub * ldt, ldt, Rm.data(),
                                    nsub, nullptr);
  const R rnorm = vnorm2<R, S>(Rm.data(), (long long)Rm.size());
  return rnorm > R(0) ? scale / (m_sqrt(scale * scale / rnorm + rnorm) * m_sqrt(rnorm)) : R(1);
}

// subspacesep(S, nsub) (ordschur.jl:118-140).
template <class R, class S> R subspacesep(int n, const S* T, int ldt, int nsub) {
  const int p = n - nsub;
  const S* A = T;
  const S* B = T + nsub + (long long)nsub * ldt;
  R scale = 1;
  auto f = [&](std::vector<S>& x) { scale = trsylvester<R, S>(false, nsub, p, A, ldt, B, ldt, x.data(), nsub, nullptr); };
  auto fh = [&](std::vector<S>& x) { scale = trsylvester<R, S>(true, nsub, p, A, ldt, B, ldt, x.data(), nsub, nullptr); };
  const R est = norm1est<R, S>(nsub * p, f, fh);
  return scale / est;
}

}  // namespace orc
