// CPU restatement of GenericSchur.jl's generalized Sylvester solvers and condition
// estimates for complex generalized Schur forms -- TEST INFRASTRUCTURE ONLY (the checker of
// the GPU kernels; never part of the product path):
//   trsylvester!(A, B, C, D, E, F)     src/gsylvester.jl:23-99
//   adjtrsylvester!(A, B, C, D, E, F)  src/gsylvester.jl:103-155
//   _trgsep (look-ahead)               src/gcondition.jl:8-115
//   eigvalscond(S::GeneralizedSchur)   src/gcondition.jl:121-165
//   subspacesep(S::GeneralizedSchur; pnorm = :F)  src/gcondition.jl:169-260
// Column-major; A, D m x m, B, E n x n upper triangular; C, F m x n.
#pragma once
#include <vector>
#include "eigvecs_oracle.hpp"

namespace orc {

// returns the scale of the last 2 x 2 solve, as the reference does
template <class R>
R gtrsyl(int m, int n, const cx<R>* A, const cx<R>* B, cx<R>* C, const cx<R>* D, const cx<R>* E, cx<R>* F) {
  typedef cx<R> Cx;
  R scale = R(1);
#define AM(i, j) A[((i) - 1) + (long long)((j) - 1) * m]
#define DM(i, j) D[((i) - 1) + (long long)((j) - 1) * m]
#define BM(i, j) B[((i) - 1) + (long long)((j) - 1) * n]
#define EM(i, j) E[((i) - 1) + (long long)((j) - 1) * n]
#define CM(i, j) C[((i) - 1) + (long long)((j) - 1) * m]
#define FM(i, j) F[((i) - 1) + (long long)((j) - 1) * m]
  for (int j = 1; j <= n; ++j)
    for (int i = m; i >= 1; --i) {
      Cx Z[4] = {AM(i, i), DM(i, i), -BM(j, j), -EM(j, j)};
      Cx rhs[2] = {CM(i, j), FM(i, j)};
      bool pert = false;
      scale = safe_lu_solve<R>(2, Z, rhs, &pert);
      CM(i, j) = rhs[0];
      FM(i, j) = rhs[1];
      if (scale != R(1))
        for (int k = 1; k <= n; ++k)
          for (int r = 1; r <= m; ++r) { CM(r, k) = CM(r, k) * scale; FM(r, k) = FM(r, k) * scale; }
      if (i > 1) {
        const Cx al = -rhs[0];
        for (int r = 1; r <= i - 1; ++r) { CM(r, j) += al * AM(r, i); FM(r, j) += al * DM(r, i); }
      }
      if (j < n) {
        const Cx al = rhs[1];
        for (int k = j + 1; k <= n; ++k) { CM(i, k) += al * BM(j, k); FM(i, k) += al * EM(j, k); }
      }
    }
  return scale;
}

template <class R>
R gadjtrsyl(int m, int n, const cx<R>* A, const cx<R>* B, cx<R>* C, const cx<R>* D, const cx<R>* E, cx<R>* F) {
  typedef cx<R> Cx;
  R scale = R(1);
  for (int i = 1; i <= m; ++i)
    for (int j = n; j >= 1; --j) {
      Cx Z[4] = {conj(AM(i, i)), -conj(BM(j, j)), conj(DM(i, i)), -conj(EM(j, j))};
      Cx rhs[2] = {CM(i, j), FM(i, j)};
      bool pert = false;
      scale = safe_lu_solve<R>(2, Z, rhs, &pert);
      CM(i, j) = rhs[0];
      FM(i, j) = rhs[1];
      if (scale != R(1))
        for (int k = 1; k <= n; ++k)
          for (int r = 1; r <= m; ++r) { CM(r, k) = CM(r, k) * scale; FM(r, k) = FM(r, k) * scale; }
      for (int jj = 1; jj <= j - 1; ++jj) FM(i, jj) += rhs[0] * conj(BM(jj, j)) + rhs[1] * conj(EM(jj, j));
      for (int ii = i + 1; ii <= m; ++ii) CM(ii, j) -= rhs[0] * conj(AM(i, ii)) + rhs[1] * conj(DM(i, ii));
    }
  return scale;
}

// _ssq (util.jl:466-505) step on one complex value
template <class R> inline void ssq_step(R& scale, R& sumsq, cx<R> x) {
  const R parts[2] = {m_abs(x.re), m_abs(x.im)};
  for (R t1 : parts)
    if (t1 > R(0) || t1 != t1) {
      if (scale < t1) { sumsq = R(1) + sumsq * (scale / t1) * (scale / t1); scale = t1; }
      else sumsq += (t1 / scale) * (t1 / scale);
    }
}

// _trgsep with the look-ahead choice of zlatdf (gcondition.jl:8-115)
template <class R>
R trgsep(int m, int n, const cx<R>* A, const cx<R>* B, const cx<R>* D, const cx<R>* E) {
  typedef cx<R> Cx;
  std::vector<Cx> Cv((size_t)m * n, Cx(R(0))), Fv((size_t)m * n, Cx(R(0)));
  Cx* C = Cv.data();
  Cx* F = Fv.data();
  R dif = R(0);
  R rdscale = R(0), rdsum = R(1);
  bool started = false;
  for (int j = 1; j <= n; ++j)
    for (int i = m; i >= 1; --i) {
      const Cx Z[4] = {AM(i, i), DM(i, i), -BM(j, j), -EM(j, j)};
      // lu(Z) with partial pivoting on |re| + |im| (LAPACK getrf)
      int p0 = 0, p1 = 1;
      if (abs1(Z[1]) > abs1(Z[0])) { p0 = 1; p1 = 0; }
      const Cx u11 = Z[p0], u12 = Z[p0 + 2];
      const Cx l21 = Z[p1] / u11;
      const Cx u22 = Z[p1 + 2] - l21 * u12;
      Cx rhs[2] = {CM(i, j), FM(i, j)};
      Cx x[2] = {rhs[p0], rhs[p1]};
      Cx pmone(R(-1));
      const Cx bp = x[0] + Cx(R(1)), bm = x[0] - Cx(R(1));
      R splus = R(1);
      splus += (conj(l21) * l21).re;
      const R sminu = (conj(l21) * x[1]).re;
      splus *= x[0].re;
      if (splus > sminu) x[0] = bp;
      else if (sminu > splus) x[0] = bm;
      else { x[0] += pmone; pmone = Cx(R(1)); }
      x[1] -= x[0] * l21;
      Cx w[2] = {x[0], x[1] + Cx(R(1))};
      x[1] -= Cx(R(1));
      R sp = R(0), sm = R(0);
      const Cx U[2] = {u11, u22};
      for (int k = 1; k >= 0; --k) {
        const Cx t = Cx(R(1)) / U[k];
        w[k] = w[k] * t;
        x[k] = x[k] * t;
        if (k == 0) {
          w[0] -= w[1] * (u12 * t);
          x[0] -= x[1] * (u12 * t);
        }
        sp += cabs(w[k]);
        sm += cabs(x[k]);
      }
      if (sp > sm) { x[0] = w[0]; x[1] = w[1]; }
      const Cx xs[2] = {x[p0], x[p1]};
      x[0] = xs[0];
      x[1] = xs[1];
      if (!started) { rdscale = R(1); rdsum = R(0); started = true; }
      ssq_step(rdscale, rdsum, x[0]);
      ssq_step(rdscale, rdsum, x[1]);
      if (rdscale != R(0)) dif = m_sqrt(R(2) * R(m) * R(n)) / (rdscale * m_sqrt(rdsum));
      CM(i, j) = x[0];
      FM(i, j) = x[1];
      if (i > 1) {
        const Cx al = -x[0];
        for (int r = 1; r <= i - 1; ++r) { CM(r, j) += al * AM(r, i); FM(r, j) += al * DM(r, i); }
      }
      if (j < n) {
        const Cx al = x[1];
        for (int k = j + 1; k <= n; ++k) { CM(i, k) += al * BM(j, k); FM(i, k) += al * EM(j, k); }
      }
    }
  return dif;
#undef AM
#undef DM
#undef BM
#undef EM
#undef CM
#undef FM
}

template <class R>
void sub_block(int n, const cx<R>* S, int r0, int c0, int rows, int cols, std::vector<cx<R>>& out) {
  out.resize((size_t)rows * cols);
  for (int j = 0; j < cols; ++j)
    for (int i = 0; i < rows; ++i) out[i + (size_t)j * rows] = S[(r0 + i) + (long long)(c0 + j) * n];
}

// eigvalscond(S::GeneralizedSchur, nsub) => (pl, pr)
template <class R>
void geigvalscond(int n, const cx<R>* S, const cx<R>* T, int nsub, R* pl, R* pr) {
  if (nsub == 0 || nsub == n) { *pl = R(1); *pr = R(1); return; }
  const int n1 = nsub, n2 = n - nsub;
  std::vector<cx<R>> S11, S22, T11, T22, Rm, Lm;
  sub_block(n, S, 0, 0, n1, n1, S11);
  sub_block(n, S, n1, n1, n2, n2, S22);
  sub_block(n, T, 0, 0, n1, n1, T11);
  sub_block(n, T, n1, n1, n2, n2, T22);
  sub_block(n, S, 0, n1, n1, n2, Rm);
  sub_block(n, T, 0, n1, n1, n2, Lm);
  const R scale = gtrsyl<R>(n1, n2, S11.data(), S22.data(), Rm.data(), T11.data(), T22.data(), Lm.data());
  auto proj = [&](const std::vector<cx<R>>& X) {
    R sc = R(0), sq = R(1);
    bool started = false;
    for (const auto& x : X) {
      if (!started) { sc = R(1); sq = R(0); started = true; }
      ssq_step(sc, sq, x);
    }
    const R p = started ? sc * m_sqrt(sq) : R(0);
    return p == R(0) ? R(1) : scale / (m_sqrt(scale * scale / p + p) * m_sqrt(p));
  };
  *pl = proj(Rm);
  *pr = proj(Lm);
}

// subspacesep(S::GeneralizedSchur, nsub; pnorm = :F) => [sep_u, sep_l]
template <class R>
void gsubspacesep(int n, const cx<R>* S, const cx<R>* T, int nsub, R* sep) {
  const int n1 = nsub, n2 = n - nsub;
  std::vector<cx<R>> S11, S22, T11, T22;
  sub_block(n, S, 0, 0, n1, n1, S11);
  sub_block(n, S, n1, n1, n2, n2, S22);
  sub_block(n, T, 0, 0, n1, n1, T11);
  sub_block(n, T, n1, n1, n2, n2, T22);
  sep[0] = trgsep<R>(n1, n2, S11.data(), S22.data(), T11.data(), T22.data());
  sep[1] = trgsep<R>(n2, n1, S22.data(), S11.data(), T22.data(), T11.data());
}

}  // namespace orc
