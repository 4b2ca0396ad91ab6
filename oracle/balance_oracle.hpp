// CPU oracle of the balancing step (TEST INFRASTRUCTURE ONLY; the shipped library
// never links this): a restatement of balance! and of the Balancer's lmul!/ldiv!
// (src/balance.jl:33-261), used by eigen! (src/pirates.jl:63-89).  1-based index
// macros so that the loops read against the reference line by line; column-major.
// Kept as written there: the 2-norms of the "pr" variant with sf(c, r) = c + r, and
// _findamax (src/norm1est.jl:76-99), which compares |x|^2 for complex entries.
#pragma once
#include <vector>
#include "scalar.hpp"

namespace orc {

template <class R> inline bool bal_zero(R x) { return x == R(0); }
template <class R> inline bool bal_zero(cx<R> x) { return x.re == R(0) && x.im == R(0); }
template <class R> inline R bal_abs(R x) { return m_abs(x); }
template <class R> inline R bal_abs(cx<R> x) { return cabs(x); }
template <class R> inline R bal_amax(R x) { return m_abs(x); }
template <class R> inline R bal_amax(cx<R> x) { return x.re * x.re + x.im * x.im; }
// _findamax returns the largest |x|, found through |x|^2 for complex entries
template <class R> inline R bal_amax_fin(R m, R) { return m; }
template <class R> inline R bal_amax_fin(R m, cx<R>) { return m_sqrt(m); }

// 2-norm of a strided vector (scaled sum of squares)
template <class R, class S> R bal_norm2(const S* x, int n, long long inc) {
  R scale = 0, ssq = 1;
  bool any = false;
  for (int i = 0; i < n; ++i) {
    const R a = bal_abs<R>(x[i * inc]);
    if (a != R(0)) {
      if (!any) { scale = a; ssq = 1; any = true; }
      else if (scale < a) { ssq = R(1) + ssq * (scale / a) * (scale / a); scale = a; }
      else { ssq += (a / scale) * (a / scale); }
    }
  }
  return any ? scale * m_sqrt(ssq) : R(0);
}

// balance!(A; scale, permute) (balance.jl:33-185).  sp (n) receives the permutation
// record (1-based), D (n) the scale factors; returns 0, or 2 on NaN.
template <class R, class S>
int balance(int n, S* a, int lda, bool do_scale, bool do_permute, int* ilo_out, int* ihi_out, int* sp, R* D,
            int* trivial_out) {
#define BA(i, j) a[((i) - 1) + (long long)((j) - 1) * lda]
  const R beta = R(2);
  const R factor = R(0.95);
  const R sfmin1 = std::numeric_limits<R>::min() / std::numeric_limits<R>::epsilon();
  const R sfmax1 = R(1) / sfmin1;
  const R sfmin2 = sfmin1 * beta;
  const R sfmax2 = R(1) / sfmin2;
  (void)sfmax1;
  for (int i = 0; i < n; ++i) { D[i] = R(1); sp[i] = 0; }
  int ilo = 1, ihi = n;
  bool trivial = true;
  auto swapcols = [&](int p, int q, int rows) {
    for (int i = 1; i <= rows; ++i) { S t = BA(i, p); BA(i, p) = BA(i, q); BA(i, q) = t; }
  };
  auto swaprows = [&](int p, int q, int c0) {
    for (int i = c0; i <= n; ++i) { S t = BA(p, i); BA(p, i) = BA(q, i); BA(q, i) = t; }
  };
  if (do_permute) {
    // rows that make the lower part upper triangular (balance.jl:62-95)
    ihi = n + 1;
    int js = 0;
    while (ihi > 1) {
      ihi -= 1;
      bool exch = false;
      int ms = 0;
      for (int j = ihi; j >= 1; --j) {
        exch = true;
        js = j;
        for (int i = 1; i <= ihi; ++i) {
          if (i == j) continue;
          if (!bal_zero(BA(j, i))) exch = false;
        }
        if (exch) { ms = ihi; break; }
      }
      if (exch) {
        sp[ms - 1] = js;
        if (js != ms) {
          trivial = false;
          swapcols(js, ms, ihi);
          swaprows(js, ms, ilo);
        }
      } else {
        break;
      }
    }
    // columns that make the left part upper triangular (balance.jl:96-130)
    if (ihi > 1) {
      ilo = 0;
      while (ilo < n) {
        ilo += 1;
        bool exch = false;
        int ms = 0;
        int js2 = 0;
        for (int j = ilo; j <= ihi; ++j) {
          js2 = j;
          exch = true;
          for (int i = ilo; i <= ihi; ++i) {
            if (i == j) continue;
            if (!bal_zero(BA(i, j))) exch = false;
          }
          if (exch) { ms = ilo; break; }
        }
        if (exch) {
          sp[ms - 1] = js2;
          if (ms != js2) {
            trivial = false;
            swapcols(js2, ms, ihi);
            swaprows(js2, ms, ilo);
          }
        } else {
          break;
        }
      }
    }
  }
  if (do_scale) {
    // balance.jl:135-181 (algo = :pr, p = 1)
    bool converged = false;
    long long sweeps = 0;
    while (!converged) {
      converged = true;
      if (++sweeps > 100000) break;
      for (int i = ilo; i <= ihi; ++i) {
        R c = bal_norm2<R>(&BA(ilo, i), ihi - ilo + 1, 1);
        R r = bal_norm2<R>(&BA(i, ilo), ihi - ilo + 1, lda);
        R ca = bal_amax<R>(BA(ilo, i)), ra = bal_amax<R>(BA(i, ilo));
        for (int k = ilo + 1; k <= ihi; ++k) {
          const R x = bal_amax<R>(BA(k, i)), y = bal_amax<R>(BA(i, k));
          if (x > ca) ca = x;
          if (y > ra) ra = y;
        }
        ca = bal_amax_fin<R>(ca, S());
        ra = bal_amax_fin<R>(ra, S());
        if (c == R(0) || r == R(0)) continue;
        R g = r / beta;
        const R s = c + r;
        R f = R(1);
        while (c < r / beta) {
          if (c >= g || m_max(m_max(f, c), ca) >= sfmax2 || m_min(m_min(r, g), ra) <= sfmin2) break;
          const R chk = c + f + ca + r + g + ra;
          if (chk != chk) return 2;
          f *= beta; c *= beta; ca *= beta; r /= beta; g /= beta; ra /= beta;
        }
        g = c / beta;
        while (r <= c / beta) {
          if (g < r || m_max(r, ra) >= sfmax2 || m_min(m_min(f, c), m_min(g, ca)) <= sfmin2) break;
          f /= beta; c /= beta; g /= beta; ca /= beta; r *= beta; ra *= beta;
        }
        if (f != R(1)) trivial = false;
        if (c + r >= factor * s) continue;
        converged = false;
        D[i - 1] *= f;
        const R rf = R(1) / f;
        for (int j = ilo; j <= n; ++j) BA(i, j) = BA(i, j) * rf;
        for (int j = 1; j <= ihi; ++j) BA(j, i) = BA(j, i) * f;
      }
    }
  }
  *ilo_out = ilo;
  *ihi_out = ihi;
  *trivial_out = trivial ? 1 : 0;
  return 0;
#undef BA
}

// lmul!(B, V) (inverse = false, right eigenvectors) and ldiv!(B, V) (inverse = true,
// left eigenvectors) on an n x m matrix V (balance.jl:189-261).
template <class R, class S>
void balancer_apply(int n, int m, S* v, int ldv, int ilo, int ihi, const int* sp, const R* D, bool trivial,
                    bool inverse) {
#define BV(i, j) v[((i) - 1) + (long long)((j) - 1) * ldv]
  if (trivial) return;
  if (ilo != ihi)
    for (int i = 1; i <= n; ++i) {
      const R d = inverse ? R(1) / D[i - 1] : D[i - 1];
      for (int j = 1; j <= m; ++j) BV(i, j) = BV(i, j) * d;
    }
  for (int j = ilo - 1; j >= 1; --j) {
    const int mm = sp[j - 1];
    if (mm == j) continue;
    for (int i = 1; i <= m; ++i) { S t = BV(j, i); BV(j, i) = BV(mm, i); BV(mm, i) = t; }
  }
  for (int j = ihi + 1; j <= n; ++j) {
    const int mm = sp[j - 1];
    if (mm == j) continue;
    for (int i = 1; i <= m; ++i) { S t = BV(j, i); BV(j, i) = BV(mm, i); BV(mm, i) = t; }
  }
#undef BV
}

}  // namespace orc
