// CPU oracle, eigenvector part: restatement of GenericSchur.jl's eigenvector
// back-substitution, its scaled triangular solvers and the real->complex Schur
// conversion.  TEST INFRASTRUCTURE ONLY (see gschur_oracle.hpp).  Loops use
// 1-based indices through the IDX macros to follow the cited reference lines;
// quirks of the reference (e.g. which column norms a call receives) are kept as
// written and marked "as written".
#pragma once
#include <vector>
#include "gschur_oracle.hpp"

namespace orc {

// _usolve!: upper-triangular solve A[1:n,1:n] x = s b with xLATRS-style scaling
// (util.jl:128-293).  x holds b on entry.  cnorm may be rescaled and restored.
template <class R, class S>
R usolve(const S* a, int lda, int n, S* x, R* cnorm) {
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * lda]
  auto cabs1half = [](S z) { return m_abs(re_of(z) / R(2)) + m_abs((abs1(z) - m_abs(re_of(z))) / R(2)); };
  const R half = R(1) / R(2);
  const R smallnum = safemin<R>() / lim<R>::eps();
  const R bignum = R(1) / smallnum;
  R xscale = 1;
  R tmax = m_abs(cnorm[0]);
  for (int j = 2; j <= n; ++j) tmax = m_max(tmax, m_abs(cnorm[j - 1]));
  R tscale;
  if (tmax <= bignum * half) {
    tscale = 1;
  } else {
    tscale = half / (smallnum * tmax);
    for (int j = 0; j < n; ++j) cnorm[j] *= tscale;
  }
  R xmax = cabs1half(x[0]);
  for (int j = 2; j <= n; ++j) xmax = m_max(xmax, cabs1half(x[j - 1]));
  R xbound = xmax;
  R grow;
  if (tscale != R(1)) {
    grow = 0;
  } else {
    grow = half / m_max(xbound, smallnum);
    xbound = grow;
    bool toosmall = false;
    for (int j = n; j >= 1; --j) {
      toosmall = (grow <= smallnum);
      if (toosmall) break;
      S tjjs = A_(j, j);
      R tjj = abs1(tjjs);
      if (tjj >= smallnum) xbound = m_min(xbound, m_min(R(1), tjj) * grow);
      else xbound = 0;
      if (tjj + cnorm[j - 1] >= smallnum) grow *= (tjj / (tjj + cnorm[j - 1]));
      else grow = 0;
    }
    if (!toosmall) grow = xbound;
  }
  if (grow * tscale > smallnum) {
    for (int j = n; j >= 1; --j) {
      S xj = x[j - 1] / A_(j, j);
      x[j - 1] = xj;
      for (int i = j - 1; i >= 1; --i) x[i - 1] -= A_(i, j) * xj;
    }
  } else {
    if (xmax > bignum * half) {
      xscale = (bignum * half) / xmax;
      for (int i = 0; i < n; ++i) x[i] *= xscale;
      xmax = bignum;
    } else {
      xmax *= 2;
    }
    for (int j = n; j >= 1; --j) {
      R xj = abs1(x[j - 1]);
      S tjjs = A_(j, j) * tscale;
      R tjj = abs1(tjjs);
      if (tjj > smallnum) {
        if (tjj < R(1)) {
          if (xj > tjj * bignum) {
            R rec = R(1) / xj;
            for (int i = 0; i < n; ++i) x[i] *= rec;
            xscale *= rec;
            xmax *= rec;
          }
        }
        x[j - 1] = x[j - 1] / tjjs;
        xj = abs1(x[j - 1]);
      } else if (tjj > R(0)) {
        if (xj > tjj * bignum) {
          R rec = (tjj * bignum) / xj;
          if (cnorm[j - 1] > R(1)) rec /= cnorm[j - 1];
          for (int i = 0; i < n; ++i) x[i] *= rec;
          xscale *= rec;
          xmax *= rec;
        }
        x[j - 1] = x[j - 1] / tjjs;
        xj = abs1(x[j - 1]);
      } else {
        for (int i = 0; i < n; ++i) x[i] = S(0);
        x[j - 1] = S(1);
        xscale = 0;
        xmax = 0;
      }
      if (xj > R(1)) {
        R rec = R(1) / xj;
        if (cnorm[j - 1] > (bignum - xmax) * rec) {
          rec *= half;
          for (int i = 0; i < n; ++i) x[i] *= rec;
          xscale *= rec;
        }
      } else if (xj * cnorm[j - 1] > bignum - xmax) {
        for (int i = 0; i < n; ++i) x[i] *= half;
        xscale *= half;
      }
      if (j > 1) {
        S xjt = x[j - 1] * tscale;
        for (int i = 1; i <= j - 1; ++i) x[i - 1] -= xjt * A_(i, j);
        xmax = abs1(x[0]);
        for (int i = 2; i <= j - 1; ++i) xmax = m_max(xmax, abs1(x[i - 1]));
      }
    }
    xscale /= tscale;
  }
  if (tscale != R(1))
    for (int i = 0; i < n; ++i) cnorm[i] *= R(1) / tscale;
  return xscale;
#undef A_
}

// _cusolve!: conjugate-transpose upper-triangular solve A^H x = s b with scaling
// (util.jl:301-461).
template <class R, class S>
R cusolve(const S* a, int lda, int n, S* x, R* cnorm) {
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * lda]
  auto cabs1half = [](S z) { return m_abs(re_of(z) / R(2)) + m_abs((abs1(z) - m_abs(re_of(z))) / R(2)); };
  const R half = R(1) / R(2);
  const R smallnum = safemin<R>() / lim<R>::eps();
  const R bignum = R(1) / smallnum;
  R xscale = 1;
  R tmax = m_abs(cnorm[0]);
  for (int j = 2; j <= n; ++j) tmax = m_max(tmax, m_abs(cnorm[j - 1]));
  R tscale;
  if (tmax <= bignum * half) {
    tscale = 1;
  } else {
    tscale = half / (smallnum * tmax);
    for (int j = 0; j < n; ++j) cnorm[j] *= tscale;
  }
  R xmax = cabs1half(x[0]);
  for (int j = 2; j <= n; ++j) xmax = m_max(xmax, cabs1half(x[j - 1]));
  R xbound = xmax;
  R grow;
  if (tscale != R(1)) {
    grow = 0;
  } else {
    grow = half / m_max(xbound, smallnum);
    xbound = grow;
    bool toosmall = false;
    for (int j = 1; j <= n; ++j) {
      toosmall = (grow <= smallnum);
      if (toosmall) break;
      R xj = R(1) + cnorm[j - 1];
      grow = m_min(grow, xbound / xj);
      R tjj = abs1(A_(j, j));
      if (tjj >= smallnum) {
        if (xj > tjj) xbound *= (tjj / xj);
      } else {
        xbound = 0;
      }
    }
    if (!toosmall) grow = m_min(grow, xbound);
  }
  if (grow * tscale > smallnum) {
    for (int j = 1; j <= n; ++j) {
      S zz = x[j - 1];
      for (int i = 1; i <= j - 1; ++i) zz -= cj(A_(i, j)) * x[i - 1];
      x[j - 1] = zz / cj(A_(j, j));
    }
  } else {
    if (xmax > bignum * half) {
      xscale = (bignum * half) / xmax;
      for (int i = 0; i < n; ++i) x[i] *= xscale;
      xmax = bignum;
    } else {
      xmax *= 2;
    }
    for (int j = 1; j <= n; ++j) {
      R xj = abs1(x[j - 1]);
      S uscale = S(tscale);
      R rec = R(1) / m_max(xmax, R(1));
      S tjjs = cj(A_(j, j)) * tscale;
      if (cnorm[j - 1] > (bignum - xj) * rec) {
        rec *= half;
        R tjj = abs1(tjjs);
        if (tjj > R(1)) {
          rec = m_min(R(1), rec * tjj);
          uscale = uscale / tjjs;
        }
        if (rec < R(1)) {
          for (int i = 0; i < n; ++i) x[i] *= rec;
          xscale *= rec;
          xmax *= rec;
        }
      }
      S csumj = S(0);
      for (int i = 1; i <= j - 1; ++i) csumj += (cj(A_(i, j)) * uscale) * x[i - 1];
      bool uscale_nan = m_isnan(re_of(uscale)) || m_isnan(abs1(uscale));
      if (uscale == S(tscale) || uscale_nan) {
        x[j - 1] -= csumj;
        xj = abs1(x[j - 1]);
        tjjs = cj(A_(j, j)) * tscale;
        R tjj = abs1(tjjs);
        if (tjj > smallnum) {
          if (tjj < R(1)) {
            if (xj > tjj * bignum) {
              R rec2 = R(1) / xj;
              for (int i = 0; i < n; ++i) x[i] *= rec2;
              xscale *= rec2;
              xmax *= rec2;
            }
          }
          x[j - 1] = x[j - 1] / tjjs;
        } else if (tjj > R(0)) {
          if (xj > tjj * bignum) {
            R rec2 = (tjj * bignum) / xj;
            for (int i = 0; i < n; ++i) x[i] *= rec2;
            xscale *= rec2;
            xmax *= rec2;
          }
          x[j - 1] = x[j - 1] / tjjs;
        } else {
          for (int i = 0; i < n; ++i) x[i] = S(0);
          x[j - 1] = S(1);
          xscale = 0;
          xmax = 0;
        }
      } else {
        x[j - 1] = x[j - 1] / tjjs - csumj;
      }
      xmax = m_max(xmax, abs1(x[j - 1]));
    }
    xscale /= tscale;
  }
  if (tscale != R(1))
    for (int i = 0; i < n; ++i) cnorm[i] *= R(1) / tscale;
  return xscale;
#undef A_
}

// _safe_lu_solve!: complete-pivoting LU solve of a small complex system with
// scaling and perturbation (util.jl:603-687).  a is nn x nn column-major, b length nn.
template <class R>
R safe_lu_solve(int nn, cx<R>* a, cx<R>* b, bool* perturbed) {
  typedef cx<R> C;
#define A_(i, j) a[((i) - 1) + ((j) - 1) * nn]
  *perturbed = false;
  const R smallnum = lim<R>::fmin() / lim<R>::eps();
  R smin = 0;
  for (int j = 1; j <= nn; ++j)
    for (int i = 1; i <= nn; ++i) smin = m_max(smin, cabs(A_(i, j)));
  smin = m_max(lim<R>::eps() * smin, smallnum);
  int jpiv[16] = {0};  // nn <= 16
  for (int i = 1; i <= nn - 1; ++i) {
    R xmax = 0;
    int ipsv = i, jpsv = i;
    for (int ip = i; ip <= nn; ++ip)
      for (int jp = i; jp <= nn; ++jp)
        if (cabs(A_(ip, jp)) >= xmax) { xmax = cabs(A_(ip, jp)); ipsv = ip; jpsv = jp; }
    if (ipsv != i) {
      for (int j = 1; j <= nn; ++j) { C t1 = A_(ipsv, j), t2 = A_(i, j); A_(ipsv, j) = t2; A_(i, j) = t1; }
      C tb = b[i - 1]; b[i - 1] = b[ipsv - 1]; b[ipsv - 1] = tb;
    }
    if (jpsv != i)
      for (int j = 1; j <= nn; ++j) { C t1 = A_(j, jpsv), t2 = A_(j, i); A_(j, jpsv) = t2; A_(j, i) = t1; }
    jpiv[i - 1] = jpsv;
    if (cabs(A_(i, i)) < smin) { *perturbed = true; A_(i, i) = C(smin); }
    for (int j = i + 1; j <= nn; ++j) {
      A_(j, i) = A_(j, i) / A_(i, i);
      b[j - 1] -= A_(j, i) * b[i - 1];
      for (int k = i + 1; k <= nn; ++k) A_(j, k) -= A_(j, i) * A_(i, k);
    }
  }
  if (cabs(A_(nn, nn)) < smin) { *perturbed = true; A_(nn, nn) = C(smin); }
  jpiv[nn - 1] = nn;
  R scale = 1;
  R aa = R(8) * smallnum;
  bool needscl = false;
  for (int i = 1; i <= nn; ++i)
    if (aa * cabs(b[i - 1]) > cabs(A_(i, i))) { needscl = true; break; }
  if (needscl) {
    R bmax = 0;
    for (int i = 0; i < nn; ++i) bmax = m_max(bmax, cabs(b[i]));
    scale = (R(1) / R(8)) / bmax;
    for (int i = 0; i < nn; ++i) b[i] *= scale;
  }
  for (int i = 1; i <= nn; ++i) {
    int k = nn + 1 - i;
    C t = C(1) / A_(k, k);
    b[k - 1] *= t;
    for (int j = k + 1; j <= nn; ++j) b[k - 1] -= (t * A_(k, j)) * b[j - 1];
  }
  for (int i = 1; i <= nn - 1; ++i) {
    int jj = jpiv[nn - i - 1];
    if (jj != nn - i) { C t = b[nn - i - 1]; b[nn - i - 1] = b[jj - 1]; b[jj - 1] = t; }
  }
  return scale;
#undef A_
}

// _xsolve: solve (a*A - b*D) X = s*B for a 1x1 or 2x2 real block A, complex b
// (util.jl:698-751).  A given as na x na column-major (already transposed by the
// caller where the reference passes an adjoint view).  B is overwritten with X.
template <class R>
R xsolve(R a, const R* A, int na, cx<R> b, cx<R>* B, R smin, R* xnorm, bool* perturbed) {
  typedef cx<R> C;
  R s = 1;
  const R small = R(2) * safemin<R>();
  const R bignum = s / small;
  smin = m_max(smin, small);
  *perturbed = false;
  if (na == 1) {
    R csr = a * A[0] - b.re;
    R csi = -b.im;
    R cnorm = m_abs(csr) + m_abs(csi);
    if (cnorm < smin) { *perturbed = true; csr = smin; csi = 0; cnorm = smin; }
    R bnorm = abs1(B[0]);
    if (cnorm < R(1) && bnorm > R(1) && bnorm > bignum * cnorm) s = R(1) / bnorm;
    C x = (B[0] * s) / C(csr, csi);
    *xnorm = abs1(x);
    B[0] = x;
    return s;
  }
  R cmax = 0;
  C m[4];
  for (int j = 1; j <= na; ++j)
    for (int i = 1; i <= na; ++i) {
      C zz = C(a * A[(i - 1) + (j - 1) * na]);
      if (i == j) zz -= b;
      m[(i - 1) + (j - 1) * na] = zz;
      cmax = m_max(cmax, abs1(zz));
    }
  if (cmax < smin) {
    *perturbed = true;
    R bnorm = 0;
    for (int i = 0; i < na; ++i) bnorm = m_max(bnorm, abs1(B[i]));
    if (smin < R(1) && bnorm > R(1) && bnorm > bignum * smin) s = R(1) / bnorm;
    R t1 = s / smin;
    for (int i = 0; i < na; ++i) B[i] *= t1;
  } else {
    bool pert2 = false;
    s = safe_lu_solve<R>(na, m, B, &pert2);
  }
  *xnorm = norm2_cplx(B, na);
  return s;
}

// _enormalize!: unit 2-norm columns with the largest-modulus entry made real
// (util.jl:572-592).
template <class R> void enormalize(int n, cx<R>* v, int ldv) {
  for (int j = 0; j < n; ++j) {
    cx<R>* col = v + (long long)j * ldv;
    R s = R(1) / norm2_cplx(col, n);
    R t = abs2(col[0]);
    int i0 = 0;
    for (int i = 1; i < n; ++i) {
      R u = abs2(col[i]);
      if (u > t) { i0 = i; t = u; }
    }
    cx<R> f = conj(col[i0]) * (s / m_sqrt(t));
    for (int i = 0; i < n; ++i) col[i] = col[i] * f;
    col[i0] = cx<R>(col[i0].re);
  }
}

// Complex right eigenvectors (ztrevc logic), vectors.jl:45-131.  T is modified
// temporarily and restored.  z may be null (then vectors of T itself).
template <class R>
void geigvecs_cplx(int n, cx<R>* t, int ldt, const cx<R>* z, int ldz, cx<R>* vec, int ldv) {
  typedef cx<R> C;
#define T_(i, j) t[((i) - 1) + (long long)((j) - 1) * ldt]
#define Z_(i, j) z[((i) - 1) + (long long)((j) - 1) * ldz]
#define V_(i, j) vec[((i) - 1) + (long long)((j) - 1) * ldv]
  const R ulp = lim<R>::eps();
  const R smallnum = safemin<R>() * R(n);
  std::vector<C> v(n + 1), tdiag(n + 1);
  std::vector<R> tnorms(n + 1, R(0));
  for (int k = 1; k <= n; ++k) tdiag[k - 1] = T_(k, k);
  for (int j = 2; j <= n; ++j)
    for (int i = 1; i <= j - 1; ++i) tnorms[j - 1] += cabs(T_(i, j));
  for (int ki = n; ki >= 1; --ki) {
    R smin = m_max(ulp * abs1(T_(ki, ki)), smallnum);
    v[0] = C(1);
    for (int k = 1; k <= ki - 1; ++k) v[k - 1] = -T_(k, ki);
    for (int k = 1; k <= ki - 1; ++k) {
      T_(k, k) -= T_(ki, ki);
      if (abs1(T_(k, k)) < smin) T_(k, k) = C(smin);
    }
    R vscale;
    if (ki > 1) {
      vscale = usolve<R, C>(t, ldt, ki - 1, v.data(), tnorms.data());
      v[ki - 1] = C(vscale);
    } else {
      vscale = 1;
    }
    if (z) {
      for (int j = 1; j <= n; ++j) {
        C acc = Z_(j, ki) * vscale;
        for (int i = 1; i <= ki - 1; ++i) acc += Z_(j, i) * v[i - 1];
        V_(j, ki) = acc;
      }
    } else {
      for (int j = 1; j <= ki; ++j) V_(j, ki) = v[j - 1];
      for (int j = ki + 1; j <= n; ++j) V_(j, ki) = C(0);
    }
    R t0 = abs1(V_(1, ki));
    for (int i = 2; i <= n; ++i) t0 = m_max(t0, abs1(V_(i, ki)));
    R remax = R(1) / t0;
    for (int i = 1; i <= n; ++i) V_(i, ki) *= remax;
    for (int k = 1; k <= ki - 1; ++k) T_(k, k) = tdiag[k - 1];
  }
#undef T_
#undef Z_
#undef V_
}

// Complex left eigenvectors, vectors.jl:372-460.
template <class R>
void gleigvecs_cplx(int n, cx<R>* t, int ldt, const cx<R>* z, int ldz, cx<R>* vec, int ldv) {
  typedef cx<R> C;
#define T_(i, j) t[((i) - 1) + (long long)((j) - 1) * ldt]
#define Z_(i, j) z[((i) - 1) + (long long)((j) - 1) * ldz]
#define V_(i, j) vec[((i) - 1) + (long long)((j) - 1) * ldv]
  const R ulp = lim<R>::eps();
  const R smallnum = safemin<R>() * R(n);
  std::vector<C> v(n + 1), tdiag(n + 1);
  std::vector<R> tnorms(n + 1, R(0));
  for (int k = 1; k <= n; ++k) tdiag[k - 1] = T_(k, k);
  for (int j = 2; j <= n; ++j)
    for (int i = 1; i <= j - 1; ++i) tnorms[j - 1] += abs1(T_(i, j));
  for (int ki = 1; ki <= n; ++ki) {
    R smin = m_max(ulp * abs1(T_(ki, ki)), smallnum);
    for (int k = ki + 1; k <= n; ++k) v[k - 1] = -conj(T_(ki, k));
    for (int k = 1; k <= ki; ++k) v[k - 1] = C(0);
    for (int k = ki + 1; k <= n; ++k) {
      T_(k, k) -= T_(ki, ki);
      if (abs1(T_(k, k)) < smin) T_(k, k) = C(smin);
    }
    R vscale;
    if (ki < n) {
      // as written at vectors.jl:417-420: the full tnorms vector is passed, so the
      // solver sees the norms of columns 1..n-ki
      vscale = cusolve<R, C>(&T_(ki + 1, ki + 1), ldt, n - ki, &v[ki], tnorms.data());
      v[ki - 1] = C(vscale);
    } else {
      v[n - 1] = C(1);
      vscale = 1;
    }
    if (z) {
      for (int j = 1; j <= n; ++j) {
        C acc = Z_(j, ki) * vscale;
        for (int i = ki + 1; i <= n; ++i) acc += Z_(j, i) * v[i - 1];
        V_(j, ki) = acc;
      }
    } else {
      for (int j = ki; j <= n; ++j) V_(j, ki) = v[j - 1];
      for (int j = 1; j <= ki - 1; ++j) V_(j, ki) = C(0);
    }
    R t0 = abs1(V_(1, ki));
    for (int i = 2; i <= n; ++i) t0 = m_max(t0, abs1(V_(i, ki)));
    R remax = R(1) / t0;
    for (int i = 1; i <= n; ++i) V_(i, ki) *= remax;
    for (int k = ki + 1; k <= n; ++k) T_(k, k) = tdiag[k - 1];
  }
#undef T_
#undef Z_
#undef V_
}

// Real right eigenvectors of a quasi-triangular T (dtrevc logic), vectors.jl:133-362.
// Output vec is complex n x n.
template <class R>
void geigvecs_real(int n, const R* t, int ldt, const R* z, int ldz, cx<R>* vec, int ldv) {
  typedef cx<R> C;
#define T_(i, j) t[((i) - 1) + (long long)((j) - 1) * ldt]
#define Z_(i, j) z[((i) - 1) + (long long)((j) - 1) * ldz]
#define V_(i, j) vec[((i) - 1) + (long long)((j) - 1) * ldv]
  const R ulp = lim<R>::eps();
  const R smallnum = safemin<R>() * (R(n) / ulp);
  const R bignum = (R(1) - ulp) / smallnum;
  const bool have_z = (z != nullptr);
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= n; ++i) V_(i, j) = C(0);
  std::vector<C> v(n + 1);
  std::vector<R> tnorms(n + 1, R(0));
  for (int j = 2; j <= n; ++j)
    for (int i = 1; i <= j - 1; ++i) tnorms[j - 1] += m_abs(T_(i, j));
  int ip = 0;
  int isel = n;
  for (int ki = n; ki >= 1; --ki) {
    if (ip == 1) {
      ip = 0;
      if (have_z) {
        for (int i = 1; i <= n; ++i) V_(i, ki) = conj(V_(i, ki + 1));
      } else {
        for (int i = 1; i <= n; ++i) V_(i, isel + 1) = conj(V_(i, isel + 2));
      }
      continue;
    }
    if (ki > 1 && T_(ki, ki - 1) != R(0)) ip = -1;
    R wr = T_(ki, ki);
    R wi = (ip == 0) ? R(0) : m_sqrt(m_abs(T_(ki, ki - 1))) * m_sqrt(m_abs(T_(ki - 1, ki)));
    R smin = m_max(ulp * (m_abs(wr) + m_abs(wi)), smallnum);
    if (ip == 0) {
      v[ki - 1] = C(1);
      for (int k = 1; k <= ki - 1; ++k) v[k - 1] = C(-T_(k, ki));
      int jnxt = ki - 1;
      for (int j = ki - 1; j >= 1; --j) {
        if (j > jnxt) continue;
        int j1 = j, j2 = j;
        if (j > 1 && T_(j, j - 1) != R(0)) { j1 = j - 1; jnxt = j - 2; }
        if (j1 == j2) {
          C x[1] = {v[j - 1]};
          R blk[1] = {T_(j, j)};
          R t1; bool pert;
          R vscale = xsolve<R>(R(1), blk, 1, C(wr), x, smin, &t1, &pert);
          if (t1 > R(1) && tnorms[j - 1] > bignum / t1) { x[0] = x[0] / t1; vscale /= t1; }
          if (vscale != R(1))
            for (int i = 1; i <= ki; ++i) v[i - 1] *= vscale;
          v[j - 1] = x[0];
          for (int i = 1; i <= j - 1; ++i) v[i - 1] = v[i - 1] - x[0] * T_(i, j);
        } else {
          C x[2] = {v[j - 2], v[j - 1]};
          R blk[4] = {T_(j - 1, j - 1), T_(j, j - 1), T_(j - 1, j), T_(j, j)};
          R t1; bool pert;
          R vscale = xsolve<R>(R(1), blk, 2, C(wr), x, smin, &t1, &pert);
          if (t1 > R(1)) {
            R beta = m_max(tnorms[j - 2], tnorms[j - 1]);
            if (beta > bignum / t1) { x[0] = x[0] / t1; x[1] = x[1] / t1; vscale /= t1; }
          }
          if (vscale != R(1))
            for (int i = 1; i <= ki; ++i) v[i - 1] *= vscale;
          v[j - 2] = x[0];
          v[j - 1] = x[1];
          for (int i = 1; i <= j - 2; ++i) v[i - 1] = v[i - 1] - x[0] * T_(i, j - 1) - x[1] * T_(i, j);
        }
      }
      if (!have_z) {
        R mx = 0;
        for (int i = 1; i <= ki; ++i) mx = m_max(mx, cabs(v[i - 1]));
        R vscale = R(1) / mx;
        for (int i = 1; i <= ki; ++i) V_(i, isel) = v[i - 1] * vscale;
      } else {
        if (ki == 1) {
          for (int i = 1; i <= n; ++i) V_(i, ki) = C(Z_(i, ki));
        } else {
          for (int i = 1; i <= n; ++i) {
            C acc(0);
            for (int k = 1; k <= ki; ++k) acc += v[k - 1] * Z_(i, k);
            V_(i, ki) = acc;
          }
          R mx = 0;
          for (int i = 1; i <= n; ++i) mx = m_max(mx, cabs(V_(i, ki)));
          R vscale = R(1) / mx;
          for (int i = 1; i <= n; ++i) V_(i, ki) *= vscale;
        }
      }
    } else {
      if (m_abs(T_(ki - 1, ki)) >= m_abs(T_(ki, ki - 1))) {
        v[ki - 2] = C(1);
        v[ki - 1] = C(R(0), wi / T_(ki - 1, ki));
      } else {
        v[ki - 2] = C(-wi / T_(ki, ki - 1));
        v[ki - 1] = C(R(0), R(1));
      }
      for (int i = 1; i <= ki - 2; ++i)
        v[i - 1] = C(-v[ki - 2].re * T_(i, ki - 1), -v[ki - 1].im * T_(i, ki));
      int jnxt = ki - 2;
      for (int j = ki - 2; j >= 1; --j) {
        if (j > jnxt) continue;
        int j1 = j, j2 = j;
        jnxt = j - 1;
        if (j > 1 && T_(j, j - 1) != R(0)) { j1 = j - 1; jnxt = j - 2; }
        if (j1 == j2) {
          C x[1] = {v[j - 1]};
          R blk[1] = {T_(j, j)};
          R t1; bool pert;
          R vscale = xsolve<R>(R(1), blk, 1, C(wr, wi), x, smin, &t1, &pert);
          if (t1 > R(1) && tnorms[j - 1] > bignum / t1) { x[0] = x[0] / t1; vscale /= t1; }
          if (vscale != R(1))
            for (int i = 1; i <= ki; ++i) v[i - 1] *= vscale;
          v[j - 1] = x[0];
          for (int i = 1; i <= j - 1; ++i) v[i - 1] = v[i - 1] - x[0] * T_(i, j);
        } else {
          C x[2] = {v[j - 2], v[j - 1]};
          R blk[4] = {T_(j - 1, j - 1), T_(j, j - 1), T_(j - 1, j), T_(j, j)};
          R t1; bool pert;
          R vscale = xsolve<R>(R(1), blk, 2, C(wr, wi), x, smin, &t1, &pert);
          if (t1 > R(1)) {
            R beta = m_max(tnorms[j - 2], tnorms[j - 1]);
            if (beta > bignum / t1) { x[0] = x[0] / t1; x[1] = x[1] / t1; vscale /= t1; }
          }
          if (vscale != R(1))
            for (int i = 1; i <= ki; ++i) v[i - 1] *= vscale;
          v[j - 2] = x[0];
          v[j - 1] = x[1];
          for (int i = 1; i <= j - 2; ++i) v[i - 1] = v[i - 1] - x[0] * T_(i, j - 1) - x[1] * T_(i, j);
        }
      }
      if (!have_z) {
        for (int k = 1; k <= ki; ++k) V_(k, isel) = conj(v[k - 1]);
        R t1 = 0;
        for (int k = 1; k <= ki; ++k) t1 = m_max(t1, abs1(V_(k, isel)));
        t1 = R(1) / t1;
        for (int k = 1; k <= ki; ++k) V_(k, isel) *= t1;
      } else {
        for (int i = 1; i <= n; ++i) {
          C acc(0);
          for (int k = 1; k <= ki; ++k) acc += v[k - 1] * Z_(i, k);
          V_(i, ki) = acc;
        }
        R mx = 0;
        for (int i = 1; i <= n; ++i) mx = m_max(mx, cabs(V_(i, ki)));
        R vscale = R(1) / mx;
        for (int i = 1; i <= n; ++i) V_(i, ki) = conj(V_(i, ki)) * vscale;
      }
    }
    isel -= (ip == 0) ? 1 : 2;
    if (ip == -1) ip = 1;
  }
#undef T_
#undef Z_
#undef V_
}

// Real left eigenvectors, vectors.jl:462-698.
template <class R>
void gleigvecs_real(int n, const R* t, int ldt, const R* z, int ldz, cx<R>* vec, int ldv) {
  typedef cx<R> C;
#define T_(i, j) t[((i) - 1) + (long long)((j) - 1) * ldt]
#define Z_(i, j) z[((i) - 1) + (long long)((j) - 1) * ldz]
#define V_(i, j) vec[((i) - 1) + (long long)((j) - 1) * ldv]
  const R ulp = lim<R>::eps();
  const R smallnum = safemin<R>() * (R(n) / ulp);
  const R bignum = (R(1) - ulp) / smallnum;
  const bool have_z = (z != nullptr);
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= n; ++i) V_(i, j) = C(0);
  std::vector<C> v(n + 1);
  std::vector<R> tnorms(n + 1, R(0));
  for (int j = 2; j <= n; ++j)
    for (int i = 1; i <= j - 1; ++i) tnorms[j - 1] += m_abs(T_(i, j));
  int ip = 0;
  int isel = 1;
  for (int ki = 1; ki <= n; ++ki) {
    if (ip == -1) {
      ip = 0;
      if (have_z) {
        for (int i = 1; i <= n; ++i) V_(i, ki) = conj(V_(i, ki - 1));
      } else {
        for (int i = 1; i <= n; ++i) V_(i, isel - 1) = conj(V_(i, isel - 2));
      }
      continue;
    }
    if (ki < n && T_(ki + 1, ki) != R(0)) ip = 1;
    R wr = T_(ki, ki);
    R wi = (ip == 0) ? R(0) : m_sqrt(m_abs(T_(ki, ki + 1))) * m_sqrt(m_abs(T_(ki + 1, ki)));
    R smin = m_max(ulp * (m_abs(wr) + m_abs(wi)), smallnum);
    if (ip == 0) {
      v[ki - 1] = C(1);
      for (int k = ki + 1; k <= n; ++k) v[k - 1] = C(-T_(ki, k));
      R vmax = 1;
      R vcrit = bignum;
      int jnxt = ki + 1;
      for (int j = ki + 1; j <= n; ++j) {
        if (j < jnxt) continue;
        int j1 = j, j2 = j;
        jnxt = j + 1;
        if (j < n && T_(j + 1, j) != R(0)) { j2 = j + 1; jnxt = j + 2; }
        if (j1 == j2) {
          if (tnorms[j - 1] > vcrit) {
            R t1 = R(1) / vmax;
            for (int i = ki; i <= n; ++i) v[i - 1] *= t1;
            vmax = 1;
            vcrit = bignum;
          }
          C acc(0);
          for (int i = ki + 1; i <= j - 1; ++i) acc += v[i - 1] * T_(i, j);
          C x[1] = {v[j - 1] - acc};
          R blk[1] = {T_(j, j)};
          R xn; bool pert;
          R vscale = xsolve<R>(R(1), blk, 1, C(wr), x, smin, &xn, &pert);
          if (vscale != R(1))
            for (int i = ki; i <= n; ++i) v[i - 1] *= vscale;
          v[j - 1] = x[0];
          vmax = m_max(cabs(v[j - 1]), vmax);
          vcrit = bignum / vmax;
        } else {
          R beta = m_max(tnorms[j], tnorms[j - 1]);
          if (beta > vcrit) {
            R t1 = R(1) / vmax;
            for (int i = ki; i <= n; ++i) v[i - 1] *= t1;
            vmax = 1;
            vcrit = bignum;
          }
          C acc0(0), acc1(0);
          for (int i = ki + 1; i <= j - 1; ++i) {
            acc0 += v[i - 1] * T_(i, j);
            acc1 += v[i - 1] * T_(i, j + 1);
          }
          C x[2] = {v[j - 1] - acc0, v[j] - acc1};
          // transpose of T[j:j+1, j:j+1]
          R blk[4] = {T_(j, j), T_(j, j + 1), T_(j + 1, j), T_(j + 1, j + 1)};
          R xn; bool pert;
          R vscale = xsolve<R>(R(1), blk, 2, C(wr), x, smin, &xn, &pert);
          if (vscale != R(1))
            for (int i = ki; i <= n; ++i) v[i - 1] *= vscale;
          v[j - 1] = x[0];
          v[j] = x[1];
          vmax = m_max(cabs(v[j - 1]), m_max(cabs(v[j]), vmax));
          vcrit = bignum / vmax;
        }
      }
      if (!have_z) {
        R mx = 0;
        for (int i = ki; i <= n; ++i) mx = m_max(mx, cabs(v[i - 1]));
        R vscale = R(1) / mx;
        for (int i = ki; i <= n; ++i) V_(i, isel) = v[i - 1] * vscale;
      } else {
        if (ki == n) {
          for (int i = 1; i <= n; ++i) V_(i, ki) = C(Z_(i, ki));
        } else {
          for (int i = 1; i <= n; ++i) {
            C acc(0);
            for (int k = ki; k <= n; ++k) acc += v[k - 1] * Z_(i, k);
            V_(i, ki) = acc;
          }
          R mx = 0;
          for (int i = 1; i <= n; ++i) mx = m_max(mx, cabs(V_(i, ki)));
          R vscale = R(1) / mx;
          for (int i = 1; i <= n; ++i) V_(i, ki) *= vscale;
        }
      }
    } else {
      if (m_abs(T_(ki, ki + 1)) >= m_abs(T_(ki + 1, ki))) {
        v[ki - 1] = C(wi / T_(ki, ki + 1));
        v[ki] = C(R(0), R(1));
      } else {
        v[ki - 1] = C(1);
        v[ki] = C(R(0), -wi / T_(ki + 1, ki));
      }
      for (int i = ki + 2; i <= n; ++i)
        v[i - 1] = C(-v[ki - 1].re * T_(ki, i), -v[ki].im * T_(ki + 1, i));
      R vmax = 1;
      R vcrit = bignum;
      int jnxt = ki + 2;
      for (int j = ki + 1; j <= n; ++j) {
        if (j < jnxt) continue;
        int j1 = j, j2 = j;
        jnxt = j + 1;
        if (j < n && T_(j + 1, j) != R(0)) { j1 = j + 1; jnxt = j + 2; }
        if (j1 == j2) {
          if (tnorms[j - 1] > vcrit) {
            R t1 = R(1) / vmax;
            for (int i = ki; i <= n; ++i) v[i - 1] *= t1;
            vmax = 1;
            vcrit = bignum;
          }
          C acc(0);
          for (int i = ki + 2; i <= j - 1; ++i) acc += v[i - 1] * T_(i, j);
          C x[1] = {v[j - 1] - acc};
          R blk[1] = {T_(j, j)};
          R xn; bool pert;
          R vscale = xsolve<R>(R(1), blk, 1, C(wr, -wi), x, smin, &xn, &pert);
          if (vscale != R(1))
            for (int i = ki; i <= n; ++i) v[i - 1] *= vscale;
          v[j - 1] = x[0];
          vmax = m_max(abs1(v[j - 1]), vmax);
          vcrit = bignum / vmax;
        } else {
          R beta = m_max(tnorms[j - 2], tnorms[j - 1]);  // as written at vectors.jl:653
          if (beta > vcrit) {
            R t1 = R(1) / vmax;
            for (int i = ki; i <= n; ++i) v[i - 1] *= t1;
            vmax = 1;
            vcrit = bignum;
          }
          C acc0(0), acc1(0);
          for (int i = ki + 2; i <= j - 1; ++i) {
            acc0 += v[i - 1] * T_(i, j);
            acc1 += v[i - 1] * T_(i, j + 1);
          }
          C x[2] = {v[j - 1] - acc0, v[j] - acc1};
          R blk[4] = {T_(j, j), T_(j, j + 1), T_(j + 1, j), T_(j + 1, j + 1)};
          R xn; bool pert;
          R vscale = xsolve<R>(R(1), blk, 2, C(wr, -wi), x, smin, &xn, &pert);
          if (vscale != R(1))
            for (int i = ki; i <= n; ++i) v[i - 1] *= vscale;
          v[j - 1] = x[0];
          v[j] = x[1];
          vmax = m_max(abs1(x[0]), m_max(abs1(x[1]), vmax));
          vcrit = bignum / vmax;
        }
      }
      if (!have_z) {
        for (int k = ki; k <= n; ++k) V_(k, isel) = v[k - 1];
        R t1 = 0;
        for (int k = ki; k <= n; ++k) t1 = m_max(t1, abs1(V_(k, isel)));
        t1 = R(1) / t1;
        for (int k = ki; k <= n; ++k) V_(k, isel) *= t1;
      } else {
        for (int i = 1; i <= n; ++i) {
          C acc(0);
          for (int k = ki; k <= n; ++k) acc += v[k - 1] * Z_(i, k);
          V_(i, ki) = acc;
        }
        R mx = 0;
        for (int i = 1; i <= n; ++i) mx = m_max(mx, cabs(V_(i, ki)));
        R vscale = R(1) / mx;
        for (int i = 1; i <= n; ++i) V_(i, ki) *= vscale;
      }
    }
    isel += (ip == 0) ? 1 : 2;
    if (ip == 1) ip = -1;
  }
#undef T_
#undef Z_
#undef V_
}

// triangularize: standard-form real quasi-triangular Schur -> complex triangular
// Schur by one unitary rotation per 2x2 block (triang.jl:9-43).
template <class R>
void triangularize(int n, const R* tr, int ldt, const R* zr, int ldz, cx<R>* tc, cx<R>* zc, cx<R>* w) {
  typedef cx<R> C;
#define TR_(i, j) tr[((i) - 1) + (long long)((j) - 1) * ldt]
#define TC_(i, j) tc[((i) - 1) + (long long)((j) - 1) * n]
#define ZC_(i, j) zc[((i) - 1) + (long long)((j) - 1) * n]
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= n; ++i) {
      TC_(i, j) = C(TR_(i, j));
      ZC_(i, j) = C(zr[(i - 1) + (long long)(j - 1) * ldz]);
    }
  for (int j = n; j >= 2; --j) {
    if (TR_(j, j - 1) != R(0)) {
      R s = m_sqrt(m_abs(TR_(j, j - 1)));
      R c = m_sqrt(m_abs(TR_(j - 1, j)));
      R r = m_hypot(s, c);
      C gc(c / r);                 // Givens c (complex, real-valued)
      C gs(R(0), -(s / r));        // Givens s = -i * s/r
      const int p = j - 1, q = j;
      for (int k = 1; k <= n; ++k) {  // lmul!(G, T)
        C a1 = TC_(p, k), a2 = TC_(q, k);
        TC_(p, k) = gc * a1 + gs * a2;
        TC_(q, k) = -conj(gs) * a1 + gc * a2;
      }
      for (int k = 1; k <= n; ++k) {  // rmul!(T, G')
        C a1 = TC_(k, p), a2 = TC_(k, q);
        TC_(k, p) = a1 * gc + a2 * conj(gs);
        TC_(k, q) = -(a1 * gs) + a2 * gc;
      }
      for (int k = 1; k <= n; ++k) {  // rmul!(Z, G')
        C a1 = ZC_(k, p), a2 = ZC_(k, q);
        ZC_(k, p) = a1 * gc + a2 * conj(gs);
        ZC_(k, q) = -(a1 * gs) + a2 * gc;
      }
    }
  }
  for (int j = 1; j <= n; ++j)
    for (int i = j + 1; i <= n; ++i) TC_(i, j) = C(0);
  for (int j = 1; j <= n; ++j) w[j - 1] = TC_(j, j);
#undef TR_
#undef TC_
#undef ZC_
}

}  // namespace orc
