// CPU oracle: a restatement of GenericSchur.jl's dense non-symmetric Schur path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links or calls this
// code; tests, the smoke check and bench.py's CPU-baseline leg use it as the
// checker.  Every routine cites the reference file:line it restates.  Indices in
// the bodies are 1-based through the IDX macros so that each loop can be read
// against the reference line by line; storage is column-major (Julia layout).
//
// Parity status: pinned by the reference's own known answers (the Godunov matrix,
// test/testfuncs.jl:127-142, exact eigenvalues {-4,-2,-1,0,1,2,4}) and by its
// property tests (test/real.jl:24-99, test/complex.jl:1-61, test/testfuncs.jl:5-86),
// restated in tests/.  The reference itself (Julia) cannot run in this build
// environment, so no element-wise golden outputs of the reference exist.
#pragma once
#include <vector>
#include <algorithm>
#include "scalar.hpp"

namespace orc {

enum { ORC_OK = 0, ORC_UNCONVERGED = 1, ORC_BADARG = 2 };

// ---------------------------------------------------------------------------
// util.jl
// ---------------------------------------------------------------------------

// _norm2 for real vectors, scaled sum of squares (util.jl:506-525).
template <class R> R norm2_real(const R* x, int n) {
  if (n < 1) return R(0);
  if (n == 1) return m_abs(x[0]);
  R scale = 0, ssq = 0;
  for (int i = 0; i < n; ++i) {
    if (x[i] != R(0)) {
      R a = m_abs(x[i]);
      if (scale < a) { ssq = R(1) + ssq * (scale / a) * (scale / a); scale = a; }
      else { ssq += (a / scale) * (a / scale); }
    }
  }
  return scale * m_sqrt(ssq);
}

// _norm2 for complex vectors (util.jl:527-557).
template <class R> R norm2_cplx(const cx<R>* x, int n) {
  if (n < 1) return R(0);
  if (n == 1) return cabs(x[0]);
  R scale = 0, ssq = 0;
  for (int i = 0; i < n; ++i) {
    R parts[2] = {x[i].re, x[i].im};
    for (int p = 0; p < 2; ++p) {
      if (parts[p] != R(0)) {
        R a = m_abs(parts[p]);
        if (scale < a) { ssq = R(1) + ssq * (scale / a) * (scale / a); scale = a; }
        else { ssq += (a / scale) * (a / scale); }
      }
    }
  }
  return scale * m_sqrt(ssq);
}

// _hypot3 (util.jl:562-570).
template <class R> R hypot3(R x, R y, R z) {
  R xa = m_abs(x), ya = m_abs(y), za = m_abs(z);
  R w = m_max(xa, m_max(ya, za));
  R rw = R(1) / w;
  return w * m_sqrt((rw * xa) * (rw * xa) + (rw * ya) * (rw * ya) + (rw * za) * (rw * za));
}

// safescale! (xLASCL): multiply by cto/cfrom without over/underflow (util.jl:41-80).
template <class R, class S> void safescale(S* a, long long len, R cfrom, R cto) {
  R smlnum = safemin<R>();
  R bignum = R(1) / smlnum;
  R cfromc = cfrom, ctoc = cto;
  bool done = false;
  while (!done) {
    R cfrom1 = cfromc * smlnum;
    R mul;
    if (cfrom1 == cfromc) {
      mul = ctoc / cfromc; done = true;
    } else {
      R cto1 = ctoc / bignum;
      if (cto1 == ctoc) {
        mul = cto; done = true; cfromc = R(1);
      } else if (m_abs(cfrom1) > m_abs(ctoc) && ctoc != R(0)) {
        // as written at util.jl:64-67 (LAPACK's xLASCL sets cfromc = cfrom1 here)
        mul = smlnum; done = false; cfromc = R(1);
      } else if (m_abs(cto1) > m_abs(cfromc)) {
        // as written at util.jl:68-71 (LAPACK's xLASCL sets ctoc = cto1 here)
        mul = bignum; done = false; cfromc = cfrom1;
      } else {
        mul = ctoc / cfromc; done = true;
      }
    }
    for (long long i = 0; i < len; ++i) a[i] = a[i] * mul;
  }
}

// _scale!: scale A when max|a_ij| is outside [smlnum, bignum] (util.jl:14-29).
// norm(A, Inf) of a matrix in Julia is the largest element modulus.
template <class R, class S>
bool scale_matrix(int n, S* a, int lda, R* cscale_out, R* anrm_out) {
  R smlnum = m_sqrt(safemin<R>()) / lim<R>::eps();
  R bignum = R(1) / smlnum;
  R anrm = 0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      R v = modulus(a[i + (long long)j * lda]);
      if (m_isnan(v)) anrm = v;
      else if (!(v <= anrm)) anrm = v;
    }
  bool scaleA = false;
  R cscale = 1;
  if (anrm > R(0) && anrm < smlnum) { scaleA = true; cscale = smlnum; }
  else if (anrm > bignum) { scaleA = true; cscale = bignum; }
  if (scaleA) {
    for (int j = 0; j < n; ++j) safescale<R, S>(a + (long long)j * lda, n, anrm, cscale);
  }
  *cscale_out = cscale;
  *anrm_out = anrm;
  return scaleA;
}

// ---------------------------------------------------------------------------
// householder.jl
// ---------------------------------------------------------------------------

// Real reflector (xLARFG) with underflow protection (householder.jl:12-54).
// On return x[0] = beta, x[1..n-1] = essential part of v; returns tau.
template <class R> R reflector_real(R* x, int n) {
  if (n <= 1) return R(0);
  R sfmin = R(2) * lim<R>::fmin() / lim<R>::eps();
  R alpha = x[0];
  R xnorm = norm2_real(x + 1, n - 1);
  if (xnorm == R(0)) return R(0);
  R beta = -m_copysign(m_hypot(alpha, xnorm), alpha);
  int kount = 0;
  bool smallb = m_abs(beta) < sfmin;
  if (smallb) {
    R rsfmin = R(1) / sfmin;
    while (smallb) {
      ++kount;
      for (int j = 1; j < n; ++j) x[j] *= rsfmin;
      beta *= rsfmin;
      alpha *= rsfmin;
      smallb = (m_abs(beta) < sfmin) && (kount < 20);
    }
    xnorm = norm2_real(x + 1, n - 1);
    beta = -m_copysign(m_hypot(alpha, xnorm), alpha);
  }
  R tau = (beta - alpha) / beta;
  R t = R(1) / (alpha - beta);
  for (int j = 1; j < n; ++j) x[j] *= t;
  for (int j = 0; j < kount; ++j) beta *= sfmin;
  x[0] = beta;
  return tau;
}

// Complex reflector (xLARFG) giving a real beta (householder.jl:56-102).
template <class R> cx<R> reflector_cplx(cx<R>* x, int n) {
  if (n < 1) return cx<R>(0);
  R sfmin = lim<R>::fmin() / lim<R>::eps();
  cx<R> alpha = x[0];
  R ar = alpha.re, ai = alpha.im;
  R xnorm = norm2_cplx(x + 1, n - 1);
  if (xnorm == R(0) && ai == R(0)) return cx<R>(0);
  R beta = -m_copysign(hypot3(ar, ai, xnorm), ar);
  int kount = 0;
  bool smallb = m_abs(beta) < sfmin;
  if (smallb) {
    R rsfmin = R(1) / sfmin;
    while (smallb) {
      ++kount;
      for (int j = 1; j < n; ++j) x[j] *= rsfmin;
      beta *= rsfmin;
      ar *= rsfmin;
      ai *= rsfmin;
      smallb = (m_abs(beta) < sfmin) && (kount < 20);
    }
    xnorm = norm2_cplx(x + 1, n - 1);
    alpha = cx<R>(ar, ai);
    beta = -m_copysign(hypot3(ar, ai, xnorm), ar);
  }
  cx<R> tau((beta - ar) / beta, -ai / beta);
  cx<R> t = R(1) / (alpha - cx<R>(beta));
  for (int j = 1; j < n; ++j) x[j] = x[j] * t;
  for (int j = 0; j < kount; ++j) beta *= sfmin;
  x[0] = cx<R>(beta);
  return tau;
}

template <class R> inline R reflector(R* x, int n) { return reflector_real(x, n); }
template <class R> inline cx<R> reflector(cx<R>* x, int n) { return reflector_cplx(x, n); }

// ---------------------------------------------------------------------------
// hessenberg.jl
// ---------------------------------------------------------------------------

// Unblocked Householder Hessenberg reduction (hessenberg.jl:3-17) with the
// reflector applications lmul!(H', .) (householder.jl:157-172) and rmul!(., H)
// (householder.jl:140-155).  tau has n-1 entries; reflector i's essential part
// is stored below the subdiagonal of column i.
template <class S> void hessenberg(int n, S* a, int lda, S* tau) {
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * lda]
  std::vector<S> x(n > 0 ? n : 1);
  for (int i = 1; i <= n - 1; ++i) {
    S t = reflector(&A_(i + 1, i), n - i);
    tau[i - 1] = t;
    // u = [1; A[i+2:n, i]]
    const int m = n - i;  // length of u
    // lmul!(H', A[i+1:n, i+1:n]): A <- (I - conj(t) u u^H) A
    for (int j = i + 1; j <= n; ++j) {
      S va = A_(i + 1, j);
      for (int r = 2; r <= m; ++r) va += cj(A_(i + r, i)) * A_(i + r, j);
      va = cj(t) * va;
      A_(i + 1, j) -= va;
      for (int r = 2; r <= m; ++r) A_(i + r, j) -= va * A_(i + r, i);
    }
    // rmul!(A[:, i+1:n], H): x = A1*v + a1; a1 -= t x; A1 -= t x v^H
    for (int r = 1; r <= n; ++r) {
      S s = S(0);
      for (int c = 2; c <= m; ++c) s += A_(r, i + c) * A_(i + c, i);
      x[r - 1] = s + A_(r, i + 1);
    }
    for (int r = 1; r <= n; ++r) A_(r, i + 1) -= t * x[r - 1];
    for (int c = 2; c <= m; ++c) {
      S yc = cj(A_(i + c, i));
      for (int r = 1; r <= n; ++r) A_(r, i + c) += x[r - 1] * (-t) * yc;
    }
  }
#undef A_
}

// Form Q from the Hessenberg reflectors (hessenberg.jl:150-166, which shifts the
// reflectors one column right and forms the packed-QR Q of the trailing (n-1)x(n-1)
// block).  Restated as backward accumulation: Q = H(1) H(2) ... H(n-1),
// H(i) = I - tau_i u_i u_i^H acting on rows/cols i+1..n.
template <class S> void materialize_q(int n, const S* a, int lda, const S* tau, S* q, int ldq) {
#define A_(i, j) a[((i) - 1) + (long long)((j) - 1) * lda]
#define Q_(i, j) q[((i) - 1) + (long long)((j) - 1) * ldq]
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= n; ++i) Q_(i, j) = (i == j) ? S(1) : S(0);
  std::vector<S> u(n > 0 ? n : 1);
  for (int i = n - 1; i >= 1; --i) {
    // u over rows i+1..n: u[i+1] = 1, u[i+1+r] = A[i+1+r, i]
    const int m = n - i;
    u[0] = S(1);
    for (int r = 1; r < m; ++r) u[r] = A_(i + 1 + r, i);
    S t = tau[i - 1];
    for (int j = i + 1; j <= n; ++j) {
      S s = S(0);
      for (int r = 0; r < m; ++r) s += cj(u[r]) * Q_(i + 1 + r, j);
      s = t * s;
      for (int r = 0; r < m; ++r) Q_(i + 1 + r, j) -= s * u[r];
    }
  }
#undef A_
#undef Q_
}

// ---------------------------------------------------------------------------
// GenericSchur.jl: real Hessenberg QR (double shift)
// ---------------------------------------------------------------------------

// _gs2x2!: standardise a real 2x2 block (dlanv2), GenericSchur.jl:716-803.
// h = {a, b, c, d} = {H11, H12, H21, H22}; returns cs, sn and eigenvalues.
template <class R> void gs2x2(R* h, R* cs_out, R* sn_out, R* w1r, R* w1i, R* w2r, R* w2i) {
  R a = h[0], b = h[1], c = h[2], d = h[3];
  auto sgn = [](R x) { return (x < R(0)) ? R(-1) : R(1); };
  const R half = R(1) / R(2);
  const R small = R(4) * lim<R>::eps();
  R cs, sn;
  if (c == R(0)) {
    cs = 1; sn = 0;
  } else if (b == R(0)) {
    cs = 0; sn = 1;
    R ta = a; a = d; b = -c; c = 0; d = ta;
  } else if ((a - d) == R(0) && (b * c < R(0))) {
    cs = 1; sn = 0;
  } else {
    R asubd = a - d;
    R p = half * asubd;
    R bcmax = m_max(m_abs(b), m_abs(c));
    R bcmis = m_min(m_abs(b), m_abs(c)) * sgn(b) * sgn(c);
    R scale = m_max(m_abs(p), bcmax);
    R z = (p / scale) * p + (bcmax / scale) * bcmis;
    if (z >= small) {
      z = p + m_sqrt(scale) * m_sqrt(z) * sgn(p);
      a = d + z;
      d -= (bcmax / z) * bcmis;
      R tau = m_hypot(c, z);
      cs = z / tau;
      sn = c / tau;
      b -= c;
      c = 0;
    } else {
      R sigma = b + c;
      R tau = m_hypot(sigma, asubd);
      cs = m_sqrt(half * (R(1) + m_abs(sigma) / tau));
      sn = -(p / (tau * cs)) * sgn(sigma);
      R aa = a * cs + b * sn;
      R bb = -a * sn + b * cs;
      R cc = c * cs + d * sn;
      R dd = -c * sn + d * cs;
      a = aa * cs + cc * sn;
      b = bb * cs + dd * sn;
      c = -aa * sn + cc * cs;
      d = -bb * sn + dd * cs;
      R midad = half * (a + d);
      a = midad;
      d = a;
      if (c != R(0)) {
        if (b != R(0)) {
          if (b * c >= R(0)) {
            R sab = m_sqrt(m_abs(b));
            R sac = m_sqrt(m_abs(c));
            p = sab * sac * sgn(c);
            tau = R(1) / m_sqrt(m_abs(b + c));
            a = midad + p;
            d = midad - p;
            b -= c;
            c = 0;
            R cs1 = sab * tau;
            R sn1 = sac * tau;
            R ncs = cs * cs1 - sn * sn1;
            R nsn = cs * sn1 + sn * cs1;
            cs = ncs; sn = nsn;
          }
        } else {
          b = -c; c = 0;
          R ncs = -sn, nsn = cs;
          cs = ncs; sn = nsn;
        }
      }
    }
  }
  if (c == R(0)) {
    *w1r = a; *w1i = 0; *w2r = d; *w2i = 0;
  } else {
    R rti = m_sqrt(m_abs(b)) * m_sqrt(m_abs(c));
    *w1r = a; *w1i = rti; *w2r = d; *w2i = -rti;
  }
  h[0] = a; h[1] = b; h[2] = c; h[3] = d;
  *cs_out = cs; *sn_out = sn;
}

// doubleShiftQR!: one implicit double-shift Francis sweep (GenericSchur.jl:837-952).
template <class R>
void double_shift_qr(int n, R* h, int ldh, R* z, int ldz, int nz, R r1r, R r1i, R r2r, R r2i,
                     int istart, int iend) {
#define H_(i, j) h[((i) - 1) + (long long)((j) - 1) * ldh]
#define Z_(i, j) z[((i) - 1) + (long long)((j) - 1) * ldz]
  const int i1 = 1, i2 = n;
  const R eps = lim<R>::eps();
  R v[3] = {0, 0, 0};
  int mx = istart;
  for (int m = iend - 2; m >= istart; --m) {
    R h21s = H_(m + 1, m);
    R s = m_abs(H_(m, m) - r2r) + m_abs(r2i) + m_abs(h21s);
    h21s /= s;
    v[0] = h21s * H_(m, m + 1) + (H_(m, m) - r1r) * ((H_(m, m) - r2r) / s) - r1i * (r2i / s);
    v[1] = h21s * (H_(m, m) + H_(m + 1, m + 1) - r1r - r2r);
    v[2] = h21s * H_(m + 2, m + 1);
    s = m_abs(v[0]) + m_abs(v[1]) + m_abs(v[2]);
    v[0] /= s; v[1] /= s; v[2] /= s;
    if (m > istart &&
        m_abs(H_(m, m - 1)) * (m_abs(v[1]) + m_abs(v[2])) <=
            eps * m_abs(v[0]) * (m_abs(H_(m - 1, m - 1)) + m_abs(H_(m, m)) + m_abs(H_(m + 1, m + 1)))) {
      mx = m;
      break;
    }
  }
  for (int k = mx; k <= iend - 1; ++k) {
    int nr = std::min(3, iend - k + 1);
    if (k > mx)
      for (int ii = 0; ii < nr; ++ii) v[ii] = H_(k + ii, k - 1);
    R tau1 = reflector_real(v, nr);
    if (k > mx) {
      H_(k, k - 1) = v[0];
      H_(k + 1, k - 1) = 0;
      if (k < iend - 1) H_(k + 2, k - 1) = 0;
    } else if (mx > istart) {
      H_(k, k - 1) *= (R(1) - tau1);
    }
    R v2 = v[1];
    R tau2 = tau1 * v2;
    if (nr == 3) {
      R v3 = v[2];
      R tau3 = tau1 * v3;
      for (int j = k; j <= i2; ++j) {
        R ss = H_(k, j) + v2 * H_(k + 1, j) + v3 * H_(k + 2, j);
        H_(k, j) -= ss * tau1;
        H_(k + 1, j) -= ss * tau2;
        H_(k + 2, j) -= ss * tau3;
      }
      for (int j = i1; j <= std::min(k + 3, iend); ++j) {
        R ss = H_(j, k) + v2 * H_(j, k + 1) + v3 * H_(j, k + 2);
        H_(j, k) -= ss * tau1;
        H_(j, k + 1) -= ss * tau2;
        H_(j, k + 2) -= ss * tau3;
      }
      if (z)
        for (int j = 1; j <= nz; ++j) {
          R ss = Z_(j, k) + v2 * Z_(j, k + 1) + v3 * Z_(j, k + 2);
          Z_(j, k) -= ss * tau1;
          Z_(j, k + 1) -= ss * tau2;
          Z_(j, k + 2) -= ss * tau3;
        }
    } else if (nr == 2) {
      for (int j = k; j <= i2; ++j) {
        R ss = H_(k, j) + v2 * H_(k + 1, j);
        H_(k, j) -= ss * tau1;
        H_(k + 1, j) -= ss * tau2;
      }
      for (int j = i1; j <= iend; ++j) {
        R ss = H_(j, k) + v2 * H_(j, k + 1);
        H_(j, k) -= ss * tau1;
        H_(j, k + 1) -= ss * tau2;
      }
      if (z)
        for (int j = 1; j <= nz; ++j) {
          R ss = Z_(j, k) + v2 * Z_(j, k + 1);
          Z_(j, k) -= ss * tau1;
          Z_(j, k + 1) -= ss * tau2;
        }
    }
  }
#undef H_
#undef Z_
}

// gschur!(H::Hessenberg{<:Real}, Z): real Hessenberg QR driver (GenericSchur.jl:513-699).
// On return h holds the quasi-triangular T (entries below the first subdiagonal
// zeroed), z is updated, w = (wr, wi).  Returns ORC_OK or ORC_UNCONVERGED.
template <class R>
int gschur_hess_real(int n, R* h, int ldh, R* z, int ldz, R* wr, R* wi, long long maxiter) {
#define H_(i, j) h[((i) - 1) + (long long)((j) - 1) * ldh]
#define Z_(i, j) z[((i) - 1) + (long long)((j) - 1) * ldz]
  for (int j = 1; j <= n; ++j)
    for (int i = j + 2; i <= n; ++i) H_(i, j) = 0;  // triu!(HH, -1)
  const R eps = lim<R>::eps();
  const R smallnum = lim<R>::fmin() * (R(n) / eps);
  const R threeq = R(3) / R(4);
  const R m7_16 = R(-7) / R(16);
  int iwcur = n;
  auto putw = [&](R re, R im) { wr[iwcur - 1] = re; wi[iwcur - 1] = im; --iwcur; };
  long long iter = 0;
  int iend = n;
  int istart = 1;
  while (iend >= 1) {
    istart = 1;
    int iterqr = 0;
    bool deflate = false;
    while (true) {
      ++iter;
      if (iter > maxiter) return ORC_UNCONVERGED;
      bool split = false;
      for (int k = iend; k >= istart + 1; --k) {
        if (m_abs(H_(k, k - 1)) < smallnum) {
          split = true;
        } else {
          R hkk = H_(k, k), hkm1 = H_(k - 1, k - 1);
          R t = m_abs(hkm1) + m_abs(hkk);
          if (t == R(0)) {
            if (k > 2) t += m_abs(H_(k - 1, k - 2));
            if (k + 1 <= n) t += m_abs(H_(k + 1, k));
          }
          R ahkkm1 = m_abs(H_(k, k - 1));
          if (ahkkm1 <= t * eps) {
            R ahkm1k = m_abs(H_(k - 1, k));
            R ab = m_max(ahkkm1, ahkm1k);
            R ba = m_min(ahkkm1, ahkm1k);
            R aa = m_max(m_abs(hkk), m_abs(hkm1 - hkk));
            R bb = m_min(m_abs(hkk), m_abs(hkm1 - hkk));
            R s = aa + bb;  // as written at GenericSchur.jl:586
            if (ba * (ab / s) <= m_max(smallnum, eps * (bb * (aa / s)))) split = true;
          }
        }
        if (split) { istart = k; break; }
      }
      if (!split) istart = 1;
      if (istart > 1) H_(istart, istart - 1) = 0;
      if (istart >= iend - 1) { deflate = true; break; }
      ++iterqr;
      R h11, h12, h21, h22;
      if (iterqr == 10) {
        R s = m_abs(H_(istart + 1, istart)) + m_abs(H_(istart + 2, istart + 1));
        h11 = threeq * s + H_(istart, istart);
        h12 = m7_16 * s; h21 = s; h22 = h11;
      } else if (iterqr == 20) {
        R s = m_abs(H_(iend, iend - 1)) + m_abs(H_(iend - 1, iend - 2));
        h11 = threeq * s + H_(iend, iend);
        h12 = m7_16 * s; h21 = s; h22 = h11;
      } else {
        h11 = H_(iend - 1, iend - 1); h21 = H_(iend, iend - 1);
        h12 = H_(iend - 1, iend); h22 = H_(iend, iend);
      }
      R s = m_abs(h11) + m_abs(h12) + m_abs(h21) + m_abs(h22);
      R r1r, r2r, r1i, r2i;
      if (s == R(0)) {
        r1r = r2r = r1i = r2i = 0;
      } else {
        h11 /= s; h12 /= s; h21 /= s; h22 /= s;
        R tr = (h11 + h22) / R(2);
        R d = (h11 - tr) * (h22 - tr) - h12 * h21;
        R rtd = m_sqrt(m_abs(d));
        if (d >= R(0)) {
          r1r = tr * s; r2r = r1r; r1i = rtd * s; r2i = -r1i;
        } else {
          r1r = tr + rtd; r2r = tr - rtd;
          if (m_abs(r1r - h22) <= m_abs(r2r - h22)) { r1r *= s; r2r = r1r; }
          else { r2r *= s; r1r = r2r; }
          r1i = r2i = 0;
        }
      }
      double_shift_qr(n, h, ldh, z, ldz, z ? n : 0, r1r, r1i, r2r, r2i, istart, iend);
    }
    if (deflate && istart >= iend) {
      putw(H_(iend, iend), R(0));
    } else if (deflate && istart + 1 == iend) {
      R h2[4] = {H_(iend - 1, iend - 1), H_(iend - 1, iend), H_(iend, iend - 1), H_(iend, iend)};
      R cs, sn, w1r, w1i, w2r, w2i;
      gs2x2(h2, &cs, &sn, &w1r, &w1i, &w2r, &w2i);
      putw(w2r, w2i);
      putw(w1r, w1i);
      const int p = iend - 1, q = iend;
      for (int j = istart; j <= n; ++j) {  // lmul!(G, HH[:, istart:n])
        R a1 = H_(p, j), a2 = H_(q, j);
        H_(p, j) = cs * a1 + sn * a2;
        H_(q, j) = -sn * a1 + cs * a2;
      }
      for (int i = 1; i <= iend; ++i) {  // rmul!(HH[1:iend, :], G')
        R a1 = H_(i, p), a2 = H_(i, q);
        H_(i, p) = cs * a1 + sn * a2;
        H_(i, q) = -sn * a1 + cs * a2;
      }
      H_(p, p) = h2[0]; H_(p, q) = h2[1]; H_(q, p) = h2[2]; H_(q, q) = h2[3];
      if (iend > 2) H_(iend - 1, iend - 2) = 0;
      if (z)
        for (int i = 1; i <= n; ++i) {
          R a1 = Z_(i, p), a2 = Z_(i, q);
          Z_(i, p) = cs * a1 + sn * a2;
          Z_(i, q) = -sn * a1 + cs * a2;
        }
    }
    iend = istart - 1;
  }
  for (int j = 1; j <= n; ++j)
    for (int i = j + 2; i <= n; ++i) H_(i, j) = 0;  // triu(HH, -1)
  return ORC_OK;
#undef H_
#undef Z_
}

// ---------------------------------------------------------------------------
// GenericSchur.jl: complex Hessenberg QR (single shift)
// ---------------------------------------------------------------------------

// singleShiftQR! (GenericSchur.jl:374-504).
template <class R>
void single_shift_qr(int n, cx<R>* h, int ldh, cx<R>* z, int ldz, cx<R> shift, int istart, int iend) {
#define H_(i, j) h[((i) - 1) + (long long)((j) - 1) * ldh]
#define Z_(i, j) z[((i) - 1) + (long long)((j) - 1) * ldz]
  typedef cx<R> C;
  const R ulp = lim<R>::eps();
  int istart1 = -1;
  C v[2];
  bool flag = false;
  for (int mm = iend - 1; mm >= istart + 1; --mm) {
    C h11 = H_(mm, mm), h22 = H_(mm + 1, mm + 1);
    C h11s = h11 - shift;
    R h21 = H_(mm + 1, mm).re;
    R s = abs1(h11s) + m_abs(h21);
    h11s = h11s / s;
    h21 /= s;
    v[0] = h11s; v[1] = C(h21);
    R h10 = H_(mm, mm - 1).re;
    if (m_abs(h10) * m_abs(h21) <= ulp * (abs1(h11s) * (abs1(h11) + abs1(h22)))) {
      istart1 = mm; flag = true; break;
    }
  }
  if (!flag) {
    istart1 = istart;
    C h11 = H_(istart, istart);
    C h11s = h11 - shift;
    R h21 = H_(istart + 1, istart).re;
    R s = abs1(h11s) + m_abs(h21);
    h11s = h11s / s;
    h21 /= s;
    v[0] = h11s; v[1] = C(h21);
  }
  for (int k = istart1; k <= iend - 1; ++k) {
    if (k > istart1) { v[0] = H_(k, k - 1); v[1] = H_(k + 1, k - 1); }
    C tau1 = reflector_cplx(v, 2);
    if (k > istart1) { H_(k, k - 1) = v[0]; H_(k + 1, k - 1) = C(0); }
    C v2 = v[1];
    R tau2 = (tau1 * v2).re;
    for (int j = k; j <= n; ++j) {
      C ss = conj(tau1) * H_(k, j) + H_(k + 1, j) * tau2;
      H_(k, j) -= ss;
      H_(k + 1, j) -= ss * v2;
    }
    for (int j = 1; j <= std::min(k + 2, iend); ++j) {
      C ss = tau1 * H_(j, k) + H_(j, k + 1) * tau2;
      H_(j, k) -= ss;
      H_(j, k + 1) -= ss * conj(v2);
    }
    if (z)
      for (int j = 1; j <= n; ++j) {
        C ss = tau1 * Z_(j, k) + Z_(j, k + 1) * tau2;
        Z_(j, k) -= ss;
        Z_(j, k + 1) -= ss * conj(v2);
      }
    if (k == istart1 && istart1 > istart) {
      C t = C(1) - tau1;
      t = t / cabs(t);
      H_(istart1 + 1, istart1) *= conj(t);
      if (istart1 + 2 <= iend) H_(istart1 + 2, istart1 + 1) *= t;
      for (int j = istart1; j <= iend; ++j) {
        if (j != istart1 + 1) {
          for (int c = j + 1; c <= n; ++c) H_(j, c) *= t;
          for (int r = 1; r <= j - 1; ++r) H_(r, j) *= conj(t);
          if (z)
            for (int r = 1; r <= n; ++r) Z_(r, j) *= conj(t);
        }
      }
    }
  }
  C t = H_(iend, iend - 1);
  if (t.im != R(0)) {
    R rt = cabs(t);
    H_(iend, iend - 1) = C(rt);
    t = t / rt;
    for (int c = iend + 1; c <= n; ++c) H_(iend, c) *= conj(t);
    for (int r = 1; r <= iend - 1; ++r) H_(r, iend) *= t;
    if (z)
      for (int r = 1; r <= n; ++r) Z_(r, iend) *= t;
  }
#undef H_
#undef Z_
}

// gschur!(H::Hessenberg{Complex}, Z) (GenericSchur.jl:194-335).
template <class R>
int gschur_hess_cplx(int n, cx<R>* h, int ldh, cx<R>* z, int ldz, cx<R>* w, long long maxiter,
                     long long maxinner, bool checksd) {
#define H_(i, j) h[((i) - 1) + (long long)((j) - 1) * ldh]
  typedef cx<R> C;
  if (checksd)
    for (int j = 1; j <= n - 1; ++j)
      if (H_(j + 1, j).im != R(0)) return ORC_BADARG;
  const R ulp = lim<R>::eps();
  const R smallnum = safemin<R>() * (R(n) / ulp);
  const R half = R(1) / R(2);
  const R threeq = R(3) / R(4);
  for (int j = 1; j <= n - 1; ++j)
    for (int i = j + 2; i <= n; ++i) H_(i, j) = C(0);
  long long it = 0;
  int iend = n;
  while (iend >= 1) {
    int istart = 1;
    bool deflated = false;
    for (long long its = 0; its <= maxinner; ++its) {
      ++it;
      if (it > maxiter) return ORC_UNCONVERGED;
      for (int k = iend - 1; k >= istart; --k) {
        if (abs1(H_(k + 1, k)) <= smallnum) { istart = k + 1; break; }
        R tst = abs1(H_(k, k)) + abs1(H_(k + 1, k + 1));
        if (tst == R(0)) {
          if (k - 1 >= 1) tst += m_abs(H_(k, k - 1).re);
          if (k + 2 <= n) tst += m_abs(H_(k + 2, k + 1).re);
        }
        if (m_abs(H_(k + 1, k).re) <= ulp * tst) {
          R ab = m_max(abs1(H_(k + 1, k)), abs1(H_(k, k + 1)));
          R ba = m_min(abs1(H_(k + 1, k)), abs1(H_(k, k + 1)));
          R aa = m_max(abs1(H_(k + 1, k + 1)), abs1(H_(k, k) - H_(k + 1, k + 1)));
          R bb = m_min(abs1(H_(k + 1, k + 1)), abs1(H_(k, k) - H_(k + 1, k + 1)));
          R s = aa + ab;
          if (ba * (ab / s) <= m_max(smallnum, ulp * (bb * (aa / s)))) { istart = k + 1; break; }
        }
      }
      if (istart > 1) H_(istart, istart - 1) = C(0);
      if (istart >= iend) { iend -= 1; deflated = true; break; }
      C t;
      if (its % 30 == 10) {
        R s = threeq * m_abs(H_(istart + 1, istart).re);
        t = C(s) + H_(istart, istart);
      } else if (its % 30 == 20) {
        R s = threeq * m_abs(H_(iend, iend - 1).re);
        t = C(s) + H_(iend, iend);
      } else {
        t = H_(iend, iend);
        C u = csqrt(H_(iend - 1, iend)) * csqrt(H_(iend, iend - 1));
        R s = abs1(u);
        if (s != R(0)) {
          C x = (H_(iend - 1, iend - 1) - t) * half;
          R sx = abs1(x);
          s = m_max(s, abs1(x));
          C xs = x / s, us = u / s;
          C y = csqrt(xs * xs + us * us) * s;
          if (sx > R(0)) {
            C xn = x / sx;
            if (xn.re * y.re + xn.im * y.im < R(0)) y = -y;
          }
          t -= u * (u / (x + y));
        }
      }
      single_shift_qr(n, h, ldh, z, ldz, t, istart, iend);
    }
    if (!deflated) {
      // maxinner exhausted without deflation: the reference's for-loop ends and the
      // outer loop re-enters with the same iend; maxiter eventually stops it.
    }
  }
  for (int j = 1; j <= n; ++j) w[j - 1] = H_(j, j);
  for (int j = 1; j <= n; ++j)
    for (int i = j + 1; i <= n; ++i) H_(i, j) = C(0);  // triu(HH)
  return ORC_OK;
#undef H_
}

// ---------------------------------------------------------------------------
// Drivers gschur!(A) (GenericSchur.jl:805-835 real, 350-372 complex)
// ---------------------------------------------------------------------------

template <class R>
int gschur_real(int n, R* a, int lda, R* z, int ldz, R* wr, R* wi, bool wantZ, bool scale,
                long long maxiter) {
  R cscale = 1, anrm = 1;
  bool scaleA = false;
  if (scale) scaleA = scale_matrix<R, R>(n, a, lda, &cscale, &anrm);
  std::vector<R> tau(n > 1 ? n - 1 : 1);
  hessenberg<R>(n, a, lda, tau.data());
  if (wantZ) materialize_q<R>(n, a, lda, tau.data(), z, ldz);
  int st = gschur_hess_real<R>(n, a, lda, wantZ ? z : nullptr, ldz, wr, wi, maxiter);
  if (st != ORC_OK) return st;
  if (scaleA) {
    for (int j = 0; j < n; ++j) safescale<R, R>(a + (long long)j * lda, n, cscale, anrm);
    safescale<R, R>(wr, n, cscale, anrm);
    safescale<R, R>(wi, n, cscale, anrm);
  }
  return ORC_OK;
}

template <class R>
int gschur_cplx(int n, cx<R>* a, int lda, cx<R>* z, int ldz, cx<R>* w, bool wantZ, bool scale,
                long long maxiter, long long maxinner) {
  R cscale = 1, anrm = 1;
  bool scaleA = false;
  if (scale) scaleA = scale_matrix<R, cx<R>>(n, a, lda, &cscale, &anrm);
  std::vector<cx<R>> tau(n > 1 ? n - 1 : 1);
  hessenberg<cx<R>>(n, a, lda, tau.data());
  if (wantZ) materialize_q<cx<R>>(n, a, lda, tau.data(), z, ldz);
  int st = gschur_hess_cplx<R>(n, a, lda, wantZ ? z : nullptr, ldz, w, maxiter, maxinner, false);
  if (st != ORC_OK) return st;
  if (scaleA) {
    for (int j = 0; j < n; ++j) safescale<R, cx<R>>(a + (long long)j * lda, n, cscale, anrm);
    for (int j = 0; j < n; ++j) w[j] = a[j + (long long)j * lda];
  }
  return ORC_OK;
}

}  // namespace orc
