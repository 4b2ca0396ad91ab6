// CPU restatement of GenericSchur.jl's divide-and-conquer eigensolver for real symmetric
// tridiagonal matrices -- TEST INFRASTRUCTURE ONLY (the checker of the GPU path):
//   _gschur!(A::SymTridiagonal, ::DivideAndConquer, Z)   src/symtri_dc.jl:6-104
//   _dcschur_core!    107-196      _dcmerge!   200-217     _dcdeflate!  221-425
//   _dcsecular!       431-489      _dcroot!    777-927     _dcroot2!    929-972
//   _dcnewton         976-1163     _initialize_n / _update_w_n / _next_step_n  492-620
//   _initialize / _update_w / _next_step                                       622-775
// Kept as the reference has them: _dcnewton's first quadratic step without the division
// by 2c (symtri_dc.jl:1011), its first function evaluation at dscale[1] for all three poles
// (1061-1069) and sclinv = small2 in both scaling branches (1047-1053).  The leaves and
// the small blocks use the QR iteration of hermitian_oracle.hpp (maxiter = 30 m).
// The reference's norm(s0) and mul! run through BLAS; here they are plain loops.
#pragma once
#include <algorithm>
#include <numeric>
#include <vector>
#include "hermitian_oracle.hpp"

namespace orc {

struct DcParts {
  double psi, phi, dpsi, dphi, dw;
};

inline double dc_sq(double x) { return x * x; }

// _dcroot2! (929-972); i 1-based; d, z, delta length 2
inline double dcroot2(int i, const double* d, const double* z, double* delta, double rho) {
  const double D = d[1] - d[0];
  double lam, tau;
  if (i == 1) {
    const double w = 1.0 + 2.0 * rho * (dc_sq(z[1]) - dc_sq(z[0])) / D;
    if (w > 0) {
      const double b = D + rho * (dc_sq(z[0]) + dc_sq(z[1]));
      const double c = rho * dc_sq(z[0]) * D;
      tau = 2.0 * c / (b + std::sqrt(b * b - 4.0 * c));
      lam = d[0] + tau;
      delta[0] = -z[0] / tau;
      delta[1] = z[1] / (D - tau);
    } else {
      const double b = -D + rho * (dc_sq(z[0]) + dc_sq(z[1]));
      const double c = rho * dc_sq(z[1]) * D;
      if (b > 0) tau = -2.0 * c / (b + std::sqrt(b * b + 4.0 * c));
      else tau = (b - std::sqrt(b * b + 4.0 * c)) / 2.0;
      lam = d[1] + tau;
      delta[0] = -z[0] / (D + tau);
      delta[1] = -z[1] / tau;
    }
  } else {
    const double b = -D + rho * (dc_sq(z[0]) + dc_sq(z[1]));
    const double c = rho * dc_sq(z[1]) * D;
    if (b > 0) tau = (b + std::sqrt(b * b + 4.0 * c)) / 2.0;
    else tau = 2.0 * c / (-b + std::sqrt(b * b + 4.0 * c));
    lam = d[1] + tau;
    delta[0] = -z[0] / (D + tau);
    delta[1] = -z[1] / tau;
  }
  const double t = std::sqrt(dc_sq(delta[0]) + dc_sq(delta[1]));
  delta[0] = delta[0] / t;
  delta[1] = delta[1] / t;
  return lam;
}

// _dcnewton (976-1163): d, z the three poles and numerators; returns tau
inline double dcnewton(int kniter, bool orig, double rho, const double* d, const double* z, double finit, bool* conv) {
  const int maxit = 40;
  const double eps = lim<double>::eps();
  double lbd, ubd;
  if (orig) { lbd = d[1]; ubd = d[2]; } else { lbd = d[0]; ubd = d[1]; }
  if (finit < 0) lbd = 0.0;
  else ubd = 0.0;
  int niter = 1;
  double tau = 0.0;
  if (kniter == 2) {
    double t, c, a, b;
    if (orig) {
      t = (d[2] - d[1]) / 2.0;
      c = rho + z[0] / ((d[0] - d[1]) - t);
      a = c * (d[1] + d[2]) + z[1] + z[2];
      b = c * d[1] * d[2] + z[1] * d[2] + z[2] * d[1];
    } else {
      t = (d[0] - d[1]) / 2.0;
      c = rho + z[2] / ((d[2] - d[1]) - t);
      a = c * (d[0] + d[1]) + z[0] + z[1];
      b = c * d[0] * d[1] + z[0] * d[1] + z[1] * d[0];
    }
    t = std::max(std::max(std::fabs(a), std::fabs(b)), std::fabs(c));
    a /= t;
    b /= t;
    c /= t;
    if (c == 0) tau = b / a;
    else if (a < 0) tau = a - std::sqrt(std::fabs(a * a - 4.0 * b * c));
    else tau = 2.0 * b / (a + std::sqrt(std::fabs(a * a - 4.0 * b * c)));
    if (tau < lbd || tau > ubd) tau = (lbd + ubd) / 2.0;
    if (d[0] == tau || d[1] == tau || d[2] == tau) {
      tau = 0.0;
    } else {
      t = finit + tau * z[0] / (d[0] * (d[0] - tau)) + tau * z[1] / (d[1] * (d[1] - tau)) +
          tau * z[2] / (d[2] * (d[2] - tau));
      if (t <= 0) lbd = tau;
      else ubd = tau;
      if (std::fabs(finit) <= std::fabs(t)) tau = 0.0;
    }
  }
  const double small1 = std::ldexp(1.0, -341), sminv1 = 1.0 / small1;
  const double small2 = small1 * small1, sminv2 = sminv1 * sminv1;
  double t = orig ? std::min(std::fabs(d[1] - tau), std::fabs(d[2] - tau))
                  : std::min(std::fabs(d[0] - tau), std::fabs(d[1] - tau));
  const bool scale = t <= small1;
  double ds[3], zs[3], sclinv = 1.0;
  if (scale) {
    double sclfac;
    if (t <= small2) { sclfac = sminv2; sclinv = small2; }
    else { sclfac = sminv1; sclinv = small2; }
    for (int q = 0; q < 3; ++q) { ds[q] = d[q] * sclfac; zs[q] = z[q] * sclfac; }
    tau *= sclfac;
    lbd *= sclfac;
    ubd *= sclfac;
  } else {
    for (int q = 0; q < 3; ++q) { ds[q] = d[q]; zs[q] = z[q]; }
  }
  double fc = 0.0, df = 0.0, ddf = 0.0;
  for (int q = 0; q < 3; ++q) {
    const double tt = 1.0 / (ds[0] - tau);
    const double t1 = zs[q] * tt, t2 = t1 * tt, t3 = t2 * tt;
    fc += t1 / ds[q];
    df += t2;
    ddf += t3;
  }
  double f = finit + tau * fc;
  if (std::fabs(f) <= 0) {
    if (scale) tau *= sclinv;
    *conv = true;
    return tau;
  }
  if (f <= 0) lbd = tau;
  else ubd = tau;
  bool converged = false;
  for (int it = niter + 1; it <= maxit; ++it) {
    double t1, t2;
    if (orig) { t1 = ds[1] - tau; t2 = ds[2] - tau; }
    else { t1 = ds[0] - tau; t2 = ds[1] - tau; }
    double a = (t1 + t2) * f - t1 * t2 * df;
    double b = t1 * t2 * f;
    double c = f - (t1 + t2) * df + t1 * t2 * ddf;
    const double tm = std::max(std::max(std::fabs(a), std::fabs(b)), std::fabs(c));
    a /= tm;
    b /= tm;
    c /= tm;
    double eta;
    if (c == 0) eta = b / a;
    else if (a <= 0) eta = (a - std::sqrt(std::fabs(a * a - 4.0 * b * c))) / (2.0 * c);
    else eta = 2.0 * b / (a + std::sqrt(std::fabs(a * a - 4.0 * b * c)));
    if (f * eta >= 0) eta = -f / df;
    tau += eta;
    if (tau < lbd || tau > ubd) tau = (lbd + ubd) / 2.0;
    fc = 0.0;
    double erretm = 0.0;
    df = 0.0;
    ddf = 0.0;
    for (int q = 0; q < 3; ++q) {
      if ((ds[q] - tau) != 0) {
        const double tt = 1.0 / (ds[q] - tau);
        const double u1 = zs[q] * tt, u2 = u1 * tt, u3 = u2 * tt, u4 = u1 / ds[q];
        fc += u4;
        erretm += std::fabs(u4);
        df += u2;
        ddf += u3;
      } else {
        converged = true;
        break;
      }
    }
    if (converged) break;
    f = finit + tau * fc;
    erretm = 8.0 * (std::fabs(finit) + std::fabs(tau) * erretm) + std::fabs(tau) * df;
    if ((std::fabs(f) <= 4.0 * eps * erretm) || ((ubd - lbd) <= 4.0 * eps * std::fabs(tau))) {
      converged = true;
      break;
    }
    if (f <= 0) lbd = tau;
    else ubd = tau;
  }
  if (scale) tau *= sclinv;
  *conv = converged;
  return tau;
}

// _dcroot! (777-927): root i (1-based) of the secular equation of (d, z, rho), n = len;
// delta (n) receives d - lambda; returns lambda, *conv the convergence flag.
inline double dcroot(int n, int i, const double* dd, const double* zz, double* dl, double rho, bool* conv) {
  const int maxit = 30;
  // 1-based views
  const double* d = dd - 1;
  const double* z = zz - 1;
  double* delta = dl - 1;
  *conv = true;
  if (n == 1) {
    delta[1] = 1.0;
    return d[1] + rho * dc_sq(z[1]);
  }
  if (n == 2) return dcroot2(i, dd, zz, dl, rho);
  const double eps = lim<double>::eps();
  const double rhoinv = 1.0 / rho;
  double dltlb, dltub, w, tau, erretm;
  if (i == n) {
    const int ii = n - 1;
    const double midpt = rho / 2.0;
    for (int j = 1; j <= n; ++j) delta[j] = (d[j] - d[i]) - midpt;
    // _initialize_n
    {
      double psi = 0.0;
      for (int j = 1; j <= n - 2; ++j) psi += dc_sq(z[j]) / delta[j];
      const double c = rhoinv + psi;
      w = c + dc_sq(z[ii]) / delta[ii] + dc_sq(z[n]) / delta[n];
      const double D = d[n] - d[n - 1];
      const double a = -c * D + dc_sq(z[n - 1]) + dc_sq(z[n]);
      const double b = dc_sq(z[n]) * D;
      auto quad = [&]() {
        return a < 0 ? 2.0 * b / (std::sqrt(a * a + 4.0 * b * c) - a) : (a + std::sqrt(a * a + 4.0 * b * c)) / (2.0 * c);
      };
      if (w <= 0) {
        const double t = dc_sq(z[n - 1]) / (d[n] - d[n - 1] + rho) + dc_sq(z[n]) / rho;
        tau = (c <= t) ? rho : quad();
        dltlb = midpt;
        dltub = rho;
      } else {
        tau = quad();
        dltlb = 0.0;
        dltub = midpt;
      }
    }
    for (int j = 1; j <= n; ++j) delta[j] = (d[j] - d[i]) - tau;
    double dpsi, dphi;
    auto update_n = [&]() {
      dpsi = 0.0;
      double psi = 0.0;
      erretm = 0.0;
      for (int j = 1; j <= ii; ++j) {
        const double t = z[j] / delta[j];
        psi += z[j] * t;
        dpsi += t * t;
        erretm += psi;
      }
      erretm = std::fabs(erretm);
      const double t = z[n] / delta[n];
      const double phi = z[n] * t;
      dphi = t * t;
      erretm = 8.0 * (-phi - psi) + erretm - phi + rhoinv + std::fabs(tau) * (dpsi + dphi);
      w = rhoinv + phi + psi;
    };
    auto step_n = [&](int iter) {
      double c = w - delta[n - 1] * dpsi - delta[n] * dphi;
      if (iter <= 2) c = std::fabs(c);
      const double a = (delta[n - 1] + delta[n]) * w - delta[n - 1] * delta[n] * (dpsi + dphi);
      const double b = delta[n - 1] * delta[n] * w;
      double eta;
      if (c == 0) eta = dltub - tau;
      else if (a >= 0) eta = (a + std::sqrt(std::fabs(a * a - 4.0 * b * c))) / (2.0 * c);
      else eta = 2.0 * b / (a - std::sqrt(std::fabs(a * a - 4.0 * b * c)));
      if (w * eta > 0) eta = -w / (dpsi + dphi);
      const double t = tau + eta;
      if (t > dltub || t < dltlb) eta = w < 0 ? (dltub - tau) / 2.0 : (dltlb - tau) / 2.0;
      return eta;
    };
    update_n();
    if (std::fabs(w) < eps * erretm) return d[i] + tau;
    if (w <= 0) dltlb = std::max(dltlb, tau);
    else dltub = std::min(dltub, tau);
    int niter = 2;
    double eta = step_n(niter);
    for (int j = 1; j <= n; ++j) delta[j] = delta[j] - eta;
    tau += eta;
    update_n();
    for (niter = 3; niter <= maxit; ++niter) {
      if (std::fabs(w) < eps * erretm) return d[i] + tau;
      if (w <= 0) dltlb = std::max(dltlb, tau);
      else dltub = std::min(dltub, tau);
      eta = step_n(niter);
      for (int j = 1; j <= n; ++j) delta[j] = delta[j] - eta;
      tau += eta;
      update_n();
    }
    *conv = false;
    return d[i] + tau;
  }
  // i < n
  const int ip1 = i + 1;
  const double D = d[ip1] - d[i];
  const double midpt = D / 2.0;
  for (int j = 1; j <= n; ++j) delta[j] = (d[j] - d[i]) - midpt;
  bool orig;
  {
    double psi = 0.0;
    for (int j = 1; j <= i - 1; ++j) psi = psi + dc_sq(z[j]) / delta[j];
    double phi = 0.0;
    for (int j = n; j >= i + 2; --j) phi = phi + dc_sq(z[j]) / delta[j];
    const double c = rhoinv + psi + phi;
    w = c + dc_sq(z[i]) / delta[i] + dc_sq(z[ip1]) / delta[ip1];
    orig = w > 0;
    if (orig) {
      const double a = c * D + dc_sq(z[i]) + dc_sq(z[ip1]);
      const double b = dc_sq(z[i]) * D;
      if (a > 0) tau = 2.0 * b / (a + std::sqrt(std::fabs(a * a - 4.0 * b * c)));
      else tau = (a - std::sqrt(std::fabs(a * a - 4.0 * b * c))) / (2.0 * c);
      dltlb = 0.0;
      dltub = midpt;
    } else {
      const double a = c * D - dc_sq(z[i]) - dc_sq(z[ip1]);
      const double b = dc_sq(z[ip1]) * D;
      if (a < 0) tau = 2.0 * b / (a - std::sqrt(std::fabs(a * a + 4.0 * b * c)));
      else tau = -(a + std::sqrt(std::fabs(a * a + 4.0 * b * c))) / (2.0 * c);
      dltlb = -midpt;
      dltub = 0.0;
    }
  }
  const int ii = orig ? i : i + 1;
  const double dorg = d[ii];
  for (int j = 1; j <= n; ++j) delta[j] = (d[j] - dorg) - tau;
  DcParts P;
  double w0;
  auto update = [&](double etaq) {
    double dpsi = 0.0, psi = 0.0;
    erretm = 0.0;
    for (int j = 1; j <= ii - 1; ++j) {
      const double t = z[j] / delta[j];
      psi += z[j] * t;
      dpsi += t * t;
      erretm += psi;
    }
    erretm = std::fabs(erretm);
    double phi = 0.0, dphi = 0.0;
    for (int j = n; j >= ii + 1; --j) {
      const double t = z[j] / delta[j];
      phi += z[j] * t;
      dphi += t * t;
      erretm += phi;
    }
    w0 = rhoinv + phi + psi;
    double t = z[ii] / delta[ii];
    const double dw = dpsi + dphi + t * t;
    t = z[ii] * t;
    w = rhoinv + phi + psi + t;
    erretm = 8.0 * (phi - psi) + erretm + 2.0 * rhoinv + 3.0 * std::fabs(t) + std::fabs(tau + etaq) * dw;
    P = DcParts{psi, phi, dpsi, dphi, dw};
  };
  auto step = [&](int niter, bool switch3, bool sw) {
    double dpsi = P.dpsi, dphi = P.dphi;
    const double psi = P.psi, phi = P.phi, dw = P.dw;
    const int iip1 = ii + 1, iim1 = ii - 1;
    double eta;
    if (!switch3) {
      double c;
      if (!sw) {
        if (orig) c = w - delta[ip1] * dw - (d[i] - d[ip1]) * dc_sq(z[i] / delta[i]);
        else c = w - delta[i] * dw - (d[ip1] - d[i]) * dc_sq(z[ip1] / delta[ip1]);
      } else {
        const double t = z[ii] / delta[ii];
        if (orig) dpsi += t * t;
        else dphi += t * t;
        c = w - delta[i] * dpsi - delta[ip1] * dphi;
      }
      double a = (delta[i] + delta[ip1]) * w - delta[i] * delta[ip1] * dw;
      const double b = delta[i] * delta[ip1] * w;
      if (c == 0) {
        if (a == 0) {
          if (orig) a = dc_sq(z[i]) + dc_sq(delta[ip1]) * (dpsi + dphi);
          else a = dc_sq(z[ip1]) + dc_sq(delta[i]) * (dpsi + dphi);
        }
        eta = b / a;
      } else if (a <= 0) {
        eta = (a - std::sqrt(std::fabs(a * a - 4.0 * b * c))) / (2.0 * c);
      } else {
        eta = 2.0 * b / (a + std::sqrt(std::fabs(a * a - 4.0 * b * c)));
      }
    } else {
      const double t = rhoinv + psi + phi;
      double c, zz3[3];
      if (orig) {
        const double t1 = dc_sq(z[iim1] / delta[iim1]);
        c = t - delta[iip1] * (dpsi + dphi) - (d[iim1] - d[iip1]) * t1;
        zz3[0] = dc_sq(z[iim1]);
        zz3[2] = dc_sq(delta[iip1]) * ((dpsi - t1) + dphi);
      } else {
        const double t1 = dc_sq(z[iip1] / delta[iip1]);
        c = t - delta[iim1] * (dpsi + dphi) - (d[iip1] - d[iim1]) * t1;
        zz3[0] = dc_sq(delta[iim1]) * (dpsi + (dphi - t1));
        zz3[2] = dc_sq(z[iip1]);
      }
      zz3[1] = dc_sq(z[ii]);
      bool cv;
      eta = dcnewton(niter, orig, c, &delta[iim1], zz3, w, &cv);
    }
    if (w * eta > 0) eta = -w / dw;
    const double t = tau + eta;
    if (t > dltub || t < dltlb) eta = w < 0 ? (dltub - tau) / 2.0 : (dltlb - tau) / 2.0;
    return eta;
  };
  update(0.0);
  bool switch3 = orig ? (w0 < 0) : (w0 > 0);
  if (ii == 1 || ii == n) switch3 = false;
  if (std::fabs(w) < eps * erretm) return dorg + tau;
  if (w <= 0) dltlb = std::max(dltlb, tau);
  else dltub = std::min(dltub, tau);
  int niter = 2;
  double eta = step(niter, switch3, false);
  double prev_w = w;
  for (int j = 1; j <= n; ++j) delta[j] = delta[j] - eta;
  update(eta);
  bool sw = false;
  if (orig) { if (-w > std::fabs(prev_w) / 10.0) sw = true; }
  else if (w > std::fabs(prev_w) / 10.0) sw = true;
  tau += eta;
  for (niter = 3; niter <= maxit; ++niter) {
    if (std::fabs(w) < eps * erretm) return dorg + tau;
    if (w <= 0) dltlb = std::max(dltlb, tau);
    else dltub = std::min(dltub, tau);
    eta = step(niter, switch3, sw);
    for (int j = 1; j <= n; ++j) delta[j] = delta[j] - eta;
    tau += eta;
    prev_w = w;
    update(0.0);
    if ((w * prev_w > 0) && (std::fabs(w) > std::fabs(prev_w) / 10.0)) sw = !sw;
  }
  *conv = false;
  return dorg + tau;
}

// stable sortperm (0-based positions)
inline std::vector<int> dc_sortperm(const double* v, int n) {
  std::vector<int> p(n);
  std::iota(p.begin(), p.end(), 0);
  std::stable_sort(p.begin(), p.end(), [&](int a, int b) { return v[a] < v[b]; });
  return p;
}

// _dcmerge! with _dcdeflate! and _dcsecular! (200-489) on the block d (n), Q (n x n, ld
// ldq), indexq (1-based local indices); returns false when a root did not converge.
inline bool dc_merge(int n, double* d, double* Q, int ldq, int* indexq, double rho, int n1) {
#define QM(i, j) Q[((i) - 1) + (size_t)((j) - 1) * ldq]
  const int n2 = n - n1, n1p1 = n1 + 1;
  std::vector<double> z(n + 1);
  for (int j = 1; j <= n1; ++j) z[j] = QM(n1, j);
  for (int j = n1p1; j <= n; ++j) z[j] = QM(n1p1, j);
  // _dcdeflate!
  const double t0 = 1.0 / std::sqrt(2.0);
  for (int j = 1; j <= n; ++j) z[j] = z[j] * t0;
  if (rho < 0)
    for (int j = n1p1; j <= n; ++j) z[j] = z[j] * -1.0;
  rho = std::fabs(2.0 * rho);
  for (int j = n1p1; j <= n; ++j) indexq[j - 1] += n1;
  std::vector<double> w(n + 1, 0.0), lam(n + 1);
  for (int j = 1; j <= n; ++j) lam[j] = d[indexq[j - 1] - 1];
  std::vector<int> indexc(n + 1), index(n + 1), indexp(n + 1, 0);
  {
    const std::vector<int> p = dc_sortperm(&lam[1], n);
    for (int j = 1; j <= n; ++j) indexc[j] = p[j - 1] + 1;
  }
  for (int j = 1; j <= n; ++j) index[j] = indexq[indexc[j] - 1];
  double zmax = 0.0, dmax = 0.0;
  for (int j = 1; j <= n; ++j) { zmax = std::max(zmax, std::fabs(z[j])); dmax = std::max(dmax, std::fabs(d[j - 1])); }
  const double tol = 8.0 * lim<double>::eps() * std::max(zmax, dmax);
  if (rho * zmax <= tol) {
    std::vector<double> Qt((size_t)n * n);
    for (int j = 1; j <= n; ++j) {
      const int i = index[j];
      for (int r = 1; r <= n; ++r) Qt[(r - 1) + (size_t)(j - 1) * n] = QM(r, i);
      lam[j] = d[i - 1];
    }
    for (int j = 1; j <= n; ++j)
      for (int r = 1; r <= n; ++r) QM(r, j) = Qt[(r - 1) + (size_t)(j - 1) * n];
    for (int j = 1; j <= n; ++j) d[j - 1] = lam[j];
    for (int j = 1; j <= n; ++j) indexq[j - 1] = j;
    return true;
  }
  std::vector<int> coltype(n + 1, 1);
  for (int j = n1p1; j <= n; ++j) coltype[j] = 3;
  int k = 0, k2 = n + 1, nclose = 0, jj = 0, pj = 0;
  bool bdone = false;
  for (int j = 1; j <= n; ++j) {
    jj = j;
    const int nj = index[j];
    if (rho * std::fabs(z[nj]) <= tol) {
      k2 -= 1;
      coltype[nj] = 4;
      indexp[k2] = nj;
      if (j == n) { bdone = true; break; }
    } else {
      pj = nj;
      break;
    }
  }
  if (!bdone) {
    while (jj < n) {
      jj += 1;
      const int nj = index[jj];
      if (rho * std::fabs(z[nj]) <= tol) {
        k2 -= 1;
        coltype[nj] = 4;
        indexp[k2] = nj;
      } else {
        double s = z[pj], c = z[nj];
        const double tau = m_hypot(c, s);
        double t = d[nj - 1] - d[pj - 1];
        c /= tau;
        s = -s / tau;
        if (std::fabs(t * c * s) <= tol) {
          nclose += 1;
          z[nj] = tau;
          z[pj] = 0.0;
          if (coltype[nj] != coltype[pj]) coltype[nj] = 2;
          coltype[pj] = 4;
          // rmul!(Q, Givens(pj, nj, c, s)')
          for (int r = 1; r <= n; ++r) {
            const double a1 = QM(r, pj), a2 = QM(r, nj);
            QM(r, pj) = a1 * c + a2 * s;
            QM(r, nj) = -a1 * s + a2 * c;
          }
          t = d[pj - 1] * (c * c) + d[nj - 1] * (s * s);
          d[nj - 1] = d[pj - 1] * (s * s) + d[nj - 1] * (c * c);
          d[pj - 1] = t;
          k2 -= 1;
          int i = 1;
          if (k2 + i > n) {
            indexp[k2 + i - 1] = pj;
          } else {
            while (k2 + i <= n) {
              if (d[pj - 1] < d[indexp[k2 + i] - 1]) {
                indexp[k2 + i - 1] = indexp[k2 + i];
                indexp[k2 + i] = pj;
                i += 1;
              } else {
                indexp[k2 + i - 1] = pj;
                break;
              }
            }
          }
          pj = nj;
        } else {
          k += 1;
          lam[k] = d[pj - 1];
          w[k] = z[pj];
          indexp[k] = pj;
          pj = nj;
        }
      }
    }
  }
  k += 1;
  lam[k] = d[pj - 1];
  w[k] = z[pj];
  indexp[k] = pj;
  int cc[5] = {0, 0, 0, 0, 0};
  for (int j = 1; j <= n; ++j) cc[coltype[j]] += 1;
  int psm[5] = {0, 1, 1 + cc[1], 1 + cc[1] + cc[2], 1 + cc[1] + cc[2] + cc[3]};
  k = n - cc[4];
  for (int j = 1; j <= n; ++j) {
    const int js = indexp[j], ct = coltype[js];
    index[psm[ct]] = js;
    indexc[psm[ct]] = j;
    psm[ct] += 1;
  }
  // Q2 blocks
  const int c1 = cc[1], c2 = cc[2], c3 = cc[3], c4 = cc[4];
  std::vector<double> Q12((size_t)n1 * (c1 + c2)), Q34((size_t)n2 * (c2 + c3)), Q5((size_t)n * c4);
  int i = 1;
  for (int j = 1; j <= c1; ++j, ++i) {
    const int js = index[i];
    for (int r = 1; r <= n1; ++r) Q12[(r - 1) + (size_t)(j - 1) * n1] = QM(r, js);
    z[i] = d[js - 1];
  }
  for (int j = 1; j <= c2; ++j, ++i) {
    const int js = index[i];
    for (int r = 1; r <= n1; ++r) Q12[(r - 1) + (size_t)(c1 + j - 1) * n1] = QM(r, js);
    for (int r = 1; r <= n2; ++r) Q34[(r - 1) + (size_t)(j - 1) * n2] = QM(n1 + r, js);
    z[i] = d[js - 1];
  }
  for (int j = 1; j <= c3; ++j, ++i) {
    const int js = index[i];
    for (int r = 1; r <= n2; ++r) Q34[(r - 1) + (size_t)(c2 + j - 1) * n2] = QM(n1 + r, js);
    z[i] = d[js - 1];
  }
  for (int j = 1; j <= c4; ++j, ++i) {
    const int js = index[i];
    for (int r = 1; r <= n; ++r) Q5[(r - 1) + (size_t)(j - 1) * n] = QM(r, js);
    z[i] = d[js - 1];
  }
  if (k < n)
    for (int j = 1; j <= c4; ++j) {
      for (int r = 1; r <= n; ++r) QM(r, k + j) = Q5[(r - 1) + (size_t)(j - 1) * n];
      d[k + j - 1] = z[k + j];
    }
  if (k == 0) {
    for (int j = 1; j <= n; ++j) indexq[j - 1] = j;
    return true;
  }
  // _dcsecular!
  for (int j = 1; j <= k; ++j) {
    bool conv;
    d[j - 1] = dcroot(k, j, &lam[1], &w[1], &QM(1, j), rho, &conv);
    if (!conv) return false;
  }
  std::vector<double> S((size_t)k * k);  // the rank-one eigenvectors, rows in type order
  if (k == 1) {
    S[0] = QM(1, 1);
  } else if (k == 2) {
    for (int j = 1; j <= 2; ++j) {
      const double w1 = QM(1, j), w2 = QM(2, j);
      const double ww[3] = {0.0, w1, w2};
      S[0 + (size_t)(j - 1) * 2] = ww[indexc[1]];
      S[1 + (size_t)(j - 1) * 2] = ww[indexc[2]];
    }
  } else {
    std::vector<double> s0(k + 1);
    for (int j = 1; j <= k; ++j) s0[j] = w[j];
    for (int j = 1; j <= k; ++j) w[j] = QM(j, j);
    for (int j = 1; j <= k; ++j) {
      for (int q = 1; q <= j - 1; ++q) w[q] = w[q] * (QM(q, j) / (lam[q] - lam[j]));
      for (int q = j + 1; q <= k; ++q) w[q] = w[q] * (QM(q, j) / (lam[q] - lam[j]));
    }
    for (int q = 1; q <= k; ++q) {
      const double sg = s0[q] > 0 ? 1.0 : (s0[q] < 0 ? -1.0 : 0.0);
      w[q] = sg * std::sqrt(-w[q]);
    }
    for (int j = 1; j <= k; ++j) {
      double sc = 0.0, ss = 1.0;
      for (int q = 1; q <= k; ++q) {
        s0[q] = w[q] / QM(q, j);
        const double a = std::fabs(s0[q]);
        if (a > 0) {
          if (sc < a) { ss = 1.0 + ss * (sc / a) * (sc / a); sc = a; }
          else ss += (a / sc) * (a / sc);
        }
      }
      const double t = sc * std::sqrt(ss);
      for (int q = 1; q <= k; ++q) S[(q - 1) + (size_t)(j - 1) * k] = s0[indexc[q]] / t;
    }
  }
  // updated eigenvectors: Q[n1+1:n, 1:k] = [Q2_3 Q2_4] S[c1+1 : c1+n23, :],
  // Q[1:n1, 1:k] = [Q2_1 Q2_2] S[1 : n12, :]
  const int n12 = c1 + c2, n23 = c2 + c3;
  for (int j = 1; j <= k; ++j) {
    for (int r = 1; r <= n2; ++r) {
      double acc = 0.0;
      for (int q = 1; q <= n23; ++q) acc += Q34[(r - 1) + (size_t)(q - 1) * n2] * S[(c1 + q - 1) + (size_t)(j - 1) * k];
      QM(n1 + r, j) = acc;
    }
    for (int r = 1; r <= n1; ++r) {
      double acc = 0.0;
      for (int q = 1; q <= n12; ++q) acc += Q12[(r - 1) + (size_t)(q - 1) * n1] * S[(q - 1) + (size_t)(j - 1) * k];
      QM(r, j) = acc;
    }
  }
  const std::vector<int> p = dc_sortperm(d, n);
  for (int j = 1; j <= n; ++j) indexq[j - 1] = p[j - 1] + 1;
  return true;
#undef QM
}

// _dcschur_core! (107-196): d (n), e (n-1), Q (n x n, ld ldq, the identity on entry)
inline bool dc_core(int n, double* d, double* e, double* Q, int ldq, int nqrmax) {
  std::vector<int> itree(1, n);
  int nsub = 1;
  while (itree[nsub - 1] > nqrmax) {
    itree.resize(2 * nsub);
    for (int j = nsub; j >= 1; --j) {
      itree[2 * j - 1] = itree[j - 1] >> 1;
      itree[2 * j - 2] = (itree[j - 1] + 1) >> 1;
    }
    nsub *= 2;
  }
  for (int j = 2; j <= nsub; ++j) itree[j - 1] += itree[j - 2];
  for (int i = 1; i <= nsub - 1; ++i) {
    const int i1 = itree[i - 1] + 1, i2 = i1 - 1;
    d[i2 - 1] -= std::fabs(e[i2 - 1]);
    d[i1 - 1] -= std::fabs(e[i2 - 1]);
  }
  std::vector<int> indexq(n);
  for (int i = 0; i <= nsub - 1; ++i) {
    const int submat = i == 0 ? 1 : itree[i - 1] + 1;
    const int msz = i == 0 ? itree[0] : itree[i] - itree[i - 1];
    std::vector<double> W((size_t)msz * msz, 0.0);
    for (int q = 0; q < msz; ++q) W[q + (size_t)q * msz] = 1.0;
    steqr<double, double>(msz, d + submat - 1, e + submat - 1, W.data(), msz, msz, 30LL * msz);
    for (int c = 0; c < msz; ++c)
      for (int r = 0; r < msz; ++r) Q[(submat - 1 + r) + (size_t)(submat - 1 + c) * ldq] = W[r + (size_t)c * msz];
    for (int j = 0; j < msz; ++j) indexq[submat - 1 + j] = j + 1;
  }
  while (nsub > 1) {
    for (int i = 0; i <= nsub - 2; i += 2) {
      int submat, msz, msd2;
      if (i == 0) {
        submat = 1;
        msz = itree[1];
        msd2 = itree[0];
      } else {
        submat = itree[i - 1] + 1;
        msz = itree[i + 1] - itree[i - 1];
        msd2 = (msz + 1) >> 1;
      }
      const double rho = e[submat + msd2 - 2];
      if (!dc_merge(msz, d + submat - 1, Q + (submat - 1) + (size_t)(submat - 1) * ldq, ldq, &indexq[submat - 1], rho,
                    msd2))
        return false;
      itree[(i >> 1)] = itree[i + 1];
    }
    nsub >>= 1;
  }
  return true;
}

// _gschur!(SymTridiagonal(d, e), DivideAndConquer(), Z) (6-104): d receives the
// eigenvalues in the algorithm's order; Z (n x n, ld ldz, or null) is multiplied from the
// right by the eigenvectors.  Returns 0, or 1 when a secular equation did not converge.
inline int stedc(int n, double* d, double* e, double* Z, int ldz, int nqrmax = 25) {
  if (n == 0) return 0;
  if (n == 1) {
    if (Z) Z[0] = 1.0;
    return 0;
  }
  const double epsT = lim<double>::eps();
  if (n <= nqrmax) {
    steqr<double, double>(n, d, e, Z, ldz, Z ? n : 0, 30LL * n);
    return 0;
  }
  int istart = 1;
  while (istart <= n) {
    int ifinish = istart;
    while (ifinish < n) {
      const double tiny = epsT * std::sqrt(std::fabs(d[ifinish - 1])) * std::sqrt(std::fabs(d[ifinish]));
      if (std::fabs(e[ifinish - 1]) <= tiny) break;
      ifinish += 1;
    }
    const int m = ifinish - istart + 1;
    if (m == 1) {
      istart = ifinish + 1;
      continue;
    }
    double* dv = d + istart - 1;
    double* ev = e + istart - 1;
    std::vector<double> W((size_t)m * m, 0.0);
    for (int q = 0; q < m; ++q) W[q + (size_t)q * m] = 1.0;
    if (m > nqrmax) {
      double t1 = 0.0, t2 = 0.0;
      for (int q = 0; q < m; ++q) t1 = std::max(t1, std::fabs(dv[q]));
      for (int q = 0; q < m - 1; ++q) t2 = std::max(t2, std::fabs(ev[q]));
      const double orgnrm = std::max(t1, t2);
      for (int q = 0; q < m; ++q) dv[q] *= (1.0 / orgnrm);
      for (int q = 0; q < m - 1; ++q) ev[q] *= (1.0 / orgnrm);
      if (!dc_core(m, dv, ev, W.data(), m, nqrmax)) return 1;
      for (int q = 0; q < m; ++q) dv[q] *= orgnrm;
    } else {
      steqr<double, double>(m, dv, ev, Z ? W.data() : nullptr, m, Z ? m : 0, 30LL * m);
    }
    if (Z) {
      std::vector<double> Zt((size_t)n * m);
      for (int c = 0; c < m; ++c)
        for (int r = 0; r < n; ++r) Zt[r + (size_t)c * n] = Z[r + (size_t)(istart - 1 + c) * ldz];
      for (int c = 0; c < m; ++c)
        for (int r = 0; r < n; ++r) {
          double acc = 0.0;
          for (int q = 0; q < m; ++q) acc += Zt[r + (size_t)q * n] * W[q + (size_t)c * m];
          Z[r + (size_t)(istart - 1 + c) * ldz] = acc;
        }
    }
    istart = ifinish + 1;
  }
  return 0;
}

}  // namespace orc
