// Divide-and-conquer eigensolver of real symmetric tridiagonal matrices
// (src/symtri_dc.jl, after LAPACK's xSTEDC / xLAED0-6) on the GPU.
//
// run_stedc is _gschur!(A, DivideAndConquer(), Z) (symtri_dc.jl:6-104): the matrix splits at
// negligible off-diagonals; blocks of order <= 25 take the QR iteration, larger ones are
// scaled and run through _dcschur_core! (107-196):
//   * the subproblem tree is index arithmetic on the host;
//   * the rank-one cuts and the leaves (QR iteration, one warp per leaf, k_steqr_leaves)
//     run in one launch each;
//   * each level of merges (_dcmerge!, 200-217) runs as a handful of launches over all the
//     level's merges at once:
//       k_dc_prep     z (last row of Q1, first row of Q2), lambda = d[indexq], the tolerance
//       k_dc_rank     sortperm of lambda (stable, by counting ranks)
//       k_dc_deflate  _dcdeflate! (221-425): one CTA per merge; the small-z and close-pair
//                     tests evaluated for all positions in parallel, then thread 0 walks the
//                     reference's scan (re-testing a pair only after a rotation) and records
//                     the Givens rotations, which the CTA applies to Q row by row; the
//                     column-type counts and partition by ballot scans
//       k_dc_gather / k_dc_place  the gathers of Q2 by column type and the deflated columns
//                     to the end, one warp per column over all the level's merges
//       k_dc_secular  the roots of the secular equation, one warp per root (_dcroot!,
//                     777-927, with _dcroot2!, _dcnewton and the i = n / i < n helpers;
//                     the lanes split the sums over the poles)
//       k_dc_lowner / k_dc_vecs   the eigenvectors of the rank-one problem (_dcsecular!,
//                     441-472)
//       the update Q = Q2 S (_dcsecular!, 474-488) as two GEMMs per merge: the FP64 product on
//       the BF16 tensor cores (gemm_f64_tc.cu) for large merges, a plain FP64 kernel over all
//       small merges of the level at once
//       k_dc_rank     indexq = sortperm(d)
// The reference's quirks are kept (the _dcnewton ones are in dcnewton below).  The
// reference's norm(s0) and mul! run through BLAS; here they are a scaled sum of squares and
// the GEMMs above, so the results agree with the reference to rounding, not to the bit.
#include <algorithm>
#include <cstring>
#include <vector>

#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kDcQrMax = 25;        // nqrmax: largest leaf order before a split
constexpr int kDcT = 512;           // threads of the per-merge CTAs
constexpr int kDcSmall = 256;       // merges of at most this order multiply with k_dc_gemm_small
constexpr double kDcEps = 2.220446049250313e-16;

struct DcMerge {
  int off, n, n1, pad;
  long long qoff;  // doubles: the merge's Q2 blocks (2 n^2)
  long long soff;  // doubles: the merge's k x k rank-one eigenvectors S (n^2)
};
struct DcInfo {
  int k, c1, c2, c3, c4, nrot, trivial, pad;
  double rho, tol;
};

__device__ __forceinline__ double dsq(double x) { return x * x; }
// 1-based index clamped into [1, n]: rank collisions (NaN input) leave slots unwritten, and
// every index that addresses memory stays inside its merge whatever the data
__device__ __forceinline__ int clamp1(int i, int n) { return i < 1 ? 1 : (i > n ? n : i); }

template <int NT> __device__ double block_max_d(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = red[0];
  for (int q = 1; q < NT / 32; ++q) r = fmax(r, red[q]);
  __syncthreads();
  return r;
}

// ---- the secular equation (symtri_dc.jl:492-1163) -----------------------------------------
__device__ double dc_root2(int i, const double* d, const double* z, double* delta, double rho) {
  const double D = d[1] - d[0];
  double lam, tau;
  if (i == 1) {
    const double w = 1.0 + 2.0 * rho * (dsq(z[1]) - dsq(z[0])) / D;
    if (w > 0) {
      const double b = D + rho * (dsq(z[0]) + dsq(z[1]));
      const double c = rho * dsq(z[0]) * D;
      tau = 2.0 * c / (b + sqrt(b * b - 4.0 * c));
      lam = d[0] + tau;
      delta[0] = -z[0] / tau;
      delta[1] = z[1] / (D - tau);
    } else {
      const double b = -D + rho * (dsq(z[0]) + dsq(z[1]));
      const double c = rho * dsq(z[1]) * D;
      tau = b > 0 ? -2.0 * c / (b + sqrt(b * b + 4.0 * c)) : (b - sqrt(b * b + 4.0 * c)) / 2.0;
      lam = d[1] + tau;
      delta[0] = -z[0] / (D + tau);
      delta[1] = -z[1] / tau;
    }
  } else {
    const double b = -D + rho * (dsq(z[0]) + dsq(z[1]));
    const double c = rho * dsq(z[1]) * D;
    tau = b > 0 ? (b + sqrt(b * b + 4.0 * c)) / 2.0 : 2.0 * c / (-b + sqrt(b * b + 4.0 * c));
    lam = d[1] + tau;
    delta[0] = -z[0] / (D + tau);
    delta[1] = -z[1] / tau;
  }
  const double t = sqrt(dsq(delta[0]) + dsq(delta[1]));
  delta[0] = delta[0] / t;
  delta[1] = delta[1] / t;
  return lam;
}

// _dcnewton (976-1163).  Kept from the reference: the first quadratic step has no
// division by 2c (1011), the first evaluation uses dscale[1] for all three poles
// (1061-1069), and sclinv = small2 in both scaling branches (1047-1053).
__device__ double dc_newton(int kniter, bool orig, double rho, const double* d, const double* z, double finit) {
  const int maxit = 40;
  double lbd = orig ? d[1] : d[0], ubd = orig ? d[2] : d[1];
  if (finit < 0) lbd = 0.0;
  else ubd = 0.0;
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
    t = fmax(fmax(fabs(a), fabs(b)), fabs(c));
    a /= t;
    b /= t;
    c /= t;
    if (c == 0) tau = b / a;
    else if (a < 0) tau = a - sqrt(fabs(a * a - 4.0 * b * c));
    else tau = 2.0 * b / (a + sqrt(fabs(a * a - 4.0 * b * c)));
    if (tau < lbd || tau > ubd) tau = (lbd + ubd) / 2.0;
    if (d[0] == tau || d[1] == tau || d[2] == tau) {
      tau = 0.0;
    } else {
      t = finit + tau * z[0] / (d[0] * (d[0] - tau)) + tau * z[1] / (d[1] * (d[1] - tau)) +
          tau * z[2] / (d[2] * (d[2] - tau));
      if (t <= 0) lbd = tau;
      else ubd = tau;
      if (fabs(finit) <= fabs(t)) tau = 0.0;
    }
  }
  const double small1 = 0x1p-341, sminv1 = 0x1p341, small2 = 0x1p-682, sminv2 = 0x1p682;
  const double t0 = orig ? fmin(fabs(d[1] - tau), fabs(d[2] - tau)) : fmin(fabs(d[0] - tau), fabs(d[1] - tau));
  const bool scale = t0 <= small1;
  double ds[3], zs[3], sclinv = 1.0;
  const double sclfac = t0 <= small2 ? sminv2 : sminv1;
  for (int q = 0; q < 3; ++q) {
    ds[q] = scale ? d[q] * sclfac : d[q];
    zs[q] = scale ? z[q] * sclfac : z[q];
  }
  if (scale) {
    sclinv = small2;
    tau *= sclfac;
    lbd *= sclfac;
    ubd *= sclfac;
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
  if (fabs(f) <= 0) return scale ? tau * sclinv : tau;
  if (f <= 0) lbd = tau;
  else ubd = tau;
  for (int it = 2; it <= maxit; ++it) {
    const double t1 = orig ? ds[1] - tau : ds[0] - tau, t2 = orig ? ds[2] - tau : ds[1] - tau;
    double a = (t1 + t2) * f - t1 * t2 * df;
    double b = t1 * t2 * f;
    double c = f - (t1 + t2) * df + t1 * t2 * ddf;
    const double tm = fmax(fmax(fabs(a), fabs(b)), fabs(c));
    a /= tm;
    b /= tm;
    c /= tm;
    double eta;
    if (c == 0) eta = b / a;
    else if (a <= 0) eta = (a - sqrt(fabs(a * a - 4.0 * b * c))) / (2.0 * c);
    else eta = 2.0 * b / (a + sqrt(fabs(a * a - 4.0 * b * c)));
    if (f * eta >= 0) eta = -f / df;
    tau += eta;
    if (tau < lbd || tau > ubd) tau = (lbd + ubd) / 2.0;
    fc = 0.0;
    double erretm = 0.0;
    df = 0.0;
    ddf = 0.0;
    bool hit = false;
    for (int q = 0; q < 3; ++q) {
      if ((ds[q] - tau) != 0) {
        const double tt = 1.0 / (ds[q] - tau);
        const double u1 = zs[q] * tt, u2 = u1 * tt, u3 = u2 * tt, u4 = u1 / ds[q];
        fc += u4;
        erretm += fabs(u4);
        df += u2;
        ddf += u3;
      } else {
        hit = true;
        break;
      }
    }
    if (hit) break;
    f = finit + tau * fc;
    erretm = 8.0 * (fabs(finit) + fabs(tau) * erretm) + fabs(tau) * df;
    if ((fabs(f) <= 4.0 * kDcEps * erretm) || ((ubd - lbd) <= 4.0 * kDcEps * fabs(tau))) break;
    if (f <= 0) lbd = tau;
    else ubd = tau;
  }
  return scale ? tau * sclinv : tau;
}

// _dcroot! (777-927): root i (1-based) of the secular equation of (d, z, rho) of order n;
// delta (n, stride 1) receives d - lambda.
__device__ double dc_root(int n, int i, const double* __restrict__ dd, const double* __restrict__ zz,
                          double* __restrict__ dl, double rho, bool* conv) {
  const int maxit = 30;
  const double* d = dd - 1;
  const double* z = zz - 1;
  double* delta = dl - 1;
  *conv = true;
  if (n == 1) {
    delta[1] = 1.0;
    return d[1] + rho * dsq(z[1]);
  }
  if (n == 2) return dc_root2(i, dd, zz, dl, rho);
  const double rhoinv = 1.0 / rho;
  double dltlb, dltub, w, tau, erretm;
  if (i == n) {
    const int ii = n - 1;
    const double midpt = rho / 2.0;
    for (int j = 1; j <= n; ++j) delta[j] = (d[j] - d[i]) - midpt;
    {
      double psi = 0.0;
      for (int j = 1; j <= n - 2; ++j) psi += dsq(z[j]) / delta[j];
      const double c = rhoinv + psi;
      w = c + dsq(z[ii]) / delta[ii] + dsq(z[n]) / delta[n];
      const double D = d[n] - d[n - 1];
      const double a = -c * D + dsq(z[n - 1]) + dsq(z[n]);
      const double b = dsq(z[n]) * D;
      const double q = a < 0 ? 2.0 * b / (sqrt(a * a + 4.0 * b * c) - a) : (a + sqrt(a * a + 4.0 * b * c)) / (2.0 * c);
      if (w <= 0) {
        const double t = dsq(z[n - 1]) / (d[n] - d[n - 1] + rho) + dsq(z[n]) / rho;
        tau = (c <= t) ? rho : q;
        dltlb = midpt;
        dltub = rho;
      } else {
        tau = q;
        dltlb = 0.0;
        dltub = midpt;
      }
    }
    for (int j = 1; j <= n; ++j) delta[j] = (d[j] - d[i]) - tau;
    double dpsi = 0.0, dphi = 0.0;
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
      erretm = fabs(erretm);
      const double t = z[n] / delta[n];
      const double phi = z[n] * t;
      dphi = t * t;
      erretm = 8.0 * (-phi - psi) + erretm - phi + rhoinv + fabs(tau) * (dpsi + dphi);
      w = rhoinv + phi + psi;
    };
    auto step_n = [&](int iter) {
      double c = w - delta[n - 1] * dpsi - delta[n] * dphi;
      if (iter <= 2) c = fabs(c);
      const double a = (delta[n - 1] + delta[n]) * w - delta[n - 1] * delta[n] * (dpsi + dphi);
      const double b = delta[n - 1] * delta[n] * w;
      double eta;
      if (c == 0) eta = dltub - tau;
      else if (a >= 0) eta = (a + sqrt(fabs(a * a - 4.0 * b * c))) / (2.0 * c);
      else eta = 2.0 * b / (a - sqrt(fabs(a * a - 4.0 * b * c)));
      if (w * eta > 0) eta = -w / (dpsi + dphi);
      const double t = tau + eta;
      if (t > dltub || t < dltlb) eta = w < 0 ? (dltub - tau) / 2.0 : (dltlb - tau) / 2.0;
      return eta;
    };
    update_n();
    if (fabs(w) < kDcEps * erretm) return d[i] + tau;
    if (w <= 0) dltlb = fmax(dltlb, tau);
    else dltub = fmin(dltub, tau);
    double eta = step_n(2);
    for (int j = 1; j <= n; ++j) delta[j] = delta[j] - eta;
    tau += eta;
    update_n();
    for (int niter = 3; niter <= maxit; ++niter) {
      if (fabs(w) < kDcEps * erretm) return d[i] + tau;
      if (w <= 0) dltlb = fmax(dltlb, tau);
      else dltub = fmin(dltub, tau);
      eta = step_n(niter);
      for (int j = 1; j <= n; ++j) delta[j] = delta[j] - eta;
      tau += eta;
      update_n();
    }
    *conv = false;
    return d[i] + tau;
  }
  const int ip1 = i + 1;
  const double D = d[ip1] - d[i];
  const double midpt = D / 2.0;
  for (int j = 1; j <= n; ++j) delta[j] = (d[j] - d[i]) - midpt;
  bool orig;
  {
    double psi = 0.0;
    for (int j = 1; j <= i - 1; ++j) psi = psi + dsq(z[j]) / delta[j];
    double phi = 0.0;
    for (int j = n; j >= i + 2; --j) phi = phi + dsq(z[j]) / delta[j];
    const double c = rhoinv + psi + phi;
    w = c + dsq(z[i]) / delta[i] + dsq(z[ip1]) / delta[ip1];
    orig = w > 0;
    if (orig) {
      const double a = c * D + dsq(z[i]) + dsq(z[ip1]);
      const double b = dsq(z[i]) * D;
      tau = a > 0 ? 2.0 * b / (a + sqrt(fabs(a * a - 4.0 * b * c))) : (a - sqrt(fabs(a * a - 4.0 * b * c))) / (2.0 * c);
      dltlb = 0.0;
      dltub = midpt;
    } else {
      const double a = c * D - dsq(z[i]) - dsq(z[ip1]);
      const double b = dsq(z[ip1]) * D;
      tau = a < 0 ? 2.0 * b / (a - sqrt(fabs(a * a + 4.0 * b * c))) : -(a + sqrt(fabs(a * a + 4.0 * b * c))) / (2.0 * c);
      dltlb = -midpt;
      dltub = 0.0;
    }
  }
  const int ii = orig ? i : i + 1;
  const double dorg = d[ii];
  for (int j = 1; j <= n; ++j) delta[j] = (d[j] - dorg) - tau;
  double Ppsi = 0.0, Pphi = 0.0, Pdpsi = 0.0, Pdphi = 0.0, Pdw = 0.0, w0 = 0.0;
  auto update = [&](double etaq) {
    double dpsi = 0.0, psi = 0.0;
    erretm = 0.0;
    for (int j = 1; j <= ii - 1; ++j) {
      const double t = z[j] / delta[j];
      psi += z[j] * t;
      dpsi += t * t;
      erretm += psi;
    }
    erretm = fabs(erretm);
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
    erretm = 8.0 * (phi - psi) + erretm + 2.0 * rhoinv + 3.0 * fabs(t) + fabs(tau + etaq) * dw;
    Ppsi = psi; Pphi = phi; Pdpsi = dpsi; Pdphi = dphi; Pdw = dw;
  };
  auto step = [&](int niter, bool switch3, bool sw) {
    double dpsi = Pdpsi, dphi = Pdphi;
    const double dw = Pdw;
    const int iip1 = ii + 1, iim1 = ii - 1;
    double eta;
    if (!switch3) {
      double c;
      if (!sw) {
        if (orig) c = w - delta[ip1] * dw - (d[i] - d[ip1]) * dsq(z[i] / delta[i]);
        else c = w - delta[i] * dw - (d[ip1] - d[i]) * dsq(z[ip1] / delta[ip1]);
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
          if (orig) a = dsq(z[i]) + dsq(delta[ip1]) * (dpsi + dphi);
          else a = dsq(z[ip1]) + dsq(delta[i]) * (dpsi + dphi);
        }
        eta = b / a;
      } else if (a <= 0) {
        eta = (a - sqrt(fabs(a * a - 4.0 * b * c))) / (2.0 * c);
      } else {
        eta = 2.0 * b / (a + sqrt(fabs(a * a - 4.0 * b * c)));
      }
    } else {
      const double t = rhoinv + Ppsi + Pphi;
      double c, z3[3];
      if (orig) {
        const double t1 = dsq(z[iim1] / delta[iim1]);
        c = t - delta[iip1] * (dpsi + dphi) - (d[iim1] - d[iip1]) * t1;
        z3[0] = dsq(z[iim1]);
        z3[2] = dsq(delta[iip1]) * ((dpsi - t1) + dphi);
      } else {
        const double t1 = dsq(z[iip1] / delta[iip1]);
        c = t - delta[iim1] * (dpsi + dphi) - (d[iip1] - d[iim1]) * t1;
        z3[0] = dsq(delta[iim1]) * (dpsi + (dphi - t1));
        z3[2] = dsq(z[iip1]);
      }
      z3[1] = dsq(z[ii]);
      const double d3[3] = {delta[iim1], delta[ii], delta[iip1]};
      eta = dc_newton(niter, orig, c, d3, z3, w);
    }
    if (w * eta > 0) eta = -w / dw;
    const double t = tau + eta;
    if (t > dltub || t < dltlb) eta = w < 0 ? (dltub - tau) / 2.0 : (dltlb - tau) / 2.0;
    return eta;
  };
  update(0.0);
  bool switch3 = orig ? (w0 < 0) : (w0 > 0);
  if (ii == 1 || ii == n) switch3 = false;
  if (fabs(w) < kDcEps * erretm) return dorg + tau;
  if (w <= 0) dltlb = fmax(dltlb, tau);
  else dltub = fmin(dltub, tau);
  double eta = step(2, switch3, false);
  double prev_w = w;
  for (int j = 1; j <= n; ++j) delta[j] = delta[j] - eta;
  update(eta);
  bool sw = orig ? (-w > fabs(prev_w) / 10.0) : (w > fabs(prev_w) / 10.0);
  tau += eta;
  for (int niter = 3; niter <= maxit; ++niter) {
    if (fabs(w) < kDcEps * erretm) return dorg + tau;
    if (w <= 0) dltlb = fmax(dltlb, tau);
    else dltub = fmin(dltub, tau);
    eta = step(niter, switch3, sw);
    for (int j = 1; j <= n; ++j) delta[j] = delta[j] - eta;
    tau += eta;
    prev_w = w;
    update(0.0);
    if ((w * prev_w > 0) && (fabs(w) > fabs(prev_w) / 10.0)) sw = !sw;
  }
  *conv = false;
  return dorg + tau;
}

// The same root with one warp: lanes split the sums over the poles and the updates of
// delta; the butterfly sums leave the same value in every lane, so the scalar steps run
// identically in all lanes.  The running erretm sums of the reference (erretm += psi after
// each term) are the weighted sums sum_i t_i (ii - i + 1) and sum_i t_i (i - ii).
__device__ __forceinline__ double wsum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ double dc_root_warp(int n, int i, const double* __restrict__ dd, const double* __restrict__ zz,
                               double* __restrict__ dl, double rho, bool* conv, int lane) {
  const int maxit = 30;
  const double* d = dd - 1;
  const double* z = zz - 1;
  double* delta = dl - 1;
  *conv = true;
  if (n <= 2) {
    double lam = 0.0;
    if (lane == 0) lam = dc_root(n, i, dd, zz, dl, rho, conv);
    __syncwarp();
    lam = __shfl_sync(0xffffffffu, lam, 0);
    return lam;
  }
  const double rhoinv = 1.0 / rho;
  double dltlb, dltub, w, tau, erretm;
  auto set_delta = [&](double org, double sh) {
    for (int j = 1 + lane; j <= n; j += 32) delta[j] = (d[j] - org) - sh;
    __syncwarp();
  };
  auto shift_delta = [&](double eta) {
    for (int j = 1 + lane; j <= n; j += 32) delta[j] = delta[j] - eta;
    __syncwarp();
  };
  if (i == n) {
    const int ii = n - 1;
    const double midpt = rho / 2.0;
    set_delta(d[i], midpt);
    {
      double ps = 0.0;
      for (int j = 1 + lane; j <= n - 2; j += 32) ps += dsq(z[j]) / delta[j];
      const double psi = wsum(ps);
      const double c = rhoinv + psi;
      w = c + dsq(z[ii]) / delta[ii] + dsq(z[n]) / delta[n];
      const double D = d[n] - d[n - 1];
      const double a = -c * D + dsq(z[n - 1]) + dsq(z[n]);
      const double b = dsq(z[n]) * D;
      const double q = a < 0 ? 2.0 * b / (sqrt(a * a + 4.0 * b * c) - a) : (a + sqrt(a * a + 4.0 * b * c)) / (2.0 * c);
      if (w <= 0) {
        const double t = dsq(z[n - 1]) / (d[n] - d[n - 1] + rho) + dsq(z[n]) / rho;
        tau = (c <= t) ? rho : q;
        dltlb = midpt;
        dltub = rho;
      } else {
        tau = q;
        dltlb = 0.0;
        dltub = midpt;
      }
    }
    set_delta(d[i], tau);
    double dpsi = 0.0, dphi = 0.0;
    auto update_n = [&]() {
      double ps = 0.0, dps = 0.0, er = 0.0;
      for (int j = 1 + lane; j <= ii; j += 32) {
        const double t = z[j] / delta[j];
        const double zt = z[j] * t;
        ps += zt;
        dps += t * t;
        er += zt * (double)(ii - j + 1);
      }
      const double psi = wsum(ps);
      dpsi = wsum(dps);
      erretm = fabs(wsum(er));
      const double t = z[n] / delta[n];
      const double phi = z[n] * t;
      dphi = t * t;
      erretm = 8.0 * (-phi - psi) + erretm - phi + rhoinv + fabs(tau) * (dpsi + dphi);
      w = rhoinv + phi + psi;
    };
    auto step_n = [&](int iter) {
      double c = w - delta[n - 1] * dpsi - delta[n] * dphi;
      if (iter <= 2) c = fabs(c);
      const double a = (delta[n - 1] + delta[n]) * w - delta[n - 1] * delta[n] * (dpsi + dphi);
      const double b = delta[n - 1] * delta[n] * w;
      double eta;
      if (c == 0) eta = dltub - tau;
      else if (a >= 0) eta = (a + sqrt(fabs(a * a - 4.0 * b * c))) / (2.0 * c);
      else eta = 2.0 * b / (a - sqrt(fabs(a * a - 4.0 * b * c)));
      if (w * eta > 0) eta = -w / (dpsi + dphi);
      const double t = tau + eta;
      if (t > dltub || t < dltlb) eta = w < 0 ? (dltub - tau) / 2.0 : (dltlb - tau) / 2.0;
      return eta;
    };
    update_n();
    if (fabs(w) < kDcEps * erretm) return d[i] + tau;
    if (w <= 0) dltlb = fmax(dltlb, tau);
    else dltub = fmin(dltub, tau);
    double eta = step_n(2);
    shift_delta(eta);
    tau += eta;
    update_n();
    for (int niter = 3; niter <= maxit; ++niter) {
      if (fabs(w) < kDcEps * erretm) return d[i] + tau;
      if (w <= 0) dltlb = fmax(dltlb, tau);
      else dltub = fmin(dltub, tau);
      eta = step_n(niter);
      shift_delta(eta);
      tau += eta;
      update_n();
    }
    *conv = false;
    return d[i] + tau;
  }
  const int ip1 = i + 1;
  const double D = d[ip1] - d[i];
  const double midpt = D / 2.0;
  set_delta(d[i], midpt);
  bool orig;
  {
    double ps = 0.0, ph = 0.0;
    for (int j = 1 + lane; j <= n; j += 32) {
      if (j <= i - 1) ps += dsq(z[j]) / delta[j];
      else if (j >= i + 2) ph += dsq(z[j]) / delta[j];
    }
    const double psi = wsum(ps), phi = wsum(ph);
    const double c = rhoinv + psi + phi;
    w = c + dsq(z[i]) / delta[i] + dsq(z[ip1]) / delta[ip1];
    orig = w > 0;
    if (orig) {
      const double a = c * D + dsq(z[i]) + dsq(z[ip1]);
      const double b = dsq(z[i]) * D;
      tau = a > 0 ? 2.0 * b / (a + sqrt(fabs(a * a - 4.0 * b * c))) : (a - sqrt(fabs(a * a - 4.0 * b * c))) / (2.0 * c);
      dltlb = 0.0;
      dltub = midpt;
    } else {
      const double a = c * D - dsq(z[i]) - dsq(z[ip1]);
      const double b = dsq(z[ip1]) * D;
      tau = a < 0 ? 2.0 * b / (a - sqrt(fabs(a * a + 4.0 * b * c))) : -(a + sqrt(fabs(a * a + 4.0 * b * c))) / (2.0 * c);
      dltlb = -midpt;
      dltub = 0.0;
    }
  }
  const int ii = orig ? i : i + 1;
  const double dorg = d[ii];
  set_delta(dorg, tau);
  double Ppsi = 0.0, Pphi = 0.0, Pdpsi = 0.0, Pdphi = 0.0, Pdw = 0.0, w0 = 0.0;
  auto update = [&](double etaq) {
    double ps = 0.0, dps = 0.0, erp = 0.0, ph = 0.0, dph = 0.0, erf = 0.0;
    for (int j = 1 + lane; j <= n; j += 32) {
      if (j == ii) continue;
      const double t = z[j] / delta[j];
      const double zt = z[j] * t;
      if (j < ii) {
        ps += zt;
        dps += t * t;
        erp += zt * (double)(ii - j);
      } else {
        ph += zt;
        dph += t * t;
        erf += zt * (double)(j - ii);
      }
    }
    const double psi = wsum(ps), dpsi = wsum(dps), phi = wsum(ph), dphi = wsum(dph);
    erretm = fabs(wsum(erp)) + wsum(erf);
    w0 = rhoinv + phi + psi;
    double t = z[ii] / delta[ii];
    const double dw = dpsi + dphi + t * t;
    t = z[ii] * t;
    w = rhoinv + phi + psi + t;
    erretm = 8.0 * (phi - psi) + erretm + 2.0 * rhoinv + 3.0 * fabs(t) + fabs(tau + etaq) * dw;
    Ppsi = psi; Pphi = phi; Pdpsi = dpsi; Pdphi = dphi; Pdw = dw;
  };
  auto step = [&](int niter, bool switch3, bool sw) {
    double dpsi = Pdpsi, dphi = Pdphi;
    const double dw = Pdw;
    const int iip1 = ii + 1, iim1 = ii - 1;
    double eta;
    if (!switch3) {
      double c;
      if (!sw) {
        if (orig) c = w - delta[ip1] * dw - (d[i] - d[ip1]) * dsq(z[i] / delta[i]);
        else c = w - delta[i] * dw - (d[ip1] - d[i]) * dsq(z[ip1] / delta[ip1]);
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
          if (orig) a = dsq(z[i]) + dsq(delta[ip1]) * (dpsi + dphi);
          else a = dsq(z[ip1]) + dsq(delta[i]) * (dpsi + dphi);
        }
        eta = b / a;
      } else if (a <= 0) {
        eta = (a - sqrt(fabs(a * a - 4.0 * b * c))) / (2.0 * c);
      } else {
        eta = 2.0 * b / (a + sqrt(fabs(a * a - 4.0 * b * c)));
      }
    } else {
      const double t = rhoinv + Ppsi + Pphi;
      double c, z3[3];
      if (orig) {
        const double t1 = dsq(z[iim1] / delta[iim1]);
        c = t - delta[iip1] * (dpsi + dphi) - (d[iim1] - d[iip1]) * t1;
        z3[0] = dsq(z[iim1]);
        z3[2] = dsq(delta[iip1]) * ((dpsi - t1) + dphi);
      } else {
        const double t1 = dsq(z[iip1] / delta[iip1]);
        c = t - delta[iim1] * (dpsi + dphi) - (d[iip1] - d[iim1]) * t1;
        z3[0] = dsq(delta[iim1]) * (dpsi + (dphi - t1));
        z3[2] = dsq(z[iip1]);
      }
      z3[1] = dsq(z[ii]);
      const double d3[3] = {delta[iim1], delta[ii], delta[iip1]};
      eta = dc_newton(niter, orig, c, d3, z3, w);
    }
    if (w * eta > 0) eta = -w / dw;
    const double t = tau + eta;
    if (t > dltub || t < dltlb) eta = w < 0 ? (dltub - tau) / 2.0 : (dltlb - tau) / 2.0;
    return eta;
  };
  update(0.0);
  bool switch3 = orig ? (w0 < 0) : (w0 > 0);
  if (ii == 1 || ii == n) switch3 = false;
  if (fabs(w) < kDcEps * erretm) return dorg + tau;
  if (w <= 0) dltlb = fmax(dltlb, tau);
  else dltub = fmin(dltub, tau);
  double eta = step(2, switch3, false);
  double prev_w = w;
  shift_delta(eta);
  update(eta);
  bool sw = orig ? (-w > fabs(prev_w) / 10.0) : (w > fabs(prev_w) / 10.0);
  tau += eta;
  for (int niter = 3; niter <= maxit; ++niter) {
    if (fabs(w) < kDcEps * erretm) return dorg + tau;
    if (w <= 0) dltlb = fmax(dltlb, tau);
    else dltub = fmin(dltub, tau);
    eta = step(niter, switch3, sw);
    shift_delta(eta);
    tau += eta;
    prev_w = w;
    update(0.0);
    if ((w * prev_w > 0) && (fabs(w) > fabs(prev_w) / 10.0)) sw = !sw;
  }
  *conv = false;
  return dorg + tau;
}

// ---- kernels ------------------------------------------------------------------------------
__global__ void k_dc_split(int n, const double* __restrict__ d, const double* __restrict__ e, int* __restrict__ brk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const double tiny = kDcEps * sqrt(fabs(d[i])) * sqrt(fabs(d[i + 1]));
  brk[i] = fabs(e[i]) <= tiny ? 1 : 0;
}

// orgnrm = max(max |d|, max |e|) of the block; d, e scaled by 1 / orgnrm (symtri_dc.jl:63-69)
__global__ void __launch_bounds__(1024) k_dc_scale(double* d, double* e, int m, double* orgnrm) {
  __shared__ double red[32];
  double t1 = 0.0, t2 = 0.0;
  for (int i = threadIdx.x; i < m; i += 1024) t1 = fmax(t1, fabs(d[i]));
  for (int i = threadIdx.x; i < m - 1; i += 1024) t2 = fmax(t2, fabs(e[i]));
  t1 = block_max_d<1024>(t1, red);
  t2 = block_max_d<1024>(t2, red);
  const double nrm = fmax(t1, t2), r = 1.0 / nrm;
  for (int i = threadIdx.x; i < m; i += 1024) d[i] *= r;
  for (int i = threadIdx.x; i < m - 1; i += 1024) e[i] *= r;
  if (threadIdx.x == 0) *orgnrm = nrm;
}

__global__ void k_dc_unscale(double* d, int m, const double* orgnrm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) d[i] *= *orgnrm;
}

// the rank-one cuts between the leaves (symtri_dc.jl:128-134); pos: 0-based last row of
// the left leaf
__global__ void k_dc_cuts(int ncut, const int* __restrict__ pos, double* d, const double* __restrict__ e) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ncut) return;
  const int i2 = pos[q];
  const double a = fabs(e[i2]);
  d[i2] -= a;
  d[i2 + 1] -= a;
}

// z, lambda = d[indexq] and the deflation tolerance of each merge (_dcmerge! 203-205,
// _dcdeflate! 221-245)
__global__ void __launch_bounds__(256) k_dc_prep(const DcMerge* __restrict__ mg, DcInfo* info,
                                                 const double* __restrict__ e, const double* __restrict__ d,
                                                 const double* __restrict__ Q, long long ld, int* indexq, double* z,
                                                 double* lam) {
  __shared__ double red[8];
  const DcMerge M = mg[blockIdx.x];
  const int o = M.off, n = M.n, n1 = M.n1;
  const double* Qb = Q + o + (size_t)o * ld;
  const double rho = e[o + n1 - 1];
  const double t0 = 1.0 / sqrt(2.0);
  double zm = 0.0, dm = 0.0;
  for (int j = threadIdx.x; j < n; j += 256) {
    double zj = j < n1 ? Qb[(n1 - 1) + (size_t)j * ld] : Qb[n1 + (size_t)j * ld];
    zj = zj * t0;
    if (rho < 0 && j >= n1) zj = zj * -1.0;
    z[o + j] = zj;
    int iq = clamp1(indexq[o + j], n);
    if (j >= n1) {
      iq += n1;
      indexq[o + j] = iq;
    }
    lam[o + j] = d[o + clamp1(iq, n) - 1];
    zm = fmax(zm, fabs(zj));
    dm = fmax(dm, fabs(d[o + j]));
  }
  zm = block_max_d<256>(zm, red);
  dm = block_max_d<256>(dm, red);
  if (threadIdx.x == 0) {
    DcInfo I{};
    I.rho = fabs(2.0 * rho);
    I.tol = 8.0 * kDcEps * fmax(zm, dm);
    I.trivial = I.rho * zm <= I.tol ? 1 : 0;
    info[blockIdx.x] = I;
  }
}

// Stable sortperm of v within each merge by counting ranks: out[off + rank] = j + 1.
// only_k: skip merges whose k is 0 (their indexq is set by k_dc_deflate).
__global__ void __launch_bounds__(256) k_dc_rank(const DcMerge* __restrict__ mg, const DcInfo* __restrict__ info,
                                                 const double* __restrict__ v, int* out, int only_k) {
  __shared__ double tile[2048];
  const DcMerge M = mg[blockIdx.x];
  if (only_k && info[blockIdx.x].k == 0) return;
  const int o = M.off, n = M.n;
  if ((int)(blockIdx.y * 256) >= n) return;
  const int j = blockIdx.y * 256 + threadIdx.x;
  const double x = j < n ? v[o + j] : 0.0;
  int r = 0;
  for (int t0 = 0; t0 < n; t0 += 2048) {
    const int cnt = min(2048, n - t0);
    __syncthreads();
    for (int q = threadIdx.x; q < cnt; q += 256) tile[q] = v[o + t0 + q];
    __syncthreads();
    if (j < n)
      for (int q = 0; q < cnt; ++q) {
        const double y = tile[q];
        r += (y < x || (y == x && t0 + q < j)) ? 1 : 0;
      }
  }
  if (j < n) out[o + r] = j + 1;
}

// _dcdeflate! (221-425), one CTA per merge.  Q2 region of the merge: [Q2_1 Q2_2] (n1 x
// (c1 + c2), ld n1) at qoff, [Q2_3 Q2_4] (n2 x (c2 + c3), ld n2) at qoff + n1^2, Q2_5
// (n x c4, ld n) at qoff + n1^2 + n2^2.
__global__ void __launch_bounds__(kDcT) k_dc_deflate(const DcMerge* __restrict__ mg, DcInfo* info, double* dg,
                                                     double* Q, long long ld, int* indexqg, double* zg,
                                                     double* lamg, double* wg, int* indexcg, int* indexg,
                                                     int* indexpg, int* coltypeg, int* rpg, int* rng_,
                                                     double* rcg, double* rsg, double* Q2, int* sfg, int* sprevg,
                                                     double* scg, double* ssg, double* stg) {
  __shared__ int sh[8];
  const DcMerge M = mg[blockIdx.x];
  const int o = M.off, n = M.n, n1 = M.n1, tid = threadIdx.x;
  double* Qb = Q + o + (size_t)o * ld;
  double* d = dg + o;
  double* z = zg + o;
  double* lam = lamg + o;
  double* w = wg + o;
  int* indexq = indexqg + o;
  int* indexc = indexcg + o;
  int* index = indexg + o;
  int* indexp = indexpg + o;
  int* coltype = coltypeg + o;
  int* rp = rpg + o;
  int* rn = rng_ + o;
  double* rc = rcg + o;
  double* rs = rsg + o;
  int* sf = sfg + o;        // per sorted position: bit 0 small z, bit 1 close pair with the previous candidate
  int* sprev = sprevg + o;  // inclusive max-scan of the positions whose z is not small
  double* sc = scg + o;     // the close-pair test's c, s, tau on the unrotated values
  double* ss = ssg + o;
  double* st = stg + o;
  (void)Q2;
  DcInfo I = info[blockIdx.x];
  for (int j = tid; j < n; j += kDcT) {
    index[j] = clamp1(indexq[clamp1(indexc[j], n) - 1], n);
    coltype[j] = j < n1 ? 1 : 3;
    indexp[j] = 0;
    w[j] = 0.0;
  }
  __syncthreads();
  if (I.trivial) {
    // d follows its sorted order; k_dc_gather / k_dc_place reorganize Q's columns (233-243)
    for (int j = tid; j < n; j += kDcT) lam[j] = d[clamp1(index[j], n) - 1];
    __syncthreads();
    for (int j = tid; j < n; j += kDcT) {
      d[j] = lam[j];
      indexq[j] = j + 1;
    }
    if (tid == 0) {
      I.k = 0;
      I.nrot = 0;
      info[blockIdx.x] = I;
    }
    return;
  }
  // The reference's scan (244-367) decides, in sorted order, whether each z is small and
  // whether each remaining candidate forms a close pair with the previous one.  Only the
  // rotations of close pairs change z and d (of those two columns), so the tests can be
  // evaluated first for every position in parallel on the values before any rotation; the
  // sequential walk (thread 0) then re-evaluates a pair only right after a rotation, with
  // the same expressions in the same order.
  const double rho = I.rho, tol = I.tol;
  const unsigned FULL = 0xffffffffu;
  const int lane = tid & 31, wid = tid >> 5;
  __shared__ int s_red[kDcT / 32];
  __shared__ int s_carry;
  // pass 1: small-z flags and the inclusive max-scan of the positions whose z is not small
  if (tid == 0) s_carry = -1;
  __syncthreads();
  for (int t0 = 0; t0 < n; t0 += kDcT) {
    const int j = t0 + tid;
    int v = -1;
    if (j < n) {
      const bool sm = rho * fabs(z[clamp1(index[j], n) - 1]) <= tol;
      sf[j] = sm ? 1 : 0;
      v = sm ? -1 : j;
    }
    int x = v;
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(FULL, x, off);
      if (lane >= off) x = max(x, y);
    }
    if (lane == 31) s_red[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int wv = lane < kDcT / 32 ? s_red[lane] : -1;
      for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(FULL, wv, off);
        if (lane >= off) wv = max(wv, y);
      }
      if (lane < kDcT / 32) s_red[lane] = wv;
    }
    __syncthreads();
    const int incl = max(max(x, wid > 0 ? s_red[wid - 1] : -1), s_carry);
    if (j < n) sprev[j] = incl;
    __syncthreads();
    if (tid == kDcT - 1) s_carry = incl;
    __syncthreads();
  }
  // pass 2: the close-pair test of (previous candidate, j) on the unrotated values
  for (int j = tid; j < n; j += kDcT) {
    if (sf[j] & 1) continue;
    const int p = j > 0 ? sprev[j - 1] : -1;
    if (p < 0) continue;
    const int nj = clamp1(index[j], n), pjv = clamp1(index[p], n);
    double sv = z[pjv - 1], c = z[nj - 1];
    const double tau = hypot(c, sv);
    const double t = d[nj - 1] - d[pjv - 1];
    c /= tau;
    sv = -sv / tau;
    sc[j] = c;
    ss[j] = sv;
    st[j] = tau;
    if (fabs(t * c * sv) <= tol) sf[j] |= 2;
  }
  __syncthreads();
  // pass 3: the reference's walk
  if (tid == 0) {
    double* D = d - 1;  // 1-based views
    double* Z = z - 1;
    double* L = lam - 1;
    double* Wv = w - 1;
    int* IX = index - 1;
    int* IP = indexp - 1;
    int* CT = coltype - 1;
    int k = 0, k2 = n + 1, jj = 1, pj = 0, nrot = 0;
    for (; jj <= n; ++jj) {
      const int nj = clamp1(IX[jj], n);
      if (sf[jj - 1] & 1) {
        k2 -= 1;
        CT[nj] = 4;
        IP[k2] = nj;
      } else {
        pj = nj;
        break;
      }
    }
    bool rotated = false;
    for (jj = jj + 1; jj <= n; ++jj) {
      const int nj = clamp1(IX[jj], n);
      const int f = sf[jj - 1];
      if (f & 1) {
        k2 -= 1;
        CT[nj] = 4;
        IP[k2] = nj;
        continue;
      }
      double c, sv, tau;
      bool close;
      if (!rotated) {
        c = sc[jj - 1];
        sv = ss[jj - 1];
        tau = st[jj - 1];
        close = (f & 2) != 0;
      } else {
        sv = Z[pj];
        c = Z[nj];
        tau = hypot(c, sv);
        const double t = D[nj] - D[pj];
        c /= tau;
        sv = -sv / tau;
        close = fabs(t * c * sv) <= tol;
      }
      if (close) {
        Z[nj] = tau;
        Z[pj] = 0.0;
        if (CT[nj] != CT[pj]) CT[nj] = 2;
        CT[pj] = 4;
        rp[nrot] = pj;
        rn[nrot] = nj;
        rc[nrot] = c;
        rs[nrot] = sv;
        ++nrot;
        const double t = D[pj] * (c * c) + D[nj] * (sv * sv);
        D[nj] = D[pj] * (sv * sv) + D[nj] * (c * c);
        D[pj] = t;
        k2 -= 1;
        int i = 1;
        if (k2 + i > n) {
          IP[k2 + i - 1] = pj;
        } else {
          while (k2 + i <= n) {
            if (D[pj] < D[clamp1(IP[k2 + i], n)]) {
              IP[k2 + i - 1] = IP[k2 + i];
              IP[k2 + i] = pj;
              i += 1;
            } else {
              IP[k2 + i - 1] = pj;
              break;
            }
          }
        }
        pj = nj;
        rotated = true;
      } else {
        k += 1;
        L[k] = D[pj];
        Wv[k] = Z[pj];
        IP[k] = pj;
        pj = nj;
        rotated = false;
      }
    }
    if (pj < 1) pj = 1;  // every z small: the trivial branch above takes that case (NaN input aside)
    k += 1;
    L[k] = D[pj];
    Wv[k] = Z[pj];
    IP[k] = pj;
    sh[5] = nrot;
  }
  __syncthreads();
  // pass 4: the column-type counts and the stable partition of the positions by type
  // (_dcdeflate! 372-382), four ballot scans per tile
  __shared__ int s_cnt[4], s_wt[4][kDcT / 32], s_base[4];
  if (tid < 4) s_cnt[tid] = 0;
  __syncthreads();
  for (int j = tid; j < n; j += kDcT) {
    int ct = coltype[j];
    if (ct < 1 || ct > 4) ct = 4;
    atomicAdd(&s_cnt[ct - 1], 1);
  }
  __syncthreads();
  if (tid == 0) {
    s_base[0] = 1;
    s_base[1] = 1 + s_cnt[0];
    s_base[2] = 1 + s_cnt[0] + s_cnt[1];
    s_base[3] = 1 + s_cnt[0] + s_cnt[1] + s_cnt[2];
  }
  __syncthreads();
  for (int t0 = 0; t0 < n; t0 += kDcT) {
    const int j = t0 + tid;  // 0-based position in indexp order
    int js = 1, ct = 0;
    if (j < n) {
      js = clamp1(indexp[j], n);
      ct = coltype[js - 1];
      if (ct < 1 || ct > 4) ct = 4;
    }
    unsigned mask[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) mask[t] = __ballot_sync(FULL, ct == t + 1);
    if (lane == 0)
#pragma unroll
      for (int t = 0; t < 4; ++t) s_wt[t][wid] = __popc(mask[t]);
    __syncthreads();
    if (j < n) {
      const int t = ct - 1;
      int before = 0;
      for (int q = 0; q < wid; ++q) before += s_wt[t][q];
      const int pos = s_base[t] + before + __popc(mask[t] & ((1u << lane) - 1u));
      if (pos <= n) {
        index[pos - 1] = js;
        indexc[pos - 1] = j + 1;
      }
    }
    __syncthreads();
    if (tid < 4) {
      int tot = 0;
      for (int q = 0; q < kDcT / 32; ++q) tot += s_wt[tid][q];
      s_base[tid] += tot;
    }
    __syncthreads();
  }
  if (tid == 0) {
    I.c1 = s_cnt[0];
    I.c2 = s_cnt[1];
    I.c3 = s_cnt[2];
    I.c4 = s_cnt[3];
    I.k = n - I.c4;
    I.nrot = sh[5];
    info[blockIdx.x] = I;
    sh[0] = I.k; sh[1] = I.c1; sh[2] = I.c2; sh[3] = I.c3; sh[4] = I.c4;
  }
  __syncthreads();
  const int k = sh[0], nrot = sh[5];
  // rmul!(Q, Givens(pj, nj, c, s)') for the recorded rotations, in order, row by row
  if (nrot > 0)
    for (int r = tid; r < n; r += kDcT)
      for (int q = 0; q < nrot; ++q) {
        double* a = Qb + r + (size_t)(rp[q] - 1) * ld;
        double* b = Qb + r + (size_t)(rn[q] - 1) * ld;
        const double a1 = *a, a2 = *b, c = rc[q], s = rs[q];
        *a = a1 * c + a2 * s;
        *b = -a1 * s + a2 * c;
      }
  __syncthreads();
  if (k == 0)
    for (int j = tid; j < n; j += kDcT) indexq[j] = j + 1;
}

// The gathers of _dcdeflate! (393-421): the merge's columns of Q in column-type order into
// [Q2_1 Q2_2] (rows 1:n1 of types 1, 2), [Q2_3 Q2_4] (rows n1+1:n of types 2, 3) and Q2_5 (all
// rows of the deflated type 4), and z <- d in that order; for a trivial merge (every z
// negligible) the columns in sorted order into the scratch.  One warp per column, lanes
// over rows, all merges of the level at once.
constexpr int kDcGW = 8;  // warps (columns) per CTA of the gather / place kernels
__global__ void __launch_bounds__(32 * kDcGW) k_dc_gather(const DcMerge* __restrict__ mg,
                                                          const DcInfo* __restrict__ info, const double* __restrict__ dg,
                                                          const double* __restrict__ Q, long long ld,
                                                          const int* __restrict__ indexg, double* zg, double* Q2) {
  const DcMerge M = mg[blockIdx.x];
  const DcInfo I = info[blockIdx.x];
  const int n = M.n, n1 = M.n1, n2 = n - n1, lane = threadIdx.x & 31;
  const int i = blockIdx.y * kDcGW + (threadIdx.x >> 5);
  if (i >= n) return;
  const double* Qb = Q + M.off + (size_t)M.off * ld;
  double* W2 = Q2 + M.qoff;
  const int js = clamp1(indexg[M.off + i], n) - 1;
  const double* src = Qb + (size_t)js * ld;
  if (I.trivial) {
    for (int r = lane; r < n; r += 32) W2[r + (size_t)i * n] = src[r];
    return;
  }
  const int c1 = I.c1, c2 = I.c2, c3 = I.c3, k = I.k;
  double* Q12 = W2;
  double* Q34 = W2 + (size_t)n1 * n1;
  double* Q5 = Q34 + (size_t)n2 * n2;
  if (i < c1 + c2) {
    for (int r = lane; r < n1; r += 32) Q12[r + (size_t)i * n1] = src[r];
    if (i >= c1)
      for (int r = lane; r < n2; r += 32) Q34[r + (size_t)(i - c1) * n2] = src[n1 + r];
  } else if (i < c1 + c2 + c3) {
    for (int r = lane; r < n2; r += 32) Q34[r + (size_t)(i - c1) * n2] = src[n1 + r];
  } else {
    for (int r = lane; r < n; r += 32) Q5[r + (size_t)(i - k) * n] = src[r];
  }
  if (lane == 0) zg[M.off + i] = dg[M.off + js];
}

// The deflated columns and values to the end of the merge's block (_dcdeflate! 415-421);
// for a trivial merge the sorted columns back into Q.
__global__ void __launch_bounds__(32 * kDcGW) k_dc_place(const DcMerge* __restrict__ mg,
                                                         const DcInfo* __restrict__ info, double* dg, double* Q,
                                                         long long ld, const double* __restrict__ zg,
                                                         const double* __restrict__ Q2) {
  const DcMerge M = mg[blockIdx.x];
  const DcInfo I = info[blockIdx.x];
  const int n = M.n, n1 = M.n1, n2 = n - n1, lane = threadIdx.x & 31;
  const int j = blockIdx.y * kDcGW + (threadIdx.x >> 5);
  double* Qb = Q + M.off + (size_t)M.off * ld;
  const double* W2 = Q2 + M.qoff;
  if (I.trivial) {
    if (j >= n) return;
    for (int r = lane; r < n; r += 32) Qb[r + (size_t)j * ld] = W2[r + (size_t)j * n];
    return;
  }
  const int k = I.k;
  if (k >= n || j >= I.c4) return;
  const double* Q5 = W2 + (size_t)n1 * n1 + (size_t)n2 * n2;
  for (int r = lane; r < n; r += 32) Qb[r + (size_t)(k + j) * ld] = Q5[r + (size_t)j * n];
  if (lane == 0) dg[M.off + k + j] = zg[M.off + k + j];
}

// the secular equation's roots: d[j] and delta in column j of the merge's block of Q; one
// warp per root (kDcRW roots per CTA)
constexpr int kDcRW = 4;
__global__ void __launch_bounds__(32 * kDcRW) k_dc_secular(const DcMerge* __restrict__ mg,
                                                           const DcInfo* __restrict__ info,
                                                           const double* __restrict__ lam,
                                                           const double* __restrict__ w, double* d, double* Q,
                                                           long long ld, int* status) {
  const DcMerge M = mg[blockIdx.x];
  const DcInfo I = info[blockIdx.x];
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.y * kDcRW + (threadIdx.x >> 5);
  if (j >= I.k) return;
  const int o = M.off;
  bool conv = true;
  const double lamj = dc_root_warp(I.k, j + 1, lam + o, w + o, Q + o + (size_t)(o + j) * ld, I.rho, &conv, lane);
  if (lane == 0) {
    d[o + j] = lamj;
    if (!conv) atomicOr(status, 1);
  }
}

// w[i] = sign(w0[i]) sqrt(-Q[i,i] prod_{j != i} Q[i,j] / (lam[i] - lam[j])) for k >= 3
// (_dcsecular! 451-462)
__global__ void __launch_bounds__(128) k_dc_lowner(const DcMerge* __restrict__ mg, const DcInfo* __restrict__ info,
                                                   const double* __restrict__ lam, const double* __restrict__ w,
                                                   double* w2, const double* __restrict__ Q, long long ld) {
  const DcMerge M = mg[blockIdx.x];
  const DcInfo I = info[blockIdx.x];
  const int i = blockIdx.y * 128 + threadIdx.x, k = I.k, o = M.off;
  if (k < 3 || i >= k) return;
  const double* Qb = Q + o + (size_t)o * ld;
  const double li = lam[o + i];
  double v = Qb[i + (size_t)i * ld];
  for (int j = 0; j < k; ++j)
    if (j != i) v = v * (Qb[i + (size_t)j * ld] / (li - lam[o + j]));
  const double s0 = w[o + i];
  const double sg = s0 > 0 ? 1.0 : (s0 < 0 ? -1.0 : 0.0);
  w2[o + i] = sg * sqrt(-v);
}

// The rank-one problem's eigenvectors, rows in column-type order: S (k x k) (_dcsecular!
// 441-472)
__global__ void __launch_bounds__(128) k_dc_vecs(const DcMerge* __restrict__ mg, const DcInfo* __restrict__ info,
                                                 const double* __restrict__ w2, const int* __restrict__ indexc,
                                                 const double* __restrict__ Q, long long ld, double* Sg) {
  const DcMerge M = mg[blockIdx.x];
  const DcInfo I = info[blockIdx.x];
  const int j = blockIdx.y * 128 + threadIdx.x, k = I.k, o = M.off;
  if (j >= k) return;
  const double* q = Q + o + (size_t)(o + j) * ld;
  double* S = Sg + M.soff + (size_t)j * k;
  if (k == 1) {
    S[0] = q[0];
    return;
  }
  if (k == 2) {
    const double ww[2] = {q[0], q[1]};
    S[0] = ww[clamp1(indexc[o], 2) - 1];
    S[1] = ww[clamp1(indexc[o + 1], 2) - 1];
    return;
  }
  double sc = 0.0, ss = 1.0;
  for (int r = 0; r < k; ++r) {
    const double a = fabs(w2[o + r] / q[r]);
    if (a > 0) {
      if (sc < a) {
        ss = 1.0 + ss * (sc / a) * (sc / a);
        sc = a;
      } else {
        ss += (a / sc) * (a / sc);
      }
    }
  }
  const double t = sc * sqrt(ss);
  for (int r = 0; r < k; ++r) {
    const int ic = clamp1(indexc[o + r], k) - 1;
    S[r] = (w2[o + ic] / q[ic]) / t;
  }
}

// Q[:, 1:k] = [Q2_1 Q2_2; Q2_3 Q2_4] S for the small merges of a level (k > 0, n <= maxn),
// one thread per output entry
__global__ void __launch_bounds__(256) k_dc_gemm_small(const DcMerge* __restrict__ mg, const DcInfo* __restrict__ info,
                                                       const double* __restrict__ Q2, const double* __restrict__ Sg,
                                                       double* Q, long long ld, int maxn) {
  const DcMerge M = mg[blockIdx.x];
  const DcInfo I = info[blockIdx.x];
  const int n = M.n, n1 = M.n1, n2 = n - n1, k = I.k;
  if (k == 0 || n > maxn) return;
  const long long e = (long long)blockIdx.y * 256 + threadIdx.x;
  if (e >= (long long)n * k) return;
  const int r = (int)(e % n), j = (int)(e / n);
  const double* S = Sg + M.soff + (size_t)j * k;
  const double* Q12 = Q2 + M.qoff;
  const double* Q34 = Q12 + (size_t)n1 * n1;
  double acc = 0.0;
  if (r < n1) {
    for (int q = 0; q < I.c1 + I.c2; ++q) acc = fma(Q12[r + (size_t)q * n1], S[q], acc);
  } else {
    for (int q = 0; q < I.c2 + I.c3; ++q) acc = fma(Q34[(r - n1) + (size_t)q * n2], S[I.c1 + q], acc);
  }
  Q[(M.off + r) + (size_t)(M.off + j) * ld] = acc;
}

__global__ void k_dc_zero(double* C, int rows, int cols, long long ldc) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)rows * cols) return;
  C[(e % rows) + (size_t)(e / rows) * ldc] = 0.0;
}

// C (rows x cols, ldc) = A (rows x q, lda) B (q x cols, ldb), one thread per entry
__global__ void k_dc_gemm_plain(int rows, int cols, int q, const double* __restrict__ A, long long lda,
                                const double* __restrict__ B, long long ldb, double* C, long long ldc) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)rows * cols) return;
  const int r = (int)(e % rows), j = (int)(e / rows);
  double acc = 0.0;
  for (int t = 0; t < q; ++t) acc = fma(A[r + (size_t)t * lda], B[t + (size_t)j * ldb], acc);
  C[r + (size_t)j * ldc] = acc;
}

__global__ void k_dc_or_err(int* status, const int* err) {
  if (*err) atomicOr(status, 4);
}

// ---- workspace ------------------------------------------------------------------------------
struct DcWs {
  double *Qc, *Zt, *Q2, *S, *z, *lam, *w, *w2, *rc, *rs, *orgnrm, *sc, *ss, *st;
  int *indexq, *indexc, *index, *indexp, *coltype, *rp, *rn, *brk, *ioff, *imsz, *cuts, *status, *sf, *sprev;
  DcMerge* mg;
  DcInfo* info;
  char* gemm;
  size_t bytes;
};

DcWs dc_ws(int n, int zcplx, char* base) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    off = (off + 255) & ~size_t(255);
    const size_t at = off;
    off += bytes;
    return base ? base + at : nullptr;
  };
  const size_t nn = (size_t)n * n, D = sizeof(double), I = sizeof(int);
  DcWs W;
  W.Qc = (double*)take(nn * D);
  W.Zt = (double*)take(nn * D * (zcplx ? 2 : 1));
  W.Q2 = (double*)take(2 * nn * D);
  W.S = (double*)take(nn * D);
  W.z = (double*)take(n * D);
  W.lam = (double*)take(n * D);
  W.w = (double*)take(n * D);
  W.w2 = (double*)take(n * D);
  W.rc = (double*)take(n * D);
  W.rs = (double*)take(n * D);
  W.orgnrm = (double*)take(D);
  W.sc = (double*)take(n * D);
  W.ss = (double*)take(n * D);
  W.st = (double*)take(n * D);
  W.sf = (int*)take(n * I);
  W.sprev = (int*)take(n * I);
  W.indexq = (int*)take(n * I);
  W.indexc = (int*)take(n * I);
  W.index = (int*)take(n * I);
  W.indexp = (int*)take(n * I);
  W.coltype = (int*)take(n * I);
  W.rp = (int*)take(n * I);
  W.rn = (int*)take(n * I);
  W.brk = (int*)take(n * I);
  W.ioff = (int*)take(n * I);
  W.imsz = (int*)take(n * I);
  W.cuts = (int*)take(n * I);
  W.status = (int*)take(4 * I);
  W.mg = (DcMerge*)take((n / 2 + 2) * sizeof(DcMerge));
  W.info = (DcInfo*)take((n / 2 + 2) * sizeof(DcInfo));
  W.gemm = take(gemm_tc_ws_bytes(2 * n, n, n));
  W.bytes = off;
  return W;
}

#define DC_CK(x)                                   \
  do {                                             \
    const cudaError_t e_ = (x);                    \
    if (e_ != cudaSuccess) return e_;              \
  } while (0)

int blocks_for(long long work, int nt) { return (int)std::max<long long>(1, (work + nt - 1) / nt); }

// C = A B with the tensor-core FP64 product when large, the plain kernel otherwise
cudaError_t dc_gemm(int rows, int cols, int q, const double* A, long long lda, const double* B, long long ldb,
                    double* C, long long ldc, const DcWs& W, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  if (q <= 0) {
    k_dc_zero<<<blocks_for((long long)rows * cols, 256), 256, 0, s>>>(C, rows, cols, ldc);
    return cudaGetLastError();
  }
  if ((double)rows * cols * q < 4.0e6) {
    k_dc_gemm_plain<<<blocks_for((long long)rows * cols, 256), 256, 0, s>>>(rows, cols, q, A, lda, B, ldb, C, ldc);
    return cudaGetLastError();
  }
  int* err = gemm_tc_err_word(rows, cols, q, W.gemm);
  DC_CK(cudaMemsetAsync(err, 0, sizeof(int), s));
  DC_CK(launch_gemm_tc(rows, cols, q, A, (int)lda, 0, B, (int)ldb, C, (int)ldc, W.gemm, s));
  k_dc_or_err<<<1, 1, 0, s>>>(W.status, err);
  return cudaGetLastError();
}

// _dcschur_core! (107-196) on d, e (m), Qc (m x m, ld m)
cudaError_t dc_core(int m, double* d, double* e, const DcWs& W, int num_sms, cudaStream_t s) {
  (void)num_sms;
  std::vector<int> itree(1, m);
  int nsub = 1;
  while (itree[nsub - 1] > kDcQrMax) {
    itree.resize(2 * nsub);
    for (int j = nsub; j >= 1; --j) {
      itree[2 * j - 1] = itree[j - 1] >> 1;
      itree[2 * j - 2] = (itree[j - 1] + 1) >> 1;
    }
    nsub *= 2;
  }
  for (int j = 2; j <= nsub; ++j) itree[j - 1] += itree[j - 2];
  // rank-one cuts and leaves
  std::vector<int> cuts, loff(nsub), lmsz(nsub), iq(m);
  for (int i = 1; i <= nsub - 1; ++i) cuts.push_back(itree[i - 1] - 1);
  int maxm = 0;
  for (int i = 0; i < nsub; ++i) {
    loff[i] = i == 0 ? 0 : itree[i - 1];
    lmsz[i] = i == 0 ? itree[0] : itree[i] - itree[i - 1];
    maxm = std::max(maxm, lmsz[i]);
    for (int j = 0; j < lmsz[i]; ++j) iq[loff[i] + j] = j + 1;
  }
  DC_CK(cudaMemsetAsync(W.Qc, 0, sizeof(double) * (size_t)m * m, s));
  if (!cuts.empty()) {
    DC_CK(cudaMemcpyAsync(W.cuts, cuts.data(), sizeof(int) * cuts.size(), cudaMemcpyHostToDevice, s));
    k_dc_cuts<<<blocks_for((long long)cuts.size(), 128), 128, 0, s>>>((int)cuts.size(), W.cuts, d, e);
    DC_CK(cudaGetLastError());
  }
  DC_CK(cudaMemcpyAsync(W.ioff, loff.data(), sizeof(int) * nsub, cudaMemcpyHostToDevice, s));
  DC_CK(cudaMemcpyAsync(W.imsz, lmsz.data(), sizeof(int) * nsub, cudaMemcpyHostToDevice, s));
  DC_CK(cudaMemcpyAsync(W.indexq, iq.data(), sizeof(int) * m, cudaMemcpyHostToDevice, s));
  DC_CK(launch_steqr_leaves(nsub, W.ioff, W.imsz, maxm, d, e, W.Qc, m, 1, W.status, s));
  // merge up the tree
  std::vector<DcMerge> mg;
  std::vector<DcInfo> info;
  while (nsub > 1) {
    mg.clear();
    long long qoff = 0, soff = 0;
    int nmax = 0;
    for (int i = 0; i <= nsub - 2; i += 2) {
      DcMerge M{};
      if (i == 0) {
        M.off = 0;
        M.n = itree[1];
        M.n1 = itree[0];
      } else {
        M.off = itree[i - 1];
        M.n = itree[i + 1] - itree[i - 1];
        M.n1 = (M.n + 1) >> 1;
      }
      M.qoff = qoff;
      M.soff = soff;
      qoff += 2LL * M.n * M.n;
      soff += (long long)M.n * M.n;
      nmax = std::max(nmax, M.n);
      mg.push_back(M);
      itree[(i >> 1)] = itree[i + 1];
    }
    const int nm = (int)mg.size();
    DC_CK(cudaMemcpyAsync(W.mg, mg.data(), sizeof(DcMerge) * nm, cudaMemcpyHostToDevice, s));
    k_dc_prep<<<nm, 256, 0, s>>>(W.mg, W.info, e, d, W.Qc, m, W.indexq, W.z, W.lam);
    DC_CK(cudaGetLastError());
    const dim3 gr(nm, (nmax + 255) / 256);
    k_dc_rank<<<gr, 256, 0, s>>>(W.mg, W.info, W.lam, W.indexc, 0);
    DC_CK(cudaGetLastError());
    k_dc_deflate<<<nm, kDcT, 0, s>>>(W.mg, W.info, d, W.Qc, m, W.indexq, W.z, W.lam, W.w, W.indexc, W.index, W.indexp,
                                     W.coltype, W.rp, W.rn, W.rc, W.rs, W.Q2, W.sf, W.sprev, W.sc, W.ss, W.st);
    DC_CK(cudaGetLastError());
    const dim3 gg(nm, (nmax + kDcGW - 1) / kDcGW);
    k_dc_gather<<<gg, 32 * kDcGW, 0, s>>>(W.mg, W.info, d, W.Qc, m, W.index, W.z, W.Q2);
    k_dc_place<<<gg, 32 * kDcGW, 0, s>>>(W.mg, W.info, d, W.Qc, m, W.z, W.Q2);
    DC_CK(cudaGetLastError());
    info.resize(nm);
    DC_CK(cudaMemcpyAsync(info.data(), W.info, sizeof(DcInfo) * nm, cudaMemcpyDeviceToHost, s));
    DC_CK(cudaStreamSynchronize(s));
    int kmax = 0;
    for (const DcInfo& I : info) kmax = std::max(kmax, I.k);
    if (kmax > 0) {
      const dim3 gk(nm, (kmax + 127) / 128);
      k_dc_secular<<<dim3(nm, (kmax + kDcRW - 1) / kDcRW), 32 * kDcRW, 0, s>>>(W.mg, W.info, W.lam, W.w, d, W.Qc,
                                                                                  m, W.status);
      k_dc_lowner<<<gk, 128, 0, s>>>(W.mg, W.info, W.lam, W.w, W.w2, W.Qc, m);
      k_dc_vecs<<<gk, 128, 0, s>>>(W.mg, W.info, W.w2, W.indexc, W.Qc, m, W.S);
      DC_CK(cudaGetLastError());
      long long small_work = 0;
      for (int q = 0; q < nm; ++q)
        if (mg[q].n <= kDcSmall) small_work = std::max(small_work, (long long)mg[q].n * info[q].k);
      if (small_work > 0) {
        k_dc_gemm_small<<<dim3(nm, (unsigned)((small_work + 255) / 256)), 256, 0, s>>>(W.mg, W.info, W.Q2, W.S, W.Qc,
                                                                                        m, kDcSmall);
        DC_CK(cudaGetLastError());
      }
      for (int q = 0; q < nm; ++q) {
        const DcMerge& M = mg[q];
        const DcInfo& I = info[q];
        if (M.n <= kDcSmall || I.k == 0) continue;
        const int n1 = M.n1, n2 = M.n - M.n1;
        double* Qb = W.Qc + M.off + (size_t)M.off * m;
        const double* Q12 = W.Q2 + M.qoff;
        const double* Q34 = Q12 + (size_t)n1 * n1;
        const double* S = W.S + M.soff;
        DC_CK(dc_gemm(n2, I.k, I.c2 + I.c3, Q34, n2, S + I.c1, I.k, Qb + n1, m, W, s));
        DC_CK(dc_gemm(n1, I.k, I.c1 + I.c2, Q12, n1, S, I.k, Qb, m, W, s));
      }
      k_dc_rank<<<gr, 256, 0, s>>>(W.mg, W.info, d, W.indexq, 1);
      DC_CK(cudaGetLastError());
    }
    nsub >>= 1;
  }
  return cudaSuccess;
}

}  // namespace

size_t stedc_ws_bytes(int n, int zcplx) { return dc_ws(std::max(n, 1), zcplx, nullptr).bytes + 256; }

cudaError_t run_stedc(int n, double* d, double* e, double* Z, long long ldz, int zcplx, char* ws, int num_sms,
                      cudaStream_t s, int* status) {
  *status = 0;
  if (n == 0) return cudaSuccess;
  const DcWs W = dc_ws(n, zcplx, ws);
  DC_CK(cudaMemsetAsync(W.status, 0, 4 * sizeof(int), s));
  if (n == 1) {
    if (Z) {
      const double one[2] = {1.0, 0.0};
      DC_CK(cudaMemcpyAsync(Z, one, zcplx ? 2 * sizeof(double) : sizeof(double), cudaMemcpyHostToDevice, s));
      DC_CK(cudaStreamSynchronize(s));
    }
    return cudaSuccess;
  }
  const int rmul = zcplx ? 2 : 1;  // a complex Z times a real matrix: its interleaved real view
  auto update_z = [&](int c0, int mb) -> cudaError_t {
    if (!Z) return cudaSuccess;
    double* Zc = Z + (size_t)rmul * c0 * ldz;
    DC_CK(cudaMemcpy2DAsync(W.Zt, sizeof(double) * rmul * n, Zc, sizeof(double) * rmul * ldz, sizeof(double) * rmul * n,
                            mb, cudaMemcpyDeviceToDevice, s));
    return dc_gemm(rmul * n, mb, mb, W.Zt, (long long)rmul * n, W.Qc, mb, Zc, (long long)rmul * ldz, W, s);
  };
  if (n <= kDcQrMax) {
    // the whole problem by the QR iteration on Qc, then Z = Z Qc
    const int zero = 0;
    DC_CK(cudaMemcpyAsync(W.ioff, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
    DC_CK(cudaMemcpyAsync(W.imsz, &n, sizeof(int), cudaMemcpyHostToDevice, s));
    DC_CK(launch_steqr_leaves(1, W.ioff, W.imsz, n, d, e, W.Qc, n, Z ? 1 : 0, W.status, s));
    DC_CK(update_z(0, n));
  } else {
    k_dc_split<<<blocks_for(n, 256), 256, 0, s>>>(n, d, e, W.brk);
    DC_CK(cudaGetLastError());
    std::vector<int> brk(n - 1);
    DC_CK(cudaMemcpyAsync(brk.data(), W.brk, sizeof(int) * (n - 1), cudaMemcpyDeviceToHost, s));
    DC_CK(cudaStreamSynchronize(s));
    int istart = 0;
    while (istart < n) {
      int ifinish = istart;
      while (ifinish < n - 1 && !brk[ifinish]) ++ifinish;
      const int mb = ifinish - istart + 1;
      if (mb > 1) {
        double* dv = d + istart;
        double* ev = e + istart;
        if (mb > kDcQrMax) {
          k_dc_scale<<<1, 1024, 0, s>>>(dv, ev, mb, W.orgnrm);
          DC_CK(cudaGetLastError());
          DC_CK(dc_core(mb, dv, ev, W, num_sms, s));
          DC_CK(update_z(istart, mb));
          k_dc_unscale<<<blocks_for(mb, 256), 256, 0, s>>>(dv, mb, W.orgnrm);
          DC_CK(cudaGetLastError());
        } else {
          const int zero = 0;
          DC_CK(cudaMemcpyAsync(W.ioff, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
          DC_CK(cudaMemcpyAsync(W.imsz, &mb, sizeof(int), cudaMemcpyHostToDevice, s));
          DC_CK(launch_steqr_leaves(1, W.ioff, W.imsz, mb, dv, ev, W.Qc, mb, Z ? 1 : 0, W.status, s));
          DC_CK(update_z(istart, mb));
        }
        // the host values above are read by the copies before the next block reuses them
        DC_CK(cudaStreamSynchronize(s));
      }
      istart = ifinish + 1;
    }
  }
  DC_CK(cudaMemcpyAsync(status, W.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  DC_CK(cudaStreamSynchronize(s));
  return cudaSuccess;
}

}  // namespace gsk
