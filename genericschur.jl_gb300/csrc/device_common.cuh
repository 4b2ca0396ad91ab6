// Device helpers shared by the Schur kernels: IEEE constants, the small
// Householder reflectors used by the Francis sweeps, and the standard-form 2x2
// Schur block.  Everything here runs in FP64 on the CUDA cores (sm_103a has no
// FP64 tensor-core MMA kind that would be faster than DFMA on this part).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gsk {

constexpr double kEps = 2.220446049250313e-16;       // eps(Float64) = 2^-52
constexpr double kFmin = 2.2250738585072014e-308;    // floatmin(Float64)
constexpr double kSafemin = 2.2250738585072014e-308; // safemin(Float64) (util.jl:5-12)

// Block reductions over the whole CTA.  `red` is shared scratch of >= 32 entries.
template <int NT, class V>
__device__ __forceinline__ V block_max(V v, V* red) {
  for (int o = 16; o > 0; o >>= 1) {
    V w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v || w != w) ? w : v;
  }
  if constexpr (NT > 32) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    v = red[0];
#pragma unroll
    for (int i = 1; i < NT / 32; ++i) {
      V w = red[i];
      v = (w > v || w != w) ? w : v;
    }
    __syncthreads();
  }
  return v;
}

template <int NT, class V>
__device__ __forceinline__ V block_sum(V v, V* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if constexpr (NT > 32) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    v = red[0];
#pragma unroll
    for (int i = 1; i < NT / 32; ++i) v += red[i];
    __syncthreads();
  }
  return v;
}

// safescale! multiplier sequence (util.jl:41-80, kept as written there): fills
// mul[0..k) with the factors to apply in order and returns k (at most 8).
__device__ inline int safescale_factors(double cfrom, double cto, double* mul) {
  const double smlnum = kSafemin;
  const double bignum = 1.0 / smlnum;
  double cfromc = cfrom, ctoc = cto;
  int k = 0;
  bool done = false;
  while (!done && k < 8) {
    double cfrom1 = cfromc * smlnum;
    double m;
    if (cfrom1 == cfromc) {
      m = ctoc / cfromc; done = true;
    } else {
      double cto1 = ctoc / bignum;
      if (cto1 == ctoc) {
        m = cto; done = true; cfromc = 1.0;
      } else if (fabs(cfrom1) > fabs(ctoc) && ctoc != 0.0) {
        m = smlnum; done = false; cfromc = 1.0;
      } else if (fabs(cto1) > fabs(cfromc)) {
        m = bignum; done = false; cfromc = cfrom1;
      } else {
        m = ctoc / cfromc; done = true;
      }
    }
    mul[k++] = m;
  }
  return k;
}

// Real Householder reflector of length 2 or 3 (householder.jl:12-54 semantics):
// given x = (alpha, x1[, x2]) returns tau and overwrites x with (beta, v1[, v2]).
// The 2-norm uses one square root when all entries lie in a range where squaring
// cannot over/underflow, and falls back to the scaled form otherwise.
__device__ __forceinline__ double reflector_small(double& a, double& x1, double& x2, int nr) {
  if (nr <= 1) return 0.0;
  const double ax1 = fabs(x1), ax2 = (nr == 3) ? fabs(x2) : 0.0;
  if (ax1 == 0.0 && ax2 == 0.0) return 0.0;
  const double aa = fabs(a);
  const double big = fmax(aa, fmax(ax1, ax2));
  double beta;
  if (big < 1.0e150 && big > 1.0e-150) {
    beta = sqrt(fma(a, a, fma(x1, x1, x2 * x2)));
  } else {
    const double r = 1.0 / big;
    const double sa = a * r, s1 = x1 * r, s2 = x2 * r;
    beta = big * sqrt(fma(sa, sa, fma(s1, s1, s2 * s2)));
  }
  const double sfmin = 2.0 * kFmin / kEps;
  beta = -copysign(beta, a);
  int kount = 0;
  if (fabs(beta) < sfmin) {
    // underflow-guard rescaling loop (householder.jl:25-42)
    const double rsfmin = 1.0 / sfmin;
    double al = a;
    do {
      ++kount;
      x1 *= rsfmin; x2 *= rsfmin; beta *= rsfmin; al *= rsfmin;
    } while (fabs(beta) < sfmin && kount < 20);
    a = al;
    beta = -copysign(sqrt(fma(a, a, fma(x1, x1, x2 * x2))), a);
  }
  const double rb = 1.0 / beta;
  const double t = 1.0 / (a - beta);
  const double tau = (beta - a) * rb;
  x1 *= t;
  x2 *= t;
  for (int j = 0; j < kount; ++j) beta *= sfmin;
  a = beta;
  return tau;
}

// Standard-form 2x2 real Schur block (dlanv2 logic, GenericSchur.jl:716-803).
__device__ inline void gs2x2(double& a, double& b, double& c, double& d, double& cs, double& sn,
                             double& w1r, double& w1i, double& w2r, double& w2i) {
  auto sgn = [](double x) { return (x < 0.0) ? -1.0 : 1.0; };
  const double half = 0.5;
  const double small = 4.0 * kEps;
  if (c == 0.0) {
    cs = 1.0; sn = 0.0;
  } else if (b == 0.0) {
    cs = 0.0; sn = 1.0;
    double ta = a; a = d; b = -c; c = 0.0; d = ta;
  } else if ((a - d) == 0.0 && (b * c < 0.0)) {
    cs = 1.0; sn = 0.0;
  } else {
    double asubd = a - d;
    double p = half * asubd;
    double bcmax = fmax(fabs(b), fabs(c));
    double bcmis = fmin(fabs(b), fabs(c)) * sgn(b) * sgn(c);
    double scale = fmax(fabs(p), bcmax);
    double z = (p / scale) * p + (bcmax / scale) * bcmis;
    if (z >= small) {
      z = p + sqrt(scale) * sqrt(z) * sgn(p);
      a = d + z;
      d -= (bcmax / z) * bcmis;
      double tau = hypot(c, z);
      cs = z / tau;
      sn = c / tau;
      b -= c;
      c = 0.0;
    } else {
      double sigma = b + c;
      double tau = hypot(sigma, asubd);
      cs = sqrt(half * (1.0 + fabs(sigma) / tau));
      sn = -(p / (tau * cs)) * sgn(sigma);
      double aa = a * cs + b * sn;
      double bb = -a * sn + b * cs;
      double cc = c * cs + d * sn;
      double dd = -c * sn + d * cs;
      a = aa * cs + cc * sn;
      b = bb * cs + dd * sn;
      c = -aa * sn + cc * cs;
      d = -bb * sn + dd * cs;
      double midad = half * (a + d);
      a = midad;
      d = a;
      if (c != 0.0) {
        if (b != 0.0) {
          if (b * c >= 0.0) {
            double sab = sqrt(fabs(b));
            double sac = sqrt(fabs(c));
            p = sab * sac * sgn(c);
            tau = 1.0 / sqrt(fabs(b + c));
            a = midad + p;
            d = midad - p;
            b -= c;
            c = 0.0;
            double cs1 = sab * tau;
            double sn1 = sac * tau;
            double ncs = cs * cs1 - sn * sn1;
            double nsn = cs * sn1 + sn * cs1;
            cs = ncs; sn = nsn;
          }
        } else {
          b = -c; c = 0.0;
          double ncs = -sn, nsn = cs;
          cs = ncs; sn = nsn;
        }
      }
    }
  }
  if (c == 0.0) {
    w1r = a; w1i = 0.0; w2r = d; w2i = 0.0;
  } else {
    double rti = sqrt(fabs(b)) * sqrt(fabs(c));
    w1r = a; w1i = rti; w2r = d; w2i = -rti;
  }
}

}  // namespace gsk

namespace gsk {
// LinearAlgebra.givensAlgorithm (LAPACK 3.x dlartg): safmn2 = 2^-485, safmx2 = 2^485.
__device__ inline void givens_alg(double f, double g, double& cs, double& sn, double& r) {
  const double mn2 = 0x1p-485, mx2 = 0x1p485;
  if (g == 0.0) { cs = 1.0; sn = 0.0; r = f; return; }
  if (f == 0.0) { cs = 0.0; sn = 1.0; r = g; return; }
  double f1 = f, g1 = g, scale = fmax(fabs(f1), fabs(g1));
  double rr;
  if (scale >= mx2) {
    int count = 0;
    do { ++count; f1 *= mn2; g1 *= mn2; scale = fmax(fabs(f1), fabs(g1)); } while (!(scale < mx2 || count >= 20));
    rr = sqrt(f1 * f1 + g1 * g1);
    cs = f1 / rr; sn = g1 / rr;
    for (int q = 0; q < count; ++q) rr *= mx2;
  } else if (scale <= mn2) {
    int count = 0;
    do { ++count; f1 *= mx2; g1 *= mx2; scale = fmax(fabs(f1), fabs(g1)); } while (!(scale > mn2) && count < 40);
    rr = sqrt(f1 * f1 + g1 * g1);
    cs = f1 / rr; sn = g1 / rr;
    for (int q = 0; q < count; ++q) rr *= mn2;
  } else {
    rr = sqrt(f1 * f1 + g1 * g1);
    cs = f1 / rr; sn = g1 / rr;
  }
  if (fabs(f) > fabs(g) && cs < 0.0) { cs = -cs; sn = -sn; rr = -rr; }
  r = rr;
}

}  // namespace gsk

// ---- complex FP64 helpers (double2 = (re, im)) -------------------------------
namespace gsk {
__device__ __forceinline__ double2 zmk(double r, double i) { return make_double2(r, i); }
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zneg(double2 a) { return make_double2(-a.x, -a.y); }
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 zscal(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// a + b * c
__device__ __forceinline__ double2 zfma(double2 b, double2 c, double2 a) {
  return make_double2(fma(b.x, c.x, fma(-b.y, c.y, a.x)), fma(b.x, c.y, fma(b.y, c.x, a.y)));
}
// a - b * c
__device__ __forceinline__ double2 zfms(double2 b, double2 c, double2 a) {
  return make_double2(fma(-b.x, c.x, fma(b.y, c.y, a.x)), fma(-b.x, c.y, fma(-b.y, c.x, a.y)));
}
// a + conj(b) * c
__device__ __forceinline__ double2 zfmac(double2 b, double2 c, double2 a) {
  return make_double2(fma(b.x, c.x, fma(b.y, c.y, a.x)), fma(b.x, c.y, fma(-b.y, c.x, a.y)));
}
__device__ __forceinline__ double zabs1(double2 a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ double zabs(double2 a) { return hypot(a.x, a.y); }
// Smith's complex division
__device__ inline double2 zdiv(double2 a, double2 b) {
  if (fabs(b.y) <= fabs(b.x)) {
    const double r = b.y / b.x, d = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  const double r = b.x / b.y, d = b.y + b.x * r;
  return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
// principal square root
__device__ inline double2 zsqrt(double2 z) {
  const double x = z.x, y = z.y;
  if (x == 0.0 && y == 0.0) return make_double2(0.0, y);
  const double t = sqrt((fabs(x) + hypot(x, y)) * 0.5);
  if (x >= 0.0) return make_double2(t, y / (2.0 * t));
  return make_double2(fabs(y) / (2.0 * t), copysign(t, y));
}
// 2-element complex reflector (householder.jl:56-102 for length 2): returns tau,
// overwrites (a, x1) with (beta, v1); beta is real.
__device__ inline double2 zreflector2(double2& a, double2& x1) {
  const double xnorm = hypot(x1.x, x1.y);
  if (xnorm == 0.0 && a.y == 0.0) return make_double2(0.0, 0.0);
  const double big = fmax(fmax(fabs(a.x), fabs(a.y)), xnorm);
  double beta;
  if (big < 1.0e150 && big > 1.0e-150) {
    beta = sqrt(fma(a.x, a.x, fma(a.y, a.y, xnorm * xnorm)));
  } else {
    const double r = 1.0 / big, p = a.x * r, q = a.y * r, s = xnorm * r;
    beta = big * sqrt(fma(p, p, fma(q, q, s * s)));
  }
  beta = -copysign(beta, a.x);
  const double sfmin = kFmin / kEps;
  int kount = 0;
  if (fabs(beta) < sfmin) {
    const double rsfmin = 1.0 / sfmin;
    do {
      ++kount;
      x1 = zscal(x1, rsfmin); beta *= rsfmin; a = zscal(a, rsfmin);
    } while (fabs(beta) < sfmin && kount < 20);
    const double xn = hypot(x1.x, x1.y);
    beta = -copysign(sqrt(fma(a.x, a.x, fma(a.y, a.y, xn * xn))), a.x);
  }
  const double2 tau = make_double2((beta - a.x) / beta, -a.y / beta);
  const double2 t = zdiv(make_double2(1.0, 0.0), make_double2(a.x - beta, a.y));
  x1 = zmul(x1, t);
  for (int j = 0; j < kount; ++j) beta *= sfmin;
  a = make_double2(beta, 0.0);
  return tau;
}
}  // namespace gsk

// ---- Newton-refined reciprocal and reciprocal square root ---------------------
// Each FP64 instruction costs a full warp slot of the FP64 pipe on this part, so
// the serial reflector math of the bulge chase is built from the hardware's
// approximate seeds (rsqrt.approx / rcp.approx, ~23 correct bits) refined by two
// Newton-Raphson steps each: y <- y + y (1 - s y^2) / 2 and r <- r + r (1 - d r),
// which square the relative error per step (23 -> 46 -> past 53 bits).  Inputs are
// kept inside [1e-290, 1e290] by the callers; extreme values take the scaled path.
namespace gsk {
__device__ __forceinline__ double rsqrt_nr(double s) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(s));
  double h = s * y;
  double e = fma(-h, y, 1.0);
  y = fma(0.5 * y, e, y);
  h = s * y;
  e = fma(-h, y, 1.0);
  return fma(0.5 * y, e, y);
}
__device__ __forceinline__ double rcp_nr(double d) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}

// Real reflector of length 2 or 3 (householder.jl:12-54) in ~20 FP64 instructions:
// with s = ||(a, x1, x2)||, beta = -sign(a) s, tau = (beta - a)/beta = 1 + |a|/s and
// 1/(a - beta) = sign(a)/(|a| + s).  Falls back to reflector_small outside the safe
// range.  Returns tau; (a, x1, x2) <- (beta, v1, v2).
__device__ __forceinline__ double reflector_fast(double& a, double& x1, double& x2, int nr) {
  if (nr < 3) x2 = 0.0;
  const double xs = fma(x1, x1, x2 * x2);
  if (xs == 0.0) return 0.0;
  const double ss = fma(a, a, xs);
  if (!(ss > 1.0e-290 && ss < 1.0e290)) return reflector_small(a, x1, x2, nr);
  const double y = rsqrt_nr(ss);
  const double s = ss * y;
  const double aa = fabs(a);
  const double tau = fma(aa, y, 1.0);
  const double t = copysign(rcp_nr(aa + s), a);
  x1 *= t;
  x2 *= t;
  a = -copysign(s, a);
  return tau;
}
}  // namespace gsk

namespace gsk {
// 2-element complex reflector (householder.jl:56-102) from Newton-refined seeds:
// s = ||(a, x1)||, beta = -sign(Re a) s, tau = (1 + |Re a|/s, sign(Re a) Im a / s),
// 1/(a - beta) = conj(d)/|d|^2 with d = (Re a + sign(Re a) s, Im a).  Falls back to
// zreflector2 outside the safe range.
__device__ __forceinline__ double2 zreflector2_fast(double2& a, double2& x1) {
  if (x1.x == 0.0 && x1.y == 0.0 && a.y == 0.0) return make_double2(0.0, 0.0);
  const double xs = fma(x1.x, x1.x, x1.y * x1.y);
  const double ss = fma(a.x, a.x, fma(a.y, a.y, xs));
  if (!(ss > 1.0e-290 && ss < 1.0e290)) return zreflector2(a, x1);
  const double y = rsqrt_nr(ss);
  const double s = ss * y;
  const double aa = fabs(a.x);
  const double sy = copysign(y, a.x);
  const double2 tau = make_double2(fma(aa, y, 1.0), a.y * sy);
  const double dr = a.x + copysign(s, a.x);
  const double r = rcp_nr(fma(dr, dr, a.y * a.y));
  const double2 t = make_double2(dr * r, -a.y * r);
  x1 = zmul(x1, t);
  a = make_double2(-copysign(s, a.x), 0.0);
  return tau;
}
}  // namespace gsk

namespace gsk {
// FP32 counterpart of reflector_fast for the FP32 stage of the mixed-precision form:
// the same closed form with the hardware reciprocal square root and a correctly
// rounded reciprocal; outside [1e-30, 1e30] the FP64 scaled path takes over.
__device__ __forceinline__ float reflector_fast(float& a, float& x1, float& x2, int nr) {
  if (nr < 3) x2 = 0.0f;
  if (x1 == 0.0f && x2 == 0.0f) return 0.0f;
  const float ss = fmaf(a, a, fmaf(x1, x1, x2 * x2));
  if (!(ss > 1.0e-30f && ss < 1.0e30f)) {
    double ad = a, x1d = x1, x2d = x2;
    const double t = reflector_small(ad, x1d, x2d, nr);
    a = (float)ad; x1 = (float)x1d; x2 = (float)x2d;
    return (float)t;
  }
  const float y = rsqrtf(ss);
  const float s = ss * y;
  const float aa = fabsf(a);
  const float tau = fmaf(aa, y, 1.0f);
  const float t = copysignf(__frcp_rn(aa + s), a);
  x1 *= t;
  x2 *= t;
  a = -copysignf(s, a);
  return tau;
}

// Floating-point constants of the working precision.
template <class T> struct Prec;
template <> struct Prec<double> {
  static constexpr double eps = 2.220446049250313e-16, fmin = 2.2250738585072014e-308;
  static constexpr double safe_lo = 1.0e-150, safe_hi = 1.0e150;
};
template <> struct Prec<float> {
  static constexpr float eps = 1.1920929e-07f, fmin = 1.17549435e-38f;
  static constexpr float safe_lo = 1.0e-15f, safe_hi = 1.0e15f;
};

// ---- CTA-wide helpers: 2-norm and Householder reflector of a vector in global memory ----
// Largest component magnitude (re and im separately) of x[0..m), over the CTA.
template <class S> __device__ __forceinline__ double comp_max(S v);
template <> __device__ __forceinline__ double comp_max<double>(double v) { return fabs(v); }
template <> __device__ __forceinline__ double comp_max<double2>(double2 v) { return fmax(fabs(v.x), fabs(v.y)); }
template <class S> __device__ __forceinline__ double comp_ssq(S v, double inv);
template <> __device__ __forceinline__ double comp_ssq<double>(double v, double inv) { const double a = v * inv; return a * a; }
template <> __device__ __forceinline__ double comp_ssq<double2>(double2 v, double inv) {
  const double a = v.x * inv, b = v.y * inv;
  return fma(a, a, b * b);
}

// 2-norm of x[0..m) without overflow (one CTA of NT threads).
template <class S, int NT>
__device__ double cta_norm2(const S* x, int m, double* red) {
  double mx = 0.0;
  for (int k = threadIdx.x; k < m; k += NT) mx = fmax(mx, comp_max(x[k]));
  mx = block_max<NT>(mx, red);
  if (!(mx > 0.0) || !isfinite(mx)) return mx;
  const double inv = 1.0 / mx;
  double ss = 0.0;
  for (int k = threadIdx.x; k < m; k += NT) ss += comp_ssq(x[k], inv);
  ss = block_sum<NT>(ss, red);
  return mx * sqrt(ss);
}

__device__ __forceinline__ double hypot3d(double a, double b, double c) {
  const double m = fmax(fabs(a), fmax(fabs(b), fabs(c)));
  if (!(m > 0.0) || !isfinite(m)) return m;
  const double x = a / m, y = b / m, z = c / m;
  return m * sqrt(fma(x, x, fma(y, y, z * z)));
}

// _reflector! (householder.jl:12-102) on x[0..m) by one CTA of NT threads: x[0] <- beta
// (real), the tail scaled to the essential part; returns tau.  All threads call it.
template <int NT>
__device__ double cta_reflector(double* x, int m, double* red) {
  if (m <= 1) return 0.0;
  const double sfmin = 2.0 * Prec<double>::fmin / Prec<double>::eps;
  double alpha = x[0];
  double xnorm = cta_norm2<double, NT>(x + 1, m - 1, red);
  if (xnorm == 0.0) return 0.0;
  double beta = -copysign(hypot(alpha, xnorm), alpha);
  int kount = 0;
  if (fabs(beta) < sfmin) {
    const double rs = 1.0 / sfmin;
    bool smallb = true;
    while (smallb) {
      ++kount;
      __syncthreads();
      for (int k = 1 + threadIdx.x; k < m; k += NT) x[k] *= rs;
      beta *= rs;
      alpha *= rs;
      smallb = fabs(beta) < sfmin && kount < 20;
    }
    __syncthreads();
    xnorm = cta_norm2<double, NT>(x + 1, m - 1, red);
    beta = -copysign(hypot(alpha, xnorm), alpha);
  }
  const double tau = (beta - alpha) / beta;
  const double t = 1.0 / (alpha - beta);
  __syncthreads();
  for (int k = 1 + threadIdx.x; k < m; k += NT) x[k] *= t;
  for (int j = 0; j < kount; ++j) beta *= sfmin;
  __syncthreads();
  if (threadIdx.x == 0) x[0] = beta;
  return tau;
}
template <int NT>
__device__ double2 cta_reflector(double2* x, int m, double* red) {
  if (m < 1) return make_double2(0.0, 0.0);
  const double sfmin = Prec<double>::fmin / Prec<double>::eps;
  double ar = x[0].x, ai = x[0].y;
  double xnorm = m > 1 ? cta_norm2<double2, NT>(x + 1, m - 1, red) : 0.0;
  if (xnorm == 0.0 && ai == 0.0) return make_double2(0.0, 0.0);
  double beta = -copysign(hypot3d(ar, ai, xnorm), ar);
  int kount = 0;
  if (fabs(beta) < sfmin) {
    const double rs = 1.0 / sfmin;
    bool smallb = true;
    while (smallb) {
      ++kount;
      __syncthreads();
      for (int k = 1 + threadIdx.x; k < m; k += NT) x[k] = make_double2(x[k].x * rs, x[k].y * rs);
      beta *= rs;
      ar *= rs;
      ai *= rs;
      smallb = fabs(beta) < sfmin && kount < 20;
    }
    __syncthreads();
    xnorm = m > 1 ? cta_norm2<double2, NT>(x + 1, m - 1, red) : 0.0;
    beta = -copysign(hypot3d(ar, ai, xnorm), ar);
  }
  const double2 tau = make_double2((beta - ar) / beta, -ai / beta);
  const double2 t = zdiv(make_double2(1.0, 0.0), make_double2(ar - beta, ai));
  __syncthreads();
  for (int k = 1 + threadIdx.x; k < m; k += NT) x[k] = zmul(x[k], t);
  for (int j = 0; j < kount; ++j) beta *= sfmin;
  __syncthreads();
  if (threadIdx.x == 0) x[0] = make_double2(beta, 0.0);
  return tau;
}

}  // namespace gsk
