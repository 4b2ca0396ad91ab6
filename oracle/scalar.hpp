// Scalar support for the CPU oracle (test infrastructure only: the product path
// never links this).  Provides a minimal complex type and the math functions the
// restated algorithms need, for float, double and a 113-bit quad type.
//
// The quad type stands in for the reference's BigFloat oracle: GenericSchur.jl's
// own known-answer test (test/real.jl:142-157) runs at 80 bits, so 113 bits is
// more than the reference requires there.
#pragma once
#include <cmath>
#include <cfloat>
#include <cstdint>
#include <limits>

#if defined(__x86_64__) || defined(__i386__)
extern "C" {
#include <quadmath.h>
}
typedef __float128 qreal;
#define ORC_HAVE_FLOAT128 1
#else
// aarch64 (and other LP64 Linux targets with IEEE binary128 long double)
typedef long double qreal;
#endif

namespace orc {

// ---- real math wrappers -------------------------------------------------
inline float m_sqrt(float x) { return std::sqrt(x); }
inline double m_sqrt(double x) { return std::sqrt(x); }
inline float m_abs(float x) { return std::fabs(x); }
inline double m_abs(double x) { return std::fabs(x); }
inline float m_hypot(float x, float y) { return std::hypot(x, y); }
inline double m_hypot(double x, double y) { return std::hypot(x, y); }
inline float m_copysign(float x, float y) { return std::copysign(x, y); }
inline double m_copysign(double x, double y) { return std::copysign(x, y); }
inline bool m_isnan(float x) { return std::isnan(x); }
inline bool m_isnan(double x) { return std::isnan(x); }

#ifdef ORC_HAVE_FLOAT128
inline qreal m_sqrt(qreal x) { return sqrtq(x); }
inline qreal m_abs(qreal x) { return fabsq(x); }
inline qreal m_hypot(qreal x, qreal y) { return hypotq(x, y); }
inline qreal m_copysign(qreal x, qreal y) { return copysignq(x, y); }
inline bool m_isnan(qreal x) { return isnanq(x); }
#else
inline qreal m_sqrt(qreal x) { return sqrtl(x); }
inline qreal m_abs(qreal x) { return fabsl(x); }
inline qreal m_hypot(qreal x, qreal y) { return hypotl(x, y); }
inline qreal m_copysign(qreal x, qreal y) { return copysignl(x, y); }
inline bool m_isnan(qreal x) { return std::isnan(x); }
#endif

template <class R> inline R m_max(R a, R b) { return (a < b) ? b : a; }
template <class R> inline R m_min(R a, R b) { return (b < a) ? b : a; }

// IEEE constants per type: eps = 2^-(p-1), floatmin, floatmax.
template <class R> struct lim;
template <> struct lim<float> {
  static float eps() { return FLT_EPSILON; }
  static float fmin() { return FLT_MIN; }
  static float fmax() { return FLT_MAX; }
};
template <> struct lim<double> {
  static double eps() { return DBL_EPSILON; }
  static double fmin() { return DBL_MIN; }
  static double fmax() { return DBL_MAX; }
};
template <> struct lim<qreal> {
#ifdef ORC_HAVE_FLOAT128
  static qreal eps() { return FLT128_EPSILON; }
  static qreal fmin() { return FLT128_MIN; }
  static qreal fmax() { return FLT128_MAX; }
#else
  static qreal eps() { return LDBL_EPSILON; }
  static qreal fmin() { return LDBL_MIN; }
  static qreal fmax() { return LDBL_MAX; }
#endif
};

// safemin: floatmin unless 1/floatmax is larger (util.jl:5-12).
template <class R> inline R safemin() {
  R sfmin = lim<R>::fmin();
  R small = R(1) / lim<R>::fmax();
  if (small >= sfmin) sfmin = small * (R(1) + lim<R>::eps());
  return sfmin;
}

// ---- complex -------------------------------------------------------------
template <class R> struct cx {
  R re, im;
  cx() : re(0), im(0) {}
  cx(R r) : re(r), im(0) {}
  cx(R r, R i) : re(r), im(i) {}
};
template <class R> inline cx<R> operator+(cx<R> a, cx<R> b) { return cx<R>(a.re + b.re, a.im + b.im); }
template <class R> inline cx<R> operator-(cx<R> a, cx<R> b) { return cx<R>(a.re - b.re, a.im - b.im); }
template <class R> inline cx<R> operator-(cx<R> a) { return cx<R>(-a.re, -a.im); }
template <class R> inline cx<R> operator*(cx<R> a, cx<R> b) {
  return cx<R>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <class R> inline cx<R> operator*(cx<R> a, R s) { return cx<R>(a.re * s, a.im * s); }
template <class R> inline cx<R> operator*(R s, cx<R> a) { return cx<R>(a.re * s, a.im * s); }
template <class R> inline cx<R> operator/(cx<R> a, R s) { return cx<R>(a.re / s, a.im / s); }
// Smith's algorithm for complex division (robust against overflow of |b|^2).
template <class R> inline cx<R> operator/(cx<R> a, cx<R> b) {
  if (m_abs(b.im) <= m_abs(b.re)) {
    if (b.re == R(0) && b.im == R(0)) return cx<R>(a.re / b.re, a.im / b.re);
    R r = b.im / b.re, d = b.re + b.im * r;
    return cx<R>((a.re + a.im * r) / d, (a.im - a.re * r) / d);
  } else {
    R r = b.re / b.im, d = b.im + b.re * r;
    return cx<R>((a.re * r + a.im) / d, (a.im * r - a.re) / d);
  }
}
template <class R> inline cx<R> operator/(R s, cx<R> b) { return cx<R>(s) / b; }
template <class R> inline cx<R>& operator+=(cx<R>& a, cx<R> b) { a = a + b; return a; }
template <class R> inline cx<R>& operator-=(cx<R>& a, cx<R> b) { a = a - b; return a; }
template <class R> inline cx<R>& operator*=(cx<R>& a, cx<R> b) { a = a * b; return a; }
template <class R> inline cx<R>& operator*=(cx<R>& a, R s) { a = a * s; return a; }
template <class R> inline bool operator==(cx<R> a, cx<R> b) { return a.re == b.re && a.im == b.im; }
template <class R> inline bool operator!=(cx<R> a, cx<R> b) { return !(a == b); }
template <class R> inline cx<R> conj(cx<R> a) { return cx<R>(a.re, -a.im); }
template <class R> inline R cabs(cx<R> a) { return m_hypot(a.re, a.im); }
template <class R> inline R abs1(cx<R> a) { return m_abs(a.re) + m_abs(a.im); }
template <class R> inline R abs1(R a) { return m_abs(a); }
template <class R> inline R abs2(cx<R> a) { return a.re * a.re + a.im * a.im; }
template <class R> inline bool cisnan(cx<R> a) { return m_isnan(a.re) || m_isnan(a.im); }
// principal square root
template <class R> inline cx<R> csqrt(cx<R> z) {
  R x = z.re, y = z.im;
  if (x == R(0) && y == R(0)) return cx<R>(R(0), y);
  R t = m_sqrt((m_abs(x) + m_hypot(x, y)) / R(2));
  if (x >= R(0)) return cx<R>(t, y / (R(2) * t));
  return cx<R>(m_abs(y) / (R(2) * t), m_copysign(t, y));
}

// Real/complex helpers used by generic code.
template <class R> inline R re_of(R a) { return a; }
template <class R> inline R re_of(cx<R> a) { return a.re; }
template <class R> inline R cj(R a) { return a; }
template <class R> inline cx<R> cj(cx<R> a) { return conj(a); }
template <class R> inline R modulus(R a) { return m_abs(a); }
template <class R> inline R modulus(cx<R> a) { return cabs(a); }

}  // namespace orc
