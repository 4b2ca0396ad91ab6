// 256-bit binary floating point for the CPU oracle (test infrastructure only): the
// precision of Julia's default BigFloat, which is what the reference's own BigFloat
// Schur runs use (BigFloat is MPFR with 256-bit significands and round-to-nearest).
//
// The type wraps the MPFR library (libmpfr.so.6, present on the build machine without its
// development headers), declared here by hand from MPFR's public C interface: the
// value struct (precision, sign, exponent, limb pointer) and the functions the restated
// algorithms need.  Every operation rounds to nearest at 256 bits, as BigFloat does.
// The exponent range is widened to MPFR's maximum, as Julia does at start-up, so the
// reference's underflow/overflow guards (which test against floatmin/floatmax of the
// working type) behave as they do for BigFloat.
#pragma once
#include <cstdint>

extern "C" {
typedef long mpfr_prec_t;
typedef int mpfr_sign_t;
typedef long mpfr_exp_t;
typedef struct {
  mpfr_prec_t _mpfr_prec;
  mpfr_sign_t _mpfr_sign;
  mpfr_exp_t _mpfr_exp;
  void* _mpfr_d;
} orc_mpfr_struct;
typedef orc_mpfr_struct* orc_mpfr_ptr;
typedef const orc_mpfr_struct* orc_mpfr_srcptr;
typedef int orc_mpfr_rnd_t;  // MPFR_RNDN = 0

void mpfr_init2(orc_mpfr_ptr, mpfr_prec_t);
void mpfr_clear(orc_mpfr_ptr);
int mpfr_set4(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_rnd_t, int);
int mpfr_set_d(orc_mpfr_ptr, double, orc_mpfr_rnd_t);
int mpfr_set_si(orc_mpfr_ptr, long, orc_mpfr_rnd_t);
double mpfr_get_d(orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_add(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_sub(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_mul(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_div(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_sqrt(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_hypot(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_neg(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_abs(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_copysign(orc_mpfr_ptr, orc_mpfr_srcptr, orc_mpfr_srcptr, orc_mpfr_rnd_t);
int mpfr_cmp(orc_mpfr_srcptr, orc_mpfr_srcptr);
int mpfr_nan_p(orc_mpfr_srcptr);
int mpfr_mul_2si(orc_mpfr_ptr, orc_mpfr_srcptr, long, orc_mpfr_rnd_t);
mpfr_exp_t mpfr_get_emin_min(void);
mpfr_exp_t mpfr_get_emax_max(void);
int mpfr_set_emin(mpfr_exp_t);
int mpfr_set_emax(mpfr_exp_t);
}

namespace orc {

constexpr long kMpBits = 256;

class mp256 {
 public:
  mp256() { mpfr_init2(v_, kMpBits); mpfr_set_si(v_, 0, 0); }
  mp256(double d) { mpfr_init2(v_, kMpBits); mpfr_set_d(v_, d, 0); }
  mp256(int i) { mpfr_init2(v_, kMpBits); mpfr_set_si(v_, i, 0); }
  mp256(long i) { mpfr_init2(v_, kMpBits); mpfr_set_si(v_, i, 0); }
  mp256(long long i) { mpfr_init2(v_, kMpBits); mpfr_set_si(v_, (long)i, 0); }
  mp256(const mp256& o) { mpfr_init2(v_, kMpBits); mpfr_set4(v_, o.v_, 0, o.v_->_mpfr_sign); }
  mp256& operator=(const mp256& o) {
    if (this != &o) mpfr_set4(v_, o.v_, 0, o.v_->_mpfr_sign);
    return *this;
  }
  ~mp256() { mpfr_clear(v_); }
  explicit operator double() const { return mpfr_get_d(v_, 0); }
  orc_mpfr_ptr p() { return v_; }
  orc_mpfr_srcptr p() const { return v_; }

 private:
  orc_mpfr_struct v_[1];
};

// Widen the exponent range to MPFR's maximum (as Julia does for BigFloat); call once
// before any computation.
inline void mp256_init_range() {
  mpfr_set_emin(mpfr_get_emin_min());
  mpfr_set_emax(mpfr_get_emax_max());
}

#define ORC_MP_BINOP(OP, FN)                                                            \
  inline mp256 operator OP(const mp256& a, const mp256& b) {                            \
    mp256 r;                                                                            \
    FN(r.p(), a.p(), b.p(), 0);                                                         \
    return r;                                                                           \
  }                                                                                     \
  inline mp256 operator OP(const mp256& a, double b) { return a OP mp256(b); }          \
  inline mp256 operator OP(double a, const mp256& b) { return mp256(a) OP b; }          \
  inline mp256 operator OP(const mp256& a, int b) { return a OP mp256(b); }             \
  inline mp256 operator OP(int a, const mp256& b) { return mp256(a) OP b; }             \
  inline mp256& operator OP##=(mp256& a, const mp256& b) {                              \
    FN(a.p(), a.p(), b.p(), 0);                                                         \
    return a;                                                                           \
  }
ORC_MP_BINOP(+, mpfr_add)
ORC_MP_BINOP(-, mpfr_sub)
ORC_MP_BINOP(*, mpfr_mul)
ORC_MP_BINOP(/, mpfr_div)
#undef ORC_MP_BINOP

inline mp256 operator-(const mp256& a) {
  mp256 r;
  mpfr_neg(r.p(), a.p(), 0);
  return r;
}

#define ORC_MP_CMP(OP)                                                                         \
  inline bool operator OP(const mp256& a, const mp256& b) {                                    \
    return !mpfr_nan_p(a.p()) && !mpfr_nan_p(b.p()) && mpfr_cmp(a.p(), b.p()) OP 0;            \
  }                                                                                            \
  inline bool operator OP(const mp256& a, double b) { return a OP mp256(b); }                  \
  inline bool operator OP(double a, const mp256& b) { return mp256(a) OP b; }                  \
  inline bool operator OP(const mp256& a, int b) { return a OP mp256(b); }                     \
  inline bool operator OP(int a, const mp256& b) { return mp256(a) OP b; }
ORC_MP_CMP(<)
ORC_MP_CMP(>)
ORC_MP_CMP(<=)
ORC_MP_CMP(>=)
ORC_MP_CMP(==)
#undef ORC_MP_CMP
inline bool operator!=(const mp256& a, const mp256& b) { return !(a == b); }
inline bool operator!=(const mp256& a, double b) { return !(a == mp256(b)); }
inline bool operator!=(const mp256& a, int b) { return !(a == mp256(b)); }

inline mp256 m_sqrt(const mp256& x) { mp256 r; mpfr_sqrt(r.p(), x.p(), 0); return r; }
inline mp256 m_abs(const mp256& x) { mp256 r; mpfr_abs(r.p(), x.p(), 0); return r; }
inline mp256 m_hypot(const mp256& x, const mp256& y) { mp256 r; mpfr_hypot(r.p(), x.p(), y.p(), 0); return r; }
inline mp256 m_copysign(const mp256& x, const mp256& y) {
  mp256 r;
  mpfr_copysign(r.p(), x.p(), y.p(), 0);
  return r;
}
inline bool m_isnan(const mp256& x) { return mpfr_nan_p(x.p()) != 0; }
inline mp256 mp_pow2(long e) { mp256 r(1); mpfr_mul_2si(r.p(), r.p(), e, 0); return r; }

}  // namespace orc
