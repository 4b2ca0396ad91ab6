// The oracle's Schur restatement (gschur_oracle.hpp) run in 256-bit MPFR arithmetic:
// the precision of the reference's own BigFloat runs.  TEST INFRASTRUCTURE ONLY: it
// generates the high-precision fixtures under tests/golden/ on the build machine (which
// has libmpfr.so.6); the GPU machines use the committed fixtures.
//
// C-ABI (inputs and outputs in double; the whole decomposition and the residuals run at
// 256 bits):
//   or_gschur_mp  (n, a, t, z, wr, wi, resid)  real Schur   (GenericSchur.jl:805-835)
//   or_gschur_zmp (n, a, t, z, w, resid)       complex Schur (GenericSchur.jl:350-372)
// resid[0] = ||A - Z T Z^H||_F / ||A||_F, resid[1] = ||Z^H Z - I||_F.
#include <vector>

#include "scalar.hpp"
#include "mp256.hpp"

namespace orc {
// BigFloat's constants at 256 bits with MPFR's widest exponent range: eps = 2^-255,
// floatmin = 2^(emin - 1), floatmax just below 2^emax.
template <> struct lim<mp256> {
  static mp256 eps() { return mp_pow2(1 - kMpBits); }
  static mp256 fmin() { return mp_pow2(mpfr_get_emin_min() - 1); }
  static mp256 fmax() { return mp_pow2(mpfr_get_emax_max() - 1); }
};
}  // namespace orc

#include "gschur_oracle.hpp"

using namespace orc;

namespace {

template <class S> S conj_of(const S& x) { return x; }
template <class R> cx<R> conj_of(const cx<R>& x) { return conj(x); }
template <class R> R sq_of(const R& x) { return x * x; }
template <class R> R sq_of(const cx<R>& x) { return abs2(x); }

// ||A - Z T Z^H||_F / ||A||_F and ||Z^H Z - I||_F in the working precision.
template <class R, class S>
void residuals(int n, const std::vector<S>& a0, const std::vector<S>& t, const std::vector<S>& z, double* resid) {
  std::vector<S> zt((size_t)n * n, S(0));
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k) {
      const S tkj = t[k + (size_t)j * n];
      if (tkj == S(0)) continue;
      for (int i = 0; i < n; ++i) zt[i + (size_t)j * n] += z[i + (size_t)k * n] * tkj;
    }
  R num(0), den(0), orth(0);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      S s(0), o(0);
      for (int k = 0; k < n; ++k) {
        s += zt[i + (size_t)k * n] * conj_of(z[j + (size_t)k * n]);
        o += conj_of(z[k + (size_t)i * n]) * z[k + (size_t)j * n];
      }
      if (i == j) o -= S(1);
      num += sq_of(a0[i + (size_t)j * n] - s);
      den += sq_of(a0[i + (size_t)j * n]);
      orth += sq_of(o);
    }
  resid[0] = (double)(m_sqrt(num) / m_sqrt(den));
  resid[1] = (double)m_sqrt(orth);
}

}  // namespace

extern "C" {

int or_gschur_mp(int n, const double* a_in, double* t_out, double* z_out, double* wr, double* wi, double* resid) {
  mp256_init_range();
  std::vector<mp256> a((size_t)n * n), a0((size_t)n * n), z((size_t)n * n), mwr(n), mwi(n);
  for (size_t i = 0; i < (size_t)n * n; ++i) a[i] = a0[i] = mp256(a_in[i]);
  const int st = gschur_real<mp256>(n, a.data(), n, z.data(), n, mwr.data(), mwi.data(), true, true, 100LL * n);
  if (st) return st;
  for (size_t i = 0; i < (size_t)n * n; ++i) { t_out[i] = (double)a[i]; z_out[i] = (double)z[i]; }
  for (int i = 0; i < n; ++i) { wr[i] = (double)mwr[i]; wi[i] = (double)mwi[i]; }
  if (resid) residuals<mp256>(n, a0, a, z, resid);
  return 0;
}

int or_gschur_zmp(int n, const double* a_in, double* t_out, double* z_out, double* w_out, double* resid) {
  typedef cx<mp256> M;
  mp256_init_range();
  std::vector<M> a((size_t)n * n), a0((size_t)n * n), z((size_t)n * n), w(n);
  for (size_t i = 0; i < (size_t)n * n; ++i) a[i] = a0[i] = M(mp256(a_in[2 * i]), mp256(a_in[2 * i + 1]));
  const int st = gschur_cplx<mp256>(n, a.data(), n, z.data(), n, w.data(), true, true, 100LL * n, 30LL * n);
  if (st) return st;
  for (size_t i = 0; i < (size_t)n * n; ++i) {
    t_out[2 * i] = (double)a[i].re; t_out[2 * i + 1] = (double)a[i].im;
    z_out[2 * i] = (double)z[i].re; z_out[2 * i + 1] = (double)z[i].im;
  }
  for (int i = 0; i < n; ++i) { w_out[2 * i] = (double)w[i].re; w_out[2 * i + 1] = (double)w[i].im; }
  if (resid) residuals<mp256>(n, a0, a, z, resid);
  return 0;
}

}  // extern "C"
