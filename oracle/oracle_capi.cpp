// C entry points of the CPU oracle (test infrastructure only; see gschur_oracle.hpp).
// Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg through
// ctypes.  Complex arrays are interleaved (re, im) doubles, column-major.
#include <cstring>
#include <vector>
#include "gschur_oracle.hpp"
#include "eigvecs_oracle.hpp"
#include "balance_oracle.hpp"
#include "condition_oracle.hpp"
#include "hermitian_oracle.hpp"
#include "qz_oracle.hpp"
#include "gcondition_oracle.hpp"
#include "stedc_oracle.hpp"

using namespace orc;
typedef cx<double> zc;

extern "C" {

int or_version(void) { return 1; }

// ---- real, double --------------------------------------------------------
int or_gschur_d(int n, double* a, int lda, double* z, int ldz, double* wr, double* wi, int wantz,
                int scale, long long maxiter) {
  if (maxiter <= 0) maxiter = 100LL * n;
  return gschur_real<double>(n, a, lda, z, ldz, wr, wi, wantz != 0, scale != 0, maxiter);
}

int or_gschur_s(int n, float* a, int lda, float* z, int ldz, float* wr, float* wi, int wantz,
                int scale, long long maxiter) {
  if (maxiter <= 0) maxiter = 100LL * n;
  return gschur_real<float>(n, a, lda, z, ldz, wr, wi, wantz != 0, scale != 0, maxiter);
}

// Hessenberg reduction + Q (hessenberg.jl:3-17, 150-166); a overwritten with H (reflectors
// below the subdiagonal), tau n-1 entries, q n x n.
int or_hessenberg_d(int n, double* a, int lda, double* tau, double* q, int ldq) {
  hessenberg<double>(n, a, lda, tau);
  if (q) materialize_q<double>(n, a, lda, tau, q, ldq);
  return 0;
}

int or_hessenberg_z(int n, double* a, int lda, double* tau, double* q, int ldq) {
  hessenberg<zc>(n, (zc*)a, lda, (zc*)tau);
  if (q) materialize_q<zc>(n, (zc*)a, lda, (zc*)tau, (zc*)q, ldq);
  return 0;
}

// ---- complex, double -----------------------------------------------------
int or_gschur_z(int n, double* a, int lda, double* z, int ldz, double* w, int wantz, int scale,
                long long maxiter, long long maxinner) {
  if (maxiter <= 0) maxiter = 100LL * n;
  if (maxinner <= 0) maxinner = 30LL * n;
  return gschur_cplx<double>(n, (zc*)a, lda, (zc*)z, ldz, (zc*)w, wantz != 0, scale != 0, maxiter,
                             maxinner);
}

// Complex Hessenberg QR on an already-Hessenberg H (GenericSchur.jl:194-335),
// checksd = true (raises on a non-real subdiagonal: returns 2).
int or_gschur_hess_z(int n, double* h, int ldh, double* z, int ldz, double* w, long long maxiter) {
  if (maxiter <= 0) maxiter = 100LL * n;
  return gschur_hess_cplx<double>(n, (zc*)h, ldh, (zc*)z, ldz, (zc*)w, maxiter, 30LL * n, true);
}

int or_gschur_hess_d(int n, double* h, int ldh, double* z, int ldz, double* wr, double* wi,
                     long long maxiter) {
  if (maxiter <= 0) maxiter = 100LL * n;
  return gschur_hess_real<double>(n, h, ldh, z, ldz, wr, wi, maxiter);
}

// ---- quad precision (113-bit) ----------------------------------------------
// Inputs/outputs in double; the whole decomposition runs in quad.  Also returns
// the quad-precision residuals ||A - Z T Z^H||_F / ||A||_F and ||Z^H Z - I||_F.
int or_gschur_q(int n, const double* a_in, double* t_out, double* z_out, double* wr, double* wi,
                double* resid) {
  std::vector<qreal> a((size_t)n * n), a0((size_t)n * n), z((size_t)n * n), qwr(n), qwi(n);
  for (size_t i = 0; i < (size_t)n * n; ++i) a[i] = a0[i] = (qreal)a_in[i];
  int st = gschur_real<qreal>(n, a.data(), n, z.data(), n, qwr.data(), qwi.data(), true, true,
                              100LL * n);
  if (st) return st;
  for (size_t i = 0; i < (size_t)n * n; ++i) { t_out[i] = (double)a[i]; z_out[i] = (double)z[i]; }
  for (int i = 0; i < n; ++i) { wr[i] = (double)qwr[i]; wi[i] = (double)qwi[i]; }
  if (resid) {
    // ||A - Z T Z^T||_F / ||A||_F and ||Z^T Z - I||_F in quad
    std::vector<qreal> zt((size_t)n * n, 0);
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) {
        qreal tkj = a[k + (size_t)j * n];
        if (tkj == 0) continue;
        for (int i = 0; i < n; ++i) zt[i + (size_t)j * n] += z[i + (size_t)k * n] * tkj;
      }
    qreal num = 0, den = 0, orth = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        qreal s = 0;
        for (int k = 0; k < n; ++k) s += zt[i + (size_t)k * n] * z[j + (size_t)k * n];
        qreal d = a0[i + (size_t)j * n] - s;
        num += d * d;
        den += a0[i + (size_t)j * n] * a0[i + (size_t)j * n];
        qreal o = 0;
        for (int k = 0; k < n; ++k) o += z[k + (size_t)i * n] * z[k + (size_t)j * n];
        o -= (i == j) ? 1 : 0;
        orth += o * o;
      }
    resid[0] = (double)(m_sqrt(num) / m_sqrt(den));
    resid[1] = (double)m_sqrt(orth);
  }
  return 0;
}

// Complex quad: a_in interleaved complex double.
int or_gschur_zq(int n, const double* a_in, double* t_out, double* z_out, double* w_out,
                 double* resid) {
  typedef cx<qreal> Q;
  std::vector<Q> a((size_t)n * n), a0((size_t)n * n), z((size_t)n * n), w(n);
  for (size_t i = 0; i < (size_t)n * n; ++i) a[i] = a0[i] = Q((qreal)a_in[2 * i], (qreal)a_in[2 * i + 1]);
  int st = gschur_cplx<qreal>(n, a.data(), n, z.data(), n, w.data(), true, true, 100LL * n, 30LL * n);
  if (st) return st;
  for (size_t i = 0; i < (size_t)n * n; ++i) {
    t_out[2 * i] = (double)a[i].re; t_out[2 * i + 1] = (double)a[i].im;
    z_out[2 * i] = (double)z[i].re; z_out[2 * i + 1] = (double)z[i].im;
  }
  for (int i = 0; i < n; ++i) { w_out[2 * i] = (double)w[i].re; w_out[2 * i + 1] = (double)w[i].im; }
  if (resid) {
    std::vector<Q> zt((size_t)n * n);
    for (int j = 0; j < n; ++j)
      for (int k = 0; k <= j; ++k) {
        Q tkj = a[k + (size_t)j * n];
        for (int i = 0; i < n; ++i) zt[i + (size_t)j * n] += z[i + (size_t)k * n] * tkj;
      }
    qreal num = 0, den = 0, orth = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        Q s;
        for (int k = 0; k < n; ++k) s += zt[i + (size_t)k * n] * conj(z[j + (size_t)k * n]);
        Q d = a0[i + (size_t)j * n] - s;
        num += abs2(d);
        den += abs2(a0[i + (size_t)j * n]);
        Q o;
        for (int k = 0; k < n; ++k) o += conj(z[k + (size_t)i * n]) * z[k + (size_t)j * n];
        if (i == j) o -= Q(1);
        orth += abs2(o);
      }
    resid[0] = (double)(m_sqrt(num) / m_sqrt(den));
    resid[1] = (double)m_sqrt(orth);
  }
  return 0;
}

// ---- eigenvectors ------------------------------------------------------------
// left = 0: right eigenvectors (vectors.jl:133-362 real / 45-131 complex);
// left = 1: left eigenvectors (vectors.jl:462-698 / 372-460).
// normalize = 1 applies _enormalize! (util.jl:572-592), as geigvecs does (vectors.jl:12-20).
int or_eigvecs_d(int n, const double* t, const double* z, double* v, int left, int normalize) {
  if (left) gleigvecs_real<double>(n, t, n, z, n, (zc*)v, n);
  else geigvecs_real<double>(n, t, n, z, n, (zc*)v, n);
  if (normalize) enormalize<double>(n, (zc*)v, n);
  return 0;
}

int or_eigvecs_z(int n, const double* t, const double* z, double* v, int left, int normalize) {
  std::vector<zc> tt((size_t)n * n);
  std::memcpy(tt.data(), t, sizeof(zc) * (size_t)n * n);
  if (left) gleigvecs_cplx<double>(n, tt.data(), n, (const zc*)z, n, (zc*)v, n);
  else geigvecs_cplx<double>(n, tt.data(), n, (const zc*)z, n, (zc*)v, n);
  if (normalize) enormalize<double>(n, (zc*)v, n);
  return 0;
}

int or_triangularize_d(int n, const double* t, const double* z, double* tc, double* zc_out, double* w) {
  triangularize<double>(n, t, n, z, n, (zc*)tc, (zc*)zc_out, (zc*)w);
  return 0;
}

// balance! (balance.jl:33-185): out3 = {ilo, ihi, trivial}, sp / D of length n.
int or_balance_d(int n, double* a, int lda, int scale, int permute, int* out3, int* sp, double* d) {
  return balance<double, double>(n, a, lda, scale != 0, permute != 0, &out3[0], &out3[1], sp, d, &out3[2]);
}
int or_balance_z(int n, double* a, int lda, int scale, int permute, int* out3, int* sp, double* d) {
  return balance<double, zc>(n, (zc*)a, lda, scale != 0, permute != 0, &out3[0], &out3[1], sp, d, &out3[2]);
}
// lmul!(B, V) / ldiv!(B, V) on complex V (n x m)
int or_balancer_apply_z(int n, int m, double* v, int ldv, int ilo, int ihi, const int* sp, const double* d,
                        int trivial, int inverse) {
  balancer_apply<double, zc>(n, m, (zc*)v, ldv, ilo, ihi, sp, d, trivial != 0, inverse != 0);
  return 0;
}

// trsylvester! / adjtrsylvester! (sylvester.jl:11-139) on C (m x p, in place);
// out2 = {scale, perturbed}.
int or_trsylv_d(int adj, int m, int p, const double* a, int lda, const double* b, int ldb, double* c, int ldc,
                double* out2) {
  bool pert = false;
  out2[0] = trsylvester<double, double>((adj & 1) != 0, m, p, a, lda, b, ldb, c, ldc, &pert, (adj & 2) != 0);
  out2[1] = pert ? 1.0 : 0.0;
  return 0;
}
int or_trsylv_z(int adj, int m, int p, const double* a, int lda, const double* b, int ldb, double* c, int ldc,
                double* out2) {
  bool pert = false;
  out2[0] = trsylvester<double, zc>((adj & 1) != 0, m, p, (const zc*)a, lda, (const zc*)b, ldb, (zc*)c, ldc, &pert, (adj & 2) != 0);
  out2[1] = pert ? 1.0 : 0.0;
  return 0;
}
// eigvalscond / subspacesep (ordschur.jl:84-140) of the leading nsub block of T (n x n).
int or_econd_d(int n, const double* t, int ldt, int nsub, double* out2) {
  out2[0] = eigvalscond<double, double>(n, t, ldt, nsub);
  out2[1] = subspacesep<double, double>(n, t, ldt, nsub);
  return 0;
}
int or_econd_z(int n, const double* t, int ldt, int nsub, double* out2) {
  out2[0] = eigvalscond<double, zc>(n, (const zc*)t, ldt, nsub);
  out2[1] = subspacesep<double, zc>(n, (const zc*)t, ldt, nsub);
  return 0;
}

// geigen! / geigvals! of Hermitian(A, uplo) (GenericSchur.jl:126-146): w ascending, V
// (when wantv) the eigenvectors; A overwritten.  Returns 1 if the sweep limit was hit.
int or_heev_d(int n, double* a, int lda, int upper, int wantv, double* w, double* v) {
  return heev<double, double>(n, a, lda, upper != 0, wantv != 0, w, v, n);
}
int or_heev_z(int n, double* a, int lda, int upper, int wantv, double* w, double* v) {
  return heev<double, zc>(n, (zc*)a, lda, upper != 0, wantv != 0, w, (zc*)v, n);
}
// _hehessenberg! (hessenberg.jl:26-96): d (n), e (n-1), tau (n-1), A overwritten.
int or_hetrd_d(int n, double* a, int lda, int upper, double* d, double* e, double* tau) {
  if (upper) he_tridiag_U<double, double>(n, a, lda, tau, d, e);
  else he_tridiag_L<double, double>(n, a, lda, tau, d, e);
  return 0;
}
int or_hetrd_z(int n, double* a, int lda, int upper, double* d, double* e, double* tau) {
  if (upper) he_tridiag_U<double, zc>(n, (zc*)a, lda, (zc*)tau, d, e);
  else he_tridiag_L<double, zc>(n, (zc*)a, lda, (zc*)tau, d, e);
  return 0;
}
// _gschur!(SymTridiagonal(d, e), QRIteration(), Z) (symtridiag.jl:79-183) with Z n x n
// (wantz) or none.
// _gschur!(SymTridiagonal(d, e), DivideAndConquer(), Z) with Z (n x n) multiplied in
// place when wantz; 1 when a secular equation did not converge.
int or_stedc_d(int n, double* d, double* e, double* z, int wantz) { return stedc(n, d, e, wantz ? z : nullptr, n); }

int or_steqr_d(int n, double* d, double* e, double* z, int wantz) {
  return steqr<double, double>(n, d, e, wantz ? z : nullptr, n, wantz ? n : 0, 30LL * n);
}

// ggschur!(A, B) for complex pencils (generalized.jl:21-80): A <- S, B <- T, Q, Z (n x n
// each, wanted when non-null), alpha, beta.  Returns 1 at the iteration limit.
int or_ggschur_z(int n, double* a, double* b, double* q, double* z, double* alpha, double* beta, int scale) {
  return ggschur_cplx<double>(n, (zc*)a, n, (zc*)b, n, (zc*)q, (zc*)z, (zc*)alpha, (zc*)beta, scale != 0, 100LL * n);
}

// Eigenvectors of a complex generalized Schur pair (src/vectors.jl:723-1038): right (left
// = 0, back-transformed by X = Z) or left (left = 1, X = Q); X may be null.  V n x n.
int or_ggevc_z(int n, const double* s, const double* p, const double* x, double* v, int left) {
  if (left)
    ggevc_left<double>(n, (const zc*)s, (const zc*)p, (const zc*)x, (zc*)v);
  else
    ggevc_right<double>(n, (const zc*)s, (const zc*)p, (const zc*)x, (zc*)v);
  return 0;
}

// ggschur!(A, B) for real pencils (src/rgeneralized.jl:10-66): A <- S (quasi-triangular),
// B <- T, Q, Z (when non-null), alpha = alr + i ali, beta.  Returns 1 at the iteration limit.
int or_ggschur_d(int n, double* a, double* b, double* q, double* z, double* alr, double* ali, double* be, int scale) {
  return ggschur_real<double>(n, a, n, b, n, q, z, alr, ali, be, scale != 0, 100LL * n);
}

// Eigenvectors of a real generalized Schur pair (src/vectors.jl:1040-1513): right (left = 0,
// back-transformed by X = Z) or left (left = 1, X = Q); X may be null.  V n x n complex.
int or_rgevc_d(int n, const double* s, const double* p, const double* x, double* v, int left) {
  if (left)
    rgevc_left<double>(n, s, p, x, (zc*)v);
  else
    rgevc_right<double>(n, s, p, x, (zc*)v);
  return 0;
}

// gordschur!(S, T, Q, Z, select) for a complex generalized Schur form (src/ordschur.jl:
// 147-305), in place; alpha, beta the new diagonals.  Returns 0 or 1 + j1 of a rejected swap.
int or_ggordschur_z(int n, double* s, double* t, double* q, double* z, const int* select, int scale, double* al,
                    double* be) {
  return gordschur_cplx<double>(n, (zc*)s, (zc*)t, (zc*)q, (zc*)z, select, scale != 0, (zc*)al, (zc*)be);
}

// gordschur!(S, T, Q, Z, select) of a real generalized Schur pair; alpha interleaved complex
int or_ggordschur_d(int n, double* s, double* t, double* q, double* z, const int* select, int scale, double* alpha,
                    double* beta) {
  return gordschur_real<double>(n, s, t, q, z, select, scale != 0, (zc*)alpha, beta);
}

// trsylvester!(A, B, C, D, E, F) (adj = 0) / adjtrsylvester! (adj = 1) for complex triangular
// A, D (m x m), B, E (n x n); C, F (m x n) overwritten; returns the reference's scale.
double or_gtrsyl_z(int m, int n, const double* a, const double* b, double* c, const double* d, const double* e,
                   double* f, int adj) {
  if (adj) return gadjtrsyl<double>(m, n, (const zc*)a, (const zc*)b, (zc*)c, (const zc*)d, (const zc*)e, (zc*)f);
  return gtrsyl<double>(m, n, (const zc*)a, (const zc*)b, (zc*)c, (const zc*)d, (const zc*)e, (zc*)f);
}
// eigvalscond / subspacesep (pnorm = :F) of a complex generalized Schur form (gcondition.jl)
int or_gcond_z(int n, const double* s, const double* t, int nsub, double* out, int sep) {
  if (sep) gsubspacesep<double>(n, (const zc*)s, (const zc*)t, nsub, out);
  else geigvalscond<double>(n, (const zc*)s, (const zc*)t, nsub, &out[0], &out[1]);
  return 0;
}

int or_gs2x2_d(double* h, double* cs, double* sn, double* w) {
  gs2x2<double>(h, cs, sn, &w[0], &w[1], &w[2], &w[3]);
  return 0;
}

int or_reflector_d(double* x, int n, double* tau) {
  *tau = reflector_real<double>(x, n);
  return 0;
}

// ---- batched (CPU baseline) --------------------------------------------------
// Ragged batch: matrix b has order ns[b], column-major at a + offs[b] (doubles, or
// complex pairs for the _z form).  Runs the reference algorithm per matrix, OpenMP
// over the batch.  Returns the number of matrices that failed to converge.
int or_gschur_batched_d(int count, const long long* offs, const int* ns, double* a, double* z,
                        double* wr, double* wi, const long long* woffs, int* status, int nthreads) {
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : bad)
  for (int b = 0; b < count; ++b) {
    int n = ns[b];
    int st = gschur_real<double>(n, a + offs[b], n, z + offs[b], n, wr + woffs[b], wi + woffs[b], true,
                                 true, 100LL * n);
    if (status) status[b] = st;
    bad += (st != 0);
  }
  return bad;
}

int or_gschur_batched_z(int count, const long long* offs, const int* ns, double* a, double* z,
                        double* w, const long long* woffs, int* status, int nthreads) {
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : bad)
  for (int b = 0; b < count; ++b) {
    int n = ns[b];
    int st = gschur_cplx<double>(n, (zc*)(a + 2 * offs[b]), n, (zc*)(z + 2 * offs[b]), n,
                                 (zc*)(w + 2 * woffs[b]), true, true, 100LL * n, 30LL * n);
    if (status) status[b] = st;
    bad += (st != 0);
  }
  return bad;
}

}  // extern "C"
