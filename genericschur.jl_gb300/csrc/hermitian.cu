// Hermitian / real symmetric eigenproblems: geigen! / geigvals! (GenericSchur.jl:126-146)
// with the default QRIteration, hessenberg!(Hermitian) (hessenberg.jl:26-130) and
// _gschur!(::SymTridiagonal, QRIteration, Z) (symtridiag.jl:79-368).
//
// 1. Tridiagonalization (zhetd2, lower form): the matrix is kept full (both triangles,
//    exactly Hermitian) in a device work array so that every access is a column read.
//    Step i, two launches:
//      k_he_matvec  w = tau A22 v, warp per column j (w_j = tau sum_k conj(A22[k,j]) v_k),
//                   per-CTA partial dots; the last CTA (ticket) forms
//                   alpha = -(tau/2) w^H v;
//      k_he_update  A22 -= v w'^H + w' v^H with w' = w + alpha v; the last CTA restores
//                   the subdiagonal entry and computes the reflector of column i+1.
//    Memory bound: 3 passes over the trailing block per step (n^3 element accesses).
//    Hermitian(A, :U) is the lower form applied to J A J (J the index reversal): the
//    reference's :U sweep (hessenberg.jl:60-96) takes the same reflectors with their
//    tails in the opposite order, so the results agree up to summation order.
// 2. Q = H_1 ... H_{n-1} accumulated backwards into the identity (k_he_formq, one launch
//    per reflector, warp per column: y_j = u^H Q[:,j], Q[:,j] -= tau u y_j).
// 3. Tridiagonal QR (k_steqr): one cooperative kernel.  Thread 0 of block 0 runs the
//    reference's state machine (splits, scaling, QL or QR per block, 2x2 deflation,
//    Givens sweeps with LinearAlgebra's givensAlgorithm); each sweep's rotations go to a
//    double buffer, and all other threads apply the previous sweep's rotations to their
//    rows of Z (a carry in a register along the sweep) while the next sweep is computed.
//    Phases end at a grid barrier with an iteration limit (cooperative launch: all blocks
//    are resident).  The sweep recurrence is one serial FP64 chain; Z costs nothing extra.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kHeT = 256;

template <class S> struct Hs;
template <> struct Hs<double> {
  static __device__ __forceinline__ double zero() { return 0.0; }
  static __device__ __forceinline__ double one() { return 1.0; }
  static __device__ __forceinline__ double from(double r) { return r; }
  static __device__ __forceinline__ double conj(double a) { return a; }
  static __device__ __forceinline__ double re(double a) { return a; }
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
  // c + conj(a) b
  static __device__ __forceinline__ double fmac(double a, double b, double c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __device__ __forceinline__ double scal(double a, double s) { return a * s; }
  static __device__ __forceinline__ bool is0(double a) { return a == 0.0; }
  static __device__ __forceinline__ double shfl(double a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
};
template <> struct Hs<double2> {
  static __device__ __forceinline__ double2 zero() { return make_double2(0.0, 0.0); }
  static __device__ __forceinline__ double2 one() { return make_double2(1.0, 0.0); }
  static __device__ __forceinline__ double2 from(double r) { return make_double2(r, 0.0); }
  static __device__ __forceinline__ double2 conj(double2 a) { return zconj(a); }
  static __device__ __forceinline__ double re(double2 a) { return a.x; }
  static __device__ __forceinline__ double2 mul(double2 a, double2 b) { return zmul(a, b); }
  static __device__ __forceinline__ double2 fma(double2 a, double2 b, double2 c) { return zfma(a, b, c); }
  static __device__ __forceinline__ double2 fmac(double2 a, double2 b, double2 c) { return zfmac(a, b, c); }
  static __device__ __forceinline__ double2 add(double2 a, double2 b) { return zadd(a, b); }
  static __device__ __forceinline__ double2 sub(double2 a, double2 b) { return zsub(a, b); }
  static __device__ __forceinline__ double2 scal(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
  static __device__ __forceinline__ bool is0(double2 a) { return a.x == 0.0 && a.y == 0.0; }
  static __device__ __forceinline__ double2 shfl(double2 a, int o) {
    return make_double2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
  }
};

template <class S> __device__ __forceinline__ S warp_sum(S v) {
  for (int o = 16; o > 0; o >>= 1) v = Hs<S>::add(v, Hs<S>::shfl(v, o));
  return v;
}

// Control block of the tridiagonalization (device memory).
template <class S> struct HeCtl {
  S tau;          // reflector of the current step
  S alpha;        // -(tau/2) w^H v
  unsigned t_mv;  // ticket of k_he_matvec
  unsigned t_up;  // ticket of k_he_update
};

// Full Hermitian matrix B (ld n) in the lower-form frame from the triangle `upper` of A.
template <class S>
__global__ void k_he_prep(const S* __restrict__ A, long long lda, int n, int upper, S* __restrict__ B) {
  const size_t tot = (size_t)n * n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % n), l = (int)(e / n);
    S v;
    if (!upper) v = (k >= l) ? A[k + l * lda] : Hs<S>::conj(A[l + k * lda]);
    else v = (k >= l) ? A[(n - 1 - k) + (n - 1 - l) * lda] : Hs<S>::conj(A[(n - 1 - l) + (n - 1 - k) * lda]);
    if (k == l) v = Hs<S>::from(Hs<S>::re(v));
    B[e] = v;
  }
}

// Reflector of column i (0-based) of B: x = B[i+1:n, i].  One CTA.  Writes tau, e[i],
// d[i], sets B[i+1, i] = 1 (the head of v during the step).
template <class S>
__device__ void he_step_reflector(S* B, int n, int i, HeCtl<S>* ctl, S* tau, double* d, double* e, double* red) {
  S* x = B + (size_t)i * n + (i + 1);
  const int m = n - 1 - i;
  const S t = cta_reflector<kHeT>(x, m, red);
  __syncthreads();
  if (threadIdx.x == 0) {
    e[i] = Hs<S>::re(x[0]);
    d[i] = Hs<S>::re(B[(size_t)i * n + i]);
    tau[i] = t;
    ctl->tau = t;
    x[0] = Hs<S>::one();
  }
}

template <class S>
__global__ void __launch_bounds__(kHeT) k_he_first(S* B, int n, HeCtl<S>* ctl, S* tau, double* d, double* e) {
  __shared__ double red[kHeT / 32];
  if (n == 1) {
    if (threadIdx.x == 0) d[0] = Hs<S>::re(B[0]);
    return;
  }
  he_step_reflector<S>(B, n, 0, ctl, tau, d, e, red);
}

// w_j = tau sum_k conj(B[k, j]) v_k for j in [i+1, n); warp per column.  partial[cta] =
// sum over the CTA's columns of conj(w_j) v_j; the last CTA forms alpha.
template <class S>
__global__ void __launch_bounds__(kHeT) k_he_matvec(const S* __restrict__ B, int n, int i, S* __restrict__ W,
                                                     S* __restrict__ partial, HeCtl<S>* ctl) {
  using O = Hs<S>;
  __shared__ S wsum[kHeT / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int m = n - 1 - i;
  const S* v = B + (size_t)i * n + (i + 1);  // v[0] = 1 is stored
  const S tau = ctl->tau;
  S acc = O::zero();
  for (int jj = blockIdx.x * (kHeT / 32) + wid; jj < m; jj += gridDim.x * (kHeT / 32)) {
    const S* col = B + (size_t)(i + 1 + jj) * n + (i + 1);
    S s = O::zero();
    for (int k = lane; k < m; k += 32) s = O::fmac(col[k], v[k], s);
    s = warp_sum(s);
    const S w = O::mul(tau, s);
    if (lane == 0) W[jj] = w;
    acc = O::fmac(w, v[jj], acc);  // conj(w_j) v_j
  }
  if (lane == 0) wsum[wid] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    S p = wsum[0];
    for (int q = 1; q < kHeT / 32; ++q) p = O::add(p, wsum[q]);
    partial[blockIdx.x] = p;
    __threadfence();
    last = atomicAdd(&ctl->t_mv, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    S dw = O::zero();
    for (int b = 0; b < (int)gridDim.x; ++b) dw = O::add(dw, partial[b]);
    ctl->alpha = O::mul(O::scal(tau, -0.5), dw);
    ctl->t_mv = 0;
  }
}

// A22 -= v w'^H + w' v^H, w' = w + alpha v (diagonal kept real).  CTA per column block;
// the last CTA puts e[i] back below the diagonal and forms the next reflector.
template <class S>
__global__ void __launch_bounds__(kHeT) k_he_update(S* B, int n, int i, const S* __restrict__ W, HeCtl<S>* ctl,
                                                     S* tau, double* d, double* e) {
  using O = Hs<S>;
  __shared__ double red[kHeT / 32];
  __shared__ bool last;
  const int m = n - 1 - i;
  const S* v = B + (size_t)i * n + (i + 1);
  const S alpha = ctl->alpha;
  for (int jj = blockIdx.x; jj < m; jj += gridDim.x) {
    const S vj = v[jj];
    const S wj = O::fma(alpha, vj, W[jj]);
    const S cvj = O::conj(vj), cwj = O::conj(wj);
    S* col = B + (size_t)(i + 1 + jj) * n + (i + 1);
    for (int k = threadIdx.x; k < m; k += kHeT) {
      const S vk = v[k];
      const S wk = O::fma(alpha, vk, W[k]);
      // a - (v_k conj(w_j) + w_k conj(v_j))
      S upd = O::fma(wk, cvj, O::mul(vk, cwj));
      S a = O::sub(col[k], upd);
      if (k == jj) a = O::from(O::re(a));
      col[k] = a;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&ctl->t_up, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    B[(size_t)i * n + (i + 1)] = O::from(e[i]);
    ctl->t_up = 0;
  }
  if (i + 1 <= n - 2) {
    he_step_reflector<S>(B, n, i + 1, ctl, tau, d, e, red);
  } else if (threadIdx.x == 0) {
    d[n - 1] = O::re(B[(size_t)(n - 1) * n + (n - 1)]);
  }
}

// Backward accumulation, reflector i: Q[i+1:, j] -= tau u (u^H Q[i+1:, j]) for j > i,
// u = [1; B[i+2:n, i]].  Warp per column.
template <class S>
__global__ void __launch_bounds__(kHeT) k_he_formq(const S* __restrict__ B, int n, int i, const S* __restrict__ tau,
                                                    S* Q) {
  using O = Hs<S>;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int m = n - 1 - i;
  const S* u = B + (size_t)i * n + (i + 1);
  const S t = tau[i];
  if (O::is0(t)) return;
  for (int jj = blockIdx.x * (kHeT / 32) + wid; jj < m; jj += gridDim.x * (kHeT / 32)) {
    S* q = Q + (size_t)(i + 1 + jj) * n + (i + 1);
    S s = O::zero();
    for (int k = lane; k < m; k += 32) s = O::fmac(k == 0 ? O::one() : u[k], q[k], s);
    s = warp_sum(s);
    const S ts = O::mul(t, s);
    for (int k = lane; k < m; k += 32) {
      const S uk = k == 0 ? O::one() : u[k];
      q[k] = O::sub(q[k], O::mul(ts, uk));
    }
  }
}

template <class S>
__global__ void k_he_identity(S* Q, int n) {
  const size_t tot = (size_t)n * n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x)
    Q[e] = Hs<S>::from((e % n) == (e / n) ? 1.0 : 0.0);
}

// Write the factors back into A's triangle (`upper` reverses the frame): B's lower
// triangle (diagonal real, subdiagonal e, reflector tails below).
template <class S>
__global__ void k_he_store(const S* __restrict__ B, int n, int upper, S* A, long long lda) {
  const size_t tot = (size_t)n * n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % n), l = (int)(e / n);
    if (k < l) continue;
    if (!upper) A[k + l * lda] = B[e];
    else A[(n - 1 - k) + (n - 1 - l) * lda] = B[e];
  }
}

// V[:, j] = Z[:, p[j]] (rows reversed when `rev`).
template <class S>
__global__ void k_he_gather(const S* __restrict__ Z, int n, const int* __restrict__ p, int rev, S* V, long long ldv) {
  const size_t tot = (size_t)n * n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(e % n), j = (int)(e / n);
    V[r + j * ldv] = Z[(rev ? (n - 1 - r) : r) + (size_t)p[j] * n];
  }
}

// ---- tridiagonal QR (symtridiag.jl:79-368) -------------------------------------------

// givensAlgorithm on its plain branch (2^-485 < max(|f|, |g|) < 2^485) from one Newton-
// refined reciprocal square root: c = f / r, s = g / r, r = sqrt(f^2 + g^2) to ~1 ulp with
// a third of the serial FP64 instructions of sqrt and two divisions.  The branch tests
// run on the bit patterns (integer pipe).  Outside [2^-480, 2^480) the exact routine runs.
__device__ __forceinline__ void givens_fast(double f, double g, double& cs, double& sn, double& r) {
  const unsigned long long bf = (unsigned long long)__double_as_longlong(f) & 0x7fffffffffffffffULL;
  const unsigned long long bg = (unsigned long long)__double_as_longlong(g) & 0x7fffffffffffffffULL;
  if (bg == 0) { cs = 1.0; sn = 0.0; r = f; return; }
  if (bf == 0) { cs = 0.0; sn = 1.0; r = g; return; }
  const unsigned long long bm = bf > bg ? bf : bg;
  if (bm >= 0x21F0000000000000ULL && bm < 0x5DF0000000000000ULL) {
    const double ss = fma(f, f, g * g);
    const double inv = rsqrt_nr(ss);
    double c = f * inv, s = g * inv, rr = ss * inv;
    if (bf > bg && __double_as_longlong(f) < 0) { c = -c; s = -s; rr = -rr; }
    cs = c; sn = s; r = rr;
    return;
  }
  givens_alg(f, g, cs, sn, r);
}

// _dgz_sym2x2 (symtridiag.jl:370-427)
__device__ void dgz_sym2x2(double a, double b, double c, bool wantvec, double& rt1, double& rt2, double& cs1,
                           double& sn1) {
  const double sm = a + c, df = a - c, adf = fabs(df), tb = 2.0 * b, ab = fabs(tb);
  double acmx, acmn;
  if (fabs(a) > fabs(c)) { acmx = a; acmn = c; } else { acmx = c; acmn = a; }
  const double rt = hypot(ab, adf);
  int sgn1;
  if (sm < 0.0) {
    rt1 = (sm - rt) / 2.0; sgn1 = -1;
    rt2 = (acmx / rt1) * acmn - (b / rt1) * b;
  } else if (sm > 0.0) {
    rt1 = (sm + rt) / 2.0; sgn1 = 1;
    rt2 = (acmx / rt1) * acmn - (b / rt1) * b;
  } else {
    rt1 = rt / 2.0; rt2 = -rt / 2.0; sgn1 = 1;
  }
  cs1 = 0.0; sn1 = 0.0;
  if (wantvec) {
    double cs;
    int sgn2;
    if (df > 0.0) { cs = df + rt; sgn2 = 1; } else { cs = df - rt; sgn2 = -1; }
    if (fabs(cs) > ab) {
      const double ct = -tb / cs;
      sn1 = 1.0 / sqrt(1.0 + ct * ct);
      cs1 = ct * sn1;
    } else if (ab == 0.0) {
      cs1 = 1.0; sn1 = 0.0;
    } else {
      const double tn = -cs / tb;
      cs1 = 1.0 / sqrt(1.0 + tn * tn);
      sn1 = tn * cs1;
    }
    if (sgn1 == sgn2) { const double tn = cs1; cs1 = -sn1; sn1 = tn; }
  }
}

// safescale! of x[0..len) by the lanes of one warp (each element gets the factors in order).
__device__ void safescale_vec(double* x, int len, double cfrom, double cto, int lane) {
  double mul[8];
  const int k = safescale_factors(cfrom, cto, mul);
  for (int i = lane; i < len; i += 32)
    for (int q = 0; q < k; ++q) x[i] *= mul[q];
  __syncwarp();
}

// State of the sweep machine (thread 0 only; persists across phases).
struct StState {
  int l1, l, lend, lsave, lendsave, iscale, mode;  // mode 0: next block, 1: QL, 2: QR
  double anorm;
  long long sweeps;
  int status;
};

// One emitted phase: count rotations (c, s) applied in order to the column pairs
// (i0 - k, i0 - k + 1) (dir = -1) or (i0 + k, i0 + k + 1) (dir = +1), 1-based.
struct StPhase {
  int i0, count, dir, done;
};

// Runs the state machine until it emits a phase of rotations (returns 1) or finishes
// (returns 0).  Executed by all 32 lanes of one warp with identical values (an FP64
// instruction costs the same for one lane or 32), so that the scans for splits and
// negligible off-diagonals test 32 positions per instruction (ballot, first hit); every
// lane stores the same values, so each lane reads back its own writes.  d, e 1-based
// through the macros.
__device__ int st_advance(StState& s, int n, double* __restrict__ d, double* __restrict__ e,
                          double* __restrict__ cb, double* __restrict__ sb, StPhase* ph, bool wantZ,
                          long long maxsweeps, int lane) {
#define D(i) d[(i) - 1]
#define E(i) e[(i) - 1]
  const unsigned FULL = 0xffffffffu;
  const double epsT = Prec<double>::eps, eps2 = epsT * epsT;
  const double safmin = Prec<double>::fmin, safmax = 1.0 / safmin;
  const double ssfmax = sqrt(safmax) / 3.0, ssfmin = sqrt(safmin) / eps2;
  for (;;) {
    if (s.mode == 0) {
      if (s.l1 > n) return 0;
      if (s.l1 > 1) E(s.l1 - 1) = 0.0;
      // _st_findsplit_fwd!: first m >= l1 with e[m] == 0 or negligible
      int msplit = n;
      for (int base = s.l1; base <= n - 1; base += 32) {
        const int m = base + lane;
        int hit = 0;
        if (m <= n - 1) {
          const double tst = fabs(E(m));
          if (tst == 0.0) hit = 1;
          else if (tst <= sqrt(fabs(D(m))) * sqrt(fabs(D(m + 1))) * epsT) hit = 2;
        }
        const unsigned bal = __ballot_sync(FULL, hit != 0);
        if (bal) {
          const int first = __ffs(bal) - 1;
          msplit = base + first;
          if (__shfl_sync(FULL, hit, first) == 2) E(msplit) = 0.0;
          break;
        }
      }
      s.l = s.l1;
      s.lsave = s.l;
      s.lend = msplit;
      s.lendsave = s.lend;
      s.l1 = msplit + 1;
      if (s.lend == s.l) continue;
      // opnorm(SymTridiagonal(d[l:lend], e[l:lend-1]), Inf)
      double an = 0.0;
      for (int i = s.l + lane; i <= s.lend; i += 32) {
        double t = fabs(D(i));
        if (i > s.l) t += fabs(E(i - 1));
        if (i < s.lend) t += fabs(E(i));
        if (t > an || t != t) an = t;
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_xor_sync(FULL, an, o);
        if (w > an || w != w) an = w;
      }
      s.anorm = an;
      s.iscale = 0;
      if (an == 0.0) continue;
      if (an > ssfmax) {
        s.iscale = 1;
        safescale_vec(&D(s.l), s.lend - s.l + 1, an, ssfmax, lane);
        safescale_vec(&E(s.l), s.lend - s.l, an, ssfmax, lane);
      } else if (an < ssfmin) {
        s.iscale = 2;
        safescale_vec(&D(s.l), s.lend - s.l + 1, an, ssfmin, lane);
        safescale_vec(&E(s.l), s.lend - s.l, an, ssfmin, lane);
      }
      if (fabs(D(s.lend)) < fabs(D(s.l))) { s.lend = s.lsave; s.l = s.lendsave; }
      s.mode = s.lend > s.l ? 1 : 2;
      continue;
    }
    if (s.mode == 1) {
      if (!(s.l <= s.lend)) {
        s.mode = 3;
        continue;
      }
      const int l = s.l, lend = s.lend;
      // first m in [l, lend) with a negligible e[m]
      int ms = lend;
      for (int base = l; base <= lend - 1; base += 32) {
        const int m = base + lane;
        bool hit = false;
        if (m <= lend - 1) {
          const double em = E(m);
          hit = em * em <= (eps2 * fabs(D(m))) * fabs(D(m + 1)) + safmin;
        }
        const unsigned bal = __ballot_sync(FULL, hit);
        if (bal) { ms = base + __ffs(bal) - 1; break; }
      }
      if (ms < lend) E(ms) = 0.0;
      double p = D(l);
      if (ms == l) {
        D(l) = p;
        s.l = l + 1;
        continue;
      }
      if (ms == l + 1) {
        double rt1, rt2, cs, sn;
        dgz_sym2x2(D(l), E(l), D(l + 1), wantZ, rt1, rt2, cs, sn);
        D(l) = rt1; D(l + 1) = rt2; E(l) = 0.0;
        s.l = l + 2;
        if (wantZ) { cb[0] = cs; sb[0] = sn; ph->i0 = l; ph->count = 1; ph->dir = -1; return 1; }
        continue;
      }
      if (++s.sweeps > maxsweeps) { s.status = 1; return 0; }
      double g = (D(l + 1) - p) / (2.0 * E(l));
      double r = hypot(g, 1.0);
      g = D(ms) - p + (E(l) / (g + copysign(r, g)));
      double sn = 1.0, c = 1.0;
      p = 0.0;
      int q = 0;
      double dn = D(ms);  // d[i+1] of the next step, carried
      for (int i = ms - 1; i >= l; --i, ++q) {
        const double ei = E(i), di = D(i);
        const double f = sn * ei, b = c * ei;
        givens_fast(g, f, c, sn, r);
        if (i < ms - 1) E(i + 1) = r;
        g = dn - p;
        r = fma(di - g, sn, 2.0 * c * b);
        p = sn * r;
        D(i + 1) = g + p;
        g = fma(c, r, -b);
        dn = di;
        if (wantZ) { cb[q] = c; sb[q] = -sn; }
      }
      D(l) -= p;
      E(l) = g;
      if (wantZ) { ph->i0 = ms - 1; ph->count = ms - l; ph->dir = -1; return 1; }
      continue;
    }
    if (s.mode == 2) {
      if (!(s.l >= s.lend)) {
        s.mode = 3;
        continue;
      }
      const int l = s.l, lend = s.lend;
      // first m in (lend, l], descending, with a negligible e[m-1]
      int ms = lend;
      for (int top = l; top >= lend + 1; top -= 32) {
        const int m = top - lane;
        bool hit = false;
        if (m >= lend + 1) {
          const double em = E(m - 1);
          hit = em * em <= (eps2 * fabs(D(m))) * fabs(D(m - 1)) + safmin;
        }
        const unsigned bal = __ballot_sync(FULL, hit);
        if (bal) { ms = top - (__ffs(bal) - 1); break; }
      }
      if (ms > lend) E(ms - 1) = 0.0;
      double p = D(l);
      if (ms == l) {
        D(l) = p;
        s.l = l - 1;
        continue;
      }
      if (ms == l - 1) {
        double rt1, rt2, cs, sn;
        dgz_sym2x2(D(l - 1), E(l - 1), D(l), wantZ, rt1, rt2, cs, sn);
        D(l - 1) = rt1; D(l) = rt2; E(l - 1) = 0.0;
        s.l = l - 2;
        if (wantZ) { cb[0] = cs; sb[0] = sn; ph->i0 = ms; ph->count = 1; ph->dir = 1; return 1; }
        continue;
      }
      if (++s.sweeps > maxsweeps) { s.status = 1; return 0; }
      double g = (D(l - 1) - p) / (2.0 * E(l - 1));
      double r = hypot(g, 1.0);
      g = D(ms) - p + (E(l - 1) / (g + copysign(r, g)));
      double sn = 1.0, c = 1.0;
      p = 0.0;
      int q = 0;
      double dc = D(ms);  // d[i] of the next step, carried
      for (int i = ms; i <= l - 1; ++i, ++q) {
        const double ei = E(i), dn = D(i + 1);
        const double f = sn * ei, b = c * ei;
        givens_fast(g, f, c, sn, r);
        if (i != ms) E(i - 1) = r;
        g = dc - p;
        r = fma(dn - g, sn, 2.0 * c * b);
        p = sn * r;
        D(i) = g + p;
        g = fma(c, r, -b);
        dc = dn;
        if (wantZ) { cb[q] = c; sb[q] = sn; }
      }
      D(l) -= p;
      E(l - 1) = g;
      if (wantZ) { ph->i0 = ms; ph->count = l - ms; ph->dir = 1; return 1; }
      continue;
    }
    // mode 3: the block is done; undo its scaling
    if (s.iscale == 1) {
      safescale_vec(&D(s.lsave), s.lendsave - s.lsave + 1, ssfmax, s.anorm, lane);
      safescale_vec(&E(s.lsave), s.lendsave - s.lsave, ssfmax, s.anorm, lane);
    } else if (s.iscale == 2) {
      safescale_vec(&D(s.lsave), s.lendsave - s.lsave + 1, ssfmin, s.anorm, lane);
      safescale_vec(&E(s.lsave), s.lendsave - s.lsave, ssfmin, s.anorm, lane);
    }
    s.mode = 0;
  }
#undef D
#undef E
}

// Grid barrier for a cooperative launch (all blocks resident): arrival counter and a
// generation word; the wait gives up after ~4 s and raises err.
__device__ void grid_barrier(unsigned* count, unsigned* gen, unsigned nblocks, int* err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = gen;
    const unsigned g = *vgen;
    __threadfence();
    if (atomicAdd(count, 1u) == nblocks - 1) {
      *count = 0;
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      long long it = 0;
      while (*vgen == g) {
        if (++it > (1LL << 25)) { atomicOr(err, 1); break; }
        __nanosleep(128);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

struct StCtl {
  unsigned count, gen;
  int err;
  int done;        // set by the sweep thread
  int status;
  StPhase ph[2];
};

// Apply one phase of rotations to row r of Z (n columns, ld ldz).
template <class S>
__device__ __forceinline__ void apply_phase(S* Z, long long ldz, int r, const StPhase& p, const double* cb,
                                            const double* sb) {
  using O = Hs<S>;
  if (p.count <= 0) return;
  S* z = Z + r;
  if (p.dir < 0) {
    S carry = z[(size_t)p.i0 * ldz];  // column i0 + 1 (1-based)
    for (int q = 0; q < p.count; ++q) {
      const int i = p.i0 - q;  // rotation on (i, i+1), 1-based
      const S a = z[(size_t)(i - 1) * ldz];
      const double c = cb[q], s = sb[q];
      const S ni = O::add(O::scal(a, c), O::scal(carry, s));
      const S ni1 = O::sub(O::scal(carry, c), O::scal(a, s));
      z[(size_t)i * ldz] = ni1;
      carry = ni;
    }
    z[(size_t)(p.i0 - p.count) * ldz] = carry;
  } else {
    S carry = z[(size_t)(p.i0 - 1) * ldz];  // column i0
    for (int q = 0; q < p.count; ++q) {
      const int i = p.i0 + q;
      const S b = z[(size_t)i * ldz];
      const double c = cb[q], s = sb[q];
      const S ni = O::add(O::scal(carry, c), O::scal(b, s));
      const S ni1 = O::sub(O::scal(b, c), O::scal(carry, s));
      z[(size_t)(i - 1) * ldz] = ni;
      carry = ni1;
    }
    z[(size_t)(p.i0 + p.count - 1) * ldz] = carry;
  }
}

// The cooperative sweep kernel.  rot: 2 buffers x 2 x n doubles (c, s).
// With smem_de (2 n doubles of dynamic shared memory), d and e live in shared memory
// during the iteration: the recurrence reads them at every step.
template <class S>
__global__ void __launch_bounds__(kHeT) k_steqr(int n, double* dg, double* eg, S* Z, long long ldz, int nz,
                                                 double* rot, StCtl* ctl, long long maxsweeps, int smem_de) {
  extern __shared__ double sde[];
  const bool wantZ = Z != nullptr && nz > 0;
  const bool chain = blockIdx.x == 0 && threadIdx.x < 32;  // warp 0 of block 0, lanes in lockstep
  const int lane = threadIdx.x & 31;
  double* d = dg;
  double* e = eg;
  StState st;
  if (chain) {
    st.l1 = 1; st.l = 0; st.lend = 0; st.lsave = 0; st.lendsave = 0; st.iscale = 0; st.mode = 0;
    st.anorm = 0.0; st.sweeps = 0; st.status = 0;
    if (smem_de) {
      d = sde;
      e = sde + n;
      for (int i = lane; i < n; i += 32) { d[i] = dg[i]; e[i] = i < n - 1 ? eg[i] : 0.0; }
      __syncwarp();
    }
  }
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nzt = (long long)gridDim.x * blockDim.x - 32;  // warp 0 of block 0 runs the chain
  bool finished = false;
  for (int k = 0;; ++k) {
    const int b = k & 1;
    if (chain) {
      StPhase* ph = &ctl->ph[b];
      if (!finished) {
        const int emitted = st_advance(st, n, d, e, rot + (size_t)b * 2 * n, rot + (size_t)b * 2 * n + n, ph, wantZ,
                                       maxsweeps, lane);
        if (!emitted) {
          finished = true;
          ph->count = 0;
          ctl->status = st.status;
          if (smem_de) {
            __syncwarp();
            for (int i = lane; i < n; i += 32) { dg[i] = d[i]; if (i < n - 1) eg[i] = e[i]; }
          }
        }
      } else {
        ph->count = 0;
      }
      ph->done = finished ? 1 : 0;
      __threadfence();
    }
    if (wantZ && k >= 1 && gtid >= 32) {
      const int pb = b ^ 1;
      const StPhase p = ctl->ph[pb];
      const double* cb = rot + (size_t)pb * 2 * n;
      const double* sb = cb + n;
      for (long long r = gtid - 32; r < nz; r += nzt) apply_phase<S>(Z, ldz, (int)r, p, cb, sb);
    }
    if (!wantZ) {
      if (chain) ctl->done = 1;
      return;  // one thread did all the work
    }
    grid_barrier(&ctl->count, &ctl->gen, gridDim.x, &ctl->err);
    const volatile StCtl* vc = ctl;
    if (vc->err) return;
    // phase k's buffer was emitted empty and phase k-1's is applied: done
    if (vc->ph[b].done && vc->ph[b].count == 0) return;
  }
}

// The QR iteration on many small independent tridiagonals at once (the leaves of a
// divide-and-conquer tree, symtri_dc.jl:145-168, and its small isolated blocks): one warp
// per problem, d and e in shared memory, the rotations of each emitted phase applied to
// the problem's diagonal block of Q (rows of the block = lanes) right away.  Q's block is
// set to the identity first; the rest of Q is not touched.
constexpr int kLeafMax = 64;
constexpr int kLeafWarps = 4;
__global__ void __launch_bounds__(32 * kLeafWarps) k_steqr_leaves(int nprob, const int* __restrict__ off,
                                                                  const int* __restrict__ msz, double* dg, double* eg,
                                                                  double* Q, long long ldq, int wantq, int* status) {
  __shared__ double sd[kLeafWarps][kLeafMax + 1], se[kLeafWarps][kLeafMax + 1];
  __shared__ double scb[kLeafWarps][kLeafMax], ssb[kLeafWarps][kLeafMax];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * kLeafWarps + wid;
  if (b >= nprob) return;
  const int o = off[b], m = msz[b];
  double* d = sd[wid];
  double* e = se[wid];
  for (int i = lane; i <= m; i += 32) {
    d[i] = i < m ? dg[o + i] : 0.0;
    e[i] = i < m - 1 ? eg[o + i] : 0.0;
  }
  double* Qb = wantq ? Q + o + (size_t)o * ldq : nullptr;
  if (wantq)
    for (int c = 0; c < m; ++c)
      for (int r = lane; r < m; r += 32) Qb[r + (size_t)c * ldq] = r == c ? 1.0 : 0.0;
  __syncwarp();
  StState st;
  st.l1 = 1; st.l = 0; st.lend = 0; st.lsave = 0; st.lendsave = 0; st.iscale = 0; st.mode = 0;
  st.anorm = 0.0; st.sweeps = 0; st.status = 0;
  StPhase ph;
  ph.i0 = 0; ph.count = 0; ph.dir = 0; ph.done = 0;
  const long long maxsweeps = 30LL * m;
  for (;;) {
    const int emitted = st_advance(st, m, d, e, scb[wid], ssb[wid], &ph, wantq != 0, maxsweeps, lane);
    __syncwarp();
    if (!emitted) break;
    for (int r = lane; r < m; r += 32) apply_phase<double>(Qb, ldq, r, ph, scb[wid], ssb[wid]);
    __syncwarp();
  }
  for (int i = lane; i < m; i += 32) {
    dg[o + i] = d[i];
    if (i < m - 1) eg[o + i] = e[i];
  }
  if (lane == 0 && st.status) atomicOr(status, 2);
}

int grid_of(size_t work) { return (int)std::min<size_t>((work + 255) / 256, 4096); }

}  // namespace

template <class S>
cudaError_t launch_he_tridiag(const S* A, long long lda, int n, int upper, S* B, S* W, S* partial, int npart,
                              HeCtlBuf* cbuf, S* tau, double* d, double* e, int num_sms, cudaStream_t s) {
  HeCtl<S>* ctl = reinterpret_cast<HeCtl<S>*>(cbuf);
  k_he_prep<S><<<grid_of((size_t)n * n), 256, 0, s>>>(A, lda, n, upper, B);
  cudaError_t err = cudaMemsetAsync(ctl, 0, sizeof(HeCtl<S>), s);
  if (err != cudaSuccess) return err;
  k_he_first<S><<<1, kHeT, 0, s>>>(B, n, ctl, tau, d, e);
  for (int i = 0; i <= n - 2; ++i) {
    const int m = n - 1 - i;
    const int gmv = std::max(1, std::min(npart, (m + 7) / 8));
    k_he_matvec<S><<<gmv, kHeT, 0, s>>>(B, n, i, W, partial, ctl);
    const int gup = std::max(1, std::min(4 * num_sms, m));
    k_he_update<S><<<gup, kHeT, 0, s>>>(B, n, i, W, ctl, tau, d, e);
  }
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_he_formq(const S* B, int n, const S* tau, S* Q, int num_sms, cudaStream_t s) {
  k_he_identity<S><<<grid_of((size_t)n * n), 256, 0, s>>>(Q, n);
  for (int i = n - 2; i >= 0; --i) {
    const int m = n - 1 - i;
    const int g = std::max(1, std::min(4 * num_sms, (m + 7) / 8));
    k_he_formq<S><<<g, kHeT, 0, s>>>(B, n, i, tau, Q);
  }
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_he_store(const S* B, int n, int upper, S* A, long long lda, cudaStream_t s) {
  k_he_store<S><<<grid_of((size_t)n * n), 256, 0, s>>>(B, n, upper, A, lda);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_he_gather(const S* Z, int n, const int* p, int rev, S* V, long long ldv, cudaStream_t s) {
  k_he_gather<S><<<grid_of((size_t)n * n), 256, 0, s>>>(Z, n, p, rev, V, ldv);
  return cudaGetLastError();
}

size_t steqr_ctl_bytes() { return sizeof(StCtl); }

cudaError_t launch_steqr_leaves(int nprob, const int* off, const int* msz, int maxm, double* d, double* e, double* Q,
                                long long ldq, int wantq, int* status, cudaStream_t s) {
  if (nprob == 0) return cudaSuccess;
  if (maxm > kLeafMax) return cudaErrorInvalidValue;
  k_steqr_leaves<<<(nprob + kLeafWarps - 1) / kLeafWarps, 32 * kLeafWarps, 0, s>>>(nprob, off, msz, d, e, Q, ldq, wantq,
                                                                                  status);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_steqr(int n, double* d, double* e, S* Z, long long ldz, int nz, double* rot, void* ctl,
                         long long maxsweeps, int num_sms, cudaStream_t s) {
  cudaError_t err = cudaMemsetAsync(ctl, 0, sizeof(StCtl), s);
  if (err != cudaSuccess) return err;
  StCtl* c = reinterpret_cast<StCtl*>(ctl);
  // d, e in shared memory when they fit
  int smem_de = (size_t)2 * n * sizeof(double) <= 200 * 1024 ? 1 : 0;
  const size_t smem = smem_de ? (size_t)2 * n * sizeof(double) : 0;
  static size_t attr_set = 0;
  if (smem > 48 * 1024 && attr_set < smem) {
    err = cudaFuncSetAttribute(k_steqr<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (err != cudaSuccess) return err;
    attr_set = 200 * 1024;
  }
  if (Z == nullptr || nz == 0) {
    k_steqr<S><<<1, 32, smem, s>>>(n, d, e, nullptr, 0, 0, rot, c, maxsweeps, smem_de);
    return cudaGetLastError();
  }
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_steqr<S>, kHeT, smem);
  if (err != cudaSuccess) return err;
  int blocks = (int)std::min<long long>(((long long)nz + 32 + kHeT - 1) / kHeT, (long long)num_sms * std::max(per_sm, 1));
  blocks = std::max(blocks, 1);
  void* args[] = {&n, &d, &e, &Z, &ldz, &nz, &rot, &c, &maxsweeps, &smem_de};
  return cudaLaunchCooperativeKernel((const void*)k_steqr<S>, dim3(blocks), dim3(kHeT), args, smem, s);
}

#define GS_HE_INST(S)                                                                                                 \
  template cudaError_t launch_he_tridiag<S>(const S*, long long, int, int, S*, S*, S*, int, HeCtlBuf*, S*, double*,    \
                                            double*, int, cudaStream_t);                                              \
  template cudaError_t launch_he_formq<S>(const S*, int, const S*, S*, int, cudaStream_t);                            \
  template cudaError_t launch_he_store<S>(const S*, int, int, S*, long long, cudaStream_t);                           \
  template cudaError_t launch_he_gather<S>(const S*, int, const int*, int, S*, long long, cudaStream_t);              \
  template cudaError_t launch_steqr<S>(int, double*, double*, S*, long long, int, double*, void*, long long, int,      \
                                       cudaStream_t);
GS_HE_INST(double)
GS_HE_INST(double2)
#undef GS_HE_INST

}  // namespace gsk
