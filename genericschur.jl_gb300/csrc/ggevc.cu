// Eigenvectors of a complex generalized Schur pair (S, P upper triangular, P with a real
// diagonal): geigvecs(S::GeneralizedSchur; left) (vectors.jl:22-33) with the reference's
// ztgevc restatements _geigvecs (right, vectors.jl:723-842) and _gleigvecs (left,
// vectors.jl:845-1038).
//
// For eigenvalue k the coefficients (a, b) of (a S - b P) x = 0 are scaled against
// under/overflow, then a triangular solve with the diagonal floored at dmin and the
// reference's rescaling of the partial solution; the result is back-transformed by Z
// (right) or Q (left) and scaled to max |re| + |im| = 1.
//
// One thread per eigenvector, CTAs over blocks of eigenvectors.  All threads of a CTA step
// through the columns j in the same order, so every read of S, P and the back-transform
// matrix is a broadcast; a thread whose eigenvector does not involve column j is masked.
// The partial solutions live in a scratch array with one row per index i, so a warp's
// accesses to it are coalesced.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kGgT = 64;

#define SS(i, j) S[((i) - 1) + (size_t)((j) - 1) * n]
#define PP(i, j) P[((i) - 1) + (size_t)((j) - 1) * n]
#define XX(i) X[(size_t)((i) - 1) * n + col]

// Column 1-norms of the strictly upper parts (snorms, pnorms) and the largest column
// norm including the diagonal (anorm, bnorm as IEEE bits, atomicMax) -- vectors.jl:752-762.
__global__ void k_gg_norms(int n, const double2* __restrict__ S, const double2* __restrict__ P,
                           double* __restrict__ sn, double* __restrict__ pn, unsigned long long* __restrict__ ab) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > n) return;
  double s = 0.0, p = 0.0;
  for (int i = 1; i <= j - 1; ++i) {
    s += zabs1(SS(i, j));
    p += zabs1(PP(i, j));
  }
  sn[j - 1] = s;
  pn[j - 1] = p;
  const double a = (j == 1) ? zabs1(SS(1, 1)) : s + zabs1(SS(j, j));
  const double b = (j == 1) ? zabs1(PP(1, 1)) : p + zabs1(PP(j, j));
  atomicMax(ab, (unsigned long long)__double_as_longlong(a));
  atomicMax(ab + 1, (unsigned long long)__double_as_longlong(b));
}

struct GgCoef {
  double acoeff;
  double2 bcoeff;
  bool ok;  // false: singular pencil (unit eigenvector)
};

// vectors.jl:775-812 (right) / 930-967 (left)
__device__ GgCoef gg_coeffs(int n, const double2* S, const double2* P, int k, double anorm, double bnorm) {
  const double ulp = kEps, safmin = kSafemin;
  const double smallnum = safmin * ((double)n / ulp);
  const double bigx = 1.0 / smallnum;
  const double ascale = 1.0 / fmax(anorm, safmin), bscale = 1.0 / fmax(bnorm, safmin);
  GgCoef c;
  const double2 skk = SS(k, k);
  const double pkk = PP(k, k).x;
  if (zabs1(skk) <= safmin && fabs(pkk) <= safmin) {
    c.ok = false;
    c.acoeff = 0.0;
    c.bcoeff = make_double2(0.0, 0.0);
    return c;
  }
  const double t = 1.0 / fmax(fmax(zabs1(skk) * ascale, fabs(pkk) * bscale), safmin);
  const double2 salpha = zscal(zscal(skk, t), ascale);
  const double sbeta = (t * pkk) * bscale;
  double ac = sbeta * ascale;
  double2 bc = zscal(salpha, bscale);
  const bool lsa = fabs(sbeta) >= safmin && fabs(ac) < smallnum;
  const bool lsb = zabs1(salpha) >= safmin && zabs1(bc) < smallnum;
  double s = 1.0;
  if (lsa) s = (smallnum / fabs(sbeta)) * fmin(anorm, bigx);
  if (lsb) s = fmax(s, (smallnum / zabs1(salpha)) * fmin(bnorm, bigx));
  if (lsa || lsb) {
    s = fmin(s, 1.0 / (safmin * fmax(fmax(1.0, fabs(ac)), zabs1(bc))));
    ac = lsa ? ascale * (s * sbeta) : ac * s;
    bc = lsb ? zscal(zscal(salpha, s), bscale) : zscal(bc, s);
  }
  c.ok = true;
  c.acoeff = ac;
  c.bcoeff = bc;
  return c;
}

// a S[i,j] - b P[i,j]
__device__ __forceinline__ double2 gg_comb(double a, double2 b, double2 s, double2 p) {
  return zfms(b, p, zscal(s, a));
}

// Right eigenvector ki = col + 1: solution into X (column col), sing[col] on a singular pencil.
__global__ void __launch_bounds__(kGgT) k_ggevc_right(int n, const double2* __restrict__ S,
                                                     const double2* __restrict__ P, const double* __restrict__ sn,
                                                     const double* __restrict__ pn,
                                                     const unsigned long long* __restrict__ ab,
                                                     double2* __restrict__ X, int* __restrict__ sing) {
  const int col = blockIdx.x * kGgT + threadIdx.x;
  const int ki = col + 1;
  const bool live_t = col < n;
  const double anorm = __longlong_as_double((long long)ab[0]), bnorm = __longlong_as_double((long long)ab[1]);
  const double ulp = kEps, safmin = kSafemin;
  const double bignum = 1.0 / ((double)n * safmin);
  GgCoef c;
  c.ok = false;
  if (live_t) c = gg_coeffs(n, S, P, ki, anorm, bnorm);
  if (live_t) sing[col] = c.ok ? 0 : 1;
  const bool act = live_t && c.ok;
  const double aca = fabs(c.acoeff), acb = zabs1(c.bcoeff);
  const double dmin = fmax(fmax(ulp * aca * anorm, ulp * acb * bnorm), safmin);
  if (act) {
    for (int i = 1; i <= n; ++i)
      XX(i) = (i < ki) ? gg_comb(c.acoeff, c.bcoeff, SS(i, ki), PP(i, ki)) : make_double2(i == ki ? 1.0 : 0.0, 0.0);
  }
  // all threads of the CTA walk j = (largest ki of the CTA) - 1 .. 1
  const int kmax = min(n, (int)(blockIdx.x + 1) * kGgT);
  for (int j = kmax - 1; j >= 1; --j) {
    const bool on = act && j < ki;
    const double2 sjj = SS(j, j), pjj = PP(j, j);
    double2 ca = make_double2(0.0, 0.0), cb = ca;
    if (on) {
      double2 d = gg_comb(c.acoeff, c.bcoeff, sjj, pjj);
      if (zabs1(d) <= dmin) d = make_double2(dmin, 0.0);
      double2 vj = XX(j);
      if (zabs1(d) < 1.0 && zabs1(vj) >= bignum * zabs1(d)) {
        const double t = 1.0 / zabs1(vj);
        for (int i = 1; i <= ki; ++i) XX(i) = zscal(XX(i), t);
        vj = XX(j);
      }
      vj = zdiv(zneg(vj), d);
      XX(j) = vj;
      if (j > 1) {
        if (zabs1(vj) > 1.0) {
          const double t = 1.0 / zabs1(vj);
          if (aca * sn[j - 1] + acb * pn[j - 1] >= bignum * t) {
            for (int i = 1; i <= ki; ++i) XX(i) = zscal(XX(i), t);
            vj = XX(j);
          }
        }
        ca = zscal(vj, c.acoeff);
        cb = zmul(c.bcoeff, vj);
      }
    }
    if (j > 1) {
      for (int i = 1; i <= j - 1; ++i) {
        const double2 sij = SS(i, j), pij = PP(i, j);
        if (on) XX(i) = zadd(XX(i), zsub(zmul(ca, sij), zmul(cb, pij)));
      }
    }
  }
}

// Left eigenvector je = col + 1.
__global__ void __launch_bounds__(kGgT) k_ggevc_left(int n, const double2* __restrict__ S,
                                                    const double2* __restrict__ P, const double* __restrict__ sn,
                                                    const double* __restrict__ pn,
                                                    const unsigned long long* __restrict__ ab,
                                                    double2* __restrict__ X, int* __restrict__ sing) {
  const int col = blockIdx.x * kGgT + threadIdx.x;
  const int je = col + 1;
  const bool live_t = col < n;
  const double anorm = __longlong_as_double((long long)ab[0]), bnorm = __longlong_as_double((long long)ab[1]);
  const double ulp = kEps, safmin = kSafemin;
  const double bignum = 1.0 / ((double)n * safmin);
  GgCoef c;
  c.ok = false;
  if (live_t) c = gg_coeffs(n, S, P, je, anorm, bnorm);
  if (live_t) sing[col] = c.ok ? 0 : 1;
  const bool act = live_t && c.ok;
  const double aca = fabs(c.acoeff), acb = zabs1(c.bcoeff);
  const double dmin = fmax(fmax(ulp * aca * anorm, ulp * acb * bnorm), safmin);
  double xmax = 1.0;
  if (act)
    for (int i = 1; i <= n; ++i) XX(i) = make_double2(i == je ? 1.0 : 0.0, 0.0);
  const int jmin = blockIdx.x * kGgT + 2;  // smallest je of the CTA + 1
  for (int j = jmin; j <= n; ++j) {
    const bool on = act && j > je;
    if (on) {
      const double t = 1.0 / xmax;
      if (aca * sn[j - 1] + acb * pn[j - 1] > bignum * t) {
        for (int r = je; r <= j - 1; ++r) XX(r) = zscal(XX(r), t);
        xmax = 1.0;
      }
    }
    double2 suma = make_double2(0.0, 0.0), sumb = suma;
    for (int jr = jmin - 1; jr <= j - 1; ++jr) {
      const double2 s = SS(jr, j), p = PP(jr, j);
      if (on && jr >= je) {
        const double2 x = XX(jr);
        suma = zfmac(s, x, suma);
        sumb = zfmac(p, x, sumb);
      }
    }
    if (on) {
      double2 sumx = zsub(zscal(suma, c.acoeff), zmul(zconj(c.bcoeff), sumb));
      double2 d = zconj(gg_comb(c.acoeff, c.bcoeff, SS(j, j), PP(j, j)));
      if (zabs1(d) <= dmin) d = make_double2(dmin, 0.0);
      if (zabs1(d) < 1.0 && zabs1(sumx) >= bignum * zabs1(d)) {
        const double t = 1.0 / zabs1(sumx);
        for (int r = je; r <= j - 1; ++r) XX(r) = zscal(XX(r), t);
        xmax *= t;
        sumx = zscal(sumx, t);
      }
      const double2 xj = zdiv(zneg(sumx), d);
      XX(j) = xj;
      xmax = fmax(xmax, zabs1(xj));
    }
  }
}

// Back-transform (V = M X, M = Z or Q, when given) and scaling to max |re|+|im| = 1
// (vectors.jl:823-839 / 1019-1035).  V column-major, ld n.
__global__ void __launch_bounds__(kGgT) k_ggevc_back(int n, const double2* __restrict__ X,
                                                    const double2* __restrict__ M, const int* __restrict__ sing,
                                                    int left, double2* __restrict__ V) {
  const int col = blockIdx.x * kGgT + threadIdx.x;
  const bool live_t = col < n;
  const int k = col + 1;
  const bool sg = live_t && sing[col];
  const double safmin = kSafemin;
  // range of X's nonzero rows: right 1..k, left k..n
  const int lo = left ? k : 1, hi = left ? n : k;
  // rows of the result that are written: all with M, else the same range
  const int r0 = M ? 1 : lo, r1 = M ? n : hi;
  const int klo = blockIdx.x * kGgT + 1, khi = min(n, (int)(blockIdx.x + 1) * kGgT);
  double xmax = 0.0;
  if (M) {
    // lockstep over rows r and inner index q: M[r, q] is a broadcast
    const int qlo = left ? klo : 1, qhi = left ? n : khi;
    for (int r = 1; r <= n; ++r) {
      double2 acc = make_double2(0.0, 0.0);
      for (int q = qlo; q <= qhi; ++q) {
        const double2 m = M[(r - 1) + (size_t)(q - 1) * n];
        if (live_t && !sg && q >= lo && q <= hi) acc = zfma(m, XX(q), acc);
      }
      if (live_t && !sg) {
        V[(r - 1) + (size_t)col * n] = acc;
        xmax = fmax(xmax, zabs1(acc));
      }
    }
  } else if (live_t && !sg) {
    for (int r = lo; r <= hi; ++r) {
      const double2 x = XX(r);
      V[(r - 1) + (size_t)col * n] = x;
      xmax = fmax(xmax, zabs1(x));
    }
  }
  if (!live_t) return;
  double2* vc = V + (size_t)col * n;
  if (sg) {
    for (int r = 1; r <= n; ++r) vc[r - 1] = make_double2(r == k ? 1.0 : 0.0, 0.0);
    return;
  }
  if (xmax > safmin) {
    const double t = 1.0 / xmax;
    for (int r = r0; r <= r1; ++r) vc[r - 1] = zscal(vc[r - 1], t);
    for (int r = 1; r < r0; ++r) vc[r - 1] = make_double2(0.0, 0.0);
    for (int r = r1 + 1; r <= n; ++r) vc[r - 1] = make_double2(0.0, 0.0);
  } else {
    for (int r = 1; r <= n; ++r) vc[r - 1] = make_double2(0.0, 0.0);
  }
}

#undef SS
#undef PP
#undef XX

}  // namespace

// Workspace bytes of launch_ggevc for order n.
size_t ggevc_ws_bytes(int n) {
  return (size_t)n * n * sizeof(double2) + 2 * (size_t)n * sizeof(double) + (size_t)n * sizeof(int) + 1024;
}

cudaError_t launch_ggevc(int n, const double2* S, const double2* P, const double2* M, int left, double2* V, void* ws,
                         cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  char* w = static_cast<char*>(ws);
  double2* X = reinterpret_cast<double2*>(w);
  w += (size_t)n * n * sizeof(double2);
  double* sn = reinterpret_cast<double*>(w);
  double* pn = sn + n;
  w += 2 * (size_t)n * sizeof(double);
  int* sing = reinterpret_cast<int*>(w);
  w += (size_t)n * sizeof(int);
  w = reinterpret_cast<char*>(((uintptr_t)w + 15) & ~uintptr_t(15));
  unsigned long long* ab = reinterpret_cast<unsigned long long*>(w);
  cudaError_t e = cudaMemsetAsync(ab, 0, 2 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  k_gg_norms<<<(n + 127) / 128, 128, 0, s>>>(n, S, P, sn, pn, ab);
  const int g = (n + kGgT - 1) / kGgT;
  if (left) k_ggevc_left<<<g, kGgT, 0, s>>>(n, S, P, sn, pn, ab, X, sing);
  else k_ggevc_right<<<g, kGgT, 0, s>>>(n, S, P, sn, pn, ab, X, sing);
  k_ggevc_back<<<g, kGgT, 0, s>>>(n, X, M, sing, left, V);
  return cudaGetLastError();
}

}  // namespace gsk
