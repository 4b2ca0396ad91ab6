// Eigenvectors from complex Schur factors, batched, one CTA per matrix.
//
// Right eigenvectors follow _geigvecs! (vectors.jl:45-131): for eigenvalue ki,
// solve (T[1:ki-1,1:ki-1] - T[ki,ki] I) x = -T[1:ki-1, ki] with the diagonal floored
// at smin and xLATRS-style overflow protection (_usolve!, util.jl:128-293), then
// v = Z[:, 1:ki] [x; scale], normalised by its largest |re|+|im| and finally by
// _enormalize! (util.jl:572-592).  Left eigenvectors follow _gleigvecs!
// (vectors.jl:372-460) with the conjugate-transposed solve (_cusolve!,
// util.jl:301-461).
//
// One thread per eigenvector.  All threads step through the columns j of T in
// the same order, so every read of T is a shared-memory broadcast; a thread whose
// eigenvalue does not involve column j is masked.  The rare systems whose growth
// bound fails (xLATRS "careful" branch) are solved afterwards by their own thread
// with the full scaling logic.  The triangular solutions X live in shared memory
// (n <= kEigSmem) or in a global scratch buffer, one row per i so that a warp's
// accesses are coalesced; V = Z X follows with each thread owning one row of V.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr double kHalf = 0.5;

__device__ __forceinline__ double cabs1half(double2 z) { return fabs(z.x * 0.5) + fabs(z.y * 0.5); }

// Shifted, floored diagonal entry: T[j,j] - lam, replaced by smin if smaller in abs1.
__device__ __forceinline__ double2 shifted_diag(double2 tjj, double2 lam, double smin) {
  double2 d = zsub(tjj, lam);
  if (zabs1(d) < smin) d = make_double2(smin, 0.0);
  return d;
}

// T is stored packed upper-triangular: column j (1-based) holds rows 1..j.
#define TT(i, j) T[((((j) - 1) * (j)) >> 1) + (i) - 1]
#define XX(i) X[((i) - 1) * ldx]

// Careful branch of _usolve! for one thread (util.jl:194-286), solving with the
// shifted diagonal; x = thread's column of X (stride ldx); returns xscale.
__device__ double usolve_careful(const double2* T, int ldt, int m, double2 lam, double smin, double2* X, int ldx,
                                 const double* cnorm, double tscale, double xmax) {
  const double smallnum = kSafemin / kEps;
  const double bignum = 1.0 / smallnum;
  double xscale = 1.0;
  if (xmax > bignum * kHalf) {
    xscale = (bignum * kHalf) / xmax;
    for (int i = 1; i <= m; ++i) XX(i) = zscal(XX(i), xscale);
    xmax = bignum;
  } else {
    xmax *= 2.0;
  }
  for (int j = m; j >= 1; --j) {
    double xj = zabs1(XX(j));
    const double2 tjjs = zscal(shifted_diag(TT(j, j), lam, smin), tscale);
    const double tjj = zabs1(tjjs);
    const double cn = cnorm[j - 1] * tscale;
    if (tjj > smallnum) {
      if (tjj < 1.0 && xj > tjj * bignum) {
        const double rec = 1.0 / xj;
        for (int i = 1; i <= m; ++i) XX(i) = zscal(XX(i), rec);
        xscale *= rec;
        xmax *= rec;
      }
      XX(j) = zdiv(XX(j), tjjs);
      xj = zabs1(XX(j));
    } else if (tjj > 0.0) {
      if (xj > tjj * bignum) {
        double rec = (tjj * bignum) / xj;
        if (cn > 1.0) rec /= cn;
        for (int i = 1; i <= m; ++i) XX(i) = zscal(XX(i), rec);
        xscale *= rec;
        xmax *= rec;
      }
      XX(j) = zdiv(XX(j), tjjs);
      xj = zabs1(XX(j));
    } else {
      for (int i = 1; i <= m; ++i) XX(i) = make_double2(0.0, 0.0);
      XX(j) = make_double2(1.0, 0.0);
      xscale = 0.0;
      xmax = 0.0;
    }
    if (xj > 1.0) {
      double rec = 1.0 / xj;
      if (cn > (bignum - xmax) * rec) {
        rec *= kHalf;
        for (int i = 1; i <= m; ++i) XX(i) = zscal(XX(i), rec);
        xscale *= rec;
      }
    } else if (xj * cn > bignum - xmax) {
      for (int i = 1; i <= m; ++i) XX(i) = zscal(XX(i), kHalf);
      xscale *= kHalf;
    }
    if (j > 1) {
      const double2 xjt = zscal(XX(j), tscale);
      for (int i = 1; i <= j - 1; ++i) XX(i) = zfms(xjt, TT(i, j), XX(i));
      xmax = zabs1(XX(1));
      for (int i = 2; i <= j - 1; ++i) xmax = fmax(xmax, zabs1(XX(i)));
    }
  }
  return xscale / tscale;
}

// Careful branch of _cusolve! (util.jl:368-454) on the trailing block starting at
// global index g0 = ki+1; local index j maps to global g0 + j - 1.
__device__ double cusolve_careful(const double2* T, int ldt, int g0, int m, double2 lam, double smin, double2* X,
                                  int ldx, const double* cnorm, double tscale, double xmax) {
  const double smallnum = kSafemin / kEps;
  const double bignum = 1.0 / smallnum;
  double xscale = 1.0;
#define XL(j) X[((g0) + (j) - 2) * ldx]
#define TL(i, j) TT((g0) + (i) - 1, (g0) + (j) - 1)
  if (xmax > bignum * kHalf) {
    xscale = (bignum * kHalf) / xmax;
    for (int i = 1; i <= m; ++i) XL(i) = zscal(XL(i), xscale);
    xmax = bignum;
  } else {
    xmax *= 2.0;
  }
  for (int j = 1; j <= m; ++j) {
    double xj = zabs1(XL(j));
    double2 uscale = make_double2(tscale, 0.0);
    double rec = 1.0 / fmax(xmax, 1.0);
    const double cn = cnorm[j - 1] * tscale;
    double2 tjjs = zscal(zconj(shifted_diag(TL(j, j), lam, smin)), tscale);
    if (cn > (bignum - xj) * rec) {
      rec *= kHalf;
      const double tjj = zabs1(tjjs);
      if (tjj > 1.0) {
        rec = fmin(1.0, rec * tjj);
        uscale = zdiv(uscale, tjjs);
      }
      if (rec < 1.0) {
        for (int i = 1; i <= m; ++i) XL(i) = zscal(XL(i), rec);
        xscale *= rec;
        xmax *= rec;
      }
    }
    double2 csumj = make_double2(0.0, 0.0);
    for (int i = 1; i <= j - 1; ++i) csumj = zfma(zmul(zconj(TL(i, j)), uscale), XL(i), csumj);
    const bool unan = (uscale.x != uscale.x) || (uscale.y != uscale.y);
    if ((uscale.x == tscale && uscale.y == 0.0) || unan) {
      XL(j) = zsub(XL(j), csumj);
      xj = zabs1(XL(j));
      tjjs = zscal(zconj(shifted_diag(TL(j, j), lam, smin)), tscale);
      const double tjj = zabs1(tjjs);
      if (tjj > smallnum) {
        if (tjj < 1.0 && xj > tjj * bignum) {
          const double r2 = 1.0 / xj;
          for (int i = 1; i <= m; ++i) XL(i) = zscal(XL(i), r2);
          xscale *= r2;
          xmax *= r2;
        }
        XL(j) = zdiv(XL(j), tjjs);
      } else if (tjj > 0.0) {
        if (xj > tjj * bignum) {
          const double r2 = (tjj * bignum) / xj;
          for (int i = 1; i <= m; ++i) XL(i) = zscal(XL(i), r2);
          xscale *= r2;
          xmax *= r2;
        }
        XL(j) = zdiv(XL(j), tjjs);
      } else {
        for (int i = 1; i <= m; ++i) XL(i) = make_double2(0.0, 0.0);
        XL(j) = make_double2(1.0, 0.0);
        xscale = 0.0;
        xmax = 0.0;
      }
    } else {
      XL(j) = zsub(zdiv(XL(j), tjjs), csumj);
    }
    xmax = fmax(xmax, zabs1(XL(j)));
  }
#undef XL
#undef TL
  return xscale / tscale;
}

// V[:, ki] = Z X[:, ki] for all ki, then the two normalisations.  Thread = row of V.
template <int NT>
__device__ void form_vectors(int n, const double2* __restrict__ Zg, const double2* X, int ldx, double2* __restrict__ Vg,
                             bool right, bool normalize, const int* cmap, double* red) {
  const int tid = threadIdx.x;
  for (int r = tid; r < n; r += NT) {
    for (int ki = 1; ki <= n; ++ki) {
      const int col = cmap ? cmap[ki - 1] : ki - 1;
      const int lo = right ? 1 : ki, hi = right ? ki : n;
      double2 acc = make_double2(0.0, 0.0);
      if (Zg) {
        for (int i = lo; i <= hi; ++i) acc = zfma(Zg[r + (long long)(i - 1) * n], X[(i - 1) * ldx + (ki - 1)], acc);
      } else {
        acc = (r + 1 >= lo && r + 1 <= hi) ? X[r * ldx + (ki - 1)] : make_double2(0.0, 0.0);
      }
      Vg[r + (long long)col * n] = acc;
    }
  }
  __syncthreads();
  // per column: 1 / max abs1, then unit 2-norm with the largest-modulus entry real
  const int lane = tid & 31, wid = tid >> 5;
  for (int ki = 1 + wid; ki <= n; ki += NT / 32) {
    double2* v = Vg + (long long)(ki - 1) * n;
    double t0 = 0.0;
    for (int r = lane; r < n; r += 32) t0 = fmax(t0, zabs1(v[r]));
    for (int o = 16; o > 0; o >>= 1) t0 = fmax(t0, __shfl_xor_sync(0xffffffffu, t0, o));
    const double remax = 1.0 / t0;
    double ss = 0.0, best = -1.0;
    int ib = 0;
    for (int r = lane; r < n; r += 32) {
      const double2 x = zscal(v[r], remax);
      v[r] = x;
      const double a2 = x.x * x.x + x.y * x.y;
      ss += a2;
      if (a2 > best) { best = a2; ib = r; }
    }
    if (!normalize) continue;
    for (int o = 16; o > 0; o >>= 1) {
      ss += __shfl_xor_sync(0xffffffffu, ss, o);
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, ib, o);
      if (ob > best || (ob == best && oi < ib)) { best = ob; ib = oi; }
    }
    // _enormalize!: f = conj(v[i0]) / (|v|_2 |v[i0]|)
    const double2 vi0 = v[ib];
    const double s = 1.0 / sqrt(ss);
    const double2 f = zscal(zconj(vi0), s / sqrt(best));
    __syncwarp();
    for (int r = lane; r < n; r += 32) {
      double2 x = zmul(v[r], f);
      if (r == ib) x.y = 0.0;
      v[r] = x;
    }
  }
  (void)red;
}

template <int NT>
__device__ void eigvecs_one(const EigBatch& eb, int b, double2* smem) {
  const int tid = threadIdx.x;
  const int n = eb.ns[b];
  if (n <= 0 || n > kSmallMax) return;  // shared memory is sized for kSmallMax; device orders are unchecked
  const long long off = eb.offs[b];
  const double2* __restrict__ Tg = eb.T + off;
  const double2* __restrict__ Zg = eb.Z ? eb.Z + off : nullptr;
  const int ldt = n;  // unused by the packed accessor
  double2* T = smem;                                  // packed upper triangle, n(n+1)/2
  double* tn = (double*)(T + (size_t)n * (n + 1) / 2); // tnorms, n
  double* red = tn + ((n + 1) & ~1);                  // 32 (tn padded to an even count so Xs is 16-byte aligned)
  double2* Xs = (double2*)(red + 32);
  const bool xsmem = (n <= kEigSmem);
  double2* X = xsmem ? Xs : eb.scratch + off;         // X[i, ki] at (i-1)*ldx + ki-1
  const int ldx = n;
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    if (i <= j) TT(i + 1, j + 1) = Tg[idx];
  }
  __syncthreads();
  const double ulp = kEps;
  const double smallnum_v = kSafemin * (double)n;     // vectors.jl:61
  const double smallnum = kSafemin / kEps;            // util.jl:134
  const double bignum = 1.0 / smallnum;

  for (int pass = 0; pass < 2; ++pass) {
    const bool right = (pass == 0);
    double2* Vg = right ? (eb.VR ? eb.VR + off : nullptr) : (eb.VL ? eb.VL + off : nullptr);
    if (!Vg) continue;
    // column norms of the strictly upper part: modulus for right, abs1 for left
    for (int j = tid; j < n; j += NT) {
      double s = 0.0;
      for (int i = 1; i <= j; ++i) s += right ? zabs(TT(i, j + 1)) : zabs1(TT(i, j + 1));
      tn[j] = s;
    }
    __syncthreads();
    const int ki = tid + 1;                 // this thread's eigenvalue (requires n <= NT)
    const bool mine = ki <= n;
    const double2 lam = mine ? TT(ki, ki) : make_double2(0.0, 0.0);
    const double smin = fmax(ulp * zabs1(lam), smallnum_v);
    // right: system rows 1..ki-1; left: rows ki+1..n
    const int m = mine ? (right ? ki - 1 : n - ki) : 0;
    // right-hand side
    if (mine) {
      if (right) {
        for (int k = 1; k <= ki - 1; ++k) X[(k - 1) * ldx + (ki - 1)] = zneg(TT(k, ki));
      } else {
        for (int k = 1; k <= n; ++k)
          X[(k - 1) * ldx + (ki - 1)] = (k > ki) ? zneg(zconj(TT(ki, k))) : make_double2(0.0, 0.0);
      }
    }
    // growth bound (util.jl:138-185 / 312-357); cnorm = tn[0..m) for the left
    // solve as the reference passes it (vectors.jl:417-420), tn[0..ki-1) for the right
    double tmax = 0.0, xmax = 0.0;
    for (int j = 1; j <= m; ++j) tmax = fmax(tmax, fabs(tn[j - 1]));
    const double tscale = (tmax <= bignum * kHalf) ? 1.0 : kHalf / (smallnum * tmax);
    for (int j = 1; j <= m; ++j) {
      const int g = right ? j : ki + j;
      xmax = fmax(xmax, cabs1half(X[(g - 1) * ldx + (ki - 1)]));
    }
    double grow = 0.0;
    if (m > 0 && tscale == 1.0) {
      grow = kHalf / fmax(xmax, smallnum);
      double xbound = grow;
      bool toosmall = false;
      if (right) {
        for (int j = m; j >= 1; --j) {
          toosmall = (grow <= smallnum);
          if (toosmall) break;
          const double tjj = zabs1(shifted_diag(TT(j, j), lam, smin));
          if (tjj >= smallnum) xbound = fmin(xbound, fmin(1.0, tjj) * grow);
          else xbound = 0.0;
          if (tjj + tn[j - 1] >= smallnum) grow *= tjj / (tjj + tn[j - 1]);
          else grow = 0.0;
        }
        if (!toosmall) grow = xbound;
      } else {
        for (int j = 1; j <= m; ++j) {
          toosmall = (grow <= smallnum);
          if (toosmall) break;
          const double xj = 1.0 + tn[j - 1];
          grow = fmin(grow, xbound / xj);
          const int g = ki + j;
          const double tjj = zabs1(shifted_diag(TT(g, g), lam, smin));
          if (tjj >= smallnum) { if (xj > tjj) xbound *= tjj / xj; }
          else xbound = 0.0;
        }
        if (!toosmall) grow = fmin(grow, xbound);
      }
    }
    const bool fast = mine && m > 0 && (grow * tscale > smallnum);
    // lockstep fast substitution
    if (right) {
      for (int j = n - 1; j >= 1; --j) {
        const bool act = fast && (j < ki);
        const double2 d = shifted_diag(TT(j, j), lam, smin);
        double2 xj = make_double2(0.0, 0.0);
        if (act) {
          xj = zdiv(X[(j - 1) * ldx + (ki - 1)], d);
          X[(j - 1) * ldx + (ki - 1)] = xj;
        }
        if (act)
          for (int i = j - 1; i >= 1; --i)
            X[(i - 1) * ldx + (ki - 1)] = zfms(TT(i, j), xj, X[(i - 1) * ldx + (ki - 1)]);
      }
    } else {
      for (int g = 2; g <= n; ++g) {
        const bool act = fast && (g > ki);
        if (act) {
          const double2 d = zconj(shifted_diag(TT(g, g), lam, smin));
          const double2 xg = zdiv(X[(g - 1) * ldx + (ki - 1)], d);
          X[(g - 1) * ldx + (ki - 1)] = xg;
          for (int h = g + 1; h <= n; ++h)
            X[(h - 1) * ldx + (ki - 1)] = zfms(zconj(TT(g, h)), xg, X[(h - 1) * ldx + (ki - 1)]);
        }
      }
    }
    double xscale = 1.0;
    if (mine && m > 0 && !fast) {
      if (right)
        xscale = usolve_careful(T, ldt, m, lam, smin, X + (ki - 1), ldx, tn, tscale, xmax);
      else
        xscale = cusolve_careful(T, ldt, ki + 1, m, lam, smin, X + (ki - 1), ldx, tn, tscale, xmax);
    }
    if (mine) X[(ki - 1) * ldx + (ki - 1)] = make_double2(xscale, 0.0);
    __syncthreads();
    form_vectors<NT>(n, Zg, X, ldx, Vg, right, eb.normalize, eb.colmap ? eb.colmap + eb.woffs[b] : nullptr, red);
    __syncthreads();
  }
}
#undef TT
#undef XX

template <int NT>
__global__ void __launch_bounds__(NT) k_eigvecs(EigBatch eb) {
  extern __shared__ double2 smem_e[];
  for (int b = blockIdx.x; b < eb.count; b += gridDim.x) eigvecs_one<NT>(eb, b, smem_e);
}

}  // namespace

// Shared memory for orders up to nmax: packed T, tnorms (padded to an even count),
// reduction scratch and, for orders <= kEigSmem, the solution block X.
size_t eigvecs_smem_bytes(int nmax) {
  size_t need = 0;
  for (int n = 1; n <= nmax; ++n) {
    const size_t x = n <= kEigSmem ? (size_t)n * n : 0;
    const size_t b = sizeof(double2) * ((size_t)n * (n + 1) / 2 + x) + sizeof(double) * (((n + 1) & ~1) + 32);
    if (b > need) need = b;
  }
  return need + 64;
}

cudaError_t launch_eigvecs_batched(const EigBatch& eb, int nmax, int num_sms, cudaStream_t s) {
  const size_t smem = eigvecs_smem_bytes(nmax);
  cudaError_t e = cudaFuncSetAttribute(k_eigvecs<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eigvecs<128>, 128, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  int grid = num_sms * per_sm;
  if (grid > eb.count) grid = eb.count;
  k_eigvecs<128><<<grid, 128, smem, s>>>(eb);
  return cudaGetLastError();
}

}  // namespace gsk
