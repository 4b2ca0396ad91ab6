// Aggressive early deflation (AED) for the large-matrix real Schur path.
//
// The reference deflates only at negligible subdiagonal entries
// (GenericSchur.jl:563-600).  The multishift path here adds the deflation window of
// Braman, Byers and Mathias ("The multishift QR algorithm. Part II: aggressive
// early deflation", SIMAX 2002): the trailing nw x nw window W = H[kwtop:ihi,
// kwtop:ihi] of the active block is put in real Schur form W = V T V^T by the
// small-matrix kernel, which turns the single coupling entry s = H[kwtop, kwtop-1]
// into the spike s V[0, :].  An eigenvalue (1x1 or 2x2 block of T) whose spike
// entries are negligible against it is converged and deflates.  Blocks are tested
// from the bottom; an undeflatable block is moved to the top of the untested
// region by swapping adjacent diagonal blocks (the direct swapping method of Bai and
// Demmel, "On swapping diagonal blocks in real Schur form", LAA 1993: a small
// Sylvester equation gives the invariant subspace, Householder reflectors rotate
// it into place, and the swap is rejected if the result is not block triangular to
// working accuracy).  The undeflated part is then brought back to Hessenberg form
// (one reflector for the spike, a Householder reduction of the undeflated block),
// and its eigenvalues are the shifts of the next multishift sweep.
//
// One CTA does all of it with T in shared memory and V in global memory (L2): the
// decisions and the 2x2/4x4 algebra of a swap run on thread 0, the row/column
// updates on all threads.  The host applies V to the rest of H and to Z by GEMMs.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kAedThreads = 256;

template <class T>
struct AedShared {
  T u1[3], u2[3];  // reflectors of a swap (u[0..2]), taus below
  T tau1, tau2;
  T cs, sn;        // rotation of a 1x1 swap or a 2x2 standardisation
  T blk[4];        // standardised 2x2 block
  T d11, d22;      // diagonal values written after a 1x1 swap / kept values
  int ok;
  int kind;        // swap kind: 11, 12, 21, 22
};

template <class T>
struct AedCtx {
  T* t;      // window, shared memory, ld ldt (0-based indices)
  int ldt;
  T* v;      // V, global, ld nw
  int nw;
  AedShared<T>* sh;
};

#define TT(i, j) a.t[(i) + (j) * a.ldt]
#define VV(i, j) a.v[(i) + (size_t)(j) * a.nw]

// Plane rotation on rows (j1, j2) for columns [c0, nw), on columns (j1, j2) for rows
// [0, r1), and on columns (j1, j2) of V:  x <- cs x + sn y, y <- cs y - sn x.
template <class T>
__device__ void rot_apply(const AedCtx<T>& a, int j1, int j2, T cs, T sn, int c0, int r1) {
  const int tid = threadIdx.x;
  for (int c = c0 + tid; c < a.nw; c += kAedThreads) {
    const T x = TT(j1, c), y = TT(j2, c);
    TT(j1, c) = cs * x + sn * y;
    TT(j2, c) = cs * y - sn * x;
  }
  for (int r = tid; r < r1; r += kAedThreads) {
    const T x = TT(r, j1), y = TT(r, j2);
    TT(r, j1) = cs * x + sn * y;
    TT(r, j2) = cs * y - sn * x;
  }
  for (int r = tid; r < a.nw; r += kAedThreads) {
    const T x = VV(r, j1), y = VV(r, j2);
    VV(r, j1) = cs * x + sn * y;
    VV(r, j2) = cs * y - sn * x;
  }
}

// (I - tau u u^T) from the left on rows j..j+2, columns [c0, c1).
template <class T>
__device__ void refl_left(const AedCtx<T>& a, const T* u, T tau, int j, int c0, int c1) {
  for (int c = c0 + threadIdx.x; c < c1; c += kAedThreads) {
    const T s = tau * (u[0] * TT(j, c) + u[1] * TT(j + 1, c) + u[2] * TT(j + 2, c));
    TT(j, c) -= s * u[0];
    TT(j + 1, c) -= s * u[1];
    TT(j + 2, c) -= s * u[2];
  }
}
// ... from the right on columns j..j+2, rows [0, r1) of T.
template <class T>
__device__ void refl_right(const AedCtx<T>& a, const T* u, T tau, int j, int r1) {
  for (int r = threadIdx.x; r < r1; r += kAedThreads) {
    const T s = tau * (TT(r, j) * u[0] + TT(r, j + 1) * u[1] + TT(r, j + 2) * u[2]);
    TT(r, j) -= s * u[0];
    TT(r, j + 1) -= s * u[1];
    TT(r, j + 2) -= s * u[2];
  }
}
// ... from the right on columns j..j+2 of V (all rows).
template <class T>
__device__ void refl_right_v(const AedCtx<T>& a, const T* u, T tau, int j) {
  for (int r = threadIdx.x; r < a.nw; r += kAedThreads) {
    const T s = tau * (VV(r, j) * u[0] + VV(r, j + 1) * u[1] + VV(r, j + 2) * u[2]);
    VV(r, j) -= s * u[0];
    VV(r, j + 1) -= s * u[1];
    VV(r, j + 2) -= s * u[2];
  }
}

// Solve T11 X - X T22 = B for X (n1 x n2, n1, n2 in {1, 2}) by Gaussian elimination
// with complete pivoting on the Kronecker system; pivots below smin are raised to
// smin (a nearly singular system only means the swap will be rejected).
__device__ void small_sylvester(int n1, int n2, const double* t11, const double* t22, const double* b,
                                double* x, double smin) {
  // unknowns x[i + j n1]; equation (i, j): sum_k t11[i,k] x[k,j] - sum_k x[i,k] t22[k,j] = b[i,j]
  const int m = n1 * n2;
  double M[4][4], r[4];
  int cp[4];
  for (int j = 0; j < n2; ++j)
    for (int i = 0; i < n1; ++i) {
      const int e = i + j * n1;
      for (int q = 0; q < m; ++q) M[e][q] = 0.0;
      for (int k = 0; k < n1; ++k) M[e][k + j * n1] += t11[i + k * n1];
      for (int k = 0; k < n2; ++k) M[e][i + k * n1] -= t22[k + j * n2];
      r[e] = b[i + j * n1];
    }
  for (int q = 0; q < m; ++q) cp[q] = q;
  for (int c = 0; c < m; ++c) {
    int pr = c, pc = c;
    double best = -1.0;
    for (int i = c; i < m; ++i)
      for (int j = c; j < m; ++j)
        if (fabs(M[i][j]) > best) { best = fabs(M[i][j]); pr = i; pc = j; }
    if (pr != c) {
      for (int j = 0; j < m; ++j) { const double t = M[c][j]; M[c][j] = M[pr][j]; M[pr][j] = t; }
      const double t = r[c]; r[c] = r[pr]; r[pr] = t;
    }
    if (pc != c) {
      for (int i = 0; i < m; ++i) { const double t = M[i][c]; M[i][c] = M[i][pc]; M[i][pc] = t; }
      const int t = cp[c]; cp[c] = cp[pc]; cp[pc] = t;
    }
    if (fabs(M[c][c]) < smin) M[c][c] = (M[c][c] < 0.0) ? -smin : smin;
    for (int i = c + 1; i < m; ++i) {
      const double f = M[i][c] / M[c][c];
      for (int j = c; j < m; ++j) M[i][j] -= f * M[c][j];
      r[i] -= f * r[c];
    }
  }
  double y[4];
  for (int c = m - 1; c >= 0; --c) {
    double s = r[c];
    for (int j = c + 1; j < m; ++j) s -= M[c][j] * y[j];
    y[c] = s / M[c][c];
  }
  for (int c = 0; c < m; ++c) x[cp[c]] = y[c];
}

// (I - tau u u^T) applied to the rows r0..r0+2 (left) / columns c0..c0+2 (right) of a
// small dense 4x4 block D (column-major, ld 4), in double.
__device__ void d_left(double* D, const double* u, double tau, int r0, int ncol) {
  for (int c = 0; c < ncol; ++c) {
    const double s = tau * (u[0] * D[r0 + 4 * c] + u[1] * D[r0 + 1 + 4 * c] + u[2] * D[r0 + 2 + 4 * c]);
    D[r0 + 4 * c] -= s * u[0];
    D[r0 + 1 + 4 * c] -= s * u[1];
    D[r0 + 2 + 4 * c] -= s * u[2];
  }
}
__device__ void d_right(double* D, const double* u, double tau, int c0, int nrow) {
  for (int r = 0; r < nrow; ++r) {
    const double s = tau * (D[r + 4 * c0] * u[0] + D[r + 4 * (c0 + 1)] * u[1] + D[r + 4 * (c0 + 2)] * u[2]);
    D[r + 4 * c0] -= s * u[0];
    D[r + 4 * (c0 + 1)] -= s * u[1];
    D[r + 4 * (c0 + 2)] -= s * u[2];
  }
}

// Standardise the 2x2 block at (j, j+1) with _gs2x2! (GenericSchur.jl:716-803) and
// apply its rotation to the rest of T and to V.  Collective.
template <class T>
__device__ void standardize(const AedCtx<T>& a, int j) {
  if (threadIdx.x == 0) {
    double p = TT(j, j), q = TT(j, j + 1), r = TT(j + 1, j), s = TT(j + 1, j + 1);
    double cs, sn, w1r, w1i, w2r, w2i;
    gs2x2(p, q, r, s, cs, sn, w1r, w1i, w2r, w2i);
    a.sh->cs = (T)cs; a.sh->sn = (T)sn;
    a.sh->blk[0] = (T)p; a.sh->blk[1] = (T)q; a.sh->blk[2] = (T)r; a.sh->blk[3] = (T)s;
  }
  __syncthreads();
  rot_apply(a, j, j + 1, a.sh->cs, a.sh->sn, j + 2, j);
  __syncthreads();
  if (threadIdx.x == 0) {
    TT(j, j) = a.sh->blk[0]; TT(j, j + 1) = a.sh->blk[1];
    TT(j + 1, j) = a.sh->blk[2]; TT(j + 1, j + 1) = a.sh->blk[3];
  }
  __syncthreads();
}

// Swap the adjacent diagonal blocks of orders n1 (at j1) and n2 (at j1+n1).
// Collective; returns false (T and V untouched) if the swap is rejected.
template <class T>
__device__ bool swap_blocks(const AedCtx<T>& a, int j1, int n1, int n2) {
  const int tid = threadIdx.x;
  const int nw = a.nw;
  const int j2 = j1 + 1, j3 = j1 + 2;
  AedShared<T>& sh = *a.sh;
  if (n1 == 1 && n2 == 1) {
    if (tid == 0) {
      const double t11 = TT(j1, j1), t22 = TT(j2, j2), t12 = TT(j1, j2);
      const double f = t12, g = t22 - t11;
      const double rr = hypot(f, g);
      sh.cs = (T)(rr > 0.0 ? f / rr : 1.0);
      sh.sn = (T)(rr > 0.0 ? g / rr : 0.0);
      sh.d11 = (T)t22;
      sh.d22 = (T)t11;
    }
    __syncthreads();
    rot_apply(a, j1, j2, sh.cs, sh.sn, j2 + 1, j1);
    __syncthreads();
    if (tid == 0) {
      TT(j1, j1) = sh.d11;
      TT(j2, j2) = sh.d22;
      TT(j2, j1) = T(0);
    }
    __syncthreads();
    return true;
  }
  const int nd = n1 + n2;
  if (tid == 0) {
    double D[16];
    for (int i = 0; i < 16; ++i) D[i] = 0.0;
    double dnorm = 0.0;
    for (int j = 0; j < nd; ++j)
      for (int i = 0; i < nd; ++i) {
        D[i + 4 * j] = TT(j1 + i, j1 + j);
        dnorm = fmax(dnorm, fabs(D[i + 4 * j]));
      }
    const double eps = (double)Prec<T>::eps;
    const double smlnum = (double)Prec<T>::fmin / eps;
    const double thresh = fmax(10.0 * eps * dnorm, smlnum);
    double t11[4], t22[4], b12[4], x[4];
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n1; ++i) t11[i + j * n1] = D[i + 4 * j];
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i < n2; ++i) t22[i + j * n2] = D[n1 + i + 4 * (n1 + j)];
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i < n1; ++i) b12[i + j * n1] = D[i + 4 * (n1 + j)];
    const double smin = fmax(eps * dnorm, smlnum);
    small_sylvester(n1, n2, t11, t22, b12, x, smin);
    const double scale = 1.0;
    double u1[3], u2[3], tau1 = 0.0, tau2 = 0.0;
    bool ok = true;
    if (n1 == 1 && n2 == 2) {
      // reflector with (scale, x11, x12) H = (0, 0, *)
      double al = x[1], x1 = scale, x2 = x[0];
      tau1 = reflector_small(al, x1, x2, 3);
      u1[0] = x1; u1[1] = x2; u1[2] = 1.0;
      const double t11s = D[0];
      d_left(D, u1, tau1, 0, 3);
      d_right(D, u1, tau1, 0, 3);
      ok = fmax(fmax(fabs(D[2]), fabs(D[2 + 4])), fabs(D[2 + 8] - t11s)) <= thresh;
      sh.d22 = (T)t11s;
      sh.kind = 12;
    } else if (n1 == 2 && n2 == 1) {
      double al = -x[0], x1 = -x[1], x2 = scale;
      tau1 = reflector_small(al, x1, x2, 3);
      u1[0] = 1.0; u1[1] = x1; u1[2] = x2;
      const double t33 = D[2 + 8];
      d_left(D, u1, tau1, 0, 3);
      d_right(D, u1, tau1, 0, 3);
      ok = fmax(fmax(fabs(D[1]), fabs(D[2])), fabs(D[0] - t33)) <= thresh;
      sh.d11 = (T)t33;
      sh.kind = 21;
    } else {
      // QR factorisation of [-X; scale I] by two reflectors
      double al = -x[0], x1 = -x[1], x2 = scale;  // x is 2x2 column-major: x11 x21 x12 x22
      tau1 = reflector_small(al, x1, x2, 3);
      u1[0] = 1.0; u1[1] = x1; u1[2] = x2;
      const double temp = -tau1 * (x[2] + u1[1] * x[3]);
      double bl = -temp * u1[1] - x[3], y1 = -temp * u1[2], y2 = scale;
      tau2 = reflector_small(bl, y1, y2, 3);
      u2[0] = 1.0; u2[1] = y1; u2[2] = y2;
      d_left(D, u1, tau1, 0, 4);
      d_right(D, u1, tau1, 0, 4);
      d_left(D, u2, tau2, 1, 4);
      d_right(D, u2, tau2, 1, 4);
      ok = fmax(fmax(fabs(D[2]), fabs(D[2 + 4])), fmax(fabs(D[3]), fabs(D[3 + 4]))) <= thresh;
      sh.kind = 22;
    }
    for (int q = 0; q < 3; ++q) { sh.u1[q] = (T)u1[q]; sh.u2[q] = (T)u2[q]; }
    sh.tau1 = (T)tau1;
    sh.tau2 = (T)tau2;
    sh.ok = ok ? 1 : 0;
  }
  __syncthreads();
  const int ok = sh.ok, kind = sh.kind;
  __syncthreads();  // everyone has read the decision before thread 0 may write the next one
  if (!ok) return false;
  if (kind == 12) {
    refl_left(a, sh.u1, sh.tau1, j1, j1, nw);
    __syncthreads();
    refl_right(a, sh.u1, sh.tau1, j1, j2 + 1);
    refl_right_v(a, sh.u1, sh.tau1, j1);
    __syncthreads();
    if (tid == 0) { TT(j3, j1) = T(0); TT(j3, j2) = T(0); TT(j3, j3) = sh.d22; }
    __syncthreads();
    standardize(a, j1);
  } else if (kind == 21) {
    refl_right(a, sh.u1, sh.tau1, j1, j3 + 1);
    refl_right_v(a, sh.u1, sh.tau1, j1);
    __syncthreads();
    refl_left(a, sh.u1, sh.tau1, j1, j2, nw);
    __syncthreads();
    if (tid == 0) { TT(j1, j1) = sh.d11; TT(j2, j1) = T(0); TT(j3, j1) = T(0); }
    __syncthreads();
    standardize(a, j2);
  } else {
    const int j4 = j1 + 3;
    refl_left(a, sh.u1, sh.tau1, j1, j1, nw);
    __syncthreads();
    refl_right(a, sh.u1, sh.tau1, j1, j4 + 1);
    __syncthreads();
    refl_left(a, sh.u2, sh.tau2, j2, j1, nw);
    __syncthreads();
    refl_right(a, sh.u2, sh.tau2, j2, j4 + 1);
    for (int r = tid; r < nw; r += kAedThreads) {
      // both V reflectors per row, in order
      T s = sh.tau1 * (VV(r, j1) * sh.u1[0] + VV(r, j1 + 1) * sh.u1[1] + VV(r, j1 + 2) * sh.u1[2]);
      VV(r, j1) -= s * sh.u1[0];
      VV(r, j1 + 1) -= s * sh.u1[1];
      VV(r, j1 + 2) -= s * sh.u1[2];
      s = sh.tau2 * (VV(r, j2) * sh.u2[0] + VV(r, j2 + 1) * sh.u2[1] + VV(r, j2 + 2) * sh.u2[2]);
      VV(r, j2) -= s * sh.u2[0];
      VV(r, j2 + 1) -= s * sh.u2[1];
      VV(r, j2 + 2) -= s * sh.u2[2];
    }
    __syncthreads();
    if (tid == 0) { TT(j3, j1) = T(0); TT(j3, j2) = T(0); TT(j4, j1) = T(0); TT(j4, j2) = T(0); }
    __syncthreads();
    standardize(a, j1);
    standardize(a, j3);
  }
  return true;
}

// dtrexc's move towards the top (GenericSchur's _trexchange!, rordschur.jl:54-166,
// iold > inew branch): the block at iold moves to inew by adjacent swaps; a 2x2 block
// that splits into two real eigenvalues on the way continues as two 1x1 blocks.
// Returns the final position, or -position - 1 if a swap was rejected.  Collective.
template <class T>
__device__ int trexchange_up(const AedCtx<T>& a, int iold, int inew) {
  const int n = a.nw;  // 1-based positions below
#define T1(i, j) a.t[((i) - 1) + ((j) - 1) * a.ldt]
  auto nbsize = [&](int j) { return (j < n && T1(j + 1, j) != T(0)) ? 2 : 1; };
  if (iold > 1 && T1(iold, iold - 1) != T(0)) iold -= 1;
  int nbold = nbsize(iold);
  if (inew > 1 && T1(inew, inew - 1) != T(0)) inew -= 1;
  if (iold == inew) return inew;
  int here = iold;
  while (here > inew) {
    if (nbold == 1 || nbold == 2) {
      const int nbnext = (here >= 3 && T1(here - 1, here - 2) != T(0)) ? 2 : 1;
      if (!swap_blocks(a, here - nbnext - 1, nbnext, nbold)) return -here - 1;
      here -= nbnext;
      if (nbold == 2 && T1(here + 1, here) == T(0)) nbold = 3;
    } else {
      // two 1x1 blocks, each swapped on its own
      int nbnext = (here >= 3 && T1(here - 1, here - 2) != T(0)) ? 2 : 1;
      if (!swap_blocks(a, here - nbnext - 1, nbnext, 1)) return -here - 1;
      if (nbnext == 1) {
        swap_blocks(a, here - 1, nbnext, 1);
        here -= 1;
      } else {
        if (T1(here, here - 1) == T(0)) nbnext = 1;
        if (nbnext == 2) {
          if (!swap_blocks(a, here - 2, 2, 1)) return -here - 1;
          here -= 2;
        } else {
          swap_blocks(a, here - 1, 1, 1);
          swap_blocks(a, here - 2, 1, 1);
          here -= 2;
        }
      }
    }
  }
#undef T1
  return here;
}

}  // namespace

// gordschur!(T, Z, select) for a real standard-form Schur pair (rordschur.jl:3-47):
// selected eigenvalues (a 2x2 block is selected if either of its eigenvalues is) move
// to the top in their order.  One CTA on T and Z in global memory (ld n).
// st[0] = 0, or k (1-based) of the block whose swap was rejected.
template <class T>
__global__ void __launch_bounds__(kAedThreads) k_ordschur_real(T* Tm, T* Zm, int n, const int* __restrict__ select,
                                                                double* wr, double* wi, int* st) {
  __shared__ AedShared<T> sh;
  AedCtx<T> a{Tm, n, Zm, n, &sh};
  const int tid = threadIdx.x;
  int ks = 0;
  bool pair = false;
  int err = 0;
  for (int k = 1; k <= n; ++k) {
    if (pair) { pair = false; continue; }
    bool sw = select[k - 1] != 0;
    if (k < n && Tm[(k - 1) * (size_t)n + k] != T(0)) {
      pair = true;
      sw = sw || select[k] != 0;
    }
    if (sw) {
      ks += 1;
      if (k != ks) {
        const int r = trexchange_up(a, k, ks);
        if (r < 0) { err = k; break; }
        ks = r;
      }
      if (pair) ks += 1;
    }
  }
  __syncthreads();
  for (int j = tid; j < n; j += kAedThreads) {
    const T d = Tm[(size_t)j * n + j];
    double im = 0.0;
    if (j + 1 < n && Tm[(size_t)j * n + j + 1] != T(0))
      im = sqrt(fabs((double)Tm[(size_t)(j + 1) * n + j])) * sqrt(fabs((double)Tm[(size_t)j * n + j + 1]));
    else if (j > 0 && Tm[(size_t)(j - 1) * n + j] != T(0))
      im = -sqrt(fabs((double)Tm[(size_t)j * n + j - 1])) * sqrt(fabs((double)Tm[(size_t)(j - 1) * n + j]));
    wr[j] = (double)d;
    wi[j] = im;
  }
  if (tid == 0) st[0] = err;
}

// gordschur!(T, Z, select) for a complex triangular Schur pair (ordschur.jl:24-74):
// selected eigenvalues move to the top in their order by adjacent swaps, each a plane
// rotation G with G [T(k,k+1); T(k+1,k+1) - T(k,k)] = [r; 0] applied as T <- G T G^H,
// Z <- Z G^H (Golub and Van Loan, Algorithm 7.6.1).  One CTA on T, Z in global memory.
__global__ void __launch_bounds__(kAedThreads) k_ordschur_cplx(double2* Tm, double2* Zm, int n,
                                                                const int* __restrict__ select, double2* w) {
  __shared__ double c_s;
  __shared__ double2 s_s;
  const int tid = threadIdx.x;
  int ks = 0;
  for (int k = 1; k <= n; ++k) {
    if (!select[k - 1]) continue;
    ks += 1;
    for (int kk = k - 1; kk >= ks; --kk) {
      // swap the diagonal entries kk, kk+1 (1-based)
      if (tid == 0) {
        const double2 f = Tm[(size_t)kk * n + (kk - 1)];                        // T(kk, kk+1)
        const double2 g = zsub(Tm[(size_t)kk * n + kk], Tm[(size_t)(kk - 1) * n + (kk - 1)]);
        const double af = hypot(f.x, f.y), ag = hypot(g.x, g.y);
        double c;
        double2 sv;
        if (ag == 0.0) { c = 1.0; sv = make_double2(0.0, 0.0); }
        else if (af == 0.0) { c = 0.0; sv = zscal(zconj(g), 1.0 / ag); }
        else {
          const double rho = hypot(af, ag);
          c = af / rho;
          sv = zscal(zmul(zscal(f, 1.0 / af), zconj(g)), 1.0 / rho);
        }
        c_s = c;
        s_s = sv;
      }
      __syncthreads();
      const double c = c_s;
      const double2 sv = s_s;
      // rows kk, kk+1 of T (all columns): [x; y] <- [c x + s y; -conj(s) x + c y]
      for (int j = tid; j < n; j += kAedThreads) {
        double2* x = &Tm[(size_t)j * n + (kk - 1)];
        double2* y = &Tm[(size_t)j * n + kk];
        const double2 a0 = *x, b0 = *y;
        *x = zadd(zscal(a0, c), zmul(sv, b0));
        *y = zsub(zscal(b0, c), zmul(zconj(sv), a0));
      }
      __syncthreads();
      // columns kk, kk+1 of T and Z (all rows): [u v] <- [c u + conj(s) v, -s u + c v]
      for (int i = tid; i < 2 * n; i += kAedThreads) {
        double2* M = i < n ? Tm : Zm;
        const int r = i < n ? i : i - n;
        double2* u = &M[(size_t)(kk - 1) * n + r];
        double2* v = &M[(size_t)kk * n + r];
        const double2 a0 = *u, b0 = *v;
        *u = zadd(zscal(a0, c), zmul(zconj(sv), b0));
        *v = zsub(zscal(b0, c), zmul(sv, a0));
      }
      __syncthreads();
    }
  }
  // triu!(T); values = diag(T)
  for (size_t idx = tid; idx < (size_t)n * n; idx += kAedThreads) {
    const int i = idx % n, j = idx / n;
    if (i > j) Tm[idx] = make_double2(0.0, 0.0);
    if (i == j) w[i] = Tm[idx];
  }
}

cudaError_t launch_ordschur_real(double* T, double* Z, int n, const int* select, double* wr, double* wi, int* st,
                                 cudaStream_t s) {
  k_ordschur_real<double><<<1, kAedThreads, 0, s>>>(T, Z, n, select, wr, wi, st);
  return cudaGetLastError();
}
cudaError_t launch_ordschur_cplx(double2* T, double2* Z, int n, const int* select, double2* w, cudaStream_t s) {
  k_ordschur_cplx<<<1, kAedThreads, 0, s>>>(T, Z, n, select, w);
  return cudaGetLastError();
}

template <class T>
__global__ void __launch_bounds__(kAedThreads) k_aed(AedArgs<T> g) {
  extern __shared__ double aed_raw[];
  __shared__ AedShared<T> sh;
  __shared__ double red[32];
  const int tid = threadIdx.x;
  const int nw = g.nw;
  const int ldt = nw | 1;
  T* t = (T*)aed_raw;
  T* vbuf = t + (size_t)nw * ldt;  // reflector vector of the Hessenberg restoration (nw)
  AedCtx<T> a{t, ldt, g.V, nw, &sh};
  if (*g.win_status != ST_OK) {
    // the window's Schur form failed: no deflation, no shifts
    if (tid == 0) { g.out[0] = nw; g.out[1] = 0; g.out[2] = 0; }
    return;
  }
  for (int idx = tid; idx < nw * nw; idx += kAedThreads) {
    const int i = idx % nw, j = idx / nw;
    TT(i, j) = (i > j + 1) ? T(0) : g.Tw[idx];
  }
  const int kwtop = g.kwtop;  // 1-based
  const T s = (kwtop > g.ilo) ? g.H[(size_t)(kwtop - 2) * g.n + (kwtop - 1)] : T(0);
  __syncthreads();
  const double ulp = (double)Prec<T>::eps;
  const double smlnum = (double)Prec<T>::fmin * ((double)g.n / ulp);
  // ---- deflation tests from the bottom.  [ns, nw) holds the deflated blocks, [pt, ns)
  // the undeflatable ones found so far, [0, pt) the untested ones.  A block whose spike
  // looks negligible where it sits is swapped down past the undeflatable group and
  // tested again there (the swaps change its spike); it deflates only if it passes at
  // its final place.  Undeflatable blocks never move, so the swap count is the number
  // of candidates times the size of the undeflatable group, not O(nw^2) as when every
  // undeflatable block is moved to the top.
  auto negligible = [&](int j, int bsz) -> bool {
    double foo, sp;
    if (bsz == 1) {
      foo = fabs((double)TT(j, j));
      sp = fabs((double)s * (double)VV(0, j));
    } else {
      foo = fabs((double)TT(j + 1, j + 1)) + sqrt(fabs((double)TT(j + 1, j))) * sqrt(fabs((double)TT(j, j + 1)));
      sp = fmax(fabs((double)s * (double)VV(0, j)), fabs((double)s * (double)VV(0, j + 1)));
    }
    if (foo == 0.0) foo = fabs((double)s);
    return sp <= fmax(smlnum, ulp * foo);
  };
  int ns = nw, pt = nw;
  while (pt > 0) {
    const int bsz = (pt >= 2 && TT(pt - 1, pt - 2) != T(0)) ? 2 : 1;
    const int j = pt - bsz;
    if (negligible(j, bsz)) {
      int here = j, nb = bsz;
      bool ok = true;
      while (here + nb < ns) {
        const int below = here + nb;
        const int nbnext = (below + 1 < nw && TT(below + 1, below) != T(0)) ? 2 : 1;
        if (!swap_blocks(a, here, nb, nbnext)) { ok = false; break; }
        here += nbnext;
        if (nb == 2 && TT(here + 1, here) == T(0)) { ok = false; break; }  // split: stop here
      }
      if (ok && here + nb == ns && negligible(here, nb)) ns -= nb;
    }
    pt = j;
  }
  // ---- eigenvalues of every block: undeflated ones are the next shifts, deflated ones final
  for (int j = tid; j < nw; j += kAedThreads) {
    double wr, wi;
    const bool top = (j + 1 < nw) && TT(j + 1, j) != T(0);
    const bool bottom = (j > 0) && TT(j, j - 1) != T(0);
    if (top) {
      wr = TT(j, j);
      wi = sqrt(fabs((double)TT(j, j + 1))) * sqrt(fabs((double)TT(j + 1, j)));
    } else if (bottom) {
      wr = TT(j, j);
      wi = -sqrt(fabs((double)TT(j - 1, j))) * sqrt(fabs((double)TT(j, j - 1)));
    } else {
      wr = TT(j, j);
      wi = 0.0;
    }
    g.ewr[j] = wr;
    g.ewi[j] = wi;
    if (j >= ns) {
      g.wr[kwtop - 1 + j] = wr;
      g.wi[kwtop - 1 + j] = wi;
    }
  }
  const int ndef = nw - ns;
  if (ndef == 0) {
    // nothing deflated: H stays as it is; only the shifts are used
    if (tid == 0) { g.out[0] = ns; g.out[1] = 0; g.out[2] = 0; }
    return;
  }
  __syncthreads();
  // ---- back to Hessenberg form: reflect the spike onto e1, then reduce T[0:ns, 0:ns]
  if (ns > 1 && s != T(0)) {
    double ls = 0.0;
    for (int i = 1 + tid; i < ns; i += kAedThreads) ls = fma((double)VV(0, i), (double)VV(0, i), ls);
    const double xs = block_sum<kAedThreads>(ls, red);
    if (tid == 0) {
      const double alpha = VV(0, 0);
      double tau = 0.0, scal = 0.0;
      if (xs > 0.0) {
        const double beta = -copysign(sqrt(fma(alpha, alpha, xs)), alpha);
        tau = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      sh.tau1 = (T)tau;
      sh.d11 = (T)scal;
    }
    __syncthreads();
    const T tau = sh.tau1, scal = sh.d11;
    if (tau != T(0)) {
      for (int i = tid; i < ns; i += kAedThreads) vbuf[i] = (i == 0) ? T(1) : VV(0, i) * scal;
      __syncthreads();
      // left on rows 0..ns-1, all columns
      for (int c = tid; c < nw; c += kAedThreads) {
        T acc = T(0);
        for (int i = 0; i < ns; ++i) acc += vbuf[i] * TT(i, c);
        acc *= tau;
        for (int i = 0; i < ns; ++i) TT(i, c) -= acc * vbuf[i];
      }
      __syncthreads();
      // right on columns 0..ns-1: rows 0..ns-1 of T, all rows of V
      for (int r = tid; r < ns + nw; r += kAedThreads) {
        if (r < ns) {
          T acc = T(0);
          for (int i = 0; i < ns; ++i) acc += TT(r, i) * vbuf[i];
          acc *= tau;
          for (int i = 0; i < ns; ++i) TT(r, i) -= acc * vbuf[i];
        } else {
          const int rv = r - ns;
          T acc = T(0);
          for (int i = 0; i < ns; ++i) acc += VV(rv, i) * vbuf[i];
          acc *= tau;
          for (int i = 0; i < ns; ++i) VV(rv, i) -= acc * vbuf[i];
        }
      }
      __syncthreads();
    }
    // Householder Hessenberg reduction of T[0:ns, 0:ns] (the reflectors leave e1 fixed)
    for (int k = 0; k + 2 < ns; ++k) {
      const int L = ns - k - 1;  // rows k+1..ns-1 of column k
      double lsq = 0.0;
      for (int i = 1 + tid; i < L; i += kAedThreads) {
        const double x = TT(k + 1 + i, k);
        lsq = fma(x, x, lsq);
      }
      const double xs2 = block_sum<kAedThreads>(lsq, red);
      if (tid == 0) {
        double al = TT(k + 1, k);
        double tau = 0.0, scal = 0.0, beta = al;
        if (xs2 > 0.0) {
          beta = -copysign(sqrt(fma(al, al, xs2)), al);
          tau = (beta - al) / beta;
          scal = 1.0 / (al - beta);
        }
        sh.tau1 = (T)tau;
        sh.d11 = (T)scal;
        sh.d22 = (T)beta;
      }
      __syncthreads();
      const T tau = sh.tau1, scal = sh.d11;
      if (tau == T(0)) { __syncthreads(); continue; }
      for (int i = tid; i < L; i += kAedThreads) vbuf[i] = (i == 0) ? T(1) : TT(k + 1 + i, k) * scal;
      __syncthreads();
      // left on rows k+1..ns-1, columns k+1..nw-1; column k becomes (beta, 0, ...)
      for (int c = k + 1 + tid; c < nw; c += kAedThreads) {
        T acc = T(0);
        for (int i = 0; i < L; ++i) acc += vbuf[i] * TT(k + 1 + i, c);
        acc *= tau;
        for (int i = 0; i < L; ++i) TT(k + 1 + i, c) -= acc * vbuf[i];
      }
      if (tid == 0) {
        TT(k + 1, k) = sh.d22;
        for (int i = 1; i < L; ++i) TT(k + 1 + i, k) = T(0);
      }
      __syncthreads();
      // right on columns k+1..ns-1: rows 0..ns-1 of T, all rows of V
      for (int r = tid; r < ns + nw; r += kAedThreads) {
        if (r < ns) {
          T acc = T(0);
          for (int i = 0; i < L; ++i) acc += TT(r, k + 1 + i) * vbuf[i];
          acc *= tau;
          for (int i = 0; i < L; ++i) TT(r, k + 1 + i) -= acc * vbuf[i];
        } else {
          const int rv = r - ns;
          T acc = T(0);
          for (int i = 0; i < L; ++i) acc += VV(rv, k + 1 + i) * vbuf[i];
          acc *= tau;
          for (int i = 0; i < L; ++i) VV(rv, k + 1 + i) -= acc * vbuf[i];
        }
      }
      __syncthreads();
    }
  }
  __syncthreads();
  // ---- the window back into H: Hessenberg part, the new coupling entry s V[0, 0]
  for (int idx = tid; idx < nw * nw; idx += kAedThreads) {
    const int i = idx % nw, j = idx / nw;
    g.H[(size_t)(kwtop - 1 + j) * g.n + (kwtop - 1 + i)] = (i > j + 1) ? T(0) : TT(i, j);
  }
  if (tid == 0) {
    if (kwtop > g.ilo) g.H[(size_t)(kwtop - 2) * g.n + (kwtop - 1)] = s * VV(0, 0);
    g.out[0] = ns;
    g.out[1] = ndef;
    g.out[2] = 1;
  }
}
#undef TT
#undef VV

template <class T>
size_t aed_smem_bytes(int nw) {
  return sizeof(T) * ((size_t)nw * (nw | 1) + nw + 2);
}

template <class T>
cudaError_t launch_aed(const AedArgs<T>& g, cudaStream_t s) {
  const size_t sm = aed_smem_bytes<T>(g.nw);
  cudaError_t e = cudaFuncSetAttribute(k_aed<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_aed<T><<<1, kAedThreads, sm, s>>>(g);
  return cudaGetLastError();
}
template cudaError_t launch_aed<double>(const AedArgs<double>&, cudaStream_t);
template cudaError_t launch_aed<float>(const AedArgs<float>&, cudaStream_t);

}  // namespace gsk
