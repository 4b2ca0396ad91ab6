// Complex Schur decomposition of one large matrix (n > 128) on the whole GPU: the
// complex counterpart of the real large path (schur_large_host.cu), replacing the
// reference's gschur!(A::StridedMatrix{Complex}) (GenericSchur.jl:350-372) with
// gschur!(H::Hessenberg{Complex}, Z) (GenericSchur.jl:194-335).
//
//   1. _scale! (util.jl:14-29): the largest |a_ij|, the safescale! factor sequence;
//   2. Householder Hessenberg reduction (hessenberg.jl:3-17 with the complex
//      _reflector!, householder.jl:56-102), Z accumulated (_materializeQ,
//      hessenberg.jl:150-166): per column one CTA forms the reflector, then grid
//      kernels apply lmul!(H', A[i+1:n, i+1:n]) and rmul!(A[:, i+1:n], H) (and the same
//      right factor to Z) as a vector pass and a rank-one update each;
//   3. QR: repeatedly take the bottom unreduced block [ilo, ihi] (the complex deflation
//      criterion of GenericSchur.jl:240-286).  Blocks of order <= 128 are finished by the
//      batched complex kernel (one CTA, shared memory), whose unitary factor U is applied
//      to the rest of H and to Z by matrix products.  Larger blocks get multishift
//      sweeps: B single-shift bulges in a chain two rows apart, the B shifts being the
//      eigenvalues of the trailing B x B block; the chain is chased in chunks whose
//      window stays in one CTA's shared memory while a grid kernel applies the logged
//      2-element reflectors to the rows and columns outside the window and to Z.  The
//      reflectors of one step have disjoint supports (rows k, k+1 of bulge b and k-2,
//      k-1 of bulge b+1), so they are computed from the state at the start of the step
//      and applied left-then-right, P^H H P.  Multishift chasing changes the shift
//      strategy of the reference's one-shift sweeps, and it does not keep the
//      subdiagonal real (the reference's phase fix-ups): parity is by backward error,
//      orthogonality and matched eigenvalues, as for the real large path;
//   4. T = triu(H), values = diag(T), the scaling undone.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

constexpr int kZT = 256;       // threads of the grid kernels
constexpr int kZRT = 512;      // threads of the reflector CTA
constexpr int kZChunk = 16;    // chase steps per chunk
constexpr int kZChunkMax = 48; // longest chunk (the chase log and the far kernel's shared memory)
constexpr int kZMaxB = 32;     // bulges per chain
constexpr int kZFarTile = 32;  // rows / columns per CTA of the far-update kernel
constexpr int kZRowPart = 64;  // columns per partial of the row-vector pass
constexpr int kZAedW = 32;     // aggressive-early-deflation window
constexpr int kZAedMax = 64;   // largest window (shared memory of k_zaed)

__device__ __forceinline__ double2 zc(double r) { return make_double2(r, 0.0); }

// ---- 1. scaling -------------------------------------------------------------------
__global__ void k_zabsmax(const double2* __restrict__ A, size_t cnt, unsigned long long* out) {
  double m = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (size_t)gridDim.x * blockDim.x) {
    const double a = hypot(A[i].x, A[i].y);
    m = (a > m || a != a) ? a : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, m, o);
    m = (w > m || w != w) ? w : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

__global__ void k_zscale(double2* A, size_t cnt, double mul) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (size_t)gridDim.x * blockDim.x)
    A[i] = zscal(A[i], mul);
}

__global__ void k_zidentity(int n, double2* Z) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  Z[idx] = zc((idx % n) == (idx / n) ? 1.0 : 0.0);
}

// ---- 2. Hessenberg reduction --------------------------------------------------------
// Reflector of column i (1-based; rows i+1..n): x[0] <- beta, u (length n) = (0, .., 0, 1,
// essential part), st[0] = tau, and the entries below the subdiagonal set to zero.
__global__ void __launch_bounds__(kZRT) k_zh_refl(int n, double2* A, int i, double2* u, double2* st) {
  __shared__ double red[32];
  double2* x = A + (size_t)(i - 1) * n + i;
  const int m = n - i;
  const double2 tau = cta_reflector<kZRT>(x, m, red);
  __syncthreads();
  for (int r = threadIdx.x; r < n; r += kZRT)
    u[r] = r < i ? zc(0.0) : (r == i ? zc(1.0) : x[r - i]);
  __syncthreads();
  for (int r = i + 1 + threadIdx.x; r < n; r += kZRT) A[(size_t)(i - 1) * n + r] = zc(0.0);
  if (threadIdx.x == 0) st[0] = tau;
}

// v_c = sum_{r >= i} conj(u_r) A(r, c) for the 0-based columns c >= i: one warp per column.
__global__ void __launch_bounds__(kZT) k_zh_leftvec(int n, const double2* __restrict__ A, int i,
                                                    const double2* __restrict__ u, double2* __restrict__ v) {
  const int lane = threadIdx.x & 31;
  const int c = i + blockIdx.x * (kZT / 32) + (threadIdx.x >> 5);
  if (c >= n) return;
  const double2* col = A + (size_t)c * n;
  double2 s = zc(0.0);
  for (int r = i + lane; r < n; r += 32) s = zfmac(u[r], col[r], s);
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  if (lane == 0) v[c] = s;
}

// A(r, c) -= conj(tau) u_r v_c for r, c >= i (0-based): lmul!(H', A[i+1:n, i+1:n]).
__global__ void __launch_bounds__(kZT) k_zh_leftupd(int n, double2* __restrict__ A, int i,
                                                    const double2* __restrict__ u, const double2* __restrict__ v,
                                                    const double2* __restrict__ st) {
  const double2 ct = zconj(st[0]);
  const int m = n - i;
  for (size_t idx = (size_t)blockIdx.x * kZT + threadIdx.x; idx < (size_t)m * m; idx += (size_t)gridDim.x * kZT) {
    const int r = i + (int)(idx % m), c = i + (int)(idx / m);
    double2& a = A[(size_t)c * n + r];
    a = zfms(zmul(ct, u[r]), v[c], a);
  }
}

// Row partials of M u over the 0-based columns c >= i, in column blocks of kZRowPart:
// pw[blk][r] (blockIdx.z: 0 = A, 1 = Z).
__global__ void __launch_bounds__(kZT) k_zh_rightvec(int n, const double2* __restrict__ A,
                                                     const double2* __restrict__ Z, int i,
                                                     const double2* __restrict__ u, double2* __restrict__ pw,
                                                     double2* __restrict__ pz, int nblk) {
  const int r = blockIdx.x * kZT + threadIdx.x;
  const int blk = blockIdx.y;
  const double2* M = blockIdx.z ? Z : A;
  if (r >= n) return;
  const int c0 = i + blk * kZRowPart, c1 = min(n, c0 + kZRowPart);
  double2 s = zc(0.0);
  for (int c = c0; c < c1; ++c) s = zfma(M[(size_t)c * n + r], u[c], s);
  (blockIdx.z ? pz : pw)[(size_t)blk * n + r] = s;
  (void)nblk;
}

// M(r, c) -= tau w_r conj(u_c) for all rows r and 0-based columns c >= i, w = the sum of
// the row partials: rmul!(A[:, i+1:n], H) and the same factor on Z.
__global__ void __launch_bounds__(kZT) k_zh_rightupd(int n, double2* __restrict__ A, double2* __restrict__ Z, int i,
                                                     const double2* __restrict__ u,
                                                     const double2* __restrict__ pw,
                                                     const double2* __restrict__ pz, int nblk,
                                                     const double2* __restrict__ st, int cpb) {
  const double2 tau = st[0];
  const int r = blockIdx.x * kZT + threadIdx.x;
  if (r >= n) return;
  double2* M = blockIdx.z ? Z : A;
  const double2* part = blockIdx.z ? pz : pw;
  double2 w = zc(0.0);
  for (int b = 0; b < nblk; ++b) w = zadd(w, part[(size_t)b * n + r]);
  const double2 tw = zmul(tau, w);
  const int c0 = i + blockIdx.y * cpb, c1 = min(n, c0 + cpb);
  for (int c = c0; c < c1; ++c) {
    double2& a = M[(size_t)c * n + r];
    a = zfms(tw, zconj(u[c]), a);
  }
}

// ---- 3. QR ----------------------------------------------------------------------------
// Deflation scan on [ilo, ihi-1] (GenericSchur.jl:240-286 with |.|_1 of the complex
// subdiagonal, which is not kept real here): the largest k whose H[k+1,k] is negligible.
__global__ void k_zdefl_scan(const double2* __restrict__ H, int n, int ilo, int ihi, int* out) {
  const int k = ilo + blockIdx.x * blockDim.x + threadIdx.x;
  if (k > ihi - 1) return;
  const double ulp = kEps, smallnum = kFmin * ((double)n / kEps);
#define HG(i, j) H[(size_t)((j) - 1) * n + ((i) - 1)]
  bool split = false;
  const double2 sd = HG(k + 1, k);
  if (zabs1(sd) <= smallnum) {
    split = true;
  } else {
    const double2 hkk = HG(k, k), hk1 = HG(k + 1, k + 1);
    double tst = zabs1(hkk) + zabs1(hk1);
    if (tst == 0.0) {
      if (k - 1 >= 1) tst += zabs1(HG(k, k - 1));
      if (k + 2 <= n) tst += zabs1(HG(k + 2, k + 1));
    }
    if (zabs1(sd) <= ulp * tst) {
      const double2 up = HG(k, k + 1);
      const double ab = fmax(zabs1(sd), zabs1(up)), ba = fmin(zabs1(sd), zabs1(up));
      const double2 df = zsub(hkk, hk1);
      const double aa = fmax(zabs1(hk1), zabs1(df)), bb = fmin(zabs1(hk1), zabs1(df));
      const double s = aa + ab;
      if (ba * (ab / s) <= fmax(smallnum, ulp * (bb * (aa / s)))) split = true;
    }
  }
#undef HG
  if (split) atomicMax(out, k);
}

struct ZChase {
  double2* H;
  double2* Z;
  int n, ilo, ihi, B, t0, w, wlo, whi;
  const double2* shifts;  // one per bulge
  int* logk;              // w*B positions (0: inactive)
  double2* logr;          // w*B*3: tau, v2, tau*v2
};

// One chunk of the chain's chase inside the window [wlo, whi] (shared memory).  At sweep
// step t bulge b sits at k = ilo + t - 2b.
__global__ void __launch_bounds__(256) k_zchase_chunk(ZChase ca) {
  extern __shared__ double2 W[];
  const int nw = ca.whi - ca.wlo + 1;
  const int ldw = nw;
  __shared__ double2 rf[kZMaxB][3];
  __shared__ int rk[kZMaxB];
  const int tid = threadIdx.x;
  const int n = ca.n;
  for (int idx = tid; idx < nw * nw; idx += blockDim.x) {
    const int i = idx % nw, j = idx / nw;
    W[i + j * ldw] = ca.H[(size_t)(ca.wlo - 1 + j) * n + (ca.wlo - 1 + i)];
  }
  __syncthreads();
#define WW(i, j) W[((i) - ca.wlo) + ((j) - ca.wlo) * ldw]
  for (int s = 0; s < ca.w; ++s) {
    const int t = ca.t0 + s;
    if (tid < ca.B) {
      const int b = tid;
      const int k = ca.ilo + t - 2 * b;
      double2 tau = zc(0.0), v2 = zc(0.0);
      const bool on = k >= ca.ilo && k <= ca.ihi - 1;
      if (on) {
        double2 a, x1;
        if (k == ca.ilo) {
          // start vector of the shift (GenericSchur.jl:409-414 at m = istart), scaled
          a = zsub(WW(k, k), ca.shifts[b]);
          x1 = WW(k + 1, k);
          const double sn = zabs1(a) + zabs1(x1);
          if (sn != 0.0) { a = zscal(a, 1.0 / sn); x1 = zscal(x1, 1.0 / sn); }
        } else {
          a = WW(k, k - 1);
          x1 = WW(k + 1, k - 1);
        }
        tau = zreflector2_fast(a, x1);
        v2 = x1;
        if (k > ca.ilo) {
          WW(k, k - 1) = a;
          WW(k + 1, k - 1) = zc(0.0);
        }
      }
      rk[b] = on ? k : 0;
      rf[b][0] = tau;
      rf[b][1] = v2;
      rf[b][2] = zmul(tau, v2);
      const size_t li = (size_t)s * ca.B + b;
      ca.logk[li] = on ? k : 0;
      ca.logr[3 * li + 0] = tau;
      ca.logr[3 * li + 1] = v2;
      ca.logr[3 * li + 2] = rf[b][2];
    }
    __syncthreads();
    // left (P^H from the left) inside the window: bulge b, columns j >= k_b
    for (int idx = tid; idx < ca.B * nw; idx += blockDim.x) {
      const int b = idx / nw, j = ca.wlo + idx % nw;
      const int k = rk[b];
      if (!k || j < k) continue;
      const double2 h0 = WW(k, j), h1 = WW(k + 1, j);
      const double2 ss = zadd(zmul(zconj(rf[b][0]), h0), zmul(zconj(rf[b][2]), h1));
      WW(k, j) = zsub(h0, ss);
      WW(k + 1, j) = zfms(ss, rf[b][1], h1);
    }
    __syncthreads();
    // right (P from the right) inside the window: bulge b, rows i <= min(k_b + 2, ihi)
    for (int idx = tid; idx < ca.B * nw; idx += blockDim.x) {
      const int b = idx / nw, i = ca.wlo + idx % nw;
      const int k = rk[b];
      if (!k || i > min(k + 2, ca.ihi)) continue;
      const double2 h0 = WW(i, k), h1 = WW(i, k + 1);
      const double2 ss = zadd(zmul(rf[b][0], h0), zmul(rf[b][2], h1));
      WW(i, k) = zsub(h0, ss);
      WW(i, k + 1) = zfms(ss, zconj(rf[b][1]), h1);
    }
    __syncthreads();
  }
#undef WW
  for (int idx = tid; idx < nw * nw; idx += blockDim.x) {
    const int i = idx % nw, j = idx / nw;
    ca.H[(size_t)(ca.wlo - 1 + j) * n + (ca.wlo - 1 + i)] = W[i + j * ldw];
  }
}

// Far updates of one chunk: tiles of columns right of the window (left updates on rows
// wlo..whi), tiles of rows above the window (right updates on columns wlo..whi), tiles
// of rows of Z (right updates).
__global__ void __launch_bounds__(256) k_zchase_far(ZChase ca, int nleft, int nright) {
  extern __shared__ double2 smz[];
  const int nw = ca.whi - ca.wlo + 1;
  const int steps = ca.w, B = ca.B;
  double2* lr = smz;                                   // steps*B*3
  double2* seg = lr + (size_t)steps * B * 3;           // nw x kZFarTile
  int* lk = (int*)(seg + (size_t)nw * kZFarTile);      // steps*B
  const int tid = threadIdx.x;
  const int n = ca.n;
  for (int idx = tid; idx < steps * B * 3; idx += blockDim.x) lr[idx] = ca.logr[idx];
  for (int idx = tid; idx < steps * B; idx += blockDim.x) lk[idx] = ca.logk[idx];
  int tile = blockIdx.x;
  if (tile < nleft) {
    const int c0 = ca.whi + 1 + tile * kZFarTile;
    const int nc = min(kZFarTile, n - c0 + 1);
    for (int idx = tid; idx < nw * kZFarTile; idx += blockDim.x) {
      const int i = idx % nw, c = idx / nw;
      seg[i + c * nw] = (c < nc) ? ca.H[(size_t)(c0 - 1 + c) * n + (ca.wlo - 1 + i)] : zc(0.0);
    }
    __syncthreads();
    for (int s = 0; s < steps; ++s) {
      for (int idx = tid; idx < B * kZFarTile; idx += blockDim.x) {
        const int b = idx / kZFarTile, c = idx % kZFarTile;
        const int k = lk[s * B + b];
        if (!k || c >= nc) continue;
        const double2* r = &lr[(s * B + b) * 3];
        double2* h = &seg[(k - ca.wlo) + c * nw];
        const double2 ss = zadd(zmul(zconj(r[0]), h[0]), zmul(zconj(r[2]), h[1]));
        h[0] = zsub(h[0], ss);
        h[1] = zfms(ss, r[1], h[1]);
      }
      __syncthreads();
    }
    for (int idx = tid; idx < nw * kZFarTile; idx += blockDim.x) {
      const int i = idx % nw, c = idx / nw;
      if (c < nc) ca.H[(size_t)(c0 - 1 + c) * n + (ca.wlo - 1 + i)] = seg[i + c * nw];
    }
    return;
  }
  tile -= nleft;
  double2* M;
  int r0, nrw;
  if (tile < nright) {
    M = ca.H;
    r0 = 1 + tile * kZFarTile;
    nrw = min(kZFarTile, ca.wlo - r0);
  } else {
    tile -= nright;
    M = ca.Z;
    r0 = 1 + tile * kZFarTile;
    nrw = min(kZFarTile, n - r0 + 1);
  }
  for (int idx = tid; idx < kZFarTile * nw; idx += blockDim.x) {
    const int i = idx % kZFarTile, j = idx / kZFarTile;
    seg[i + j * kZFarTile] = (i < nrw) ? M[(size_t)(ca.wlo - 1 + j) * n + (r0 - 1 + i)] : zc(0.0);
  }
  __syncthreads();
  for (int s = 0; s < steps; ++s) {
    for (int idx = tid; idx < B * kZFarTile; idx += blockDim.x) {
      const int b = idx / kZFarTile, i = idx % kZFarTile;
      const int k = lk[s * B + b];
      if (!k || i >= nrw) continue;
      const double2* r = &lr[(s * B + b) * 3];
      double2* h = &seg[i + (k - ca.wlo) * kZFarTile];
      const double2 ss = zadd(zmul(r[0], h[0]), zmul(r[2], h[kZFarTile]));
      h[0] = zsub(h[0], ss);
      h[kZFarTile] = zfms(ss, zconj(r[1]), h[kZFarTile]);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < kZFarTile * nw; idx += blockDim.x) {
    const int i = idx % kZFarTile, j = idx / kZFarTile;
    if (i < nrw) M[(size_t)(ca.wlo - 1 + j) * n + (r0 - 1 + i)] = seg[i + j * kZFarTile];
  }
}

// Aggressive early deflation on the trailing window [kwtop, kwtop + nw - 1] of the active
// block (Braman, Byers, Mathias 2002; the complex form of LAPACK's xLAQR3 without the
// reordering of undeflatable eigenvalues): the window's Schur form Tw = U^H H_w U and U
// come from the batched kernel; the spike s U(1, :)^H (s = H(kwtop, kwtop-1)) is tested from
// the bottom, and the trailing entries below ulp |T_jj| deflate.  When any deflate, the
// spike is folded into one entry by a reflector and the undeflated leading ns x ns part
// of the window returned to Hessenberg form, all in shared memory, with U updated; the
// host then writes the window back and applies U to the rest of H and to Z.  out[0] = ns
// (undeflated), out[1] = nd (deflated); eig = diag(Tw) (the next sweep's shifts); beta =
// the folded spike entry.
__global__ void __launch_bounds__(256) k_zaed(const double2* __restrict__ H, int n, int kwtop, int ilo,
                                              double2* Tw, double2* U, int nw, int* out, double2* eig,
                                              double2* beta_out) {
  extern __shared__ double2 sma[];
  double2* W = sma;              // nw x nw, ld nw
  double2* Us = W + nw * nw;     // nw x nw
  double2* sp = Us + nw * nw;    // nw
  double2* v = sp + nw;          // nw
  __shared__ double red[32];
  __shared__ int s_ns;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < nw * nw; idx += 256) { W[idx] = Tw[idx]; Us[idx] = U[idx]; }
  const double2 s = (kwtop > ilo) ? H[(size_t)(kwtop - 2) * n + (kwtop - 1)] : zc(0.0);
  for (int j = tid; j < nw; j += 256) sp[j] = zmul(s, zconj(U[(size_t)j * nw]));
  __syncthreads();
  if (tid == 0) {
    const double smlnum = kFmin * ((double)n / kEps);
    int ns = nw;
    while (ns > 0) {
      const double2 t = W[(ns - 1) + (size_t)(ns - 1) * nw];
      if (zabs1(sp[ns - 1]) <= fmax(smlnum, kEps * zabs1(t))) --ns;
      else break;
    }
    s_ns = ns;
    out[0] = ns;
    out[1] = nw - ns;
  }
  for (int j = tid; j < nw; j += 256) eig[j] = W[j + (size_t)j * nw];
  __syncthreads();
  const int ns = s_ns;
  if (ns == nw) return;  // nothing deflated: the window stays as it was
  for (int j = ns + tid; j < nw; j += 256) sp[j] = zc(0.0);
  __syncthreads();
  if (ns >= 1 && kwtop > ilo) {
    // fold the spike: P^H sp = beta e1, P = I - tau v v^H on the leading ns entries
    const double2 tau = cta_reflector<256>(sp, ns, red);
    __syncthreads();
    for (int k = tid; k < ns; k += 256) v[k] = (k == 0) ? zc(1.0) : sp[k];
    __syncthreads();
    // W <- P^H W (rows 0..ns-1, every column), W <- W P (columns 0..ns-1), U <- U P
    for (int c = tid; c < nw; c += 256) {
      double2 ss = zc(0.0);
      for (int k = 0; k < ns; ++k) ss = zfmac(v[k], W[k + (size_t)c * nw], ss);
      ss = zmul(zconj(tau), ss);
      for (int k = 0; k < ns; ++k) W[k + (size_t)c * nw] = zfms(ss, v[k], W[k + (size_t)c * nw]);
    }
    __syncthreads();
    for (int r = tid; r < 2 * nw; r += 256) {
      double2* M = r < nw ? W : Us;
      const int rr = r < nw ? r : r - nw;
      double2 ss = zc(0.0);
      for (int k = 0; k < ns; ++k) ss = zfma(M[rr + (size_t)k * nw], v[k], ss);
      ss = zmul(tau, ss);
      for (int k = 0; k < ns; ++k) M[rr + (size_t)k * nw] = zfms(ss, zconj(v[k]), M[rr + (size_t)k * nw]);
    }
    __syncthreads();
    // Hessenberg form of the leading ns x ns part (hessenberg.jl:3-17 on the block)
    for (int c = 0; c + 2 < ns; ++c) {
      double2* x = &W[(c + 1) + (size_t)c * nw];
      const int m = ns - c - 1;
      const double2 t = cta_reflector<256>(x, m, red);
      __syncthreads();
      for (int k = tid; k < m; k += 256) v[k] = (k == 0) ? zc(1.0) : x[k];
      __syncthreads();
      for (int k = 1 + tid; k < m; k += 256) x[k] = zc(0.0);
      // rows c+1..ns-1 from the left (columns c+1..nw-1)
      for (int cc = c + 1 + tid; cc < nw; cc += 256) {
        double2 ss = zc(0.0);
        for (int k = 0; k < m; ++k) ss = zfmac(v[k], W[(c + 1 + k) + (size_t)cc * nw], ss);
        ss = zmul(zconj(t), ss);
        for (int k = 0; k < m; ++k) W[(c + 1 + k) + (size_t)cc * nw] = zfms(ss, v[k], W[(c + 1 + k) + (size_t)cc * nw]);
      }
      __syncthreads();
      // columns c+1..ns-1 from the right (rows 0..ns-1 of W, every row of U)
      for (int r = tid; r < ns + nw; r += 256) {
        double2* M = r < ns ? W : Us;
        const int rr = r < ns ? r : r - ns;
        double2 ss = zc(0.0);
        for (int k = 0; k < m; ++k) ss = zfma(M[rr + (size_t)(c + 1 + k) * nw], v[k], ss);
        ss = zmul(t, ss);
        for (int k = 0; k < m; ++k)
          M[rr + (size_t)(c + 1 + k) * nw] = zfms(ss, zconj(v[k]), M[rr + (size_t)(c + 1 + k) * nw]);
      }
      __syncthreads();
    }
  }
  if (tid == 0) *beta_out = sp[0];
  for (int idx = tid; idx < nw * nw; idx += 256) { Tw[idx] = W[idx]; U[idx] = Us[idx]; }
}

// C (m x p, ldc) = op(A) (m x q) * B (q x p), op(A) = A (conjA = 0) or A^H (conjA = 1).
__global__ void __launch_bounds__(256) k_zgemm(int m, int p, int q, const double2* __restrict__ A, int lda,
                                               int conjA, const double2* __restrict__ B, int ldb,
                                               double2* __restrict__ C, int ldc) {
  __shared__ double2 As[16][33];
  __shared__ double2 Bs[16][33];
  const int tid = threadIdx.x;
  const int tr = tid % 16, tc = tid / 16;  // 16 x 16 threads, 2 x 2 outputs each
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  double2 acc[2][2];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) acc[a][b] = zc(0.0);
  for (int k0 = 0; k0 < q; k0 += 16) {
    for (int idx = tid; idx < 16 * 32; idx += 256) {
      const int kk = idx / 32, ii = idx % 32;
      const int i = i0 + ii, k = k0 + kk;
      double2 av = zc(0.0);
      if (i < m && k < q) av = conjA ? zconj(A[(size_t)i * lda + k]) : A[(size_t)k * lda + i];
      As[kk][ii] = av;
      const int j = j0 + ii;
      Bs[kk][ii] = (j < p && k < q) ? B[(size_t)j * ldb + k] : zc(0.0);
    }
    __syncthreads();
    for (int kk = 0; kk < 16; ++kk) {
      const double2 a0 = As[kk][tr], a1 = As[kk][tr + 16];
      const double2 b0 = Bs[kk][tc], b1 = Bs[kk][tc + 16];
      acc[0][0] = zfma(a0, b0, acc[0][0]);
      acc[0][1] = zfma(a0, b1, acc[0][1]);
      acc[1][0] = zfma(a1, b0, acc[1][0]);
      acc[1][1] = zfma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
  for (int x = 0; x < 2; ++x)
    for (int y = 0; y < 2; ++y) {
      const int i = i0 + tr + 16 * x, j = j0 + tc + 16 * y;
      if (i < m && j < p) C[(size_t)j * ldc + i] = acc[x][y];
    }
}

// dst (m x p, ld ldd) <- src (m x p, ld lds)
__global__ void k_zcopy2d(int m, int p, const double2* __restrict__ src, int lds, double2* __restrict__ dst, int ldd) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)m * p) return;
  const int i = idx % m, j = idx / m;
  dst[(size_t)j * ldd + i] = src[(size_t)j * lds + i];
}

// T = triu(H); w = diag(T)
__global__ void k_ztriu_diag(double2* H, int n, double2* w) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int i = idx % n, j = idx / n;
  if (i > j) H[idx] = zc(0.0);
  if (i == j) w[i] = H[idx];
}

__global__ void k_zvec_scale(double2* w, int n, double mul) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) w[i] = zscal(w[i], mul);
}

cudaError_t zcopy2d(int m, int p, const double2* src, int lds, double2* dst, int ldd, cudaStream_t s) {
  if (m <= 0 || p <= 0) return cudaSuccess;
  const size_t tot = (size_t)m * p;
  k_zcopy2d<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(m, p, src, lds, dst, ldd);
  return cudaGetLastError();
}

cudaError_t zgemm(int m, int p, int q, const double2* A, int lda, int conjA, const double2* B, int ldb, double2* C,
                  int ldc, cudaStream_t s) {
  if (m <= 0 || p <= 0) return cudaSuccess;
  dim3 g((m + 31) / 32, (p + 31) / 32);
  k_zgemm<<<g, 256, 0, s>>>(m, p, q, A, lda, conjA, B, ldb, C, ldc);
  return cudaGetLastError();
}

}  // namespace

size_t schur_large_cplx_ws_bytes(int n) {
  const size_t nb = kSmallMax;
  const size_t nblk = ((size_t)n + kZRowPart - 1) / kZRowPart;
  size_t b = 0;
  b += sizeof(double2) * (2 * (size_t)n + 8) + 512;                     // u, v, st
  b += 2 * sizeof(double2) * nblk * n + 512;                             // row partials of A and Z
  b += sizeof(int) * kZChunkMax * kZMaxB + sizeof(double2) * 3 * kZChunkMax * kZMaxB + 512;  // chase log
  b += sizeof(double2) * kZMaxB + 256;                                   // shifts
  b += 2 * sizeof(double2) * nb * nb + sizeof(double2) * nb + 1024;      // block, U, eigenvalues
  b += sizeof(long long) * 4 + sizeof(int) * (2 * nb + 3 * kNumBins + 24) + 768;  // meta, order, iota, sched, status, scan
  b += sizeof(double2) * (size_t)n * nb + 512;                           // product temporary
  b += sizeof(unsigned long long) * 2 + 256;
  b += sizeof(int) * 4 + sizeof(double2) * 2 + 512;                     // AED results
  return b + 16 * 256;
}

// Returns ST_OK / ST_UNCONVERGED, or -1 with *cerr set on a CUDA error.  A (device, n x n,
// ld n) is overwritten by T; Z (may be null) receives the unitary factor; w (n) the
// eigenvalues.
int schur_large_cplx_run(double2* A, double2* Z, double2* w, int n, int scale, long long maxsweeps, void* ws,
                         int num_sms, cudaStream_t s, cudaError_t* cerr) {
  cudaError_t e;
#define CKZ(...)                 \
  do {                           \
    e = (__VA_ARGS__);           \
    if (e != cudaSuccess) {      \
      *cerr = e;                 \
      return -1;                 \
    }                            \
  } while (0)
  char* p = (char*)ws;
  auto take = [&](size_t bytes) { char* q = p; p += (bytes + 255) & ~size_t(255); return (void*)q; };
  const int nb = kSmallMax;
  const int nblk = (n + kZRowPart - 1) / kZRowPart;
  double2* u = (double2*)take(sizeof(double2) * n);
  double2* v = (double2*)take(sizeof(double2) * n);
  double2* st = (double2*)take(sizeof(double2) * 8);
  double2* pw = (double2*)take(sizeof(double2) * nblk * (size_t)n);
  double2* pz = (double2*)take(sizeof(double2) * nblk * (size_t)n);
  int* logk = (int*)take(sizeof(int) * kZChunkMax * kZMaxB);
  double2* logr = (double2*)take(sizeof(double2) * 3 * kZChunkMax * kZMaxB);
  double2* dshift = (double2*)take(sizeof(double2) * kZMaxB);
  double2* blk = (double2*)take(sizeof(double2) * nb * nb);
  double2* U = (double2*)take(sizeof(double2) * nb * nb);
  double2* bw = (double2*)take(sizeof(double2) * nb);
  long long* meta = (long long*)take(sizeof(long long) * 4);
  int* order = (int*)take(sizeof(int) * (nb + 8));
  int* iota = (int*)take(sizeof(int) * (nb + 8));
  int* sched = (int*)take(sizeof(int) * (3 * kNumBins + 4));
  int* bstat = (int*)take(sizeof(int) * 4);
  int* dscan = (int*)take(sizeof(int) * 4);
  double2* tmp = (double2*)take(sizeof(double2) * (size_t)n * nb);
  unsigned long long* dmax = (unsigned long long*)take(sizeof(unsigned long long) * 2);
  int* aout = (int*)take(sizeof(int) * 4);
  double2* abeta = (double2*)take(sizeof(double2) * 2);
  const size_t nn = (size_t)n * n;
  double2* H = A;

  // ---- 1. scale (a NaN or Inf entry can only end in the iteration limit: reported as such)
  double amax = 0.0, cscale = 1.0;
  bool scaled = false;
  {
    CKZ(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), s));
    k_zabsmax<<<4 * num_sms, 256, 0, s>>>(H, nn, dmax);
    unsigned long long bits = 0;
    CKZ(cudaMemcpyAsync(&bits, dmax, sizeof(bits), cudaMemcpyDeviceToHost, s));
    CKZ(cudaStreamSynchronize(s));
    std::memcpy(&amax, &bits, sizeof(amax));
    if (!std::isfinite(amax)) return ST_UNCONVERGED;
  }
  if (scale) {
    const double smlnum = std::sqrt(kFmin) / kEps;
    const double bignum = 1.0 / smlnum;
    if (amax > 0.0 && amax < smlnum) { scaled = true; cscale = smlnum; }
    else if (amax > bignum) { scaled = true; cscale = bignum; }
    if (scaled)
      for (double m : safescale_factors_host(amax, cscale)) k_zscale<<<4 * num_sms, 256, 0, s>>>(H, nn, m);
  }

  // ---- 2. Hessenberg reduction with Z
  if (Z) {
    k_zidentity<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(n, Z);
    CKZ(cudaGetLastError());
  }
  for (int i = 1; i <= n - 2; ++i) {
    const int ic = i;  // 0-based first column of the trailing block
    k_zh_refl<<<1, kZRT, 0, s>>>(n, H, i, u, st);
    const int ncol = n - ic;
    k_zh_leftvec<<<(ncol + (kZT / 32) - 1) / (kZT / 32), kZT, 0, s>>>(n, H, ic, u, v);
    const size_t cells = (size_t)ncol * ncol;
    const unsigned gl = (unsigned)std::min<size_t>((cells + kZT - 1) / kZT, (size_t)8 * num_sms);
    k_zh_leftupd<<<gl, kZT, 0, s>>>(n, H, ic, u, v, st);
    const int nb_i = (ncol + kZRowPart - 1) / kZRowPart;
    dim3 gv((n + kZT - 1) / kZT, nb_i, Z ? 2 : 1);
    k_zh_rightvec<<<gv, kZT, 0, s>>>(n, H, Z, ic, u, pw, pz, nb_i);
    const int rows = (n + kZT - 1) / kZT;
    int cpb = (int)(((long long)ncol * rows * (Z ? 2 : 1) + 4 * num_sms - 1) / (4 * num_sms));
    cpb = std::max(8, cpb);
    dim3 gu(rows, (ncol + cpb - 1) / cpb, Z ? 2 : 1);
    k_zh_rightupd<<<gu, kZT, 0, s>>>(n, H, Z, ic, u, pw, pz, nb_i, st, cpb);
  }
  CKZ(cudaGetLastError());

  // ---- 3. QR
  // the batched complex kernel on H[lo:hi, lo:hi] (copied to blk): T_blk in blk, U (when
  // wanted) in U, eigenvalues in eig; status in bstat
  CKZ(launch_single_meta(iota, (long long*)meta, s));
  auto small_solve = [&](int lo, int hi, bool wantU, double2* eig) -> int {
    const int m = hi - lo + 1;
    CKZ(zcopy2d(m, m, H + (size_t)(lo - 1) * n + (lo - 1), n, blk, m, s));
    CplxBatch bt{};
    bt.count = 1;
    bt.ns = iota + m;
    bt.offs = meta;
    bt.woffs = meta;
    bt.A = blk;
    bt.Z = wantU ? U : nullptr;
    bt.w = eig;
    bt.status = bstat;
    bt.wantz = wantU;
    bt.scale = 0;
    bt.maxiter_mult = 100;
    bt.maxinner_mult = 30;
    CKZ(launch_single_queue(default_bin_of(m), order, sched, s));
    CKZ(launch_schur_cplx_one(bt, m, order, sched, s));
    return 0;
  };
  // the unitary factor U (m x m) of the diagonal block [lo, hi] on the rest of H and on Z
  auto apply_U = [&](int lo, int hi) -> int {
    const int m = hi - lo + 1;
    const int nr = n - hi;
    if (nr > 0) {
      CKZ(zcopy2d(m, nr, H + (size_t)hi * n + (lo - 1), n, tmp, m, s));
      CKZ(zgemm(m, nr, m, U, m, 1, tmp, m, H + (size_t)hi * n + (lo - 1), n, s));
    }
    if (lo > 1) {
      CKZ(zcopy2d(lo - 1, m, H + (size_t)(lo - 1) * n, n, tmp, lo - 1, s));
      CKZ(zgemm(lo - 1, m, m, tmp, lo - 1, 0, U, m, H + (size_t)(lo - 1) * n, n, s));
    }
    if (Z) {
      CKZ(zcopy2d(n, m, Z + (size_t)(lo - 1) * n, n, tmp, n, s));
      CKZ(zgemm(n, m, m, tmp, n, 0, U, m, Z + (size_t)(lo - 1) * n, n, s));
    }
    return 0;
  };

  // Blocks up to nmin go to the batched kernel; a sweep chases at most bmax bulges, chunk
  // steps per window; aedw is the early-deflation window (0: off).  Defaults measured on
  // GB300 with complex N(0,1/2) matrices: 12 bulges without early deflation are fastest up
  // to n ~ 700 (n = 256: 0.19 s against 0.28 s for 32 bulges), 24 bulges with a 32-wide
  // early-deflation window above (n = 1024: 1.74 s against 1.95 s).  GS_CPLX_NMIN,
  // GS_CPLX_BULGES, GS_CPLX_CHUNK and GS_CPLX_AEDW override them for tuning runs.
  const bool big = n >= 768;
  int nmin = 64, bmax = big ? 24 : 12, chunk = kZChunk, aedw = big ? kZAedW : 0;
  if (const char* ev = std::getenv("GS_CPLX_NMIN")) nmin = std::max(16, std::min(nb, std::atoi(ev)));
  if (const char* ev = std::getenv("GS_CPLX_BULGES")) bmax = std::max(1, std::min(kZMaxB, std::atoi(ev)));
  if (const char* ev = std::getenv("GS_CPLX_CHUNK")) chunk = std::max(1, std::min(kZChunkMax, std::atoi(ev)));
  if (const char* ev = std::getenv("GS_CPLX_AEDW")) aedw = std::max(0, std::min(kZAedMax, std::atoi(ev)));
  int ihi = n;
  long long sweeps = 0, since_defl = 0;
  const long long max_sweeps = maxsweeps > 0 ? maxsweeps : 100LL * n;
  std::vector<double2> hsh(kZMaxB);
  while (ihi >= 1) {
    int kmax = 0;
    if (ihi > 1) {
      CKZ(cudaMemsetAsync(dscan, 0, sizeof(int), s));
      k_zdefl_scan<<<(ihi - 1 + 255) / 256, 256, 0, s>>>(H, n, 1, ihi, dscan);
      CKZ(cudaGetLastError());
      CKZ(cudaMemcpyAsync(&kmax, dscan, sizeof(int), cudaMemcpyDeviceToHost, s));
      CKZ(cudaStreamSynchronize(s));
    }
    const int ilo = kmax > 0 ? kmax + 1 : 1;
    if (kmax > 0) CKZ(cudaMemsetAsync(H + (size_t)(ilo - 2) * n + (ilo - 1), 0, sizeof(double2), s));
    int m = ihi - ilo + 1;
    if (m <= nmin) {
      if (small_solve(ilo, ihi, Z != nullptr || ihi < n || ilo > 1, bw)) return -1;
      CKZ(zcopy2d(m, m, blk, m, H + (size_t)(ilo - 1) * n + (ilo - 1), n, s));
      const bool needU = Z != nullptr || ihi < n || ilo > 1;
      if (needU && apply_U(ilo, ihi)) return -1;
      int stv = 0;
      CKZ(cudaMemcpyAsync(&stv, bstat, sizeof(int), cudaMemcpyDeviceToHost, s));
      CKZ(cudaStreamSynchronize(s));
      if (stv != ST_OK) return ST_UNCONVERGED;
      ihi = ilo - 1;
      since_defl = 0;
      continue;
    }
    if (++sweeps > max_sweeps) return ST_UNCONVERGED;
    int B = std::min(bmax, std::max(1, (m - 8) / 4));
    ++since_defl;
    std::vector<double2> sh;
    if (aedw > 0 && since_defl % 10 != 0) {
      // aggressive early deflation on the trailing window
      const int nw = std::min(aedw, m - 1);
      const int kwtop = ihi - nw + 1;
      if (small_solve(kwtop, ihi, true, bw)) return -1;
      const size_t sm = sizeof(double2) * (2 * (size_t)nw * nw + 2 * nw);
      CKZ(cudaFuncSetAttribute(k_zaed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      k_zaed<<<1, 256, sm, s>>>(H, n, kwtop, ilo, blk, U, nw, aout, bw, abeta);
      CKZ(cudaGetLastError());
      int ao[2] = {0, 0}, wst = 0;
      std::vector<double2> ev(nw);
      CKZ(cudaMemcpyAsync(ao, aout, sizeof(ao), cudaMemcpyDeviceToHost, s));
      CKZ(cudaMemcpyAsync(&wst, bstat, sizeof(int), cudaMemcpyDeviceToHost, s));
      CKZ(cudaMemcpyAsync(ev.data(), bw, sizeof(double2) * nw, cudaMemcpyDeviceToHost, s));
      CKZ(cudaStreamSynchronize(s));
      if (wst == ST_OK) {
        const int ns = ao[0], nd = ao[1];
        if (nd > 0) {
          // the window's new form, its spike column, and U on the rest of H and on Z
          CKZ(zcopy2d(nw, nw, blk, nw, H + (size_t)(kwtop - 1) * n + (kwtop - 1), n, s));
          if (kwtop > ilo) {
            double2* col = H + (size_t)(kwtop - 2) * n + (kwtop - 1);
            CKZ(cudaMemsetAsync(col, 0, sizeof(double2) * nw, s));
            if (ns >= 1) CKZ(cudaMemcpyAsync(col, abeta, sizeof(double2), cudaMemcpyDeviceToDevice, s));
          }
          if (apply_U(kwtop, ihi)) return -1;
          ihi = kwtop + ns - 1;
          since_defl = 0;
          // deflated enough (LAPACK's nibble of 14%), or too little left: deflate again first
          if (nd * 100 >= 14 * nw || ns < 2 || ihi - ilo + 1 <= nmin) continue;
          for (int j = ns - 1; j >= 0 && (int)sh.size() < B; --j) sh.push_back(ev[j]);
        } else {
          for (int j = nw - 1; j >= 0 && (int)sh.size() < B; --j) sh.push_back(ev[j]);
        }
        m = ihi - ilo + 1;
        B = std::min(std::min(B, (int)sh.size()), std::max(1, (m - 8) / 4));
        sh.resize(B);
      }
    }
    if ((int)sh.size() == B) {
      // shifts from the deflation window
    } else if (since_defl % 10 == 0) {
      sh.assign(B, make_double2(0.0, 0.0));
      // exceptional shifts (GenericSchur.jl:302-307 pattern): bottom diagonal entries
      // moved by 3/4 of the adjacent subdiagonal magnitude
      for (int b = 0; b < B; ++b) {
        const int k = ihi - b;
        double2 hkk, sd;
        CKZ(cudaMemcpyAsync(&hkk, H + (size_t)(k - 1) * n + (k - 1), sizeof(double2), cudaMemcpyDeviceToHost, s));
        CKZ(cudaMemcpyAsync(&sd, H + (size_t)(k - 2) * n + (k - 1), sizeof(double2), cudaMemcpyDeviceToHost, s));
        CKZ(cudaStreamSynchronize(s));
        const double a = 0.75 * (std::fabs(sd.x) + std::fabs(sd.y));
        sh[b] = make_double2(hkk.x + a, hkk.y);
      }
    } else {
      // the eigenvalues of the trailing B x B block
      sh.assign(B, make_double2(0.0, 0.0));
      if (small_solve(ihi - B + 1, ihi, false, bw)) return -1;
      std::vector<double2> ev(B);
      CKZ(cudaMemcpyAsync(ev.data(), bw, sizeof(double2) * B, cudaMemcpyDeviceToHost, s));
      CKZ(cudaStreamSynchronize(s));
      // bottom-most eigenvalues (the last deflated in the block) lead the chain
      for (int b = 0; b < B; ++b) sh[b] = ev[B - 1 - b];
    }
    CKZ(cudaMemcpyAsync(dshift, sh.data(), sizeof(double2) * B, cudaMemcpyHostToDevice, s));
    const int steps = (ihi - 1 - ilo) + 2 * (B - 1) + 1;
    for (int t0 = 0; t0 < steps; t0 += chunk) {
      const int wc = std::min(chunk, steps - t0);
      const int kmin = std::max(ilo, ilo + t0 - 2 * (B - 1));
      const int kmx = std::min(ihi - 1, ilo + t0 + wc - 1);
      ZChase ca{};
      ca.H = H;
      ca.Z = Z;
      ca.n = n;
      ca.ilo = ilo;
      ca.ihi = ihi;
      ca.B = B;
      ca.t0 = t0;
      ca.w = wc;
      ca.wlo = std::max(ilo, kmin - 1);
      ca.whi = std::min(ihi, kmx + 2);
      ca.shifts = dshift;
      ca.logk = logk;
      ca.logr = logr;
      const int nw = ca.whi - ca.wlo + 1;
      size_t sm = sizeof(double2) * (size_t)nw * nw;
      CKZ(cudaFuncSetAttribute(k_zchase_chunk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      k_zchase_chunk<<<1, 256, sm, s>>>(ca);
      CKZ(cudaGetLastError());
      const int nleft = (n - ca.whi + kZFarTile - 1) / kZFarTile;
      const int nright = (ca.wlo - 1 + kZFarTile - 1) / kZFarTile;
      const int nz = Z ? (n + kZFarTile - 1) / kZFarTile : 0;
      const int tiles = nleft + nright + nz;
      if (tiles > 0) {
        sm = sizeof(double2) * ((size_t)wc * B * 3 + (size_t)nw * kZFarTile) + sizeof(int) * (size_t)wc * B + 16;
        CKZ(cudaFuncSetAttribute(k_zchase_far, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_zchase_far<<<tiles, 256, sm, s>>>(ca, nleft, nright);
        CKZ(cudaGetLastError());
      }
    }
  }

  // ---- 4. T = triu(H), values = diag(T), scaling undone
  k_ztriu_diag<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(H, n, w);
  CKZ(cudaGetLastError());
  if (scaled) {
    for (double m : safescale_factors_host(cscale, amax)) {
      k_zscale<<<4 * num_sms, 256, 0, s>>>(H, nn, m);
      k_zvec_scale<<<(n + 255) / 256, 256, 0, s>>>(w, n, m);
    }
    CKZ(cudaGetLastError());
  }
  return ST_OK;
#undef CKZ
}

}  // namespace gsk
