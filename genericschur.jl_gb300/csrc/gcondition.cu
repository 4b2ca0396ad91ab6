// Generalized Sylvester solves and condition estimates of a complex generalized Schur
// form (S, T) (src/gsylvester.jl, src/gcondition.jl).
//
//   trsylvester!(A, B, C, D, E, F)     A R - L B = s C,  D R - L E = s F   (gsylvester.jl:23-99)
//   adjtrsylvester!(A, B, C, D, E, F)  A^H R + D^H L = s C, R B^H + L E^H = -s F (:103-155)
//   _trgsep (look-ahead)               zlatdf-style growth of R, L on zero right-hand
//                                      sides; dif = sqrt(2 m n) / ||[R L]||_F (gcondition.jl:8-115)
//
// A, D are m x m and B, E n x n upper triangular; C, F (m x n) are overwritten with R, L.
// The reference solves element by element (j ascending, i descending; for the adjoint
// i ascending, j descending) and pushes each solution into the right-hand sides still to
// come.  Element (i, j) therefore needs every element of its row to the left and of its
// column below (adjoint: above and to the right), so the elements of one anti-diagonal are
// independent: k_gsyl_wave runs the anti-diagonals in turn on a cooperative grid, with a
// bounded grid barrier between levels.
//
// Each element pulls the updates the reference pushes into it, in the reference's order:
// forward: the L terms l = 0 .. j-1, then the R terms k = m-1 .. i+1; adjoint: C from the
// rows above in ascending order, F from the columns to the right in descending order.
// An SM sub-partition issues one FP64 warp instruction in tens of cycles, so an element is
// a warp: the lanes form the complex products of 32 terms at once and four lanes add them
// to the four real components of the sums, one FP64 add per term on the serial path instead
// of sixteen FP64 operations.  What remains is the dependency structure: one level after
// another, each as long as its longest element's serial sum.  The elements of a level go to
// the CTAs' first warps before any SM takes a second one.
// Products and sums are plain IEEE operations (no contraction) with the reference's
// complex formulas, so the result is the reference's to the bit on the same inputs, apart
// from hypot in the pivot tests.
//
// Rescaling: the reference scales all of C and F when a 2 x 2 solve returns a scale below
// one, through lmul!(view, scale), which LinearAlgebra defines for no such argument order,
// so that branch raises there.  The kernel flags the case and the host reports an error.
// _trgsep factors each 2 x 2 system with lu(Z), which raises SingularException on a zero
// pivot; the kernel flags that too.
#include "gs_internal.h"
#include "device_common.cuh"

namespace gsk {
namespace {

constexpr int kGsT = 256;  // threads per CTA
constexpr int kGsW = kGsT / 32;  // warps per CTA, one element each

// ---- IEEE complex arithmetic without contraction ----------------------------------------
__device__ __forceinline__ double2 xadd(double2 a, double2 b) { return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)); }
__device__ __forceinline__ double2 xsub(double2 a, double2 b) { return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y)); }
__device__ __forceinline__ double2 xmul(double2 a, double2 b) {
  return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                      __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 xscal(double2 a, double s) { return make_double2(__dmul_rn(a.x, s), __dmul_rn(a.y, s)); }
// Smith's division
__device__ double2 xdiv(double2 a, double2 b) {
  if (fabs(b.y) <= fabs(b.x)) {
    if (b.x == 0.0 && b.y == 0.0) return make_double2(__ddiv_rn(a.x, b.x), __ddiv_rn(a.y, b.x));
    const double r = __ddiv_rn(b.y, b.x), d = __dadd_rn(b.x, __dmul_rn(b.y, r));
    return make_double2(__ddiv_rn(__dadd_rn(a.x, __dmul_rn(a.y, r)), d), __ddiv_rn(__dsub_rn(a.y, __dmul_rn(a.x, r)), d));
  }
  const double r = __ddiv_rn(b.x, b.y), d = __dadd_rn(b.y, __dmul_rn(b.x, r));
  return make_double2(__ddiv_rn(__dadd_rn(__dmul_rn(a.x, r), a.y), d), __ddiv_rn(__dsub_rn(__dmul_rn(a.y, r), a.x), d));
}
__device__ __forceinline__ double xabs1(double2 a) { return __dadd_rn(fabs(a.x), fabs(a.y)); }

// _safe_lu_solve! (util.jl:603-690) of the 2 x 2 system Z (column-major), in place on b;
// returns the scale and sets *pert when a pivot was raised to smin.
__device__ double xlu2(double2 Z[4], double2 b[2], bool* pert) {
  const double eps = 2.220446049250313e-16;
  const double smallnum = 2.2250738585072014e-308 / eps;
  double smin = 0.0;
  for (int e = 0; e < 4; ++e) smin = fmax(smin, zabs(Z[e]));
  smin = fmax(__dmul_rn(eps, smin), smallnum);
  double xmax = 0.0;
  int ipsv = 1, jpsv = 1;
  for (int ip = 1; ip <= 2; ++ip)
    for (int jp = 1; jp <= 2; ++jp) {
      const double v = zabs(Z[(ip - 1) + (jp - 1) * 2]);
      if (v >= xmax) { xmax = v; ipsv = ip; jpsv = jp; }
    }
  if (ipsv != 1) {
    double2 t = Z[0]; Z[0] = Z[1]; Z[1] = t;
    t = Z[2]; Z[2] = Z[3]; Z[3] = t;
    t = b[0]; b[0] = b[1]; b[1] = t;
  }
  if (jpsv != 1) {
    double2 t = Z[0]; Z[0] = Z[2]; Z[2] = t;
    t = Z[1]; Z[1] = Z[3]; Z[3] = t;
  }
  if (zabs(Z[0]) < smin) { *pert = true; Z[0] = make_double2(smin, 0.0); }
  Z[1] = xdiv(Z[1], Z[0]);
  b[1] = xsub(b[1], xmul(Z[1], b[0]));
  Z[3] = xsub(Z[3], xmul(Z[1], Z[2]));
  if (zabs(Z[3]) < smin) { *pert = true; Z[3] = make_double2(smin, 0.0); }
  double scale = 1.0;
  const double aa = 8.0 * smallnum;
  if (__dmul_rn(aa, zabs(b[0])) > zabs(Z[0]) || __dmul_rn(aa, zabs(b[1])) > zabs(Z[3])) {
    const double bmax = fmax(zabs(b[0]), zabs(b[1]));
    scale = __ddiv_rn(0.125, bmax);
    b[0] = xscal(b[0], scale);
    b[1] = xscal(b[1], scale);
  }
  const double2 one = make_double2(1.0, 0.0);
  b[1] = xmul(b[1], xdiv(one, Z[3]));
  const double2 t = xdiv(one, Z[0]);
  b[0] = xmul(b[0], t);
  b[0] = xsub(b[0], xmul(xmul(t, Z[2]), b[1]));
  if (jpsv != 1) { const double2 u = b[0]; b[0] = b[1]; b[1] = u; }
  return scale;
}

// The look-ahead solve of _trgsep (gcondition.jl:36-96) for Z = [a -b; d -e] and the
// accumulated right-hand side (c, f): returns false on a zero pivot of lu(Z).
__device__ bool xlookahead(double2 a, double2 d, double2 mb, double2 me, double2& c, double2& f) {
  const double2 cone = make_double2(1.0, 0.0);
  // lu(Z): partial pivoting on |re| + |im|
  const bool sw = xabs1(d) > xabs1(a);
  const double2 u11 = sw ? d : a, u12 = sw ? me : mb, z21 = sw ? a : d, z22 = sw ? mb : me;
  if (u11.x == 0.0 && u11.y == 0.0) return false;
  const double2 l21 = xdiv(z21, u11);
  const double2 u22 = xsub(z22, xmul(l21, u12));
  if (u22.x == 0.0 && u22.y == 0.0) return false;
  double2 x0 = sw ? f : c, x1 = sw ? c : f;
  double2 pmone = make_double2(-1.0, 0.0);
  const double2 bp = xadd(x0, cone), bm = xsub(x0, cone);
  double splus = __dadd_rn(1.0, xmul(zconj(l21), l21).x);
  const double sminu = xmul(zconj(l21), x1).x;
  splus = __dmul_rn(splus, x0.x);
  if (splus > sminu) x0 = bp;
  else if (sminu > splus) x0 = bm;
  else { x0 = xadd(x0, pmone); pmone = cone; }
  x1 = xsub(x1, xmul(x0, l21));
  double2 w0 = x0, w1 = xadd(x1, cone);
  x1 = xsub(x1, cone);
  double sp = 0.0, sm = 0.0;
  {
    const double2 t = xdiv(cone, u22);
    w1 = xmul(w1, t);
    x1 = xmul(x1, t);
    sp = __dadd_rn(sp, zabs(w1));
    sm = __dadd_rn(sm, zabs(x1));
  }
  {
    const double2 t = xdiv(cone, u11);
    w0 = xmul(w0, t);
    x0 = xmul(x0, t);
    const double2 ut = xmul(u12, t);
    w0 = xsub(w0, xmul(w1, ut));
    x0 = xsub(x0, xmul(x1, ut));
    sp = __dadd_rn(sp, zabs(w0));
    sm = __dadd_rn(sm, zabs(x0));
  }
  if (sp > sm) { x0 = w0; x1 = w1; }
  // x = x[fZ.p]: the row permutation applied to the solution, as the reference does
  c = sw ? x1 : x0;
  f = sw ? x0 : x1;
  return true;
}

// Grid barrier of a cooperative launch: arrival counter and generation word; a wait gives
// up after about four seconds and marks the barrier broken, after which every later
// barrier of the launch returns at once.
__device__ bool gs_grid_sync(GsylBar* bar, unsigned nblocks) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = &bar->gen;
    volatile int* verr = &bar->err;
    ok = *verr == 0;
    if (ok) {
      const unsigned g = *vgen;
      __threadfence();
      if (atomicAdd(&bar->count, 1u) == nblocks - 1) {
        bar->count = 0;
        __threadfence();
        atomicAdd(&bar->gen, 1u);
      } else {
        long long it = 0;
        while (*vgen == g) {
          if (++it > (1LL << 25)) { atomicOr(&bar->err, 1); ok = 0; break; }
          __nanosleep(128);
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok;
}

// Accumulates the 32-term chunk held in pb into acc (lanes 0..3, one real component each).
__device__ __forceinline__ double chunk_sum(double acc, const double (*pb)[4], int lane, int cnt) {
  if (cnt == 32) {
#pragma unroll
    for (int u = 0; u < 32; ++u) acc = __dadd_rn(acc, pb[u][lane]);
  } else {
    for (int u = 0; u < cnt; ++u) acc = __dadd_rn(acc, pb[u][lane]);
  }
  return acc;
}

// One warp per element.  Lane u forms the complex products of terms t0 + u of the element's
// sums (the FP64 products of 32 terms in one pass); lanes 0..3 then add them, in the
// reference's order, to the four real accumulators Re C, Im C, Re F, Im F.
__global__ void __launch_bounds__(kGsT) k_gsyl_wave(GsylArgs P) {
  __shared__ double buf[kGsW][32][4];
  const int G = gridDim.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int e0 = blockIdx.x + G * w, stride = G * kGsW;
  double(*pb)[4] = buf[w];
  const int m = P.m, n = P.n;
  const double2 *A = P.A, *B = P.B, *D = P.D, *E = P.E;
  double2 *C = P.C, *F = P.F;
  const size_t lda = P.lda, ldb = P.ldb, ldd = P.ldd, lde = P.lde, ldc = P.ldc, ldf = P.ldf;
  int fl = 0;
  for (int d = 0; d <= m + n - 2; ++d) {
    if (P.mode != 1) {
      // (i, j) with (m - 1 - i) + j = d: the L terms l = 0 .. j-1, then the R terms
      // k = m-1 .. i+1, d terms in all
      const int jlo = max(0, d - (m - 1)), jhi = min(n - 1, d);
      for (int j = jlo + e0; j <= jhi; j += stride) {
        const int i = m - 1 - d + j;
        double acc = 0.0;
        if (lane < 4) {
          const double2 c0 = lane < 2 ? __ldcg(&C[i + j * ldc]) : __ldcg(&F[i + j * ldf]);
          acc = (lane & 1) ? c0.y : c0.x;
        }
        for (int t0 = 0; t0 < d; t0 += 32) {
          const int t = t0 + lane;
          if (t < d) {
            double2 x, y1, y2;
            if (t < j) {
              x = __ldcg(&F[i + t * ldf]);
              y1 = __ldg(&B[t + j * ldb]);
              y2 = __ldg(&E[t + j * lde]);
            } else {
              const int k = m - 1 - (t - j);
              x = zneg(__ldcg(&C[k + j * ldc]));
              y1 = __ldg(&A[i + k * lda]);
              y2 = __ldg(&D[i + k * ldd]);
            }
            const double2 p1 = xmul(x, y1), p2 = xmul(x, y2);
            pb[lane][0] = p1.x;
            pb[lane][1] = p1.y;
            pb[lane][2] = p2.x;
            pb[lane][3] = p2.y;
          }
          __syncwarp();
          if (lane < 4) acc = chunk_sum(acc, pb, lane, min(32, d - t0));
          __syncwarp();
        }
        const double a0 = __shfl_sync(0xffffffffu, acc, 0), a1 = __shfl_sync(0xffffffffu, acc, 1);
        const double a2 = __shfl_sync(0xffffffffu, acc, 2), a3 = __shfl_sync(0xffffffffu, acc, 3);
        if (lane == 0) {
          double2 ac = make_double2(a0, a1), af = make_double2(a2, a3);
          const double2 aii = __ldg(&A[i + i * lda]), dii = __ldg(&D[i + i * ldd]);
          const double2 mbjj = zneg(__ldg(&B[j + j * ldb])), mejj = zneg(__ldg(&E[j + j * lde]));
          if (P.mode == 0) {
            double2 Z[4] = {aii, dii, mbjj, mejj};
            double2 rhs[2] = {ac, af};
            bool pert = false;
            const double sc = xlu2(Z, rhs, &pert);
            if (pert) fl |= 1;
            if (sc != 1.0) fl |= 2;
            ac = rhs[0];
            af = rhs[1];
          } else if (!xlookahead(aii, dii, mbjj, mejj, ac, af)) {
            fl |= 4;
          }
          C[i + j * ldc] = ac;
          F[i + j * ldf] = af;
        }
        __syncwarp();
      }
    } else {
      // (i, j) with i + (n - 1 - j) = d: C takes the rows above in ascending order (i
      // terms), F the columns to the right in descending order (n - 1 - j terms); C's
      // subtractions are stored as additions of the negated terms
      const int ilo = max(0, d - (n - 1)), ihi = min(m - 1, d);
      for (int i = ilo + e0; i <= ihi; i += stride) {
        const int j = n - 1 - d + i;
        const int nC = i, nF = n - 1 - j;
        double acc = 0.0;
        if (lane < 4) {
          const double2 c0 = lane < 2 ? __ldcg(&C[i + j * ldc]) : __ldcg(&F[i + j * ldf]);
          acc = (lane & 1) ? c0.y : c0.x;
        }
        const int nmax = max(nC, nF);
        for (int t0 = 0; t0 < nmax; t0 += 32) {
          const int t = t0 + lane;
          if (t < nC) {
            const double2 x1 = __ldcg(&C[t + j * ldc]), x2 = __ldcg(&F[t + j * ldf]);
            const double2 q = xadd(xmul(x1, zconj(__ldg(&A[t + i * lda]))), xmul(x2, zconj(__ldg(&D[t + i * ldd]))));
            pb[lane][0] = -q.x;
            pb[lane][1] = -q.y;
          }
          if (t < nF) {
            const int c = n - 1 - t;
            const double2 x1 = __ldcg(&C[i + c * ldc]), x2 = __ldcg(&F[i + c * ldf]);
            const double2 q = xadd(xmul(x1, zconj(__ldg(&B[j + c * ldb]))), xmul(x2, zconj(__ldg(&E[j + c * lde]))));
            pb[lane][2] = q.x;
            pb[lane][3] = q.y;
          }
          __syncwarp();
          if (lane < 4) {
            const int cnt = min(32, (lane < 2 ? nC : nF) - t0);
            if (cnt > 0) acc = chunk_sum(acc, pb, lane, cnt);
          }
          __syncwarp();
        }
        const double a0 = __shfl_sync(0xffffffffu, acc, 0), a1 = __shfl_sync(0xffffffffu, acc, 1);
        const double a2 = __shfl_sync(0xffffffffu, acc, 2), a3 = __shfl_sync(0xffffffffu, acc, 3);
        if (lane == 0) {
          double2 Z[4] = {zconj(__ldg(&A[i + i * lda])), zneg(zconj(__ldg(&B[j + j * ldb]))),
                          zconj(__ldg(&D[i + i * ldd])), zneg(zconj(__ldg(&E[j + j * lde])))};
          double2 rhs[2] = {make_double2(a0, a1), make_double2(a2, a3)};
          bool pert = false;
          const double sc = xlu2(Z, rhs, &pert);
          if (pert) fl |= 1;
          if (sc != 1.0) fl |= 2;
          C[i + j * ldc] = rhs[0];
          F[i + j * ldf] = rhs[1];
        }
        __syncwarp();
      }
    }
    __threadfence();
    if (!gs_grid_sync(P.bar, G)) { fl |= 8; break; }
  }
  fl = __reduce_or_sync(0xffffffffu, fl);
  if (lane == 0 && fl) atomicOr(P.flag, fl);
}

}  // namespace

size_t gsyl_bar_bytes() { return sizeof(GsylBar); }

// P.bar and P.flag must be zeroed on the stream beforehand.
cudaError_t launch_gsyl(const GsylArgs& P, int num_sms, cudaStream_t s) {
  if (P.m == 0 || P.n == 0) return cudaSuccess;
  const int maxlev = std::min(P.m, P.n);
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gsyl_wave, kGsT, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  // one CTA per SM at most: element e of a level runs on CTA e mod G, warp e / G, so the
  // elements fill the SMs' first warps before any SM takes a second one
  const int G = std::max(1, std::min(num_sms, maxlev));
  GsylArgs a = P;
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)k_gsyl_wave, dim3(G), dim3(kGsT), args, 0, s);
}

}  // namespace gsk
