// Real standard-form quasi-triangular Schur pair -> complex triangular Schur pair
// (triangularize, triang.jl:9-43), batched, one CTA per matrix.
//
// For each 2x2 block [a b; c a] (bc < 0) at rows/columns (j-1, j), j = n..2, the
// unitary rotation G = [cs, -i sn; -i sn, cs] with cs = sqrt|b|/r, sn = sqrt|c|/r,
// r = hypot(sqrt|c|, sqrt|b|) is applied as T <- G T G^H, Z <- Z G^H.  Work is done
// in the complex output buffers (L2-resident); rotations of different blocks act
// on disjoint coordinates and are applied one block after another.
//
// colmap[b][ki] receives the column of the reference's real-Schur eigenvalue order
// (GenericSchur.jl:678-679 puts a + i*rti first) that complex eigenvalue ki
// corresponds to, so eigenvectors computed from the complex pair can be returned
// in the order of S.values.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

template <int NT>
__global__ void __launch_bounds__(NT) k_triangularize(TriBatch tb) {
  const int tid = threadIdx.x;
  for (int b = blockIdx.x; b < tb.count; b += gridDim.x) {
    const int n = tb.ns[b];
    const long long off = tb.offs[b];
    const double* __restrict__ Tr = tb.Tr + off;
    const double* __restrict__ Zr = tb.Zr ? tb.Zr + off : nullptr;
    double2* __restrict__ Tc = tb.Tc + off;
    double2* __restrict__ Zc = tb.Zc ? tb.Zc + off : nullptr;
    for (int idx = tid; idx < n * n; idx += NT) {
      Tc[idx] = make_double2(Tr[idx], 0.0);
      if (Zc) Zc[idx] = make_double2(Zr ? Zr[idx] : ((idx % n) == (idx / n) ? 1.0 : 0.0), 0.0);
    }
    __syncthreads();
    for (int j = n; j >= 2; --j) {
      const double sub = Tr[(j - 1) + (long long)(j - 2) * n];  // Tr[j, j-1]
      if (sub == 0.0) continue;
      const double s = sqrt(fabs(sub));
      const double cc = sqrt(fabs(Tr[(j - 2) + (long long)(j - 1) * n]));  // sqrt|Tr[j-1, j]|
      const double r = hypot(s, cc);
      const double gc = cc / r;      // Givens c (real)
      const double gs = -(s / r);    // Givens s = i * gs (purely imaginary)
      const int p = j - 2, q = j - 1;  // 0-based rows/cols of the block
      // lmul!(G, T): rows p, q; new_p = c a1 + s a2; new_q = -conj(s) a1 + c a2, s = i gs
      for (int k = tid; k < n; k += NT) {
        const double2 a1 = Tc[p + (long long)k * n], a2 = Tc[q + (long long)k * n];
        Tc[p + (long long)k * n] = make_double2(gc * a1.x - gs * a2.y, gc * a1.y + gs * a2.x);
        Tc[q + (long long)k * n] = make_double2(gc * a2.x - gs * a1.y, gc * a2.y + gs * a1.x);
      }
      __syncthreads();
      // rmul!(T, G') and rmul!(Z, G'): columns p, q; new_p = a1 c + a2 conj(s); new_q = -a1 s + a2 c
      for (int k = tid; k < n; k += NT) {
        double2 a1 = Tc[k + (long long)p * n], a2 = Tc[k + (long long)q * n];
        Tc[k + (long long)p * n] = make_double2(gc * a1.x + gs * a2.y, gc * a1.y - gs * a2.x);
        Tc[k + (long long)q * n] = make_double2(gc * a2.x + gs * a1.y, gc * a2.y - gs * a1.x);
        if (Zc) {
          a1 = Zc[k + (long long)p * n];
          a2 = Zc[k + (long long)q * n];
          Zc[k + (long long)p * n] = make_double2(gc * a1.x + gs * a2.y, gc * a1.y - gs * a2.x);
          Zc[k + (long long)q * n] = make_double2(gc * a2.x + gs * a1.y, gc * a2.y - gs * a1.x);
        }
      }
      __syncthreads();
    }
    // triu!(T), values = diag(T), column map
    for (int idx = tid; idx < n * n; idx += NT) {
      const int i = idx % n, jj = idx / n;
      if (i > jj) Tc[idx] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    for (int k = tid; k < n; k += NT) {
      const double2 d = Tc[k + (long long)k * n];
      if (tb.w) tb.w[tb.woffs[b] + k] = d;
      if (tb.colmap) {
        int dst = k;
        const bool lower = (k + 1 < n) && Tr[(k + 1) + (long long)k * n] != 0.0;  // k is first of a pair
        const bool upper = (k > 0) && Tr[k + (long long)(k - 1) * n] != 0.0;      // k is second of a pair
        if (lower && d.y < 0.0) dst = k + 1;
        if (upper && Tc[(k - 1) + (long long)(k - 1) * n].y < 0.0) dst = k - 1;
        tb.colmap[tb.woffs[b] + k] = dst;
      }
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_triangularize(const TriBatch& tb, int num_sms, cudaStream_t s) {
  int grid = tb.count < 4 * num_sms ? tb.count : 4 * num_sms;
  if (grid < 1) grid = 1;
  k_triangularize<128><<<grid, 128, 0, s>>>(tb);
  return cudaGetLastError();
}

}  // namespace gsk
