// Eigenvalue adjoint, batched: the backward pass of A -> eigenvalues(A).
//
// For eigenvalue l_i with right eigenvector x_i and left eigenvector y_i
// (A^H y_i = conj(l_i) y_i, the convention of _gleigvecs!, vectors.jl:372-460),
// first-order perturbation gives dl_i = y_i^H dA x_i / (y_i^H x_i).  For a real loss
// with cotangents g_i = dL/dRe(l_i) + i dL/dIm(l_i) the gradient with respect to A
// (dL/dRe(A) + i dL/dIm(A)) is
//     grad = sum_i g_i y_i x_i^H / conj(y_i^H x_i) = Y diag(c) X^H,  c_i = g_i / conj(s_i),
// which does not depend on how x_i and y_i are scaled.  One CTA per matrix: the
// s_i are column dot products (one warp each) and the contraction is a complex
// GEMM with the diagonal folded into Y, read through L1 from the eigenvector buffers.
#include "device_common.cuh"
#include "gs_internal.h"

namespace gsk {
namespace {

template <int NT>
__global__ void __launch_bounds__(NT) k_eig_adjoint(AdjBatch ab) {
  extern __shared__ double2 sm[];
  const int tid = threadIdx.x;
  for (int b = blockIdx.x; b < ab.count; b += gridDim.x) {
    const int n = ab.ns[b];
    if (n <= 0 || n > kSmallMax) continue;  // shared memory is sized for kSmallMax; device orders are unchecked
    const long long off = ab.offs[b];
    const double2* __restrict__ X = ab.VR + off;
    const double2* __restrict__ Y = ab.VL + off;
    const double2* __restrict__ g = ab.gbar + ab.woffs[b];
    double2* __restrict__ G = ab.grad + off;
    double2* cs = sm;  // c_i
    // s_i = y_i^H x_i, c_i = g_i / conj(s_i): one warp per column
    const int lane = tid & 31, wid = tid >> 5;
    for (int i = wid; i < n; i += NT / 32) {
      double2 s = make_double2(0.0, 0.0);
      for (int r = lane; r < n; r += 32) s = zfmac(Y[r + (long long)i * n], X[r + (long long)i * n], s);
      for (int o = 16; o > 0; o >>= 1) {
        s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
        s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
      }
      if (lane == 0) cs[i] = zdiv(g[i], zconj(s));
    }
    __syncthreads();
    // G[j, k] = sum_i Y[j, i] c_i conj(X[k, i]); a thread computes a 1 x 4 strip of G,
    // consecutive threads consecutive rows j (coalesced reads of Y, broadcast reads of X)
    for (int t = tid; t < n * ((n + 3) / 4); t += NT) {
      const int j = t % n, k0 = (t / n) * 4;
      double2 acc[4] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0),
                        make_double2(0.0, 0.0)};
      for (int i = 0; i < n; ++i) {
        const double2 yv = zmul(Y[j + (long long)i * n], cs[i]);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (k0 + q < n) acc[q] = zfma(yv, zconj(X[(k0 + q) + (long long)i * n]), acc[q]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (k0 + q < n) G[j + (long long)(k0 + q) * n] = acc[q];
    }
    __syncthreads();
  }
}

}  // namespace

size_t eig_adjoint_smem_bytes(int nmax) { return sizeof(double2) * (size_t)nmax; }

cudaError_t launch_eig_adjoint(const AdjBatch& ab, int nmax, int num_sms, cudaStream_t s) {
  const size_t smem = eig_adjoint_smem_bytes(nmax);
  cudaError_t e = cudaFuncSetAttribute(k_eig_adjoint<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eig_adjoint<256>, 256, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  int grid = num_sms * per_sm;
  if (grid > ab.count) grid = ab.count;
  if (grid < 1) grid = 1;
  k_eig_adjoint<256><<<grid, 256, smem, s>>>(ab);
  return cudaGetLastError();
}

}  // namespace gsk
