// Host driver of the large-matrix (n > 128) real Schur path, templated on the
// working precision T (double: the plain FP64 path; float: the first stage of the
// mixed-precision path).
//
//   1. _scale! (util.jl:14-29) with a device max-reduction;
//   2. Hessenberg reduction with Z accumulated (hessenberg_large.cu);
//   3. QR: repeatedly take the bottom unreduced block [ilo, ihi] (deflation scan
//      with the criterion of GenericSchur.jl:563-600).  Blocks of order <= 128 are
//      finished by the small-matrix kernel in FP64 (it returns T_blk and the
//      block's orthogonal factor U; the standard-form 2x2 blocks and the eigenvalue
//      order of the reference come from it), and U is applied to the rest of H and
//      to Z with GEMMs.  Larger blocks get multishift sweeps (schur_large.cu) whose
//      2B shifts are the eigenvalues of the trailing 2B x 2B block, again computed
//      by the small-matrix kernel;
//   4. T = triu(H, -1), scaling undone.
// The host reads two small values per sweep (the split position and the shifts).
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

template <class T>
__global__ void k_absmax_bits(const T* __restrict__ A, size_t cnt, unsigned long long* out) {
  double m = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (size_t)gridDim.x * blockDim.x) {
    const double a = fabs((double)A[i]);
    m = (a > m || a != a) ? a : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, m, o);
    m = (w > m || w != w) ? w : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

template <class T>
__global__ void k_scale(T* A, size_t cnt, double mul) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (size_t)gridDim.x * blockDim.x)
    A[i] = (T)((double)A[i] * mul);
}

template <class T>
__global__ void k_triu1(T* H, int n) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int i = idx % n, j = idx / n;
  if (i > j + 1) H[idx] = T(0);
}

// dst (m x p, ld m) <- src (m x p, ld lds), converting element type
template <class S, class D>
__global__ void k_copy2d(int m, int p, const S* __restrict__ src, int lds, D* __restrict__ dst, int ldd) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)m * p) return;
  const int i = idx % m, j = idx / m;
  dst[(size_t)j * ldd + i] = (D)src[(size_t)j * lds + i];
}

template <class S, class D>
cudaError_t copy2d(int m, int p, const S* src, int lds, D* dst, int ldd, cudaStream_t s) {
  if (m <= 0 || p <= 0) return cudaSuccess;
  const size_t tot = (size_t)m * p;
  k_copy2d<S, D><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(m, p, src, lds, dst, ldd);
  return cudaGetLastError();
}

}  // namespace

void large_tuning(int n, int* bulges, int* chunk, int* aedw, size_t tsize) {
  const char* b = std::getenv("GS_LARGE_BULGES");
  const char* c = std::getenv("GS_LARGE_CHUNK");
  const char* w = std::getenv("GS_LARGE_AEDW");
  *bulges = b ? std::max(1, std::min(kMaxBulges, std::atoi(b))) : (n >= 1024 ? 16 : 12);
  *chunk = c ? std::max(1, std::min(64, std::atoi(c))) : 16;
  // The window's Schur form costs one small-matrix solve per deflation step; in FP64
  // its latency limits the useful window to about two shifts' worth (measured on GB300:
  // 32 at n <= 2048, 48 at n = 4096), in FP32 the solve is cheap and a wider window
  // deflates more.
  const int wdef = tsize == 4 ? 64 : (n >= 3072 ? 48 : 32);
  *aedw = w ? std::max(0, std::min(kSmallMax, std::atoi(w))) : wdef;
}

int large_shift_fp32() {
  const char* f = std::getenv("GS_LARGE_SHIFT32");
  return f ? (std::atoi(f) != 0) : 0;
}

cudaError_t launch_absmax(const double* A, size_t cnt, unsigned long long* out, int num_sms, cudaStream_t s) {
  k_absmax_bits<double><<<4 * num_sms, 256, 0, s>>>(A, cnt, out);
  return cudaGetLastError();
}

// Workspace needed by schur_large_run<T>, in bytes.
size_t schur_large_ws_bytes(int n, size_t tsize) {
  const size_t nb = kSmallMax;
  size_t b = 0;
  b += tsize * std::max(hess_large_ws_elems(n), hess_blocked_ws_elems(n)) + 256;
  b += sizeof(int) * 64 * kMaxBulges + tsize * 64 * kMaxBulges * 5 + 512;  // chase log
  b += tsize * 4 * kMaxBulges + 256;                                        // shifts
  b += 3 * sizeof(double) * nb * nb + 4 * sizeof(double) * nb + 1024;       // small solve blk, U, wr, wi, meta
  b += sizeof(int) * (2 * nb + 3 * kNumBins + 16) + 512;                    // order/iota/sched/status/scan
  b += 2 * sizeof(double) * nb + sizeof(int) * 4 + 512;                      // AED eigenvalues, results
  b += tsize * (size_t)n * nb * 2 + tsize * nb * nb + 512;                  // GEMM temporaries, U in T
  return b + 16 * 256;
}

template <class T>
int schur_large_run(LargeRun<T>& r) {
  const int n = r.n;
  cudaStream_t s = r.stream;
  cudaError_t e;
#define CKL(...)                     \
  do {                               \
    e = (__VA_ARGS__);               \
    if (e != cudaSuccess) {          \
      r.cuda_error = e;              \
      return -1;                     \
    }                                \
  } while (0)
  // ---- carve the workspace
  char* p = (char*)r.ws;
  auto take = [&](size_t bytes) { char* q = p; p += (bytes + 255) & ~size_t(255); return (void*)q; };
  T* hws = (T*)take(sizeof(T) * std::max(hess_large_ws_elems(n), hess_blocked_ws_elems(n)));
  int* logk = (int*)take(sizeof(int) * 64 * kMaxBulges);
  T* logr = (T*)take(sizeof(T) * 64 * kMaxBulges * 5);
  T* dshift = (T*)take(sizeof(T) * 4 * kMaxBulges);
  const int nb = kSmallMax;
  T* blk = (T*)take(sizeof(T) * nb * nb);
  T* U = (T*)take(sizeof(T) * nb * nb);
  float* blk32 = (float*)take(sizeof(float) * nb * nb);
  double* bwr = (double*)take(sizeof(double) * nb);
  double* bwi = (double*)take(sizeof(double) * nb);
  long long* meta = (long long*)take(sizeof(long long) * 4);
  int* order = (int*)take(sizeof(int) * (nb + 8));
  int* iota = (int*)take(sizeof(int) * (nb + 8));
  int* sched = (int*)take(sizeof(int) * (3 * kNumBins + 4));
  int* bstat = (int*)take(sizeof(int) * 4);
  int* dscan = (int*)take(sizeof(int) * 4);
  T* tmp = (T*)take(sizeof(T) * (size_t)n * nb);
  T* tmp2 = (T*)take(sizeof(T) * (size_t)n * nb);
  unsigned long long* dmax = (unsigned long long*)take(sizeof(unsigned long long) * 2);
  double* aewr = (double*)take(sizeof(double) * nb);
  double* aewi = (double*)take(sizeof(double) * nb);
  int* aout = (int*)take(sizeof(int) * 4);
  T* H = r.A;
  T* Z = r.Z;
  const size_t nn = (size_t)n * n;

  // ---- 1. scale (the maximum is also the non-finite check: a NaN or Inf entry can only
  // end in the iteration limit, so it is reported as such without iterating)
  double amax = 0.0, cscale = 1.0;
  bool scaled = false;
  {
    CKL(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), s));
    k_absmax_bits<T><<<4 * r.num_sms, 256, 0, s>>>(H, nn, dmax);
    unsigned long long bits = 0;
    CKL(cudaMemcpyAsync(&bits, dmax, sizeof(bits), cudaMemcpyDeviceToHost, s));
    CKL(cudaStreamSynchronize(s));
    std::memcpy(&amax, &bits, sizeof(amax));
    if (!std::isfinite(amax)) return ST_UNCONVERGED;
  }
  if (r.scale) {
    const double smlnum = std::sqrt((double)Prec<T>::fmin) / (double)Prec<T>::eps;
    const double bignum = 1.0 / smlnum;
    if (amax > 0.0 && amax < smlnum) { scaled = true; cscale = smlnum; }
    else if (amax > bignum) { scaled = true; cscale = bignum; }
    if (scaled) {
      // factor sequence of safescale! (util.jl:41-80), applied in order
      for (double m : safescale_factors_host(amax, cscale)) k_scale<T><<<4 * r.num_sms, 256, 0, s>>>(H, nn, m);
    }
  }

  // ---- 2. Hessenberg (+ Z)
  if (n >= hess_blocked_min(sizeof(T))) {
    int herr = 0;
    CKL(hessenberg_blocked<T>(n, H, n, Z, n, nullptr, hws, r.num_sms, &herr, s));
    if (herr) {
      r.cuda_error = cudaErrorLaunchTimeout;
      return -1;
    }
  } else {
    CKL(hessenberg_large<T>(n, H, n, Z, n, nullptr, hws, s));
  }
  k_triu1<T><<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(H, n);
  CKL(cudaGetLastError());

  // ---- 3. QR
  // The small-matrix kernel in the working precision T on H[lo:hi, lo:hi] (copied to blk;
  // T_blk back in blk, U in U), or -- eigenvalues only, fp32 set -- in FP32.
  CKL(launch_single_meta(iota, meta, s));
  auto small_solve = [&](int lo, int hi, bool wantU, double* wr_out, double* wi_out, bool fp32) -> int {
    const int m = hi - lo + 1;
    if (fp32) {
      CKL(copy2d<T, float>(m, m, H + (size_t)(lo - 1) * n + (lo - 1), n, blk32, m, s));
      RealBatchT<float> bt{};
      bt.count = 1;
      bt.ns = iota + m;
      bt.offs = meta;
      bt.woffs = meta;
      bt.A = blk32;
      bt.Z = nullptr;
      bt.wr = wr_out;
      bt.wi = wi_out;
      bt.status = bstat;
      bt.wantz = 0;
      bt.scale = 0;
      bt.maxiter_mult = 100;
      CKL(launch_single_queue(default_bin_of(m), order, sched, s));
      CKL(launch_schur_real_one<float, double>(bt, m, order, sched, s));
      return 0;
    }
    CKL(copy2d<T, T>(m, m, H + (size_t)(lo - 1) * n + (lo - 1), n, blk, m, s));
    RealBatchT<T> bt{};
    bt.count = 1;
    bt.ns = iota + m;
    bt.offs = meta;
    bt.woffs = meta;
    bt.A = blk;
    bt.Z = wantU ? U : nullptr;
    bt.wr = wr_out;
    bt.wi = wi_out;
    bt.status = bstat;
    bt.wantz = wantU;
    bt.scale = 0;
    bt.maxiter_mult = 100;
    CKL(launch_single_queue(default_bin_of(m), order, sched, s));
    CKL(launch_schur_real_one<T, double>(bt, m, order, sched, s));
    return 0;
  };

  // Apply the orthogonal factor U (m x m, in U) of the diagonal block [lo, hi] to the
  // rest of H and to Z: H[lo:hi, hi+1:n] <- U^T H[lo:hi, hi+1:n], H[1:lo-1, lo:hi] <-
  // H[1:lo-1, lo:hi] U, Z[:, lo:hi] <- Z[:, lo:hi] U.
  auto apply_U = [&](int lo, int hi) -> int {
    const int m = hi - lo + 1;
    const int nr = n - hi;
    if (nr > 0) {
      CKL(copy2d<T, T>(m, nr, H + (size_t)hi * n + (lo - 1), n, tmp, m, s));
      CKL(launch_gemm<T>(m, nr, m, U, m, 1, tmp, m, H + (size_t)hi * n + (lo - 1), n, s));
    }
    if (lo > 1) {
      CKL(copy2d<T, T>(lo - 1, m, H + (size_t)(lo - 1) * n, n, tmp, lo - 1, s));
      CKL(launch_gemm<T>(lo - 1, m, m, tmp, lo - 1, 0, U, m, H + (size_t)(lo - 1) * n, n, s));
    }
    if (Z) {
      CKL(copy2d<T, T>(n, m, Z + (size_t)(lo - 1) * n, n, tmp, n, s));
      CKL(launch_gemm<T>(n, m, m, tmp, n, 0, U, m, Z + (size_t)(lo - 1) * n, n, s));
    }
    return 0;
  };

  const int NMIN = kSmallMax;
  int ihi = n;
  long long sweeps = 0, since_defl = 0;
  const long long max_sweeps = r.maxiter > 0 ? r.maxiter : 100LL * n;
  std::vector<T> hsh(4 * kMaxBulges);
  while (ihi >= 1) {
    // bottom unreduced block
    int kmax = 0;
    if (ihi > 1) {
      CKL(cudaMemsetAsync(dscan, 0, sizeof(int), s));
      CKL(launch_deflation_scan<T>(H, n, 1, ihi, dscan, s));
      CKL(cudaMemcpyAsync(&kmax, dscan, sizeof(int), cudaMemcpyDeviceToHost, s));
      CKL(cudaStreamSynchronize(s));
    }
    const int ilo = kmax > 0 ? kmax : 1;
    if (kmax > 0) CKL(cudaMemsetAsync(H + (size_t)(ilo - 2) * n + (ilo - 1), 0, sizeof(T), s));
    int m = ihi - ilo + 1;
    if (m <= NMIN) {
      // finish the block with the small-matrix kernel; eigenvalues straight into wr/wi
      if (small_solve(ilo, ihi, true, r.wr + (ilo - 1), r.wi + (ilo - 1), false)) return -1;
      CKL(copy2d<T, T>(m, m, blk, m, H + (size_t)(ilo - 1) * n + (ilo - 1), n, s));
      if (apply_U(ilo, ihi)) return -1;
      int st = 0;
      CKL(cudaMemcpyAsync(&st, bstat, sizeof(int), cudaMemcpyDeviceToHost, s));
      CKL(cudaStreamSynchronize(s));
      if (st != ST_OK) return ST_UNCONVERGED;
      ihi = ilo - 1;
      since_defl = 0;
      continue;
    }
    if (++sweeps > max_sweeps) return ST_UNCONVERGED;
    int B = std::min(r.bulges > 0 ? r.bulges : kMaxBulges, std::max(1, (m - 8) / 6));
    std::vector<double> aed_wr, aed_wi;  // shift candidates from the deflation window
    if (r.aedw > 0) {
      // aggressive early deflation on the trailing window (aed.cu)
      const int nw = std::min(r.aedw, m - 1);
      const int kwtop = ihi - nw + 1;
      if (small_solve(kwtop, ihi, true, aewr, aewi, false)) return -1;
      AedArgs<T> ag{};
      ag.H = H; ag.n = n; ag.ilo = ilo; ag.kwtop = kwtop; ag.nw = nw;
      ag.Tw = blk; ag.V = U; ag.win_status = bstat;
      ag.ewr = aewr; ag.ewi = aewi; ag.wr = r.wr; ag.wi = r.wi; ag.out = aout;
      CKL(launch_aed<T>(ag, s));
      int ao[3] = {0, 0, 0};
      std::vector<double> ewr_w(nw), ewi_w(nw);
      CKL(cudaMemcpyAsync(ao, aout, sizeof(ao), cudaMemcpyDeviceToHost, s));
      CKL(cudaMemcpyAsync(ewr_w.data(), aewr, sizeof(double) * nw, cudaMemcpyDeviceToHost, s));
      CKL(cudaMemcpyAsync(ewi_w.data(), aewi, sizeof(double) * nw, cudaMemcpyDeviceToHost, s));
      CKL(cudaStreamSynchronize(s));
      const int nsu = ao[0], nd = ao[1];
      if (ao[2]) {
        if (apply_U(kwtop, ihi)) return -1;
      }
      if (nd > 0) {
        ihi = kwtop + nsu - 1;
        since_defl = 0;
        // deflated enough (LAPACK's nibble of 14%), or too little left for a sweep: AED again
        if (nd * 100 >= 14 * nw || nsu < 2 || ihi - ilo + 1 <= NMIN) continue;
      }
      // candidate shifts: whole blocks from the bottom of the undeflated part
      for (int q = nsu - 1; q >= 0 && (int)aed_wr.size() < 2 * B;) {
        const int bs = (ewi_w[q] < 0.0 && q > 0) ? 2 : 1;
        for (int t = q - bs + 1; t <= q; ++t) { aed_wr.push_back(ewr_w[t]); aed_wi.push_back(ewi_w[t]); }
        q -= bs;
      }
      m = ihi - ilo + 1;
      B = std::min(B, std::max(1, (m - 8) / 6));
      if ((int)aed_wr.size() >= 2) B = std::min(B, (int)aed_wr.size() / 2);
    }
    const int ns = 2 * B;
    std::vector<double> ewr(ns), ewi(ns);
    ++since_defl;
    if (since_defl % 6 == 0) {
      // exceptional shifts (GenericSchur.jl:614-627 pattern) from the bottom entries
      std::vector<T> hd(3 * ns + 3);
      for (int b = 0; b < B; ++b) {
        const int k = ihi - 2 * b;
        T hkk, s1, s2;
        CKL(cudaMemcpyAsync(&hkk, H + (size_t)(k - 1) * n + (k - 1), sizeof(T), cudaMemcpyDeviceToHost, s));
        CKL(cudaMemcpyAsync(&s1, H + (size_t)(k - 2) * n + (k - 1), sizeof(T), cudaMemcpyDeviceToHost, s));
        CKL(cudaMemcpyAsync(&s2, H + (size_t)(k - 3) * n + (k - 2), sizeof(T), cudaMemcpyDeviceToHost, s));
        CKL(cudaStreamSynchronize(s));
        const double sv = std::fabs((double)s1) + std::fabs((double)s2);
        const double h11 = 0.75 * sv + (double)hkk;
        // eigenvalues of [h11, -7/16 sv; sv, h11]: h11 +- i sv sqrt(7/16)
        ewr[2 * b] = h11; ewi[2 * b] = sv * std::sqrt(7.0 / 16.0);
        ewr[2 * b + 1] = h11; ewi[2 * b + 1] = -ewi[2 * b];
      }
    } else if ((int)aed_wr.size() >= 2) {
      // the undeflated window eigenvalues (bottom-most first); fewer than 2B shorten the chain
      ewr.assign(aed_wr.begin(), aed_wr.end());
      ewi.assign(aed_wi.begin(), aed_wi.end());
    } else {
      if (small_solve(ihi - ns + 1, ihi, false, bwr, bwi, r.shift_fp32 != 0)) return -1;
      CKL(cudaMemcpyAsync(ewr.data(), bwr, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
      CKL(cudaMemcpyAsync(ewi.data(), bwi, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
      CKL(cudaStreamSynchronize(s));
    }
    // pair the shifts: conjugate pairs stay together, real shifts are paired in order
    std::vector<std::complex<double>> cpx, rl;
    const int nc = (int)ewr.size();
    for (int q = 0; q < nc; ++q) {
      if (ewi[q] > 0.0 && q + 1 < nc) { cpx.push_back({ewr[q], ewi[q]}); cpx.push_back({ewr[q + 1], ewi[q + 1]}); ++q; }
      else if (ewi[q] == 0.0) rl.push_back({ewr[q], 0.0});
    }
    std::vector<std::complex<double>> sh(cpx);
    for (auto& x : rl) sh.push_back(x);
    while ((int)sh.size() < ns) sh.push_back(sh.empty() ? std::complex<double>(0.0, 0.0) : sh.back());
    for (int b = 0; b < B; ++b) {
      hsh[4 * b + 0] = (T)sh[2 * b].real();
      hsh[4 * b + 1] = (T)sh[2 * b].imag();
      hsh[4 * b + 2] = (T)sh[2 * b + 1].real();
      hsh[4 * b + 3] = (T)sh[2 * b + 1].imag();
    }
    CKL(cudaMemcpyAsync(dshift, hsh.data(), sizeof(T) * 4 * B, cudaMemcpyHostToDevice, s));
    // chase the chain through [ilo, ihi] in chunks
    const int steps = (ihi - 1 - ilo) + 3 * (B - 1) + 1;
    const int w = r.chunk > 0 ? std::min(r.chunk, 64) : 32;
    for (int t0 = 0; t0 < steps; t0 += w) {
      const int wc = std::min(w, steps - t0);
      const int kmin = std::max(ilo, ilo + t0 - 3 * (B - 1));
      const int kmx = std::min(ihi - 1, ilo + t0 + wc - 1);
      ChaseArgs<T> ca{};
      ca.H = H;
      ca.Z = Z;
      ca.n = n;
      ca.ilo = ilo;
      ca.ihi = ihi;
      ca.B = B;
      ca.t0 = t0;
      ca.w = wc;
      ca.wlo = std::max(ilo, kmin - 1);
      ca.whi = std::min(ihi, kmx + 3);
      ca.shifts = dshift;
      ca.logk = logk;
      ca.logr = logr;
      CKL(launch_chase_chunk<T>(ca, r.num_sms, s));
    }
  }

  // ---- 4. unscale T and the eigenvalues
  k_triu1<T><<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(H, n);
  CKL(cudaGetLastError());
  if (scaled) {
    for (double m : safescale_factors_host(cscale, amax)) {
      k_scale<T><<<4 * r.num_sms, 256, 0, s>>>(H, nn, m);
      k_scale<double><<<1, 256, 0, s>>>(r.wr, n, m);
      k_scale<double><<<1, 256, 0, s>>>(r.wi, n, m);
    }
  }
  CKL(cudaGetLastError());
  return ST_OK;
#undef CKL
}

template int schur_large_run<double>(LargeRun<double>&);
template int schur_large_run<float>(LargeRun<float>&);

}  // namespace gsk
