// Internal declarations shared by the kernel translation units and the C-ABI.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

namespace gsk {

// Largest matrix order handled by the one-CTA-per-matrix kernels.
constexpr int kSmallMax = 128;

// Per-matrix status codes (also the C-ABI return codes).
enum : int { ST_OK = 0, ST_UNCONVERGED = 1, ST_BADARG = 2, ST_CUDA = 3 };
// Internal per-matrix status of the mixed batched form: the refinement handed the matrix
// back to the FP64 kernel (which overwrites it with ST_OK / ST_UNCONVERGED).
constexpr int kStFallback = 7;

// A ragged batch of column-major matrices in one packed buffer.  Matrix b has
// order ns[b] and starts at element offs[b] of A and Z; its eigenvalues start at
// woffs[b].  All pointers are device pointers.
template <class T, class W = double>
struct RealBatchT {
  int count;
  const int* ns;
  const long long* offs;
  const long long* woffs;
  T* A;            // in: A; out: T (quasi-triangular, standard form)
  T* Z;            // out: Schur vectors (ignored when wantz == 0)
  W* wr;           // out: real parts of the eigenvalues
  W* wi;           // out: imaginary parts
  int* status;     // out: ST_OK / ST_UNCONVERGED per matrix
  int wantz;
  int scale;
  int maxiter_mult;  // maxiter = maxiter_mult * n (reference default 100)
  long long maxiter_abs;  // when > 0, overrides maxiter_mult
};
using RealBatch = RealBatchT<double>;

struct CplxBatch {
  int count;
  const int* ns;
  const long long* offs;
  const long long* woffs;
  double2* A;      // in: A; out: T (upper triangular)
  double2* Z;
  double2* w;
  int* status;
  int wantz;
  int scale;
  int maxiter_mult;  // maxiter = maxiter_mult * n (reference default 100)
  int maxinner_mult; // maxinner = maxinner_mult * n (reference default 30)
  long long maxiter_abs;   // when > 0, overrides maxiter_mult
  long long maxinner_abs;  // when > 0, overrides maxinner_mult
};
// One complex matrix of order n > 128 on the whole GPU (schur_large_cplx.cu): Hessenberg
// reduction, multishift QR, blocks <= 128 by the batched kernel.  A (device, ld n) <- T,
// Z (or null) <- the unitary factor, w <- diag(T).  Returns ST_OK, ST_UNCONVERGED (sweep
// limit maxsweeps, <= 0: 100 n; or a non-finite entry), or -1 with *cerr on a CUDA error.
size_t schur_large_cplx_ws_bytes(int n);
int schur_large_cplx_run(double2* A, double2* Z, double2* w, int n, int scale, long long maxsweeps, void* ws,
                         int num_sms, cudaStream_t s, cudaError_t* cerr);

// Eigenvectors of complex Schur factors (T upper triangular), batched.  Matrix b
// has order ns[b] <= 128 at element offset offs[b] of T, Z, VR, VL and scratch.
constexpr int kEigSmem = 64;  // orders up to this keep the solution block in shared memory
struct EigBatch {
  int count;
  const int* ns;
  const long long* offs;
  const double2* T;
  const double2* Z;   // may be null: eigenvectors of T itself
  double2* VR;        // right eigenvectors (null: skip)
  double2* VL;        // left eigenvectors (null: skip)
  double2* scratch;   // solution blocks of orders > kEigSmem
  int normalize;      // apply _enormalize!
  const long long* woffs;  // per-matrix offset into colmap (with colmap)
  const int* colmap;       // optional: output column of eigenvector ki is colmap[woffs[b] + ki - 1]
};
size_t eigvecs_smem_bytes(int nmax);
// One matrix of any order (eigvecs_large.cu): workspace of eigvecs_large_ws_elems(n)
// complex elements; cmap (optional) scatters eigenvector ki to column cmap[ki]; bad[0]
// counts columns that overflowed.
size_t eigvecs_large_ws_elems(int n);
cudaError_t launch_eigvecs_large(int n, const double2* T, const double2* Z, double2* VR, double2* VL, int normalize,
                                 const int* cmap, double2* ws, int* bad, cudaStream_t s);
cudaError_t launch_enormalize(int n, int m, double2* V, int normalize, int* bad, cudaStream_t s);

// Balancing (balance.cu).
template <class S>
cudaError_t launch_bal_mark(const S* A, int lda, int lo, int hi, int rows, int* flag, int num_sms, cudaStream_t s);
cudaError_t launch_bal_pick(const int* flag, int lo, int hi, int rows, int* out, cudaStream_t s);
template <class S>
cudaError_t launch_bal_swap(S* A, int lda, int n, int p, int q, int rows, int c0, cudaStream_t s);
template <class S>
cudaError_t launch_bal_scale(S* A, int lda, int n, int ilo, int ihi, double* D, int* st, cudaStream_t s);
cudaError_t launch_bal_apply(int n, int m, const double2* V, int ldv, double2* W, const int* src, const double* D,
                             int scale, int inverse, int num_sms, cudaStream_t s);
cudaError_t launch_rconde(int n, int m, const double2* VL, const double2* VR, double* out, cudaStream_t s);

// Condition estimators (condition.cu): triangular Sylvester solves of sylvester.jl and
// the vector steps of norm1est.jl.  S = double or double2.
template <class S>
struct SylvArgs {
  const S* A;     // m x m, upper triangle read (the flipped conjugate transpose for adjoints)
  int lda;
  const S* B;     // p x p, upper triangle read
  int ldb;
  S* C;           // m x p right-hand side, overwritten by the solution
  int ldc;
  int m, p, mT, pT;
  int flip;       // C(i, j) stored at C[(m-1-i) + (p-1-j) ldc] (adjoint solves)
  int le;         // perturb |a11|_1 <= smin (trsylvester!) or < smin (adjtrsylvester!)
  int pos;        // possign: A X + X B = scale C (the B terms' sign is +)
  double smin, bignum;
  int* flag;      // |= 1 perturbed, 2 the overflow rescaling is needed, 4 non-finite entry
};
enum { N1_FILL = 0, N1_UNIT = 1, N1_ALT = 2, N1_SIGN = 3 };
// Generalized Schur of complex pencils (qz.cu): one CTA per pencil of a ragged batch.
struct QzBatch {
  int count;
  const int* ns;
  const long long* offs;   // element (double2) offsets of A, B, Q, Z
  const long long* woffs;  // offsets of alpha, beta
  double2* A;              // in: A, out: S
  double2* B;              // in: B, out: T
  double2* Q;              // out (may be null)
  double2* Z;              // out (may be null)
  double2* alpha;
  double2* beta;
  int* status;             // per pencil: 0, or 1 when the iteration limit was reached
  int scale;
  int n1;                  // ns == null: one pencil of order n1 at offset 0
};
cudaError_t launch_ggschur(const QzBatch& bt, int num_sms, cudaStream_t s);
// gordschur! of a complex generalized Schur form (qz.cu); status 0 or 1 + j1 of a rejected swap.
cudaError_t launch_ggordschur_cplx(int n, double2* S, double2* T, double2* Q, double2* Z, const int* select, int scale,
                                   double2* alpha, double2* beta, int* status, cudaStream_t s);
// Generalized Sylvester solves of complex triangular A, D (m x m), B, E (n x n) on
// C, F (m x n) (gcondition.cu).  mode 0 trsylvester!, 1 adjtrsylvester!, 2 the look-ahead
// of _trgsep.  flag bits: 1 a perturbed pivot, 2 a rescaled right-hand side, 4 a singular
// look-ahead system, 8 a grid barrier that timed out.
struct GsylBar {
  unsigned count, gen;
  int err;
};
struct GsylArgs {
  const double2 *A, *B, *D, *E;
  int lda, ldb, ldd, lde;
  double2 *C, *F;
  int ldc, ldf;
  int m, n, mode;
  int* flag;
  GsylBar* bar;
};
size_t gsyl_bar_bytes();
cudaError_t launch_gsyl(const GsylArgs& P, int num_sms, cudaStream_t s);
// gordschur! of a real generalized Schur pair (qz_real.cu); Q, Z may be NULL; status 0 or
// 1 + k of the block that could not be moved.
cudaError_t launch_ggordschur_real(int n, double* S, double* T, double* Q, double* Z, const int* select, int scale,
                                   double2* alpha, double* beta, int* status, cudaStream_t s);
// Real pencils (qz_real.cu): A, B, Q, Z real; alpha complex, beta real.
struct QzrBatch {
  int count;
  const int* ns;
  const long long* offs;   // element offsets of A, B, Q, Z
  const long long* woffs;  // offsets of alpha, beta
  double* A;               // in: A, out: S (quasi-triangular)
  double* B;               // in: B, out: T
  double* Q;               // out (may be null)
  double* Z;               // out (may be null)
  double2* alpha;
  double* beta;
  int* status;
  int scale;
  int n1;
};
cudaError_t launch_ggschur_real(const QzrBatch& bt, int num_sms, cudaStream_t s);

// Hermitian path (hermitian.cu).  S = double or double2.
struct HeCtlBuf {
  alignas(16) unsigned char bytes[64];
};
template <class S>
cudaError_t launch_he_tridiag(const S* A, long long lda, int n, int upper, S* B, S* W, S* partial, int npart,
                              HeCtlBuf* ctl, S* tau, double* d, double* e, int num_sms, cudaStream_t s);
template <class S>
cudaError_t launch_he_formq(const S* B, int n, const S* tau, S* Q, int num_sms, cudaStream_t s);
template <class S>
cudaError_t launch_he_store(const S* B, int n, int upper, S* A, long long lda, cudaStream_t s);
template <class S>
cudaError_t launch_he_gather(const S* Z, int n, const int* p, int rev, S* V, long long ldv, cudaStream_t s);
size_t steqr_ctl_bytes();
// Tridiagonal QR with the rotations applied to Z (nz rows, ld ldz) when Z != NULL.  ctl:
// steqr_ctl_bytes(); rot: 4 n doubles.  ctl holds {count, gen, err, done, status, ...}:
// err != 0 (a barrier wait gave up) at byte 8, status (sweep limit) at byte 16.
template <class S>
cudaError_t launch_steqr(int n, double* d, double* e, S* Z, long long ldz, int nz, double* rot, void* ctl,
                         long long maxsweeps, int num_sms, cudaStream_t s);
// The QR iteration on nprob independent small tridiagonals (problem b: entries off[b] ..
// off[b] + msz[b] - 1 of d and e, msz[b] <= maxm <= 64), one warp each; with wantq the
// problem's diagonal block of Q (ld ldq) is set to the identity and receives the rotations.
// status |= 2 when a problem hit its iteration limit (30 msz).
cudaError_t launch_steqr_leaves(int nprob, const int* off, const int* msz, int maxm, double* d, double* e, double* Q,
                                long long ldq, int wantq, int* status, cudaStream_t s);
// _gschur!(SymTridiagonal(d, e), DivideAndConquer(), Z) (symtri_dc.jl:6-104) on device
// d (n), e (n - 1), Z (n x n, ld ldz; interleaved complex when zcplx; or NULL): d receives
// the eigenvalues in the algorithm's order and Z is multiplied from the right by the
// eigenvectors.  ws: stedc_ws_bytes(n, zcplx) bytes.  *status: 0, 1 (a secular equation did
// not converge), 2 (a QR leaf hit its iteration limit), 4 (a wait in the tensor-core GEMM
// timed out).  Synchronises the stream.
size_t stedc_ws_bytes(int n, int zcplx);
cudaError_t run_stedc(int n, double* d, double* e, double* Z, long long ldz, int zcplx, char* ws, int num_sms,
                      cudaStream_t s, int* status);

template <class S>
cudaError_t launch_cond_maxabs(const S* M, int ld, int rows, int cols, unsigned long long* out, int nsm, cudaStream_t s);
template <class S>
cudaError_t launch_adj_copy(const S* M, int ld, int m, S* Ap, int nsm, cudaStream_t s);
template <class S>
cudaError_t launch_trsyl_levels(const SylvArgs<S>& P, cudaStream_t s);
template <class S>
cudaError_t launch_trsyl_exact(const SylvArgs<S>& P, double* out, cudaStream_t s);
template <class S>
cudaError_t launch_n1_step(int op, S* x, long long N, double arg, int nsm, cudaStream_t s);
template <class S>
cudaError_t launch_n1_stats(const S* x, long long N, long long jlast, double* out, cudaStream_t s);
template <class S>
cudaError_t launch_cond_fro(const S* x, long long N, double* out, cudaStream_t s);
cudaError_t launch_eigvecs_batched(const EigBatch& eb, int nmax, int num_sms, cudaStream_t s);

// Real quasi-triangular -> complex triangular Schur pairs (triang.jl:9-43).
struct TriBatch {
  int count;
  const int* ns;
  const long long* offs;   // element offsets of T/Z (real and complex buffers alike)
  const long long* woffs;  // offsets of w / colmap
  const double* Tr;
  const double* Zr;        // may be null (identity)
  double2* Tc;
  double2* Zc;             // may be null
  double2* w;              // may be null
  int* colmap;             // may be null
};
cudaError_t launch_triangularize(const TriBatch& tb, int num_sms, cudaStream_t s);

// Eigenvalue adjoint: grad = Y diag(gbar / conj(diag(Y^H X))) X^H per matrix.
struct AdjBatch {
  int count;
  const int* ns;
  const long long* offs;   // offsets of VR, VL, grad (complex elements)
  const long long* woffs;  // offsets of gbar
  const double2* VR;
  const double2* VL;
  const double2* gbar;
  double2* grad;
};
cudaError_t launch_eig_adjoint(const AdjBatch& ab, int nmax, int num_sms, cudaStream_t s);

// Large-matrix path (n > kSmallMax).
constexpr int kMaxBulges = 32;  // bulges per multishift chain (one lane each)
constexpr int kFarTile = 32;    // rows/columns per CTA of the far-update kernel
template <class T>
struct ChaseArgs {
  T* H;          // n x n, leading dimension n
  T* Z;          // may be null
  int n;
  int ilo, ihi;  // active block (1-based)
  int B;         // bulges in the chain
  int t0, w;     // first sweep step of this chunk and number of steps
  int wlo, whi;  // window (1-based, inclusive)
  const T* shifts;  // 4 per bulge: r1r, r1i, r2r, r2i
  int* logk;     // w*B positions (0 = inactive)
  T* logr;       // w*B*5 reflector scalars (t1, t1*v2, t1*v3, v2, v3)
};
template <class T> cudaError_t launch_chase_chunk(const ChaseArgs<T>& ca, int num_sms, cudaStream_t s);
template <class T> cudaError_t launch_deflation_scan(const T* H, int n, int ilo, int ihi, int* out, cudaStream_t s);
template <class T>
cudaError_t launch_gemm(int m, int p, int q, const T* A, int lda, int transA, const T* B, int ldb, T* C, int ldc,
                        cudaStream_t s);
size_t hess_large_ws_elems(int n);
template <class T> cudaError_t hessenberg_large(int n, T* A, int lda, T* Z, int ldz, T* tau_out, T* ws, cudaStream_t s);
// Blocked (compact-WY panel) Hessenberg reduction (hessenberg_blocked.cu): the same
// outputs as hessenberg_large; ws of hess_blocked_ws_elems(n) elements; *err_host (when
// not null; the call then synchronises) is nonzero if a grid barrier timed out.
size_t hess_blocked_ws_elems(int n);
template <class T>
cudaError_t hessenberg_blocked(int n, T* A, int lda, T* Z, int ldz, T* tau_out, T* ws, int num_sms, int* err_host,
                               cudaStream_t s);
// Orders from which the blocked reduction is used for element size tsize
// (GS_HESS_BLOCKED_MIN overrides; default 256 for FP32, unused for FP64).
int hess_blocked_min(size_t tsize);

// Aggressive early deflation on the trailing window of the active block (aed.cu).
template <class T>
struct AedArgs {
  T* H;                   // n x n, ld n
  int n;
  int ilo;                // active block start (1-based)
  int kwtop;              // window start (1-based); the window ends at ihi = kwtop + nw - 1
  int nw;
  const T* Tw;            // real Schur form of the window (nw x nw, ld nw)
  T* V;                   // its Schur vectors; updated in place to the window's final transform
  const int* win_status;  // status of the window's Schur decomposition
  double* ewr;            // eigenvalues of the window's diagonal blocks (nw)
  double* ewi;
  double* wr;             // eigenvalue outputs of the whole matrix (deflated ones written)
  double* wi;
  int* out;               // [undeflated count, deflated count, H modified]
};
template <class T> cudaError_t launch_aed(const AedArgs<T>& g, cudaStream_t s);
// Schur reordering (aed.cu): real standard form (st[0] = 0 or the rejected block) and complex.
cudaError_t launch_ordschur_real(double* T, double* Z, int n, const int* select, double* wr, double* wi, int* st,
                                 cudaStream_t s);
cudaError_t launch_ordschur_cplx(double2* T, double2* Z, int n, const int* select, double2* w, cudaStream_t s);

// One large real Schur decomposition (schur_large_host.cu).
template <class T>
struct LargeRun {
  T* A;            // in: A; out: T (device, n x n, ld n)
  T* Z;            // out: Schur vectors, or null
  double* wr;      // out: eigenvalues (device, n)
  double* wi;
  int n;
  int scale;
  long long maxiter;  // bound on multishift sweeps (<= 0: 100 n)
  void* ws;        // workspace of schur_large_ws_bytes(n, sizeof(T)) bytes
  int num_sms;
  cudaStream_t stream;
  cudaError_t cuda_error;
  int bulges;      // bulges per chain (<= kMaxBulges; 0: default)
  int chunk;       // chase steps per chunk (<= 64; 0: default)
  int shift_fp32;  // compute the sweep shifts with the FP32 small-matrix kernel
  int aedw;        // aggressive-early-deflation window (<= 128; 0: off)
};
size_t schur_large_ws_bytes(int n, size_t tsize);
// Tuning of the large path: GS_LARGE_BULGES / GS_LARGE_CHUNK / GS_LARGE_AEDW environment
// variables (read once per call), else the built-in defaults for element size tsize.
void large_tuning(int n, int* bulges, int* chunk, int* aedw, size_t tsize);
// GS_LARGE_SHIFT32=1: shifts of the FP64 path from the FP32 small-matrix kernel.
int large_shift_fp32();
template <class T> int schur_large_run(LargeRun<T>& r);  // ST_OK, ST_UNCONVERGED, or -1 (cuda_error set)

// Host copy of the safescale! factor sequence (util.jl:41-80, as written there).
inline std::vector<double> safescale_factors_host(double cfrom, double cto) {
  const double smlnum = 2.2250738585072014e-308, bignum = 1.0 / smlnum;
  std::vector<double> f;
  double cfromc = cfrom, ctoc = cto;
  bool done = false;
  while (!done && f.size() < 8) {
    const double cfrom1 = cfromc * smlnum;
    double m;
    if (cfrom1 == cfromc) { m = ctoc / cfromc; done = true; }
    else {
      const double cto1 = ctoc / bignum;
      if (cto1 == ctoc) { m = cto; done = true; cfromc = 1.0; }
      else if (std::fabs(cfrom1) > std::fabs(ctoc) && ctoc != 0.0) { m = smlnum; done = false; cfromc = 1.0; }
      else if (std::fabs(cto1) > std::fabs(cfromc)) { m = bignum; done = false; cfromc = cfrom1; }
      else { m = ctoc / cfromc; done = true; }
    }
    f.push_back(m);
  }
  return f;
}

// FP64 refinement kernels of the mixed-precision form (refine.cu).
// Tiles of the Sylvester solve: fills ts[0..nT], tbk[0..nT] (host arrays of n+1) from the
// scalar-to-block map and returns nT.
int sylv_tiles(int n, const int* blk_host, int* ts, int* tbk);
size_t sylv_part_elems(int nT);  // partial right-hand sides of one level (doubles)
cudaError_t launch_sylv_tiled(int n, int nT, const double* At, double* W, const int* bs, const int* bz,
                              const int* blk, const int* ts, const int* tbk, double* part, double floor,
                              cudaStream_t s);
// Eigenvectors of a complex generalized Schur pair (ggevc.cu): right (left = 0, M = Z)
// or left (left = 1, M = Q) into V (n x n, ld n); M may be null; ws of ggevc_ws_bytes.
size_t ggevc_ws_bytes(int n);
cudaError_t launch_ggevc(int n, const double2* S, const double2* P, const double2* M, int left, double2* V, void* ws,
                         cudaStream_t s);
// Eigenvectors of a real generalized Schur pair (rgevc.cu): complex V (n x n, ld n),
// right (left = 0, M = Z) or left (left = 1, M = Q); M may be null; ws of rgevc_ws_bytes.
size_t rgevc_ws_bytes(int n);
cudaError_t launch_rgevc(int n, const double* S, const double* P, const double* M, int left, double2* V, void* ws,
                         cudaStream_t s);
// FP64 product on the BF16 tensor cores by exact splitting (gemm_f64_tc.cu):
// C (m x p, ldc) = op(A) (m x q) B (q x p), column-major; ws of gemm_tc_ws_bytes bytes.
// The error word (gemm_tc_err_word; the caller zeroes it) becomes nonzero when a launch's
// pipeline waits time out; launches with the same (m, p, q) and ws share it.
size_t gemm_tc_ws_bytes(int m, int p, int q);
cudaError_t launch_gemm_tc(int m, int p, int q, const double* A, int lda, int transA, const double* B, int ldb,
                           double* C, int ldc, void* ws, cudaStream_t s);
int* gemm_tc_err_word(int m, int p, int q, void* ws);
cudaError_t launch_refine_elementwise(int op, int n, const double* a, double* b, double x, cudaStream_t s);
cudaError_t launch_add_f32(double* Z, const float* P, size_t cnt, cudaStream_t s);
cudaError_t launch_add_diff_f32(double* X, const float* P1, const float* P2, size_t cnt, cudaStream_t s);
cudaError_t launch_sub_f32(double* X, const float* P, size_t cnt, cudaStream_t s);
cudaError_t launch_lower_norm(int n, const double* At, const int* blk, double* out, int num_sms, cudaStream_t s);
cudaError_t launch_block_triu(int n, const double* At, const int* blk, double* T, cudaStream_t s);
cudaError_t launch_std_blocks(int n, int N, const int* bs, const int* bz, double* T, double* Z, double* cs_sn,
                              double* wr, double* wi, cudaStream_t s);
template <class S, class D> cudaError_t convert_array(const S* src, D* dst, size_t count, double scale, cudaStream_t s);
cudaError_t launch_absmax(const double* A, size_t cnt, unsigned long long* out, int num_sms, cudaStream_t s);

// Size bins of the persistent batched kernels.  `sched` holds, per bin, the
// [start, end) range of that bin inside the sorted work order and a queue ticket
// counter: sched[3*bin + {0,1,2}].
constexpr int kNumBins = 4;
__host__ __device__ constexpr int bin_max(int bin) { return 32 * (bin + 1); }  // 32, 64, 96, 128 (defaults)

// Launch shape of the persistent batched kernels, per size bin: the largest order of
// the bin (ascending, the last one kSmallMax), threads per CTA, whether the
// Hessenberg phase runs on a full copy of the matrix in shared memory, and a cap on
// resident CTAs per SM (0: as many as fit).  Chosen per GPU by the tuner
// (tune.py) and loaded with gs_set_tuning; the defaults are the hand-picked shapes.
struct BinTuning {
  int bounds[kNumBins];
  int nt[kNumBins];
  int hsmem[kNumBins];
  int ctas[kNumBins];
};
BinTuning default_tuning_real();
BinTuning default_tuning_cplx();
BinTuning default_tuning_mixed32();  // the FP32 stage of the mixed batched form
// Thread counts compiled for the FP64 real and the complex kernels (the tuner's
// candidates); other values are rejected by the table parser.  The FP32 stage of the
// mixed form compiles the same counts but 160.
constexpr int kTuneThreads[] = {64, 96, 128, 160, 192, 256};
// Table kinds: real FP64 kernel, complex kernel, FP32 stage of the mixed real form.
enum : int { kTuneReal = 0, kTuneCplx = 1, kTuneMixed32 = 2 };
// Whether (nt, hsmem) is a compiled shape of that kind whose shared memory fits for
// orders up to nmax.
bool tuning_shape_ok(int kind, int nmax, int nt, int hsmem);
size_t real_bin_smem_bytes(int nmax, int hsmem);
size_t real32_bin_smem_bytes(int nmax, int hsmem);
size_t cplx_bin_smem_bytes(int nmax, int hsmem);
struct BinBounds {
  int b[kNumBins];
};

// Sorting/binning kernel: order[] lists matrix indices grouped by bin, largest
// order first inside a bin; sched[] receives the bin ranges and zeroed counters.
// Without `bounds`, the default bins (bin_max).
cudaError_t launch_bin_sort(const int* ns, int count, int* order, int* sched, cudaStream_t s);
cudaError_t launch_bin_sort(const int* ns, int count, int* order, int* sched, const BinBounds& bounds,
                            cudaStream_t s);
// The same over the matrices whose status equals `code` only (the others are left out).
cudaError_t launch_bin_sort_status(const int* ns, int count, const int* status, int code, int* order, int* sched,
                                   const BinBounds& bounds, cudaStream_t s);

// T = double: the FP64 batched kernel; T = float: the same algorithm in FP32 (the
// Float32 entry points and the FP32 stage of the mixed-precision form).  W is the
// type of the eigenvalue outputs.  Without `tun`, the default shapes; the FP32
// instances always run the default shapes.
template <class T, class W>
cudaError_t launch_schur_batched_real(const RealBatchT<T, W>& bt, const int* order, int* sched,
                                      int num_sms, cudaStream_t* streams, int nstreams);
cudaError_t launch_schur_batched_real_tuned(const RealBatchT<double, double>& bt, const int* order, int* sched,
                                            int num_sms, cudaStream_t* streams, int nstreams, const BinTuning& tun);
cudaError_t launch_schur_batched_real32_tuned(const RealBatchT<float, float>& bt, const int* order, int* sched,
                                              int num_sms, cudaStream_t* streams, int nstreams, const BinTuning& tun);
cudaError_t launch_schur_batched_cplx(const CplxBatch& bt, const int* order, int* sched,
                                      int num_sms, cudaStream_t* streams, int nstreams);
cudaError_t launch_schur_batched_cplx_tuned(const CplxBatch& bt, const int* order, int* sched, int num_sms,
                                            cudaStream_t* streams, int nstreams, const BinTuning& tun);
// One matrix of order m (<= kSmallMax) by one CTA of the default shape of its bin, without
// the bin sort: launch_single_queue fills order/sched for that bin (default_bin_of(m));
// launch_single_meta writes iota[0..kSmallMax] and two zero offsets once, so that a batch
// of one can use ns = iota + m and offs = woffs = zeros with no host copy per call.
int default_bin_of(int m);
cudaError_t launch_single_queue(int bin, int* order, int* sched, cudaStream_t s);
cudaError_t launch_single_meta(int* iota, long long* zeros, cudaStream_t s);
template <class T, class W>
cudaError_t launch_schur_real_one(const RealBatchT<T, W>& bt, int m, const int* order, int* sched, cudaStream_t s);
cudaError_t launch_schur_cplx_one(const CplxBatch& bt, int m, const int* order, int* sched, cudaStream_t s);

// Batched real Schur in mixed precision (refine_batched.cu): FP32 Schur pairs refined to
// FP64 by Newton steps, matrices the refinement cannot finish recomputed by the FP64
// kernel (unless nofallback: then ST_UNCONVERGED).  na / nw: element extents of A and of
// the eigenvalue arrays; order / sched: count and 3 * kNumBins ints.
struct MixedBatch {
  int count;
  const int* ns;
  const long long* offs;
  const long long* woffs;
  double* A;
  double* Z;  // null: no Schur vectors wanted
  double* wr;
  double* wi;
  int* status;
  int* order;
  int* sched;
  void* ws;   // mixed_batched_ws_bytes(na, nw, Z != null): arrays indexed like A and wr
  int* iws;   // mixed_batched_iws_ints(count) ints: per-matrix and schedule scratch
  long long na, nw;
  int scale;
  int nofallback;
  unsigned long long* stats;      // 4 counters the caller zeroed: matrices refined, handed back
                                  // to FP64, Newton steps, FP64-accurate product FLOPs
  int* tc_err;                    // zeroed word, set when a tensor-core wait timed out
  cudaEvent_t ref0, ref1;         // null, or recorded around the refinement kernels
};
size_t mixed_batched_ws_bytes(long long na, long long nw, bool wantz);
constexpr size_t kMixedSchedInts = 64;  // schedules and ticket counters of one run
// per matrix: the scale exponent, the refinement's last step size and the fallback order
inline size_t mixed_batched_iws_ints(long long count) { return 3 * (size_t)count + kMixedSchedInts; }
cudaError_t launch_mixed_batched(const MixedBatch& m, int num_sms, cudaStream_t s, cudaStream_t* aux, int naux,
                                 cudaEvent_t fork, cudaEvent_t* join, const BinTuning& tun64, const BinTuning& tun32);
// Element extents of a device-resident ragged batch: out[0] = max(offs + n^2),
// out[1] = max(woffs + n) (orders clamped to [0, kSmallMax]); out must be zeroed.
cudaError_t launch_batch_extent(const int* ns, const long long* offs, const long long* woffs, int count,
                                unsigned long long* out, cudaStream_t s);

}  // namespace gsk
