/*
 * gschur_gb300 — C-ABI of the GB300 dense Schur engine.
 *
 * Drop-in boundary for GenericSchur.jl's dense non-symmetric path: every entry
 * point below names the reference function it replaces (file:line in the
 * GenericSchur.jl source tree).  Matrices are column-major (Julia layout); complex
 * data is interleaved (re, im) doubles, the memory layout of Julia's ComplexF64.
 * Plain pointers and sizes only; no CUDA or torch types appear in the signatures.
 *
 * Pointers are host pointers unless GS_DEVICE is set in `flags`, in which case
 * they are device pointers on the context's device and the call is asynchronous
 * on the context's stream (results and per-matrix status are ready once the
 * stream reaches that point).  Host-pointer calls are synchronous.
 *
 * Return codes mirror the reference's exceptions:
 *   GS_OK           0  success
 *   GS_UNCONVERGED  1  iteration limit reached   (UnconvergedException, GenericSchur.jl:39-45)
 *   GS_BADARG       2  bad size / pointer        (DimensionMismatch / ArgumentError)
 *   GS_CUDA         3  CUDA error; text from gs_last_error()
 * There is no CPU fallback: without a usable GPU every compute entry returns GS_CUDA.
 */
#ifndef GSCHUR_GB300_H
#define GSCHUR_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GS_API __attribute__((visibility("default")))
#else
#define GS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GS_OK 0
#define GS_UNCONVERGED 1
#define GS_BADARG 2
#define GS_CUDA 3

/* flags */
#define GS_WANTZ 1u   /* accumulate Schur vectors (gschur!(A; wantZ=true), GenericSchur.jl:805-826) */
#define GS_SCALE 2u   /* _scale! before and after (gschur!(A; scale=true), util.jl:14-29)          */
#define GS_DEVICE 4u  /* all array arguments are device pointers; asynchronous                    */
#define GS_GRAPH 8u   /* batched calls: replay a cached CUDA graph of the launch sequence         */
#define GS_RAW 16u    /* eigenvectors: skip _enormalize! (return the max-|re|+|im|-scaled vectors) */
#define GS_NOFALLBACK 32u /* mixed precision: report GS_UNCONVERGED instead of recomputing in FP64   */
#define GS_BAL_PERMUTE 64u /* balancing: search the row/column permutations (with GS_SCALE: scale too) */
#define GS_DC 128u         /* Hermitian eigensolver: DivideAndConquer() instead of QRIteration()       */
#define GS_MIXED 256u      /* batched real FP64: FP32 Schur + FP64 Newton refinement, same accuracy    */

typedef struct gs_context gs_context;

/* Library version (integer, major*10000 + minor*100 + patch). */
GS_API int gs_version(void);

/* Create a context on CUDA device `device` with its own non-blocking stream.
 * No reference counterpart (the reference keeps no state). */
GS_API int gs_create(gs_context** ctx, int device);
GS_API int gs_destroy(gs_context* ctx);

/* Use the caller's CUDA stream (a cudaStream_t passed as void*; NULL restores the
 * context's own stream). */
GS_API int gs_set_stream(gs_context* ctx, void* stream);

/* Text of the last error on this context (empty string if none). */
GS_API const char* gs_last_error(const gs_context* ctx);

/* Device time in milliseconds of the last compute call's kernel sequence
 * (CUDA events on the context stream; host<->device copies excluded). */
GS_API float gs_last_kernel_ms(const gs_context* ctx);

/* Launch shapes of the batched kernels (no reference counterpart: the reference has no
 * batched form).  gs_set_tuning loads a table written by the project's tuner
 * (genericschur.jl_gb300/tune.py) for this context: per size bin of the real FP64, the
 * complex, and the FP32 stage of the mixed real (GS_MIXED) batched Schur kernels, the
 * bin's largest order, threads per CTA, whether the Hessenberg phase runs in shared
 * memory, and a cap on CTAs per SM.  Text lines "kind bin nmax threads hsmem ctas_per_sm"
 * (kind real_f64, complex_f64 or mixed_f32; '#' starts a comment; bins not listed keep
 * their defaults; mixed_f32 bins keep the default bounds 32/64/96/128).  path NULL or ""
 * restores the built-in defaults.  GS_BADARG (message in gs_last_error) for an unreadable
 * file, a shape that is not compiled or does not fit in shared memory, or bounds that do
 * not increase to 128; the context keeps its previous shapes then.  Results do not depend
 * on the shapes beyond rounding.  gs_get_tuning writes the active table (same format)
 * into buf. */
GS_API int gs_set_tuning(gs_context* ctx, const char* path);
GS_API int gs_get_tuning(const gs_context* ctx, char* buf, size_t len);

/* Pinned host memory for fast host<->device staging. */
GS_API int gs_host_alloc(gs_context* ctx, void** ptr, size_t bytes);
GS_API int gs_host_free(gs_context* ctx, void* ptr);

/* ---------------------------------------------------------------------------
 * Real Schur decomposition of one n x n matrix.
 * Replaces gschur!(A::StridedMatrix{<:AbstractFloat}; wantZ, scale, maxiter)
 * (GenericSchur.jl:805-835, driving _hessenberg! hessenberg.jl:3-17,
 * _materializeQ hessenberg.jl:150-166 and gschur!(H::Hessenberg, Z)
 * GenericSchur.jl:513-699).
 *   A   [in/out] n x n, leading dimension lda; overwritten by T (upper
 *       quasi-triangular, 2x2 blocks in standard form, zeros below the first
 *       subdiagonal), as the reference returns S.T.
 *   Z   [out] n x n orthogonal Schur vectors, leading dimension ldz (GS_WANTZ).
 *   wr, wi [out] eigenvalues, in the reference's order (S.values).
 *   maxiter: iteration limit; <= 0 selects the reference default 100*n.
 * ------------------------------------------------------------------------- */
GS_API int gs_schur_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, double* Z, int64_t ldz,
                 double* wr, double* wi, unsigned flags, int64_t maxiter);

/* Float32 real Schur decomposition: gschur!(A::StridedMatrix{Float32}) computed in
 * FP32 throughout (the reference's generic code in Float32 arithmetic); same layout
 * and semantics as gs_schur_f64 with float arrays. */
GS_API int gs_schur_f32(gs_context* ctx, int64_t n, float* A, int64_t lda, float* Z, int64_t ldz,
                        float* wr, float* wi, unsigned flags, int64_t maxiter);

/* Complex Schur decomposition of one n x n ComplexF64 matrix.
 * Replaces gschur!(A::StridedMatrix{Complex}) (GenericSchur.jl:350-372) with
 * gschur!(H::Hessenberg{Complex}, Z) (GenericSchur.jl:194-335).
 *   A [in/out] interleaved complex, overwritten by upper-triangular T.
 *   w [out] n eigenvalues (interleaved complex) = diag(T).
 *   maxiter / maxinner <= 0 select the reference defaults 100*n / 30*n. */
GS_API int gs_schur_c64(gs_context* ctx, int64_t n, double* A, int64_t lda, double* Z, int64_t ldz,
                 double* w, unsigned flags, int64_t maxiter, int64_t maxinner);

/* ---------------------------------------------------------------------------
 * Batched forms (no reference counterpart: the reference handles one matrix per
 * call; these run gschur! on every matrix of a ragged batch in one persistent
 * launch sequence).  Matrix b has order ns[b] <= 128 and is stored column-major
 * with leading dimension ns[b] at element offset offs[b] of A and Z; its
 * eigenvalues start at element woffs[b] of wr/wi (or of w, complex).  status[b]
 * receives GS_OK or GS_UNCONVERGED.  Returns GS_UNCONVERGED if any matrix failed
 * (host-pointer mode) — the other matrices are still valid.  Host-pointer calls check
 * every order and offset before launching (GS_BADARG).  With GS_DEVICE the orders are
 * read on the device only: a matrix whose order lies outside [0, 128] is left untouched
 * and gets status[b] = GS_BADARG; offsets are the caller's responsibility. 
 * ------------------------------------------------------------------------- */
GS_API int gs_schur_batched_f64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                         const int64_t* woffs, double* A, double* Z, double* wr, double* wi,
                         int32_t* status, unsigned flags);

/* After a GS_MIXED batched call (GS_MIXED: FP32 Schur pairs refined to FP64 accuracy by
 * per-matrix Newton steps; matrices the refinement cannot finish are recomputed in FP64,
 * or with GS_NOFALLBACK reported GS_UNCONVERGED), info[0..5]: info[0] matrices finished by
 * the refinement, info[1] matrices handed back to the FP64 kernel (or reported), info[2]
 * Newton steps taken, info[3] FLOPs of the refinement's FP64-accurate products (per step
 * 2 n^3 each for A Z, Z^T (A Z) and Z^T Z, run on the tensor cores), info[4] device time
 * of the refinement in microseconds, info[5] device time of the FP32 stage (conversion,
 * FP32 Schur) in microseconds (both -1 if not timed).  Synchronises
 * the context stream.  GS_BADARG before the first GS_MIXED call; GS_CUDA (counters
 * filled) when a tensor-core wait timed out and its matrix was handed back. */
GS_API int gs_mixed_batched_info(gs_context* ctx, int64_t* info);

GS_API int gs_schur_batched_f32(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                                const int64_t* woffs, float* A, float* Z, float* wr, float* wi,
                                int32_t* status, unsigned flags);

GS_API int gs_schur_batched_c64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                         const int64_t* woffs, double* A, double* Z, double* w, int32_t* status,
                         unsigned flags);

/* ---------------------------------------------------------------------------
 * Eigenvectors from Schur factors.  V columns are ordered like S.values; each has
 * unit 2-norm with its largest-modulus entry real (_enormalize!, util.jl:572-592)
 * unless GS_RAW.  VR / VL may be NULL to skip right / left vectors; Z may be NULL
 * for eigenvectors of T itself.  Orders n <= 128.
 * ------------------------------------------------------------------------- */

/* Complex Schur pair (T upper triangular).  Replaces eigvecs(S::Schur{Complex}; left)
 * (pirates.jl:38-48) = geigvecs (vectors.jl:12-20) with _geigvecs! (vectors.jl:45-131,
 * _usolve! util.jl:128-293) and _gleigvecs! (vectors.jl:372-460, _cusolve! util.jl:301-461).
 * T, Z: n x n interleaved complex, leading dimension n; VR, VL: n x n complex. */
GS_API int gs_eigvecs_c64(gs_context* ctx, int64_t n, const double* T, const double* Z, double* VR, double* VL,
                          unsigned flags);

/* Real standard-form Schur pair; complex eigenvectors.  Replaces geigvecs(S::Schur{<:Real};
 * left) (vectors.jl:12-20 with _geigvecs! 133-362 / _gleigvecs! 462-698).  Computed as
 * triangularize + the complex back-substitution (identical vectors after normalisation). */
GS_API int gs_eigvecs_f64(gs_context* ctx, int64_t n, const double* T, const double* Z, double* VR, double* VL,
                          unsigned flags);

/* Real quasi-triangular Schur pair -> complex triangular Schur pair (triangularize,
 * triang.jl:9-43).  T, Z real n x n (Z may be NULL: identity); Tc, Zc complex n x n
 * (Zc may be NULL); w complex n = diag(Tc) (may be NULL).  Any n. */
GS_API int gs_triangularize_f64(gs_context* ctx, int64_t n, const double* T, const double* Z, double* Tc, double* Zc,
                                double* w, unsigned flags);

/* Batched eigenvectors (no reference counterpart).  Matrix b of order ns[b] <= 128 at
 * element offset offs[b] of T, Z, VR, VL (complex elements for complex buffers);
 * packed_len = total elements per buffer.  The real form also takes woffs (offsets
 * of each matrix's eigenvalues, as in gs_schur_batched_f64) and w_len = their total. */
GS_API int gs_eigvecs_batched_c64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                                  int64_t packed_len, const double* T, const double* Z, double* VR, double* VL,
                                  unsigned flags);
GS_API int gs_eigvecs_batched_f64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                                  const int64_t* woffs, int64_t packed_len, int64_t w_len, const double* T,
                                  const double* Z, double* VR, double* VL, unsigned flags);

/* ---------------------------------------------------------------------------
 * Eigenvalue adjoint (no reference counterpart; the reverse-mode rule of
 * A -> eigenvalues(A) built on the reference's eigenvector definitions).
 * Given complex Schur pairs (T, Z) of a batch of matrices A_b and cotangents
 * gbar_i = dL/dRe(l_i) + i dL/dIm(l_i) for their eigenvalues (in the order of
 * S.values = diag(T)), returns grad_b = dL/dRe(A_b) + i dL/dIm(A_b)
 *   = sum_i gbar_i y_i x_i^H / conj(y_i^H x_i),
 * with x_i, y_i the right / left eigenvectors recomputed on the device from (T, Z)
 * (_geigvecs!, vectors.jl:45-131; _gleigvecs!, vectors.jl:372-460).  Layout as in
 * gs_eigvecs_batched_c64; gbar and the eigenvalues use woffs / w_len. */
GS_API int gs_eig_adjoint_batched_c64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                                      const int64_t* woffs, int64_t packed_len, int64_t w_len, const double* T,
                                      const double* Z, const double* gbar, double* grad, unsigned flags);

/* Mixed-precision real Schur (no reference counterpart; same outputs as
 * gs_schur_f64).  The decomposition runs in FP32 on the GPU (Hessenberg reduction
 * and multishift QR), then FP64 Newton refinement of the Schur pair restores FP64
 * accuracy: Z is re-orthonormalised (Newton-Schulz), Z^T A Z is formed in FP64 and
 * its block-lower part removed by solving the block triangular Sylvester equation
 * of the Newton step; the 1x1/2x2 block structure is the FP32 form's, and the 2x2
 * blocks are finally put in standard form with _gs2x2! (GenericSchur.jl:716-803).
 * Z is required.  info (may be NULL) receives 4 doubles: refinement iterations,
 * final ||blocklower(Z^T A Z)||_F / ||A||_F, FP32-stage ms, refinement ms.
 * When the refinement cannot reach FP64 accuracy (eigenvalues that FP32 does not
 * separate, e.g. tight clusters relative to ||A||), the decomposition is recomputed
 * by gs_schur_f64 from the untouched input and info[0] = -1; with GS_NOFALLBACK
 * the call returns GS_UNCONVERGED instead. */
GS_API int gs_schur_mixed_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, double* Z, int64_t ldz, double* wr,
                              double* wi, unsigned flags, int64_t maxiter, double* info);

/* Hessenberg reduction with Q.  Replaces hessenberg!(A) (pirates.jl:232 ->
 * _hessenberg!, hessenberg.jl:3-17) and _materializeQ (hessenberg.jl:150-166):
 * A [in/out] is overwritten by H with the reflectors' essential parts below the
 * first subdiagonal (the packed form of the reference's Hessenberg object), tau
 * receives the n-1 reflector scalars, Q (may be NULL) the orthogonal factor with
 * A = Q H Q^T.  Any n. */
GS_API int gs_hessenberg_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, double* tau, double* Q, int64_t ldq,
                             unsigned flags);

/* ---------------------------------------------------------------------------
 * Balancing.  Replaces balance!(A; scale, permute) (balance.jl:33-185): with
 * GS_BAL_PERMUTE, row/column permutations bring A to [T1 X Y; 0 C Z; 0 0 T2] (T1, T2
 * upper triangular, C = A[ilo:ihi, ilo:ihi]); with GS_SCALE, powers of two balance the
 * rows and columns of C (2-norms, the reference's "pr" variant).  A is overwritten
 * by the balanced matrix; info receives {ilo, ihi, trivial}, sp (n) the permutation
 * record (1-based, sp[j-1] for j < ilo and j > ihi), D (n) the scale factors.
 * Returns GS_BADARG on NaN (the reference throws "NaN encountered while balancing").
 * The complex form takes interleaved ComplexF64. */
GS_API int gs_balance_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, unsigned flags, int64_t* info,
                          int64_t* sp, double* D);
GS_API int gs_balance_c64(gs_context* ctx, int64_t n, double* A, int64_t lda, unsigned flags, int64_t* info,
                          int64_t* sp, double* D);

/* The Balancer on eigenvectors: lmul!(B, V) (inverse = 0, right eigenvectors of the
 * balanced matrix -> of A) or ldiv!(B, V) (inverse = 1, left eigenvectors)
 * (balance.jl:189-261).  V: n x m interleaved complex, leading dimension ldv. */
GS_API int gs_balancer_apply_c64(gs_context* ctx, int64_t n, int64_t m, double* V, int64_t ldv, const int64_t* info,
                                 const int64_t* sp, const double* D, int inverse, unsigned flags);

/* Column normalisation of eigenvectors: each column scaled by 1 / max |v|_1, then (unless
 * GS_RAW) _enormalize! (util.jl:572-592): unit 2-norm, largest-modulus entry real. */
GS_API int gs_enormalize_c64(gs_context* ctx, int64_t n, int64_t m, double* V, int64_t ldv, unsigned flags);

/* Reciprocal eigenvalue condition numbers from left/right eigenvector matrices
 * (eigen!(A; jce = true), pirates.jl:107-113): rconde[j] = |vl_j^H vr_j| /
 * (|vl_j|_2 |vr_j|_2).  VL, VR: n x n interleaved complex, ld n. */
GS_API int gs_rconde_c64(gs_context* ctx, int64_t n, const double* VL, const double* VR, double* rconde, unsigned flags);

/* eigvalscond(S, nsub) (ordschur.jl:84-105): reciprocal condition number of the leading
 * nsub eigenvalues of the Schur factor T (n x n, leading dimension ldt; only the upper
 * triangle of each diagonal block is read, as the reference's trsylvester! reads it).
 * The result goes to the host scalar *s (with GS_DEVICE only T is a device pointer).
 * nsub = 0 or n gives 1. */
GS_API int gs_eigvalscond_f64(gs_context* ctx, int64_t n, const double* T, int64_t ldt, int64_t nsub, double* s,
                              unsigned flags);
GS_API int gs_eigvalscond_c64(gs_context* ctx, int64_t n, const double* T, int64_t ldt, int64_t nsub, double* s,
                              unsigned flags);
/* subspacesep(S, nsub) (ordschur.jl:107-140): estimated separation of the leading nsub
 * block from the rest (norm1est! over trsylvester! / adjtrsylvester!, norm1est.jl:21-74).
 * 0 < nsub < n (GS_BADARG otherwise: the reference fails on an empty block). */
GS_API int gs_subspacesep_f64(gs_context* ctx, int64_t n, const double* T, int64_t ldt, int64_t nsub, double* sep,
                              unsigned flags);
GS_API int gs_subspacesep_c64(gs_context* ctx, int64_t n, const double* T, int64_t ldt, int64_t nsub, double* sep,
                              unsigned flags);
/* trsylvester!(A, B, C; possign) (adjoint = 0) / adjtrsylvester!(A, B, C; possign)
 * (adjoint = 1) (sylvester.jl:11-139): A X - X B = scale C, resp. A^H X - X B^H = scale C,
 * with + for the B terms when possign; A (m x m) and B (n x n) upper triangular (only their
 * upper triangles are read), C (m x n) overwritten with X; *scale the reference's scale
 * (below one only when the solution would overflow), *perturbed whether a diagonal
 * difference was raised to smin.  _c64: interleaved complex. */
GS_API int gs_trsylvester_f64(gs_context* ctx, int64_t m, int64_t n, const double* A, int64_t lda, const double* B,
                              int64_t ldb, double* C, int64_t ldc, int32_t adjoint, int32_t possign, double* scale,
                              int32_t* perturbed, unsigned flags);
GS_API int gs_trsylvester_c64(gs_context* ctx, int64_t m, int64_t n, const double* A, int64_t lda, const double* B,
                              int64_t ldb, double* C, int64_t ldc, int32_t adjoint, int32_t possign, double* scale,
                              int32_t* perturbed, unsigned flags);
/* Generalized Sylvester equations of complex upper triangular A, D (m x m) and B, E
 * (n x n), interleaved complex, C and F m x n overwritten with R and L:
 *   adjoint = 0: trsylvester!(A, B, C, D, E, F) (gsylvester.jl:23-99)
 *                A R - L B = scale C,  D R - L E = scale F
 *   adjoint = 1: adjtrsylvester!(A, B, C, D, E, F) (gsylvester.jl:103-155)
 *                A^H R + D^H L = scale C,  R B^H + L E^H = -scale F
 * Only the upper triangles of A, B, D, E are read.  *scale is 1 on success; *perturbed is 1
 * when a 2 x 2 pivot was raised to smin (the reference's fourth return value).  Where a
 * 2 x 2 solve would need rescaling against overflow the call fails with GS_BADARG (the
 * reference's rescaling branch raises there).  With GS_DEVICE all arrays are device
 * pointers. */
GS_API int gs_gtrsylvester_c64(gs_context* ctx, int64_t m, int64_t n, const double* A, int64_t lda, const double* B,
                               int64_t ldb, double* C, int64_t ldc, const double* D, int64_t ldd, const double* E,
                               int64_t lde, double* F, int64_t ldf, int32_t adjoint, double* scale,
                               int32_t* perturbed, unsigned flags);
/* eigvalscond(S::GeneralizedSchur, nsub) (gcondition.jl:121-165) of a complex generalized
 * Schur pair (S, T), n x n: plpr[0] = pl, plpr[1] = pr, the reciprocal norms of the left
 * and right projectors onto the deflating subspaces of the leading nsub block. */
GS_API int gs_geigvalscond_c64(gs_context* ctx, int64_t n, const double* S, int64_t lds, const double* T,
                               int64_t ldt, int64_t nsub, double* plpr, unsigned flags);
/* subspacesep(S::GeneralizedSchur, nsub; pnorm) (gcondition.jl:169-260): sep[0], sep[1]
 * the estimated separations (Difu, Difl) of the leading nsub block from the rest.
 * pnorm = 0 (:Frobenius, the default there): the look-ahead estimate of _trgsep
 * (gcondition.jl:8-115); pnorm = 1: the one-norm estimate of norm1est! over the generalized
 * Sylvester operator and its adjoint, applied in place (0 < nsub < n). */
GS_API int gs_gsubspacesep_c64(gs_context* ctx, int64_t n, const double* S, int64_t lds, const double* T,
                               int64_t ldt, int64_t nsub, int32_t pnorm, double* sep, unsigned flags);
/* eigen!(A; jcv = true) (pirates.jl:136-153) on a Schur factor T (n x n, ld n): for each
 * j, eigenvalue j moved to the front of a copy of T by ordschur!, then rconde[j] =
 * eigvalscond(., 1) (skipped when rconde is NULL) and rcondv[j] = subspacesep(., 1)
 * (skipped when rcondv is NULL).  With GS_DEVICE, T, rconde and rcondv are device
 * pointers.  O(n^3) work, as the reference warns. */
GS_API int gs_eigen_rcond_f64(gs_context* ctx, int64_t n, const double* T, double* rconde, double* rcondv,
                              unsigned flags);
GS_API int gs_eigen_rcond_c64(gs_context* ctx, int64_t n, const double* T, double* rconde, double* rcondv,
                              unsigned flags);

/* geigen!(Hermitian(A, uplo)) / geigvals! (GenericSchur.jl:126-146) with the default
 * QRIteration (with GS_DC: DivideAndConquer(), symtri_dc.jl:6-104, n <= 32768): Householder tridiagonalization (hessenberg.jl:26-96), Q (hessenberg.jl:
 * 145-231) and the tridiagonal QL/QR iteration (symtridiag.jl:79-368).  uplo = 'L' or 'U'
 * names the triangle of A (n x n, lda) that is read; A is not modified.  w (n) receives the
 * eigenvalues in ascending order; with GS_WANTZ, V (n x n, ldv) the orthonormal
 * eigenvectors in the same order.  _c64: A and V interleaved complex, w real. */
GS_API int gs_heev_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* w, double* V,
                       int64_t ldv, unsigned flags);
GS_API int gs_heev_c64(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* w, double* V,
                       int64_t ldv, unsigned flags);
/* hessenberg!(Hermitian(A, uplo)) (hessenberg.jl:26-96): the real symmetric tridiagonal
 * (d: n, e: n-1), the reflector scalars tau (n-1; complex for _c64) and, in A's `uplo`
 * triangle, the subdiagonal (superdiagonal) entries and reflector tails as the reference
 * stores them.  A is overwritten in place. */
GS_API int gs_hetrd_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* d, double* e,
                        double* tau, unsigned flags);
GS_API int gs_hetrd_c64(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* d, double* e,
                        double* tau, unsigned flags);
/* _gschur!(SymTridiagonal(d, e), QRIteration(), Z) (symtridiag.jl:79-183): d (n) receives
 * the eigenvalues in the iteration's order (unsorted), e (n-1) is overwritten; when Z
 * (n x n, ldz) is not NULL every rotation is applied to it from the right.  Used by
 * eigen!/eigvals!(::SymTridiagonal) (symtridiag.jl:43-57), which sort afterwards. */
GS_API int gs_steqr_f64(gs_context* ctx, int64_t n, double* d, double* e, double* Z, int64_t ldz, unsigned flags);
/* _gschur!(SymTridiagonal(d, e), DivideAndConquer(), Z) (symtri_dc.jl:6-104, after LAPACK's
 * xSTEDC): the same contract as gs_steqr_f64 (d receives the eigenvalues in the algorithm's
 * order; Z, when not NULL, is multiplied from the right by the eigenvectors).  n <= 32768.
 * GS_UNCONVERGED when a secular equation fails (the reference's UnconvergedException). */
GS_API int gs_stedc_f64(gs_context* ctx, int64_t n, double* d, double* e, double* Z, int64_t ldz, unsigned flags);

/* ggschur!(A, B; wantQ, wantZ, scale) (generalized.jl:21-80) for a complex pencil: qr!(B),
 * Hessenberg-triangular reduction (_hessenberg!, 82-113) and the single-shift QZ
 * iteration (_gqz!, 125-487).  A <- S, B <- T (both upper triangular, diag(T) real and
 * non-negative), Q and Z (n x n; NULL when not wanted) unitary with A = Q S Z^H and
 * B = Q T Z^H; alpha, beta (n) the generalized eigenvalues alpha ./ beta.  Interleaved
 * complex, leading dimension n.  GS_SCALE applies _scale! to A and B as the reference's
 * default scale = true does.  GS_UNCONVERGED at the reference's 100 n iteration limit. */
GS_API int gs_ggschur_c64(gs_context* ctx, int64_t n, double* A, double* B, double* Q, double* Z, double* alpha,
                          double* beta, unsigned flags);
/* The same over a ragged batch: pencil b has order ns[b] at element offset offs[b] of the
 * packed A, B, Q, Z (packed_len complex elements each) and its alpha, beta at woffs[b]
 * (wlen elements).  One CTA per pencil.  status (count, may be NULL) receives 0 or
 * GS_UNCONVERGED per pencil. */
GS_API int gs_ggschur_batched_c64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                                  int64_t packed_len, double* A, double* B, double* Q, double* Z, const int64_t* woffs,
                                  int64_t wlen, double* alpha, double* beta, int32_t* status, unsigned flags);

/* Eigenvectors of the generalized Schur decomposition of a real pencil (the output of
 * gs_ggschur_f64: S quasi-triangular, T upper triangular, A = Q S Z^T, B = Q T Z^T).
 * Replaces geigvecs(S::GeneralizedSchur{<:Real}; left) (vectors.jl:22-33): right vectors
 * (_geigvecs, vectors.jl:1040-1283) into VR, back-transformed by Z; left vectors
 * (_gleigvecs, vectors.jl:1285-1513) into VL, back-transformed by Q.  VR, VL are complex
 * n x n (interleaved); a complex pair's second column is the conjugate of the first.
 * Either output may be NULL; Q / Z NULL give the eigenvectors of (S, T).  Columns scaled to
 * max |re| + |im| = 1.  Host pointers, or device with GS_DEVICE. */
GS_API int gs_ggeigvecs_f64(gs_context* ctx, int64_t n, const double* S, const double* T, const double* Q,
                            const double* Z, double* VR, double* VL, unsigned flags);

/* FP64 matrix product C (m x p, ldc) = op(A) (m x q) * B (q x p), op(A) = A (transA = 0)
 * or A^T (transA = 1), column-major, computed on the BF16 tensor cores by exact splitting
 * (Ozaki scheme: 10 slices of 6 bits per row of op(A) and column of B, exact FP32
 * accumulation of each slice product, FP64 sum of the 55 leading slice products).  The
 * error is below that of an FP64 dot product of the same length, measured against the
 * row maxima of op(A) and column maxima of B; Inf/NaN in a row of op(A) (column of B)
 * make that row (column) of C NaN.  No counterpart in the reference: the mixed-precision
 * refinement (gs_schur_mixed_f64) forms Z^T A Z and Z^T Z with it.  Synchronous; host
 * pointers, or device pointers with GS_DEVICE. */
GS_API int gs_gemm_f64_tc(gs_context* ctx, int64_t m, int64_t p, int64_t q, const double* A, int64_t lda,
                          int transA, const double* B, int64_t ldb, double* C, int64_t ldc, unsigned flags);

/* ggschur!(A, B; wantQ, wantZ, scale) for a real pencil (rgeneralized.jl:10-66): qr!(B),
 * the Hessenberg-triangular reduction (_hessenberg!, generalized.jl:84-113) and the real QZ
 * iteration (_gqz!, rgeneralized.jl:68-808; single and double shifts, 2 x 2 blocks of complex
 * eigenvalues with B diagonal there).  A <- S (quasi-triangular), B <- T (upper triangular,
 * non-negative diagonal), Q and Z (n x n real; NULL when not wanted) with A = Q S Z^T and
 * B = Q T Z^T; alpha (n complex, interleaved) and beta (n real) the generalized eigenvalues
 * alpha ./ beta.  Leading dimension n.  GS_SCALE applies _scale! to A and B.  GS_UNCONVERGED
 * at the reference's 100 n iteration limit. */
GS_API int gs_ggschur_f64(gs_context* ctx, int64_t n, double* A, double* B, double* Q, double* Z, double* alpha,
                          double* beta, unsigned flags);
/* The same over a ragged batch (layout as gs_ggschur_batched_c64 with real matrices, complex
 * alpha, real beta). */
GS_API int gs_ggschur_batched_f64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                                  int64_t packed_len, double* A, double* B, double* Q, double* Z, const int64_t* woffs,
                                  int64_t wlen, double* alpha, double* beta, int32_t* status, unsigned flags);

/* gordschur!(S, T, Q, Z, select) / ordschur!(F::GeneralizedSchur, select) for a complex
 * generalized Schur form (ordschur.jl:147-305): the eigenvalues with select[k] != 0 move to
 * the leading positions in their order, by adjacent swaps (_trexch2!, ztgex2 with the weak
 * and strong stability tests).  S, T, Q, Z (n x n, interleaved complex, leading dimension n)
 * in place; alpha, beta (n) the new diagonals.  GS_SCALE applies the reference's default
 * _scale! of S and T around the swaps.  GS_UNCONVERGED if a swap is rejected (the
 * reference's IllConditionException); the form is then partly reordered. */
GS_API int gs_ggordschur_c64(gs_context* ctx, int64_t n, double* S, double* T, double* Q, double* Z,
                             const int32_t* select, double* alpha, double* beta, unsigned flags);
/* gordschur!(S, T, Q, Z, select) for a real generalized Schur pair (rordschur.jl:542-627,
 * _trexchange! 629-766, _swap1or2! 768-962 after LAPACK's dtgexc / dtgex2): the 1 x 1 and
 * 2 x 2 blocks of the selected eigenvalues (a pair moves when either of its members is
 * selected) are moved to the top by orthogonal equivalences accumulated into Q and Z (either
 * may be NULL); S, T are overwritten with the reordered standardized pair, alpha (n,
 * interleaved complex) and beta (n, real) with the generalized eigenvalues.  GS_SCALE scales
 * as the reference's `scale = true` does.  GS_UNCONVERGED when a swap fails the stability
 * tests (the reference's IllConditionException). */
GS_API int gs_ggordschur_f64(gs_context* ctx, int64_t n, double* S, double* T, double* Q, double* Z,
                             const int32_t* select, double* alpha, double* beta, unsigned flags);

/* Eigenvectors of the generalized Schur decomposition of a complex pencil (the output
 * of gs_ggschur_c64: S, T upper triangular, A = Q S Z^H, B = Q T Z^H).  Replaces
 * geigvecs(S::GeneralizedSchur; left) (vectors.jl:22-33): right eigenvectors
 * (_geigvecs, vectors.jl:723-842) into VR, back-transformed by Z, with
 * beta_k A v = alpha_k B v; left eigenvectors (_gleigvecs, vectors.jl:845-1038) into VL,
 * back-transformed by Q, with conj(beta_k) A^H y = conj(alpha_k) B^H y.  Either output
 * may be NULL; Q / Z NULL give the eigenvectors of the triangular pair.  Columns scaled
 * to max |re| + |im| = 1; a singular pencil (S_kk = T_kk = 0) gives the unit vector e_k.
 * Interleaved complex, leading dimension n; host pointers, or device with GS_DEVICE. */
GS_API int gs_ggeigvecs_c64(gs_context* ctx, int64_t n, const double* S, const double* T, const double* Q,
                            const double* Z, double* VR, double* VL, unsigned flags);

/* Reordering a Schur decomposition.  Replaces gordschur!(T, Z, select) / ordschur!:
 * eigenvalues with select[k] != 0 move to the leading positions in their order.
 * Real (rordschur.jl:3-47, standard-form 2x2 blocks kept; a block is selected if
 * either of its eigenvalues is): T, Z n x n real, wr/wi the new eigenvalues.
 * Complex (ordschur.jl:24-74): T, Z interleaved complex, w the new diagonal.
 * T, Z in place, leading dimension n.  GS_UNCONVERGED if a block swap is rejected as
 * ill-conditioned (the reference's IllConditionException). */
GS_API int gs_ordschur_f64(gs_context* ctx, int64_t n, double* T, double* Z, const int32_t* select, double* wr,
                           double* wi, unsigned flags);
GS_API int gs_ordschur_c64(gs_context* ctx, int64_t n, double* T, double* Z, const int32_t* select, double* w,
                           unsigned flags);

#ifdef __cplusplus
}
#endif

#endif /* GSCHUR_GB300_H */
