/*
 * mat_gpu.h - C ABI of libmatgpu, the GB300 (sm_103a) implementation of
 * Mat's dense-factorization hot path: packed GEMM, blocked partial-pivoting
 * LU (PLU), Cholesky (LLT), blocked Householder QR and the Solve calls on top
 * of them, plus a mixed-precision (split-BF16 + iterative refinement) solve
 * and reverse-mode (adjoint) kernels.
 *
 * Conventions (all entry points):
 *   - Matrices are column-major with an explicit leading dimension, exactly
 *     like Mat's MAT<T> / __BlockMat<T> (Mat-8.3.1/Base/__Matrix.h:141-146,
 *     Mat-8.3.1/Base/__Block.h:3-34): element (r,c) lives at data[r + c*ld].
 *   - Every matrix / vector pointer is a DEVICE pointer unless the parameter
 *     name starts with "host_".  Work is enqueued on the handle's stream; the
 *     call returns after enqueueing unless documented otherwise (calls that
 *     report an `info` or a `report` synchronise the stream).
 *   - Sizes are `int`, as in Mat.  Every call returns an mg_status_t; Mat
 *     itself has no error channel (singular/non-SPD inputs fail silently,
 *     Mat-8.3.1/LU/__PLU.h:68-71, Mat-8.3.1/LU/__LLT.h:7).
 *   - There is no CPU fallback: without a CUDA device every compute call
 *     returns MG_ERR_CUDA.
 */
#ifndef MAT_GPU_H
#define MAT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mg_status {
    MG_OK = 0,
    MG_ERR_ARG = 1,          /* bad size / null pointer / bad leading dimension   */
    MG_ERR_CUDA = 2,         /* CUDA runtime error (no device, launch failure ...) */
    MG_ERR_ALLOC = 3,        /* device or pinned-host allocation failed            */
    MG_SINGULAR = 4,         /* exact zero pivot met; info = 1-based column        */
    MG_NOT_SPD = 5,          /* non-positive Cholesky pivot; info = 1-based column */
    MG_IR_STALLED = 6,       /* refinement did not reach the requested tolerance   */
    MG_FALLBACK_USED = 7,    /* mixed solve fell back to GMRES-IR or the FP64 path */
    MG_TIMEOUT = 8,          /* a bounded device-side wait gave up                 */
    MG_ERR_UNSUPPORTED = 9,  /* option not supported on this device                */
    MG_NOT_CONVERGED = 10    /* an iteration did not converge within its budget    */
} mg_status_t;

typedef struct mg_handle_s* mg_handle_t;

/* ---------------------------------------------------------------- handles */

/* Creates a handle bound to the current CUDA device.  `cuda_stream` is a
 * cudaStream_t (NULL = the legacy default stream). */
mg_status_t mg_handle_create(mg_handle_t* out, void* cuda_stream);
mg_status_t mg_handle_destroy(mg_handle_t h);
mg_status_t mg_set_stream(mg_handle_t h, void* cuda_stream);
mg_status_t mg_synchronize(mg_handle_t h);
const char* mg_status_string(mg_status_t s);
/* Last error text recorded on this handle (empty string if none). */
const char* mg_get_last_error(mg_handle_t h);
/* Number of this library's kernel launches enqueued through `h` so far. */
uint64_t mg_launch_count(mg_handle_t h);

/* Per-phase profiling: while on, each library phase (panel, trailing GEMM,
 * residual, ...) is bracketed by CUDA events on the handle's stream and
 * accumulated with the algorithmic flops / bytes it performed.  Turning it
 * on clears the records; count/get synchronise the stream. */
mg_status_t mg_profile_enable(mg_handle_t h, int on);
/* Restricts the timing to phases named `name` (NULL or "" = every phase), so
 * that timing one kernel family adds two event records per launch of it
 * only. */
mg_status_t mg_profile_only(mg_handle_t h, const char* name);
int mg_profile_count(mg_handle_t h);
mg_status_t mg_profile_get(mg_handle_t h, int i, const char** name, double* ms, long long* launches,
                           double* flops, double* bytes);

/* ------------------------------------------------------ memory utilities
 * For callers (C, cgo, JNI, ctypes) that do not link the CUDA runtime. */
mg_status_t mg_device_malloc(void** out, size_t bytes);
mg_status_t mg_device_free(void* p);
mg_status_t mg_host_malloc_pinned(void** out, size_t bytes);
mg_status_t mg_host_free_pinned(void* p);
/* Asynchronous copies on the handle's stream (kind: 0 = H2D, 1 = D2H, 2 = D2D). */
mg_status_t mg_memcpy(mg_handle_t h, void* dst, const void* src, size_t bytes, int kind);

/* ------------------------------------------------------ seeded generators
 * Counter-based, bit-identical on the host and on the device (no libm, no
 * fused operations).  Element (r,c) of a rows x cols matrix draws stream
 * index r*cols + c when `rowmajor_stream` != 0 (the "row-major fill" of the
 * benchmark configurations), else r + c*rows.  Mat's own generator is
 * time-seeded (Mat-5.1/_extra/__Random.h:2-27) and cannot be reproduced. */
void mg_host_fill_uniform(double* host_A, int rows, int cols, int ld, uint64_t seed,
                          double lo, double hi, int rowmajor_stream);
void mg_host_fill_normal(double* host_A, int rows, int cols, int ld, uint64_t seed,
                         int rowmajor_stream);
mg_status_t mg_fill_uniform(mg_handle_t h, double* A, int rows, int cols, int ld,
                            uint64_t seed, double lo, double hi, int rowmajor_stream);
mg_status_t mg_fill_normal(mg_handle_t h, double* A, int rows, int cols, int ld,
                           uint64_t seed, int rowmajor_stream);

/* ------------------------------------------------------------------ GEMM
 * C = alpha * op(A) * op(B) + beta * C, op(X) = X (trans = 0) or X^T (1).
 * With alpha = 1, beta = 0, transA = transB = 0 this is Mat's
 * `operator*(const MAT<t1>&, const MAT<t2>&)` for double
 * (Mat-8.3.1/Mul/Mul.h:204-235 -> __mulAB_2, Mul.h:155-202, which zeroes C
 * first, Mul.h:167).  With alpha = -1, beta = 1 it is the subtracting
 * trailing update __mulAB_packed_n (Mul.h:240-263).  When beta == 0, C is
 * not read (NaNs in C do not propagate). */
mg_status_t mg_dgemm(mg_handle_t h, int transA, int transB, int m, int n, int k,
                     double alpha, const double* A, int lda, const double* B, int ldb,
                     double beta, double* C, int ldc);
/* FP32 form: C = alpha op(A) op(B) + beta C on the SIMT FP32 pipe (FFMA),
 * 128 x 128 tiles, IEEE fp32 accumulation; not bit-identical to Mat's float
 * micro-kernel order.  Mat's operator* on MAT<float> (the same
 * Mul/Mul.h:204-235 template) runs this for small products and the
 * split-BF16 tensor-core GEMM (mg_sgemm_bf16x_ex, 3 terms, ordered) for
 * large ones (k >= 32, m n k >= 2^27), as do the GEMMs inside the FP32
 * Cholesky, its adjoint and the FP32 Gaussian-process loss. */
mg_status_t mg_sgemm(mg_handle_t h, int transA, int transB, int m, int n, int k, float alpha, const float* A,
                     int lda, const float* B, int ldb, float beta, float* C, int ldc);

/* ------------------------------------------------------------------- LU
 * In-place LU with partial pivoting, Mat's PLU (Mat-8.3.1/LU/__PLU.h:152-190,
 * blocked as __PLU, :93-149, block size 60): on return A holds the unit-lower
 * L strictly below the diagonal and U on and above it, and pos[0..m) (device)
 * is Mat's permutation: row i of L*U is row pos[i] of the input
 * (PLU_getP, :193-197, builds P with P(pos[i], i) = 1).  The pivot is the
 * first row holding the largest |a| of the column (:67-77).  m >= n is the
 * reference-parity domain; for m < n the trailing columns are eliminated
 * LAPACK-style (Mat leaves them un-updated after the last panel).  Returns
 * MG_SINGULAR with *info = first exactly-zero pivot column (1-based); Mat
 * has no such report and stops that panel instead.  Synchronises. */
mg_status_t mg_dgetrf(mg_handle_t h, int m, int n, double* A, int lda, int* pos, int* info);

/* mg_dgetrf without any allocation (no counterpart in Mat, whose calls each
 * allocate their packing buffers): for callers that cannot allocate device
 * memory when they factor, e.g. code running inside another system's memory
 * pool or fixed budget, or callers that must not synchronise the device the
 * way cudaMalloc/cudaFree do.  No handle: work goes on `cuda_stream` (NULL =
 * legacy default stream); the caller passes A and pos.  Scratch is one
 * file-scope device array of about 400 KiB per device, shared by every call:
 * calls that overlap on the GPU (other streams, other threads) race on it and
 * must be serialised by the caller.  Its address is looked up on the first
 * call on each device and kept, so make that first call before any stream
 * capture; a cudaDeviceReset (or other teardown of the device's primary
 * context) invalidates the kept address, and the entry point must not be
 * called on that device afterwards.  MG_ERR_UNSUPPORTED, returned before
 * anything is launched, means one of: m > 65536; more than 256 SMs; or the
 * first panel's slab does not fit shared memory: the panel is min(m, n)
 * columns wide when min(m, n) <= 90 (else 60) and its m rows are spread over
 * P = min(SMs, ceil(m / 128)) CTAs (one CTA when the slab is <= 64 KiB),
 * each holding ceil(m / P) rows x width doubles within the opt-in shared
 * memory per block (about 227 KiB on GB300: at width 90, m up to about
 * 48,000 rows; at width 60, every m <= 65536).  mg_dgetrf has the same
 * panel limit.  Otherwise the same results (bit for bit), statuses and
 * synchronisation as mg_dgetrf. */
mg_status_t mg_dgetrf_noalloc(void* cuda_stream, int m, int n, double* A, int lda, int* pos, int* info);

/* X := A^{-1} B from mg_dgetrf's factors and pos (n x n), B and X distinct.
 * Substitution order of Mat's narrow solve (Solve_direct_narrow,
 * Mat-8.3.1/LU/__Solve_direct.h:112-139) for every right-hand side. */
mg_status_t mg_dgetrs(mg_handle_t h, int n, int nrhs, const double* LU, int lda, const int* pos,
                      const double* B, int ldb, double* X, int ldx);

/* Mat's Solve_direct(A, B) (Mat-8.3.1/LU/__Solve_direct.h:146-220): A is
 * not modified (factored in a workspace copy), X = A^{-1} B.  Synchronises. */
mg_status_t mg_dgesv(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* B, int ldb,
                     double* X, int ldx, int* info);

/* Mat's Det(A) (Mat-8.3.1/LU/__Det.h:30-101) for n x n A (not modified):
 * the PLU of a copy, the parity of its row permutation, then the product
 * sign * U(0,0) * U(1,1) * ... in that order on the host, so the value
 * equals Mat's bit for bit.  An exactly singular A gives a zero.
 * Synchronises. */
mg_status_t mg_ddet(mg_handle_t h, int n, const double* A, int lda, double* det);

/* Mat's Inv(A) (Mat-8.3.1/LU/__Inv.h:212-225, with __Inv :90-161 and
 * __Inv_small :164-205) for n x n A (not modified): Ainv (ld ldinv) = A^{-1}
 * in Mat's operation order, bit for bit.  info = the first zero-pivot
 * column (1-based, status MG_SINGULAR) or 0; Mat does not check and neither
 * is the inverse skipped.  Ainv may be A when ldinv == lda.  Synchronises. */
mg_status_t mg_dinv(mg_handle_t h, int n, const double* A, int lda, double* Ainv, int ldinv, int* info);

/* Mat's LU(A, L, U) without pivoting (Mat-8.3.1/LU/__LU.h:71-108) for square
 * n x n A, in place: the unit lower factor's multipliers below the diagonal,
 * U on and above it, bit for bit Mat's.  An exactly zero pivot gives info =
 * its column + 1 and MG_SINGULAR (Mat's panel stops there; here the
 * factorization goes on, so the factors then differ from Mat's).
 * Synchronises. */
mg_status_t mg_dlu(mg_handle_t h, int n, double* A, int lda, int* info);

/* Mat's LDLT(A, L, D) (Mat-8.3.1/LU/__LLT.h:249-295, blocked __LDLT :153-209,
 * BS = 48), in place: reads the lower triangle of A (n x n), leaves Mat's
 * lower factor L (its diagonal as Mat computes it, d_j * (1/d_j)) with the
 * strict upper part zeroed, and d (device, n doubles) = diag(D); bit for bit.
 * No pivoting: an exactly zero d_j gives info = j + 1 and MG_SINGULAR (Mat
 * does not check; the factorization runs to the end).  Synchronises. */
mg_status_t mg_dldlt(mg_handle_t h, int n, double* A, int lda, double* d, int* info);

/* ------------------------------------------- symmetric eigendecomposition
 * Mat-8.1 snapshot's EVD_Q(A, E, Q, eps, EVD_QR) (Mat-8.1/EVD/EVD_Q.h:7-35,
 * EVD/__QR.h:145-169); results bit for bit those of its AVX-512 build.
 *
 * mg_dtridiag81: __EVD_Q_Householder (EVD/__QR.h:2-47) and __Householder_Q2
 * (QR/__Householder.h:124-152).  Reads the lower triangle of the symmetric A
 * (n x n), leaves the Householder reflectors below its diagonal, and writes
 * d (device, n) = the diagonal and e (device, n - 1) = the off-diagonal of
 * T = Q^T A Q, and Q (n x n).  Synchronises. */
mg_status_t mg_dtridiag81(mg_handle_t h, int n, double* A, int lda, double* Q, int ldq, double* d, double* e);

/* mg_devd_q: the whole EVD_Q with EVD_QR: A's lower triangle is read (A is
 * not modified unless A == E); E (n x n) receives diag(eigenvalues) and Q the
 * eigenvectors (A Q = Q E); w (device, n, may be NULL) the eigenvalues.  eps
 * is Mat's absolute deflation threshold on the off-diagonal.  The QR sweeps'
 * scalar recurrence runs on the host and the rotations are applied on the
 * GPU.  Mat iterates without limit; here after 64 n sweeps the call returns
 * MG_NOT_CONVERGED.  Synchronises. */
mg_status_t mg_devd_q(mg_handle_t h, int n, const double* A, int lda, double eps, double* E, int lde, double* Q,
                      int ldq, double* w);

/* mg_dsteqr81_host: the host half of mg_devd_q on its own, eigenvalues only:
 * Mat-8.1's implicit QR sweeps (EVD/__QR.h:50-142) on the tridiagonal with
 * diagonal d (host, n; overwritten with the eigenvalues, in Mat's order) and
 * off-diagonal e (host, n - 1), absolute deflation threshold eps.  rotations
 * (may be NULL) receives the number of plane rotations.  No GPU work, no
 * handle.  MG_NOT_CONVERGED after 64 n sweeps. */
mg_status_t mg_dsteqr81_host(int n, double* d, const double* e, double eps, long long* rotations);

/* ------------------------------------------------- split-precision GEMM
 * C = alpha * A * B + beta * C for fp32 column-major operands on the
 * tcgen05 BF16 tensor cores: A and B are split into `nterms` bf16 terms
 * (A = A0 + A1 + A2, A0 = bf16(A), A1 = bf16(A - A0), ...) and the products
 * of total order < nterms are accumulated in fp32 (nterms = 3: six products,
 * about fp32 accuracy; 2: three products; 1: plain bf16).  No counterpart in
 * Mat (Mat has no mixed precision); it is the trailing update of the mixed
 * LU and the split GEMM of the M=N=K=16384 benchmark configuration.
 * Uses handle workspace of nterms*(m+n)*k*2 bytes (k rounded up to 32). */
mg_status_t mg_sgemm_bf16x(mg_handle_t h, int nterms, int m, int n, int k, float alpha,
                           const float* A, int lda, const float* B, int ldb, float beta,
                           float* C, int ldc);
/* The same with options.  MG_BF16X_ORDERED: the lower-order products are
 * accumulated over all of k before the leading A0*B0 (a second pass over k
 * that reloads A0 and B0): the tensor cores round each accumulation relative
 * to the running sum, so this order is about 4x more accurate (normwise
 * 1.9e-5 against 7.2e-5 at m = n = k = 16384 with entries u*2^e, e in
 * [-8, 8]) for about 20% more time when the product is compute-bound. */
#define MG_BF16X_ORDERED 1
mg_status_t mg_sgemm_bf16x_ex(mg_handle_t h, int nterms, int flags, int m, int n, int k, float alpha,
                              const float* A, int lda, const float* B, int ldb, float beta, float* C, int ldc);
/* Device error word of the last split GEMM (MG_TIMEOUT if a bounded wait gave up). */
mg_status_t mg_bf16x_check_error(mg_handle_t h, int* device_err_flag);

/* ------------------------------------------- mixed LU + refinement solve
 * X = A^{-1} B (n x nrhs, nrhs <= 8) to FP64 normwise backward error:
 * fp32 LU with partial pivoting (fp32 panels, split-BF16 tensor-core
 * trailing updates, fp32 accumulation), then FP64 iterative refinement
 * (r = b - A x to FP64 accuracy or better (opts.residual), fp32 correction
 * solves, fp64 update) until every
 * column satisfies ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol.
 * If refinement stalls (the backward error not halving twice in a row, or
 * max_iter reached), GMRES-IR takes over: refinement steps whose correction
 * solves A d = r by FP64 GMRES (restart length 40, classical Gram-Schmidt
 * twice) left-preconditioned by the fp32 factors applied in FP64 arithmetic,
 * from x = 0 (Carson & Higham, "Accelerating the solution of linear systems
 * by iterative refinement in three precisions", SIAM J. Sci. Comput. 2018);
 * it converges well beyond plain refinement's condition-number range.  If
 * that stalls too, the solve falls back to the plain FP64 GPU solve
 * (mg_dgesv).  Either takeover returns MG_FALLBACK_USED (report.path 1 or
 * 2); with both off, or fallback off after GMRES-IR stalled, MG_IR_STALLED.
 * The mixed counterpart of Mat's Solve_direct
 * (Mat-8.3.1/LU/__Solve_direct.h:146-220), which has no mixed precision.
 * A and B are not modified.  Synchronises. */
typedef struct mg_ir_opts {
    double tol;    /* target backward error, default 1e-14 */
    int max_iter;  /* refinement iterations, default 30 */
    int nterms;    /* bf16 terms of the split updates (1..3), default 3 */
    int fallback;  /* nonzero: FP64 solve when refinement stalls (default 1) */
    int gmres;     /* nonzero: GMRES-IR when plain refinement stalls, before the
                      FP64 fallback (default 1; n up to the dataflow solves' size) */
    int panel;     /* FP32 panel pivoting: 0 = default, 1 = partial pivoting,
                      2 = tournament pivoting (one pivot agreement per 16 columns) */
    int residual;  /* arithmetic of r = b - A x: 0 = exact fixed-point integer
                      (default: every entry of A and x rounded once to 2^-63 of
                      its row's / column's largest, products and sums exact on
                      the integer pipe; an A or x with an infinity or NaN takes
                      FP64), 1 = FP64 FMA */
} mg_ir_opts;

/* R = B - A X (A n x n, X and B n x nrhs, nrhs <= 8; column-major), the
 * residual of the mixed solves on its own.  mode 0: exact fixed-point
 * integer arithmetic: every A(i,k) rounded once to a 63-bit integer in units
 * of 2^-62 of row i's largest power of two, every X(k,j) likewise per column,
 * the products and sums exact (int64 on the integer multiply-add pipe), the
 * sum rounded once to double, then R = B - that in FP64; its error is about
 * 2^-60 max|A(i,:)| max|X(:,j)| per entry, below FP64's accumulation error.
 * An A or X holding an infinity or NaN takes mode 1.  mode 1: FP64 FMA
 * (partial sums over column chunks of 2048, added in a fixed order).
 * Synchronises (mode 0). */
mg_status_t mg_dresidual(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* X,
                         int ldx, const double* B, int ldb, double* R, int ldr, int mode);

typedef struct mg_ir_report {
    int iterations;        /* refinement steps taken (plain and GMRES-IR outer steps) */
    int path;              /* 0 = refinement converged, 1 = GMRES-IR converged, 2 = FP64 fallback */
    int info;              /* first exactly-zero pivot column of the fp32 LU (1-based) */
    int gmres_iterations;  /* GMRES (inner) iterations of GMRES-IR, 0 if it did not run */
    double backward_error; /* final max-over-columns normwise backward error */
    double anorm_inf;      /* ||A||_inf */
    double factor_ms;      /* host wall time of the fp32 factorization */
    double refine_ms;      /* host wall time of the refinement loop */
    double history[32];    /* backward error before each correction */
    double pivot_growth;   /* max |U(i,j)| / max |A(i,j)| of the fp32 LU (fp64 reduction) */
} mg_ir_report;

mg_status_t mg_dsgesv_ir(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* B,
                         int ldb, double* X, int ldx, const mg_ir_opts* opts, mg_ir_report* report);

/* Mixed-precision solve for symmetric positive definite A (no mixed
 * precision in Mat; the FP64 counterpart is Mat's LLT, Mat-8.3.1/LU/__LLT.h:
 * 94-150, with the Cholesky solve): fp32 Cholesky of A's lower triangle in
 * blocks of 64 columns (fp32 diagonal blocks and block-column solves, the
 * trailing updates C -= L21 L21^T on the split-BF16 tensor cores, fp32
 * accumulation), its factor rewritten as the LU of the same matrix
 * (L D^-1)(D L^T), D = diag(L), then the refinement of mg_dsgesv_ir:
 * residuals (opts.residual) with all of A (both triangles: pass the full symmetric
 * matrix), GMRES-IR, FP64 fallback (mg_dgesv).  If the fp32 Cholesky breaks
 * down (a non-positive pivot, possible for nearly singular A) the solve
 * goes straight to the FP64 fallback (MG_FALLBACK_USED, path 2), or returns
 * MG_NOT_SPD with report.info when fallback is off.  opts.panel is ignored.
 * Synchronises. */
mg_status_t mg_dsposv_ir(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* B,
                         int ldb, double* X, int ldx, const mg_ir_opts* opts, mg_ir_report* report);

/* Mixed-precision solve through Householder QR (no mixed precision in Mat;
 * the FP64 counterpart is Mat's blocked Householder QR,
 * Mat-8.3.1/QR/__Householder_Blocked.h:63-353): n x n A factored by
 * mg_sgeqrf (fp32, the norm / beta / tau of every reflector in FP64, the
 * trailing updates on the split-BF16 tensor cores), then refined: r = b - A x
 * in FP64, d = R^{-1} Q^T r with the fp32 reflectors, T factors and R, x += d
 * in FP64.  Plain refinement solves for d in fp32 as the LU's does (Q^T and
 * the dataflow upper solve on the scaled residual; in FP64 arithmetic when
 * the dataflow grid cannot be co-resident); GMRES-IR uses the same operator
 * in FP64 arithmetic as its preconditioner; then the FP64 fallback as in
 * mg_dsgesv_ir.  The report's
 * pivot_growth is max |R| / max |A|.  opts.panel is ignored.  Synchronises. */
mg_status_t mg_dsqrsv_ir(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* B,
                         int ldb, double* X, int ldx, const mg_ir_opts* opts, mg_ir_report* report);
/* The FP32 Householder QR of that solve, for m x n A (m >= n), in place: R on
 * and above the diagonal, the reflectors v below it (v_c = 1 implicit, LAPACK
 * layout as in Mat's blocked panel, QR/__Householder_Blocked.h:63-84).
 * Panels of 128 columns, one cooperative grid each (one bounded grid
 * barrier per column; the column's sum of squares, alpha, beta = -sign(alpha)
 * ||x||, tau = (beta - alpha) / beta and the scale 1 / (alpha - beta) in
 * FP64, the reflector's dot products and updates in fp32), then T (the
 * compact WY factor, fp32, from V^T V formed inside the panel) and
 * R2 -= V (T^T (V^T R2)) with the products on the split-BF16 tensor cores.  tau: n doubles (device); T: ceil(n / 128) blocks
 * of 128 x 128 floats (device, block b column-major with ld 128).
 * Synchronises. */
mg_status_t mg_sgeqrf(mg_handle_t h, int m, int n, float* A, int lda, double* tau, float* T);

/* ----------------------------------------------- FP32 LU (mixed solve)
 * The single-precision factorizations inside mg_dsgesv_ir, exposed for
 * callers that refine on their own.  No counterpart in Mat (no mixed
 * precision there); the pivoting and the pos convention are those of Mat's
 * PLU (Mat-8.3.1/LU/__PLU.h:54-90: first row of the largest |a|, pos
 * starts as 0..m-1 and records each interchange, A(pos[i],:) = (LU)(i,:)).
 * An exactly zero pivot column is left unscaled and reported in info
 * (1-based, first such column); the call then returns MG_SINGULAR.
 *
 * mg_sgetf2: in-place unblocked panel LU of an m x n block, n <= 128 (the
 * panel of the mixed LU: one 16-CTA thread-block cluster for m <= 16384,
 * a cooperative grid beyond).  Synchronises. */
mg_status_t mg_sgetf2(mg_handle_t h, int m, int n, float* A, int lda, int* pos, int* info);
/* mg_sgetf2 with options.  MG_PANEL_TOURNAMENT: tournament pivoting on the
 * cluster path (Grigori, Demmel & Xiang's CALU, SIAM J. Matrix Anal. Appl.
 * 2011).  Per 16-column sub-panel the pivot rows are chosen by a reduction
 * tree of partial-pivoting eliminations, each level passing on the rows it
 * picked as they were when the sub-panel started: each warp over its own
 * rows, each CTA over its warps' picks, then (in every CTA alike) pairs of
 * CTAs and finally all 16 CTAs of the cluster; the 16 pivots are swapped to
 * the diagonal in order and the sub-panel eliminated without further
 * pivoting.  One cluster-wide exchange per 16 columns instead of one per
 * column.  The pivots may differ from partial pivoting's (|L| is no longer
 * bounded by 1); pos, info and the update order are as for mg_sgetf2.
 * Panels off the cluster path (m > 16384, or slabs up to 64 KiB) use partial
 * pivoting. */
#define MG_PANEL_TOURNAMENT 1
mg_status_t mg_sgetf2_ex(mg_handle_t h, int flags, int m, int n, float* A, int lda, int* pos, int* info);
/* mg_sgetrf: in-place blocked LU of an n x n fp32 matrix (blocks of 128:
 * mg_sgetf2 panels, block-row solve and trailing update on the split-BF16
 * tensor-core GEMM with 3 terms, fp32 accumulation).  Synchronises. */
mg_status_t mg_sgetrf(mg_handle_t h, int n, float* A, int lda, int* pos, int* info);

/* ------------------------------------------------ benchmark input generators
 * A = Q1 diag(sigma) Q2 with Q1, Q2 products of `nrefl` Householder
 * reflectors whose vectors are iid N(0,1) (seeded), sigma geometric from 1
 * down to sigma_min (condition number 1/sigma_min; 0 < sigma_min <= 1, else
 * MG_ERR_ARG).  Every operation has a fixed order and rounding (fused-chain
 * products, sigma from a series in basic arithmetic), so a host restatement
 * reproduces A bit for bit. */
mg_status_t mg_gen_svd_matrix(mg_handle_t h, int n, double* A, int lda, uint64_t seed, int nrefl,
                              double sigma_min);
/* S = G G^T / n + I with G iid N(0,1) (seeded, row-major stream order). */
mg_status_t mg_gen_spd_gram(mg_handle_t h, int n, double* S, int lds, uint64_t seed);

/* -------------------------------------------------------------- Cholesky
 * Mat's LLT (Mat-8.3.1/LU/__LLT.h:212-246, blocked as __LLT, :94-150,
 * block size 48), in place: reads the lower triangle of A, leaves L there and
 * zeroes the strict upper triangle.  Bit-identical to Mat's AVX-512 build.
 * Returns MG_NOT_SPD with *info = first non-positive pivot column (1-based);
 * Mat produces NaNs silently there (:7).  Synchronises. */
mg_status_t mg_dpotrf(mg_handle_t h, int n, double* A, int lda, int* info);
/* B := (L L^T)^{-1} B with L from mg_dpotrf (forward then back substitution). */
mg_status_t mg_dpotrs(mg_handle_t h, int n, int nrhs, const double* L, int ldl, double* B, int ldb);
/* FP32 Cholesky (LLT on MAT<float>, Mat-8.3.1/LU/__LLT.h:212-246): the same
 * blocking (48), kernels and conventions as mg_dpotrf in fp32, trailing
 * updates by mg_sgemm.  info / MG_NOT_SPD as mg_dpotrf.  Synchronises. */
mg_status_t mg_spotrf(mg_handle_t h, int n, float* A, int lda, int* info);

/* -------------------------------------------------------------------- QR
 * Mat's QR(A, Q, R, QR_Householder) (Mat-8.3.1/QR/QR.h:8-25, blocked
 * Householder with block size 48, __Householder_Blocked.h:215-353): A (m x n)
 * is not modified; Q (m x m, the full orthogonal factor as Mat forms it) and
 * R (m x n, zero below the diagonal) are written.  R(j,j) = -sign(x0)||x||.
 * Bit-identical to Mat's AVX-512 build when min(m, n) > 96; smaller
 * problems agree to rounding (Mat switches to its unblocked variant).
 * Synchronises. */
mg_status_t mg_dqr(mg_handle_t h, int m, int n, const double* A, int lda, double* Q, int ldq,
                   double* R, int ldr);
/* The factorization alone, in place: R on and above the diagonal of A, the
 * Householder vectors (unit first entry implied) below it, tau[min(m,n)] and
 * the upper-triangular compact-WY factors T (one 48 x 48 block per 48
 * columns, ceil(min(m,n)/48)*48*48 doubles). Synchronises. */
mg_status_t mg_dgeqrf(mg_handle_t h, int m, int n, double* A, int lda, double* tau, double* T);

/* ------------------------------------------------------------- adjoints
 * Reverse-mode calls for the Cholesky family (Mat has no derivatives; these
 * are the backward passes of LLT, Mat-8.3.1/LU/__LLT.h:212-246, of its
 * triangular solves, and of the Cholesky log-determinant).
 *
 * mg_dpotrf_backward: given L = chol(A) (lower) and Lbar (lower triangle
 * used), Abar = the symmetric gradient of the loss with respect to A, by the
 * blocked reverse-mode recurrence of Murray (2016) on Phi(L^T Lbar) (Phi =
 * lower triangle, diagonal halved).  Only L is read (no stored
 * intermediates); uses n*n doubles of handle workspace. */
mg_status_t mg_dpotrf_backward(mg_handle_t h, int n, const double* L, int ldl, const double* Lbar,
                               int ldlbar, double* Abar, int ldabar);
/* FP32 form of mg_dpotrf_backward (n*n floats of workspace). */
mg_status_t mg_spotrf_backward(mg_handle_t h, int n, const float* L, int ldl, const float* Lbar, int ldlbar,
                               float* Abar, int ldabar);
/* X = op(L)^{-1} B with L lower (trans = 0: L, 1: L^T): given X and Xbar,
 * writes Bbar = op(L)^{-T} Xbar and accumulates into the lower triangle of
 * Lbar (-tril(Bbar X^T) or -tril(X Bbar^T)); Lbar's strict upper triangle is
 * scratch. */
mg_status_t mg_dtrsm_backward(mg_handle_t h, int trans, int n, int nrhs, const double* L, int ldl,
                              const double* X, int ldx, const double* Xbar, int ldxbar, double* Bbar,
                              int ldbbar, double* Lbar, int ldlbar);
/* logdet(A) = 2 sum log L_ii for A = L L^T (host result; synchronises), and its
 * adjoint Lbar_ii += 2 gbar / L_ii. */
mg_status_t mg_dlogdet_chol(mg_handle_t h, int n, const double* L, int ldl, double* host_out);
mg_status_t mg_dlogdet_chol_backward(mg_handle_t h, int n, const double* L, int ldl, double gbar,
                                     double* Lbar, int ldlbar);
/* RBF kernel K(i,j) = sigma2 exp(-|x_i - x_j|^2 / (2 ell^2)) + jitter [i==j],
 * points X (n x 3, column-major). */
mg_status_t mg_gen_rbf_kernel(mg_handle_t h, int n, const double* X, double ell, double sigma2,
                              double jitter, double* K, int ldk);
/* Gaussian-process loss 0.5 y^T K^{-1} y + 0.5 logdet K with K the RBF kernel
 * above: forward (Cholesky, two triangular solves, logdet) and backward
 * (triangular-solve and logdet adjoints, Cholesky adjoint) in one call;
 * returns the loss and d loss / d ell on the host and, if Kbar is not NULL,
 * d loss / dK (symmetric).  Synchronises. */
mg_status_t mg_gp_loss_grad(mg_handle_t h, int n, const double* X, double ell, double sigma2, double jitter,
                            const double* y, double* host_loss, double* host_dell, double* Kbar,
                            int ldkbar);
/* FP32 form of mg_gp_loss_grad: X, y, K and every matrix step in fp32
 * (mg_spotrf, fp32 solves, fp32 Cholesky adjoint); the scalar reductions
 * (y^T K^-1 y, logdet, d loss / d ell) are summed in fp64. */
mg_status_t mg_sgp_loss_grad(mg_handle_t h, int n, const float* X, float ell, float sigma2, float jitter,
                             const float* y, double* host_loss, double* host_dell, float* Kbar, int ldkbar);

/* Measures the FP64 peaks of this GPU with dependent-free FMA / DMMA loops
 * (TFLOP/s, counting an FMA as 2 flops).  Synchronises. */
mg_status_t mg_measure_fp64_peaks(mg_handle_t h, double* dfma_tflops, double* dmma_tflops);

/* Self-test of the bounded device-side waits (no counterpart in Mat, which
 * has no error channel: a zero pivot is a silent break,
 * Mat-8.3.1/LU/__PLU.h:68-71).  Runs the library's own wait code with a
 * budget of `poll_limit` polls (1 .. 2^24): kind 0 = the grid barrier of the
 * cooperative kernels, in a cooperative launch of 8 CTAs of which CTA
 * `withhold` (0..7) never arrives; kind 1 = an mbarrier wait on a phase that
 * nothing completes.  withhold < 0 lets every wait complete.  Returns
 * MG_TIMEOUT when the wait ran out (the kernel records it and returns: no
 * trap, no hang, the handle stays usable), MG_OK otherwise.  Synchronises. */
mg_status_t mg_selftest_bounded_wait(mg_handle_t h, int kind, int withhold, unsigned poll_limit);

#ifdef __cplusplus
}
#endif

#endif /* MAT_GPU_H */
