/*
 * ddla_gb300.h -- C ABI of the GB300 (sm_103a) implementation of DDLA's dense
 * hot path: BLIS-shaped FP64 level-3 calls, the blocked LU / Cholesky / LDL^T
 * factorizations and solves, mixed-precision solves with FP64 iterative
 * refinement, batched small factorizations and two-operand einsum.
 *
 * Every entry point is `extern "C"`, takes plain pointers, sizes and element
 * strides, and returns an int32 status:
 *     0                 success
 *     < 0 (> -1000)     -(position of the first invalid argument), 1-based
 *     > 0               1-based index of the first failing pivot (singular LU
 *                       pivot, non-positive Cholesky pivot, zero LDL^T pivot);
 *                       DDLA throws LinalgException / ArgumentException there
 *     DDLA_ERR_*        runtime errors (CUDA, timeout, no convergence, memory)
 * A human-readable message for the last failure of the calling thread is
 * available from ddla_last_error().
 *
 * Matrices follow DDLA's MatrixView (DDLA/Core/MatrixView.cs:22-31): a pointer
 * to the head element plus a row stride and a column stride, in elements.
 * Either stride may be 1; a transposed view swaps them.  Flag values are the
 * BLIS values DDLA's enums carry (DDLA/Misc/Flags/*.cs).  dim/inc types are
 * 64-bit (DDLA/Alias.cs:1-3); alpha and beta are passed by pointer like the
 * `in double` of DDLA's P/Invoke declarations.
 *
 * Host-pointer entry points (ddla_d*) are synchronous drop-ins for the BLIS
 * calls DDLA makes through P/Invoke: data is copied to the device, computed
 * there and copied back before return; the caller's arrays are not retained.
 * Device entry points (ddla_dev_*) take device pointers and a handle whose
 * stream they are enqueued on; they return once enqueued unless stated.
 * All entry points are thread-safe: host-pointer calls use a per-thread handle.
 */
#ifndef DDLA_GB300_H
#define DDLA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int64_t ddla_dim_t;
typedef int64_t ddla_inc_t;

/* TransType, DDLA/Misc/Flags/TransType.cs:3-9 */
enum { DDLA_NO_TRANSPOSE = 0, DDLA_TRANSPOSE = 8, DDLA_CONJ_NO_TRANSPOSE = 16, DDLA_CONJ_TRANSPOSE = 24 };
/* UpLo, DDLA/Misc/Flags/UpLo.cs:3-9 */
enum { DDLA_ZEROS = 0x00, DDLA_LOWER = 0xC0, DDLA_UPPER = 0x60, DDLA_DENSE = 0xE0 };
/* DiagType, DDLA/Misc/Flags/DiagType.cs */
enum { DDLA_NONUNIT_DIAG = 0x000, DDLA_UNIT_DIAG = 0x100 };
/* SideType, DDLA/Misc/Flags/SideType.cs */
enum { DDLA_LEFT = 0, DDLA_RIGHT = 1 };

/* runtime status codes (all below -1000 so they never collide with argument
 * positions) */
enum {
    DDLA_OK = 0,
    DDLA_ERR_CUDA = -1001,          /* a CUDA runtime call failed */
    DDLA_ERR_NOMEM = -1002,         /* device or pinned allocation failed */
    DDLA_ERR_TIMEOUT = -1003,       /* a bounded device-side wait gave up */
    DDLA_ERR_NOT_CONVERGED = -1004, /* iterative refinement hit max_iter */
    DDLA_ERR_UNSUPPORTED = -1005,   /* valid request the library does not cover */
    DDLA_ERR_NO_DEVICE = -1006      /* no usable sm_103 device */
};

/* Precision of the O(n^3) work in the mixed solvers. */
enum {
    DDLA_PREC_FP64 = 0,      /* plain FP64 factorization (DMMA) */
    DDLA_PREC_FP32 = 1,      /* FP32 factorization, FP32 CUDA-core GEMM updates */
    DDLA_PREC_TF32X3 = 2,    /* FP32 factorization, 3xTF32 tcgen05 tensor-core GEMM updates */
    DDLA_PREC_BF16X3 = 3,    /* FP32 factorization, 3xBF16 tcgen05 tensor-core GEMM updates (x = hi + lo in
                                two bf16 parts, hi*hi + hi*lo + lo*hi, FP32 accumulation) */
    DDLA_PREC_OZAKI = 4      /* FP64-accurate GEMM from split BF16 tensor-core products */
};

/* Options of the factorization / mixed-solver calls.  Zero-initialised means
 * defaults.  (DDLA keeps these as mutable statics: LU.PLUBlockSize,
 * Cholesky.BlockSize, LDLT.BlockSize = 128, DDLA/Factorizations/LU.cs:131,235,
 * Cholesky.cs:125, LDLT.cs:139.) */
typedef struct ddla_opts {
    int32_t precision;     /* DDLA_PREC_*; 0 = FP32 for the mixed solvers, FP64 for the plain
                              factorizations (which also accept DDLA_PREC_OZAKI updates) */
    int32_t nb;            /* outer block size; 0 = automatic */
    int32_t max_iter;      /* refinement iterations; 0 = default 30; <0 = none */
    int32_t reserved;
    double tol;            /* target relative backward error; 0 = 1e-14 */
} ddla_opts;

/* Result record of a mixed-precision solve. */
typedef struct ddla_solve_report {
    int32_t iterations;        /* correction solves with the low-precision factors (classical steps, or
                                  GMRES preconditioner applications for one right-hand side) */
    int32_t converged;         /* 1 when backward_error <= tol */
    int32_t precision;         /* precision actually used for the factorization */
    int32_t info;              /* factorization status (0 or failing pivot) */
    double backward_error;     /* max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf) */
    double forward_error;      /* ||x - x_ref||_inf / ||x_ref||_inf when x_ref was given, else -1 */
    double factor_ms;          /* device time of the factorization */
    double refine_ms;          /* device time of the refinement loop */
    int32_t pivots_agree;      /* LU with a reference pivot vector (ddla_dev_dgesv_mixed_piv): how many of
                                  the n pivots of the low-precision factor equal the reference's; -1 = not
                                  measured */
    int32_t pivots_first_diff; /* first index where they differ; -1 = none or not measured */
    /* Growth monitor, computed in FP64 on the GPU from the low-precision factors (0 when the
     * factorization failed).  growth: LU max|u_ij| / max|a_ij| (the pivot growth factor);
     * Cholesky max_i sum_k l_ik^2 / max|a_ij|; LDL^T max_i (sum_k<i l_ik^2 |d_k| + |d_i|) /
     * max|a_ij| -- for Cholesky and LDL^T a bound on the entries of |L||D||L^T| relative to A,
     * which bounds the factorization's backward error.  diag_ratio: max / min over the
     * diagonal of U (LU), of L^2 (Cholesky) or of |D| (LDL^T, its pivots d_i). */
    double growth;
    double diag_ratio;
} ddla_solve_report;

/* ---------------------------------------------------------------- runtime */

/* Message describing the calling thread's last failure ("" if none). */
const char *ddla_last_error(void);
/* Library version string. */
const char *ddla_version(void);
/* Number of kernels this library has launched in this process (all threads). */
int64_t ddla_kernel_launches(void);

typedef struct ddla_handle_s *ddla_handle;
/* Create a handle bound to the current device and a stream (cudaStream_t cast
 * to void*; NULL = a new non-blocking stream owned by the handle; the legacy
 * default stream is cudaStreamLegacy, (void *)1). */
int ddla_handle_create(ddla_handle *h, void *stream);
int ddla_handle_destroy(ddla_handle h);
int ddla_handle_sync(ddla_handle h);

/* Measure this GPU's FP64 DMMA and FP32 FFMA throughput (TFLOP/s) with
 * bounded register-resident loops (no memory traffic). */
int ddla_measure_peaks(double *fp64_tflops, double *fp32_tflops);

/* Per-launch device timing of kernel classes (0 trailing-matrix GEMM update,
 * 1 LU panel, 2 TRSM, 3 row interchanges, 4 refinement FP64 residual,
 * 5 batched, 6 einsum GEMM, 7 QR T factor, 8 refinement correction solves with
 * the low-precision factors, 9 two-stage bidiagonal: band reduction with U and
 * V of stage 1, 10 its band chase, 11 its back-transformation of U and V).
 * ddla_timing_enable(1) clears the records and brackets every later
 * launch of those classes with CUDA events on its stream; ddla_timing_read
 * sums one class: total device ms, launches, algorithmic flops and bytes. */
int ddla_timing_enable(int on);
int ddla_timing_read(int cls, double *total_ms, int64_t *launches, double *flops, double *bytes);

/* Tuning parameters (no DDLA counterpart; DDLA hard-codes its blocking in
 * GEMMKernel, DDLA/Einsum/GEMMKernel.cs:11-21, and LU/Cholesky/LDLT.BlockSize).
 * Keys: "lu.nb" (LU panel width cap), "lu.lookahead" (0 turns the look-ahead
 * panel off), "chol.lookahead" (0 turns the Cholesky look-ahead off),
 * "panel.cluster" (CTAs per panel cluster), "panel.calu" (1 = tournament-
 * pivoting FP32 panels), "trsv.cluster" (0 uses
 * the chained per-block triangular solve instead of the cluster solve),
 * "trsv.chain16" (0 keeps the 4-group chained solve for 9-16 right-hand sides),
 * "trsv.cluster.size", "trsv.split.w" (near tiles per block row that the
 * one-right-hand-side cluster solve keeps on its chain while helper clusters
 * sum the far tiles; 0 = one cluster), "trsv.split.pw" (the near tile at
 * which the chain adds a row's far sum), "trsv.split.clusters" (cap on the
 * clusters of the split solve), "refine.gmres" (0 = classical refinement for one
 * right-hand side), "refine.gmres.m" (GMRES restart length),
 * "refine.gmres.relax" (factor on GMRES's 2-norm stopping target; 0 =
 * min(16, sqrt(n) / 4)),
 * "batched.nb.{32,64,128,big}", "batched.ctas_per_sm", "update.tc",
 * "update.tn", "update.tiles_per_cta", "u12.gemm", "qr.nb" (QR panel width
 * cap), "qr.cluster" (CTAs per QR panel cluster), "qr.resident" (0 factors QR
 * panels in place through L2 instead of in shared memory).  value == INT64_MIN
 * removes a key. */
int ddla_tune_set(const char *key, int64_t value);
int64_t ddla_tune_get(const char *key, int64_t dflt);

/* ------------------------------------------------ BLIS-shaped level 3 (host) */

/* C = beta*C + alpha*op(A)*op(B).  Replaces bli_dgemm,
 * DDLA/BLAS/Native/3m.cs:12-24 (wrapper DDLA/BLAS/3m.cs:10-31). */
int ddla_dgemm(int32_t transa, int32_t transb, ddla_dim_t m, ddla_dim_t n, ddla_dim_t k,
               const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
               const double *b, ddla_inc_t rsb, ddla_inc_t csb,
               const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);

/* Triangle of C (uploc) = beta*C + alpha*op(A)*op(B), C m x m.  Replaces
 * bli_dgemmt, DDLA/BLAS/Native/3m.cs:26-38 (wrapper DDLA/BLAS/3m.cs:44-70). */
int ddla_dgemmt(int32_t uploc, int32_t transa, int32_t transb, ddla_dim_t m, ddla_dim_t k,
                const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);

/* Triangle of C = beta*C + alpha*op(A)*op(A)^T.  Replaces bli_dsyrk,
 * DDLA/BLAS/Native/3m.cs:96-106 (wrapper DDLA/BLAS/3m.cs:118-138). */
int ddla_dsyrk(int32_t uploc, int32_t transa, ddla_dim_t m, ddla_dim_t k,
               const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
               const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);

/* C = beta*C + alpha*A*op(B) (left) or beta*C + alpha*op(B)*A (right), A
 * symmetric (m x m left, n x n right) and read only in its uploa triangle;
 * conja is accepted and ignored (real data).  Replaces bli_dsymm,
 * DDLA/BLAS/Native/3m.cs:81-94 (wrapper DDLA/BLAS/3m.cs:83-106). */
int ddla_dsymm(int32_t sidea, int32_t uploa, int32_t conja, int32_t transb, ddla_dim_t m, ddla_dim_t n,
               const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
               const double *b, ddla_inc_t rsb, ddla_inc_t csb,
               const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);

/* Triangle of C (uploc, m x m) = beta*C + alpha*op(A)*op(B)^T +
 * alpha*op(B)*op(A)^T, op(A) and op(B) m x k.  Replaces bli_dsyr2k,
 * DDLA/BLAS/Native/3m.cs:108-120 (wrapper DDLA/BLAS/3m.cs:149-172). */
int ddla_dsyr2k(int32_t uploc, int32_t transa, int32_t transb, ddla_dim_t m, ddla_dim_t k,
                const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);

/* B = alpha*op(A)*B (left) or alpha*B*op(A) (right) in place, A triangular
 * (uploa, diaga; the other triangle and a unit diagonal are never read).
 * Replaces bli_dtrmm, DDLA/BLAS/Native/3m.cs:122-133 (wrapper
 * DDLA/BLAS/3m.cs:185-204). */
int ddla_dtrmm(int32_t sidea, int32_t uploa, int32_t transa, int32_t diaga, ddla_dim_t m, ddla_dim_t n,
               const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
               double *b, ddla_inc_t rsb, ddla_inc_t csb);

/* C = beta*C + alpha*op(A)*op(B) (left) or beta*C + alpha*op(B)*op(A)
 * (right), A triangular, C m x n.  Replaces bli_dtrmm3,
 * DDLA/BLAS/Native/3m.cs:135-149 (wrapper DDLA/BLAS/3m.cs:225-250). */
int ddla_dtrmm3(int32_t sidea, int32_t uploa, int32_t transa, int32_t diaga, int32_t transb, ddla_dim_t m,
                ddla_dim_t n, const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);

/* Left: solve op(A) X = alpha B; Right: X op(A) = alpha B; B <- X.  Replaces
 * bli_dtrsm, DDLA/BLAS/Native/3m.cs:151-162 (wrapper DDLA/BLAS/3m.cs:287-305). */
int ddla_dtrsm(int32_t side, int32_t uploa, int32_t transa, int32_t diaga, ddla_dim_t m, ddla_dim_t n,
               const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
               double *b, ddla_inc_t rsb, ddla_inc_t csb);

/* ------------------------------------------------ QR (host) */

/* Householder QR in place: R on and above the diagonal, the Householder
 * vectors u_j (u_j(j) = 1 implicit) below it.  T (t_rows x n, element strides
 * rst / cst) receives, for every block of t_rows columns starting at j0, the
 * upper triangular UT factor S of that block in T[0:b, j0:j0+b]
 * (S(j,j) = tau_j, S(i,j) = u_i^T u_j); the rest of T is not written.
 * QR.QRDecompose(A, T), DDLA/Factorizations/QR.cs:130-149, 314-389; DDLA
 * sizes T with QR.CreateT (QR.cs:124-128): t_rows = min(256, max(m, n)).
 * opts (may be NULL): precision DDLA_PREC_OZAKI runs the large block-reflector
 * products through the split-precision tensor-core GEMM (FP64-level accuracy),
 * nb caps the panel width. */
int ddla_dgeqrf(ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa,
                double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst, const ddla_opts *opts);
/* B (m x nrhs) = Q^T B (trans != 0) or Q B with the factors of ddla_dgeqrf.
 * QR.ApplyQT / ApplyQ, QR.cs:79-109 (ApplyQlhfc / ApplyQlnfc, QR.cs:417-534). */
int ddla_dormqr(int32_t trans, ddla_dim_t m, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa,
                ddla_inc_t csa, const double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst,
                double *b, ddla_inc_t rsb, ddla_inc_t csb);
/* X (n x nrhs) = least-squares solution of A X = B (m >= n): Q^T B, then R.
 * QR.Solve, QR.cs:151-168, 391-415. */
int ddla_dgeqrs(ddla_dim_t m, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                const double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst,
                const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx);
/* Q (m x m) = H_0 H_1 ... H_{k-1}.  QR.FormQ(A, T, Q), QR.cs:179-201. */
int ddla_dorgqr(ddla_dim_t m, ddla_dim_t n, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                const double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst,
                double *q, ddla_inc_t rsq, ddla_inc_t csq);

/* ------------------------------------------------ tridiagonal reduction (host) */

/* Householder reduction of the symmetric n x n A (its lower triangle is read)
 * to tridiagonal form: on return A holds Q with Q^T A Q = tridiag(d, e),
 * d (n) the diagonal, e (n - 1) the subdiagonal, T (t_rows x n) the block
 * factors of the reflectors.  Tridiagonaling.Tridiag(A, T, d, e),
 * DDLA/Transformations/Tridiagonaling.cs:33-56 (Step :72-112, FormQ
 * :122-203); DDLA sizes T with CreateT (:15-19): t_rows = min(64, n).
 * opts (may be NULL): precision DDLA_PREC_OZAKI forms Q with split-precision
 * block-reflector products. */
int ddla_dsytrd(ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *t, ddla_dim_t t_rows,
                ddla_inc_t rst, ddla_inc_t cst, double *d, double *e, const ddla_opts *opts);

/* ------------------------------------------------ bidiagonal reduction (host) */

/* One-stage Householder reduction of A (m x n, m >= n) to upper bidiagonal
 * form: U^T A V = bidiag(d, e) with U (m x m) and V (n x n) orthogonal; A is
 * overwritten by the reflectors.  Bidiagonaling.Bidiag2 (HHStepBlock and
 * BuildUV), DDLA/Transformations/Bidiagonaling.cs:48-143.  opts (may be NULL):
 * precision DDLA_PREC_OZAKI forms U and V with split-precision products. */
int ddla_dbidiag(ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *d, double *e,
                 double *u, ddla_inc_t rsu, ddla_inc_t csu, double *v, ddla_inc_t rsv, ddla_inc_t csv,
                 const ddla_opts *opts);
/* Two-stage reduction of A (m x n, m >= n) to upper bidiagonal form, the one
 * DDLA's SVD calls: Bidiagonaling.Bidiag through TwoStageBidiag,
 * DDLA/Transformations/Bidiagonaling.cs:14-33 and 334-582.  Stage 1 reduces
 * A to an upper band of width 32 with blocked QR / LQ steps (Ge2Bd), stage 2
 * chases the band to the bidiagonal with small reflectors (Bd2Bi), whose
 * products are accumulated into U and V.  U^T A_in V = bidiag(d, e); A is
 * overwritten (band and zeros).  opts (may be NULL): precision
 * DDLA_PREC_OZAKI runs stage 1's block-reflector products through the
 * split-precision tensor-core GEMM.  DDLA_ERR_TIMEOUT if a bounded wait of
 * the band chase gave up. */
int ddla_dbidiag_twostage(ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *d,
                          double *e, double *u, ddla_inc_t rsu, ddla_inc_t csu, double *v, ddla_inc_t rsv,
                          ddla_inc_t csv, const ddla_opts *opts);

/* ------------------------------------------------ factorizations (host) */

/* In-place LU with partial pivoting; piv[i] is RELATIVE (row i swapped with
 * row i + piv[i]) exactly as LU.PLUDecompose, DDLA/Factorizations/LU.cs:251-264. */
int ddla_dgetrf(ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, int32_t *piv, const ddla_opts *opts);
/* Solve with the factors of ddla_dgetrf (trans != 0: A^T X = B).
 * LU.PLUSolve, LU.cs:266-287, 431-465. */
int ddla_dgetrs(int32_t trans, ddla_dim_t n, ddla_dim_t nrhs, const double *lu, ddla_inc_t rsa, ddla_inc_t csa,
                const int32_t *piv, double *b, ddla_inc_t rsb, ddla_inc_t csb);
/* In-place LU without pivoting, LU.LUDecompose, LU.cs:133-142, 169-203. */
int ddla_dgetrf_nopiv(ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, const ddla_opts *opts);
/* LU.LUSolve, LU.cs:144-167, 205-231. */
int ddla_dgetrs_nopiv(int32_t trans, ddla_dim_t n, ddla_dim_t nrhs, const double *lu, ddla_inc_t rsa, ddla_inc_t csa,
                      double *b, ddla_inc_t rsb, ddla_inc_t csb);
/* In-place Cholesky of the uplo triangle, Cholesky.CholDecompose,
 * DDLA/Factorizations/Cholesky.cs:52-69. */
int ddla_dpotrf(int32_t uplo, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, const ddla_opts *opts);
/* Cholesky.CholeskySolve, Cholesky.cs:102-123, 210-226. */
int ddla_dpotrs(int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                double *b, ddla_inc_t rsb, ddla_inc_t csb);
/* In-place unpivoted LDL^T, LDLT.LDLTDecompose, DDLA/Factorizations/LDLT.cs:56-73. */
int ddla_dldlt(int32_t uplo, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, const ddla_opts *opts);
/* LDLT.LDLTSolve, LDLT.cs:105-126, 267-295. */
int ddla_dldlts(int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                double *b, ddla_inc_t rsb, ddla_inc_t csb);

/* Mixed-precision solves: factor in opts->precision, refine in FP64 until the
 * relative backward error is <= opts->tol.  A and B are read only; X receives
 * the solution.  x_ref (may be NULL) is an oracle solution for the forward
 * error.  Any number of right-hand sides: they are refined in blocks of 16
 * with the same factors (the report gives the worst block).  No reference
 * counterpart: DDLA's LU(A).Solve / Cholesky(A).Solve / LDLT.Solve
 * (LU.cs:64-100, Cholesky.cs:71-88, LDLT.cs:75-100) are FP64-only.
 * ddla_dsysv_mixed is the unpivoted LDL^T of DDLA's LDLT (LDLT.cs:56-295) in
 * FP32 with FP64 refinement: like DDLA's it needs A's leading blocks
 * non-singular; the report's growth and diag_ratio tell how much the
 * unpivoted factorization amplified A. */
int ddla_dgesv_mixed(ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                     const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx,
                     const double *x_ref, const ddla_opts *opts, ddla_solve_report *report);
int ddla_dposv_mixed(int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                     const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx,
                     const double *x_ref, const ddla_opts *opts, ddla_solve_report *report);
int ddla_dsysv_mixed(int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                     const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx,
                     const double *x_ref, const ddla_opts *opts, ddla_solve_report *report);

/* ------------------------------------------------ device-resident variants */
/* Same semantics as the host calls; pointers are device pointers; work is
 * enqueued on the handle's stream.  Factorization statuses > 0 are produced
 * on the device: these calls synchronize the stream to return them. */
int ddla_dev_dgemm(ddla_handle h, int32_t transa, int32_t transb, ddla_dim_t m, ddla_dim_t n, ddla_dim_t k,
                   double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                   const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                   double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);
/* FP64 GEMM with a selectable arithmetic: DDLA_PREC_FP64 (DMMA, same as
 * ddla_dev_dgemm) or DDLA_PREC_OZAKI (error-free BF16 slices on the tensor
 * cores, FP64-level accuracy: |error| <= a small multiple of 2^-53 k
 * max_l|a_il| max_l|b_lj|).  The reference GEMM (DDLA/BLAS/Native/3m.cs:12-24)
 * has a single FP64 arithmetic; the precision argument has no counterpart there. */
int ddla_dev_dgemm_ex(ddla_handle h, int32_t precision, int32_t transa, int32_t transb, ddla_dim_t m, ddla_dim_t n,
                      ddla_dim_t k, double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                      const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                      double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);
int ddla_dev_dgemmt(ddla_handle h, int32_t uploc, int32_t transa, int32_t transb, ddla_dim_t m, ddla_dim_t k,
                    double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                    const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                    double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);
int ddla_dev_dtrsm(ddla_handle h, int32_t side, int32_t uploa, int32_t transa, int32_t diaga, ddla_dim_t m,
                   ddla_dim_t n, double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                   double *b, ddla_inc_t rsb, ddla_inc_t csb);
int ddla_dev_dsymm(ddla_handle h, int32_t sidea, int32_t uploa, int32_t conja, int32_t transb, ddla_dim_t m,
                   ddla_dim_t n, double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                   const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                   double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);
int ddla_dev_dsyr2k(ddla_handle h, int32_t uploc, int32_t transa, int32_t transb, ddla_dim_t m, ddla_dim_t k,
                    double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                    const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                    double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);
/* In place: the product is formed from a copy of B kept in the handle's
 * scratch (m*n doubles). */
int ddla_dev_dtrmm(ddla_handle h, int32_t sidea, int32_t uploa, int32_t transa, int32_t diaga, ddla_dim_t m,
                   ddla_dim_t n, double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                   double *b, ddla_inc_t rsb, ddla_inc_t csb);
int ddla_dev_dtrmm3(ddla_handle h, int32_t sidea, int32_t uploa, int32_t transa, int32_t diaga, int32_t transb,
                    ddla_dim_t m, ddla_dim_t n, double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                    const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                    double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc);
int ddla_dev_dbidiag(ddla_handle h, ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *d,
                     double *e, double *u, ddla_inc_t rsu, ddla_inc_t csu, double *v, ddla_inc_t rsv, ddla_inc_t csv,
                     const ddla_opts *opts);
int ddla_dev_dbidiag_twostage(ddla_handle h, ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa,
                              ddla_inc_t csa, double *d, double *e, double *u, ddla_inc_t rsu, ddla_inc_t csu,
                              double *v, ddla_inc_t rsv, ddla_inc_t csv, const ddla_opts *opts);
int ddla_dev_dsytrd(ddla_handle h, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *t,
                    ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst, double *d, double *e, const ddla_opts *opts);
int ddla_dev_dgeqrf(ddla_handle h, ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa,
                    double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst, const ddla_opts *opts);
int ddla_dev_dormqr(ddla_handle h, int32_t trans, ddla_dim_t m, ddla_dim_t n, ddla_dim_t nrhs, const double *a,
                    ddla_inc_t rsa, ddla_inc_t csa, const double *t, ddla_dim_t t_rows, ddla_inc_t rst,
                    ddla_inc_t cst, double *b, ddla_inc_t rsb, ddla_inc_t csb);
int ddla_dev_dgeqrs(ddla_handle h, ddla_dim_t m, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa,
                    ddla_inc_t csa, const double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst,
                    const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx);
int ddla_dev_dorgqr(ddla_handle h, ddla_dim_t m, ddla_dim_t n, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                    const double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst,
                    double *q, ddla_inc_t rsq, ddla_inc_t csq);
int ddla_dev_dgetrf(ddla_handle h, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, int32_t *piv,
                    const ddla_opts *opts);
int ddla_dev_dgetrs(ddla_handle h, int32_t trans, ddla_dim_t n, ddla_dim_t nrhs, const double *lu, ddla_inc_t rsa,
                    ddla_inc_t csa, const int32_t *piv, double *b, ddla_inc_t rsb, ddla_inc_t csb);
int ddla_dev_dpotrf(ddla_handle h, int32_t uplo, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa,
                    const ddla_opts *opts);
int ddla_dev_dpotrs(ddla_handle h, int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa,
                    ddla_inc_t csa, double *b, ddla_inc_t rsb, ddla_inc_t csb);
int ddla_dev_dldlt(ddla_handle h, int32_t uplo, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa,
                   const ddla_opts *opts);
int ddla_dev_dldlts(ddla_handle h, int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa,
                    ddla_inc_t csa, double *b, ddla_inc_t rsb, ddla_inc_t csb);
/* Mixed solves on device data (A, B row-major contiguous n x n, n x nrhs;
 * X n x nrhs row-major).  Synchronous (returns the report). */
int ddla_dev_dgesv_mixed(ddla_handle h, ddla_dim_t n, ddla_dim_t nrhs, const double *a, const double *b, double *x,
                         const double *x_ref, const ddla_opts *opts, ddla_solve_report *report);
int ddla_dev_dposv_mixed(ddla_handle h, int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a,
                         const double *b, double *x, const double *x_ref, const ddla_opts *opts,
                         ddla_solve_report *report);
int ddla_dev_dsysv_mixed(ddla_handle h, int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a,
                         const double *b, double *x, const double *x_ref, const ddla_opts *opts,
                         ddla_solve_report *report);
/* ddla_dev_dgesv_mixed that also hands out the low-precision factor's pivots
 * (piv_out, device, n entries, DDLA's relative convention of LU.cs:367-374;
 * may be NULL) and compares them with piv_ref (device, n; may be NULL), for
 * instance the pivots of an FP64 ddla_dev_dgetrf of the same A: the report's
 * pivots_agree and pivots_first_diff say how far the FP32 factorization
 * followed the FP64 pivot sequence.  No DDLA counterpart (DDLA's
 * LU(A).Solve, LU.cs:64-100, is FP64-only). */
int ddla_dev_dgesv_mixed_piv(ddla_handle h, ddla_dim_t n, ddla_dim_t nrhs, const double *a, const double *b,
                             double *x, const double *x_ref, const int32_t *piv_ref, int32_t *piv_out,
                             const ddla_opts *opts, ddla_solve_report *report);

/* FP32 GEMM C = alpha*A*B + beta*C on device data in the precision the mixed
 * factorizations use for their trailing updates: DDLA_PREC_FP32 (CUDA-core
 * FFMA), DDLA_PREC_TF32X3 (tcgen05 tensor cores, 3xTF32 split products,
 * FP32 accumulation in TMEM) or DDLA_PREC_BF16X3 (tcgen05, two-part BF16
 * split, 3 products, FP32 accumulation; only the update shape beta = 1,
 * k <= 64, else DDLA_ERR_UNSUPPORTED).  No DDLA counterpart (DDLA is FP64
 * only). */
int ddla_dev_sgemm_tc(ddla_handle h, int32_t precision, int64_t m, int64_t n, int64_t k, float alpha, const float *a,
                      int64_t rsa, int64_t csa, const float *b, int64_t rsb, int64_t csb, float beta, float *c,
                      int64_t rsc, int64_t csc);

/* Allocation-free triangular solve (no counterpart in the reference; DDLA has
 * no GPU code).  Solves op(tri(A)) X = X in place for n <= DDLA_NOALLOC_MAX_N
 * and nrhs <= DDLA_NOALLOC_MAX_RHS, X row-major on the device with leading
 * dimension ldx, A a device view (rsa, csa), on `stream` (cudaStream_t cast to
 * void*; NULL = legacy default stream).  It is for callers that must not
 * allocate device memory -- for example a real-time loop that may not block
 * on cudaMalloc, or an application whose memory is owned by its own pool
 * allocator: every other device entry point grows a handle workspace on
 * first use, this one never calls cudaMalloc, cudaFree or any allocating
 * routine.  Its scratch (the inverted diagonal blocks and the block flags) is
 * one fixed 1 MiB + 256 B array in the library's device image, held by every
 * GPU that loads the library until the process exits.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress) and
 * should therefore come before any stream capture.  All calls share the one
 * array: calls whose work overlaps on the GPU (different streams, threads)
 * race and must be serialized by the caller.  Every call is synchronous: it
 * copies the solve's error word back to host memory and synchronizes `stream`
 * before it returns 0, a negative argument position, DDLA_ERR_TIMEOUT or
 * DDLA_ERR_CUDA. */
#define DDLA_NOALLOC_MAX_N 2048
#define DDLA_NOALLOC_MAX_RHS 16
int ddla_dev_dtrsv_noalloc(void *stream, int32_t uplo, int32_t trans, int32_t diag, int64_t n, int64_t nrhs,
                           const double *a, int64_t rsa, int64_t csa, double *x, int64_t ldx);

/* ------------------------------------------------ batched small factorizations */

/* Plan for `count` square row-major matrices of uneven size (1 <= n[i] <= 1024,
 * host array), each factored and solved with one right-hand side in ONE
 * persistent kernel launch captured into a CUDA graph (no DDLA counterpart:
 * DDLA factors one matrix per LU / Cholesky object).  kind[i]: 0 = LU with
 * partial pivoting (LU.PLUDecompose), 1 = LU without pivoting
 * (LU.LUDecompose), 2 = lower Cholesky (Cholesky.CholDecompose).
 * Device buffers, packed in item order: d_a holds the matrices back to back
 * (sum n^2 doubles; plain mode overwrites them with the factors), d_b / d_x /
 * d_piv the vectors (sum n each), d_info / d_iters one int per item (failing
 * pivot or 0; refinement steps or -1 when not converged).  mixed != 0 factors
 * in FP32 and refines in FP64 until the item's own FP64 backward-error
 * estimate is at most opts->tol / 2 (default tol 1e-14; the half leaves room
 * for a recomputation with another summation order). */
int ddla_batched_plan_create(ddla_handle h, int64_t count, const int32_t *n, const int32_t *kind, int32_t mixed,
                             double *d_a, const double *d_b, double *d_x, int32_t *d_piv, int32_t *d_info,
                             int32_t *d_iters, const ddla_opts *opts, void **plan);
/* Replay the plan's graph on the handle's stream (asynchronous). */
int ddla_batched_plan_exec(void *plan);
/* Algorithmic flops of one execution, persistent grid size, shared memory. */
int ddla_batched_plan_info(void *plan, double *flops, int32_t *grid, int64_t *smem_bytes);
int ddla_batched_plan_destroy(void *plan);

/* ------------------------------------------------ einsum (two operands) */

/* One mode of a contraction: length and element strides in A, B, C (0 when
 * the mode does not occur in that operand). */
typedef struct ddla_contract_mode {
    int64_t len, sa, sb, sc;
} ddla_contract_mode;

/* Lowered contraction: batch modes, then the M (A,C), N (B,C) and K (A,B)
 * mode lists after folding; `swapped` means the operand roles were exchanged
 * (A's strides are in `sb`).  Produced by ddla_contract_plan. */
typedef struct ddla_contract_desc {
    int32_t nbatch, nm, nn, nk, swapped, reserved;
    ddla_contract_mode batch[48];
    ddla_contract_mode m[16];
    ddla_contract_mode n[16];
    ddla_contract_mode k[16];
} ddla_contract_desc;

/* Index analysis of MArray.Contract(result, "ab,bc->ac", alpha, left, right)
 * (DDLA/Einsum/MArray.Contract.cs:48-125; IndiceUtils.Diagonal / Divide / Fold,
 * DDLA/Utilities/IndiceUtils.cs:18-245): ranks, lengths and element strides of
 * the three tensors. */
int ddla_contract_plan(const char *expr, int32_t rank_a, const int64_t *len_a, const int64_t *str_a, int32_t rank_b,
                       const int64_t *len_b, const int64_t *str_b, int32_t rank_c, const int64_t *len_c,
                       const int64_t *str_c, ddla_contract_desc *out);
/* C += alpha * contraction(A, B) on device data (MArray.Contract's
 * accumulating overload, MArray.Contract.cs:48-50).  precision: DDLA_PREC_FP64
 * (DMMA) or DDLA_PREC_OZAKI (FP64-accurate split BF16 tensor-core products). */
int ddla_dev_contract(ddla_handle h, const ddla_contract_desc *d, double alpha, const double *a, const double *b,
                      double *c, int32_t precision);
/* Same on host arrays: a/b/c point at the element with all indices 0 and
 * na/nb/nc are the element counts spanned by each tensor. */
int ddla_contract(const ddla_contract_desc *d, double alpha, const double *a, int64_t na, const double *b,
                  int64_t nb, double *c, int64_t nc, int32_t precision);

/* ------------------------------------------------ multi-operand einsum */

/* out = beta*out + alpha*einsum(expr, inputs) for any number of inputs
 * ("ab,bc,cd->ad").  MArray.Einsum (DDLA/Einsum/MArray.Contract.cs:409-427):
 * beta = 1 is Einsum(result, expr, alpha, inputs), beta = 0 the returning
 * form.  The pairwise order is DDLA's greedy path
 * (DDLA/Einsum/EinsumTree/EinsumState.cs:45-419); intermediates stay on the
 * device.  One input is contracted with the scalar 1 (transpose, diagonal,
 * sums), where DDLA returns the input unchanged (EinsumNodes.cs:97-100).
 * Tensor i has ranks[i] modes with lengths lens[i][.] and element strides
 * strides[i][.]; precision DDLA_PREC_FP64 or DDLA_PREC_OZAKI. */
int ddla_dev_einsum(ddla_handle h, const char *expr, int32_t n_inputs, const int32_t *ranks,
                    const int64_t *const *lens, const int64_t *const *strides, const double *const *inputs,
                    double alpha, double beta, int32_t rank_out, const int64_t *len_out, const int64_t *str_out,
                    double *out, int32_t precision);
/* Host arrays: counts[i] / out_count are the element spans from index 0. */
int ddla_einsum(const char *expr, int32_t n_inputs, const int32_t *ranks, const int64_t *const *lens,
                const int64_t *const *strides, const double *const *inputs, const int64_t *counts, double alpha,
                double beta, int32_t rank_out, const int64_t *len_out, const int64_t *str_out, double *out,
                int64_t out_count, int32_t precision);
/* The pairwise path, "ab,bc->ac;ac,cd->ad" (NUL-terminated, at most buflen
 * bytes). */
int ddla_einsum_path(const char *expr, int32_t n_inputs, const int32_t *ranks, const int64_t *const *lens, char *buf,
                     int32_t buflen);

#ifdef __cplusplus
}
#endif
#endif /* DDLA_GB300_H */
