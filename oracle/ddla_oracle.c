/*
 * ddla_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of DDLA's FP64 dense hot path, used as the parity oracle by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  It is
 * never linked into, loaded by, or called from the product library
 * (ddla_gb300/), which must fail loudly when its CUDA build is missing.
 *
 * Parity status: UNPINNED.  DDLA (C#/.NET) cannot be built or run here (no .NET
 * runtime; its micro-kernel needs x86 AVX2; its factorizations P/Invoke a
 * closed Windows BLIS DLL) and it ships no golden vectors.  This file is pinned
 * instead against (a) the property checks of DDLA's own tests at their sizes and
 * tolerances and (b) an independent LAPACK (scipy) on the same inputs -- see
 * tests/test_oracle.py.
 *
 * Every routine cites the reference file:line it restates (paths relative to
 * the DDLA repository root).  BLIS routines that DDLA delegates to (gemm, trsm,
 * syrk, ger, amaxv, scalv) follow BLIS's documented typed-API semantics, with
 * the blocking structure of DDLA's managed provider where one exists.
 *
 * Conventions: a matrix is (pointer to head element, rows, cols, row stride,
 * column stride) in elements, exactly like DDLA's MatrixView
 * (DDLA/Core/MatrixView.cs:22-31); transposition swaps rows/cols and strides
 * (DDLA/Core/MatrixView.cs:481).  Flag values are BLIS's
 * (DDLA/Misc/Flags/*.cs).  Status: 0 ok, >0 = 1-based index of the failing
 * pivot (DDLA throws LinalgException / ArgumentException there), <0 = bad
 * argument.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;

enum { TR_NO = 0, TR_T = 8 };            /* TransType  DDLA/Misc/Flags/TransType.cs:3-9 */
enum { UL_LOWER = 0xC0, UL_UPPER = 0x60, UL_DENSE = 0xE0 }; /* UpLo DDLA/Misc/Flags/UpLo.cs:3-9 */
enum { DG_NONUNIT = 0, DG_UNIT = 0x100 }; /* DiagType DDLA/Misc/Flags/DiagType.cs */
enum { SD_LEFT = 0, SD_RIGHT = 1 };        /* SideType DDLA/Misc/Flags/SideType.cs */

/* GEMMKernel blocking constants, DDLA/Einsum/GEMMKernel.cs:11-21 */
#define MC 510
#define NC 512
#define KC 144
#define MR 6
#define NR 8
#define KR 6
/* Block sizes of the factorizations: LU.cs:131,235, Cholesky.cs:125, LDLT.cs:139 */
#define NB 128

typedef struct { double *p; i64 r, c, rs, cs; } mat;

static inline double *AT(mat A, i64 i, i64 j) { return A.p + i * A.rs + j * A.cs; }
static inline mat mk(double *p, i64 r, i64 c, i64 rs, i64 cs) { mat m = {p, r, c, rs, cs}; return m; }
static inline mat tr(mat A) { mat m = {A.p, A.c, A.r, A.cs, A.rs}; return m; }
static inline mat sub(mat A, i64 i, i64 ni, i64 j, i64 nj) {
    mat m = {A.p + i * A.rs + j * A.cs, ni, nj, A.rs, A.cs}; return m;
}
static inline int flip_uplo(int u) { return u == UL_LOWER ? UL_UPPER : (u == UL_UPPER ? UL_LOWER : u); }
static inline i64 align_up(i64 x, i64 a) { return (x + a - 1) / a * a; }

static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_get_threads(void) { return g_threads; }
int orc_has_openmp(void) {
#ifdef _OPENMP
    return 1;
#else
    return 0;
#endif
}

/* ------------------------------------------------------------------------ */
/* Level-1/2 primitives                                                      */
/* ------------------------------------------------------------------------ */

/* Scal on a matrix (triangle): alpha==0 sets zero, alpha!=1 multiplies.
 * DDLA/BLAS/Managed/1m.cs:251-300, DDLA/BLAS/Managed/1v.cs:294-300. */
static void scal_m(int uplo, double alpha, mat A) {
    if (alpha == 1.0) return;
    for (i64 i = 0; i < A.r; i++) {
        i64 j0 = 0, j1 = A.c;
        if (uplo == UL_LOWER) j1 = i + 1 < A.c ? i + 1 : A.c;
        if (uplo == UL_UPPER) j0 = i;
        for (i64 j = j0; j < j1; j++) {
            double *x = AT(A, i, j);
            *x = (alpha == 0.0) ? 0.0 : *x * alpha;
        }
    }
}

/* bli_damaxv as documented by DDLA (DDLA/BLAS/1v.cs:29-42): index of the first
 * element of largest |x|; NaN compares smaller than every other value; an
 * empty vector gives 0. */
i64 orc_damax(i64 n, const double *x, i64 inc) {
    i64 best = 0;
    double bv = -1.0;
    for (i64 i = 0; i < n; i++) {
        double v = fabs(x[i * inc]);
        if (v > bv) { bv = v; best = i; }
    }
    return best;
}

static void swap_rows(mat A, i64 i, i64 j) {   /* MatrixView.SwapRow, Managed/1v.cs:324-328 */
    if (i == j) return;
    for (i64 c = 0; c < A.c; c++) { double t = *AT(A, i, c); *AT(A, i, c) = *AT(A, j, c); *AT(A, j, c) = t; }
}

/* A += alpha * x * y^T (bli_dger, DDLA/BLAS/2m.cs:35-49): column-wise axpy with
 * the scalar alpha*y[j], fused multiply-add. */
static void ger(double alpha, const double *x, i64 incx, const double *y, i64 incy, mat A) {
    for (i64 j = 0; j < A.c; j++) {
        double s = alpha * y[j * incy];
        for (i64 i = 0; i < A.r; i++) *AT(A, i, j) = fma(x[i * incx], s, *AT(A, i, j));
    }
}

/* Symmetric rank-1 on one triangle: A += alpha*x*x^T (managed SyR,
 * DDLA/BLAS/Managed/2m.cs:381-421: row i gets fma(x[j], alpha*x[i], A[i][j])). */
static void syr(int uplo, double alpha, const double *x, i64 incx, mat A) {
    for (i64 i = 0; i < A.r; i++) {
        double s = alpha * x[i * incx];
        i64 j0 = uplo == UL_LOWER ? 0 : i, j1 = uplo == UL_LOWER ? i + 1 : A.c;
        for (i64 j = j0; j < j1; j++) *AT(A, i, j) = fma(x[j * incx], s, *AT(A, i, j));
    }
}

/* x *= 1/alpha (InvScal: native DDLA/BLAS/1v.cs:97-103 rejects alpha==0; the
 * managed one DDLA/BLAS/Managed/1v.cs:283-292 also rejects non-finite alpha
 * and skips alpha==1).  Returns 0 or -1 when DDLA would throw. */
static int invscal(double alpha, double *x, i64 n, i64 inc, int managed) {
    if (alpha == 0.0) return -1;
    if (managed && !isfinite(alpha)) return -1;
    if (managed && alpha == 1.0) return 0;
    double s = 1.0 / alpha;
    for (i64 i = 0; i < n; i++) x[i * inc] *= s;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* GEMM: DDLA's managed BLIS-style 5-loop algorithm                          */
/* ------------------------------------------------------------------------ */

/* 6x8 micro-kernel, DDLA/Einsum/GEMMKernel.cs:36-233: for each k (ascending) one
 * fused multiply-add per output element into a fresh accumulator; output tile
 * stored row-major. */
static void micro(i64 kc, const double *a, const double *b, double *c) {
    double acc[MR][NR];
    for (int r = 0; r < MR; r++) for (int s = 0; s < NR; s++) acc[r][s] = 0.0;
    for (i64 k = 0; k < kc; k++) {
        const double *ak = a + k * MR, *bk = b + k * NR;
        for (int r = 0; r < MR; r++) {
            double av = ak[r];
            for (int s = 0; s < NR; s++) acc[r][s] = fma(av, bk[s], acc[r][s]);
        }
    }
    for (int r = 0; r < MR; r++) for (int s = 0; s < NR; s++) c[r * NR + s] = acc[r][s];
}

/* GEPack, DDLA/BLAS/Managed/3m/Packing.cs:30-101: panels of `blk` rows, each
 * stored [col][row] with zero padding of the ragged last panel. */
static void pack(mat S, double *buf, int blk) {
    i64 np = align_up(S.r, blk) / blk;
    /* a copy: splitting it over threads changes no arithmetic */
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1 && np >= 16)
#endif
    for (i64 pi = 0; pi < np; pi++) {
        double *dst = buf + pi * S.c * blk;
        i64 r0 = pi * blk, ar = S.r - r0 < blk ? S.r - r0 : blk;
        for (i64 col = 0; col < S.c; col++)
            for (int r = 0; r < blk; r++) *dst++ = r < ar ? *AT(S, r0 + r, col) : 0.0;
    }
}

/* Macro kernel, DDLA/BLAS/Managed/3m/MacroKernel.cs:69-96 (GEMM) and :147-216
 * (GEMMT masks).  tri: 0 = full tile add via fused axpy (Managed/1m.cs:86-158),
 * UL_LOWER/UL_UPPER = masked scalar add alpha*t + c (MacroKernel.cs:177-211). */
static void macro(i64 mc, i64 nc, i64 kc, double alpha, const double *bufA, const double *bufB,
                  mat C, int tri, i64 diag0) {
    i64 ip = align_up(mc, MR) / MR;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1 && ip >= 8)
#endif
    for (i64 i = 0; i < ip; i++) {
        double t[MR * NR];
        i64 amr = mc - i * MR < MR ? mc - i * MR : MR;
        for (i64 j = 0; j < align_up(nc, NR); j += NR) {
            i64 anr = nc - j < NR ? nc - j : NR;
            mat Ct = sub(C, i * MR, amr, j, anr);
            if (tri == 0) {
                micro(kc, bufA + i * kc * MR, bufB + j * kc, t);
                for (i64 r = 0; r < amr; r++)
                    for (i64 s = 0; s < anr; s++) *AT(Ct, r, s) = fma(t[r * NR + s], alpha, *AT(Ct, r, s));
            } else {
                i64 diag = diag0 + i * MR - j;
                if (tri == UL_UPPER && diag >= anr) continue;
                if (tri == UL_LOWER && diag <= -amr) continue;
                micro(kc, bufA + i * kc * MR, bufB + j * kc, t);
                for (i64 r = 0; r < amr; r++) {
                    i64 s0 = 0, s1 = anr;
                    if (tri == UL_UPPER) { s0 = r + diag; if (s0 > anr) s0 = anr; if (s0 < 0) s0 = 0; }
                    else { s1 = r + diag + 1; if (s1 < 0) s1 = 0; if (s1 > anr) s1 = anr; }
                    for (i64 s = s0; s < s1; s++) *AT(Ct, r, s) = alpha * t[r * NR + s] + *AT(Ct, r, s);
                }
            }
        }
    }
}

/* GeMMInner / GeMMT loops, DDLA/BLAS/Managed/3m/GeMM.cs:14-73 and
 * DDLA/BLAS/Managed/3m.cs:75-130.  C is already beta-scaled. */
static void gemm_core(double alpha, mat A, mat B, mat C, int tri) {
    i64 m = C.r, n = C.c, k = A.c;
    if (C.cs < C.rs) {              /* prefer row-major C: solve the transposed problem */
        mat T = A; A = tr(B); B = tr(T); C = tr(C);
        m = C.r; n = C.c;
        if (tri) tri = flip_uplo(tri);
    }
    if (m == 0 || n == 0 || k == 0) return;
    i64 mce = MC < align_up(m, MR) ? MC : align_up(m, MR);
    i64 nce = NC < align_up(n, NR) ? NC : align_up(n, NR);
    double *bufA = (double *)malloc(sizeof(double) * mce * KC);
    double *bufB = (double *)malloc(sizeof(double) * KC * nce);
    for (i64 ic = 0; ic < m; ic += MC) {
        i64 mc = m - ic < MC ? m - ic : MC;
        for (i64 pc = 0; pc < k; pc += KC) {
            i64 kc = k - pc < KC ? k - pc : KC;
            pack(sub(A, ic, mc, pc, kc), bufA, MR);
            for (i64 jc = 0; jc < n; jc += NC) {
                i64 nc = n - jc < NC ? n - jc : NC;
                pack(tr(sub(B, pc, kc, jc, nc)), bufB, NR);
                macro(mc, nc, kc, alpha, bufA, bufB, sub(C, ic, mc, jc, nc), tri, ic - jc);
            }
        }
    }
    free(bufA); free(bufB);
}

/* C = beta*C + alpha*op(A)*op(B); DDLA/BLAS/Managed/3m.cs:13-39 (beta first). */
void orc_dgemm(int ta, int tb, i64 m, i64 n, i64 k, double alpha,
               const double *a, i64 rsa, i64 csa, const double *b, i64 rsb, i64 csb,
               double beta, double *c, i64 rsc, i64 csc) {
    mat A = mk((double *)a, ta == TR_T ? k : m, ta == TR_T ? m : k, rsa, csa);
    mat B = mk((double *)b, tb == TR_T ? n : k, tb == TR_T ? k : n, rsb, csb);
    if (ta == TR_T) A = tr(A);
    if (tb == TR_T) B = tr(B);
    mat C = mk(c, m, n, rsc, csc);
    if (m == 0 || n == 0) return;
    scal_m(UL_DENSE, beta, C);
    if (k == 0) return;
    gemm_core(alpha, A, B, C, 0);
}

/* C(uplo triangle) = beta*C + alpha*op(A)*op(B); DDLA/BLAS/Managed/3m.cs:51-131. */
void orc_dgemmt(int uplo, int ta, int tb, i64 m, i64 k, double alpha,
                const double *a, i64 rsa, i64 csa, const double *b, i64 rsb, i64 csb,
                double beta, double *c, i64 rsc, i64 csc) {
    mat A = mk((double *)a, ta == TR_T ? k : m, ta == TR_T ? m : k, rsa, csa);
    mat B = mk((double *)b, tb == TR_T ? m : k, tb == TR_T ? k : m, rsb, csb);
    if (ta == TR_T) A = tr(A);
    if (tb == TR_T) B = tr(B);
    mat C = mk(c, m, m, rsc, csc);
    if (m == 0) return;
    scal_m(uplo, beta, C);
    if (k == 0) return;
    gemm_core(alpha, A, B, C, uplo);
}

/* SYRK as GEMMT(A, A^T), DDLA/BLAS/Managed/3m.cs:200-216. */
void orc_dsyrk(int uplo, int ta, i64 m, i64 k, double alpha, const double *a, i64 rsa, i64 csa,
               double beta, double *c, i64 rsc, i64 csc) {
    mat A = mk((double *)a, ta == TR_T ? k : m, ta == TR_T ? m : k, rsa, csa);
    if (ta == TR_T) A = tr(A);
    mat C = mk(c, m, m, rsc, csc);
    if (m == 0) return;
    scal_m(uplo, beta, C);
    if (k == 0) return;
    gemm_core(alpha, A, tr(A), C, uplo);
}

/* ------------------------------------------------------------------------ */
/* SYMM / SYR2K / TRMM / TRMM3                                               */
/* ------------------------------------------------------------------------ */

/* A structured operand as DDLA's packing sees it: kind 0 dense, 1 symmetric
 * (stored in `uplo`), 2 triangular (`uplo` nonzero triangle, `unit` implicit
 * unit diagonal). */
enum { SK_DENSE = 0, SK_SYM = 1, SK_TRI = 2 };
typedef struct { mat M; int kind, uplo, unit; } smat;

static smat sm(mat M, int kind, int uplo, int unit) { smat S = {M, kind, uplo, unit}; return S; }
static smat str_s(smat S) { S.M = tr(S.M); S.uplo = flip_uplo(S.uplo); return S; }

/* Element (i, j): SYPack mirrors the unstored triangle, TRPack reads zeros
 * outside the triangle and 1 on a unit diagonal
 * (DDLA/BLAS/Managed/3m/Packing.cs:172-197 and 282-340). */
static double sget(smat S, i64 i, i64 j) {
    int outside = S.uplo == UL_LOWER ? (j > i) : (j < i);
    if (S.kind == SK_SYM && outside) return *AT(S.M, j, i);
    if (S.kind == SK_TRI) {
        if (outside) return 0.0;
        if (i == j && S.unit) return 1.0;
    }
    return *AT(S.M, i, j);
}

/* pack(sub(S, i0, ni, j0, nj), buf, blk) for a structured operand. */
static void spack(smat S, i64 i0, i64 ni, i64 j0, i64 nj, double *buf, int blk) {
    i64 np = align_up(ni, blk) / blk;
    for (i64 pi = 0; pi < np; pi++) {
        double *dst = buf + pi * nj * blk;
        i64 r0 = pi * blk, ar = ni - r0 < blk ? ni - r0 : blk;
        for (i64 col = 0; col < nj; col++)
            for (int r = 0; r < blk; r++) *dst++ = r < ar ? sget(S, i0 + r0 + r, j0 + col) : 0.0;
    }
}

/* SyMMInner / TrMM3Inner, DDLA/BLAS/Managed/3m/SyMM.cs:13-71 and
 * TrMM3.cs:13-76: the GeMM loops with structured packing.  C is already
 * beta-scaled. */
static void gemm_core_s(double alpha, smat A, smat B, mat C) {
    i64 m = C.r, n = C.c, k = A.M.c;
    if (C.cs < C.rs) {
        smat T = A; A = str_s(B); B = str_s(T); C = tr(C);
        m = C.r; n = C.c;
    }
    if (m == 0 || n == 0 || k == 0) return;
    i64 mce = MC < align_up(m, MR) ? MC : align_up(m, MR);
    i64 nce = NC < align_up(n, NR) ? NC : align_up(n, NR);
    double *bufA = (double *)malloc(sizeof(double) * mce * KC);
    double *bufB = (double *)malloc(sizeof(double) * KC * nce);
    smat Bt = str_s(B);
    for (i64 ic = 0; ic < m; ic += MC) {
        i64 mc = m - ic < MC ? m - ic : MC;
        for (i64 pc = 0; pc < k; pc += KC) {
            i64 kc = k - pc < KC ? k - pc : KC;
            spack(A, ic, mc, pc, kc, bufA, MR);
            for (i64 jc = 0; jc < n; jc += NC) {
                i64 nc = n - jc < NC ? n - jc : NC;
                spack(Bt, jc, nc, pc, kc, bufB, NR);
                macro(mc, nc, kc, alpha, bufA, bufB, sub(C, ic, mc, jc, nc), 0, 0);
            }
        }
    }
    free(bufA); free(bufB);
}

static mat opm(const double *p, i64 r, i64 c, i64 rs, i64 cs, int t) {
    return t == TR_T ? tr(mk((double *)p, c, r, rs, cs)) : mk((double *)p, r, c, rs, cs);
}

/* bli_dsymm semantics (DDLA/BLAS/3m.cs:83-106; managed DDLA/BLAS/Managed/3m.cs:
 * 144-188): C = beta*C + alpha*A*op(B) (left) / alpha*op(B)*A (right), A
 * symmetric in its `uplo` triangle. */
void orc_dsymm(int side, int uplo, int conja, int tb, i64 m, i64 n, double alpha,
               const double *a, i64 rsa, i64 csa, const double *b, i64 rsb, i64 csb,
               double beta, double *c, i64 rsc, i64 csc) {
    (void)conja;
    i64 na = side == SD_LEFT ? m : n;
    smat A = sm(mk((double *)a, na, na, rsa, csa), SK_SYM, uplo, 0);
    smat B = sm(opm(b, m, n, rsb, csb, tb), SK_DENSE, UL_DENSE, 0);
    mat C = mk(c, m, n, rsc, csc);
    if (m == 0 || n == 0) return;
    scal_m(UL_DENSE, beta, C);
    if (side == SD_LEFT) gemm_core_s(alpha, A, B, C);
    else gemm_core_s(alpha, B, A, C);
}

/* bli_dsyr2k semantics (DDLA/BLAS/3m.cs:149-172): two triangle-only GEMMs as
 * DDLA/BLAS/Managed/3m.cs:227-246 does. */
void orc_dsyr2k(int uplo, int ta, int tb, i64 m, i64 k, double alpha,
                const double *a, i64 rsa, i64 csa, const double *b, i64 rsb, i64 csb,
                double beta, double *c, i64 rsc, i64 csc) {
    mat A = opm(a, m, k, rsa, csa, ta), B = opm(b, m, k, rsb, csb, tb);
    mat C = mk(c, m, m, rsc, csc);
    if (m == 0) return;
    scal_m(uplo, beta, C);
    if (k == 0) return;
    gemm_core(alpha, A, tr(B), C, uplo);
    gemm_core(alpha, B, tr(A), C, uplo);
}

/* bli_dtrmm3 semantics (DDLA/BLAS/3m.cs:225-250; managed
 * DDLA/BLAS/Managed/3m.cs:308-356): C = beta*C + alpha*op(A)*op(B) (left) or
 * alpha*op(B)*op(A) (right), A triangular. */
void orc_dtrmm3(int side, int uplo, int ta, int diag, int tb, i64 m, i64 n, double alpha,
                const double *a, i64 rsa, i64 csa, const double *b, i64 rsb, i64 csb,
                double beta, double *c, i64 rsc, i64 csc) {
    i64 na = side == SD_LEFT ? m : n;
    smat A = sm(mk((double *)a, na, na, rsa, csa), SK_TRI, uplo, diag == DG_UNIT);
    if (ta == TR_T) A = str_s(A);
    smat B = sm(opm(b, m, n, rsb, csb, tb), SK_DENSE, UL_DENSE, 0);
    mat C = mk(c, m, n, rsc, csc);
    if (m == 0 || n == 0) return;
    scal_m(UL_DENSE, beta, C);
    if (side == SD_LEFT) gemm_core_s(alpha, A, B, C);
    else gemm_core_s(alpha, B, A, C);
}

/* bli_dtrmm semantics (DDLA/BLAS/3m.cs:185-204): B = alpha*op(A)*B (left) or
 * alpha*B*op(A) (right) in place.  DDLA's managed TrMM
 * (DDLA/BLAS/Managed/3m/TrMM.cs:14-207) walks KC blocks with a TrMV per
 * column of the diagonal block; this restatement forms the same product with
 * the structured GEMM of TRMM3 from a copy of B, so the two agree to rounding. */
void orc_dtrmm(int side, int uplo, int ta, int diag, i64 m, i64 n, double alpha,
               const double *a, i64 rsa, i64 csa, double *b, i64 rsb, i64 csb) {
    if (m == 0 || n == 0) return;
    double *t = (double *)malloc(sizeof(double) * m * n);
    for (i64 i = 0; i < m; i++)
        for (i64 j = 0; j < n; j++) t[i * n + j] = b[i * rsb + j * csb];
    orc_dtrmm3(side, uplo, ta, diag, TR_NO, m, n, alpha, a, rsa, csa, t, n, 1, 0.0, b, rsb, csb);
    free(t);
}

/* ------------------------------------------------------------------------ */
/* TRSM / TRSV                                                              */
/* ------------------------------------------------------------------------ */

/* Triangular solve with one vector, column-oriented (DDLA/BLAS/Managed/2m.cs:625-865). */
static void trsv(int uplo, int unit, mat A, double *x, i64 inc) {
    i64 n = A.r;
    if (uplo == UL_LOWER) {
        for (i64 j = 0; j < n; j++) {
            if (!unit) x[j * inc] /= *AT(A, j, j);
            double xj = -x[j * inc];
            for (i64 i = j + 1; i < n; i++) x[i * inc] = fma(*AT(A, i, j), xj, x[i * inc]);
        }
    } else {
        for (i64 j = n - 1; j >= 0; j--) {
            if (!unit) x[j * inc] /= *AT(A, j, j);
            double xj = -x[j * inc];
            for (i64 i = 0; i < j; i++) x[i * inc] = fma(*AT(A, i, j), xj, x[i * inc]);
        }
    }
}

/* Left solve tri(A)*X = B in KC-row blocks: GEMM update of the block from the
 * solved part, then a TRSV per column (DDLA/BLAS/Managed/3m/TrSM.cs:62-122). */
static void trsm_left(int uplo, int unit, mat A, mat B) {
    i64 m = B.r;
    if (uplo == UL_LOWER) {
        for (i64 i0 = 0; i0 < m; i0 += KC) {
            i64 b = m - i0 < KC ? m - i0 : KC;
            if (i0 > 0) gemm_core(-1.0, sub(A, i0, b, 0, i0), sub(B, 0, i0, 0, B.c), sub(B, i0, b, 0, B.c), 0);
            mat A11 = sub(A, i0, b, i0, b);
            /* the column solves are independent of one another */
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1 && B.c >= 64)
#endif
            for (i64 j = 0; j < B.c; j++) trsv(UL_LOWER, unit, A11, AT(B, i0, j), B.rs);
        }
    } else {
        for (i64 i1 = m; i1 > 0; i1 -= KC) {
            i64 b = i1 < KC ? i1 : KC, i0 = i1 - b;
            if (i1 < m) gemm_core(-1.0, sub(A, i0, b, i1, m - i1), sub(B, i1, m - i1, 0, B.c), sub(B, i0, b, 0, B.c), 0);
            mat A11 = sub(A, i0, b, i0, b);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1 && B.c >= 64)
#endif
            for (i64 j = 0; j < B.c; j++) trsv(UL_UPPER, unit, A11, AT(B, i0, j), B.rs);
        }
    }
}

/* bli_dtrsm semantics (DDLA/BLAS/3m.cs:276-305): Left solves op(A)*X = alpha*B,
 * Right solves X*op(A) = alpha*B, B overwritten.  alpha is applied first
 * (DDLA/BLAS/Managed/3m.cs:434).  A right solve is the left solve of the
 * transposed system. */
void orc_dtrsm(int side, int uplo, int ta, int diag, i64 m, i64 n, double alpha,
               const double *a, i64 rsa, i64 csa, double *b, i64 rsb, i64 csb) {
    i64 na = side == SD_LEFT ? m : n;
    mat A = mk((double *)a, na, na, rsa, csa);
    mat B = mk(b, m, n, rsb, csb);
    if (m == 0 || n == 0) return;
    scal_m(UL_DENSE, alpha, B);
    if (ta == TR_T) { A = tr(A); uplo = flip_uplo(uplo); }
    if (side == SD_RIGHT) { A = tr(A); uplo = flip_uplo(uplo); B = tr(B); }
    trsm_left(uplo, diag == DG_UNIT, A, B);
}

/* ------------------------------------------------------------------------ */
/* Householder QR, DDLA/Factorizations/QR.cs (UT transform, as libflame)     */
/* ------------------------------------------------------------------------ */

#define QR_BLOCKED_ABOVE 256   /* QR.BlockSize, QR.cs:16; blocked iff n > 256 (QR.cs:139-149) */

/* Vector 2-norm (NrmF of a vector, bli_dnormfv): plain sum of squares. */
static double nrm2(const double *x, i64 n, i64 inc) {
    double s = 0.0;
    for (i64 i = 0; i < n; i++) s = fma(x[i * inc], x[i * inc], s);
    return sqrt(s);
}

/* BuildHouseHolder, DDLA/Transformations/HouseHolder.cs:34-58: chi <- rho,
 * x <- u2 = x / (chi - rho), tau = (1 + |u2|^2) / 2; an all-zero x gives the
 * reflection chi <- -chi with tau = 1/2. */
static void house_build(double *chi, double *x, i64 n, i64 inc, double *tau) {
    double len = nrm2(x, n, inc);
    if (len == 0.0) { *chi = -*chi; *tau = 0.5; return; }
    double alpha = hypot(*chi, len);
    double rho = -copysign(alpha, *chi);
    double miu = *chi - rho;
    *chi = rho;
    double s = 1.0 / miu;                   /* InvScal = scal by 1/alpha, BLAS/1v.cs:97-103 */
    for (i64 i = 0; i < n; i++) x[i * inc] *= s;
    double sc = len / fabs(miu);
    *tau = (1.0 + sc * sc) / 2.0;
}

/* ApplyHouseHolder(Left), HouseHolder.cs:95-115: w = a1 + A2^T u2, w /= tau,
 * a1 -= w, A2 -= u2 w^T.  a1 is a 1 x c row, A2 n x c, u2 n long. */
static void house_apply_left(double tau, const double *u2, i64 incu, mat a1, mat A2) {
    i64 c = a1.c;
    if (c == 0 || tau == 0.0) return;
    double *w = (double *)malloc(sizeof(double) * c);
    for (i64 j = 0; j < c; j++) w[j] = *AT(a1, 0, j);
    for (i64 j = 0; j < c; j++)
        for (i64 i = 0; i < A2.r; i++) w[j] = fma(*AT(A2, i, j), u2[i * incu], w[j]);
    double s = 1.0 / tau;
    for (i64 j = 0; j < c; j++) { w[j] *= s; *AT(a1, 0, j) -= w[j]; }
    for (i64 i = 0; i < A2.r; i++) {
        double ui = -u2[i * incu];
        for (i64 j = 0; j < c; j++) *AT(A2, i, j) = fma(ui, w[j], *AT(A2, i, j));
    }
    free(w);
}

/* QRDecUnblock, QR.cs:314-350: one reflector per column; T(i, i) = tau_i and
 * T(0:i, i) = A(i, 0:i)^T + A(i+1:, 0:i)^T A(i+1:, i) = u_j^T u_i. */
static void qr_unblock(mat A, mat T) {
    i64 m = A.r, n = A.c, k = m < n ? m : n;
    for (i64 i = 0; i < k; i++) {
        double *tau = AT(T, i, i);
        house_build(AT(A, i, i), AT(A, i + 1 < m ? i + 1 : i, i), m - i - 1, A.rs, tau);
        house_apply_left(*tau, AT(A, i + 1 < m ? i + 1 : i, i), A.rs, sub(A, i, 1, i + 1, n - i - 1),
                         sub(A, i + 1, m - i - 1, i + 1, n - i - 1));
        for (i64 j = 0; j < i; j++) {
            double t = *AT(A, i, j);
            for (i64 r = i + 1; r < m; r++) t = fma(*AT(A, r, j), *AT(A, r, i), t);
            *AT(T, j, i) = t;
        }
    }
}

/* One block of ApplyQlhfc (QR.cs:417-467, trans) or ApplyQlnfc (QR.cs:469-533):
 * W = B1 (copy); W = A11^T W; W += A21^T B2; W = S^-T W (trans) or S^-1 W;
 * B2 -= A21 W; W = -A11 W; B1 += W.  A11 unit lower (b x b), A21 below it. */
static void qr_apply_one(int trans, mat A11, mat A21, mat S, mat B1, mat B2) {
    i64 b = A11.r, c = B1.c;
    if (c == 0) return;
    double *w = (double *)malloc(sizeof(double) * b * c);
    mat W = mk(w, b, c, c, 1);
    for (i64 i = 0; i < b; i++) for (i64 j = 0; j < c; j++) *AT(W, i, j) = *AT(B1, i, j);
    orc_dtrmm(SD_LEFT, UL_LOWER, TR_T, DG_UNIT, b, c, 1.0, A11.p, A11.rs, A11.cs, w, c, 1);
    if (A21.r > 0) gemm_core(1.0, tr(A21), B2, W, 0);
    orc_dtrsm(SD_LEFT, UL_UPPER, trans ? TR_T : TR_NO, DG_NONUNIT, b, c, 1.0, S.p, S.rs, S.cs, w, c, 1);
    if (A21.r > 0) gemm_core(-1.0, A21, W, B2, 0);
    orc_dtrmm(SD_LEFT, UL_LOWER, TR_NO, DG_UNIT, b, c, -1.0, A11.p, A11.rs, A11.cs, w, c, 1);
    for (i64 i = 0; i < b; i++) for (i64 j = 0; j < c; j++) *AT(B1, i, j) += *AT(W, i, j);
    free(w);
}

/* Q^T B (trans, blocks first to last) or Q B (last to first); blocks of T.r
 * columns over the k = min(m, n) reflectors.  ApplyQlnfc (QR.cs:479-503) sizes
 * its first (= last) block by T.Cols % block, which is the same partition when
 * m >= n; this follows the forward partition in both directions. */
static void qr_apply(int trans, mat A, mat T, mat B) {
    i64 m = A.r, k = A.r < A.c ? A.r : A.c, tb = T.r;
    i64 nblk = (k + tb - 1) / tb;
    for (i64 bi = 0; bi < nblk; bi++) {
        i64 blk = trans ? bi : nblk - 1 - bi;
        i64 j0 = blk * tb, b = k - j0 < tb ? k - j0 : tb;
        qr_apply_one(trans, sub(A, j0, b, j0, b), sub(A, j0 + b, m - j0 - b, j0, b), sub(T, 0, b, j0, b),
                     sub(B, j0, b, 0, B.c), sub(B, j0 + b, m - j0 - b, 0, B.c));
    }
}

/* QR.QRDecompose(A, T) (QR.cs:139-149): unblocked (QR.cs:314-350) when
 * n <= 256, else QRDecBlock (QR.cs:352-389) in blocks of T.Rows columns, each
 * factored unblocked and applied to the columns on its right with
 * ApplyQlhfc.  Returns -7 if T is too short for the unblocked form. */
int orc_dgeqrf(i64 m, i64 n, double *a, i64 rsa, i64 csa, double *t, i64 t_rows, i64 rst, i64 cst) {
    mat A = mk(a, m, n, rsa, csa), T = mk(t, t_rows, n, rst, cst);
    i64 k = m < n ? m : n;
    if (k == 0) return 0;
    if (n <= QR_BLOCKED_ABOVE) {
        if (t_rows < k) return -7;
        qr_unblock(A, T);
        return 0;
    }
    for (i64 j0 = 0; j0 < k; j0 += t_rows) {
        i64 b = k - j0 < t_rows ? k - j0 : t_rows;
        mat Ab1 = sub(A, j0, m - j0, j0, b), S = sub(T, 0, b, j0, b);
        qr_unblock(Ab1, S);
        if (j0 + b < n)
            qr_apply_one(1, sub(A, j0, b, j0, b), sub(A, j0 + b, m - j0 - b, j0, b), S,
                         sub(A, j0, b, j0 + b, n - j0 - b), sub(A, j0 + b, m - j0 - b, j0 + b, n - j0 - b));
    }
    return 0;
}

/* ApplyQT / ApplyQ (QR.cs:79-109): B (m x nrhs) = Q^T B or Q B. */
void orc_dormqr(int trans, i64 m, i64 n, i64 nrhs, const double *a, i64 rsa, i64 csa, const double *t, i64 t_rows,
                i64 rst, i64 cst, double *b, i64 rsb, i64 csb) {
    if (m == 0 || n == 0 || nrhs == 0) return;
    qr_apply(trans != 0, mk((double *)a, m, n, rsa, csa), mk((double *)t, t_rows, n, rst, cst),
             mk(b, m, nrhs, rsb, csb));
}

/* QR.Solve (QR.cs:391-415): Y = Q^T B, then R X = Y(0:n). */
void orc_dgeqrs(i64 m, i64 n, i64 nrhs, const double *a, i64 rsa, i64 csa, const double *t, i64 t_rows, i64 rst,
                i64 cst, const double *b, i64 rsb, i64 csb, double *x, i64 rsx, i64 csx) {
    if (n == 0 || nrhs == 0) return;
    double *y = (double *)malloc(sizeof(double) * m * nrhs);
    for (i64 i = 0; i < m; i++) for (i64 j = 0; j < nrhs; j++) y[i * nrhs + j] = b[i * rsb + j * csb];
    qr_apply(1, mk((double *)a, m, n, rsa, csa), mk((double *)t, t_rows, n, rst, cst), mk(y, m, nrhs, nrhs, 1));
    orc_dtrsm(SD_LEFT, UL_UPPER, TR_NO, DG_NONUNIT, n, nrhs, 1.0, a, rsa, csa, y, nrhs, 1);
    for (i64 i = 0; i < n; i++) for (i64 j = 0; j < nrhs; j++) x[i * rsx + j * csx] = y[i * nrhs + j];
    free(y);
}

/* QR.FormQ(A, T, Q) (QR.cs:192-201): Q = I, then Q = H_0 ... H_{k-1} Q. */
void orc_dorgqr(i64 m, i64 n, const double *a, i64 rsa, i64 csa, const double *t, i64 t_rows, i64 rst, i64 cst,
                double *q, i64 rsq, i64 csq) {
    for (i64 i = 0; i < m; i++) for (i64 j = 0; j < m; j++) q[i * rsq + j * csq] = i == j ? 1.0 : 0.0;
    orc_dormqr(0, m, n, m, a, rsa, csa, t, t_rows, rst, cst, q, rsq, csq);
}

/* ------------------------------------------------------------------------ */
/* Tridiagonal reduction, DDLA/Transformations/Tridiagonaling.cs             */
/* ------------------------------------------------------------------------ */

/* BuildHH, Tridiagonaling.cs:205-230: x(0) <- 1, x(1:) <- x(1:)/(chi - sigma)
 * with sigma = sign(chi) |x|, tau = (1 + |u(1:)|^2) / 2; a zero tail gives
 * sigma = -chi, tau = 1/2. */
static void trd_build(double *x, i64 n, i64 inc, double *sigma, double *tau) {
    double chi = x[0];
    double len = nrm2(x + inc, n - 1, inc);
    if (len == 0.0) { *sigma = -chi; x[0] = 1.0; *tau = 0.5; return; }
    double lenx = hypot(chi, len);
    *sigma = copysign(lenx, chi);
    double inv = 1.0 / (chi - *sigma);
    x[0] = 1.0;
    for (i64 i = 1; i < n; i++) x[i * inc] *= inv;
    len *= inv;
    *tau = (1.0 + len * len) / 2.0;
}

/* Tridiag(A, T, d, e), Tridiagonaling.cs:33-56 with Step (:72-112) and FormQ
 * (:122-203): one Householder reflector per column from the lower triangle
 * (SyMV, then the symmetric rank-2 update of the trailing matrix), T holding
 * the block factors per block of t_rows columns; A is then overwritten by Q
 * (Q^T A Q = tridiag(d, e)).  FormQ shifts the vectors one column right and
 * accumulates Q' = H_0 ... H_{n-2} on the trailing (n-1) x (n-1) identity;
 * here that product is formed with the blocked ApplyQlnfc of the QR. */
int orc_dsytrd(i64 n, double *a, i64 rsa, i64 csa, double *t, i64 t_rows, i64 rst, i64 cst, double *d, double *e) {
    mat A = mk(a, n, n, rsa, csa), T = mk(t, t_rows, n, rst, cst);
    if (n == 0) return 0;
    double *p = (double *)malloc(sizeof(double) * (size_t)n);
    for (i64 index = 0; index < n; index += t_rows) {
        i64 block = n - index < t_rows ? n - index : t_rows;
        for (i64 il = 0; il < block; il++) {
            i64 i = index + il;
            d[i] = *AT(A, i, i);
            if (i >= n - 1) continue;
            i64 m = n - i - 1;
            double *x = AT(A, i + 1, i);
            double sigma, tau;
            trd_build(x, m, A.rs, &sigma, &tau);
            *AT(T, il, i) = tau;
            /* p = A22 x (lower storage), Managed SyMV */
            for (i64 r = 0; r < m; r++) p[r] = 0.0;
            for (i64 r = 0; r < m; r++) {
                for (i64 c = 0; c <= r; c++) {
                    double v = *AT(A, i + 1 + r, i + 1 + c);
                    p[r] = fma(v, x[c * A.rs], p[r]);
                    if (c != r) p[c] = fma(v, x[r * A.rs], p[c]);
                }
            }
            double dot = 0.0;
            for (i64 r = 0; r < m; r++) dot = fma(x[r * A.rs], p[r], dot);
            double beta = dot / (2.0 * tau);
            double s = 1.0 / tau;
            for (i64 r = 0; r < m; r++) p[r] = (p[r] - beta * x[r * A.rs]) * s;
            /* A22 -= x p^T + p x^T on the lower triangle (Rank2, alpha = -1) */
            for (i64 r = 0; r < m; r++)
                for (i64 c = 0; c <= r; c++) {
                    double *v = AT(A, i + 1 + r, i + 1 + c);
                    *v = *v - (x[r * A.rs] * p[c] + p[r] * x[c * A.rs]);
                }
            /* t01 = A20^T x over this block's earlier columns */
            for (i64 j = 0; j < il; j++) {
                double acc = 0.0;
                for (i64 r = 0; r < m; r++) acc = fma(*AT(A, i + 1 + r, index + j), x[r * A.rs], acc);
                *AT(T, j, i) = acc;
            }
            x[0] = sigma;
            e[i] = sigma;
        }
    }
    free(p);
    /* FormQ */
    for (i64 j = n - 2; j > 0; j--)
        for (i64 r = j + 1; r < n; r++) *AT(A, r, j) = *AT(A, r, j - 1);
    if (n > 1) {
        i64 m = n - 1;
        double *q = (double *)malloc(sizeof(double) * (size_t)(m * m));
        mat Ap = sub(A, 1, m, 1, m), Tp = sub(T, 0, t_rows, 0, m);
        for (i64 r = 0; r < m; r++) for (i64 c = 0; c < m; c++) q[r * m + c] = r == c ? 1.0 : 0.0;
        qr_apply(0, Ap, Tp, mk(q, m, m, m, 1));
        for (i64 r = 0; r < m; r++) for (i64 c = 0; c < m; c++) *AT(Ap, r, c) = q[r * m + c];
        free(q);
    }
    for (i64 k = 0; k < n; k++) { *AT(A, 0, k) = k == 0 ? 1.0 : 0.0; *AT(A, k, 0) = k == 0 ? 1.0 : 0.0; }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* One-stage bidiagonal reduction, DDLA/Transformations/Bidiagonaling.cs     */
/* ------------------------------------------------------------------------ */

#define BD_BLOCK 128   /* Bidiagonaling.BlockSize, :62 */

/* Bidiag2(A, U, V, d, e), Bidiagonaling.cs:48-60: HHStepBlock (:64-123) and
 * BuildUV (:125-143) for m >= n.  Per column g: the column reflector (BuildHH
 * of Tridiagonaling, u(g) = 1 kept in A), d(g) = sigma, A(g:, g+1:) -= u
 * (u^T A(g:, g+1:)) / tau, TU(0:j, g) = A(g, j) + A(g+1:, j)^T u(g+1:) over the
 * block's earlier columns; then (except for the last column) the row
 * reflector of A(g, g+1:), e(g) = sigma, A(g+1:, g+1:) -= (A v) v^T / tau and
 * TV(0:j, g) likewise from the rows above.  U (m x m) and V (n x n) start as
 * the identity and receive the block reflectors (ApplyQ, :159-182: backward
 * blocks, the first one T.Cols % block wide, which the QR's partition matches
 * when it divides evenly and is otherwise the same product). */
int orc_dbidiag(i64 m, i64 n, double *a, i64 rsa, i64 csa, double *tu, i64 tu_rows, double *tv, i64 tv_rows,
                double *d, double *e, double *u, i64 rsu, i64 csu, double *v, i64 rsv, i64 csv) {
    if (m < n) return -1;
    mat A = mk(a, m, n, rsa, csa);
    mat TU = mk(tu, tu_rows, n, n, 1), TV = mk(tv, tv_rows, n, n, 1);
    if (n == 0) return 0;
    double *buf = (double *)malloc(sizeof(double) * (size_t)(m > n ? m : n));
    for (i64 bs = 0; bs < n; bs += BD_BLOCK) {
        i64 block = n - bs < BD_BLOCK ? n - bs : BD_BLOCK;
        i64 be = bs + block;
        for (i64 il = 0; il < block; il++) {
            i64 g = bs + il;
            double tau, sig;
            /* column reflector */
            trd_build(AT(A, g, g), m - g, A.rs, &sig, &tau);
            d[g] = sig;
            *AT(TU, il, g) = tau;
            i64 nr = n - g - 1;
            for (i64 c = 0; c < nr; c++) {
                double acc = 0.0;
                for (i64 r = g; r < m; r++) acc = fma(*AT(A, r, g), *AT(A, r, g + 1 + c), acc);
                buf[c] = acc * (1.0 / tau);
            }
            for (i64 r = g; r < m; r++) {
                double ur = -*AT(A, r, g);
                for (i64 c = 0; c < nr; c++) *AT(A, r, g + 1 + c) = fma(ur, buf[c], *AT(A, r, g + 1 + c));
            }
            for (i64 j = 0; j < il; j++) {
                double acc = *AT(A, g, bs + j);
                for (i64 r = g + 1; r < m; r++) acc = fma(*AT(A, r, bs + j), *AT(A, r, g), acc);
                *AT(TU, j, g) = acc;
            }
            /* row reflector (Bidiagonaling.cs:92-119) */
            if ((g < n - 1 && il < block - 1) || be < n) {
                trd_build(AT(A, g, g + 1), nr, A.cs, &sig, &tau);
                e[g] = sig;
                *AT(TV, il, g) = tau;
                i64 mr = m - g - 1;
                for (i64 r = 0; r < mr; r++) {
                    double acc = 0.0;
                    for (i64 c = 0; c < nr; c++) acc = fma(*AT(A, g + 1 + r, g + 1 + c), *AT(A, g, g + 1 + c), acc);
                    buf[r] = acc * (1.0 / tau);
                }
                for (i64 r = 0; r < mr; r++) {
                    double br = -buf[r];
                    for (i64 c = 0; c < nr; c++)
                        *AT(A, g + 1 + r, g + 1 + c) = fma(br, *AT(A, g, g + 1 + c), *AT(A, g + 1 + r, g + 1 + c));
                }
                for (i64 j = 0; j < il; j++) {
                    double acc = *AT(A, bs + j, g + 1);
                    for (i64 c = g + 2; c < n; c++) acc = fma(*AT(A, bs + j, c), *AT(A, g, c), acc);
                    *AT(TV, j, g) = acc;
                }
            }
        }
    }
    free(buf);
    /* BuildUV: U = H_0 ... H_{n-1} I, V = [1, 0; 0, G_0 ... G_{n-2} I] */
    mat U = mk(u, m, m, rsu, csu), V = mk(v, n, n, rsv, csv);
    for (i64 r = 0; r < m; r++) for (i64 c = 0; c < m; c++) *AT(U, r, c) = r == c ? 1.0 : 0.0;
    for (i64 r = 0; r < n; r++) for (i64 c = 0; c < n; c++) *AT(V, r, c) = r == c ? 1.0 : 0.0;
    qr_apply(0, A, TU, U);
    if (n > 1) qr_apply(0, tr(sub(A, 0, n - 1, 1, n - 1)), sub(TV, 0, tv_rows, 0, n - 1), sub(V, 1, n - 1, 0, n));
    return 0;
}

/* ------------------------------------------------------------------------ */
/* LU with partial pivoting, DDLA/Factorizations/LU.cs                      */
/* ------------------------------------------------------------------------ */

/* PLUDecUnblock, LU.cs:344-374: per column AMax (relative pivot), swap whole
 * panel rows, InvScal (native: throws on 0), GeR(-1).  `row0` is the global
 * index of the panel's first row for the status code. */
static int plu_unblock(mat A, int *piv, i64 row0) {
    i64 len = A.r < A.c ? A.r : A.c;
    for (i64 i = 0; i < len; i++) {
        i64 ip = orc_damax(A.r - i, AT(A, i, i), A.rs);
        piv[i] = (int)ip;
        if (ip != 0) swap_rows(sub(A, i, A.r - i, 0, A.c), 0, ip);
        double a11 = *AT(A, i, i);
        if (invscal(a11, AT(A, i + 1, i), A.r - i - 1, A.rs, 0)) return (int)(row0 + i + 1);
        ger(-1.0, AT(A, i + 1, i), A.rs, AT(A, i, i + 1), A.cs, sub(A, i + 1, A.r - i - 1, i + 1, A.c - i - 1));
    }
    return 0;
}

/* ApplyPivInternel (Left), LU.cs:376-404: forward applies swaps i <-> i+p[i]
 * in increasing i, backward in decreasing i. */
static void apply_piv(mat X, const int *piv, i64 np, int forward) {
    if (X.r == 0 || X.c == 0) return;
    /* every column sees the swaps in the same order, so column strips are
     * independent */
    const i64 strip = 256, ns = (X.c + strip - 1) / strip;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1 && ns >= 4)
#endif
    for (i64 t = 0; t < ns; t++) {
        mat S = sub(X, 0, X.r, t * strip, X.c - t * strip < strip ? X.c - t * strip : strip);
        if (forward) { for (i64 i = 0; i < np; i++) if (piv[i] > 0) swap_rows(S, i, i + piv[i]); }
        else { for (i64 i = np - 1; i >= 0; i--) if (piv[i] > 0) swap_rows(S, i, i + piv[i]); }
    }
}

/* PLUDecompose / PLUDecBlock, LU.cs:251-264, 289-342 (blocked iff n >= 128). */
int orc_dgetrf(i64 n, double *a, i64 rs, i64 cs, int *piv) {
    mat A = mk(a, n, n, rs, cs);
    if (n < NB) return plu_unblock(A, piv, 0);
    for (i64 j0 = 0; j0 < n; j0 += NB) {
        i64 b = n - j0 < NB ? n - j0 : NB;
        int info = plu_unblock(sub(A, j0, n - j0, j0, b), piv + j0, j0);
        if (info) return info;
        apply_piv(sub(A, j0, n - j0, 0, j0), piv + j0, b, 1);
        apply_piv(sub(A, j0, n - j0, j0 + b, n - j0 - b), piv + j0, b, 1);
        i64 r = n - j0 - b;
        if (r > 0) {
            mat A11 = sub(A, j0, b, j0, b), A12 = sub(A, j0, b, j0 + b, r);
            trsm_left(UL_LOWER, 1, A11, A12);
            gemm_core(-1.0, sub(A, j0 + b, r, j0, b), A12, sub(A, j0 + b, r, j0 + b, r), 0);
        }
    }
    return 0;
}

/* PLUSolveInternel, LU.cs:431-465. */
void orc_dgetrs(int trans, i64 n, i64 nrhs, const double *a, i64 rs, i64 cs, const int *piv,
                double *b, i64 rsb, i64 csb) {
    if (n == 0 || nrhs == 0) return;
    mat B = mk(b, n, nrhs, rsb, csb);
    if (!trans) {
        apply_piv(B, piv, n, 1);
        orc_dtrsm(SD_LEFT, UL_LOWER, TR_NO, DG_UNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
        orc_dtrsm(SD_LEFT, UL_UPPER, TR_NO, DG_NONUNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
    } else {
        orc_dtrsm(SD_LEFT, UL_UPPER, TR_T, DG_NONUNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
        orc_dtrsm(SD_LEFT, UL_LOWER, TR_T, DG_UNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
        apply_piv(B, piv, n, 0);
    }
}

/* LU without pivoting: LUDecUnblock LU.cs:188-203 (pivots 0..n-2 checked),
 * LUDecBlock LU.cs:169-186 (blocked iff n > 128). */
static int lu_unblock(mat A, i64 row0) {
    i64 len = A.r < A.c ? A.r : A.c;
    for (i64 i = 0; i + 1 < len; i++) {
        if (invscal(*AT(A, i, i), AT(A, i + 1, i), A.r - i - 1, A.rs, 0)) return (int)(row0 + i + 1);
        ger(-1.0, AT(A, i + 1, i), A.rs, AT(A, i, i + 1), A.cs, sub(A, i + 1, A.r - i - 1, i + 1, A.c - i - 1));
    }
    return 0;
}

int orc_dgetrf_nopiv(i64 n, double *a, i64 rs, i64 cs) {
    mat A = mk(a, n, n, rs, cs);
    if (n <= NB) return lu_unblock(A, 0);
    for (i64 j0 = 0; j0 < n; j0 += NB) {
        i64 b = n - j0 < NB ? n - j0 : NB, r = n - j0 - b;
        mat A11 = sub(A, j0, b, j0, b);
        int info = lu_unblock(A11, j0);
        if (info) return info;
        if (r > 0) {
            mat A12 = sub(A, j0, b, j0 + b, r), A21 = sub(A, j0 + b, r, j0, b);
            trsm_left(UL_LOWER, 1, A11, A12);
            trsm_left(UL_LOWER, 0, tr(A11), tr(A21));       /* X * U11 = A21 */
            gemm_core(-1.0, A21, A12, sub(A, j0 + b, r, j0 + b, r), 0);
        }
    }
    return 0;
}

/* LUSolveInternal, LU.cs:205-231 for trans == 0.  For trans != 0 this solves
 * A^T X = B (U^T first, then L^T); DDLA's code applies the two transposed
 * solves in the opposite order. */
void orc_dgetrs_nopiv(int trans, i64 n, i64 nrhs, const double *a, i64 rs, i64 cs,
                      double *b, i64 rsb, i64 csb) {
    if (n == 0 || nrhs == 0) return;
    if (!trans) {
        orc_dtrsm(SD_LEFT, UL_LOWER, TR_NO, DG_UNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
        orc_dtrsm(SD_LEFT, UL_UPPER, TR_NO, DG_NONUNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
    } else {
        orc_dtrsm(SD_LEFT, UL_UPPER, TR_T, DG_NONUNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
        orc_dtrsm(SD_LEFT, UL_LOWER, TR_T, DG_UNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
    }
}

/* ------------------------------------------------------------------------ */
/* Cholesky, DDLA/Factorizations/Cholesky.cs                                */
/* ------------------------------------------------------------------------ */

/* CholeskyLowerUnblock, Cholesky.cs:127-140 with Sqrt :228-236 (finite <= 0
 * throws) and managed InvScaled (non-finite throws). */
static int chol_lower_unblock(mat A, i64 row0) {
    for (i64 i = 0; i < A.r; i++) {
        double *a11 = AT(A, i, i);
        if (isfinite(*a11) && *a11 <= 0) return (int)(row0 + i + 1);
        *a11 = sqrt(*a11);
        if (invscal(*a11, AT(A, i + 1, i), A.r - i - 1, A.rs, 1)) return (int)(row0 + i + 1);
        syr(UL_LOWER, -1.0, AT(A, i + 1, i), A.rs, sub(A, i + 1, A.r - i - 1, i + 1, A.r - i - 1));
    }
    return 0;
}

/* CholeskyUpperUnblock, Cholesky.cs:162-186: dot-product form, no <=0 check
 * (sqrt of a negative gives NaN which the managed InvScaled then rejects). */
static int chol_upper_unblock(mat A, i64 row0) {
    i64 n = A.r;
    for (i64 i = 0; i < n; i++) {
        double *a11 = AT(A, i, i);
        double d = 0.0;
        for (i64 p = 0; p < i; p++) d = fma(*AT(A, p, i), *AT(A, p, i), d);
        *a11 -= d;
        *a11 = sqrt(*a11);
        /* a12 -= A02^T a01 */
        for (i64 j = i + 1; j < n; j++) {
            double s = 0.0;
            for (i64 p = 0; p < i; p++) s = fma(*AT(A, p, j), *AT(A, p, i), s);
            *AT(A, i, j) -= s;
        }
        if (invscal(*a11, AT(A, i, i + 1), n - i - 1, A.cs, 1)) return (int)(row0 + i + 1);
    }
    return 0;
}

int orc_dpotrf(int uplo, i64 n, double *a, i64 rs, i64 cs) {
    mat A = mk(a, n, n, rs, cs);
    if (n <= NB) return uplo == UL_LOWER ? chol_lower_unblock(A, 0) : chol_upper_unblock(A, 0);
    for (i64 j0 = 0; j0 < n; j0 += NB) {
        i64 b = n - j0 < NB ? n - j0 : NB, r = n - j0 - b;
        mat A11 = sub(A, j0, b, j0, b);
        if (uplo == UL_LOWER) {
            /* CholeskyLowerBlock, Cholesky.cs:142-160 */
            int info = chol_lower_unblock(A11, j0);
            if (info) return info;
            if (r > 0) {
                mat A21 = sub(A, j0 + b, r, j0, b);
                trsm_left(UL_LOWER, 0, A11, tr(A21));       /* A21 * L11^-T: L11 X^T = A21^T */
                gemm_core(-1.0, A21, tr(A21), sub(A, j0 + b, r, j0 + b, r), UL_LOWER);
            }
        } else {
            /* CholeskyUpperBlock, Cholesky.cs:188-208 */
            int info = chol_upper_unblock(A11, j0);
            if (info) return info;
            if (r > 0) {
                mat A12 = sub(A, j0, b, j0 + b, r);
                trsm_left(UL_LOWER, 0, tr(A11), A12);         /* U11^T X = A12 */
                gemm_core(-1.0, tr(A12), A12, sub(A, j0 + b, r, j0 + b, r), UL_UPPER);
            }
        }
    }
    return 0;
}

/* CholeskySolveUncheck, Cholesky.cs:210-226. */
void orc_dpotrs(int uplo, i64 n, i64 nrhs, const double *a, i64 rs, i64 cs, double *b, i64 rsb, i64 csb) {
    if (n == 0 || nrhs == 0) return;
    if (uplo == UL_LOWER) {
        orc_dtrsm(SD_LEFT, UL_LOWER, TR_NO, DG_NONUNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
        orc_dtrsm(SD_LEFT, UL_UPPER, TR_NO, DG_NONUNIT, n, nrhs, 1.0, a, cs, rs, b, rsb, csb);
    } else {
        orc_dtrsm(SD_LEFT, UL_LOWER, TR_NO, DG_NONUNIT, n, nrhs, 1.0, a, cs, rs, b, rsb, csb);
        orc_dtrsm(SD_LEFT, UL_UPPER, TR_NO, DG_NONUNIT, n, nrhs, 1.0, a, rs, cs, b, rsb, csb);
    }
}

/* ------------------------------------------------------------------------ */
/* LDL^T without pivoting, DDLA/Factorizations/LDLT.cs                      */
/* ------------------------------------------------------------------------ */

/* LDLTLowerUnblock LT.cs:141-158 / LDLTUpperUnblock :204-221: only the first
 * n-1 diagonals are tested against zero. */
static int ldlt_unblock(int uplo, mat A, i64 row0) {
    i64 n = A.r;
    for (i64 i = 0; i + 1 < n; i++) {
        double a11 = *AT(A, i, i);
        if (a11 == 0) return (int)(row0 + i + 1);
        mat A22 = sub(A, i + 1, n - i - 1, i + 1, n - i - 1);
        if (uplo == UL_LOWER) {
            if (invscal(a11, AT(A, i + 1, i), n - i - 1, A.rs, 1)) return (int)(row0 + i + 1);
            syr(UL_LOWER, -a11, AT(A, i + 1, i), A.rs, A22);
        } else {
            if (invscal(a11, AT(A, i, i + 1), n - i - 1, A.cs, 0)) return (int)(row0 + i + 1);
            syr(UL_UPPER, -a11, AT(A, i, i + 1), A.cs, A22);
        }
    }
    return 0;
}

/* LDLTLowerBlock LDLT.cs:160-202 / LDLTUpperBlock :223-265 (blocked iff n > 128). */
int orc_dldlt(int uplo, i64 n, double *a, i64 rs, i64 cs) {
    mat A = mk(a, n, n, rs, cs);
    if (n <= NB) return ldlt_unblock(uplo, A, 0);
    double *work = (double *)malloc(sizeof(double) * (size_t)(n - NB) * NB);
    int info = 0;
    for (i64 j0 = 0; j0 < n && !info; j0 += NB) {
        i64 b = n - j0 < NB ? n - j0 : NB, r = n - j0 - b;
        mat A11 = sub(A, j0, b, j0, b);
        info = ldlt_unblock(uplo, A11, j0);
        if (info || r == 0) break;
        if (uplo == UL_LOWER) {
            mat A21 = sub(A, j0 + b, r, j0, b);
            trsm_left(UL_LOWER, 1, A11, tr(A21));         /* A21 * L11^-T, unit */
            mat Y = mk(work, r, b, b, 1);
            for (i64 i = 0; i < r; i++) for (i64 j = 0; j < b; j++) *AT(Y, i, j) = *AT(A21, i, j);
            for (i64 j = 0; j < b && !info; j++)
                if (invscal(*AT(A11, j, j), AT(A21, 0, j), r, A21.rs, 1)) info = (int)(j0 + j + 1);
            if (!info) gemm_core(-1.0, Y, tr(A21), sub(A, j0 + b, r, j0 + b, r), UL_LOWER);
        } else {
            mat A12 = sub(A, j0, b, j0 + b, r);
            trsm_left(UL_LOWER, 1, tr(A11), A12);           /* U11^T X = A12, unit */
            mat Y = mk(work, b, r, r, 1);
            for (i64 i = 0; i < b; i++) for (i64 j = 0; j < r; j++) *AT(Y, i, j) = *AT(A12, i, j);
            for (i64 i = 0; i < b && !info; i++)
                if (invscal(*AT(A11, i, i), AT(A12, i, 0), r, A12.cs, 1)) info = (int)(j0 + i + 1);
            if (!info) gemm_core(-1.0, tr(A12), Y, sub(A, j0 + b, r, j0 + b, r), UL_UPPER);
        }
    }
    free(work);
    return info;
}

/* LDLTSolveUncheck, LDLT.cs:267-295. */
int orc_dldlts(int uplo, i64 n, i64 nrhs, const double *a, i64 rs, i64 cs, double *b, i64 rsb, i64 csb) {
    if (n == 0 || nrhs == 0) return 0;
    i64 lrs = uplo == UL_LOWER ? rs : cs, lcs = uplo == UL_LOWER ? cs : rs;   /* L view */
    orc_dtrsm(SD_LEFT, UL_LOWER, TR_NO, DG_UNIT, n, nrhs, 1.0, a, lrs, lcs, b, rsb, csb);
    for (i64 i = 0; i < n; i++)
        if (invscal(a[i * rs + i * cs], b + i * rsb, nrhs, csb, 1)) return (int)(i + 1);
    orc_dtrsm(SD_LEFT, UL_UPPER, TR_NO, DG_UNIT, n, nrhs, 1.0, a, lcs, lrs, b, rsb, csb);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Einsum: MArray.Contract index analysis + block-scatter GEMM               */
/* ------------------------------------------------------------------------ */

#define ORC_MAXMODE 16
typedef struct { i64 len, sa, sb, sc; } orc_mode;   /* TripleIndice */
typedef struct {
    int nbatch, nm, nn, nk, swapped;
    orc_mode batch[3 * ORC_MAXMODE];
    orc_mode m[ORC_MAXMODE];   /* len, sa (operand-A stride), sc */
    orc_mode n[ORC_MAXMODE];   /* len, sb (operand-B stride), sc */
    orc_mode k[ORC_MAXMODE];   /* len, sa, sb */
} orc_contract_desc;

typedef struct { char sym; i64 len, s1, s2, s3; int used; } ent;

/* IndiceUtils.Diagonal, DDLA/Utilities/IndiceUtils.cs:18-48: a repeated
 * symbol becomes one mode whose stride is the sum of the strides. */
static int diagonal(const char *sym, int rank, const i64 *len, const i64 *str, ent *out, int *cnt) {
    *cnt = 0;
    if ((int)strlen(sym) != rank) return -1;
    for (int i = 0; i < rank; i++) {
        int f = -1;
        for (int j = 0; j < *cnt; j++) if (out[j].sym == sym[i]) f = j;
        if (f >= 0) {
            if (out[f].len != len[i]) return -1;
            out[f].s1 += str[i];
        } else {
            ent e = {sym[i], len[i], str[i], 0, 0, 0};
            out[(*cnt)++] = e;
        }
    }
    return 0;
}

/* IndiceUtils.Fold for two-stride modes, IndiceUtils.cs:186-244: an outer mode
 * whose strides equal (len*stride) of an inner mode absorbs it. */
static void fold2(orc_mode *v, int *cnt, int first, int second) {
    /* first/second: which stride fields are the pair (0 = sa, 1 = sb, 2 = sc) */
    int changed = 1;
    while (changed) {
        changed = 0;
        for (int o = 0; o < *cnt && !changed; o++)
            for (int in = 0; in < *cnt && !changed; in++) {
                if (o == in) continue;
                i64 so[3] = {v[o].sa, v[o].sb, v[o].sc}, si[3] = {v[in].sa, v[in].sb, v[in].sc};
                if (so[first] == v[in].len * si[first] && so[second] == v[in].len * si[second]) {
                    v[o].len *= v[in].len;
                    v[o].sa = v[in].sa; v[o].sb = v[in].sb; v[o].sc = v[in].sc;
                    for (int t = in; t + 1 < *cnt; t++) v[t] = v[t + 1];
                    (*cnt)--;
                    changed = 1;
                }
            }
    }
}

static void sort_desc(orc_mode *v, int cnt, int field) {
    for (int i = 1; i < cnt; i++) {     /* stable insertion sort */
        orc_mode x = v[i];
        i64 kx = field == 0 ? x.sa : field == 1 ? x.sb : x.sc;
        int j = i - 1;
        while (j >= 0) {
            i64 kj = field == 0 ? v[j].sa : field == 1 ? v[j].sb : v[j].sc;
            if (kj >= kx) break;
            v[j + 1] = v[j]; j--;
        }
        v[j + 1] = x;
    }
}

/* MArray.Contract(result, expr, alpha, left, right) index analysis,
 * DDLA/Einsum/MArray.Contract.cs:48-125 with IndiceUtils.Divide
 * (IndiceUtils.cs:73-125).  Modes of length 1 are dropped as in :175-180. */
int orc_contract_plan(const char *expr, int ra, const i64 *la, const i64 *sa,
                      int rb, const i64 *lb, const i64 *sb, int rc, const i64 *lc, const i64 *sc,
                      orc_contract_desc *d) {
    char sA[ORC_MAXMODE + 1], sB[ORC_MAXMODE + 1], sC[ORC_MAXMODE + 1];
    int ns = 0, which = 0;
    char *dst[3] = {sA, sB, sC};
    for (const char *p = expr; *p; p++) {
        if (*p == ' ') continue;
        if (*p == ',') { if (which != 0) return -1; dst[which][ns] = 0; which = 1; ns = 0; continue; }
        if (*p == '-' && p[1] == '>') { if (which != 1) return -1; dst[which][ns] = 0; which = 2; ns = 0; p++; continue; }
        if (ns >= ORC_MAXMODE) return -1;
        dst[which][ns++] = *p;
    }
    if (which != 2) return -1;
    dst[2][ns] = 0;
    ent A[ORC_MAXMODE], B[ORC_MAXMODE], C[ORC_MAXMODE];
    int na, nb, nc;
    if (diagonal(sA, ra, la, sa, A, &na) || diagonal(sB, rb, lb, sb, B, &nb) || diagonal(sC, rc, lc, sc, C, &nc)) return -2;
    memset(d, 0, sizeof(*d));
    orc_mode abc[ORC_MAXMODE], cc[ORC_MAXMODE], ao[ORC_MAXMODE], bo[ORC_MAXMODE];
    int nabc = 0, ncc = 0, nao = 0, nbo = 0;
    for (int i = 0; i < na; i++) A[i].used = A[i].len <= 1;
    for (int i = 0; i < nb; i++) B[i].used = B[i].len <= 1;
    for (int i = 0; i < nc; i++) C[i].used = C[i].len <= 1;
    for (int ic = 0; ic < nc; ic++) {
        if (C[ic].used) continue;
        int fa = -1, fb = -1;
        for (int i = 0; i < na; i++) if (!A[i].used && A[i].sym == C[ic].sym) fa = i;
        for (int i = 0; i < nb; i++) if (!B[i].used && B[i].sym == C[ic].sym) fb = i;
        if (fa >= 0 && A[fa].len != C[ic].len) return -2;
        if (fb >= 0 && B[fb].len != C[ic].len) return -2;
        orc_mode md = {C[ic].len, fa >= 0 ? A[fa].s1 : 0, fb >= 0 ? B[fb].s1 : 0, C[ic].s1};
        if (fa >= 0 && fb >= 0) abc[nabc++] = md;
        else if (fa >= 0) d->m[d->nm++] = md;
        else if (fb >= 0) d->n[d->nn++] = md;
        else cc[ncc++] = md;
        if (fa >= 0) A[fa].used = 1;
        if (fb >= 0) B[fb].used = 1;
        C[ic].used = 1;
    }
    for (int i = 0; i < na; i++) {
        if (A[i].used) continue;
        int fb = -1;
        for (int j = 0; j < nb; j++) if (!B[j].used && B[j].sym == A[i].sym) fb = j;
        if (fb >= 0) {
            if (B[fb].len != A[i].len) return -2;
            orc_mode md = {A[i].len, A[i].s1, B[fb].s1, 0};
            d->k[d->nk++] = md; B[fb].used = 1;
        } else { orc_mode md = {A[i].len, A[i].s1, 0, 0}; ao[nao++] = md; }
        A[i].used = 1;
    }
    for (int j = 0; j < nb; j++) if (!B[j].used) { orc_mode md = {B[j].len, 0, B[j].s1, 0}; bo[nbo++] = md; }
    /* batch order: ABC by descending C stride, then C-only, A-only, B-only (Contract.cs:68-89) */
    sort_desc(abc, nabc, 2); sort_desc(cc, ncc, 2); sort_desc(ao, nao, 0); sort_desc(bo, nbo, 1);
    for (int i = 0; i < nabc; i++) d->batch[d->nbatch++] = abc[i];
    for (int i = 0; i < ncc; i++) d->batch[d->nbatch++] = cc[i];
    for (int i = 0; i < nao; i++) d->batch[d->nbatch++] = ao[i];
    for (int i = 0; i < nbo; i++) d->batch[d->nbatch++] = bo[i];
    /* Fold + sort (Contract.cs:91-99): M by (sa, sc) sorted on C stride, N by
     * (sb, sc) on C stride, K by (sa, sb) on A stride. */
    fold2(d->m, &d->nm, 0, 2); sort_desc(d->m, d->nm, 2);
    fold2(d->n, &d->nn, 1, 2); sort_desc(d->n, d->nn, 2);
    fold2(d->k, &d->nk, 0, 1); sort_desc(d->k, d->nk, 0);
    if (d->nm == 0) { orc_mode u = {1, 1, 1, 1}; d->m[d->nm++] = u; }
    if (d->nn == 0) { orc_mode u = {1, 1, 1, 1}; d->n[d->nn++] = u; }
    if (d->nk == 0) { orc_mode u = {1, 1, 1, 1}; d->k[d->nk++] = u; }
    /* Operand swap when N's innermost C stride is 1 (Contract.cs:101-121). */
    if (d->n[d->nn - 1].sc == 1) {
        d->swapped = 1;
        orc_mode tmp[ORC_MAXMODE];
        int t = d->nm;
        memcpy(tmp, d->m, sizeof(tmp));
        memcpy(d->m, d->n, sizeof(tmp)); d->nm = d->nn;
        memcpy(d->n, tmp, sizeof(tmp)); d->nn = t;
        for (int i = 0; i < d->nm; i++) { i64 s = d->m[i].sb; d->m[i].sb = 0; d->m[i].sa = s; }
        for (int i = 0; i < d->nn; i++) { i64 s = d->n[i].sa; d->n[i].sa = 0; d->n[i].sb = s; }
        for (int i = 0; i < d->nk; i++) { i64 s = d->k[i].sa; d->k[i].sa = d->k[i].sb; d->k[i].sb = s; }
        for (int i = 0; i < d->nbatch; i++) { i64 s = d->batch[i].sa; d->batch[i].sa = d->batch[i].sb; d->batch[i].sb = s; }
    }
    return 0;
}

static i64 total_len(const orc_mode *v, int cnt) { i64 t = 1; for (int i = 0; i < cnt; i++) t *= v[i].len; return t; }

/* Offsets of every flattened index of a mode list (BlockScatterMatrix scatter
 * vectors, DDLA/Einsum/BlockScatterMatrix.cs:205-324); the last mode varies
 * fastest. */
static void scatter(const orc_mode *v, int cnt, int field, i64 *out) {
    i64 tot = total_len(v, cnt);
    for (i64 f = 0; f < tot; f++) {
        i64 rem = f, off = 0;
        for (int i = cnt - 1; i >= 0; i--) {
            i64 idx = rem % v[i].len; rem /= v[i].len;
            i64 s = field == 0 ? v[i].sa : field == 1 ? v[i].sb : v[i].sc;
            off += idx * s;
        }
        out[f] = off;
    }
}

/* BlockScatterContract_Silent, DDLA/Einsum/MArray.Contract.cs:313-405: for each
 * batch index, C[m,n] += alpha * sum_k A[m,k] B[k,n] with the MC/KC/NC
 * blocking, K padded to KR with zeros, the 6x8 micro-kernel and a fused
 * C += alpha*tile (BSMBlock.UnpackAxpy, DDLA/Einsum/BSMBlock.cs:195-305).
 * Operands are (A, B) after the plan's optional swap. */
void orc_contract_exec(const orc_contract_desc *d, double alpha, const double *a, const double *b, double *c) {
    if (alpha == 0.0) return;
    if (d->swapped) { const double *t = a; a = b; b = t; }
    i64 m = total_len(d->m, d->nm), n = total_len(d->n, d->nn), k = total_len(d->k, d->nk);
    i64 *rA = malloc(sizeof(i64) * m), *rC = malloc(sizeof(i64) * m);
    i64 *cB = malloc(sizeof(i64) * n), *cC = malloc(sizeof(i64) * n);
    i64 *kA = malloc(sizeof(i64) * k), *kB = malloc(sizeof(i64) * k);
    scatter(d->m, d->nm, 0, rA); scatter(d->m, d->nm, 2, rC);
    scatter(d->n, d->nn, 1, cB); scatter(d->n, d->nn, 2, cC);
    scatter(d->k, d->nk, 0, kA); scatter(d->k, d->nk, 1, kB);
    i64 nbt = total_len(d->batch, d->nbatch);
    i64 kmax = align_up(k < KC ? k : KC, KR);
    double *bufA = malloc(sizeof(double) * align_up(m < MC ? m : MC, MR) * kmax);
    double *bufB = malloc(sizeof(double) * align_up(n < NC ? n : NC, NR) * kmax);
    for (i64 bt = 0; bt < nbt; bt++) {
        i64 rem = bt, oa = 0, ob = 0, oc = 0;
        for (int i = d->nbatch - 1; i >= 0; i--) {
            i64 idx = rem % d->batch[i].len; rem /= d->batch[i].len;
            oa += idx * d->batch[i].sa; ob += idx * d->batch[i].sb; oc += idx * d->batch[i].sc;
        }
        for (i64 i0 = 0; i0 < m; i0 += MC) {
            i64 ic = m - i0 < MC ? m - i0 : MC;
            for (i64 q = 0; q < k; q += KC) {
                i64 qc = k - q < KC ? k - q : KC, qa = align_up(qc, KR);
                for (i64 p = 0; p < align_up(ic, MR) / MR; p++)
                    for (i64 kk = 0; kk < qa; kk++)
                        for (int r = 0; r < MR; r++) {
                            i64 row = i0 + p * MR + r;
                            bufA[(p * qa + kk) * MR + r] = (row < i0 + ic && kk < qc) ? a[oa + rA[row] + kA[q + kk]] : 0.0;
                        }
                for (i64 j0 = 0; j0 < n; j0 += NC) {
                    i64 jc = n - j0 < NC ? n - j0 : NC;
                    for (i64 p = 0; p < align_up(jc, NR) / NR; p++)
                        for (i64 kk = 0; kk < qa; kk++)
                            for (int s = 0; s < NR; s++) {
                                i64 col = j0 + p * NR + s;
                                bufB[(p * qa + kk) * NR + s] = (col < j0 + jc && kk < qc) ? b[ob + kB[q + kk] + cB[col]] : 0.0;
                            }
                    i64 ip = align_up(ic, MR) / MR;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1 && ip >= 8)
#endif
                    for (i64 p = 0; p < ip; p++) {
                        double t[MR * NR];
                        for (i64 s0 = 0; s0 < align_up(jc, NR); s0 += NR) {
                            micro(qa, bufA + p * qa * MR, bufB + (s0 / NR) * qa * NR, t);
                            for (int r = 0; r < MR; r++) {
                                i64 row = i0 + p * MR + r;
                                if (row >= i0 + ic) break;
                                for (int s = 0; s < NR; s++) {
                                    i64 col = j0 + s0 + s;
                                    if (col >= j0 + jc) break;
                                    double *cp = c + oc + rC[row] + cC[col];
                                    *cp = fma(t[r * NR + s], alpha, *cp);
                                }
                            }
                        }
                    }
                }
            }
        }
    }
    free(rA); free(rC); free(cB); free(cC); free(kA); free(kB); free(bufA); free(bufB);
}

int orc_contract_desc_size(void) { return (int)sizeof(orc_contract_desc); }

/* ------------------------------------------------------------------------ */
/* Batched small solves (the batched workload's checker)                     */
/* ------------------------------------------------------------------------ */

/* Factor and solve `count` independent square row-major systems packed back
 * to back (a: sum n_i^2 doubles, b / x / piv: sum n_i entries), item i with
 * kind 0 = PLUDecompose + PLUSolve (LU.cs:251-287), 1 = LUDecompose + LUSolve
 * (LU.cs:133-167), 2 = lower CholDecompose + CholeskySolve (Cholesky.cs:52-123).
 * a is factored in place, x = solution of the original system, info[i] the
 * failing pivot or 0.  Items run in parallel; each one is the serial
 * restatement above (the factorizations' own threading stays off inside). */
void orc_batched(i64 count, const int *n, const int *kind, double *a, const double *b, double *x, int *piv,
                 int *info) {
    i64 *ao = (i64 *)malloc(sizeof(i64) * (count + 1)), *vo = (i64 *)malloc(sizeof(i64) * (count + 1));
    ao[0] = vo[0] = 0;
    for (i64 i = 0; i < count; i++) { ao[i + 1] = ao[i] + (i64)n[i] * n[i]; vo[i + 1] = vo[i] + n[i]; }
    int saved = g_threads;
    int outer = g_threads;
    g_threads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8) num_threads(outer) if (outer > 1)
#endif
    for (i64 i = 0; i < count; i++) {
        const i64 ni = n[i];
        double *ai = a + ao[i], *xi = x + vo[i];
        int *pi = piv + vo[i];
        memcpy(xi, b + vo[i], sizeof(double) * ni);
        memset(pi, 0, sizeof(int) * ni);
        int rc;
        if (kind[i] == 0) {
            rc = orc_dgetrf(ni, ai, ni, 1, pi);
            if (!rc) orc_dgetrs(0, ni, 1, ai, ni, 1, pi, xi, 1, 1);
        } else if (kind[i] == 1) {
            rc = orc_dgetrf_nopiv(ni, ai, ni, 1);
            if (!rc) orc_dgetrs_nopiv(0, ni, 1, ai, ni, 1, xi, 1, 1);
        } else {
            rc = orc_dpotrf(UL_LOWER, ni, ai, ni, 1);
            if (!rc) orc_dpotrs(UL_LOWER, ni, 1, ai, ni, 1, xi, 1, 1);
        }
        info[i] = rc;
    }
    g_threads = saved;
    free(ao); free(vo);
}

/* ------------------------------------------------------------------------ */
/* Two-stage bidiagonal reduction, DDLA/Transformations/Bidiagonaling.cs     */
/* (Bidiag -> TwoStageBidiag, :14-33 and :334-582)                           */
/* ------------------------------------------------------------------------ */

#define BD2_BLOCK 32   /* TwoStageBidiag.MaxBlockSize, Bidiagonaling.cs:336 */

/* BidHelper.BuildHH (Bidiagonaling.cs:705-718): |x| from the sum of squares,
 * rho = -sign(a11) |x|, x2 *= 1 / (a11 - rho), tau = (1 + |x2|^2) / 2. */
static void bd2_build_hh(double *a11, double *x, i64 n, i64 inc, double *tau) {
    double xsq = 0.0;
    for (i64 i = 0; i < n; i++) xsq = fma(x[i * inc], x[i * inc], xsq);
    double alphasq = *a11 * *a11 + xsq;
    double alpha = sqrt(alphasq);
    double sign = *a11 > 0 ? 1.0 : (*a11 < 0 ? -1.0 : 0.0);   /* Math.Sign */
    double rho = -sign * alpha;
    double miu = *a11 - rho;
    double s = 1.0 / miu;
    for (i64 i = 0; i < n; i++) x[i * inc] *= s;
    double t = 0.0;
    for (i64 i = 0; i < n; i++) t = fma(x[i * inc], x[i * inc], t);
    *tau = 1.0 + t;
    *a11 = rho;
    *tau /= 2.0;
}

/* BidHelper.ApplyHH (Bidiagonaling.cs:752-764), per column of A2:
 * w = a12 + a21 . a22, w /= tau, a12 -= w, a22 -= w a21. */
static void bd2_apply_hh(const double *a21, i64 n, i64 inc, mat A2, double tau) {
    for (i64 c = 0; c < A2.c; c++) {
        double dot = 0.0;
        for (i64 i = 0; i < n; i++) dot = fma(a21[i * inc], *AT(A2, 1 + i, c), dot);
        double w = *AT(A2, 0, c) + dot;
        w /= tau;
        *AT(A2, 0, c) -= w;
        for (i64 i = 0; i < n; i++) *AT(A2, 1 + i, c) = fma(-w, a21[i * inc], *AT(A2, 1 + i, c));
    }
}

/* BidHelper.QRUnblock (Bidiagonaling.cs:594-615): the QR of one block column
 * with its UT factor: T(i, i) = tau_i, T(0:i, i) = A(i, 0:i)^T + A20^T a21. */
static void bd2_qr_unblock(mat A, mat T) {
    i64 m = A.r, n = A.c, k = m < n ? m : n;
    for (i64 i = 0; i < k; i++) {
        double *x = AT(A, i + 1 < m ? i + 1 : i, i);
        bd2_build_hh(AT(A, i, i), x, m - i - 1, A.rs, AT(T, i, i));
        bd2_apply_hh(x, m - i - 1, A.rs, sub(A, i, m - i, i + 1, n - i - 1), *AT(T, i, i));
        for (i64 j = 0; j < i; j++) {
            double t = *AT(A, i, j);
            for (i64 r = i + 1; r < m; r++) t = fma(*AT(A, r, j), *AT(A, r, i), t);
            *AT(T, j, i) = t;
        }
    }
}

/* Bd2Bi_StepSide (Bidiagonaling.cs:539-551): the reflector of A's first
 * column (HouseHolder.BuildHouseHolder) applied from the left to the other
 * columns; tau and the vector go to t, the column's tail is cleared. */
static void bd2_step_side(mat A, double *t, i64 tinc) {
    i64 len = A.r - 1;
    double *chi = AT(A, 0, 0);
    double *x = AT(A, A.r > 1 ? 1 : 0, 0);
    house_build(chi, x, len, A.rs, &t[0]);
    house_apply_left(t[0], x, A.rs, sub(A, 0, 1, 1, A.c - 1), sub(A, 1, len, 1, A.c - 1));
    for (i64 i = 0; i < len; i++) { t[(1 + i) * tinc] = x[i * A.rs]; x[i * A.rs] = 0.0; }
}

/* Bd2Bi_StepCycle (Bidiagonaling.cs:489-516): chase row i's band to the
 * superdiagonal, alternating right (transposed view) and left reflectors. */
static void bd2_step_cycle(mat A, double *tu, double *tv, i64 tinc, i64 block) {
    i64 is = 1, ie = is + block, ie2 = ie + block;
    i64 rows = A.r;
    if (rows <= ie) {
        bd2_step_side(tr(sub(A, 0, A.r, is, A.c - is)), tv + is * tinc, tinc);
        bd2_step_side(sub(A, is, A.r - is, is, A.c - is), tu + is * tinc, tinc);
        return;
    }
    bd2_step_side(tr(sub(A, 0, ie, is, ie - is)), tv + is * tinc, tinc);
    while (ie2 < rows) {
        bd2_step_side(sub(A, is, ie - is, is, ie2 - is), tu + is * tinc, tinc);
        bd2_step_side(tr(sub(A, is, ie2 - is, ie, ie2 - ie)), tv + ie * tinc, tinc);
        is += block; ie += block; ie2 += block;
    }
    bd2_step_side(sub(A, is, ie - is, is, A.c - is), tu + is * tinc, tinc);
    bd2_step_side(tr(sub(A, is, A.r - is, ie, A.c - ie)), tv + ie * tinc, tinc);
    bd2_step_side(sub(A, ie, A.r - ie, ie, A.c - ie), tu + ie * tinc, tinc);
}

/* Bd2Bi_Back (Bidiagonaling.cs:553-558): Q <- Q H, H = I - u u^T / tau with
 * u = (1, t[1..]) (ApplyHouseHolder on Q^T from the left). */
static void bd2_back(const double *t, i64 tinc, i64 len, mat Q) {
    if (len <= 0) return;
    mat QT = tr(Q);
    double *u2 = (double *)malloc(sizeof(double) * (len > 1 ? len - 1 : 1));
    for (i64 i = 0; i + 1 < len; i++) u2[i] = t[(1 + i) * tinc];
    house_apply_left(t[0], u2, 1, sub(QT, 0, 1, 0, QT.c), sub(QT, 1, len - 1, 0, QT.c));
    free(u2);
}

/* Bidiagonaling.Bidiag(A, U, V, d, e) through TwoStageBidiag, m >= n: A is a
 * work copy (overwritten), U m x m, V n x n, d (n), e (n - 1).  Ge2Bd
 * (Bidiagonaling.cs:384-474): blocks of BD2_BLOCK columns, each a QR of the
 * block column (its reflector applied to the columns right of it) and an LQ
 * of the block row right of it (a QR of its transpose, applied to the rows
 * below); U and V from the two sets of block reflectors (ApplyQlnfc), which
 * leaves an upper band of width BD2_BLOCK.  Bd2Bi (:478-487): for each row a
 * bulge-chasing cycle of small reflectors down the band, stored in TU2 / TV2,
 * then every cycle's reflectors applied to U and V. */
int orc_dbidiag2s(i64 m, i64 n, double *a, i64 rsa, i64 csa, double *u, i64 rsu, i64 csu, double *v, i64 rsv,
                  i64 csv, double *d, double *e) {
    if (m < n) return -1;
    if (n == 0) return 0;
    mat W = mk(a, m, n, rsa, csa), U = mk(u, m, m, rsu, csu), V = mk(v, n, n, rsv, csv);
    const i64 bs = n < BD2_BLOCK ? n : BD2_BLOCK;          /* TUBlockSize */
    const i64 tvc = n - bs;
    double *tu = (double *)calloc((size_t)bs * n, sizeof(double));
    double *tv = (double *)calloc((size_t)bs * (tvc > 0 ? tvc : 1), sizeof(double));
    mat TU = mk(tu, bs, n, n, 1), TV = mk(tv, bs, tvc > 0 ? tvc : 1, tvc > 0 ? tvc : 1, 1);
    for (i64 i = 0; i < m; i++) for (i64 j = 0; j < m; j++) *AT(U, i, j) = i == j;
    for (i64 i = 0; i < n; i++) for (i64 j = 0; j < n; j++) *AT(V, i, j) = i == j;
    /* Ge2Bd */
    for (i64 i0 = 0; i0 < n; ) {
        i64 b = n - i0 < BD2_BLOCK ? n - i0 : BD2_BLOCK;
        mat AB1 = sub(W, i0, m - i0, i0, b), AB2 = sub(W, i0, m - i0, i0 + b, n - i0 - b);
        mat TUT1 = sub(TU, 0, b, i0, b);
        bd2_qr_unblock(AB1, TUT1);
        qr_apply_one(1, sub(AB1, 0, b, 0, b), sub(AB1, b, m - i0 - b, 0, b), TUT1, sub(AB2, 0, b, 0, AB2.c),
                     sub(AB2, b, m - i0 - b, 0, AB2.c));
        i64 c22 = n - i0 - b;
        if (c22 > 0) {
            i64 b2 = c22 < BD2_BLOCK ? c22 : b;   /* the ragged last block row: block2 = A22.Cols */
            mat R = tr(sub(W, i0, b2, i0 + b, c22));           /* c22 x b2 */
            mat below = tr(sub(W, i0 + b2, m - i0 - b2, i0 + b, c22));
            mat TVT1 = sub(TV, 0, b2, i0, b2);
            bd2_qr_unblock(R, TVT1);
            qr_apply_one(1, sub(R, 0, b2, 0, b2), sub(R, b2, c22 - b2, 0, b2), TVT1, sub(below, 0, b2, 0, below.c),
                         sub(below, b2, c22 - b2, 0, below.c));
        }
        i0 += b;
    }
    qr_apply(0, W, TU, U);
    for (i64 i = 0; i < m; i++) for (i64 j = 0; j < i && j < n; j++) *AT(W, i, j) = 0.0;
    if (tvc > 0) {
        mat A = tr(sub(W, 0, tvc, bs, tvc));
        qr_apply(0, A, TV, sub(V, bs, tvc, bs, tvc));
        for (i64 i = 0; i < tvc; i++) for (i64 j = 0; j < i; j++) *AT(A, i, j) = 0.0;
    }
    /* Bd2Bi */
    double *tu2 = (double *)calloc((size_t)n * n, sizeof(double));
    double *tv2 = (double *)calloc((size_t)n * n, sizeof(double));
    for (i64 i = 0; i + 1 < n; i++)
        bd2_step_cycle(sub(W, i, n - i, i, n - i), tu2 + i * n + i, tv2 + i * n + i, 1, bs);
    for (i64 i = 0; i + 1 < n; i++) {
        const i64 rows = n - i, maxu = (rows - 2) / bs + 1;
        for (i64 k = 0; k < maxu; k++) {
            i64 is = 1 + k * bs, ie = is + bs < rows ? is + bs : rows;
            bd2_back(tv2 + i * n + i + is, 1, ie - is, sub(V, 0, n, i + is, ie - is));
            bd2_back(tu2 + i * n + i + is, 1, ie - is, sub(U, 0, m, i + is, ie - is));
        }
    }
    for (i64 i = 0; i < n; i++) d[i] = *AT(W, i, i);
    for (i64 i = 0; i + 1 < n; i++) e[i] = *AT(W, i, i + 1);
    free(tu); free(tv); free(tu2); free(tv2);
    return 0;
}
