// Triangular solve with many right-hand sides (BLIS trsm semantics).
//
// The problem is first normalised to a left solve with a non-transposed
// triangle (a right solve X*op(A) = B is the left solve op(A)^T X^T = B^T; a
// transposed triangle is the other triangle of the transposed view), then
// solved in blocks of TB rows: a diagonal-block kernel (one thread per
// right-hand-side column, triangle and columns in shared memory) followed by
// a GEMM update of the remaining rows, forward for lower and backward for
// upper triangles -- the block structure of DDLA's managed TrSM
// (DDLA/BLAS/Managed/3m/TrSM.cs:62-122, blocks of KC rows, GEMM + TRSV).
#include "common.cuh"

namespace ddla {
namespace {

constexpr int TB = 64;   // rows per diagonal block
// right-hand-side columns per CTA (one thread each); keeps the triangle plus
// the column block within 48 KB of static shared memory
template <typename T>
constexpr int cw() { return sizeof(T) == 8 ? 32 : 64; }

template <typename T>
__global__ void k_scale(T alpha, T *B, i64 m, i64 n, i64 rs, i64 cs) {
    i64 tot = m * n;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        i64 i = e / n, j = e % n;
        T *p = B + i * rs + j * cs;
        *p = (alpha == T(0)) ? T(0) : *p * alpha;
    }
}

// Solve tri(A11) X = B1 for a bs x bs triangle (bs <= TB), columns split over
// CTAs, one thread per column, four partial sums per dot product.
template <typename T>
__global__ void __launch_bounds__(cw<T>())
    k_trsm_diag(int bs, i64 n, const T *__restrict__ A, i64 rsa, i64 csa, T *B, i64 rsb, i64 csb, int lower,
                int unit) {
    constexpr int CW = cw<T>();
    __shared__ T L[TB][TB];
    __shared__ T X[TB][CW];
    const int t = threadIdx.x;
    const i64 c = (i64)blockIdx.x * CW + t;
    for (int e = t; e < bs * bs; e += CW) {
        int i = e / bs, j = e % bs;
        L[i][j] = A[i * rsa + j * csa];
    }
    if (c < n)
        for (int i = 0; i < bs; i++) X[i][t] = B[i * rsb + c * csb];
    __syncthreads();
    if (c >= n) return;
    if (lower) {
        for (int i = 0; i < bs; i++) {
            T s0 = X[i][t], s1 = 0, s2 = 0, s3 = 0;
            int p = 0;
            for (; p + 3 < i; p += 4) {
                s0 -= L[i][p] * X[p][t];
                s1 -= L[i][p + 1] * X[p + 1][t];
                s2 -= L[i][p + 2] * X[p + 2][t];
                s3 -= L[i][p + 3] * X[p + 3][t];
            }
            for (; p < i; p++) s0 -= L[i][p] * X[p][t];
            T s = (s0 + s1) + (s2 + s3);
            X[i][t] = unit ? s : s / L[i][i];
        }
    } else {
        for (int i = bs - 1; i >= 0; i--) {
            T s0 = X[i][t], s1 = 0, s2 = 0, s3 = 0;
            int p = i + 1;
            for (; p + 3 < bs; p += 4) {
                s0 -= L[i][p] * X[p][t];
                s1 -= L[i][p + 1] * X[p + 1][t];
                s2 -= L[i][p + 2] * X[p + 2][t];
                s3 -= L[i][p + 3] * X[p + 3][t];
            }
            for (; p < bs; p++) s0 -= L[i][p] * X[p][t];
            T s = (s0 + s1) + (s2 + s3);
            X[i][t] = unit ? s : s / L[i][i];
        }
    }
    for (int i = 0; i < bs; i++) B[i * rsb + c * csb] = X[i][t];
}

template <typename T>
int scale(cudaStream_t s, T alpha, View<T> B) {
    if (alpha == T(1) || B.rows == 0 || B.cols == 0) return 0;
    i64 tot = B.rows * B.cols;
    int blocks = (int)((tot + 255) / 256 < 4096 ? (tot + 255) / 256 : 4096);
    k_scale<T><<<blocks, 256, 0, s>>>(alpha, B.p, B.rows, B.cols, B.rs, B.cs);
    DDLA_LAUNCHED();
    return 0;
}

template <typename T>
int diag_solve(cudaStream_t s, int bs, View<const T> A11, View<T> B1, bool lower, bool unit) {
    i64 n = B1.cols;
    constexpr int CW = cw<T>();
    unsigned grid = (unsigned)((n + CW - 1) / CW);
    k_trsm_diag<T><<<grid, CW, 0, s>>>(bs, n, A11.p, A11.rs, A11.cs, B1.p, B1.rs, B1.cs, lower ? 1 : 0,
                                       unit ? 1 : 0);
    DDLA_LAUNCHED();
    return 0;
}

}  // namespace

template <typename T>
int gemm_any(ddla_handle h, int prec, i64 m, i64 n, i64 k, T alpha, View<const T> A, View<const T> B, T beta,
             View<T> C, int uplo);

template <typename T>
int trsm(ddla_handle h, int side, int uplo, int trans, int diag, i64 m, i64 n, T alpha, View<const T> A,
         View<T> B) {
    if (m == 0 || n == 0) return 0;
    cudaStream_t s = h->stream;
    DDLA_TRY(scale<T>(s, alpha, B));
    if (trans & DDLA_TRANSPOSE) {
        A = A.t();
        uplo = flip_uplo(uplo);
    }
    if (side == DDLA_RIGHT) {
        A = A.t();
        uplo = flip_uplo(uplo);
        B = B.t();
        i64 t = m;
        m = n;
        n = t;
    }
    const bool unit = (diag == DDLA_UNIT_DIAG);
    const int prec = sizeof(T) == 8 ? DDLA_PREC_FP64 : DDLA_PREC_FP32;
    if (uplo == DDLA_LOWER) {
        for (i64 i0 = 0; i0 < m; i0 += TB) {
            int bs = (int)(m - i0 < TB ? m - i0 : TB);
            DDLA_TRY(diag_solve<T>(s, bs, A.sub(i0, bs, i0, bs), B.sub(i0, bs, 0, n), true, unit));
            i64 r = m - i0 - bs;
            if (r > 0) {
                View<const T> B1{B.p + i0 * B.rs, bs, n, B.rs, B.cs};
                DDLA_TRY(gemm_any<T>(h, prec, r, n, bs, T(-1), A.sub(i0 + bs, r, i0, bs), B1, T(1),
                                     B.sub(i0 + bs, r, 0, n), DDLA_DENSE));
            }
        }
    } else {
        for (i64 i1 = m; i1 > 0; i1 -= TB) {
            int bs = (int)(i1 < TB ? i1 : TB);
            i64 i0 = i1 - bs;
            DDLA_TRY(diag_solve<T>(s, bs, A.sub(i0, bs, i0, bs), B.sub(i0, bs, 0, n), false, unit));
            if (i0 > 0) {
                View<const T> B1{B.p + i0 * B.rs, bs, n, B.rs, B.cs};
                DDLA_TRY(gemm_any<T>(h, prec, i0, n, bs, T(-1), A.sub(0, i0, i0, bs), B1, T(1), B.sub(0, i0, 0, n),
                                     DDLA_DENSE));
            }
        }
    }
    return 0;
}

template int trsm<double>(ddla_handle, int, int, int, int, i64, i64, double, View<const double>, View<double>);
template int trsm<float>(ddla_handle, int, int, int, int, i64, i64, float, View<const float>, View<float>);

}  // namespace ddla
