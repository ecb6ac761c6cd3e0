// Internal definitions shared by the CUDA translation units of libddla_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/ddla_gb300.h"

namespace ddla {

typedef int64_t i64;

// ------------------------------------------------------------------ status
// Thread-local last error message and a process-wide kernel launch counter.
void set_error(const std::string &msg);
extern std::atomic<int64_t> g_launches;
inline void count_launch(int64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

struct Status {
    int code = 0;
};

#define DDLA_CUDA(expr)                                                                          \
    do {                                                                                         \
        cudaError_t e_ = (expr);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            cudaGetLastError();                                                                  \
            ::ddla::set_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " at " +      \
                              __FILE__ + ":" + std::to_string(__LINE__) + " in " #expr);         \
            return DDLA_ERR_CUDA;                                                                \
        }                                                                                        \
    } while (0)

#define DDLA_LAUNCHED()                                                                          \
    do {                                                                                         \
        ::ddla::count_launch();                                                                  \
        cudaError_t e_ = cudaGetLastError();                                                     \
        if (e_ != cudaSuccess) {                                                                 \
            ::ddla::set_error(std::string("kernel launch failed: ") + cudaGetErrorString(e_) +   \
                              " at " + __FILE__ + ":" + std::to_string(__LINE__));               \
            return DDLA_ERR_CUDA;                                                                \
        }                                                                                        \
    } while (0)

#define DDLA_TRY(expr)                   \
    do {                                 \
        int s_ = (expr);                 \
        if (s_ != 0) return s_;          \
    } while (0)

// ------------------------------------------------------------------ views
// Strided matrix view in elements, DDLA's MatrixView layout.
template <typename T>
struct View {
    T *p;
    i64 rows, cols, rs, cs;
    __host__ __device__ T &at(i64 i, i64 j) const { return p[i * rs + j * cs]; }
    __host__ __device__ View t() const { return View{p, cols, rows, cs, rs}; }
    __host__ __device__ View sub(i64 i, i64 ni, i64 j, i64 nj) const {
        return View{p + i * rs + j * cs, ni, nj, rs, cs};
    }
};

inline int flip_uplo(int u) { return u == DDLA_LOWER ? DDLA_UPPER : (u == DDLA_UPPER ? DDLA_LOWER : u); }

// ------------------------------------------------------------------ handle
struct Workspace {
    void *ptr = nullptr;
    size_t bytes = 0;
};

}  // namespace ddla

struct ddla_handle_s {
    int device = 0;
    int sm_count = 0;
    int max_cluster = 8;         // largest cluster size the panel kernel may use
    size_t smem_optin = 0;       // max dynamic shared memory per block
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // Growable device scratch areas (indexed by purpose).
    ddla::Workspace ws[25];
    // Pinned host staging for host-pointer calls.
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
    int *d_info = nullptr;       // device status words (info, timeout flags)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // look-ahead: high-priority side stream for the next panel, and the
    // events ordering it against the main stream (created on first use)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_ready = nullptr, ev_panel = nullptr;
};

namespace ddla {

// Scratch slots.  A slot may be reallocated by its next user, so a buffer
// must not be held across a call that uses the same slot:
//   WS_A/B/C   host staging of operands, mixed-solver vectors
//   WS_TMP     TRSM copies, row-permutation temporaries
//   WS_PIV     LU panel touched-row lists      WS_F32  FP32 factor copy
//   WS_X       device pivots                   WS_MISC TRSV flags, permutations
//   WS_TRI     inverted diagonal blocks        WS_Y    LDL^T Y block
//   WS_PERM    row permutation kept by getrf   WS_TC   tensor-core split operands
//   WS_INV     inverted diagonal blocks of a factorization, kept for all of
//              its refinement solves
//   WS_PINV    inverses of the LU panels' L11 blocks (two, by panel parity)
//   WS_QR      QR: tau, a panel's block factor, the block-reflector scratch
//   WS_SPLIT   partial products of split-k FP64 GEMMs
//   WS_QRU     QR: explicit copy of a block's Householder vectors
//   WS_TRD     tridiagonal reduction: vectors and partial sums
//   WS_TRDQ    tridiagonal reduction: Q of the trailing block before its copy
//   WS_RHS     mixed solves: a block of right-hand sides
//   WS_BD2     two-stage bidiagonal reduction: block factors, chase reflectors
//   WS_NEXT    LU look-ahead: the next panel's columns after the previous step
//   WS_TRSV    split triangular solve: block flags, row states, far sums
//   WS_TRSVM   cluster triangular solve: diagonal-block inverses times the last tiles
enum WsSlot {
    WS_A = 0, WS_B = 1, WS_C = 2, WS_TMP = 3, WS_PIV = 4, WS_F32 = 5, WS_X = 6, WS_MISC = 7,
    WS_TRI = 8, WS_Y = 9, WS_PERM = 10, WS_TC = 11, WS_TC2 = 12, WS_INV = 13, WS_PINV = 14, WS_QR = 15,
    WS_SPLIT = 16, WS_QRU = 17, WS_TRD = 18, WS_TRDQ = 19, WS_RHS = 20, WS_BD2 = 21, WS_NEXT = 22,
    WS_TRSV = 23, WS_TRSVM = 24
};

// Order of the diagonal blocks that the triangular solves invert.
constexpr int TRI_TB = 64;

// Where an LU panel loads its rows from when the work of the previous step
// was done out of place (panel.cu next_prep): rows from ld, and U12 rows to
// copy to u12_dst (strides of the panel's own view) before factoring.
template <typename T>
struct PanelLoad {
    const T *ld;
    i64 ld_rs, ld_cs;
    const T *u12_src;
    T *u12_dst;
    int u12_rows;
};

// Raises the kernel's dynamic shared-memory limit to everything the device
// allows beside its static shared memory; returns that limit in *avail.
int max_dyn_smem(const void *fn, size_t optin, size_t *avail);

// Tuning parameter lookup (tune.cu); dflt when the key was never set.
int64_t tune_get(const char *key, int64_t dflt);

// Returns a device buffer of at least `bytes` from slot `slot` (grown on demand).
int workspace(ddla_handle h, int slot, size_t bytes, void **out);
int pinned(ddla_handle h, size_t bytes, void **out);
// The calling thread's default handle (created on first use).
int default_handle(ddla_handle *out);

// Device status words in h->d_info.
enum InfoSlot { INFO_PIVOT = 0, INFO_TIMEOUT = 1, INFO_COUNT = 4 };
int reset_info(ddla_handle h);
// Reads the device info words (synchronizes the stream).  Returns the first
// failing pivot (1-based, 0 = none) in *pivot; DDLA_ERR_TIMEOUT if a bounded
// wait gave up.
int read_info(ddla_handle h, int *pivot);

// ------------------------------------------------------------------ kernels
// GEMM: C = alpha*A*B + beta*C on device views (A m x k, B k x n, C m x n).
// uplo = DDLA_DENSE for a full C, DDLA_LOWER / DDLA_UPPER for GEMMT (only that
// triangle of C is written; tiles outside it are skipped).
// batch > 1 runs `batch` independent products with element offsets
// sa/sb/sc between consecutive problems.
int gemm_f64(cudaStream_t s, i64 m, i64 n, i64 k, double alpha, View<const double> A, View<const double> B,
             double beta, View<double> C, int uplo = DDLA_DENSE, i64 batch = 1, i64 sa = 0, i64 sb = 0, i64 sc = 0);
int gemm_f32(cudaStream_t s, i64 m, i64 n, i64 k, float alpha, View<const float> A, View<const float> B,
             float beta, View<float> C, int uplo = DDLA_DENSE);
// Structured FP64 operands of gemm_f64_struct: kind in bits 0-1, then flags.
// OP_TRI operands may be trapezoidal (element (i, j) is zero for j > i when
// OP_LOWER, for j < i otherwise).
enum OpMode : int { OP_DENSE = 0, OP_SYM = 1, OP_TRI = 2, OP_LOWER = 4, OP_UNIT = 8 };
int gemm_f64_struct(cudaStream_t s, i64 m, i64 n, i64 k, double alpha, View<const double> A, int amode,
                    View<const double> B, int bmode, double beta, View<double> C, int uplo = DDLA_DENSE);
// The same with the k range split over extra CTAs when C has too few tiles to
// fill the GPU (partial products in the handle's WS_SPLIT scratch, summed in a
// fixed order, so results do not depend on scheduling).
int gemm_f64_struct_h(ddla_handle h, i64 m, i64 n, i64 k, double alpha, View<const double> A, int amode,
                      View<const double> B, int bmode, double beta, View<double> C, int uplo = DDLA_DENSE);

// Triangular solve, B <- op(A)^-1 alpha B (left) or alpha B op(A)^-1 (right).
template <typename T>
int trsm(ddla_handle h, int side, int uplo, int trans, int diag, i64 m, i64 n, T alpha, View<const T> A, View<T> B);

// Precision-dispatching GEMM used by the factorization drivers.
template <typename T>
int gemm_any(ddla_handle h, int prec, i64 m, i64 n, i64 k, T alpha, View<const T> A, View<const T> B, T beta,
             View<T> C, int uplo = DDLA_DENSE);

// Factorization drivers (device data, row/col strides arbitrary).
// d_perm (optional, n ints): receives the row permutation of the
// factorization (row k of P*A is row d_perm[k] of A).
template <typename T>
int getrf(ddla_handle h, i64 n, View<T> A, int32_t *d_piv, int prec, int nb, int *d_perm = nullptr);
// Solve with the factors and the permutation vector of getrf.
template <typename T>
int getrs_perm(ddla_handle h, i64 n, i64 nrhs, View<const T> LU, const int *d_perm, View<T> B);
template <typename T>
int getrs(ddla_handle h, int trans, i64 n, i64 nrhs, View<const T> LU, const int32_t *d_piv, View<T> B);
template <typename T>
int getrf_nopiv(ddla_handle h, i64 n, View<T> A, int prec, int nb);
template <typename T>
int getrs_nopiv(ddla_handle h, int trans, i64 n, i64 nrhs, View<const T> LU, View<T> B);
template <typename T>
int potrf(ddla_handle h, int uplo, i64 n, View<T> A, int prec, int nb);
template <typename T>
int potrs(ddla_handle h, int uplo, i64 n, i64 nrhs, View<const T> A, View<T> B);
template <typename T>
int ldlt(ddla_handle h, int uplo, i64 n, View<T> A, int prec, int nb);
template <typename T>
int ldlts(ddla_handle h, int uplo, i64 n, i64 nrhs, View<const T> A, View<T> B);

// Householder QR in DDLA's UT-transform storage (qr.cu); T has tb rows and
// holds the factor of every block of tb columns.
// prec DDLA_PREC_OZAKI runs the block reflectors' large products through the
// split-precision tensor-core GEMM; wcap caps the panel width (0 = automatic).
int geqrf(ddla_handle h, i64 m, i64 n, View<double> A, View<double> T, i64 tb, int prec = DDLA_PREC_FP64,
          int wcap = 0);
// oz_min_b: smallest block that takes the split-precision products (0 = 64).
int ormqr(ddla_handle h, bool trans, i64 m, i64 n, View<const double> A, View<const double> T, i64 tb,
          View<double> B, int prec = DDLA_PREC_FP64, int oz_min_b = 0);
int geqrs(ddla_handle h, i64 m, i64 n, View<const double> A, View<const double> T, i64 tb, View<const double> B,
          View<double> Y, View<double> X);
int orgqr(ddla_handle h, i64 m, i64 n, View<const double> A, View<const double> T, i64 tb, View<double> Q,
          int prec = DDLA_PREC_FP64);
// One block reflector of those factors (qr.cu): S (b x b) = triu(U^T U) with
// tau on the diagonal for the unit-lower m x b U stored below Ub's diagonal,
// and C = (I - U S^-1 U^T)^T C (trans) or (I - U S^-1 U^T) C with W a
// b x C.cols scratch.
int qr_tfactor(ddla_handle h, View<const double> Ub, i64 b, const double *tau, View<double> S);
int qr_apply_block(ddla_handle h, bool trans, View<const double> Ub, i64 b, View<const double> S, View<double> Cm,
                   double *W, int prec = DDLA_PREC_FP64, int oz_min_b = 0);
// Tridiagonaling.Tridiag on device data (tridiag.cu): A (lower triangle read)
// becomes Q, d (n) and e (n - 1) the tridiagonal, T (tb rows) the factors.
int sytrd(ddla_handle h, i64 n, View<double> A, View<double> T, i64 tb, double *d, double *e,
          int prec = DDLA_PREC_FP64);
// Bidiagonaling.Bidiag2 on device data (bidiag.cu), m >= n: A becomes the
// reflectors, d (n) / e (n - 1) the upper bidiagonal, U (m x m) and V (n x n)
// the orthogonal factors with U^T A V = bidiag(d, e).
int bidiag(ddla_handle h, i64 m, i64 n, View<double> A, double *d, double *e, View<double> U, View<double> V,
           int prec = DDLA_PREC_FP64);
// Bidiagonaling.Bidiag (two-stage) on device data (bidiag2s.cu), m >= n: A
// becomes the band and zeros, U (m x m) and V (n x n) the orthogonal factors
// with U^T A V = bidiag(d, e).
int bidiag2s(ddla_handle h, i64 m, i64 n, View<double> A, View<double> U, View<double> V, double *d, double *e,
             int prec = DDLA_PREC_FP64);

// Triangular-solve building blocks (trsm.cu): inverses of the 64 x 64
// diagonal blocks, and the chained whole-system solve for <= 16 columns.
template <typename T>
int tri_inverse(ddla_handle h, bool lower, bool unit, View<const T> A, i64 n, T *inv);
template <typename T>
int trsv_apply(ddla_handle h, bool lower, View<const T> A, i64 n, const T *inv, T *X, i64 ldx, int nr,
               const T *mlast = nullptr);
// M_p = inv(A_pp) A_{p,p-1} (lower) or inv(A_pp) A_{p,p+1} (upper), TB x TB per
// block row, for trsv_apply's one-right-hand-side cluster solve.
template <typename T>
int tri_mlast(ddla_handle h, bool lower, View<const T> A, i64 n, const T *inv, T *M);
// Y = X element by element (any strides; trsm.cu).
template <typename T>
int copy2d_on(cudaStream_t s, View<const T> X, View<T> Y);
// Rows of B reordered by a permutation (forward: row k <- row perm[k]).
template <typename T>
int permute_rows(ddla_handle h, View<T> B, const int *perm, i64 n, bool forward);

}  // namespace ddla
