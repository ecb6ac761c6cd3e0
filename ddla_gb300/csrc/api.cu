// C ABI of libddla_gb300: handles, workspaces, host staging and the extern "C"
// entry points declared in include/ddla_gb300.h.
//
// Host-pointer entry points replace DDLA's P/Invoke calls into BLIS
// (DDLA/BLAS/Native/3m.cs:12-162) and its factorization classes
// (DDLA/Factorizations/LU.cs, Cholesky.cs, LDLT.cs).  They validate arguments
// the way DDLA's checked wrappers do (DDLA/BLAS/3m.cs:10-315: empty problems
// return early, mismatched shapes are rejected), stage the strided host views
// into device buffers, run the device implementation on the calling thread's
// handle and copy results back before returning.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace ddla {

std::atomic<int64_t> g_launches{0};
static thread_local std::string t_error;
void set_error(const std::string &msg) { t_error = msg; }

int workspace(ddla_handle h, int slot, size_t bytes, void **out) {
    Workspace &w = h->ws[slot];
    if (w.bytes < bytes) {
        if (w.ptr) {
            cudaStreamSynchronize(h->stream);
            cudaFree(w.ptr);
            w.ptr = nullptr;
            w.bytes = 0;
        }
        size_t want = bytes + bytes / 8 + 256;
        if (cudaMalloc(&w.ptr, want) != cudaSuccess) {
            cudaGetLastError();
            set_error("device workspace allocation of " + std::to_string(want) + " bytes failed");
            return DDLA_ERR_NOMEM;
        }
        w.bytes = want;
    }
    *out = w.ptr;
    return 0;
}

int max_dyn_smem(const void *fn, size_t optin, size_t *avail) {
    cudaFuncAttributes fa;
    DDLA_CUDA(cudaFuncGetAttributes(&fa, fn));
    size_t lim = optin > fa.sharedSizeBytes ? optin - fa.sharedSizeBytes : 0;
    DDLA_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim));
    *avail = lim;
    return 0;
}

int pinned(ddla_handle h, size_t bytes, void **out) {
    if (h->pinned_bytes < bytes) {
        if (h->pinned) {
            cudaStreamSynchronize(h->stream);
            cudaFreeHost(h->pinned);
        }
        h->pinned = nullptr;
        h->pinned_bytes = 0;
        if (cudaMallocHost(&h->pinned, bytes) != cudaSuccess) {
            cudaGetLastError();
            set_error("pinned host allocation failed");
            return DDLA_ERR_NOMEM;
        }
        h->pinned_bytes = bytes;
    }
    *out = h->pinned;
    return 0;
}

int reset_info(ddla_handle h) {
    static const int init[INFO_COUNT] = {INT32_MAX, 0, 0, 0};
    DDLA_CUDA(cudaMemcpyAsync(h->d_info, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    return 0;
}

int read_info(ddla_handle h, int *pivot) {
    int v[INFO_COUNT];
    DDLA_CUDA(cudaMemcpyAsync(v, h->d_info, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    DDLA_CUDA(cudaStreamSynchronize(h->stream));
    *pivot = (v[INFO_PIVOT] == INT32_MAX) ? 0 : v[INFO_PIVOT];
    if (v[INFO_TIMEOUT]) {
        set_error("a bounded device-side wait gave up");
        return DDLA_ERR_TIMEOUT;
    }
    return 0;
}

static int handle_init(ddla_handle h, void *stream) {
    DDLA_CUDA(cudaGetDevice(&h->device));
    cudaDeviceProp prop;
    DDLA_CUDA(cudaGetDeviceProperties(&prop, h->device));
    if (prop.major < 10) {
        set_error(std::string("device ") + prop.name + " is not a Blackwell (sm_10x) GPU");
        return DDLA_ERR_NO_DEVICE;
    }
    h->sm_count = prop.multiProcessorCount;
    h->smem_optin = prop.sharedMemPerBlockOptin;
    if (stream) {
        h->stream = (cudaStream_t)stream;
        h->own_stream = false;
    } else {
        DDLA_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    DDLA_CUDA(cudaMalloc(&h->d_info, sizeof(int) * INFO_COUNT));
    DDLA_CUDA(cudaEventCreate(&h->ev0));
    DDLA_CUDA(cudaEventCreate(&h->ev1));
    return reset_info(h);
}

static void handle_free(ddla_handle h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto &w : h->ws)
        if (w.ptr) cudaFree(w.ptr);
    if (h->pinned) cudaFreeHost(h->pinned);
    if (h->d_info) cudaFree(h->d_info);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->side) {
        cudaStreamSynchronize(h->side);
        cudaStreamDestroy(h->side);
    }
    if (h->ev_ready) cudaEventDestroy(h->ev_ready);
    if (h->ev_panel) cudaEventDestroy(h->ev_panel);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int default_handle(ddla_handle *out) {
    static thread_local ddla_handle t_handle = nullptr;
    if (!t_handle) {
        ddla_handle h = new ddla_handle_s();
        int rc = handle_init(h, nullptr);
        if (rc) {
            handle_free(h);
            return rc;
        }
        t_handle = h;
    }
    *out = t_handle;
    return 0;
}

// ------------------------------------------------------------------ staging
// A host view staged into a device buffer; the device copy keeps the host
// orientation when one stride is 1 (2-D copies), else is packed row-major.
struct Staged {
    double *d = nullptr;
    View<double> view{};
};

static bool rowwise(i64 rows, i64 cols, i64 rs, i64 cs) { return cs == 1 && (rows <= 1 || rs >= cols); }
static bool colwise(i64 rows, i64 cols, i64 rs, i64 cs) { return rs == 1 && (cols <= 1 || cs >= rows); }

static int stage_in(ddla_handle h, int slot, const double *hp, i64 rows, i64 cols, i64 rs, i64 cs, bool copy,
                    Staged *out) {
    size_t bytes = sizeof(double) * (size_t)(rows * cols > 0 ? rows * cols : 1);
    void *d;
    DDLA_TRY(workspace(h, slot, bytes, &d));
    out->d = (double *)d;
    if (rows == 0 || cols == 0) {
        out->view = View<double>{out->d, rows, cols, cols, 1};
        return 0;
    }
    if (rowwise(rows, cols, rs, cs)) {
        out->view = View<double>{out->d, rows, cols, cols, 1};
        if (copy)
            DDLA_CUDA(cudaMemcpy2DAsync(out->d, cols * 8, hp, (rows > 1 ? rs : cols) * 8, cols * 8, rows,
                                        cudaMemcpyHostToDevice, h->stream));
    } else if (colwise(rows, cols, rs, cs)) {
        out->view = View<double>{out->d, rows, cols, 1, rows};
        if (copy)
            DDLA_CUDA(cudaMemcpy2DAsync(out->d, rows * 8, hp, (cols > 1 ? cs : rows) * 8, rows * 8, cols,
                                        cudaMemcpyHostToDevice, h->stream));
    } else {
        out->view = View<double>{out->d, rows, cols, cols, 1};
        if (copy) {
            void *pin;
            DDLA_TRY(pinned(h, bytes, &pin));
            DDLA_CUDA(cudaStreamSynchronize(h->stream));
            double *pp = (double *)pin;
            for (i64 i = 0; i < rows; i++)
                for (i64 j = 0; j < cols; j++) pp[i * cols + j] = hp[i * rs + j * cs];
            DDLA_CUDA(cudaMemcpyAsync(out->d, pp, bytes, cudaMemcpyHostToDevice, h->stream));
            DDLA_CUDA(cudaStreamSynchronize(h->stream));
        }
    }
    return 0;
}

// Copies the device view back to the host view; `tri` limits the copy to one
// triangle (DDLA_LOWER / DDLA_UPPER incl. diagonal) so the other triangle of
// the caller's array is never touched.
static int stage_out(ddla_handle h, const Staged &s, double *hp, i64 rows, i64 cols, i64 rs, i64 cs,
                     int tri = DDLA_DENSE) {
    if (rows == 0 || cols == 0) return 0;
    const View<double> &v = s.view;
    if (tri == DDLA_DENSE && rowwise(rows, cols, rs, cs) && v.cs == 1) {
        DDLA_CUDA(cudaMemcpy2DAsync(hp, (rows > 1 ? rs : cols) * 8, v.p, cols * 8, cols * 8, rows,
                                    cudaMemcpyDeviceToHost, h->stream));
        DDLA_CUDA(cudaStreamSynchronize(h->stream));
        return 0;
    }
    if (tri == DDLA_DENSE && colwise(rows, cols, rs, cs) && v.rs == 1) {
        DDLA_CUDA(cudaMemcpy2DAsync(hp, (cols > 1 ? cs : rows) * 8, v.p, rows * 8, rows * 8, cols,
                                    cudaMemcpyDeviceToHost, h->stream));
        DDLA_CUDA(cudaStreamSynchronize(h->stream));
        return 0;
    }
    size_t bytes = sizeof(double) * (size_t)(rows * cols);
    void *pin;
    DDLA_TRY(pinned(h, bytes, &pin));
    DDLA_CUDA(cudaMemcpyAsync(pin, v.p, bytes, cudaMemcpyDeviceToHost, h->stream));
    DDLA_CUDA(cudaStreamSynchronize(h->stream));
    const double *pp = (const double *)pin;
    for (i64 i = 0; i < rows; i++)
        for (i64 j = 0; j < cols; j++) {
            if (tri == DDLA_LOWER && j > i) continue;
            if (tri == DDLA_UPPER && j < i) continue;
            hp[i * rs + j * cs] = pp[i * v.rs + j * v.cs];
        }
    return 0;
}

static int fprec(const ddla_opts *o) {
    return (o && o->precision == DDLA_PREC_OZAKI) ? DDLA_PREC_OZAKI : DDLA_PREC_FP64;
}

static View<const double> cv(const View<double> &v) { return View<const double>{v.p, v.rows, v.cols, v.rs, v.cs}; }

template <typename T>
int gemm_any(ddla_handle h, int prec, i64 m, i64 n, i64 k, T alpha, View<const T> A, View<const T> B, T beta,
             View<T> C, int uplo);

int gemm_ozaki(ddla_handle h, i64 m, i64 n, i64 k, double alpha, View<const double> A, View<const double> B,
               double beta, View<double> C, int uplo = DDLA_DENSE, i64 batch = 1,
               const i64 *d_offsets = nullptr);

template <>
int gemm_any<double>(ddla_handle h, int prec, i64 m, i64 n, i64 k, double alpha, View<const double> A,
                     View<const double> B, double beta, View<double> C, int uplo) {
    if (prec == DDLA_PREC_OZAKI) return gemm_ozaki(h, m, n, k, alpha, A, B, beta, C, uplo);
    return gemm_f64(h->stream, m, n, k, alpha, A, B, beta, C, uplo);
}

int gemm_tc(ddla_handle h, int prec, i64 m, i64 n, i64 k, float alpha, View<const float> A, View<const float> B,
            float beta, View<float> C, int uplo);

template <>
int gemm_any<float>(ddla_handle h, int prec, i64 m, i64 n, i64 k, float alpha, View<const float> A,
                    View<const float> B, float beta, View<float> C, int uplo) {
    if (prec == DDLA_PREC_TF32X3 || prec == DDLA_PREC_BF16X3)
        return gemm_tc(h, prec, m, n, k, alpha, A, B, beta, C, uplo);
    return gemm_f32(h->stream, m, n, k, alpha, A, B, beta, C, uplo);
}

}  // namespace ddla

using namespace ddla;

// ------------------------------------------------------------------ argument checks
#define CHECK_ARG(cond, pos)                                                         \
    do {                                                                             \
        if (!(cond)) {                                                               \
            set_error(std::string("invalid argument ") + std::to_string(pos) + ": " #cond); \
            return -(pos);                                                           \
        }                                                                            \
    } while (0)

static bool valid_trans(int t) { return t == DDLA_NO_TRANSPOSE || t == DDLA_TRANSPOSE || t == DDLA_CONJ_NO_TRANSPOSE || t == DDLA_CONJ_TRANSPOSE; }
static bool is_trans(int t) { return (t & DDLA_TRANSPOSE) != 0; }
static bool valid_tri(int u) { return u == DDLA_LOWER || u == DDLA_UPPER; }

static bool valid_conj(int c) { return c == 0 || c == 0x10; }  // ConjType, DDLA/Misc/Flags/ConjType.cs

// op(X) as a view of shape rows x cols, X stored with strides (rs, cs).
static View<const double> op_view(const double *p, i64 rows, i64 cols, i64 rs, i64 cs, int trans) {
    if (is_trans(trans)) return View<const double>{p, cols, rows, rs, cs}.t();
    return View<const double>{p, rows, cols, rs, cs};
}

// Structured-operand mode of a triangular op(A) (transposing flips the triangle).
static int tri_mode(int uplo, int trans, int diag) {
    int u = is_trans(trans) ? flip_uplo(uplo) : uplo;
    return OP_TRI | (u == DDLA_LOWER ? OP_LOWER : 0) | (diag == DDLA_UNIT_DIAG ? OP_UNIT : 0);
}

// SYMM on device views: A the symmetric na x na operand, opB m x n.
// DDLA/BLAS/Managed/3m.cs:144-188 (the operands trade places on the right).
static int symm_dev(ddla_handle h, int side, int uplo, i64 m, i64 n, double alpha, View<const double> A,
                    View<const double> opB, double beta, View<double> C) {
    int mode = OP_SYM | (uplo == DDLA_LOWER ? OP_LOWER : 0);
    if (side == DDLA_LEFT) return gemm_f64_struct(h->stream, m, n, m, alpha, A, mode, opB, OP_DENSE, beta, C);
    return gemm_f64_struct(h->stream, m, n, n, alpha, opB, OP_DENSE, A, mode, beta, C);
}

// TRMM3 on device views: A the stored na x na triangle, opB m x n.
// DDLA/BLAS/Managed/3m.cs:308-356.
static int trmm3_dev(ddla_handle h, int side, int uplo, int ta, int diag, i64 m, i64 n, double alpha,
                     View<const double> A, View<const double> opB, double beta, View<double> C) {
    View<const double> opA = is_trans(ta) ? A.t() : A;
    int mode = tri_mode(uplo, ta, diag);
    if (side == DDLA_LEFT) return gemm_f64_struct(h->stream, m, n, m, alpha, opA, mode, opB, OP_DENSE, beta, C);
    return gemm_f64_struct(h->stream, m, n, n, alpha, opB, OP_DENSE, opA, mode, beta, C);
}

// SYR2K as two triangle-only GEMMs, DDLA/BLAS/Managed/3m.cs:227-246.
static int syr2k_dev(ddla_handle h, int uplo, i64 m, i64 k, double alpha, View<const double> opA,
                     View<const double> opB, double beta, View<double> C) {
    DDLA_TRY(gemm_f64(h->stream, m, m, k, alpha, opA, opB.t(), beta, C, uplo));
    return gemm_f64(h->stream, m, m, k, alpha, opB, opA.t(), 1.0, C, uplo);
}

#define GET_HANDLE(h)                  \
    ddla_handle h;                     \
    do {                               \
        int rc_ = default_handle(&h);  \
        if (rc_) return rc_;           \
    } while (0)

extern "C" {

const char *ddla_last_error(void) { return t_error.c_str(); }
const char *ddla_version(void) { return "ddla_gb300 0.1 (sm_103a)"; }
int64_t ddla_kernel_launches(void) { return g_launches.load(); }

int ddla_handle_create(ddla_handle *h, void *stream) {
    CHECK_ARG(h != nullptr, 1);
    ddla_handle x = new ddla_handle_s();
    int rc = handle_init(x, stream);
    if (rc) {
        handle_free(x);
        return rc;
    }
    *h = x;
    return 0;
}

int ddla_handle_destroy(ddla_handle h) {
    handle_free(h);
    return 0;
}

int ddla_handle_sync(ddla_handle h) {
    DDLA_CUDA(cudaStreamSynchronize(h->stream));
    return 0;
}

// ------------------------------------------------------------------ level 3, device
int ddla_dev_dgemm(ddla_handle h, int32_t ta, int32_t tb, ddla_dim_t m, ddla_dim_t n, ddla_dim_t k, double alpha,
                   const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b, ddla_inc_t rsb,
                   ddla_inc_t csb, double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(valid_trans(ta), 2);
    CHECK_ARG(valid_trans(tb), 3);
    CHECK_ARG(m >= 0, 4);
    CHECK_ARG(n >= 0, 5);
    CHECK_ARG(k >= 0, 6);
    if (m == 0 || n == 0) return 0;
    View<const double> A{a, is_trans(ta) ? k : m, is_trans(ta) ? m : k, rsa, csa};
    View<const double> B{b, is_trans(tb) ? n : k, is_trans(tb) ? k : n, rsb, csb};
    if (is_trans(ta)) A = A.t();
    if (is_trans(tb)) B = B.t();
    return gemm_f64(h->stream, m, n, k, alpha, A, B, beta, View<double>{c, m, n, rsc, csc});
}

int ddla_dev_dgemm_ex(ddla_handle h, int32_t precision, int32_t ta, int32_t tb, ddla_dim_t m, ddla_dim_t n,
                      ddla_dim_t k, double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b,
                      ddla_inc_t rsb, ddla_inc_t csb, double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(precision == DDLA_PREC_FP64 || precision == DDLA_PREC_OZAKI, 2);
    CHECK_ARG(valid_trans(ta), 3);
    CHECK_ARG(valid_trans(tb), 4);
    CHECK_ARG(m >= 0, 5);
    CHECK_ARG(n >= 0, 6);
    CHECK_ARG(k >= 0, 7);
    if (m == 0 || n == 0) return 0;
    View<const double> A{a, is_trans(ta) ? k : m, is_trans(ta) ? m : k, rsa, csa};
    View<const double> B{b, is_trans(tb) ? n : k, is_trans(tb) ? k : n, rsb, csb};
    if (is_trans(ta)) A = A.t();
    if (is_trans(tb)) B = B.t();
    View<double> C{c, m, n, rsc, csc};
    if (precision == DDLA_PREC_OZAKI) return gemm_ozaki(h, m, n, k, alpha, A, B, beta, C);
    return gemm_f64(h->stream, m, n, k, alpha, A, B, beta, C);
}

int ddla_dev_dgemmt(ddla_handle h, int32_t uplo, int32_t ta, int32_t tb, ddla_dim_t m, ddla_dim_t k, double alpha,
                    const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b, ddla_inc_t rsb,
                    ddla_inc_t csb, double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(valid_tri(uplo), 2);
    CHECK_ARG(valid_trans(ta), 3);
    CHECK_ARG(valid_trans(tb), 4);
    CHECK_ARG(m >= 0, 5);
    CHECK_ARG(k >= 0, 6);
    if (m == 0) return 0;
    View<const double> A{a, is_trans(ta) ? k : m, is_trans(ta) ? m : k, rsa, csa};
    View<const double> B{b, is_trans(tb) ? m : k, is_trans(tb) ? k : m, rsb, csb};
    if (is_trans(ta)) A = A.t();
    if (is_trans(tb)) B = B.t();
    return gemm_f64(h->stream, m, m, k, alpha, A, B, beta, View<double>{c, m, m, rsc, csc}, uplo);
}

int ddla_dev_dtrsm(ddla_handle h, int32_t side, int32_t uplo, int32_t ta, int32_t diag, ddla_dim_t m, ddla_dim_t n,
                   double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa, double *b, ddla_inc_t rsb,
                   ddla_inc_t csb) {
    CHECK_ARG(side == DDLA_LEFT || side == DDLA_RIGHT, 2);
    CHECK_ARG(valid_tri(uplo), 3);
    CHECK_ARG(valid_trans(ta), 4);
    CHECK_ARG(diag == DDLA_UNIT_DIAG || diag == DDLA_NONUNIT_DIAG, 5);
    CHECK_ARG(m >= 0, 6);
    CHECK_ARG(n >= 0, 7);
    if (m == 0 || n == 0) return 0;
    i64 na = side == DDLA_LEFT ? m : n;
    return trsm<double>(h, side, uplo, ta, diag, m, n, alpha, View<const double>{a, na, na, rsa, csa},
                        View<double>{b, m, n, rsb, csb});
}

int ddla_dev_dsymm(ddla_handle h, int32_t side, int32_t uplo, int32_t conja, int32_t tb, ddla_dim_t m, ddla_dim_t n,
                   double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b, ddla_inc_t rsb,
                   ddla_inc_t csb, double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(side == DDLA_LEFT || side == DDLA_RIGHT, 2);
    CHECK_ARG(valid_tri(uplo), 3);
    CHECK_ARG(valid_conj(conja), 4);
    CHECK_ARG(valid_trans(tb), 5);
    CHECK_ARG(m >= 0, 6);
    CHECK_ARG(n >= 0, 7);
    if (m == 0 || n == 0) return 0;
    i64 na = side == DDLA_LEFT ? m : n;
    return symm_dev(h, side, uplo, m, n, alpha, View<const double>{a, na, na, rsa, csa},
                    op_view(b, m, n, rsb, csb, tb), beta, View<double>{c, m, n, rsc, csc});
}

int ddla_dev_dsyr2k(ddla_handle h, int32_t uplo, int32_t ta, int32_t tb, ddla_dim_t m, ddla_dim_t k, double alpha,
                    const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b, ddla_inc_t rsb,
                    ddla_inc_t csb, double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(valid_tri(uplo), 2);
    CHECK_ARG(valid_trans(ta), 3);
    CHECK_ARG(valid_trans(tb), 4);
    CHECK_ARG(m >= 0, 5);
    CHECK_ARG(k >= 0, 6);
    if (m == 0) return 0;
    return syr2k_dev(h, uplo, m, k, alpha, op_view(a, m, k, rsa, csa, ta), op_view(b, m, k, rsb, csb, tb), beta,
                     View<double>{c, m, m, rsc, csc});
}

int ddla_dev_dtrmm(ddla_handle h, int32_t side, int32_t uplo, int32_t ta, int32_t diag, ddla_dim_t m, ddla_dim_t n,
                   double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa, double *b, ddla_inc_t rsb,
                   ddla_inc_t csb) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(side == DDLA_LEFT || side == DDLA_RIGHT, 2);
    CHECK_ARG(valid_tri(uplo), 3);
    CHECK_ARG(valid_trans(ta), 4);
    CHECK_ARG(diag == DDLA_UNIT_DIAG || diag == DDLA_NONUNIT_DIAG, 5);
    CHECK_ARG(m >= 0, 6);
    CHECK_ARG(n >= 0, 7);
    if (m == 0 || n == 0) return 0;
    i64 na = side == DDLA_LEFT ? m : n;
    void *tmp;
    DDLA_TRY(workspace(h, WS_TMP, sizeof(double) * (size_t)(m * n), &tmp));
    View<double> Bc{(double *)tmp, m, n, n, 1};
    View<double> Bv{b, m, n, rsb, csb};
    DDLA_TRY(copy2d_on<double>(h->stream, cv(Bv), Bc));
    return trmm3_dev(h, side, uplo, ta, diag, m, n, alpha, View<const double>{a, na, na, rsa, csa}, cv(Bc), 0.0, Bv);
}

int ddla_dev_dtrmm3(ddla_handle h, int32_t side, int32_t uplo, int32_t ta, int32_t diag, int32_t tb, ddla_dim_t m,
                    ddla_dim_t n, double alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b,
                    ddla_inc_t rsb, ddla_inc_t csb, double beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(side == DDLA_LEFT || side == DDLA_RIGHT, 2);
    CHECK_ARG(valid_tri(uplo), 3);
    CHECK_ARG(valid_trans(ta), 4);
    CHECK_ARG(diag == DDLA_UNIT_DIAG || diag == DDLA_NONUNIT_DIAG, 5);
    CHECK_ARG(valid_trans(tb), 6);
    CHECK_ARG(m >= 0, 7);
    CHECK_ARG(n >= 0, 8);
    if (m == 0 || n == 0) return 0;
    i64 na = side == DDLA_LEFT ? m : n;
    return trmm3_dev(h, side, uplo, ta, diag, m, n, alpha, View<const double>{a, na, na, rsa, csa},
                     op_view(b, m, n, rsb, csb, tb), beta, View<double>{c, m, n, rsc, csc});
}

// ------------------------------------------------------------------ level 3, host
int ddla_dgemm(int32_t ta, int32_t tb, ddla_dim_t m, ddla_dim_t n, ddla_dim_t k, const double *alpha,
               const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b, ddla_inc_t rsb, ddla_inc_t csb,
               const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(valid_trans(ta), 1);
    CHECK_ARG(valid_trans(tb), 2);
    CHECK_ARG(m >= 0, 3);
    CHECK_ARG(n >= 0, 4);
    CHECK_ARG(k >= 0, 5);
    CHECK_ARG(alpha != nullptr, 6);
    CHECK_ARG(beta != nullptr, 13);
    if (m == 0 || n == 0) return 0;
    GET_HANDLE(h);
    i64 ar = is_trans(ta) ? k : m, ac = is_trans(ta) ? m : k;
    i64 br = is_trans(tb) ? n : k, bc = is_trans(tb) ? k : n;
    Staged sa, sb, sc;
    DDLA_TRY(stage_in(h, WS_A, a, ar, ac, rsa, csa, k > 0, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, br, bc, rsb, csb, k > 0, &sb));
    DDLA_TRY(stage_in(h, WS_C, c, m, n, rsc, csc, *beta != 0.0, &sc));
    View<const double> A = cv(sa.view), B = cv(sb.view);
    if (is_trans(ta)) A = A.t();
    if (is_trans(tb)) B = B.t();
    DDLA_TRY(gemm_f64(h->stream, m, n, k, *alpha, A, B, *beta, sc.view));
    return stage_out(h, sc, c, m, n, rsc, csc);
}

int ddla_dgemmt(int32_t uplo, int32_t ta, int32_t tb, ddla_dim_t m, ddla_dim_t k, const double *alpha,
                const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(valid_tri(uplo), 1);
    CHECK_ARG(valid_trans(ta), 2);
    CHECK_ARG(valid_trans(tb), 3);
    CHECK_ARG(m >= 0, 4);
    CHECK_ARG(k >= 0, 5);
    CHECK_ARG(alpha != nullptr, 6);
    CHECK_ARG(beta != nullptr, 13);
    if (m == 0) return 0;
    GET_HANDLE(h);
    i64 ar = is_trans(ta) ? k : m, ac = is_trans(ta) ? m : k;
    i64 br = is_trans(tb) ? m : k, bc = is_trans(tb) ? k : m;
    Staged sa, sb, sc;
    DDLA_TRY(stage_in(h, WS_A, a, ar, ac, rsa, csa, k > 0, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, br, bc, rsb, csb, k > 0, &sb));
    DDLA_TRY(stage_in(h, WS_C, c, m, m, rsc, csc, *beta != 0.0, &sc));
    View<const double> A = cv(sa.view), B = cv(sb.view);
    if (is_trans(ta)) A = A.t();
    if (is_trans(tb)) B = B.t();
    DDLA_TRY(gemm_f64(h->stream, m, m, k, *alpha, A, B, *beta, sc.view, uplo));
    return stage_out(h, sc, c, m, m, rsc, csc, uplo);
}

int ddla_dsyrk(int32_t uplo, int32_t ta, ddla_dim_t m, ddla_dim_t k, const double *alpha, const double *a,
               ddla_inc_t rsa, ddla_inc_t csa, const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(valid_tri(uplo), 1);
    CHECK_ARG(valid_trans(ta), 2);
    CHECK_ARG(m >= 0, 3);
    CHECK_ARG(k >= 0, 4);
    CHECK_ARG(alpha != nullptr, 5);
    CHECK_ARG(beta != nullptr, 9);
    if (m == 0) return 0;
    GET_HANDLE(h);
    i64 ar = is_trans(ta) ? k : m, ac = is_trans(ta) ? m : k;
    Staged sa, sc;
    DDLA_TRY(stage_in(h, WS_A, a, ar, ac, rsa, csa, k > 0, &sa));
    DDLA_TRY(stage_in(h, WS_C, c, m, m, rsc, csc, *beta != 0.0, &sc));
    View<const double> A = cv(sa.view);
    if (is_trans(ta)) A = A.t();
    DDLA_TRY(gemm_f64(h->stream, m, m, k, *alpha, A, A.t(), *beta, sc.view, uplo));
    return stage_out(h, sc, c, m, m, rsc, csc, uplo);
}

int ddla_dtrsm(int32_t side, int32_t uplo, int32_t ta, int32_t diag, ddla_dim_t m, ddla_dim_t n,
               const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa, double *b, ddla_inc_t rsb,
               ddla_inc_t csb) {
    CHECK_ARG(side == DDLA_LEFT || side == DDLA_RIGHT, 1);
    CHECK_ARG(valid_tri(uplo), 2);
    CHECK_ARG(valid_trans(ta), 3);
    CHECK_ARG(diag == DDLA_UNIT_DIAG || diag == DDLA_NONUNIT_DIAG, 4);
    CHECK_ARG(m >= 0, 5);
    CHECK_ARG(n >= 0, 6);
    CHECK_ARG(alpha != nullptr, 7);
    if (m == 0 || n == 0) return 0;
    GET_HANDLE(h);
    i64 na = side == DDLA_LEFT ? m : n;
    Staged sa, sb;
    DDLA_TRY(stage_in(h, WS_A, a, na, na, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, m, n, rsb, csb, true, &sb));
    DDLA_TRY(trsm<double>(h, side, uplo, ta, diag, m, n, *alpha, cv(sa.view), sb.view));
    return stage_out(h, sb, b, m, n, rsb, csb);
}

int ddla_dsymm(int32_t side, int32_t uplo, int32_t conja, int32_t tb, ddla_dim_t m, ddla_dim_t n, const double *alpha,
               const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b, ddla_inc_t rsb, ddla_inc_t csb,
               const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(side == DDLA_LEFT || side == DDLA_RIGHT, 1);
    CHECK_ARG(valid_tri(uplo), 2);
    CHECK_ARG(valid_conj(conja), 3);
    CHECK_ARG(valid_trans(tb), 4);
    CHECK_ARG(m >= 0, 5);
    CHECK_ARG(n >= 0, 6);
    CHECK_ARG(alpha != nullptr, 7);
    CHECK_ARG(beta != nullptr, 14);
    if (m == 0 || n == 0) return 0;
    GET_HANDLE(h);
    i64 na = side == DDLA_LEFT ? m : n;
    Staged sa, sb, sc;
    DDLA_TRY(stage_in(h, WS_A, a, na, na, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, is_trans(tb) ? n : m, is_trans(tb) ? m : n, rsb, csb, true, &sb));
    DDLA_TRY(stage_in(h, WS_C, c, m, n, rsc, csc, *beta != 0.0, &sc));
    View<const double> B = cv(sb.view);
    if (is_trans(tb)) B = B.t();
    DDLA_TRY(symm_dev(h, side, uplo, m, n, *alpha, cv(sa.view), B, *beta, sc.view));
    return stage_out(h, sc, c, m, n, rsc, csc);
}

int ddla_dsyr2k(int32_t uplo, int32_t ta, int32_t tb, ddla_dim_t m, ddla_dim_t k, const double *alpha,
                const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b, ddla_inc_t rsb, ddla_inc_t csb,
                const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(valid_tri(uplo), 1);
    CHECK_ARG(valid_trans(ta), 2);
    CHECK_ARG(valid_trans(tb), 3);
    CHECK_ARG(m >= 0, 4);
    CHECK_ARG(k >= 0, 5);
    CHECK_ARG(alpha != nullptr, 6);
    CHECK_ARG(beta != nullptr, 13);
    if (m == 0) return 0;
    GET_HANDLE(h);
    i64 ar = is_trans(ta) ? k : m, ac = is_trans(ta) ? m : k;
    i64 br = is_trans(tb) ? k : m, bc = is_trans(tb) ? m : k;
    Staged sa, sb, sc;
    DDLA_TRY(stage_in(h, WS_A, a, ar, ac, rsa, csa, k > 0, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, br, bc, rsb, csb, k > 0, &sb));
    DDLA_TRY(stage_in(h, WS_C, c, m, m, rsc, csc, *beta != 0.0, &sc));
    View<const double> A = cv(sa.view), B = cv(sb.view);
    if (is_trans(ta)) A = A.t();
    if (is_trans(tb)) B = B.t();
    DDLA_TRY(syr2k_dev(h, uplo, m, k, *alpha, A, B, *beta, sc.view));
    return stage_out(h, sc, c, m, m, rsc, csc, uplo);
}

int ddla_dtrmm(int32_t side, int32_t uplo, int32_t ta, int32_t diag, ddla_dim_t m, ddla_dim_t n, const double *alpha,
               const double *a, ddla_inc_t rsa, ddla_inc_t csa, double *b, ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(side == DDLA_LEFT || side == DDLA_RIGHT, 1);
    CHECK_ARG(valid_tri(uplo), 2);
    CHECK_ARG(valid_trans(ta), 3);
    CHECK_ARG(diag == DDLA_UNIT_DIAG || diag == DDLA_NONUNIT_DIAG, 4);
    CHECK_ARG(m >= 0, 5);
    CHECK_ARG(n >= 0, 6);
    CHECK_ARG(alpha != nullptr, 7);
    if (m == 0 || n == 0) return 0;
    GET_HANDLE(h);
    i64 na = side == DDLA_LEFT ? m : n;
    Staged sa, sb, sc;
    DDLA_TRY(stage_in(h, WS_A, a, na, na, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, m, n, rsb, csb, true, &sb));
    DDLA_TRY(stage_in(h, WS_C, b, m, n, rsb, csb, false, &sc));   // product lands here, then back in b
    DDLA_TRY(trmm3_dev(h, side, uplo, ta, diag, m, n, *alpha, cv(sa.view), cv(sb.view), 0.0, sc.view));
    return stage_out(h, sc, b, m, n, rsb, csb);
}

int ddla_dtrmm3(int32_t side, int32_t uplo, int32_t ta, int32_t diag, int32_t tb, ddla_dim_t m, ddla_dim_t n,
                const double *alpha, const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *b, ddla_inc_t rsb,
                ddla_inc_t csb, const double *beta, double *c, ddla_inc_t rsc, ddla_inc_t csc) {
    CHECK_ARG(side == DDLA_LEFT || side == DDLA_RIGHT, 1);
    CHECK_ARG(valid_tri(uplo), 2);
    CHECK_ARG(valid_trans(ta), 3);
    CHECK_ARG(diag == DDLA_UNIT_DIAG || diag == DDLA_NONUNIT_DIAG, 4);
    CHECK_ARG(valid_trans(tb), 5);
    CHECK_ARG(m >= 0, 6);
    CHECK_ARG(n >= 0, 7);
    CHECK_ARG(alpha != nullptr, 8);
    CHECK_ARG(beta != nullptr, 15);
    if (m == 0 || n == 0) return 0;
    GET_HANDLE(h);
    i64 na = side == DDLA_LEFT ? m : n;
    Staged sa, sb, sc;
    DDLA_TRY(stage_in(h, WS_A, a, na, na, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, is_trans(tb) ? n : m, is_trans(tb) ? m : n, rsb, csb, true, &sb));
    DDLA_TRY(stage_in(h, WS_C, c, m, n, rsc, csc, *beta != 0.0, &sc));
    View<const double> B = cv(sb.view);
    if (is_trans(tb)) B = B.t();
    DDLA_TRY(trmm3_dev(h, side, uplo, ta, diag, m, n, *alpha, cv(sa.view), B, *beta, sc.view));
    return stage_out(h, sc, c, m, n, rsc, csc);
}

// ------------------------------------------------------------------ QR
int ddla_dev_dgeqrf(ddla_handle h, ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *t,
                    ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst, const ddla_opts *opts) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(m >= 0, 2);
    CHECK_ARG(n >= 0, 3);
    CHECK_ARG(t_rows >= 1, 8);
    CHECK_ARG(!opts || opts->precision == 0 || opts->precision == DDLA_PREC_FP64 ||
                  opts->precision == DDLA_PREC_OZAKI, 11);
    if (m == 0 || n == 0) return 0;
    return geqrf(h, m, n, View<double>{a, m, n, rsa, csa}, View<double>{t, t_rows, n, rst, cst}, t_rows, fprec(opts),
                 opts ? opts->nb : 0);
}

int ddla_dev_dormqr(ddla_handle h, int32_t trans, ddla_dim_t m, ddla_dim_t n, ddla_dim_t nrhs, const double *a,
                    ddla_inc_t rsa, ddla_inc_t csa, const double *t, ddla_dim_t t_rows, ddla_inc_t rst,
                    ddla_inc_t cst, double *b, ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(m >= 0, 3);
    CHECK_ARG(n >= 0, 4);
    CHECK_ARG(nrhs >= 0, 5);
    CHECK_ARG(t_rows >= 1, 10);
    if (m == 0 || n == 0 || nrhs == 0) return 0;
    return ormqr(h, trans != 0, m, n, View<const double>{a, m, n, rsa, csa},
                 View<const double>{t, t_rows, n, rst, cst}, t_rows, View<double>{b, m, nrhs, rsb, csb});
}

int ddla_dev_dgeqrs(ddla_handle h, ddla_dim_t m, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa,
                    ddla_inc_t csa, const double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst,
                    const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(m >= 0, 2);
    CHECK_ARG(n >= 0 && n <= m, 3);
    CHECK_ARG(nrhs >= 0, 4);
    CHECK_ARG(t_rows >= 1, 9);
    if (n == 0 || nrhs == 0) return 0;
    void *y;
    DDLA_TRY(workspace(h, WS_Y, sizeof(double) * (size_t)(m * nrhs), &y));
    return geqrs(h, m, n, View<const double>{a, m, n, rsa, csa}, View<const double>{t, t_rows, n, rst, cst}, t_rows,
                 View<const double>{b, m, nrhs, rsb, csb}, View<double>{(double *)y, m, nrhs, nrhs, 1},
                 View<double>{x, n, nrhs, rsx, csx});
}

int ddla_dev_dorgqr(ddla_handle h, ddla_dim_t m, ddla_dim_t n, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                    const double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst, double *q, ddla_inc_t rsq,
                    ddla_inc_t csq) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(m >= 0, 2);
    CHECK_ARG(n >= 0, 3);
    CHECK_ARG(t_rows >= 1, 8);
    if (m == 0) return 0;
    return orgqr(h, m, n, View<const double>{a, m, n, rsa, csa}, View<const double>{t, t_rows, n, rst, cst}, t_rows,
                 View<double>{q, m, m, rsq, csq});
}

int ddla_dgeqrf(ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *t, ddla_dim_t t_rows,
                ddla_inc_t rst, ddla_inc_t cst, const ddla_opts *opts) {
    CHECK_ARG(m >= 0, 1);
    CHECK_ARG(n >= 0, 2);
    CHECK_ARG(t_rows >= 1, 7);
    CHECK_ARG(!opts || opts->precision == 0 || opts->precision == DDLA_PREC_FP64 ||
                  opts->precision == DDLA_PREC_OZAKI, 10);
    if (m == 0 || n == 0) return 0;
    GET_HANDLE(h);
    Staged sa, st;
    DDLA_TRY(stage_in(h, WS_A, a, m, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_C, t, t_rows, n, rst, cst, true, &st));
    DDLA_TRY(geqrf(h, m, n, sa.view, st.view, t_rows, fprec(opts), opts ? opts->nb : 0));
    DDLA_TRY(stage_out(h, sa, a, m, n, rsa, csa));
    return stage_out(h, st, t, t_rows, n, rst, cst);
}

int ddla_dormqr(int32_t trans, ddla_dim_t m, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa,
                ddla_inc_t csa, const double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst, double *b,
                ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(m >= 0, 2);
    CHECK_ARG(n >= 0, 3);
    CHECK_ARG(nrhs >= 0, 4);
    CHECK_ARG(t_rows >= 1, 9);
    if (m == 0 || n == 0 || nrhs == 0) return 0;
    GET_HANDLE(h);
    Staged sa, st, sb;
    DDLA_TRY(stage_in(h, WS_A, a, m, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_C, t, t_rows, n, rst, cst, true, &st));
    DDLA_TRY(stage_in(h, WS_B, b, m, nrhs, rsb, csb, true, &sb));
    DDLA_TRY(ormqr(h, trans != 0, m, n, cv(sa.view), cv(st.view), t_rows, sb.view));
    return stage_out(h, sb, b, m, nrhs, rsb, csb);
}

int ddla_dgeqrs(ddla_dim_t m, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                const double *t, ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst, const double *b, ddla_inc_t rsb,
                ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx) {
    CHECK_ARG(m >= 0, 1);
    CHECK_ARG(n >= 0 && n <= m, 2);
    CHECK_ARG(nrhs >= 0, 3);
    CHECK_ARG(t_rows >= 1, 8);
    if (n == 0 || nrhs == 0) return 0;
    GET_HANDLE(h);
    Staged sa, st, sb, sx;
    DDLA_TRY(stage_in(h, WS_A, a, m, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_C, t, t_rows, n, rst, cst, true, &st));
    DDLA_TRY(stage_in(h, WS_B, b, m, nrhs, rsb, csb, true, &sb));
    DDLA_TRY(stage_in(h, WS_F32, x, n, nrhs, rsx, csx, false, &sx));
    void *y;
    DDLA_TRY(workspace(h, WS_Y, sizeof(double) * (size_t)(m * nrhs), &y));
    DDLA_TRY(geqrs(h, m, n, cv(sa.view), cv(st.view), t_rows, cv(sb.view),
                   View<double>{(double *)y, m, nrhs, nrhs, 1}, sx.view));
    return stage_out(h, sx, x, n, nrhs, rsx, csx);
}

int ddla_dorgqr(ddla_dim_t m, ddla_dim_t n, const double *a, ddla_inc_t rsa, ddla_inc_t csa, const double *t,
                ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst, double *q, ddla_inc_t rsq, ddla_inc_t csq) {
    CHECK_ARG(m >= 0, 1);
    CHECK_ARG(n >= 0, 2);
    CHECK_ARG(t_rows >= 1, 7);
    if (m == 0) return 0;
    GET_HANDLE(h);
    Staged sa, st, sq;
    DDLA_TRY(stage_in(h, WS_A, a, m, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_C, t, t_rows, n, rst, cst, true, &st));
    DDLA_TRY(stage_in(h, WS_B, q, m, m, rsq, csq, false, &sq));
    DDLA_TRY(orgqr(h, m, n, cv(sa.view), cv(st.view), t_rows, sq.view));
    return stage_out(h, sq, q, m, m, rsq, csq);
}

// ------------------------------------------------------------------ tridiagonal reduction
int ddla_dev_dsytrd(ddla_handle h, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *t,
                    ddla_dim_t t_rows, ddla_inc_t rst, ddla_inc_t cst, double *d, double *e, const ddla_opts *opts) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(n >= 0, 2);
    CHECK_ARG(t_rows >= 1, 7);
    CHECK_ARG(d != nullptr || n == 0, 10);
    CHECK_ARG(e != nullptr || n <= 1, 11);
    CHECK_ARG(!opts || opts->precision == 0 || opts->precision == DDLA_PREC_FP64 ||
                  opts->precision == DDLA_PREC_OZAKI, 12);
    if (n == 0) return 0;
    return sytrd(h, n, View<double>{a, n, n, rsa, csa}, View<double>{t, t_rows, n, rst, cst}, t_rows, d, e,
                 fprec(opts));
}

int ddla_dsytrd(ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *t, ddla_dim_t t_rows, ddla_inc_t rst,
                ddla_inc_t cst, double *d, double *e, const ddla_opts *opts) {
    CHECK_ARG(n >= 0, 1);
    CHECK_ARG(t_rows >= 1, 6);
    CHECK_ARG(d != nullptr || n == 0, 9);
    CHECK_ARG(e != nullptr || n <= 1, 10);
    CHECK_ARG(!opts || opts->precision == 0 || opts->precision == DDLA_PREC_FP64 ||
                  opts->precision == DDLA_PREC_OZAKI, 11);
    if (n == 0) return 0;
    GET_HANDLE(h);
    Staged sa, st;
    DDLA_TRY(stage_in(h, WS_A, a, n, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_C, t, t_rows, n, rst, cst, true, &st));
    void *de;
    DDLA_TRY(workspace(h, WS_PIV, sizeof(double) * (size_t)(2 * n), &de));
    double *dd = (double *)de, *ed = dd + n;
    DDLA_TRY(sytrd(h, n, sa.view, st.view, t_rows, dd, ed, fprec(opts)));
    DDLA_TRY(stage_out(h, sa, a, n, n, rsa, csa));
    DDLA_TRY(stage_out(h, st, t, t_rows, n, rst, cst));
    DDLA_CUDA(cudaMemcpyAsync(d, dd, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
    if (n > 1) DDLA_CUDA(cudaMemcpyAsync(e, ed, sizeof(double) * (size_t)(n - 1), cudaMemcpyDeviceToHost, h->stream));
    DDLA_CUDA(cudaStreamSynchronize(h->stream));
    return 0;
}

// ------------------------------------------------------------------ bidiagonal reduction
int ddla_dev_dbidiag(ddla_handle h, ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *d,
                     double *e, double *u, ddla_inc_t rsu, ddla_inc_t csu, double *v, ddla_inc_t rsv, ddla_inc_t csv,
                     const ddla_opts *opts) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(m >= 0, 2);
    CHECK_ARG(n >= 0 && n <= m, 3);
    CHECK_ARG(d != nullptr || n == 0, 7);
    CHECK_ARG(e != nullptr || n <= 1, 8);
    CHECK_ARG(u != nullptr || m == 0, 9);
    CHECK_ARG(v != nullptr || n == 0, 12);
    CHECK_ARG(!opts || opts->precision == 0 || opts->precision == DDLA_PREC_FP64 ||
                  opts->precision == DDLA_PREC_OZAKI, 15);
    if (n == 0) return 0;
    return bidiag(h, m, n, View<double>{a, m, n, rsa, csa}, d, e, View<double>{u, m, m, rsu, csu},
                  View<double>{v, n, n, rsv, csv}, fprec(opts));
}

int ddla_dbidiag(ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *d, double *e,
                 double *u, ddla_inc_t rsu, ddla_inc_t csu, double *v, ddla_inc_t rsv, ddla_inc_t csv,
                 const ddla_opts *opts) {
    CHECK_ARG(m >= 0, 1);
    CHECK_ARG(n >= 0 && n <= m, 2);
    CHECK_ARG(d != nullptr || n == 0, 6);
    CHECK_ARG(e != nullptr || n <= 1, 7);
    CHECK_ARG(u != nullptr || m == 0, 8);
    CHECK_ARG(v != nullptr || n == 0, 11);
    CHECK_ARG(!opts || opts->precision == 0 || opts->precision == DDLA_PREC_FP64 ||
                  opts->precision == DDLA_PREC_OZAKI, 14);
    if (n == 0) return 0;
    GET_HANDLE(h);
    Staged sa, su, sv;
    DDLA_TRY(stage_in(h, WS_A, a, m, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, u, m, m, rsu, csu, false, &su));
    DDLA_TRY(stage_in(h, WS_C, v, n, n, rsv, csv, false, &sv));
    void *de;
    DDLA_TRY(workspace(h, WS_PIV, sizeof(double) * (size_t)(2 * n), &de));
    double *dd = (double *)de, *ed = dd + n;
    DDLA_TRY(bidiag(h, m, n, sa.view, dd, ed, su.view, sv.view, fprec(opts)));
    DDLA_TRY(stage_out(h, sa, a, m, n, rsa, csa));
    DDLA_TRY(stage_out(h, su, u, m, m, rsu, csu));
    DDLA_TRY(stage_out(h, sv, v, n, n, rsv, csv));
    DDLA_CUDA(cudaMemcpyAsync(d, dd, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
    if (n > 1) DDLA_CUDA(cudaMemcpyAsync(e, ed, sizeof(double) * (size_t)(n - 1), cudaMemcpyDeviceToHost, h->stream));
    DDLA_CUDA(cudaStreamSynchronize(h->stream));
    return 0;
}

int ddla_dev_dbidiag_twostage(ddla_handle h, ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa,
                              ddla_inc_t csa, double *d, double *e, double *u, ddla_inc_t rsu, ddla_inc_t csu,
                              double *v, ddla_inc_t rsv, ddla_inc_t csv, const ddla_opts *opts) {
    CHECK_ARG(h != nullptr, 1);
    CHECK_ARG(m >= 0, 2);
    CHECK_ARG(n >= 0 && n <= m, 3);
    CHECK_ARG(d != nullptr || n == 0, 7);
    CHECK_ARG(e != nullptr || n <= 1, 8);
    CHECK_ARG(u != nullptr || m == 0, 9);
    CHECK_ARG(v != nullptr || n == 0, 12);
    CHECK_ARG(!opts || opts->precision == 0 || opts->precision == DDLA_PREC_FP64 ||
                  opts->precision == DDLA_PREC_OZAKI, 15);
    if (n == 0) return 0;
    return bidiag2s(h, m, n, View<double>{a, m, n, rsa, csa}, View<double>{u, m, m, rsu, csu},
                    View<double>{v, n, n, rsv, csv}, d, e, fprec(opts));
}

int ddla_dbidiag_twostage(ddla_dim_t m, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, double *d,
                          double *e, double *u, ddla_inc_t rsu, ddla_inc_t csu, double *v, ddla_inc_t rsv,
                          ddla_inc_t csv, const ddla_opts *opts) {
    CHECK_ARG(m >= 0, 1);
    CHECK_ARG(n >= 0 && n <= m, 2);
    CHECK_ARG(d != nullptr || n == 0, 6);
    CHECK_ARG(e != nullptr || n <= 1, 7);
    CHECK_ARG(u != nullptr || m == 0, 8);
    CHECK_ARG(v != nullptr || n == 0, 11);
    CHECK_ARG(!opts || opts->precision == 0 || opts->precision == DDLA_PREC_FP64 ||
                  opts->precision == DDLA_PREC_OZAKI, 14);
    if (n == 0) return 0;
    GET_HANDLE(h);
    Staged sa, su, sv;
    DDLA_TRY(stage_in(h, WS_A, a, m, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, u, m, m, rsu, csu, false, &su));
    DDLA_TRY(stage_in(h, WS_C, v, n, n, rsv, csv, false, &sv));
    void *de;
    DDLA_TRY(workspace(h, WS_PIV, sizeof(double) * (size_t)(2 * n), &de));
    double *dd = (double *)de, *ed = dd + n;
    DDLA_TRY(bidiag2s(h, m, n, sa.view, su.view, sv.view, dd, ed, fprec(opts)));
    DDLA_TRY(stage_out(h, sa, a, m, n, rsa, csa));
    DDLA_TRY(stage_out(h, su, u, m, m, rsu, csu));
    DDLA_TRY(stage_out(h, sv, v, n, n, rsv, csv));
    DDLA_CUDA(cudaMemcpyAsync(d, dd, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
    if (n > 1) DDLA_CUDA(cudaMemcpyAsync(e, ed, sizeof(double) * (size_t)(n - 1), cudaMemcpyDeviceToHost, h->stream));
    DDLA_CUDA(cudaStreamSynchronize(h->stream));
    return 0;
}

// ------------------------------------------------------------------ factorizations, device
int ddla_dev_dgetrf(ddla_handle h, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, int32_t *piv,
                    const ddla_opts *opts) {
    CHECK_ARG(n >= 0, 2);
    CHECK_ARG(piv != nullptr || n == 0, 6);
    if (n == 0) return 0;
    DDLA_TRY(reset_info(h));
    DDLA_TRY(getrf<double>(h, n, View<double>{a, n, n, rsa, csa}, piv, fprec(opts), opts ? opts->nb : 0));
    int info;
    DDLA_TRY(read_info(h, &info));
    return info;
}

int ddla_dev_dgetrs(ddla_handle h, int32_t trans, ddla_dim_t n, ddla_dim_t nrhs, const double *lu, ddla_inc_t rsa,
                    ddla_inc_t csa, const int32_t *piv, double *b, ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(n >= 0, 3);
    CHECK_ARG(nrhs >= 0, 4);
    if (n == 0 || nrhs == 0) return 0;
    return getrs<double>(h, trans, n, nrhs, View<const double>{lu, n, n, rsa, csa}, piv,
                         View<double>{b, n, nrhs, rsb, csb});
}

int ddla_dev_dpotrf(ddla_handle h, int32_t uplo, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa,
                    const ddla_opts *opts) {
    CHECK_ARG(valid_tri(uplo), 2);
    CHECK_ARG(n >= 0, 3);
    if (n == 0) return 0;
    DDLA_TRY(reset_info(h));
    DDLA_TRY(potrf<double>(h, uplo, n, View<double>{a, n, n, rsa, csa}, fprec(opts), opts ? opts->nb : 0));
    int info;
    DDLA_TRY(read_info(h, &info));
    return info;
}

int ddla_dev_dpotrs(ddla_handle h, int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa,
                    ddla_inc_t csa, double *b, ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(valid_tri(uplo), 2);
    if (n == 0 || nrhs == 0) return 0;
    return potrs<double>(h, uplo, n, nrhs, View<const double>{a, n, n, rsa, csa}, View<double>{b, n, nrhs, rsb, csb});
}

int ddla_dev_dldlt(ddla_handle h, int32_t uplo, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa,
                   const ddla_opts *opts) {
    CHECK_ARG(valid_tri(uplo), 2);
    CHECK_ARG(n >= 0, 3);
    if (n == 0) return 0;
    DDLA_TRY(reset_info(h));
    DDLA_TRY(ldlt<double>(h, uplo, n, View<double>{a, n, n, rsa, csa}, fprec(opts), opts ? opts->nb : 0));
    int info;
    DDLA_TRY(read_info(h, &info));
    return info;
}

int ddla_dev_dldlts(ddla_handle h, int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa,
                    ddla_inc_t csa, double *b, ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(valid_tri(uplo), 2);
    if (n == 0 || nrhs == 0) return 0;
    DDLA_TRY(reset_info(h));
    DDLA_TRY(ldlts<double>(h, uplo, n, nrhs, View<const double>{a, n, n, rsa, csa},
                           View<double>{b, n, nrhs, rsb, csb}));
    int info;
    DDLA_TRY(read_info(h, &info));
    return info;
}

// ------------------------------------------------------------------ factorizations, host
int ddla_dgetrf(ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, int32_t *piv, const ddla_opts *opts) {
    CHECK_ARG(n >= 0, 1);
    CHECK_ARG(piv != nullptr || n == 0, 5);
    if (n == 0) return 0;
    GET_HANDLE(h);
    Staged sa;
    DDLA_TRY(stage_in(h, WS_A, a, n, n, rsa, csa, true, &sa));
    int32_t *dp;
    DDLA_TRY(workspace(h, WS_X, sizeof(int32_t) * (size_t)n, (void **)&dp));
    DDLA_TRY(reset_info(h));
    DDLA_TRY(getrf<double>(h, n, sa.view, dp, fprec(opts), opts ? opts->nb : 0));
    int info;
    DDLA_TRY(read_info(h, &info));
    DDLA_CUDA(cudaMemcpyAsync(piv, dp, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
    DDLA_TRY(stage_out(h, sa, a, n, n, rsa, csa));
    return info;
}

int ddla_dgetrs(int32_t trans, ddla_dim_t n, ddla_dim_t nrhs, const double *lu, ddla_inc_t rsa, ddla_inc_t csa,
                const int32_t *piv, double *b, ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(n >= 0, 2);
    CHECK_ARG(nrhs >= 0, 3);
    CHECK_ARG(piv != nullptr || n == 0, 7);
    if (n == 0 || nrhs == 0) return 0;
    GET_HANDLE(h);
    Staged sa, sb;
    DDLA_TRY(stage_in(h, WS_A, lu, n, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, n, nrhs, rsb, csb, true, &sb));
    int32_t *dp;
    DDLA_TRY(workspace(h, WS_X, sizeof(int32_t) * (size_t)n, (void **)&dp));
    DDLA_CUDA(cudaMemcpyAsync(dp, piv, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, h->stream));
    DDLA_TRY(getrs<double>(h, trans, n, nrhs, cv(sa.view), dp, sb.view));
    return stage_out(h, sb, b, n, nrhs, rsb, csb);
}

int ddla_dgetrf_nopiv(ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, const ddla_opts *opts) {
    CHECK_ARG(n >= 0, 1);
    if (n == 0) return 0;
    GET_HANDLE(h);
    Staged sa;
    DDLA_TRY(stage_in(h, WS_A, a, n, n, rsa, csa, true, &sa));
    DDLA_TRY(reset_info(h));
    DDLA_TRY(getrf_nopiv<double>(h, n, sa.view, fprec(opts), opts ? opts->nb : 0));
    int info;
    DDLA_TRY(read_info(h, &info));
    DDLA_TRY(stage_out(h, sa, a, n, n, rsa, csa));
    return info;
}

int ddla_dgetrs_nopiv(int32_t trans, ddla_dim_t n, ddla_dim_t nrhs, const double *lu, ddla_inc_t rsa,
                      ddla_inc_t csa, double *b, ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(n >= 0, 2);
    CHECK_ARG(nrhs >= 0, 3);
    if (n == 0 || nrhs == 0) return 0;
    GET_HANDLE(h);
    Staged sa, sb;
    DDLA_TRY(stage_in(h, WS_A, lu, n, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, n, nrhs, rsb, csb, true, &sb));
    DDLA_TRY(getrs_nopiv<double>(h, trans, n, nrhs, cv(sa.view), sb.view));
    return stage_out(h, sb, b, n, nrhs, rsb, csb);
}

int ddla_dpotrf(int32_t uplo, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, const ddla_opts *opts) {
    CHECK_ARG(valid_tri(uplo), 1);
    CHECK_ARG(n >= 0, 2);
    if (n == 0) return 0;
    GET_HANDLE(h);
    Staged sa;
    DDLA_TRY(stage_in(h, WS_A, a, n, n, rsa, csa, true, &sa));
    DDLA_TRY(reset_info(h));
    DDLA_TRY(potrf<double>(h, uplo, n, sa.view, fprec(opts), opts ? opts->nb : 0));
    int info;
    DDLA_TRY(read_info(h, &info));
    DDLA_TRY(stage_out(h, sa, a, n, n, rsa, csa, uplo));
    return info;
}

int ddla_dpotrs(int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                double *b, ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(valid_tri(uplo), 1);
    CHECK_ARG(n >= 0, 2);
    CHECK_ARG(nrhs >= 0, 3);
    if (n == 0 || nrhs == 0) return 0;
    GET_HANDLE(h);
    Staged sa, sb;
    DDLA_TRY(stage_in(h, WS_A, a, n, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, n, nrhs, rsb, csb, true, &sb));
    DDLA_TRY(potrs<double>(h, uplo, n, nrhs, cv(sa.view), sb.view));
    return stage_out(h, sb, b, n, nrhs, rsb, csb);
}

int ddla_dldlt(int32_t uplo, ddla_dim_t n, double *a, ddla_inc_t rsa, ddla_inc_t csa, const ddla_opts *opts) {
    CHECK_ARG(valid_tri(uplo), 1);
    CHECK_ARG(n >= 0, 2);
    if (n == 0) return 0;
    GET_HANDLE(h);
    Staged sa;
    DDLA_TRY(stage_in(h, WS_A, a, n, n, rsa, csa, true, &sa));
    DDLA_TRY(reset_info(h));
    DDLA_TRY(ldlt<double>(h, uplo, n, sa.view, fprec(opts), opts ? opts->nb : 0));
    int info;
    DDLA_TRY(read_info(h, &info));
    DDLA_TRY(stage_out(h, sa, a, n, n, rsa, csa, uplo));
    return info;
}

int ddla_dldlts(int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                double *b, ddla_inc_t rsb, ddla_inc_t csb) {
    CHECK_ARG(valid_tri(uplo), 1);
    CHECK_ARG(n >= 0, 2);
    CHECK_ARG(nrhs >= 0, 3);
    if (n == 0 || nrhs == 0) return 0;
    GET_HANDLE(h);
    Staged sa, sb;
    DDLA_TRY(stage_in(h, WS_A, a, n, n, rsa, csa, true, &sa));
    DDLA_TRY(stage_in(h, WS_B, b, n, nrhs, rsb, csb, true, &sb));
    DDLA_TRY(reset_info(h));
    DDLA_TRY(ldlts<double>(h, uplo, n, nrhs, cv(sa.view), sb.view));
    int info;
    DDLA_TRY(read_info(h, &info));
    if (info) return info;
    return stage_out(h, sb, b, n, nrhs, rsb, csb);
}

}  // extern "C"
