// Blocked right-looking factorizations and their solves on device data.
//
//   getrf   LU with partial pivoting   DDLA/Factorizations/LU.cs:251-342
//   getrf_nopiv  LU without pivoting   LU.cs:133-203
//   potrf   Cholesky (lower / upper)   DDLA/Factorizations/Cholesky.cs:52-208
//   ldlt    unpivoted LDL^T            DDLA/Factorizations/LDLT.cs:56-265
//
// Each step factors a diagonal block (or, for LU, a whole column panel) with a
// single-kernel on-chip factorization, solves the off-diagonal block with
// TRSM and updates the trailing matrix with one GEMM / GEMMT in the requested
// precision.  Failure statuses (1-based pivot index) are accumulated on the
// device with atomicMin and read once at the end.
#include <climits>

#include "common.cuh"
#include "timing.cuh"

namespace ddla {

template <typename T>
int panel_width_for(ddla_handle h, i64 m);
template <typename T>
int panel_factor(ddla_handle h, cudaStream_t s, View<T> X, i64 pc, int w, int32_t *d_piv, i64 row_base, int *d_info,
                 T *inv, int slot, const PanelLoad<T> *pl = nullptr);
template <typename T>
bool panel_fused_ok(ddla_handle h, i64 m, int w);
int next_prep(ddla_handle h, cudaStream_t s, View<const float> F, i64 w0, i64 w1, int slot, const float *inv,
              float *Tb);
template <typename T>
int panel_swap_cols(ddla_handle h, View<T> X, i64 ncols, i64 skip0, i64 skipw, int *perm, int slot);
template <typename T>
int copy2d_on(cudaStream_t s, View<const T> X, View<T> Y);
template <typename T>
int panel_swap_rest(ddla_handle h, View<T> X, i64 pc, int w, int *perm, int slot);
template <typename T>
int apply_perm(ddla_handle h, View<T> B, const int32_t *d_piv, i64 n, bool forward);

namespace {

constexpr int DIAG_MAX = 128;
constexpr int DIAG_THREADS = 1024;

enum DiagKind { DK_CHOL = 0, DK_LDLT = 1, DK_LU_NOPIV = 2 };

// Unblocked factorization of one bs x bs diagonal block held in shared memory.
//   DK_CHOL: lower Cholesky of the lower triangle (Cholesky.cs:127-140): a
//            finite pivot <= 0 fails (Sqrt, :228-236), a non-finite square
//            root fails (managed InvScaled, DDLA/BLAS/Managed/1v.cs:283-292).
//   DK_LDLT: lower LDL^T (LDLT.cs:141-158): pivots 0..bs-2 must be non-zero
//            and finite.
//   DK_LU_NOPIV: LU without pivoting (LU.cs:188-203): pivots 0..bs-2 non-zero.
// `upper` factors the transposed view (A = U^T U, U^T D U), which yields the
// upper-triangle results of DDLA's upper variants.
template <typename T>
__global__ void __launch_bounds__(DIAG_THREADS)
    k_diag(T *A, i64 rs, i64 cs, int bs, int kind, int *info, i64 row_base) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *S = (T *)smem_raw;
    const int LD = bs + 1;
    const int tid = threadIdx.x;
    __shared__ int s_fail;
    for (int e = tid; e < bs * bs; e += DIAG_THREADS) {
        int i = e / bs, j = e % bs;
        S[i * LD + j] = A[i * rs + j * cs];
    }
    if (tid == 0) s_fail = 0;
    __syncthreads();
    const int last = (kind == DK_CHOL) ? bs : bs - 1;
    for (int i = 0; i < last; i++) {
        T piv = S[i * LD + i];
        bool fail = false;
        if (kind == DK_CHOL) {
            if (isfinite(piv) && piv <= T(0)) fail = true;
            else {
                piv = sqrt(piv);
                if (!isfinite(piv) || piv == T(0)) fail = true;
            }
        } else {
            if (piv == T(0) || (kind == DK_LDLT && !isfinite(piv))) fail = true;
        }
        if (fail) {
            if (tid == 0) { atomicMin(info, (int)(row_base + i + 1)); s_fail = 1; }
            break;
        }
        __syncthreads();
        if (tid == 0 && kind == DK_CHOL) S[i * LD + i] = piv;
        const T rinv = T(1) / piv;
        // scale column i below the diagonal
        for (int r = i + 1 + tid; r < bs; r += DIAG_THREADS) S[r * LD + i] *= rinv;
        __syncthreads();
        // trailing update
        const int nr = bs - i - 1;
        if (kind == DK_LU_NOPIV) {
            for (int e = tid; e < nr * nr; e += DIAG_THREADS) {
                int r = i + 1 + e / nr, c = i + 1 + e % nr;
                S[r * LD + c] = fma(S[r * LD + i], -S[i * LD + c], S[r * LD + c]);
            }
        } else {
            const T alpha = (kind == DK_CHOL) ? T(-1) : -piv;
            for (int e = tid; e < nr * nr; e += DIAG_THREADS) {
                int r = i + 1 + e / nr, c = i + 1 + e % nr;
                if (c > r) continue;
                T sc = alpha * S[r * LD + i];
                S[r * LD + c] = fma(S[c * LD + i], sc, S[r * LD + c]);
            }
        }
        __syncthreads();
    }
    __syncthreads();
    for (int e = tid; e < bs * bs; e += DIAG_THREADS) {
        int i = e / bs, j = e % bs;
        if (kind != DK_LU_NOPIV && j > i) continue;  // only the factored triangle
        A[i * rs + j * cs] = S[i * LD + j];
    }
}

// Scale columns j of X (m x b) by 1/d_j where d_j = D(j,j); rows == false
// scales columns, rows == true scales rows of X (b x m) by 1/d_i.  Zero or
// non-finite d fails (managed InvScaled).
template <typename T>
__global__ void k_scale_by_diag(T *X, i64 rs, i64 cs, i64 m, int b, const T *D, i64 drs, i64 dcs, bool rows,
                                int *info, i64 row_base) {
    i64 tot = m * b;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        i64 r = e / b;
        int j = (int)(e % b);
        T d = D[j * drs + j * dcs];
        if (d == T(0) || !isfinite(d)) {
            if (r == 0) atomicMin(info, (int)(row_base + j + 1));
            continue;
        }
        T *p = rows ? &X[(i64)j * rs + r * cs] : &X[r * rs + (i64)j * cs];
        *p *= T(1) / d;
    }
}

template <typename T>
__global__ void k_copy(const T *X, i64 rs, i64 cs, i64 m, i64 n, T *Y, i64 ld) {
    i64 tot = m * n;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        i64 i = e / n, j = e % n;
        Y[i * ld + j] = X[i * rs + j * cs];
    }
}

// The same factorizations with the block in registers: G x G threads,
// thread (tr, tc) owning the R x R elements (tr R + u, tc R + v).  Per column: the owner of the
// diagonal forms the pivot, the owners of the column (and, without pivoting,
// of the row) publish the scaled column / the pivot row in shared memory,
// every thread updates its elements -- two barriers per column and no index
// arithmetic per element.  The arithmetic per element is k_diag's, operation
// for operation, so the results are the same bits.
template <typename T, int R, int G>
__global__ void __launch_bounds__(G *G)
    k_diag_reg(T *A, i64 rs, i64 cs, int bs, int kind, int *info, i64 row_base) {
    __shared__ T lcol[G * R], urow[G * R];
    __shared__ T s_piv;
    __shared__ int s_fail;
    const int tid = threadIdx.x, tr = tid / G, tc = tid % G;
    T a[R][R];
#pragma unroll
    for (int u = 0; u < R; u++)
#pragma unroll
        for (int v = 0; v < R; v++) {
            const int r = tr * R + u, c = tc * R + v;
            a[u][v] = (r < bs && c < bs) ? A[r * rs + c * cs] : T(0);
        }
    const int last = (kind == DK_CHOL) ? bs : bs - 1;
    for (int i = 0; i < last; i++) {
        const int oi = i / R, li = i - oi * R;
        if (tr == oi && tc == oi) {
            T piv = T(0);
#pragma unroll
            for (int u = 0; u < R; u++)
                if (u == li) piv = a[u][u];
            bool fail = false;
            if (kind == DK_CHOL) {
                if (isfinite(piv) && piv <= T(0)) fail = true;
                else {
                    piv = sqrt(piv);
                    if (!isfinite(piv) || piv == T(0)) fail = true;
                }
#pragma unroll
                for (int u = 0; u < R; u++)
                    if (u == li && !fail) a[u][u] = piv;
            } else {
                if (piv == T(0) || (kind == DK_LDLT && !isfinite(piv))) fail = true;
            }
            s_piv = piv;
            s_fail = fail ? 1 : 0;
        }
        __syncthreads();
        if (s_fail) {
            if (tid == 0) atomicMin(info, (int)(row_base + i + 1));
            break;
        }
        const T piv = s_piv, rinv = T(1) / piv;
        if (tc == oi) {
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int r = tr * R + u;
#pragma unroll
                for (int v = 0; v < R; v++)
                    if (v == li && r > i && r < bs) {
                        const T l = a[u][v] * rinv;
                        a[u][v] = l;
                        lcol[r] = l;
                    }
            }
        }
        if (kind == DK_LU_NOPIV && tr == oi) {
#pragma unroll
            for (int u = 0; u < R; u++)
                if (u == li)
#pragma unroll
                    for (int v = 0; v < R; v++) {
                        const int c = tc * R + v;
                        if (c > i && c < bs) urow[c] = a[u][v];
                    }
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < R; u++) {
            const int r = tr * R + u;
            if (r <= i || r >= bs) continue;
            const T lr = lcol[r];
            const T sc = (kind == DK_CHOL) ? -lr : -piv * lr;
#pragma unroll
            for (int v = 0; v < R; v++) {
                const int c = tc * R + v;
                if (c <= i || c >= bs) continue;
                if (kind == DK_LU_NOPIV) a[u][v] = fma(lr, -urow[c], a[u][v]);
                else if (c <= r) a[u][v] = fma(lcol[c], sc, a[u][v]);
            }
        }
    }
#pragma unroll
    for (int u = 0; u < R; u++)
#pragma unroll
        for (int v = 0; v < R; v++) {
            const int r = tr * R + u, c = tc * R + v;
            if (r >= bs || c >= bs) continue;
            if (kind != DK_LU_NOPIV && c > r) continue;   // only the factored triangle
            A[r * rs + c * cs] = a[u][v];
        }
}

template <typename T>
int diag_kernel(ddla_handle h, View<T> A11, int bs, int kind, i64 row_base) {
    // 16 x 16 threads (8 warps: cheap barriers) with 4 x 4 elements each for
    // bs <= 64; 32 x 32 threads with 4 x 4 FP32 elements for bs <= 128
    if (bs <= 64) {
        k_diag_reg<T, 4, 16><<<1, 256, 0, h->stream>>>(A11.p, A11.rs, A11.cs, bs, kind, h->d_info + INFO_PIVOT,
                                                       row_base);
        DDLA_LAUNCHED();
        return 0;
    }
    if constexpr (sizeof(T) == 4) {   // (4 x 4 doubles per thread would spill at 1024 threads)
        if (bs <= 128) {
            k_diag_reg<T, 4, 32><<<1, DIAG_THREADS, 0, h->stream>>>(A11.p, A11.rs, A11.cs, bs, kind,
                                                                   h->d_info + INFO_PIVOT, row_base);
            DDLA_LAUNCHED();
            return 0;
        }
    }
    size_t smem = sizeof(T) * (size_t)bs * (bs + 1);
    static size_t avail[2] = {0, 0};
    if (!avail[sizeof(T) == 8]) DDLA_TRY(max_dyn_smem((const void *)k_diag<T>, h->smem_optin, &avail[sizeof(T) == 8]));
    if (smem > avail[sizeof(T) == 8]) {
        set_error("diagonal block does not fit in shared memory");
        return DDLA_ERR_UNSUPPORTED;
    }
    k_diag<T><<<1, DIAG_THREADS, smem, h->stream>>>(A11.p, A11.rs, A11.cs, bs, kind, h->d_info + INFO_PIVOT,
                                                   row_base);
    DDLA_LAUNCHED();
    return 0;
}

int grid_for(i64 tot) { return (int)((tot + 255) / 256 < 8192 ? ((tot + 255) / 256 > 0 ? (tot + 255) / 256 : 1) : 8192); }

template <typename T>
int prec_of(int prec) {
    if (sizeof(T) == 8) return prec == DDLA_PREC_OZAKI ? DDLA_PREC_OZAKI : DDLA_PREC_FP64;
    return prec == DDLA_PREC_FP64 || prec == DDLA_PREC_OZAKI ? DDLA_PREC_FP32 : prec;
}

int pick_nb(int nb, int dflt) { return nb > 0 ? (nb > DIAG_MAX ? DIAG_MAX : nb) : dflt; }

}  // namespace

// ------------------------------------------------------------------ LU (pivoted)
// U12 columns in place: X[0:b, c] <- inv(L11)[0:b, 0:b] X[0:b, c] for the
// U12CW columns of this CTA (inv row-major, ld TRI_TB).  The CTA reads its
// columns whole into shared memory first, so the product can overwrite them;
// thread t forms column t % U12CW, rows t / U12CW + 8 i.
constexpr int U12CW = 32;
template <typename T>
__global__ void __launch_bounds__(256) k_u12_inplace(T *X, i64 rs, i64 cs, int b, i64 ncol, const T *inv) {
    __shared__ T si[TRI_TB][TRI_TB + 1];
    __shared__ T sx[TRI_TB][U12CW + 1];
    const i64 c0 = (i64)blockIdx.x * U12CW;
    const int tid = threadIdx.x;
    for (int e = tid; e < b * b; e += 256) si[e / b][e % b] = inv[(e / b) * TRI_TB + (e % b)];
    for (int e = tid; e < b * U12CW; e += 256) {
        const int r = e / U12CW, c = e % U12CW;
        sx[r][c] = (c0 + c < ncol) ? X[r * rs + (c0 + c) * cs] : T(0);
    }
    __syncthreads();
    const int c = tid % U12CW, r0 = tid / U12CW;   // 8 row groups
    if (c0 + c >= ncol) return;
    for (int r = r0; r < b; r += 256 / U12CW) {
        T acc = T(0);
        for (int k = 0; k < b; k++) acc = fma(si[r][k], sx[k][c], acc);
        X[r * rs + (c0 + c) * cs] = acc;
    }
}

__global__ void k_iota(int *p, i64 n) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x) p[e] = (int)e;
}

// The handle's high-priority side stream and its two events, created on first
// use by the look-ahead factorizations.
static int ensure_side(ddla_handle h) {
    if (h->side) return 0;
    int lo = 0, hi = 0;
    DDLA_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    DDLA_CUDA(cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, hi));
    DDLA_CUDA(cudaEventCreateWithFlags(&h->ev_ready, cudaEventDisableTiming));
    DDLA_CUDA(cudaEventCreateWithFlags(&h->ev_panel, cudaEventDisableTiming));
    return 0;
}

template <typename T>
int getrf(ddla_handle h, i64 n, View<T> A, int32_t *d_piv, int prec, int nb, int *d_perm) {
    if (n == 0) return 0;
    prec = prec_of<T>(prec);
    cudaStream_t s = h->stream;
    if (d_perm) {
        k_iota<<<grid_for(n), 256, 0, s>>>(d_perm, n);
        DDLA_LAUNCHED();
    }
    int w = panel_width_for<T>(h, n);
    if (w == 0) w = 8;
    if (nb <= 0) nb = (int)tune_get("lu.nb", 0);
    if (nb > 0 && nb < w) w = nb < 8 ? 8 : nb;
    // Look-ahead of depth one: after panel k's interchanges and U12 solve, the
    // columns of panel k+1 are updated first and panel k+1 is factored on a
    // high-priority side stream while the main stream updates the rest of the
    // trailing matrix.  The panel touches only its own columns; its row
    // interchanges on the other columns are applied on the main stream after
    // the big update (panel_swap_rest), so the two streams never overlap in
    // memory.
    const bool ahead = tune_get("lu.lookahead", 1) != 0 && n > 2 * (i64)w;
    if (ahead) DDLA_TRY(ensure_side(h));
    // the panel kernel also forms inv(L11) (double-buffered by panel parity:
    // panel k+1 writes its inverse while the main stream still uses panel k's)
    T *pinv;
    DDLA_TRY(workspace(h, WS_PINV, sizeof(T) * 2 * TRI_TB * TRI_TB, (void **)&pinv));
    auto inv_of = [&](i64 j0) { return pinv + ((j0 / w) & 1) * TRI_TB * TRI_TB; };
    auto panel = [&](cudaStream_t st, i64 j0, int b, const PanelLoad<T> *pl = nullptr) -> int {
        Timed t(st, TC_PANEL, 2.0 * b * b * ((n - j0) - b / 3.0), 2.0 * sizeof(T) * (n - j0) * (double)b);
        return panel_factor<T>(h, st, A.sub(j0, n - j0, 0, n), j0, b, d_piv + j0, j0, h->d_info + INFO_PIVOT,
                               inv_of(j0), (int)((j0 / w) & 1), pl);
    };
    // FP32: the work between two panels (the next panel's interchanges, U12
    // and update) runs as one out-of-place launch (next_prep) instead of
    // three, and the next panel loads its rows from that launch's output
    const bool fused = ahead && sizeof(T) == 4 && tune_get("lu.nextprep", 1) != 0 &&
                       panel_fused_ok<T>(h, n - (i64)w, w);
    T *tb = nullptr;
    if (fused) DDLA_TRY(workspace(h, WS_NEXT, sizeof(T) * (size_t)n * w, (void **)&tb));
    // U12 columns [c, c + nc) of the row block of panel j0: inv(L11) times a
    // copy of them (the same blocked inverse the general TRSM applies)
    const int tprec = sizeof(T) == 8 ? DDLA_PREC_FP64 : DDLA_PREC_FP32;
    T *tmp;
    DDLA_TRY(workspace(h, WS_TMP, sizeof(T) * (size_t)w * n, (void **)&tmp));
    auto u12 = [&](i64 j0, int b, i64 c, i64 nc) -> int {
        if (nc <= 0) return 0;
        Timed t(s, TC_TRSM, (double)b * b * nc, sizeof(T) * (2.0 * b * nc + b * b));
        View<T> blk = A.sub(j0, b, c, nc);
        if (nc <= 4 * U12CW * 152 || tune_get("u12.gemm", 0) == 0) {
            // one kernel, in place: each CTA owns 32 whole columns
            k_u12_inplace<T><<<(unsigned)((nc + U12CW - 1) / U12CW), 256, 0, s>>>(blk.p, blk.rs, blk.cs, b, nc,
                                                                                  inv_of(j0));
            DDLA_LAUNCHED();
            return 0;
        }
        View<T> Tm{tmp + c, b, nc, n, 1};
        DDLA_TRY(copy2d_on<T>(s, View<const T>{blk.p, b, nc, blk.rs, blk.cs}, Tm));
        return gemm_any<T>(h, tprec, b, nc, b, T(1), View<const T>{inv_of(j0), b, b, TRI_TB, 1},
                           View<const T>{Tm.p, b, nc, n, 1}, T(0), blk, DDLA_DENSE);
    };
    DDLA_TRY(panel(s, 0, (int)(n < w ? n : w)));
    for (i64 j0 = 0; j0 < n; j0 += w) {
        const int b = (int)(n - j0 < w ? n - j0 : w);
        const int slot = (int)((j0 / w) & 1);
        const i64 r = n - j0 - b;
        const int b1n = (int)(r < w ? r : w);
        if (!ahead || r <= 0) {
            DDLA_TRY(panel_swap_rest<T>(h, A.sub(j0, n - j0, 0, n), j0, b, d_perm ? d_perm + j0 : nullptr, slot));
        } else if (!fused) {
            // the next panel's columns now; the rest after the next panel started
            DDLA_TRY(panel_swap_cols<T>(h, A.sub(j0, n - j0, j0 + b, b1n), b1n, b1n, 0, nullptr, slot));
        }
        if (r <= 0) break;
        View<T> A12 = A.sub(j0, b, j0 + b, r);
        View<const T> A21{A.p + (j0 + b) * A.rs + j0 * A.cs, r, b, A.rs, A.cs};
        const i64 j1 = j0 + b;
        const int b1 = (int)(r < w ? r : w);
        if (fused) {
            // the next panel's columns (interchanges, U12, update) into tb in
            // one launch, then the next panel from tb on the side stream,
            // launched before this step's big update so that its cluster
            // finds free SMs
            {
                Timed t(s, TC_UPDATE, 2.0 * r * b1 * b + (double)b * b * b1,
                        sizeof(T) * (2.0 * (r + b) * b1 + r * b + b * b));
                if constexpr (sizeof(T) == 4)
                    DDLA_TRY(next_prep(h, s, View<const float>{A.p + j0 * A.rs + j0 * A.cs, n - j0, b + b1, A.rs, A.cs},
                                       b, b1, slot, inv_of(j0), tb));
            }
            DDLA_CUDA(cudaEventRecord(h->ev_ready, s));
            DDLA_CUDA(cudaStreamWaitEvent(h->side, h->ev_ready, 0));
            const PanelLoad<T> pl{tb + (i64)b * b1, b1, 1, tb, A.p + j0 * A.rs + j1 * A.cs, b};
            DDLA_TRY(panel(h->side, j1, b1, &pl));
            DDLA_CUDA(cudaEventRecord(h->ev_panel, h->side));
            DDLA_TRY(panel_swap_cols<T>(h, A.sub(j0, n - j0, 0, n), n - b - b1, j0, (i64)b + b1,
                                        d_perm ? d_perm + j0 : nullptr, slot));
            const i64 rest = r - b1;
            if (rest > 0) {
                DDLA_TRY(u12(j0, b, j1 + b1, rest));
                Timed t(s, TC_UPDATE, 2.0 * r * rest * b, sizeof(T) * (2.0 * r * rest + r * b + b * rest));
                DDLA_TRY(gemm_any<T>(h, prec, r, rest, b, T(-1), A21,
                                     View<const T>{A12.p + b1 * A12.cs, b, rest, A12.rs, A12.cs}, T(1),
                                     A.sub(j1, r, j1 + b1, rest)));
            }
            DDLA_CUDA(cudaStreamWaitEvent(s, h->ev_panel, 0));
        } else if (ahead) {
            // next panel's columns first: their U12 part, then their update
            DDLA_TRY(u12(j0, b, j1, b1));
            {
                Timed t(s, TC_UPDATE, 2.0 * r * b1 * b, sizeof(T) * (2.0 * r * b1 + r * b + b * b1));
                // narrow: one launch on the CUDA cores (FP32) beats packing for the tensor cores
                DDLA_TRY(gemm_any<T>(h, sizeof(T) == 4 ? DDLA_PREC_FP32 : prec, r, b1, b, T(-1), A21,
                                     View<const T>{A12.p, b, b1, A12.rs, A12.cs}, T(1), A.sub(j1, r, j1, b1)));
            }
            DDLA_CUDA(cudaEventRecord(h->ev_ready, s));
            DDLA_CUDA(cudaStreamWaitEvent(h->side, h->ev_ready, 0));
            DDLA_TRY(panel(h->side, j1, b1));
            DDLA_CUDA(cudaEventRecord(h->ev_panel, h->side));
            // interchanges of every other column: left of the panel and right
            // of the next panel (the touched-row list of this panel is kept in
            // its own slot while the next panel writes the other)
            DDLA_TRY(panel_swap_cols<T>(h, A.sub(j0, n - j0, 0, n), n - b - b1, j0, (i64)b + b1,
                                        d_perm ? d_perm + j0 : nullptr, slot));
            const i64 rest = r - b1;
            if (rest > 0) {
                DDLA_TRY(u12(j0, b, j1 + b1, rest));
                Timed t(s, TC_UPDATE, 2.0 * r * rest * b, sizeof(T) * (2.0 * r * rest + r * b + b * rest));
                DDLA_TRY(gemm_any<T>(h, prec, r, rest, b, T(-1), A21,
                                     View<const T>{A12.p + b1 * A12.cs, b, rest, A12.rs, A12.cs}, T(1),
                                     A.sub(j1, r, j1 + b1, rest)));
            }
            DDLA_CUDA(cudaStreamWaitEvent(s, h->ev_panel, 0));
        } else {
            DDLA_TRY(u12(j0, b, j1, r));
            {
                View<const T> cA12{A12.p, b, r, A12.rs, A12.cs};
                Timed t(s, TC_UPDATE, 2.0 * r * r * b, sizeof(T) * (2.0 * r * r + 2.0 * r * b));
                DDLA_TRY(gemm_any<T>(h, prec, r, r, b, T(-1), A21, cA12, T(1), A.sub(j1, r, j1, r)));
            }
            DDLA_TRY(panel(s, j1, b1));
        }
    }
    return 0;
}

template <typename T>
int getrs(ddla_handle h, int trans, i64 n, i64 nrhs, View<const T> LU, const int32_t *d_piv, View<T> B) {
    if (n == 0 || nrhs == 0) return 0;
    if (!trans) {
        DDLA_TRY(apply_perm<T>(h, B, d_piv, n, true));
        DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_LOWER, DDLA_NO_TRANSPOSE, DDLA_UNIT_DIAG, n, nrhs, T(1), LU, B));
        DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_UPPER, DDLA_NO_TRANSPOSE, DDLA_NONUNIT_DIAG, n, nrhs, T(1), LU, B));
    } else {
        DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_UPPER, DDLA_TRANSPOSE, DDLA_NONUNIT_DIAG, n, nrhs, T(1), LU, B));
        DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_LOWER, DDLA_TRANSPOSE, DDLA_UNIT_DIAG, n, nrhs, T(1), LU, B));
        DDLA_TRY(apply_perm<T>(h, B, d_piv, n, false));
    }
    return 0;
}

template <typename T>
int getrs_perm(ddla_handle h, i64 n, i64 nrhs, View<const T> LU, const int *d_perm, View<T> B) {
    if (n == 0 || nrhs == 0) return 0;
    DDLA_TRY(permute_rows<T>(h, B, d_perm, n, true));
    DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_LOWER, DDLA_NO_TRANSPOSE, DDLA_UNIT_DIAG, n, nrhs, T(1), LU, B));
    DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_UPPER, DDLA_NO_TRANSPOSE, DDLA_NONUNIT_DIAG, n, nrhs, T(1), LU, B));
    return 0;
}

// ------------------------------------------------------------------ LU (no pivoting)
template <typename T>
int getrf_nopiv(ddla_handle h, i64 n, View<T> A, int prec, int nb) {
    if (n == 0) return 0;
    prec = prec_of<T>(prec);
    nb = pick_nb(nb, DIAG_MAX);
    if (n <= nb) return diag_kernel<T>(h, A, (int)n, DK_LU_NOPIV, 0);
    for (i64 j0 = 0; j0 < n; j0 += nb) {
        int b = (int)(n - j0 < nb ? n - j0 : nb);
        i64 r = n - j0 - b;
        View<T> A11 = A.sub(j0, b, j0, b);
        // every diagonal of a non-final block is tested (LU.cs:181 then the
        // next block's unblocked step); the final block leaves its last one.
        DDLA_TRY(diag_kernel<T>(h, A11, b, DK_LU_NOPIV, j0));
        if (r > 0) {
            View<const T> cA11{A11.p, b, b, A11.rs, A11.cs};
            View<T> A12 = A.sub(j0, b, j0 + b, r), A21 = A.sub(j0 + b, r, j0, b);
            DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_LOWER, DDLA_NO_TRANSPOSE, DDLA_UNIT_DIAG, b, r, T(1), cA11, A12));
            DDLA_TRY(trsm<T>(h, DDLA_RIGHT, DDLA_UPPER, DDLA_NO_TRANSPOSE, DDLA_NONUNIT_DIAG, r, b, T(1), cA11, A21));
            View<const T> cA21{A21.p, r, b, A21.rs, A21.cs}, cA12{A12.p, b, r, A12.rs, A12.cs};
            DDLA_TRY(gemm_any<T>(h, prec, r, r, b, T(-1), cA21, cA12, T(1), A.sub(j0 + b, r, j0 + b, r)));
        }
    }
    return 0;
}

template <typename T>
int getrs_nopiv(ddla_handle h, int trans, i64 n, i64 nrhs, View<const T> LU, View<T> B) {
    if (n == 0 || nrhs == 0) return 0;
    if (!trans) {
        DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_LOWER, DDLA_NO_TRANSPOSE, DDLA_UNIT_DIAG, n, nrhs, T(1), LU, B));
        DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_UPPER, DDLA_NO_TRANSPOSE, DDLA_NONUNIT_DIAG, n, nrhs, T(1), LU, B));
    } else {
        DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_UPPER, DDLA_TRANSPOSE, DDLA_NONUNIT_DIAG, n, nrhs, T(1), LU, B));
        DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_LOWER, DDLA_TRANSPOSE, DDLA_UNIT_DIAG, n, nrhs, T(1), LU, B));
    }
    return 0;
}

// ------------------------------------------------------------------ Cholesky
template <typename T>
int potrf(ddla_handle h, int uplo, i64 n, View<T> A, int prec, int nb) {
    if (n == 0) return 0;
    prec = prec_of<T>(prec);
    // FP32 factors of the mixed solver: 64-wide blocks, so the trailing
    // updates are rank-64 (the tensor-core update kernel's shape)
    nb = pick_nb(nb, sizeof(T) == 4 ? 64 : DIAG_MAX);
    // The upper factorization is the lower one of the transposed view.
    View<T> L = (uplo == DDLA_UPPER) ? A.t() : A;
    // block column j0 (width b): L11 = chol(A11), L21 = A21 L11^-T, on the
    // handle's current stream
    auto column = [&](i64 j0, int b) -> int {
        const i64 r = n - j0 - b;
        View<T> L11 = L.sub(j0, b, j0, b);
        DDLA_TRY(diag_kernel<T>(h, L11, b, DK_CHOL, j0));
        if (r > 0) {
            View<const T> cL11{L11.p, b, b, L11.rs, L11.cs};
            DDLA_TRY(trsm<T>(h, DDLA_RIGHT, DDLA_LOWER, DDLA_TRANSPOSE, DDLA_NONUNIT_DIAG, r, b, T(1), cL11,
                             L.sub(j0 + b, r, j0, b)));
        }
        return 0;
    };
    // Look-ahead of depth one (as in getrf): after block column k, the columns
    // of block k+1 are updated first, and block column k+1 is factored on the
    // high-priority side stream while the main stream updates the rest of the
    // trailing matrix.  The side stream touches only the columns of block k+1;
    // its diagonal kernel and triangular solve use the WS_TRI / WS_TMP
    // workspaces, the updates on the main stream none of them (WS_TMP is
    // largest for block 0, which the main stream solves, so it never grows
    // while the side stream holds it).
    const bool ahead = tune_get("chol.lookahead", 1) != 0 && n > 2 * (i64)nb;
    if (ahead) DDLA_TRY(ensure_side(h));
    cudaStream_t s = h->stream;
    if (ahead) DDLA_TRY(column(0, (int)nb));
    for (i64 j0 = 0; j0 < n; j0 += nb) {
        int b = (int)(n - j0 < nb ? n - j0 : nb);
        i64 r = n - j0 - b;
        if (!ahead) DDLA_TRY(column(j0, b));
        if (r <= 0) break;
        View<const T> cL21{L.p + (j0 + b) * L.rs + j0 * L.cs, r, b, L.rs, L.cs};
        const i64 j1 = j0 + b;
        if (!ahead) {
            Timed t(s, TC_UPDATE, 1.0 * r * (r + 1) * b, sizeof(T) * (1.0 * r * (r + 1) + r * b));
            DDLA_TRY(gemm_any<T>(h, prec, r, r, b, T(-1), cL21, cL21.t(), T(1), L.sub(j1, r, j1, r), DDLA_LOWER));
            continue;
        }
        const int b1 = (int)(r < nb ? r : nb);
        const i64 rest = r - b1;
        {   // block k+1's columns: its diagonal block (lower triangle) and the rows below it;
            // narrow, so FP32 on the CUDA cores for the FP32 factors
            Timed t(s, TC_UPDATE, 1.0 * b1 * (b1 + 1) * b + 2.0 * rest * b1 * b,
                    sizeof(T) * (2.0 * r * b1 + r * b));
            const int np = sizeof(T) == 4 ? DDLA_PREC_FP32 : prec;
            View<const T> top{cL21.p, b1, b, cL21.rs, cL21.cs};
            DDLA_TRY(gemm_any<T>(h, np, b1, b1, b, T(-1), top, top.t(), T(1), L.sub(j1, b1, j1, b1), DDLA_LOWER));
            if (rest > 0)
                DDLA_TRY(gemm_any<T>(h, np, rest, b1, b, T(-1),
                                     View<const T>{cL21.p + b1 * cL21.rs, rest, b, cL21.rs, cL21.cs}, top.t(), T(1),
                                     L.sub(j1 + b1, rest, j1, b1), DDLA_DENSE));
        }
        DDLA_CUDA(cudaEventRecord(h->ev_ready, s));
        DDLA_CUDA(cudaStreamWaitEvent(h->side, h->ev_ready, 0));
        h->stream = h->side;
        const int rc = column(j1, b1);
        h->stream = s;
        DDLA_TRY(rc);
        DDLA_CUDA(cudaEventRecord(h->ev_panel, h->side));
        if (rest > 0) {
            View<const T> low{cL21.p + b1 * cL21.rs, rest, b, cL21.rs, cL21.cs};
            Timed t(s, TC_UPDATE, 1.0 * rest * (rest + 1) * b, sizeof(T) * (1.0 * rest * (rest + 1) + rest * b));
            DDLA_TRY(gemm_any<T>(h, prec, rest, rest, b, T(-1), low, low.t(), T(1),
                                 L.sub(j1 + b1, rest, j1 + b1, rest), DDLA_LOWER));
        }
        DDLA_CUDA(cudaStreamWaitEvent(s, h->ev_panel, 0));
    }
    return 0;
}

template <typename T>
int potrs(ddla_handle h, int uplo, i64 n, i64 nrhs, View<const T> A, View<T> B) {
    if (n == 0 || nrhs == 0) return 0;
    View<const T> L = (uplo == DDLA_UPPER) ? A.t() : A;
    DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_LOWER, DDLA_NO_TRANSPOSE, DDLA_NONUNIT_DIAG, n, nrhs, T(1), L, B));
    DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_UPPER, DDLA_NO_TRANSPOSE, DDLA_NONUNIT_DIAG, n, nrhs, T(1), L.t(), B));
    return 0;
}

// ------------------------------------------------------------------ LDL^T
template <typename T>
int ldlt(ddla_handle h, int uplo, i64 n, View<T> A, int prec, int nb) {
    if (n == 0) return 0;
    prec = prec_of<T>(prec);
    nb = pick_nb(nb, DIAG_MAX);
    View<T> L = (uplo == DDLA_UPPER) ? A.t() : A;
    T *Y = nullptr;
    if (n > nb) DDLA_TRY(workspace(h, WS_Y, sizeof(T) * (size_t)(n - nb) * nb, (void **)&Y));
    for (i64 j0 = 0; j0 < n; j0 += nb) {
        int b = (int)(n - j0 < nb ? n - j0 : nb);
        i64 r = n - j0 - b;
        View<T> L11 = L.sub(j0, b, j0, b);
        DDLA_TRY(diag_kernel<T>(h, L11, b, DK_LDLT, j0));
        if (r > 0) {
            View<const T> cL11{L11.p, b, b, L11.rs, L11.cs};
            View<T> L21 = L.sub(j0 + b, r, j0, b);
            // A21 <- A21 L11^-T (unit), LDLT.cs:185-187
            DDLA_TRY(trsm<T>(h, DDLA_RIGHT, DDLA_LOWER, DDLA_TRANSPOSE, DDLA_UNIT_DIAG, r, b, T(1), cL11, L21));
            // Y21 = A21 (= L21 D), LDLT.cs:188-189
            k_copy<T><<<grid_for(r * b), 256, 0, h->stream>>>(L21.p, L21.rs, L21.cs, r, b, Y, b);
            DDLA_LAUNCHED();
            // A21[:, j] /= d_j, LDLT.cs:190-191
            k_scale_by_diag<T><<<grid_for(r * b), 256, 0, h->stream>>>(L21.p, L21.rs, L21.cs, r, b, L11.p, L11.rs,
                                                                      L11.cs, false, h->d_info + INFO_PIVOT, j0);
            DDLA_LAUNCHED();
            // A22 -= Y21 A21^T on the lower triangle, LDLT.cs:192-193
            View<const T> cY{Y, r, b, b, 1}, cL21{L21.p, r, b, L21.rs, L21.cs};
            DDLA_TRY(gemm_any<T>(h, prec, r, r, b, T(-1), cY, cL21.t(), T(1), L.sub(j0 + b, r, j0 + b, r),
                                 DDLA_LOWER));
        }
    }
    return 0;
}

template <typename T>
int ldlts(ddla_handle h, int uplo, i64 n, i64 nrhs, View<const T> A, View<T> B) {
    if (n == 0 || nrhs == 0) return 0;
    View<const T> L = (uplo == DDLA_UPPER) ? A.t() : A;
    DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_LOWER, DDLA_NO_TRANSPOSE, DDLA_UNIT_DIAG, n, nrhs, T(1), L, B));
    // X.row(i) /= a_ii, LDLT.cs:274-275
    k_scale_by_diag<T><<<grid_for(n * nrhs), 256, 0, h->stream>>>(B.p, B.cs, B.rs, nrhs, (int)n, A.p, A.rs, A.cs,
                                                                 false, h->d_info + INFO_PIVOT, 0);
    DDLA_LAUNCHED();
    DDLA_TRY(trsm<T>(h, DDLA_LEFT, DDLA_UPPER, DDLA_NO_TRANSPOSE, DDLA_UNIT_DIAG, n, nrhs, T(1), L.t(), B));
    return 0;
}

#define INST(T)                                                                                     \
    template int getrf<T>(ddla_handle, i64, View<T>, int32_t *, int, int, int *);                   \
    template int getrs_perm<T>(ddla_handle, i64, i64, View<const T>, const int *, View<T>);        \
    template int getrs<T>(ddla_handle, int, i64, i64, View<const T>, const int32_t *, View<T>);     \
    template int getrf_nopiv<T>(ddla_handle, i64, View<T>, int, int);                               \
    template int getrs_nopiv<T>(ddla_handle, int, i64, i64, View<const T>, View<T>);                \
    template int potrf<T>(ddla_handle, int, i64, View<T>, int, int);                                \
    template int potrs<T>(ddla_handle, int, i64, i64, View<const T>, View<T>);                      \
    template int ldlt<T>(ddla_handle, int, i64, View<T>, int, int);                                 \
    template int ldlts<T>(ddla_handle, int, i64, i64, View<const T>, View<T>);
INST(double)
INST(float)

}  // namespace ddla
