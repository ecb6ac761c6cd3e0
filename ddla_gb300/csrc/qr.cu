// Householder QR (FP64) in DDLA's UT-transform form, and its applications.
//
//   geqrf   QR.QRDecompose   DDLA/Factorizations/QR.cs:130-149, 314-389
//   ormqr   ApplyQlhfc / ApplyQlnfc (Q^T B, Q B)   QR.cs:417-534
//   geqrs   QR.Solve (least squares, m >= n)       QR.cs:151-168, 391-415
//   orgqr   QR.FormQ (Q = H_0 ... H_{k-1}, m x m)  QR.cs:179-201
//
// Storage is DDLA's: A holds R on and above the diagonal and the Householder
// vectors u_j below it (u_j(j) = 1 implicit); T (t_rows x n) holds, for every
// block of t_rows columns starting at j0, the upper triangular factor S of that
// block in T[0:b, j0:j0+b]: S(j, j) = tau_j and S(i, j) = u_i^T u_j, so that
// H_j0 ... H_j0+b-1 = I - U S^-1 U^T.  Each reflector is
// H = I - u u^T / tau with tau = u^T u / 2 (HouseHolder.BuildHouseHolder,
// DDLA/Transformations/HouseHolder.cs:34-58).
//
// GPU structure.  A panel of w <= 32 columns is factored by one thread-block
// cluster with the panel's rows spread over up to 16 CTAs (k_qr_panel): per
// column, every CTA reduces its share of the column norm and pushes it to all
// CTAs over DSMEM; after one cluster barrier every CTA forms the same
// reflector, reduces its share of u^T A for the panel's remaining columns,
// pushes those, and after a second barrier updates its rows.  The trailing
// matrix is then updated with the panel's block reflector in three FP64 DMMA
// launches that read U straight out of A as a unit-lower trapezoid
// (W = U^T C, W = S^-T W, C = C - U W).  The T blocks are formed at the end from
// U^T U (one triangle-only GEMM per block) with the panel's tau on the diagonal.
#include <cooperative_groups.h>

#include "common.cuh"
#include "timing.cuh"

namespace ddla {
int gemm_ozaki(ddla_handle h, i64 m, i64 n, i64 k, double alpha, View<const double> A, View<const double> B,
               double beta, View<double> C, int uplo = DDLA_DENSE, i64 batch = 1, const i64 *d_offsets = nullptr);
}

namespace cg = cooperative_groups;

namespace ddla {

namespace {

constexpr int QR_THREADS = 512;
constexpr int QR_WARPS = QR_THREADS / 32;
constexpr int QR_WMAX = 32;
constexpr int QR_MAXCS = 16;

struct QrPanelArgs {
    double *A;
    i64 rs, cs;
    int m, w;        // panel rows (from the diagonal down) and columns
    int rows_per;    // rows per CTA
    double *tau;     // w outputs
    double *S;       // w x w upper factor of the panel (row stride lds)
    i64 lds;
};

// Shared-memory doubles of the cross-CTA and cross-warp scratch.
constexpr int QR_SCRATCH = 2 * QR_MAXCS + QR_MAXCS * QR_WMAX + QR_WARPS * QR_WMAX + QR_WMAX + QR_WARPS + 8;

__host__ __device__ inline size_t qr_panel_smem(bool resident, int rows_per, int w) {
    return sizeof(double) * ((resident ? (size_t)rows_per * (w + 1) : 0) + QR_SCRATCH);
}

// One panel, one cluster.  RES: the CTA's rows live in shared memory (else
// they are read and written in place through L2).
template <bool RES>
__global__ void __launch_bounds__(QR_THREADS, 1) k_qr_panel(QrPanelArgs a) {
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int w = a.w, WP = w + 1;
    const int r0 = rank * a.rows_per;
    const int nr = max(0, min(a.m - r0, a.rows_per));

    extern __shared__ double qsm[];
    double *X = qsm;
    double *cl_norm = qsm + (RES ? (size_t)a.rows_per * WP : 0);  // [QR_MAXCS][2]: |x|^2 share, chi
    double *cl_dot = cl_norm + 2 * QR_MAXCS;                        // [QR_MAXCS][QR_WMAX]
    double *wred = cl_dot + QR_MAXCS * QR_WMAX;                     // [QR_WARPS][QR_WMAX]
    double *csum = wred + QR_WARPS * QR_WMAX;                       // [QR_WMAX]
    double *nred = csum + QR_WMAX;                                  // [QR_WARPS]
    double *tau_s = nred + QR_WARPS;                                // tau, 1/tau, 1/(chi-rho), rho, |x(i+1:)|

    auto at = [&](int lr, int c) -> double & {
        if (RES) return X[lr * WP + c];
        return a.A[(i64)(r0 + lr) * a.rs + (i64)c * a.cs];
    };
    if (RES) {
        for (int e = tid; e < nr * w; e += QR_THREADS) {
            int lr = e / w, c = e % w;
            X[lr * WP + c] = a.A[(i64)(r0 + lr) * a.rs + (i64)c * a.cs];
        }
    }
    __syncthreads();

    const int k = min(a.m, w);
    for (int i = 0; i < k; i++) {
        // 1. this CTA's share of |x(i+1:)|^2, and chi = x(i) from its owner
        double p = 0.0;
        for (int lr = tid; lr < nr; lr += QR_THREADS)
            if (r0 + lr > i) {
                double x = at(lr, i);
                p = fma(x, x, p);
            }
#pragma unroll
        for (int o = 16; o; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
        if (lane == 0) nred[warp] = p;
        __syncthreads();
        if (tid < CS) {
            double t = 0.0;
            for (int q = 0; q < QR_WARPS; q++) t += nred[q];
            const bool own = (i >= r0 && i < r0 + nr);
            double *dst = cluster.map_shared_rank(cl_norm, tid);
            dst[2 * rank] = t;
            dst[2 * rank + 1] = own ? at(i - r0, i) : 0.0;
        }
        cluster.sync();

        // 2. the reflector, formed once per CTA (FP64 division, square root
        // and hypot are long instruction sequences on this GPU's FP64 pipe)
        if (tid == 0) {
            double ss = 0.0, chi = 0.0;
            for (int q = 0; q < CS; q++) {
                ss += cl_norm[2 * q];
                chi += cl_norm[2 * q + 1];
            }
            const double len = sqrt(ss);
            double rho, tau, inv = 1.0;
            if (len == 0.0) {
                rho = -chi;
                tau = 0.5;
            } else {
                const double alpha = hypot(chi, len);
                rho = -copysign(alpha, chi);
                const double miu = chi - rho;
                inv = 1.0 / miu;
                const double sc = len / fabs(miu);
                tau = (1.0 + sc * sc) / 2.0;
            }
            tau_s[0] = tau;
            tau_s[1] = 1.0 / tau;
            tau_s[2] = inv;
            tau_s[3] = rho;
            tau_s[4] = len;
        }
        __syncthreads();
        {
            const double inv = tau_s[2], rho = tau_s[3];
            const bool scale = tau_s[4] != 0.0;
            for (int lr = tid; lr < nr; lr += QR_THREADS) {
                const int r = r0 + lr;
                if (r > i && scale) at(lr, i) *= inv;
                else if (r == i) at(lr, i) = rho;
            }
        }
        __syncthreads();

        // 3. this CTA's share of x(i, c) + u2^T x(i+1:, c) for every column
        // c != i of the panel (lane l: c = l for l < i, else l + 1): for c > i
        // the row a1 + u2^T A2 of the reflector's application, for c < i the
        // factor entry S(c, i) = u_c^T u_i (QR.cs:339-345)
        const int nc = w - 1;
        const int c = lane < i ? lane : lane + 1;
        if (nc > 0) {
            double acc = 0.0;
            if (c < w)
                for (int lr = warp; lr < nr; lr += QR_WARPS) {
                    const int r = r0 + lr;
                    if (r > i) acc = fma(at(lr, i), at(lr, c), acc);
                    else if (r == i) acc += at(lr, c);
                }
            wred[warp * QR_WMAX + lane] = acc;
            __syncthreads();
            if (warp == 0) {
                double t = 0.0;
                for (int q = 0; q < QR_WARPS; q++) t += wred[q * QR_WMAX + lane];
                csum[lane] = t;
            }
            __syncthreads();
            if (tid < CS * QR_WMAX) {
                const int q = tid / QR_WMAX, l = tid % QR_WMAX;
                if (l < nc) cluster.map_shared_rank(cl_dot, q)[rank * QR_WMAX + l] = csum[l];
            }
        }
        cluster.sync();

        // 4. rank-1 update of the later columns: a1 -= w, A2 -= u2 w^T with
        // w = (sum of shares) / tau; the factor column S(0:i, i) and S(i, i) = tau
        if (warp == 0) {
            double t = 0.0;
            if (lane < nc)
                for (int q = 0; q < CS; q++) t += cl_dot[q * QR_WMAX + lane];
            csum[lane] = (c > i) ? t * tau_s[1] : t;
        }
        __syncthreads();
        if (nc > 0 && c < w) {
            const double t = csum[lane];
            if (c > i) {
                const double wv = t;
                for (int lr = warp; lr < nr; lr += QR_WARPS) {
                    const int r = r0 + lr;
                    if (r > i) at(lr, c) = fma(-at(lr, i), wv, at(lr, c));
                    else if (r == i) at(lr, c) -= wv;
                }
            } else if (rank == 0 && warp == 0) {
                a.S[(i64)c * a.lds + i] = t;
            }
        }
        if (rank == 0 && tid == 0) {
            a.tau[i] = tau_s[0];
            a.S[(i64)i * a.lds + i] = tau_s[0];
        }
        __syncthreads();
    }
    if (RES) {
        for (int e = tid; e < nr * w; e += QR_THREADS) {
            int lr = e / w, c = e % w;
            a.A[(i64)(r0 + lr) * a.rs + (i64)c * a.cs] = X[lr * WP + c];
        }
    }
    // All DSMEM traffic must finish before any CTA of the cluster exits.
    cluster.sync();
}

__global__ void k_eye(double *Q, i64 m, i64 rs, i64 cs) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < m * m; e += (i64)gridDim.x * blockDim.x) {
        i64 i = e / m, j = e % m;
        Q[i * rs + j * cs] = i == j ? 1.0 : 0.0;
    }
}

// U (m x b, row-major) = the unit-lower trapezoid stored in A, explicitly
// (zeros above the diagonal, ones on it) for the split-precision products.
__global__ void k_qr_dense_u(const double *__restrict__ A, i64 rs, i64 cs, i64 m, i64 b, double *__restrict__ U) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < m * b; e += (i64)gridDim.x * blockDim.x) {
        const i64 r = e / b, c = e % b;
        U[e] = r > c ? A[r * rs + c * cs] : (r == c ? 1.0 : 0.0);
    }
}

// T(i, i) = tau(i) for the b x b factor written by the U^T U product.
__global__ void k_qr_diag(double *T, i64 rs, i64 cs, const double *tau, int b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < b) T[i * rs + i * cs] = tau[i];
}

int g_qr_cluster = 0;
size_t g_qr_smem = 0;

int qr_cluster(ddla_handle h) {
    if (g_qr_cluster) return g_qr_cluster;
    DDLA_CUDA(cudaFuncSetAttribute(k_qr_panel<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    DDLA_CUDA(cudaFuncSetAttribute(k_qr_panel<false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    size_t avail = 0;
    DDLA_TRY(max_dyn_smem((const void *)k_qr_panel<true>, h->smem_optin, &avail));
    DDLA_CUDA(cudaFuncSetAttribute(k_qr_panel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)qr_panel_smem(false, 0, QR_WMAX)));
    g_qr_smem = avail;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(QR_MAXCS);
    cfg.blockDim = dim3(QR_THREADS);
    cfg.dynamicSmemBytes = avail;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = QR_MAXCS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int cs = 0;
    if (cudaOccupancyMaxPotentialClusterSize(&cs, (const void *)k_qr_panel<true>, &cfg) != cudaSuccess || cs < 1) {
        cudaGetLastError();
        cs = 8;
    }
    int p2 = 1;
    while (p2 * 2 <= cs && p2 * 2 <= QR_MAXCS) p2 *= 2;
    g_qr_cluster = p2;
    return p2;
}

// Widest panel (<= 32) whose m rows fit in one cluster's shared memory; 0 =
// none fits (the panel is then factored in place through L2 at width 32).
int qr_width_for(ddla_handle h, i64 m) {
    const int cs = qr_cluster(h);
    if (cs <= 0) return 0;
    for (int w = QR_WMAX; w >= 8; w /= 2) {
        i64 rp = (m + cs - 1) / cs;
        if (qr_panel_smem(true, (int)rp, w) <= g_qr_smem) return w;
    }
    return 0;
}

int qr_panel(ddla_handle h, View<double> P, int w, double *tau, double *S, i64 lds) {
    Timed tm(h->stream, TC_PANEL, 2.0 * (double)P.rows * w * w, 16.0 * (double)P.rows * w);
    QrPanelArgs a;
    a.A = P.p;
    a.rs = P.rs;
    a.cs = P.cs;
    a.m = (int)P.rows;
    a.w = w;
    a.tau = tau;
    a.S = S;
    a.lds = lds;
    int cs = qr_cluster(h);
    if (cs <= 0) return cs < 0 ? cs : DDLA_ERR_UNSUPPORTED;
    const int64_t want = tune_get("qr.cluster", 0);
    if (want > 0 && want < cs) cs = (int)want;
    const i64 m = P.rows;
    // the panel is bound by the FP64 pipes of its CTAs: as many CTAs as keep
    // at least 64 rows each (and fit the rows on chip)
    int use = 1;
    while (use < cs && ((m + use - 1) / use > 64 || qr_panel_smem(true, (int)((m + use - 1) / use), w) > g_qr_smem))
        use *= 2;
    const i64 rp = (m + use - 1) / use;
    const bool res = qr_panel_smem(true, (int)rp, w) <= g_qr_smem && tune_get("qr.resident", 1) != 0;
    a.rows_per = (int)rp;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(use);
    cfg.blockDim = dim3(QR_THREADS);
    cfg.dynamicSmemBytes = qr_panel_smem(res, (int)rp, w);
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = use;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (res) DDLA_CUDA(cudaLaunchKernelEx(&cfg, k_qr_panel<true>, a));
    else DDLA_CUDA(cudaLaunchKernelEx(&cfg, k_qr_panel<false>, a));
    DDLA_LAUNCHED();
    return 0;
}

}  // namespace

// S = upper(U^T U) with tau on the diagonal, U = the m x b unit-lower
// trapezoid stored below the diagonal of Ub.  The factor of several
// consecutive blocks is the same formula over their joined columns.
int qr_tfactor(ddla_handle h, View<const double> Ub, i64 b, const double *tau, View<double> S) {
    const i64 m = Ub.rows;
    Timed tm(h->stream, TC_QR_T, (double)m * b * b, 8.0 * (double)m * b);
    View<const double> U{Ub.p, m, b, Ub.rs, Ub.cs};
    DDLA_TRY(gemm_f64_struct_h(h, b, b, m, 1.0, U.t(), OP_TRI | OP_UNIT, U, OP_TRI | OP_LOWER | OP_UNIT, 0.0,
                             View<double>{S.p, b, b, S.rs, S.cs}, DDLA_UPPER));
    k_qr_diag<<<(unsigned)((b + 127) / 128), 128, 0, h->stream>>>(S.p, S.rs, S.cs, tau, (int)b);
    DDLA_LAUNCHED();
    return 0;
}

// C = (I - U S^-1 U^T)^T C (trans) or (I - U S^-1 U^T) C, U m x b unit-lower
// trapezoid in Ub, W a b x C.cols scratch.
int qr_apply_block(ddla_handle h, bool trans, View<const double> Ub, i64 b, View<const double> S, View<double> Cm,
                   double *W, int prec, int oz_min_b) {
    const i64 m = Ub.rows, nc = Cm.cols;
    if (nc <= 0 || m <= 0) return 0;
    View<const double> U{Ub.p, m, b, Ub.rs, Ub.cs};
    View<double> Wv{W, b, nc, nc, 1};
    if (prec == DDLA_PREC_OZAKI && b >= (oz_min_b > 0 ? oz_min_b : 64) && m >= 256 && nc >= 64) {
        // split-precision tensor-core products on an explicit copy of U
        void *ud;
        DDLA_TRY(workspace(h, WS_QRU, sizeof(double) * (size_t)(m * b), &ud));
        const i64 blocks = (m * b + 255) / 256 < 4096 ? (m * b + 255) / 256 : 4096;
        k_qr_dense_u<<<(unsigned)blocks, 256, 0, h->stream>>>(Ub.p, Ub.rs, Ub.cs, m, b, (double *)ud);
        DDLA_LAUNCHED();
        View<const double> Ud{(const double *)ud, m, b, b, 1};
        {
            Timed tm(h->stream, TC_UPDATE, 2.0 * (double)m * b * nc, 8.0 * (double)m * (b + nc));
            DDLA_TRY(gemm_ozaki(h, b, nc, m, 1.0, Ud.t(), View<const double>{Cm.p, m, nc, Cm.rs, Cm.cs}, 0.0, Wv));
        }
        {
            Timed tm(h->stream, TC_TRSM, (double)b * b * nc, 8.0 * (double)b * nc);
            DDLA_TRY(trsm<double>(h, DDLA_LEFT, DDLA_UPPER, trans ? DDLA_TRANSPOSE : DDLA_NO_TRANSPOSE,
                                  DDLA_NONUNIT_DIAG, b, nc, 1.0, View<const double>{S.p, b, b, S.rs, S.cs}, Wv));
        }
        Timed tm(h->stream, TC_UPDATE, 2.0 * (double)m * b * nc, 16.0 * (double)m * nc);
        return gemm_ozaki(h, m, nc, b, -1.0, Ud, View<const double>{W, b, nc, nc, 1}, 1.0, Cm);
    }
    {
        Timed tm(h->stream, TC_UPDATE, 2.0 * (double)m * b * nc, 8.0 * (double)m * (b + nc));
        DDLA_TRY(gemm_f64_struct_h(h, b, nc, m, 1.0, U.t(), OP_TRI | OP_UNIT,
                                   View<const double>{Cm.p, m, nc, Cm.rs, Cm.cs}, OP_DENSE, 0.0, Wv));
    }
    {
        Timed tm(h->stream, TC_TRSM, (double)b * b * nc, 8.0 * (double)b * nc);
        DDLA_TRY(trsm<double>(h, DDLA_LEFT, DDLA_UPPER, trans ? DDLA_TRANSPOSE : DDLA_NO_TRANSPOSE, DDLA_NONUNIT_DIAG,
                              b, nc, 1.0, View<const double>{S.p, b, b, S.rs, S.cs}, Wv));
    }
    Timed tm(h->stream, TC_UPDATE, 2.0 * (double)m * b * nc, 16.0 * (double)m * nc);
    return gemm_f64_struct_h(h, m, nc, b, -1.0, U, OP_TRI | OP_LOWER | OP_UNIT, View<const double>{W, b, nc, nc, 1},
                             OP_DENSE, 1.0, Cm);
}

// QR of the m x n A in place; T (tb rows x n) receives the block factors.
// Two levels: panels of w <= 32 columns (one cluster kernel each, which also
// forms the panel's own factor S_w) update the rest of their block of tb
// columns; each finished block's factor goes to T and its reflector updates
// the trailing matrix with large-k products (W = U^T C, k = the block's rows).
int geqrf(ddla_handle h, i64 m, i64 n, View<double> A, View<double> T, i64 tb, int prec, int wcap) {
    const i64 k = m < n ? m : n;
    if (k == 0) return 0;
    const int64_t wt = wcap > 0 ? wcap : tune_get("qr.nb", 0);
    const i64 wmax = tb < n ? tb : n;
    // scratch: tau (k), the panel factor (32 x 32), W (max(tb, 32) x n)
    const i64 wrows = tb > QR_WMAX ? tb : QR_WMAX;
    void *ws;
    DDLA_TRY(workspace(h, WS_QR, sizeof(double) * (size_t)(k + QR_WMAX * QR_WMAX + wrows * n), &ws));
    double *tau = (double *)ws, *Sw = tau + k, *W = Sw + QR_WMAX * QR_WMAX;
    for (i64 j0 = 0; j0 < k; j0 += tb) {
        const i64 b = (k - j0) < tb ? (k - j0) : tb;
        for (i64 p = j0; p < j0 + b;) {
            const i64 mp = m - p;
            int w = qr_width_for(h, mp);
            if (w == 0) w = QR_WMAX;
            if (wt > 0 && wt < w) w = (int)wt;
            if (w > wmax) w = (int)wmax;
            const i64 pw = (j0 + b - p) < w ? (j0 + b - p) : w;
            View<double> P{A.p + p * A.rs + p * A.cs, mp, pw, A.rs, A.cs};
            DDLA_TRY(qr_panel(h, P, (int)pw, tau + p, Sw, QR_WMAX));
            if (p + pw < j0 + b) {   // the rest of this block
                View<const double> Ub{P.p, mp, pw, A.rs, A.cs};
                View<double> Cm{A.p + p * A.rs + (p + pw) * A.cs, mp, j0 + b - p - pw, A.rs, A.cs};
                DDLA_TRY(qr_apply_block(h, true, Ub, pw, View<const double>{Sw, pw, pw, QR_WMAX, 1}, Cm, W));
            }
            p += pw;
        }
        View<const double> Ub{A.p + j0 * A.rs + j0 * A.cs, m - j0, b, A.rs, A.cs};
        View<double> S{T.p + j0 * T.cs, b, b, T.rs, T.cs};
        DDLA_TRY(qr_tfactor(h, Ub, b, tau + j0, S));
        if (j0 + b < n) {   // the trailing matrix
            View<double> Cm{A.p + j0 * A.rs + (j0 + b) * A.cs, m - j0, n - j0 - b, A.rs, A.cs};
            DDLA_TRY(qr_apply_block(h, true, Ub, b, View<const double>{S.p, b, b, S.rs, S.cs}, Cm, W, prec));
        }
    }
    return 0;
}

// B (m x nrhs) = Q^T B (trans) or Q B with the factors of geqrf.
int ormqr(ddla_handle h, bool trans, i64 m, i64 n, View<const double> A, View<const double> T, i64 tb,
          View<double> B, int prec, int oz_min_b) {
    const i64 k = m < n ? m : n, nrhs = B.cols;
    if (k == 0 || nrhs == 0) return 0;
    void *ws;
    DDLA_TRY(workspace(h, WS_QR, sizeof(double) * (size_t)(tb * nrhs), &ws));
    double *W = (double *)ws;
    const i64 nblk = (k + tb - 1) / tb;
    for (i64 bi = 0; bi < nblk; bi++) {
        const i64 blk = trans ? bi : nblk - 1 - bi;   // Q^T: first block first; Q: last block first
        const i64 j0 = blk * tb, b = (k - j0) < tb ? (k - j0) : tb;
        View<const double> Ub{A.p + j0 * A.rs + j0 * A.cs, m - j0, b, A.rs, A.cs};
        View<const double> S{T.p + j0 * T.cs, b, b, T.rs, T.cs};
        View<double> Cm{B.p + j0 * B.rs, m - j0, nrhs, B.rs, B.cs};
        DDLA_TRY(qr_apply_block(h, trans, Ub, b, S, Cm, W, prec, oz_min_b));
    }
    return 0;
}

// Q (m x m) = H_0 ... H_{k-1}: Q = I, then Q = Q I.
int orgqr(ddla_handle h, i64 m, i64 n, View<const double> A, View<const double> T, i64 tb, View<double> Q, int prec) {
    if (m == 0) return 0;
    i64 blocks = (m * m + 255) / 256;
    k_eye<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, h->stream>>>(Q.p, m, Q.rs, Q.cs);
    DDLA_LAUNCHED();
    return ormqr(h, false, m, n, A, T, tb, Q, prec);
}

// Least squares X (n x nrhs) = argmin |A X - B| for m >= n; Y (m x nrhs)
// is scratch that receives Q^T B.
int geqrs(ddla_handle h, i64 m, i64 n, View<const double> A, View<const double> T, i64 tb, View<const double> B,
          View<double> Y, View<double> X) {
    DDLA_TRY(copy2d_on<double>(h->stream, B, Y));
    DDLA_TRY(ormqr(h, true, m, n, A, T, tb, Y, DDLA_PREC_FP64));
    View<double> Yt{Y.p, n, Y.cols, Y.rs, Y.cs};
    DDLA_TRY(trsm<double>(h, DDLA_LEFT, DDLA_UPPER, DDLA_NO_TRANSPOSE, DDLA_NONUNIT_DIAG, n, Y.cols, 1.0,
                          View<const double>{A.p, n, n, A.rs, A.cs}, Yt));
    return copy2d_on<double>(h->stream, View<const double>{Y.p, n, Y.cols, Y.rs, Y.cs}, X);
}

}  // namespace ddla
