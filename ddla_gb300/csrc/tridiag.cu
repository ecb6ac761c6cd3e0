// Reduction of a symmetric matrix to tridiagonal form (FP64), DDLA's
// Tridiagonaling.Tridiag (DDLA/Transformations/Tridiagonaling.cs:33-230):
// one Householder reflector per column built from the lower triangle
// (BuildHH: sigma = sign(chi) |x|, u(0) = 1, tau = (1 + |u(1:)|^2) / 2),
// p = A22 u, p = (p - (u^T p / 2 tau) u) / tau, A22 -= u p^T + p u^T, and the
// block factors T(0:i, i) = A20^T u, T(i, i) = tau per block of T's rows;
// then A is overwritten by Q with Q^T A Q = tridiag(d, e).
//
// The reduction is a BLAS-2 sweep per column over the trailing triangle; on
// GB300 its 4/3 n^3 flops run on the FP64 pipe.  Each column costs three
// launches:
//   k_trd_column   one CTA: the pending rank-2 update of column i, d(i), the
//                  reflector of column i (norm reduced in a fixed order);
//   k_trd_sweep    one CTA per 64 x 64 tile of the trailing lower triangle:
//                  applies the pending rank-2 update of the previous column
//                  and forms this column's A22 u from the updated tile (row
//                  and column partial sums, so only the lower triangle is
//                  read); extra CTAs form the partial sums of A20^T u;
//   k_trd_reduce   one CTA per 64-row block: p in a fixed order, the block's
//                  share of u^T p, and (CTA 0) the T column.
// The finishing of p (beta, 1/tau) is applied by its consumers, so no pass
// over p is spent on it.  Q is formed from the vectors, which sit below the
// subdiagonal exactly as a QR's vectors sit below the diagonal of A[1:, 0:n-1],
// with the QR's block-reflector code (ormqr on the identity).
#include <cmath>

#include "common.cuh"
#include "timing.cuh"

namespace ddla {

namespace {

constexpr int TT = 64;            // tile edge
constexpr int SW_THREADS = 256;   // one 4 x 4 block of the 64 x 64 tile per thread

struct TrdWs {
    double *u[2];   // reflector vectors by column parity (full length n)
    double *p;      // unscaled p = A22 u of the last column (full length n)
    double *tau;    // tau per column
    double *tinv;   // 1 / tau per column (one FP64 division per column, not per thread)
    double *dotp;   // per 64-row block share of u^T p
    double *prow;   // [tile][64] row partial sums
    double *pcol;   // [tile][64] column partial sums
    double *pt;     // [chunk][64] partial sums of A20^T u
    double *beta;   // per column: u^T p / (2 tau), formed by the last reducing CTA
    unsigned *ticket;
};

struct TrdArgs {
    double *A;
    i64 rs, cs;
    int n, i;        // column
    int il;          // column within its T block
    int nt;          // 64-row blocks of the trailing matrix of column i
    TrdWs w;
    double *T;
    i64 rst, cst;
    double *d, *e;
};

// p of column j at global row g, finished: (p - beta u) / tau with
// beta = u^T p / (2 tau) from the block shares.
__device__ __forceinline__ double p_fin(const TrdWs &w, const double *u, double beta, double inv_tau, int g) {
    return (w.p[g] - beta * u[g]) * inv_tau;
}


__global__ void __launch_bounds__(1024) k_trd_column(TrdArgs a) {
    const int n = a.n, i = a.i, tid = threadIdx.x;
    __shared__ double red[32];
    __shared__ double bc[4];
    double *A = a.A;
    auto at = [&](int r, int c) -> double & { return A[(i64)r * a.rs + (i64)c * a.cs]; };
    // 1. the pending rank-2 update of column i (from column i - 1)
    if (i > 0) {
        const double *uo = a.w.u[(i - 1) & 1];
        const double inv = a.w.tinv[i - 1];
        const double beta = a.w.beta[i - 1];
        const double ui = uo[i], pi = p_fin(a.w, uo, beta, inv, i);
        for (int r = i + tid; r < n; r += blockDim.x) {
            const double ur = uo[r], pr = p_fin(a.w, uo, beta, inv, r);
            at(r, i) = at(r, i) - (ur * pi + pr * ui);
        }
        __syncthreads();
    }
    if (tid == 0) a.d[i] = at(i, i);
    if (i >= n - 1) return;
    // 2. the reflector of x = A(i+1:, i)
    double s = 0.0;
    for (int r = i + 2 + tid; r < n; r += blockDim.x) {
        const double v = at(r, i);
        s = fma(v, v, s);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((tid & 31) == 0) red[tid >> 5] = s;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += red[q];
        const double chi = at(i + 1, i), len = sqrt(t);
        double sigma, tau, inv = 1.0;
        if (len == 0.0) {
            sigma = -chi;
            tau = 0.5;
        } else {
            const double lenx = hypot(chi, len);
            sigma = copysign(lenx, chi);
            inv = 1.0 / (chi - sigma);
            const double ll = len * inv;
            tau = (1.0 + ll * ll) / 2.0;
        }
        bc[0] = sigma;
        bc[1] = tau;
        bc[2] = inv;
        bc[3] = len;
    }
    __syncthreads();
    const double sigma = bc[0], tau = bc[1], inv = bc[2];
    const bool zero = bc[3] == 0.0;
    double *u = a.w.u[i & 1];
    for (int r = i + 1 + tid; r < n; r += blockDim.x) {
        double v;
        if (r == i + 1) {
            v = 1.0;
            at(r, i) = sigma;
        } else {
            v = zero ? at(r, i) : at(r, i) * inv;
            at(r, i) = v;
        }
        u[r] = v;
    }
    if (tid == 0) {
        a.w.tau[i] = tau;
        a.w.tinv[i] = 1.0 / tau;
        a.e[i] = sigma;
        a.T[(i64)a.il * a.rst + (i64)i * a.cst] = tau;
    }
}

// Tile (R, C), C <= R, of the trailing triangle of column i (origin i + 1).
__device__ __forceinline__ void tile_of(int t, int &R, int &C) {
    int r = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((r + 1) * (r + 2) / 2 <= t) r++;
    while (r * (r + 1) / 2 > t) r--;
    R = r;
    C = t - r * (r + 1) / 2;
}

template <bool rowmajor>
__global__ void __launch_bounds__(SW_THREADS) k_trd_sweep(TrdArgs a) {
    const int n = a.n, i = a.i, o = i + 1;
    const int nt = a.nt, ntiles = nt * (nt + 1) / 2;
    const int tid = threadIdx.x;
    const double *un = a.w.u[i & 1];
    __shared__ double vr[3][TT];   // tile rows: u of column i, u and finished p of column i - 1
    __shared__ double vc[3][TT];   // tile columns: the same
    __shared__ double ysm[16][TT + 1];
    __shared__ double zsm[16][TT + 1];
    double *A = a.A;
    // a tile (R, C) of the trailing triangle, or (chunk) rows q*64.. of the
    // block's earlier columns i - il .. i - 1 for A20^T u
    const bool chunk = (int)blockIdx.x >= ntiles;
    const int il = a.il;
    int gr0, gc0;
    if (chunk) {
        gr0 = o + ((int)blockIdx.x - ntiles) * TT;
        gc0 = i - il;
    } else {
        int R, C;
        tile_of(blockIdx.x, R, C);
        gr0 = o + R * TT;
        gc0 = o + C * TT;
    }
    const bool pend = !chunk && i > 0;
    const double *uo = i > 0 ? a.w.u[(i - 1) & 1] : nullptr;
    double beta = 0.0, inv = 0.0;
    if (pend) {
        inv = a.w.tinv[i - 1];
        beta = a.w.beta[i - 1];
    }
    if (tid < TT) {
        const int g = gr0 + tid;
        vr[0][tid] = g < n ? un[g] : 0.0;
        vr[1][tid] = (pend && g < n) ? uo[g] : 0.0;
        vr[2][tid] = (pend && g < n) ? p_fin(a.w, uo, beta, inv, g) : 0.0;
    } else if (tid < 2 * TT) {
        const int t = tid - TT, g = gc0 + t;
        const bool ok = !chunk && g < n;
        vc[0][t] = ok ? un[g] : 0.0;
        vc[1][t] = (pend && ok) ? uo[g] : 0.0;
        vc[2][t] = (pend && ok) ? p_fin(a.w, uo, beta, inv, g) : 0.0;
    }
    __syncthreads();
    // thread: a 4 x 4 block, 4 consecutive fast (contiguous) indices from fq,
    // 4 slow indices from sq; the row sums y and column sums z of the block
    // stay in registers until one shared-memory reduction
    const int fg = tid & 15, sgp = tid >> 4;
    const int fq = fg * 4, sq = sgp * 4;
    double yy[4] = {0.0, 0.0, 0.0, 0.0}, zz[4] = {0.0, 0.0, 0.0, 0.0};   // by row / by column of the block
#pragma unroll
    for (int ks = 0; ks < 4; ks++) {
#pragma unroll
        for (int kf = 0; kf < 4; kf++) {
            const int r = rowmajor ? sq + ks : fq + kf, c = rowmajor ? fq + kf : sq + ks;
            const int gr = gr0 + r, gc = gc0 + c;
            const bool ok = chunk ? (gr < n && c < il) : (gr < n && gc < n && gr >= gc);
            if (!ok) continue;
            double *ptr = A + (i64)gr * a.rs + (i64)gc * a.cs;
            double v = *ptr;
            if (pend) {
                v = fma(-vr[1][r], vc[2][c], fma(-vr[2][r], vc[1][c], v));
                *ptr = v;
            }
            const int ri = rowmajor ? ks : kf, ci = rowmajor ? kf : ks;
            yy[ri] = fma(v, vc[0][c], yy[ri]);
            if (gr != gc) zz[ci] = fma(v, vr[0][r], zz[ci]);
        }
    }
    // row sums: rows of this thread's block, one column group each; column sums likewise
    const int rq = rowmajor ? sq : fq, cq = rowmajor ? fq : sq;
    const int cgid = rowmajor ? fg : sgp, rgid = rowmajor ? sgp : fg;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        ysm[cgid][rq + k] = yy[k];
        zsm[rgid][cq + k] = zz[k];
    }
    __syncthreads();
    if (tid < TT) {
        double y = 0.0, z = 0.0;
#pragma unroll
        for (int g = 0; g < 16; g++) {
            y += ysm[g][tid];
            z += zsm[g][tid];
        }
        if (chunk) {
            if (tid < il) a.w.pt[(i64)((int)blockIdx.x - ntiles) * TT + tid] = z;
        } else {
            const i64 tix = (i64)blockIdx.x * TT;
            a.w.prow[tix + tid] = y;
            a.w.pcol[tix + tid] = z;
        }
    }
}

// 4 threads per row: quarter q sums every 4th partial from q on (independent
// loads in flight), then the quarters are added in order.
constexpr int RD_THREADS = 4 * TT;

__global__ void __launch_bounds__(RD_THREADS) k_trd_reduce(TrdArgs a) {
    const int n = a.n, i = a.i, o = i + 1, nt = a.nt;
    const int B = blockIdx.x, tid = threadIdx.x, row = tid & (TT - 1), q = tid >> 6;
    const int g = o + B * TT + row;
    const double *un = a.w.u[i & 1];
    __shared__ double part[4][TT];
    __shared__ double red[2];
    // terms: row partials of tiles (B, C <= B) for C = 0..B, then column
    // partials of tiles (R >= B, B) for R = B..nt-1
    const int nterm = B + 1 + (nt - B);
    double acc = 0.0;
    for (int t = q; t < nterm; t += 4) {
        const double v = t <= B ? a.w.prow[((i64)(B * (B + 1) / 2 + t)) * TT + row]
                                : a.w.pcol[((i64)((B + t - B - 1) * (B + t - B) / 2 + B)) * TT + row];
        acc += v;
    }
    part[q][row] = acc;
    __syncthreads();
    if (tid < TT) {
        const double p = part[0][tid] + part[1][tid] + part[2][tid] + part[3][tid];
        double dp = 0.0;
        if (g < n) {
            a.w.p[g] = p;
            dp = p * un[g];
        }
#pragma unroll
        for (int s = 16; s; s >>= 1) dp += __shfl_xor_sync(0xffffffffu, dp, s);
        if ((tid & 31) == 0) red[tid >> 5] = dp;
    }
    __syncthreads();
    __shared__ bool last;
    if (tid == 0) {
        a.w.dotp[B] = red[0] + red[1];
        // the last CTA to finish sums the shares in block order
        __threadfence();
        last = atomicAdd(a.w.ticket, 1u) == (unsigned)(nt - 1);
    }
    __syncthreads();
    if (last && tid == 0) {
        __threadfence();
        double t = 0.0;
        for (int b = 0; b < nt; b++) t += ((volatile double *)a.w.dotp)[b];
        a.w.beta[i] = t / (2.0 * a.w.tau[i]);
        *a.w.ticket = 0u;
    }
    if (B == 0 && tid < a.il) {
        double t = 0.0;
        for (int qq = 0; qq < nt; qq++) t += a.w.pt[(i64)qq * TT + tid];
        a.T[(i64)tid * a.rst + (i64)i * a.cst] = t;
    }
}

__global__ void k_trd_q_border(double *A, i64 rs, i64 cs, int n) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        A[(i64)k * cs] = k == 0 ? 1.0 : 0.0;
        A[(i64)k * rs] = k == 0 ? 1.0 : 0.0;
    }
}

}  // namespace

// Tridiag(A, T, d, e) on device data; T has tb rows; prec selects the Q
// formation's block-reflector products (FP64 or Ozaki).
int sytrd(ddla_handle h, i64 n, View<double> A, View<double> T, i64 tb, double *d, double *e, int prec) {
    if (n <= 0) return 0;
    if (n > (i64)1 << 30) {
        set_error("sytrd: n too large");
        return DDLA_ERR_UNSUPPORTED;
    }
    cudaStream_t s = h->stream;
    const i64 ntm = (n + TT - 1) / TT;
    const size_t nd = (size_t)(3 * n + n + ntm + 2 * ntm * (ntm + 1) / 2 * TT + ntm * TT + 2 * n + 16);
    void *ws;
    DDLA_TRY(workspace(h, WS_TRD, sizeof(double) * nd, &ws));
    TrdWs w;
    double *q = (double *)ws;
    w.u[0] = q;
    w.u[1] = q + n;
    w.p = q + 2 * n;
    w.tau = q + 3 * n;
    w.dotp = q + 4 * n;
    w.prow = w.dotp + ntm;
    w.pcol = w.prow + ntm * (ntm + 1) / 2 * TT;
    w.pt = w.pcol + ntm * (ntm + 1) / 2 * TT;
    w.beta = w.pt + ntm * TT;
    w.tinv = w.beta + n;
    w.ticket = (unsigned *)(w.tinv + n);
    DDLA_CUDA(cudaMemsetAsync(w.ticket, 0, sizeof(unsigned), s));
    TrdArgs a;
    a.A = A.p;
    a.rs = A.rs;
    a.cs = A.cs;
    a.n = (int)n;
    a.w = w;
    a.T = T.p;
    a.rst = T.rs;
    a.cst = T.cs;
    a.d = d;
    a.e = e;
    // the sweep's fast (coalesced) index follows the unit stride
    const bool rowmajor = A.cs == 1 || (A.rs != 1 && llabs(A.cs) <= llabs(A.rs));
    {
        Timed tm(s, TC_PANEL, 4.0 * (double)n * n * n / 3.0, 8.0 * (double)n * n * n / 3.0);
        for (i64 i = 0; i < n; i++) {
            a.i = (int)i;
            a.il = (int)(i % tb);
            const i64 m = n - i - 1;
            a.nt = (int)((m + TT - 1) / TT);
            k_trd_column<<<1, 1024, 0, s>>>(a);
            DDLA_LAUNCHED();
            if (m <= 0) break;
            const int ntiles = a.nt * (a.nt + 1) / 2 + (a.il > 0 ? a.nt : 0);
            if (rowmajor) k_trd_sweep<true><<<ntiles, SW_THREADS, 0, s>>>(a);
            else k_trd_sweep<false><<<ntiles, SW_THREADS, 0, s>>>(a);
            DDLA_LAUNCHED();
            k_trd_reduce<<<a.nt, RD_THREADS, 0, s>>>(a);
            DDLA_LAUNCHED();
        }
        DDLA_CUDA(cudaGetLastError());
    }
    // Q: the vectors of columns 0 .. n-2 lie below the diagonal of A[1:, 0:n-1]
    if (n > 1) {
        Timed tm(s, TC_UPDATE, 4.0 * (double)n * n * n / 3.0, 0.0);
        const i64 m = n - 1;
        void *qb;
        DDLA_TRY(workspace(h, WS_TRDQ, sizeof(double) * (size_t)(m * m), &qb));
        View<double> Q{(double *)qb, m, m, m, 1};
        DDLA_TRY(orgqr(h, m, m, View<const double>{A.p + A.rs, m, m, A.rs, A.cs},
                       View<const double>{T.p, tb, m, T.rs, T.cs}, tb, Q, prec));
        DDLA_TRY(copy2d_on<double>(s, View<const double>{Q.p, m, m, m, 1},
                                   View<double>{A.p + A.rs + A.cs, m, m, A.rs, A.cs}));
    }
    k_trd_q_border<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(A.p, A.rs, A.cs, (int)n);
    DDLA_LAUNCHED();
    return 0;
}

}  // namespace ddla
