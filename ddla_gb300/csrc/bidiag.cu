// One-stage bidiagonal reduction (FP64, m >= n), DDLA's Bidiagonaling.Bidiag2
// (DDLA/Transformations/Bidiagonaling.cs:48-143): per column g a column
// reflector (Tridiagonaling.BuildHH; u(g) = 1 stays in A), d(g) = sigma,
// A(g:, g+1:) -= u (u^T A(g:, g+1:)) / tau; then, except for the last column,
// a row reflector of A(g, g+1:), e(g) = sigma, A(g+1:, g+1:) -= (A v) v^T / tau.
// TU / TV (blocks of 128 columns) receive the UT factors of both reflector
// sets; U (m x m) and V (n x n) are formed from them with the QR's block
// reflectors (BuildUV).
//
// GPU structure, per column (each rank-1 update is applied by the next pass
// over the same part of A, fused with the product that pass exists for):
//   k_bd_vec (col)   one CTA: the pending row update of column g, its reflector
//   k_bd_sweep (L)   64 x 64 tiles of A(g:, g+1:): pending row update, then
//                    column sums with u; extra tiles: TU's A20^T u
//   k_bd_reduce (L)  w = (column sums) / tau in a fixed order; TU column
//   k_bd_vec (row)   one CTA: the pending column update of row g, its reflector
//   k_bd_sweep (R)   tiles of A(g+1:, g+1:): pending column update, then row
//                    sums with v; extra tiles: TV's A02 v
//   k_bd_reduce (R)  y = (row sums) / tau; TV column
#include <cmath>

#include "common.cuh"
#include "timing.cuh"

namespace ddla {

namespace {

constexpr int BT = 64;           // tile edge
constexpr int BD_NB = 128;       // Bidiagonaling.BlockSize
constexpr int BS_THREADS = 256;  // one 4 x 4 block per thread
constexpr int BR_THREADS = 256;  // reduce: 4 threads per output element

struct BdWs {
    double *u, *v;      // column / row reflector (full length m / n)
    double *w, *y;      // finished u^T A / tau (length n) and A v / tau (length m)
    double *part;       // [tile][64] partial sums
    double *tpart;      // [chunk][64] partial sums of the T column
    double *scal;       // per step: tau, 1/tau
};

struct BdArgs {
    double *A;
    i64 rs, cs;
    int m, n, g;
    int il, bs;          // step within its 128-block, block start
    int left;            // 1: column step, 0: row step
    // sweep geometry: main tiles cover rows [r0, m) x cols [c0, n)
    int r0, c0, nrb, ncb, nmain;
    int tchunks, thalves;   // T-column tiles: chunks along the long side x halves of il
    BdWs w;
    double *TU, *TV;
    double *d, *e;
};

// Column g (left) or row g (right) of A: apply the pending rank-1 update of
// the other side, then build the reflector (BuildHH, Tridiagonaling.cs:205-230).
__global__ void __launch_bounds__(1024) k_bd_vec(BdArgs a) {
    const int g = a.g, tid = threadIdx.x;
    __shared__ double red[32];
    __shared__ double bc[4];
    double *A = a.A;
    // x(k), k = 0 .. len-1: column g rows g..m-1, or row g columns g+1..n-1
    const int len = a.left ? a.m - g : a.n - g - 1;
    auto xp = [&](int k) -> double * {
        return a.left ? A + (i64)(g + k) * a.rs + (i64)g * a.cs : A + (i64)g * a.rs + (i64)(g + 1 + k) * a.cs;
    };
    // pending update: column step: A(r, g) -= y(r) v(g) (v(g) = 1, from row step g-1);
    // row step: A(g, c) -= u(g) w(c) (u(g) = 1)
    const bool pend = a.left ? g > 0 : true;
    double s = 0.0;
    for (int k = tid; k < len; k += blockDim.x) {
        double *p = xp(k);
        double v = *p;
        if (pend) v -= a.left ? a.w.y[g + k] : a.w.w[g + 1 + k];
        *p = v;
        if (k > 0) s = fma(v, v, s);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((tid & 31) == 0) red[tid >> 5] = s;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += red[q];
        const double chi = *xp(0), ln = sqrt(t);
        double sigma, tau, inv = 1.0;
        if (ln == 0.0) {
            sigma = -chi;
            tau = 0.5;
        } else {
            const double lx = hypot(chi, ln);
            sigma = copysign(lx, chi);
            inv = 1.0 / (chi - sigma);
            const double ll = ln * inv;
            tau = (1.0 + ll * ll) / 2.0;
        }
        bc[0] = sigma;
        bc[1] = tau;
        bc[2] = inv;
        bc[3] = ln;
        a.w.scal[0] = tau;
        a.w.scal[1] = 1.0 / tau;
        if (a.left) {
            a.d[g] = sigma;
            a.TU[(i64)a.il * a.n + g] = tau;
        } else {
            a.e[g] = sigma;
            a.TV[(i64)a.il * a.n + g] = tau;
        }
    }
    __syncthreads();
    const double inv = bc[2];
    const bool zero = bc[3] == 0.0;
    double *vec = a.left ? a.w.u : a.w.v;
    const int base = a.left ? g : g + 1;
    for (int k = tid; k < len; k += blockDim.x) {
        double *p = xp(k);
        double v;
        if (k == 0) v = 1.0;
        else v = zero ? *p : *p * inv;
        *p = v;
        vec[base + k] = v;
    }
}

// Main tiles: A(r, c) -= pr(r) pc(c) (the pending update), then column sums
// with u (left) or row sums with v (right).  T tiles: the same sums over the
// block's earlier columns (left: rows g.., columns bs..g-1) or rows (right:
// rows bs..g-1, columns g+1..), without an update.
template <bool rowmajor>
__global__ void __launch_bounds__(BS_THREADS) k_bd_sweep(BdArgs a) {
    const int m = a.m, n = a.n, g = a.g, tid = threadIdx.x;
    const bool left = a.left != 0;
    __shared__ double vr[2][BT];   // rows: pending row factor, sum weight
    __shared__ double vcl[2][BT];  // cols: pending col factor, sum weight
    __shared__ double ysm[16][BT + 1];
    __shared__ double zsm[16][BT + 1];
    double *A = a.A;
    const bool tchunk = (int)blockIdx.x >= a.nmain;
    int gr0, gc0, rend, cend;
    bool pend;
    if (!tchunk) {
        const int R = blockIdx.x / a.ncb, C = blockIdx.x % a.ncb;
        gr0 = a.r0 + R * BT;
        gc0 = a.c0 + C * BT;
        rend = m;
        cend = n;
        pend = left ? g > 0 : true;
    } else {
        const int t = blockIdx.x - a.nmain, q = t / a.thalves, h = t % a.thalves;
        if (left) {   // rows g.. in chunks, columns bs + 64 h ..
            gr0 = g + q * BT;
            rend = m;
            gc0 = a.bs + h * BT;
            cend = g;
        } else {      // rows bs + 64 h .., columns g+1.. in chunks
            gr0 = a.bs + h * BT;
            rend = g;
            gc0 = g + 1 + q * BT;
            cend = n;
        }
        pend = false;
    }
    if (tid < BT) {
        const int gr = gr0 + tid;
        const bool ok = gr < rend;
        // left: pending = y (rows) x v (cols), weights u on rows;
        // right: pending = u (rows) x w (cols), weights v on cols
        vr[0][tid] = (pend && ok) ? (left ? a.w.y[gr] : a.w.u[gr]) : 0.0;
        vr[1][tid] = (ok && left) ? a.w.u[gr] : 0.0;
    } else if (tid < 2 * BT) {
        const int t = tid - BT, gc = gc0 + t;
        const bool ok = gc < cend;
        vcl[0][t] = (pend && ok) ? (left ? a.w.v[gc] : a.w.w[gc]) : 0.0;
        vcl[1][t] = (ok && !left) ? a.w.v[gc] : 0.0;
    }
    __syncthreads();
    const int fg = tid & 15, sgp = tid >> 4;
    const int fq = fg * 4, sq = sgp * 4;
    double yy[4] = {0.0, 0.0, 0.0, 0.0}, zz[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int ks = 0; ks < 4; ks++) {
#pragma unroll
        for (int kf = 0; kf < 4; kf++) {
            const int r = rowmajor ? sq + ks : fq + kf, c = rowmajor ? fq + kf : sq + ks;
            const int gr = gr0 + r, gc = gc0 + c;
            if (gr >= rend || gc >= cend) continue;
            double *ptr = A + (i64)gr * a.rs + (i64)gc * a.cs;
            double v = *ptr;
            if (pend) {
                v = fma(-vr[0][r], vcl[0][c], v);
                *ptr = v;
            }
            yy[rowmajor ? ks : kf] = fma(v, vcl[1][c], yy[rowmajor ? ks : kf]);   // row sums (weights on cols)
            zz[rowmajor ? kf : ks] = fma(v, vr[1][r], zz[rowmajor ? kf : ks]);   // column sums (weights on rows)
        }
    }
    const int rq = rowmajor ? sq : fq, cq = rowmajor ? fq : sq;
    const int cgid = rowmajor ? fg : sgp, rgid = rowmajor ? sgp : fg;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        ysm[cgid][rq + k] = yy[k];
        zsm[rgid][cq + k] = zz[k];
    }
    __syncthreads();
    if (tid < BT) {
        double y = 0.0, z = 0.0;
#pragma unroll
        for (int q = 0; q < 16; q++) {
            y += ysm[q][tid];
            z += zsm[q][tid];
        }
        const double outv = left ? z : y;
        if (!tchunk) a.w.part[(i64)blockIdx.x * BT + tid] = outv;
        else a.w.tpart[(i64)((int)blockIdx.x - a.nmain) * BT + tid] = outv;
    }
}

// left: w(c) = sum over row blocks of the column sums, / tau, for the
// columns of block C = blockIdx.x; right: y(r) likewise over column blocks.
// CTA 0 also sums the T column.
__global__ void __launch_bounds__(BR_THREADS) k_bd_reduce(BdArgs a) {
    const int B = blockIdx.x, tid = threadIdx.x, k = tid & (BT - 1), q4 = tid >> 6;
    const bool left = a.left != 0;
    __shared__ double part4[4][BT];
    const bool have = left ? a.ncb > 0 : a.nrb > 0;   // the last column has no w
    const int nterm = have ? (left ? a.nrb : a.ncb) : 0;
    double acc = 0.0;
    for (int t = q4; t < nterm; t += 4) {
        const i64 tile = left ? (i64)t * a.ncb + B : (i64)B * a.ncb + t;
        acc += a.w.part[tile * BT + k];
    }
    part4[q4][k] = acc;
    __syncthreads();
    const double itau = a.w.scal[1];
    if (have && tid < BT) {
        const double s = (part4[0][tid] + part4[1][tid] + part4[2][tid] + part4[3][tid]) * itau;
        if (left) {
            const int c = a.c0 + B * BT + tid;
            if (c < a.n) a.w.w[c] = s;
        } else {
            const int r = a.r0 + B * BT + tid;
            if (r < a.m) a.w.y[r] = s;
        }
    }
    if (B == 0) {
        // T(j, g) = sum over chunks, j = 0 .. il-1 (up to two halves of 64)
        for (int j = tid; j < a.il; j += blockDim.x) {
            const int h = j / BT, kk = j % BT;
            double t = 0.0;
            for (int q = 0; q < a.tchunks; q++) t += a.w.tpart[((i64)q * a.thalves + h) * BT + kk];
            if (left) a.TU[(i64)j * a.n + a.g] = t;
            else a.TV[(i64)j * a.n + a.g] = t;
        }
    }
}

__global__ void k_bd_border(double *V, i64 rs, i64 cs, int n) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        V[(i64)k * cs] = k == 0 ? 1.0 : 0.0;
        V[(i64)k * rs] = k == 0 ? 1.0 : 0.0;
    }
}

}  // namespace

// Bidiag2 on device data: A (m x n, m >= n) is overwritten by the reflectors;
// d (n), e (n - 1), U (m x m), V (n x n).
int bidiag(ddla_handle h, i64 m, i64 n, View<double> A, double *d, double *e, View<double> U, View<double> V,
           int prec) {
    if (n <= 0) return 0;
    if (m < n) {
        set_error("bidiag: needs m >= n");
        return DDLA_ERR_UNSUPPORTED;
    }
    if (m > (i64)1 << 30) {
        set_error("bidiag: m too large");
        return DDLA_ERR_UNSUPPORTED;
    }
    cudaStream_t s = h->stream;
    const i64 nrbm = (m + BT - 1) / BT, ncbm = (n + BT - 1) / BT;
    const i64 tur = n < BD_NB ? n : BD_NB, tvr = (n - 1) < BD_NB ? (n - 1 > 0 ? n - 1 : 1) : BD_NB;
    const i64 chunks = (m + BT - 1) / BT + 1;
    const size_t nd = (size_t)(2 * m + 2 * n + nrbm * ncbm * BT + chunks * 2 * BT + 8 + tur * n + tvr * n);
    void *ws;
    DDLA_TRY(workspace(h, WS_TRD, sizeof(double) * nd, &ws));
    double *q = (double *)ws;
    BdWs w;
    w.u = q;
    w.y = q + m;
    w.v = q + 2 * m;
    w.w = q + 2 * m + n;
    w.part = q + 2 * m + 2 * n;
    w.tpart = w.part + nrbm * ncbm * BT;
    w.scal = w.tpart + chunks * 2 * BT;
    double *TU = w.scal + 8, *TV = TU + tur * n;   // row-major tur x n and tvr x n
    BdArgs a;
    a.A = A.p;
    a.rs = A.rs;
    a.cs = A.cs;
    a.m = (int)m;
    a.n = (int)n;
    a.w = w;
    a.TU = TU;
    a.TV = TV;
    a.d = d;
    a.e = e;
    const bool rowmajor = A.cs == 1 || (A.rs != 1 && llabs(A.cs) <= llabs(A.rs));
    auto sweep = [&](void) -> int {
        const int grid = a.nmain + a.tchunks * a.thalves;
        if (grid <= 0) return 0;
        if (rowmajor) k_bd_sweep<true><<<grid, BS_THREADS, 0, s>>>(a);
        else k_bd_sweep<false><<<grid, BS_THREADS, 0, s>>>(a);
        DDLA_LAUNCHED();
        return 0;
    };
    {
        Timed tm(s, TC_PANEL, 4.0 * (double)m * n * n - 4.0 * (double)n * n * n / 3.0, 0.0);
        for (i64 gi = 0; gi < n; gi++) {
            const int g = (int)gi;
            a.g = g;
            a.bs = (int)(gi / BD_NB * BD_NB);
            a.il = g - a.bs;
            // column step
            a.left = 1;
            k_bd_vec<<<1, 1024, 0, s>>>(a);
            DDLA_LAUNCHED();
            a.r0 = g;
            a.c0 = g + 1;
            a.nrb = (int)((m - g + BT - 1) / BT);
            a.ncb = (int)((n - g - 1 + BT - 1) / BT);
            a.nmain = a.nrb * a.ncb;
            a.tchunks = a.il > 0 ? a.nrb : 0;
            a.thalves = (a.il + BT - 1) / BT;
            if (a.thalves == 0) a.thalves = 1;
            DDLA_TRY(sweep());
            if (a.ncb > 0 || a.il > 0) {
                k_bd_reduce<<<a.ncb > 0 ? a.ncb : 1, BR_THREADS, 0, s>>>(a);
                DDLA_LAUNCHED();
            }
            if (g >= n - 1) break;
            // row step
            a.left = 0;
            k_bd_vec<<<1, 1024, 0, s>>>(a);
            DDLA_LAUNCHED();
            a.r0 = g + 1;
            a.c0 = g + 1;
            a.nrb = (int)((m - g - 1 + BT - 1) / BT);
            a.ncb = (int)((n - g - 1 + BT - 1) / BT);
            a.nmain = a.nrb * a.ncb;
            a.tchunks = a.il > 0 ? a.ncb : 0;
            a.thalves = (a.il + BT - 1) / BT;
            if (a.thalves == 0) a.thalves = 1;
            DDLA_TRY(sweep());
            k_bd_reduce<<<a.nrb > 0 ? a.nrb : 1, BR_THREADS, 0, s>>>(a);
            DDLA_LAUNCHED();
        }
        DDLA_CUDA(cudaGetLastError());
    }
    // BuildUV: U = H_0 ... H_{n-1} I; V = [1, 0; 0, G_0 ... G_{n-2} I]
    Timed tm(s, TC_UPDATE, 0.0, 0.0);
    DDLA_TRY(orgqr(h, m, n, View<const double>{A.p, m, n, A.rs, A.cs}, View<const double>{TU, tur, n, n, 1}, tur, U,
                   prec));
    if (n > 1) {
        DDLA_TRY(orgqr(h, n - 1, n - 1, View<const double>{A.p + A.cs, n - 1, n - 1, A.cs, A.rs},
                       View<const double>{TV, tvr, n - 1, n, 1}, tvr, View<double>{V.p + V.rs + V.cs, n - 1, n - 1, V.rs, V.cs},
                       prec));
    }
    // first row and column of V
    k_bd_border<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(V.p, V.rs, V.cs, (int)n);
    DDLA_LAUNCHED();
    return 0;
}

}  // namespace ddla
