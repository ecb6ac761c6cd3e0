// Two-stage bidiagonal reduction of an m x n matrix (m >= n): DDLA's
// Bidiagonaling.Bidiag, which its SVD calls (DDLA/Factorizations/SVD.cs:89,97),
// through TwoStageBidiag (DDLA/Transformations/Bidiagonaling.cs:334-582).
//
// Stage 1 (Ge2Bd, :384-474): blocks of 32 columns.  Each block column is
// reduced by a Householder QR (its block reflector then updates the columns
// to its right), and the block row right of it by an LQ -- a QR of its
// transpose, whose block reflector updates the rows below from the right.
// All of it runs on the QR path of this library (qr.cu: cluster panel
// kernels, FP64 DMMA or split-precision products for the block reflectors),
// on strided and transposed views of the work matrix.  U and V are then
// formed from the two sets of block reflectors (ApplyQlnfc), which leaves an
// upper band of width 32.
//
// Stage 2 (Bd2Bi, :478-582): for every row i a cycle of small reflectors
// (length <= 32) chases the band's row i to the superdiagonal, alternating a
// reflector from the right (on a transposed view) with one from the left
// (StepCycle, :489-516).  The cycles are sequential in DDLA; here consecutive
// cycles run concurrently on different CTAs of one cooperative launch: cycle
// s starts its t-th reflector only when cycle s - 1 has finished t + LAG of
// its own (or all of them).  LAG = 4 keeps every pair of reflectors that may
// run at the same time on disjoint parts of the band (the schedule test
// tests/test_bd_chase_schedule.py enumerates the regions and checks it).  The
// reflectors are stored in TU2 / TV2 (row i for cycle i) and applied to U and
// V afterwards, cycle by cycle (BackCycle, :518-537): the reflectors of one
// cycle act on disjoint column blocks, so one launch per cycle applies them
// all, a warp per (row, reflector).
//
// Every wait is bounded: on timeout the kernel sets an error word and
// returns; the host reports DDLA_ERR_TIMEOUT.
#include <algorithm>

#include "common.cuh"

namespace ddla {
namespace {

constexpr int BD2_BLOCK = 32;   // TwoStageBidiag.MaxBlockSize, Bidiagonaling.cs:336
constexpr int BD2_LAG = 4;      // reflectors cycle s - 1 stays ahead of cycle s
constexpr int BD2_THREADS = 256;
constexpr long long BD2_SPIN = 1LL << 26;

__global__ void k_zero_lower(double *A, i64 rs, i64 cs, i64 rows, i64 cols) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < rows * cols; e += (i64)gridDim.x * blockDim.x) {
        const i64 i = e / cols, j = e % cols;
        if (j < i) A[i * rs + j * cs] = 0.0;
    }
}

__global__ void k_eye2(double *Q, i64 n, i64 rs, i64 cs) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n * n; e += (i64)gridDim.x * blockDim.x)
        Q[(e / n) * rs + (e % n) * cs] = (e / n) == (e % n) ? 1.0 : 0.0;
}

__global__ void k_extract_bd(const double *A, i64 rs, i64 cs, i64 n, double *d, double *e) {
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        d[i] = A[i * rs + i * cs];
        if (i + 1 < n) e[i] = A[i * rs + (i + 1) * cs];
    }
}

// Number of reflectors of cycle i (the StepCycle sequence below).
__host__ __device__ inline int cycle_steps(i64 n, i64 i, int bs) {
    const i64 rows = n - i;
    if (rows <= 1 + bs) return 2;
    int k = 0;
    for (i64 ie2 = 1 + 2 * bs; ie2 < rows; ie2 += bs) k++;
    return 2 * k + 4;
}

struct ChaseArgs {
    double *W;
    i64 rs, cs, n;
    int bs;
    double *tu2, *tv2;   // n x n, row i = cycle i's reflectors (tau, then the vector)
    int *prog;           // reflectors finished per cycle
    int *err;
};

// StepSide (Bidiagonaling.cs:539-551) on the view M = sub(W, r0, nr, c0, nc),
// transposed when `trans`: the reflector of M's first column
// (HouseHolder.BuildHouseHolder, HouseHolder.cs:34-58) is applied from the
// left to M's other columns (ApplyHouseHolder, HouseHolder.cs:95-115); tau and
// the vector go to t, the column's tail is cleared.  All threads of the CTA.
__device__ void step_side(const ChaseArgs &a, i64 r0, i64 nr, i64 c0, i64 nc, bool trans, double *t) {
    __shared__ double s_u[BD2_BLOCK];
    __shared__ double s_tau;
    const int tid = threadIdx.x, lane = tid & 31;
    double *p = a.W + r0 * a.rs + c0 * a.cs;
    const i64 R = trans ? nc : nr, Cc = trans ? nr : nc;
    auto M = [&](i64 r, i64 c) -> double & { return trans ? p[c * a.rs + r * a.cs] : p[r * a.rs + c * a.cs]; };
    const int len = (int)(R - 1);
    if (tid < 32) {
        // every lane reads chi before the shuffles, lane 0 writes it after them
        const double x = lane < len ? M(1 + lane, 0) : 0.0;
        double chi = M(0, 0), tau, u = x;
        double s = x * x;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        const double nrm = sqrt(s);
        if (nrm == 0.0) {
            chi = -chi;
            tau = 0.5;
        } else {
            const double alpha = hypot(chi, nrm);
            const double rho = -copysign(alpha, chi);
            const double miu = chi - rho;
            chi = rho;
            u = x * (1.0 / miu);
            const double sc = nrm / fabs(miu);
            tau = (1.0 + sc * sc) / 2.0;
        }
        if (lane < len) {
            s_u[lane] = u;
            t[1 + lane] = u;
            M(1 + lane, 0) = 0.0;
        }
        if (lane == 0) {
            M(0, 0) = chi;
            t[0] = tau;
            s_tau = tau;
        }
    }
    __syncthreads();
    // w_j = a1_j + sum_l A2(l, j) u_l, w_j /= tau, a1_j -= w_j, A2(:, j) -= u w_j
    const double rt = 1.0 / s_tau;
    for (i64 j = 1 + tid; j < Cc; j += blockDim.x) {
        double w = M(0, j);
        for (int l = 0; l < len; l++) w = fma(M(1 + l, j), s_u[l], w);
        w *= rt;
        M(0, j) -= w;
        for (int l = 0; l < len; l++) M(1 + l, j) = fma(-s_u[l], w, M(1 + l, j));
    }
    __syncthreads();
}

// The bulge chase: CTA b runs cycles b, b + gridDim.x, ... in order.
__global__ void __launch_bounds__(BD2_THREADS) k_bd_chase(ChaseArgs a) {
    __shared__ int s_abort;
    const int tid = threadIdx.x;
    for (i64 s = blockIdx.x; s + 1 < a.n; s += gridDim.x) {
        const int bs = a.bs;
        const i64 rows = a.n - s;
        const int before = s > 0 ? cycle_steps(a.n, s - 1, bs) : 0;
        double *tu = a.tu2 + s * a.n + s, *tv = a.tv2 + s * a.n + s;
        int step = 0;
        bool abort = false;
        // one reflector of this cycle on sub(cycle view, r0, nr, c0, nc)
        auto side = [&](i64 r0, i64 nr, i64 c0, i64 nc, bool trans, double *t) {
            if (abort) return;
            if (s > 0) {
                const int want = step + BD2_LAG < before ? step + BD2_LAG : before;
                if (tid == 0) {
                    int ok = 0;
                    for (long long it = 0; it < BD2_SPIN; it++) {
                        if (*(volatile int *)&a.prog[s - 1] >= want) { ok = 1; break; }
                        if (*(volatile int *)a.err) break;   // another cycle gave up
                    }
                    __threadfence();
                    s_abort = !ok;
                    if (!ok) atomicExch(a.err, 1);
                }
                __syncthreads();
                abort = s_abort != 0;
                __syncthreads();
                if (abort) return;
            }
            step_side(a, s + r0, nr, s + c0, nc, trans, t);
            step++;
            if (tid == 0) {
                __threadfence();
                atomicExch(&a.prog[s], step);
            }
        };
        const i64 is0 = 1, ie0 = 1 + bs;
        if (rows <= ie0) {
            side(0, rows, is0, rows - is0, true, tv + is0);
            side(is0, rows - is0, is0, rows - is0, false, tu + is0);
        } else {
            i64 is = is0, ie = ie0, ie2 = ie0 + bs;
            side(0, ie, is, ie - is, true, tv + is);
            while (ie2 < rows) {
                side(is, ie - is, is, ie2 - is, false, tu + is);
                side(is, ie2 - is, ie, ie2 - ie, true, tv + ie);
                is += bs;
                ie += bs;
                ie2 += bs;
            }
            side(is, ie - is, is, rows - is, false, tu + is);
            side(is, rows - is, ie, rows - ie, true, tv + ie);
            side(ie, rows - ie, ie, rows - ie, false, tu + ie);
        }
        if (abort) return;
    }
}

// BackCycle of cycle i (Bidiagonaling.cs:518-537): Q <- Q H_k for every
// reflector k of the cycle, H_k = I - u u^T / tau on columns i + is_k ..
// i + ie_k of Q (ApplyHouseHolder on Q^T from the left).  A warp per
// (row of Q, reflector): lane l holds column c0 + l.
__global__ void k_bd_back(double *Q, i64 rows, i64 rs, i64 cs, const double *t2, i64 n, i64 i, int bs, int nref) {
    const int lane = threadIdx.x & 31;
    const i64 wid = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
    if (wid >= rows * nref) return;
    const i64 r = wid / nref;
    const int k = (int)(wid % nref);
    const i64 cyc = n - i;
    const i64 is = 1 + (i64)k * bs, ie = is + bs < cyc ? is + bs : cyc;
    const int len = (int)(ie - is);
    const double *t = t2 + i * n + i + is;
    const double tau = t[0];
    if (tau == 0.0) return;
    const i64 c0 = i + is;
    const double q = lane < len ? Q[r * rs + (c0 + lane) * cs] : 0.0;
    const double u = lane == 0 ? 1.0 : (lane < len ? t[lane] : 0.0);
    double w = lane == 0 ? 0.0 : q * u;
    for (int off = 16; off > 0; off >>= 1) w += __shfl_xor_sync(0xffffffffu, w, off);
    w = (__shfl_sync(0xffffffffu, q, 0) + w) * (1.0 / tau);
    if (lane == 0) Q[r * rs + c0 * cs] = q - w;
    else if (lane < len) Q[r * rs + (c0 + lane) * cs] = fma(-u, w, q);
}

}  // namespace

// Bidiagonaling.Bidiag(A, U, V, d, e) on device data: A (m x n, m >= n) is
// overwritten, U (m x m) and V (n x n) receive the orthogonal factors with
// U^T A_in V = bidiag(d, e).  prec DDLA_PREC_OZAKI runs stage 1's block
// reflector products through the split-precision tensor-core GEMM.
int bidiag2s(ddla_handle h, i64 m, i64 n, View<double> A, View<double> U, View<double> V, double *d, double *e,
             int prec) {
    if (n == 0) return 0;
    cudaStream_t s = h->stream;
    const i64 bs = n < BD2_BLOCK ? n : BD2_BLOCK;
    const i64 tvc = n - bs;
    // workspace: TU (bs x n), TV (bs x tvc), TU2, TV2 (n x n), progress, error
    const size_t nd = (size_t)bs * n + (size_t)bs * (tvc > 0 ? tvc : 1) + 2 * (size_t)n * n;
    void *ws;
    DDLA_TRY(workspace(h, WS_BD2, sizeof(double) * nd + sizeof(int) * ((size_t)n + 8), &ws));
    double *TU = (double *)ws, *TV = TU + (size_t)bs * n, *TU2 = TV + (size_t)bs * (tvc > 0 ? tvc : 1),
           *TV2 = TU2 + (size_t)n * n;
    int *prog = (int *)(TV2 + (size_t)n * n), *err = prog + n;
    DDLA_CUDA(cudaMemsetAsync(TU, 0, sizeof(double) * nd, s));
    DDLA_CUDA(cudaMemsetAsync(prog, 0, sizeof(int) * ((size_t)n + 8), s));
    auto grid_of = [](i64 tot) { return (unsigned)std::max<i64>(1, std::min<i64>((tot + 255) / 256, 8192)); };
    // ---- stage 1: Ge2Bd
    for (i64 i0 = 0; i0 < n;) {
        const i64 b = n - i0 < BD2_BLOCK ? n - i0 : BD2_BLOCK;
        View<double> AB1 = A.sub(i0, m - i0, i0, b);
        View<double> TUb{TU + i0, b, b, n, 1};
        DDLA_TRY(geqrf(h, m - i0, b, AB1, TUb, b, prec));
        const i64 c22 = n - i0 - b;
        if (c22 > 0) {
            DDLA_TRY(ormqr(h, true, m - i0, b, View<const double>{AB1.p, AB1.rows, AB1.cols, AB1.rs, AB1.cs},
                           View<const double>{TUb.p, b, b, TUb.rs, TUb.cs}, b, A.sub(i0, m - i0, i0 + b, c22), prec));
            // the block row right of it (the ragged last one takes all the remaining columns' width)
            const i64 b2 = c22 < BD2_BLOCK ? c22 : b;
            View<double> R = A.sub(i0, b2, i0 + b, c22).t();          // c22 x b2
            View<double> below = A.sub(i0 + b2, m - i0 - b2, i0 + b, c22).t();
            View<double> TVb{TV + i0, b2, b2, tvc, 1};
            DDLA_TRY(geqrf(h, c22, b2, R, TVb, b2, prec));
            DDLA_TRY(ormqr(h, true, c22, b2, View<const double>{R.p, R.rows, R.cols, R.rs, R.cs},
                           View<const double>{TVb.p, b2, b2, TVb.rs, TVb.cs}, b2, below, prec));
        }
        i0 += b;
    }
    // U and V from the block reflectors (ApplyQlnfc); A keeps the band
    k_eye2<<<grid_of(m * m), 256, 0, s>>>(U.p, m, U.rs, U.cs);
    DDLA_LAUNCHED();
    DDLA_TRY(ormqr(h, false, m, n, View<const double>{A.p, m, n, A.rs, A.cs}, View<const double>{TU, bs, n, n, 1}, bs,
                   U, prec));
    k_zero_lower<<<grid_of(m * n), 256, 0, s>>>(A.p, A.rs, A.cs, m, n);
    DDLA_LAUNCHED();
    k_eye2<<<grid_of(n * n), 256, 0, s>>>(V.p, n, V.rs, V.cs);
    DDLA_LAUNCHED();
    if (tvc > 0) {
        View<double> Al = A.sub(0, tvc, bs, tvc).t();
        DDLA_TRY(ormqr(h, false, tvc, tvc, View<const double>{Al.p, tvc, tvc, Al.rs, Al.cs},
                       View<const double>{TV, bs, tvc, tvc, 1}, bs, V.sub(bs, tvc, bs, tvc), prec));
        k_zero_lower<<<grid_of(tvc * tvc), 256, 0, s>>>(Al.p, Al.rs, Al.cs, tvc, tvc);
        DDLA_LAUNCHED();
    }
    // ---- stage 2: Bd2Bi
    if (n > 1) {
        ChaseArgs ca{A.p, A.rs, A.cs, n, (int)bs, TU2, TV2, prog, err};
        int per_sm = 0;
        DDLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bd_chase, BD2_THREADS, 0));
        const i64 cyc = n - 1;
        const int grid = (int)std::max<i64>(1, std::min<i64>(cyc, (i64)h->sm_count * std::max(per_sm, 1)));
        void *args[] = {&ca};
        DDLA_CUDA(cudaLaunchCooperativeKernel((const void *)k_bd_chase, dim3(grid), dim3(BD2_THREADS), args, 0, s));
        DDLA_LAUNCHED();
        for (i64 i = 0; i + 1 < n; i++) {
            const int nref = (int)((n - i - 2) / bs + 1);
            const i64 wv = n * nref, wu = m * nref;
            k_bd_back<<<(unsigned)((wv * 32 + 255) / 256), 256, 0, s>>>(V.p, n, V.rs, V.cs, TV2, n, i, (int)bs, nref);
            DDLA_LAUNCHED();
            k_bd_back<<<(unsigned)((wu * 32 + 255) / 256), 256, 0, s>>>(U.p, m, U.rs, U.cs, TU2, n, i, (int)bs, nref);
            DDLA_LAUNCHED();
        }
    }
    k_extract_bd<<<grid_of(n), 256, 0, s>>>(A.p, A.rs, A.cs, n, d, e);
    DDLA_LAUNCHED();
    int herr = 0;
    DDLA_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    DDLA_CUDA(cudaStreamSynchronize(s));
    if (herr) {
        set_error("bidiag (two-stage): a bounded wait of the bulge chase gave up");
        return DDLA_ERR_TIMEOUT;
    }
    return 0;
}

}  // namespace ddla
