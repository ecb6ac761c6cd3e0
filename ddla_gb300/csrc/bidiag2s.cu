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
// V afterwards (BackCycle, :518-537), 32 cycles per launch with the rows of U
// and V streamed through shared memory once per launch and the reflectors
// applied four at a time in compact WY form (k_bd_back).
//
// Every wait is bounded: on timeout the kernel sets an error word and
// returns; the host reports DDLA_ERR_TIMEOUT.
#include <algorithm>

#include "common.cuh"
#include "timing.cuh"

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

// tau of reflector j from the diagonal of its block's factor: T (bs rows,
// leading dimension ldt) holds block i0's factor at columns i0 .. i0 + bs.
__global__ void k_taus(const double *T, i64 ldt, i64 k, int bs, double *tau) {
    for (i64 j = blockIdx.x * (i64)blockDim.x + threadIdx.x; j < k; j += (i64)gridDim.x * blockDim.x)
        tau[j] = T[(j % bs) * ldt + j];
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

// Progress counters between chase cycles: a release store after the CTA's
// closing barrier publishes every thread's writes of the reflector (the
// barrier orders them before it); an acquire load by the waiting CTA's
// thread 0, followed by a barrier, makes them visible to all its threads.
__device__ __forceinline__ int prog_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void prog_release(int *p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

struct ChaseArgs {
    double *W;
    i64 rs, cs, n;
    int bs;
    double *tu2, *tv2;   // n x n, row i = cycle i's reflectors (tau, then the vector)
    int *prog;           // reflectors finished per cycle
    int *err;
    int build_solo;      // 1: warp 0 alone builds each reflector
};

// Geometry of reflector t of a cycle with `rows` rows left (Bd2Bi_StepCycle,
// Bidiagonaling.cs:489-516): the StepSide view sub(cycle, r0, nr, c0, nc),
// transposed for a reflector from the right (stored in TV2) and plain for one
// from the left (TU2); toff is its offset in the cycle's row of TU2 / TV2.
struct StepGeom {
    i64 r0, nr, c0, nc, toff;
    bool trans;
};

__device__ inline StepGeom step_geom(i64 rows, int bs, int t, int steps) {
    if (rows <= 1 + bs) {
        if (t == 0) return {0, rows, 1, rows - 1, 1, true};
        return {1, rows - 1, 1, rows - 1, 1, false};
    }
    const int K = (steps - 4) / 2;   // passes of the StepCycle loop
    if (t == 0) return {0, 1 + bs, 1, bs, 1, true};
    if (t <= 2 * K) {
        const i64 is = 1 + (i64)((t - 1) / 2) * bs, ie = is + bs;
        if ((t - 1) % 2 == 0) return {is, bs, is, 2 * (i64)bs, is, false};
        return {is, 2 * (i64)bs, ie, bs, ie, true};
    }
    const i64 is = 1 + (i64)K * bs, ie = is + bs;
    if (t == 2 * K + 1) return {is, bs, is, rows - is, is, false};
    if (t == 2 * K + 2) return {is, rows - is, ie, rows - ie, ie, true};
    return {ie, rows - ie, ie, rows - ie, ie, false};
}

// StepSide (Bidiagonaling.cs:539-551) on M = the view of g (R <= 32 rows,
// Cc <= 64 columns): the reflector of M's first column
// (HouseHolder.BuildHouseHolder, HouseHolder.cs:34-58) applied from the left
// to M's other columns (ApplyHouseHolder, HouseHolder.cs:95-115); tau and the
// vector go to t, the column's tail is cleared.  Warp 0 builds the
// reflector and shares it through one barrier (on GB300 the FP64 square
// roots and divisions cost more than the barrier: 94 against 125 ms of chase
// at n = 4096); with the tuning key bidiag2s.build_solo = 0 every warp builds
// it and no barrier is taken.  1 / tau is formed once in the build.  Four threads per column split its
// dot product, with the column's entries loaded before the reflector is
// known.  Warp 0 writes column 0 and the reflector: right after the build
// when it builds alone (no other warp reads column 0), else after the
// closing barrier.
__device__ void step_side(const ChaseArgs &a, i64 s, const StepGeom &g, double *t) {
    __shared__ double s_u[BD2_THREADS / 32][BD2_BLOCK];
    __shared__ double s_rt;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double *p = a.W + (s + g.r0) * a.rs + (s + g.c0) * a.cs;
    const i64 ers = g.trans ? a.cs : a.rs, ecs = g.trans ? a.rs : a.cs;   // M(r, c) = p[r ers + c ecs]
    const int R = (int)(g.trans ? g.nc : g.nr), Cc = (int)(g.trans ? g.nr : g.nc);
    const int len = R - 1;
    const int j = 1 + (tid >> 2), sub = tid & 3;
    const bool colv = j < Cc;
    double v[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int l = sub + 4 * i;
        v[i] = colv && l < len ? p[(1 + l) * ers + j * ecs] : 0.0;
    }
    const double a1 = colv ? p[j * ecs] : 0.0;
    // the reflector: by every warp (no barrier), or by warp 0 alone with one
    // barrier (the FP64 square roots and divisions then run once per CTA)
    const bool solo = a.build_solo != 0;
    double chi = 0.0, tau = 0.5, rtau = 2.0, u = 0.0;
    if (!solo || warp == 0) {
        const double x = lane < len ? p[(1 + lane) * ers] : 0.0;
        chi = p[0];
        u = x;
        double ss = x * x;
        for (int off = 16; off > 0; off >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, off);
        if (ss == 0.0) {
            chi = -chi;
        } else {
            const double alpha = hypot(chi, sqrt(ss));
            const double rho = -copysign(alpha, chi);
            const double miu = chi - rho;
            const double rmiu = 1.0 / miu;
            chi = rho;
            u = x * rmiu;
            tau = (1.0 + ss * rmiu * rmiu) / 2.0;   // (1 + (|x| / |miu|)^2) / 2
            rtau = 1.0 / tau;
        }
        s_u[warp][lane] = u;
        if (solo) {
            // only warp 0 reads column 0 in this mode: it stores the reflector
            // and the column now, so the closing barrier covers them (the
            // warp barrier orders every lane's read of p[0] before lane 0's store)
            if (lane == 0) s_rt = rtau;
            __syncwarp();
            if (lane < len) {
                t[1 + lane] = u;
                p[(1 + lane) * ers] = 0.0;
            }
            if (lane == 0) {
                p[0] = chi;
                t[0] = tau;
            }
        }
    }
    if (solo) __syncthreads();
    else __syncwarp();
    const double *su = s_u[solo ? 0 : warp];
    const double rt = solo ? s_rt : rtau;
    double part = 0.0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int l = sub + 4 * i;
        if (l < len) part = fma(v[i], su[l], part);
    }
    part += __shfl_xor_sync(0xffffffffu, part, 1);
    part += __shfl_xor_sync(0xffffffffu, part, 2);
    const double w = (a1 + part) * rt;
    if (colv) {
        if (sub == 0) p[j * ecs] = a1 - w;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int l = sub + 4 * i;
            if (l < len) p[(1 + l) * ers + j * ecs] = fma(-su[l], w, v[i]);
        }
    }
    __syncthreads();   // every warp has read column 0
    if (!solo && warp == 0) {
        if (lane < len) {
            t[1 + lane] = u;
            p[(1 + lane) * ers] = 0.0;
        }
        if (lane == 0) {
            p[0] = chi;
            t[0] = tau;
        }
        __syncwarp();
    }
}

// The bulge chase: CTA b runs cycles b, b + gridDim.x, ... in order; reflector
// t of cycle s waits until cycle s - 1 has finished min(t + LAG, all).
__global__ void __launch_bounds__(BD2_THREADS) k_bd_chase(ChaseArgs a) {
    __shared__ int s_abort;
    const int tid = threadIdx.x;
    for (i64 s = blockIdx.x; s + 1 < a.n; s += gridDim.x) {
        const i64 rows = a.n - s;
        const int steps = cycle_steps(a.n, s, a.bs);
        const int before = s > 0 ? cycle_steps(a.n, s - 1, a.bs) : 0;
        for (int t = 0; t < steps; t++) {
            if (tid == 0) {
                int ok = 1;
                if (s > 0) {
                    const int want = t + BD2_LAG < before ? t + BD2_LAG : before;
                    ok = 0;
                    for (long long it = 0; it < BD2_SPIN; it++) {
                        if (prog_acquire(&a.prog[s - 1]) >= want) { ok = 1; break; }
                        if (*(volatile int *)a.err) break;   // another cycle gave up
                    }
                    if (!ok) atomicExch(a.err, 1);
                }
                s_abort = !ok;
            }
            __syncthreads();   // the wait, and this CTA's previous reflector, are complete
            if (s_abort) return;
            const StepGeom g = step_geom(rows, a.bs, t, steps);
            step_side(a, s, g, (g.trans ? a.tv2 : a.tu2) + s * a.n + s + g.toff);
            if (tid == 0) prog_release(&a.prog[s], t + 1);
        }
    }
}

// BackCycle (Bidiagonaling.cs:518-537) of the cycles i0 .. i0 + G - 1 (G =
// the block width bs): Q <- Q H for every reflector H = I - u u^T / tau of
// those cycles, on U (TU2's reflectors) and V (TV2's) in one launch.
// Reflector k of cycle i0 + g acts on columns base_k + g .. + len, base_k =
// i0 + 1 + bs k.  Running k from the last down and, for each k, g upward
// keeps DDLA's order wherever two reflectors overlap: (g, k) overlaps only
// (g', k) and (g', k + 1) with g' < g, which it must follow, and (g', k) and
// (g', k - 1) with g' > g, which must follow it.  So a row of Q needs only a
// window of 2 bs - 1 columns per k: a CTA (one warp, 8 rows) keeps the
// window of its rows in shared memory, writes back the bs columns that no
// later k touches, shifts and loads the next bs; every element of U and V is
// read and written once per group of cycles.
//
// The reflectors of one k are applied four at a time in compact WY form: for
// a row q and reflectors a = 0..3 (in order), d_a = q . u_a, w S = d with S
// upper triangular, S_aa = tau_a, S_ab = u_a . u_b (a < b), and q -= sum_a
// w_a u_a -- the same product as applying them one by one.  Z = S^-1 comes
// from k_bd_back_prep.  Four threads per row: thread p sums the terms
// l = p mod 4 of the four dot products and updates the columns = p mod 4.
constexpr int BK_RB = 8;    // rows of Q per CTA
constexpr int BK_WP = 68;   // window pitch (63 columns used): 8 r + 2 p distinct banks
constexpr int BK_Q = 4;     // reflectors per WY block

__host__ __device__ inline int refl_len(i64 n, i64 i, int bs, int k) {
    // length of reflector k of cycle i, 0 if the cycle has no k-th reflector
    const i64 rem = n - i - 1 - (i64)bs * k;
    return rem <= 0 ? 0 : (int)(rem < bs ? rem : bs);
}

// Z = S^-1 of every WY block: grid (k, U/V), thread j = block j of the k.
__global__ void k_bd_back_prep(const double *tu2, const double *tv2, i64 n, int bs, i64 i0, int G, int kcount,
                               double *Zq) {
    const int k = blockIdx.x, which = blockIdx.y, j = threadIdx.x;
    if (j >= BD2_BLOCK / BK_Q) return;
    const double *T = which == 0 ? tu2 : tv2;
    int len[BK_Q];
    const double *t[BK_Q];
    double S[BK_Q][BK_Q], Z[BK_Q][BK_Q];
    for (int a = 0; a < BK_Q; a++) {
        const int g = BK_Q * j + a;
        const i64 i = i0 + g;
        len[a] = g < G ? refl_len(n, i, bs, k) : 0;
        t[a] = T + i * n + i + 1 + (i64)bs * k;
    }
    for (int a = 0; a < BK_Q; a++)
        for (int b = 0; b < BK_Q; b++) {
            double v = 0.0;
            if (a == b) v = len[a] ? t[a][0] : 1.0;
            else if (a < b && len[a] && len[b])
                for (int c = b; c < a + len[a] && c - b < len[b]; c++)
                    v = fma(c == a ? 1.0 : t[a][c - a], c == b ? 1.0 : t[b][c - b], v);
            S[a][b] = v;
            Z[a][b] = 0.0;
        }
    for (int c = 0; c < BK_Q; c++) {
        Z[c][c] = 1.0 / S[c][c];
        for (int r = c - 1; r >= 0; r--) {
            double v = 0.0;
            for (int l = r + 1; l <= c; l++) v = fma(S[r][l], Z[l][c], v);
            Z[r][c] = -v / S[r][r];
        }
    }
    double *out = Zq + (((i64)which * kcount + k) * (BD2_BLOCK / BK_Q) + j) * BK_Q * BK_Q;
    for (int a = 0; a < BK_Q; a++)
        for (int b = 0; b < BK_Q; b++) out[a * BK_Q + b] = Z[a][b];
}

__global__ void __launch_bounds__(32) k_bd_back(double *U, i64 m, i64 rsu, i64 csu, double *V, i64 rsv, i64 csv,
                                                 const double *tu2, const double *tv2, const double *Zq, i64 n,
                                                 int bs, i64 i0, int ublocks) {
    __shared__ double sQ[BK_RB * BK_WP];
    __shared__ double sU[BD2_BLOCK * BD2_BLOCK];
    __shared__ double sZ[BD2_BLOCK * BK_Q];
    const int lane = threadIdx.x, r = lane >> 2, p = lane & 3;
    const bool isu = (int)blockIdx.x < ublocks;
    const i64 rb = isu ? blockIdx.x : blockIdx.x - ublocks;
    const i64 rows = isu ? m : n, rs = isu ? rsu : rsv, cs = isu ? csu : csv;
    const double *T = isu ? tu2 : tv2;
    const i64 row = rb * BK_RB + r;
    const bool live = row < rows;
    double *qrow = (isu ? U : V) + (live ? row : 0) * rs;
    double *sq = sQ + r * BK_WP;
    const int G = (int)(n - 1 - i0 < bs ? n - 1 - i0 : bs), WW = 2 * bs - 1;
    const int kmax = (int)((n - i0 - 2) / bs), kcount = kmax + 1;
    i64 base = i0 + 1 + (i64)bs * kmax;
    for (int j = p; j < BK_WP; j += 4) sq[j] = j < WW && live && base + j < n ? qrow[(base + j) * cs] : 0.0;
    for (int k = kmax; k >= 0; k--) {
        base = i0 + 1 + (i64)bs * k;
        // the reflectors of this k, u(0) = 1, zero past their length
        int gk = 0;
        for (int e = lane; e < BD2_BLOCK * BD2_BLOCK; e += 32) {
            const int g = e >> 5, l = e & 31;
            const int len = g < G ? refl_len(n, i0 + g, bs, k) : 0;
            const double *t = T + (i0 + g) * n + i0 + g + 1 + (i64)bs * k;
            sU[e] = l < len ? (l == 0 ? 1.0 : t[l]) : 0.0;
            if (len) gk = g + 1;
        }
        for (int o = 16; o > 0; o >>= 1) gk = max(gk, __shfl_xor_sync(0xffffffffu, gk, o));
        const double *zk = Zq + ((isu ? 0 : 1) * (i64)kcount + k) * BD2_BLOCK * BK_Q;
        for (int e = lane; e < BD2_BLOCK * BK_Q; e += 32) sZ[e] = zk[e];
        __syncwarp();
        for (int g0 = 0; g0 < gk; g0 += BK_Q) {
            const double *u = sU + g0 * BD2_BLOCK;
            double d[BK_Q] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int l = p + 4 * i;
#pragma unroll
                for (int a = 0; a < BK_Q; a++) d[a] = fma(sq[g0 + a + l], u[a * BD2_BLOCK + l], d[a]);
            }
#pragma unroll
            for (int a = 0; a < BK_Q; a++) {
                d[a] += __shfl_xor_sync(0xffffffffu, d[a], 1);
                d[a] += __shfl_xor_sync(0xffffffffu, d[a], 2);
            }
            const double *z = sZ + (g0 / BK_Q) * BK_Q * BK_Q;
            double w[BK_Q];
#pragma unroll
            for (int a = 0; a < BK_Q; a++) {
                w[a] = 0.0;
#pragma unroll
                for (int b = 0; b <= a; b++) w[a] = fma(d[b], z[b * BK_Q + a], w[a]);
            }
            // columns g0 + t, t = p mod 4, t < 32 + BK_Q - 1
#pragma unroll
            for (int s2 = 0; s2 < 9; s2++) {
                const int t = p + 4 * s2;
                if (t < BD2_BLOCK + BK_Q - 1) {
                    double acc = sq[g0 + t];
#pragma unroll
                    for (int a = 0; a < BK_Q; a++) {
                        const int l = t - a;
                        if (l >= 0 && l < BD2_BLOCK) acc = fma(-w[a], u[a * BD2_BLOCK + l], acc);
                    }
                    sq[g0 + t] = acc;
                }
            }
            __syncwarp();
        }
        // columns base + bs - 1 .. base + WW are final for this group
        for (int j = (k == 0 ? 0 : bs - 1) + p; j < WW; j += 4)
            if (live && base + j < n) qrow[(base + j) * cs] = sq[j];
        if (k == 0) break;
        __syncwarp();
        for (int j = p; j < bs - 1; j += 4) sq[bs + j] = sq[j];
        __syncwarp();
        for (int j = p; j < bs; j += 4) sq[j] = live && base - bs + j < n ? qrow[(base - bs + j) * cs] : 0.0;
        __syncwarp();
    }
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
    // U and V are formed from block reflectors of up to FB columns
    const i64 FB = std::max<i64>(bs, std::min<i64>(256, tune_get("bidiag2s.form_nb", 128)));
    const size_t nd = (size_t)bs * n + (size_t)bs * (tvc > 0 ? tvc : 1) + 2 * (size_t)n * n;
    const size_t nf = (size_t)FB * FB + 2 * (size_t)n + (size_t)FB * m;
    const size_t nz = 2 * (size_t)(n / bs + 2) * BD2_BLOCK * BK_Q;
    void *ws;
    DDLA_TRY(workspace(h, WS_BD2, sizeof(double) * (nd + nf + nz) + sizeof(int) * ((size_t)n + 8), &ws));
    double *TU = (double *)ws, *TV = TU + (size_t)bs * n, *TU2 = TV + (size_t)bs * (tvc > 0 ? tvc : 1),
           *TV2 = TU2 + (size_t)n * n;
    double *Sf = TV2 + (size_t)n * n, *tauf = Sf + (size_t)FB * FB, *Wf = tauf + 2 * (size_t)n;
    double *Zq = Wf + (size_t)FB * m;
    int *prog = (int *)(Zq + nz), *err = prog + n;
    DDLA_CUDA(cudaMemsetAsync(TU, 0, sizeof(double) * nd, s));
    DDLA_CUDA(cudaMemsetAsync(prog, 0, sizeof(int) * ((size_t)n + 8), s));
    auto grid_of = [](i64 tot) { return (unsigned)std::max<i64>(1, std::min<i64>((tot + 255) / 256, 8192)); };
    // ---- stage 1: Ge2Bd
    {
    Timed tm(s, TC_BD_BAND, 4.0 * m * n * n - 4.0 * n * n * n / 3.0 + 4.0 * m * m * n - 2.0 * m * n * n, 0.0);
    for (i64 i0 = 0; i0 < n;) {
        const i64 b = n - i0 < BD2_BLOCK ? n - i0 : BD2_BLOCK;
        View<double> AB1 = A.sub(i0, m - i0, i0, b);
        View<double> TUb{TU + i0, b, b, n, 1};
        DDLA_TRY(geqrf(h, m - i0, b, AB1, TUb, b, prec));
        const i64 c22 = n - i0 - b;
        if (c22 > 0) {
            DDLA_TRY(ormqr(h, true, m - i0, b, View<const double>{AB1.p, AB1.rows, AB1.cols, AB1.rs, AB1.cs},
                           View<const double>{TUb.p, b, b, TUb.rs, TUb.cs}, b, A.sub(i0, m - i0, i0 + b, c22), prec,
                           BD2_BLOCK));
            // the block row right of it (the ragged last one takes all the remaining columns' width)
            const i64 b2 = c22 < BD2_BLOCK ? c22 : b;
            View<double> R = A.sub(i0, b2, i0 + b, c22).t();          // c22 x b2
            View<double> below = A.sub(i0 + b2, m - i0 - b2, i0 + b, c22).t();
            View<double> TVb{TV + i0, b2, b2, tvc, 1};
            DDLA_TRY(geqrf(h, c22, b2, R, TVb, b2, prec));
            DDLA_TRY(ormqr(h, true, c22, b2, View<const double>{R.p, R.rows, R.cols, R.rs, R.cs},
                           View<const double>{TVb.p, b2, b2, TVb.rs, TVb.cs}, b2, below, prec, BD2_BLOCK));
        }
        i0 += b;
    }
    // U and V from the block reflectors (ApplyQlnfc); A keeps the band.  The
    // blocks of bs reflectors are joined into blocks of FB (their factor is
    // the same triu(U^T U) with the taus on the diagonal) and applied last
    // first to the identity, each only to the columns it can change.
    auto form = [&](View<const double> R, i64 rows, i64 k, const double *T, i64 ldt, View<double> Q) -> int {
        k_taus<<<grid_of(k), 256, 0, s>>>(T, ldt, k, (int)bs, tauf);
        DDLA_LAUNCHED();
        for (i64 j0 = ((k - 1) / FB) * FB; j0 >= 0; j0 -= FB) {
            const i64 b = k - j0 < FB ? k - j0 : FB;
            View<const double> Ub = R.sub(j0, rows - j0, j0, b);
            DDLA_TRY(qr_tfactor(h, Ub, b, tauf + j0, View<double>{Sf, b, b, FB, 1}));
            DDLA_TRY(qr_apply_block(h, false, Ub, b, View<const double>{Sf, b, b, FB, 1},
                                    Q.sub(j0, rows - j0, j0, rows - j0), Wf, prec));
        }
        return 0;
    };
    k_eye2<<<grid_of(m * m), 256, 0, s>>>(U.p, m, U.rs, U.cs);
    DDLA_LAUNCHED();
    DDLA_TRY(form(View<const double>{A.p, m, n, A.rs, A.cs}, m, n, TU, n, U));
    k_zero_lower<<<grid_of(m * n), 256, 0, s>>>(A.p, A.rs, A.cs, m, n);
    DDLA_LAUNCHED();
    k_eye2<<<grid_of(n * n), 256, 0, s>>>(V.p, n, V.rs, V.cs);
    DDLA_LAUNCHED();
    if (tvc > 0) {
        View<double> Al = A.sub(0, tvc, bs, tvc).t();
        DDLA_TRY(form(View<const double>{Al.p, tvc, tvc, Al.rs, Al.cs}, tvc, tvc, TV, tvc, V.sub(bs, tvc, bs, tvc)));
        k_zero_lower<<<grid_of(tvc * tvc), 256, 0, s>>>(Al.p, Al.rs, Al.cs, tvc, tvc);
        DDLA_LAUNCHED();
    }
    }
    // ---- stage 2: Bd2Bi
    if (n > 1) {
        ChaseArgs ca{A.p, A.rs, A.cs, n, (int)bs, TU2, TV2, prog, err, (int)tune_get("bidiag2s.build_solo", 1)};
        int per_sm = 0;
        DDLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bd_chase, BD2_THREADS, 0));
        const i64 cyc = n - 1;
        const int grid = (int)std::max<i64>(1, std::min<i64>(cyc, (i64)h->sm_count * std::max(per_sm, 1)));
        void *args[] = {&ca};
        {
            Timed tm(s, TC_BD_CHASE, 0.0, 0.0);
            DDLA_CUDA(cudaLaunchCooperativeKernel((const void *)k_bd_chase, dim3(grid), dim3(BD2_THREADS), args, 0,
                                                  s));
            DDLA_LAUNCHED();
        }
        // every group of bs cycles reads and writes columns i0 + 1 .. n of U and V once
        Timed tm(s, TC_BD_BACK, 2.0 * n * n * (double)(m + n), 8.0 * n * n * (double)(m + n) / bs);
        const int ublocks = (int)((m + BK_RB - 1) / BK_RB), vblocks = (int)((n + BK_RB - 1) / BK_RB);
        for (i64 i0 = 0; i0 + 1 < n; i0 += bs) {
            const int G = (int)(n - 1 - i0 < bs ? n - 1 - i0 : bs), kcount = (int)((n - i0 - 2) / bs) + 1;
            k_bd_back_prep<<<dim3(kcount, 2), 32, 0, s>>>(TU2, TV2, n, (int)bs, i0, G, kcount, Zq);
            DDLA_LAUNCHED();
            k_bd_back<<<ublocks + vblocks, 32, 0, s>>>(U.p, m, U.rs, U.cs, V.p, V.rs, V.cs, TU2, TV2, Zq, n, (int)bs,
                                                      i0, ublocks);
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
