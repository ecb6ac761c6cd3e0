// Triangular solves (BLIS trsm semantics) built on inverted diagonal blocks.
//
// The problem is normalised to a left solve tri(A) X = alpha B with a
// non-transposed view (a right solve X op(A) = B is op(A)^T X^T = B^T; a
// transposed triangle is the other triangle of the transposed view).  The
// triangle is split into TB x TB diagonal blocks whose inverses are formed
// once (k_tri_inv, one CTA per block).  Then:
//   * few right-hand sides (<= 16): ONE kernel (k_trsv_chain) solves the whole
//     system.  Each CTA owns a block row; it takes its block in ticket order
//     (so every block it waits for is already running or done), subtracts
//     L_ij x_j as each x_j is published (flag per block, bounded spin), then
//     multiplies by inv(L_ii) and publishes x_i.  The off-diagonal tiles are
//     loaded before the wait, so HBM latency overlaps the dependency chain.
//   * many right-hand sides: per diagonal block X1 = inv(A11) B1 and the GEMM
//     update B2 -= A21 X1 (DDLA's managed TrSM has the same block structure
//     with a TRSV per column, DDLA/BLAS/Managed/3m/TrSM.cs:62-122).
#include <cooperative_groups.h>

#include <mutex>
#include <string>

#include "common.cuh"
#include "timing.cuh"

namespace ddla {
namespace {

constexpr int TB = TRI_TB;
constexpr int CHAIN_THREADS = 256;
constexpr long long SPIN_LIMIT = 1LL << 24;

template <typename T>
__global__ void k_scale(T alpha, T *B, i64 m, i64 n, i64 rs, i64 cs) {
    i64 tot = m * n;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        i64 i = e / n, j = e % n;
        T *p = B + i * rs + j * cs;
        *p = (alpha == T(0)) ? T(0) : *p * alpha;
    }
}

template <typename T>
__global__ void k_copy2d(const T *X, i64 rs, i64 cs, i64 m, i64 n, T *Y, i64 yrs, i64 ycs) {
    i64 tot = m * n;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        i64 i = e / n, j = e % n;
        Y[i * yrs + j * ycs] = X[i * rs + j * cs];
    }
}

// Inverse of each TB x TB diagonal block of tri(A) (lower/upper, unit or not),
// stored row-major per block, zero outside the triangle.  One thread per
// column of the identity; forward (lower) or backward (upper) substitution.
// Column c of the inverse by column-oriented substitution: one warp per
// column, lanes own rows lane and lane + 32; the finished entry y_k is
// broadcast with a shuffle and the lanes below (above, for upper) subtract
// its column of L.  16 warps, so the 64 columns take 4 passes.
constexpr int TI_THREADS = 512;

template <typename T>
__global__ void __launch_bounds__(TI_THREADS) k_tri_inv(const T *A, i64 rs, i64 cs, i64 n, int lower, int unit, T *inv) {
    __shared__ T L[TB][TB + 1];
    __shared__ T dinv[TB];
    const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const i64 r0 = (i64)b * TB;
    const int bs = (int)(n - r0 < TB ? n - r0 : TB);
    for (int e = tid; e < TB * TB; e += TI_THREADS) {
        const int i = e / TB, c = e % TB;
        L[i][c] = (i < bs && c < bs) ? A[(r0 + i) * rs + (r0 + c) * cs] : T(0);
    }
    __syncthreads();
    if (tid < TB) dinv[tid] = (tid < bs && !unit) ? T(1) / L[tid][tid] : T(1);
    __syncthreads();
    T *out = inv + (i64)b * TB * TB;
    for (int c = warp; c < TB; c += TI_THREADS / 32) {
        T y0 = (lane == c) ? T(1) : T(0), y1 = (lane + 32 == c) ? T(1) : T(0);
        if (c < bs) {
            if (lower) {
                for (int k = c; k < bs; k++) {
                    const T yk = __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, k & 31) * dinv[k];
                    if (lane == k) y0 = yk;
                    if (lane + 32 == k) y1 = yk;
                    if (lane > k && lane < bs) y0 -= L[lane][k] * yk;
                    if (lane + 32 > k && lane + 32 < bs) y1 -= L[lane + 32][k] * yk;
                }
            } else {
                for (int k = c; k >= 0; k--) {
                    const T yk = __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, k & 31) * dinv[k];
                    if (lane == k) y0 = yk;
                    if (lane + 32 == k) y1 = yk;
                    if (lane < k) y0 -= L[lane][k] * yk;
                    if (lane + 32 < k) y1 -= L[lane + 32][k] * yk;
                }
            }
        } else {
            y0 = y1 = T(0);
        }
        out[lane * TB + c] = lane < bs ? y0 : T(0);
        out[(lane + 32) * TB + c] = lane + 32 < bs ? y1 : T(0);
    }
}

__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Whole-system solve with <= NR right-hand sides, X row-major n x ldx.
// Thread t works on block row r = t/4, k-quarter q = t%4 (16 columns of the
// tile), reduces its partial dot products over the 4 threads of the row.
// G groups of 256 threads split the right-hand sides (NR / G each), so the
// tile products on the chain's critical path are shorter for 16 of them.
template <typename T, int NR, int G>
__global__ void __launch_bounds__(CHAIN_THREADS *G)
    k_trsv_chain(i64 n, int nblk, const T *__restrict__ A, i64 rs, i64 cs, int lower, const T *__restrict__ inv,
                 T *X, i64 ldx, int nr, int *flags, int *ticket, int *err) {
    constexpr int NC = NR / G;
    constexpr int NT = CHAIN_THREADS * G;
    __shared__ T s_acc[TB][NR];
    __shared__ T s_x[TB][NR];
    __shared__ int s_blk, s_abort;
    const int t = threadIdx.x, g = t / CHAIN_THREADS, tt = t % CHAIN_THREADS, r = tt >> 2, q = tt & 3;
    const int cb = g * NC;
    if (t == 0) {
        s_blk = atomicAdd(ticket, 1);
        s_abort = 0;
    }
    __syncthreads();
    const int logical = s_blk;
    const int blk = lower ? logical : nblk - 1 - logical;
    const i64 r0 = (i64)blk * TB;
    const int rows = (int)(n - r0 < TB ? n - r0 : TB);
    for (int e = t; e < TB * NR; e += NT) {
        int i = e / NR, c = e % NR;
        s_acc[i][c] = (i < rows && c < nr) ? X[(r0 + i) * ldx + c] : T(0);
    }
    __syncthreads();
    for (int d = 0; d < logical; d++) {
        const int j = lower ? d : nblk - 1 - d;
        const i64 c0 = (i64)j * TB;
        const int cols = (int)(n - c0 < TB ? n - c0 : TB);
        // tile row r, columns q*16 .. q*16+15 (loaded before waiting)
        T a[16];
#pragma unroll
        for (int k = 0; k < 16; k++) {
            int cc = q * 16 + k;
            a[k] = (r < rows && cc < cols) ? A[(r0 + r) * rs + (c0 + cc) * cs] : T(0);
        }
        if (t == 0) {
            long long it = 0;
            while (ld_acquire(flags + j) == 0) {
                if (++it > SPIN_LIMIT) {
                    atomicExch(err, 1);
                    s_abort = 1;
                    break;
                }
                __nanosleep(64);
            }
        }
        __syncthreads();
        if (s_abort) return;
        for (int e = t; e < TB * NR; e += NT) {
            int i = e / NR, c = e % NR;
            s_x[i][c] = (i < cols && c < nr) ? __ldcg(&X[(c0 + i) * ldx + c]) : T(0);
        }
        __syncthreads();
        T p[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) p[c] = T(0);
#pragma unroll
        for (int k = 0; k < 16; k++)
#pragma unroll
            for (int c = 0; c < NC; c++) p[c] += a[k] * s_x[q * 16 + k][cb + c];
#pragma unroll
        for (int c = 0; c < NC; c++) {
            p[c] += __shfl_xor_sync(0xffffffffu, p[c], 1);
            p[c] += __shfl_xor_sync(0xffffffffu, p[c], 2);
        }
        if (q == 0)
#pragma unroll
            for (int c = 0; c < NC; c++) s_acc[r][cb + c] -= p[c];
        __syncthreads();
    }
    // x_blk = inv(A_blk,blk) * acc
    {
        const T *iv = inv + (i64)blk * TB * TB;
        T a[16];
#pragma unroll
        for (int k = 0; k < 16; k++) a[k] = iv[r * TB + q * 16 + k];
        T p[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) p[c] = T(0);
#pragma unroll
        for (int k = 0; k < 16; k++)
#pragma unroll
            for (int c = 0; c < NC; c++) p[c] += a[k] * s_acc[q * 16 + k][cb + c];
#pragma unroll
        for (int c = 0; c < NC; c++) {
            p[c] += __shfl_xor_sync(0xffffffffu, p[c], 1);
            p[c] += __shfl_xor_sync(0xffffffffu, p[c], 2);
        }
        if (q == 0 && r < rows)
            for (int c = 0; c < NC; c++)
                if (cb + c < nr) X[(r0 + r) * ldx + cb + c] = p[c];
    }
    __syncthreads();
    if (t == 0) {
        __threadfence();
        st_release(flags + blk, 1);
    }
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
int copy2d(cudaStream_t s, View<const T> X, View<T> Y);

}  // namespace

template <typename T>
int copy2d_on(cudaStream_t s, View<const T> X, View<T> Y) {
    return copy2d<T>(s, X, Y);
}
template int copy2d_on<double>(cudaStream_t, View<const double>, View<double>);
template int copy2d_on<float>(cudaStream_t, View<const float>, View<float>);

namespace {

template <typename T>
int copy2d(cudaStream_t s, View<const T> X, View<T> Y) {
    i64 tot = X.rows * X.cols;
    if (tot == 0) return 0;
    int blocks = (int)((tot + 255) / 256 < 8192 ? (tot + 255) / 256 : 8192);
    k_copy2d<T><<<blocks, 256, 0, s>>>(X.p, X.rs, X.cs, X.rows, X.cols, Y.p, Y.rs, Y.cs);
    DDLA_LAUNCHED();
    return 0;
}

// ------------------------------------------------------------------ cluster solve
//
// Whole-system solve with <= NR right-hand sides on ONE thread-block cluster
// (up to 16 CTAs).  Logical block l (block row l of a lower triangle, block
// row nblk-1-l of an upper one) belongs to CTA l % CS.  Every CTA keeps a copy
// of the whole solution x (n x NR) in its shared memory, filled with a marker
// value that no arithmetic produces.  A CTA solves its blocks in increasing l,
// left-looking:
//   acc = b_l;  for j < l: acc -= A_lj x_j  (waiting, bounded, until this
//   lane's entries of x_j no longer hold the marker);  x_l = inv(A_ll) acc
// and then stores x_l into every CTA's copy over DSMEM: the values mark
// themselves, so the chain needs no flags and no fences.
// Each warp owns 8 rows of the block: it streams its own rows of the tiles
// A_lj and of the inverted diagonal block through its own ring of
// shared-memory stages (cp.async, STAGES-1 items ahead, in consumption
// order) and updates its own rows of acc, so the tile loop needs no CTA-wide
// barrier; the CTA synchronises only around the inverse, once per block.
constexpr int CL_THREADS = 256;
constexpr int CL_WARPS = CL_THREADS / 32;
constexpr int CL_WROWS = TB / CL_WARPS;   // rows of a tile per warp
constexpr int CL_MAXCS = 16;
constexpr int CL_TLD = TB + 4;           // padded tile row (16-byte multiple for float and double)
constexpr long long CL_SPIN = 1LL << 22;

template <typename T> struct ClStages { static constexpr int value = sizeof(T) == 4 ? 8 : 4; };

struct ClLayout {
    size_t ring, xall, acc, total;
};

template <typename T, int NR>
__host__ __device__ inline ClLayout cl_layout(int nblk) {
    ClLayout L;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = (o + bytes + 127) & ~(size_t)127;
        return at;
    };
    L.ring = take(sizeof(T) * (size_t)ClStages<T>::value * TB * CL_TLD);
    L.xall = take(sizeof(T) * (size_t)nblk * TB * NR);
    L.acc = take(sizeof(T) * TB * NR);
    L.total = o;
    return L;
}

// "Not yet written" marker of the x copies: a signaling-NaN bit pattern, which
// no arithmetic result can have (results that are NaN are quiet NaNs), so each
// value announces its own arrival and needs no flag or fence.
__device__ __forceinline__ bool cl_pending(float v) { return __float_as_uint(v) == 0x7FBADBADu; }
__device__ __forceinline__ bool cl_pending(double v) {
    return (unsigned long long)__double_as_longlong(v) == 0x7FF4DEADBEEFBADDull;
}
template <typename T> __device__ __forceinline__ T cl_marker();
template <> __device__ __forceinline__ float cl_marker<float>() { return __uint_as_float(0x7FBADBADu); }
template <> __device__ __forceinline__ double cl_marker<double>() {
    return __longlong_as_double((long long)0x7FF4DEADBEEFBADDull);
}
__device__ __forceinline__ float ld_volatile(const float *p) { return *(const volatile float *)p; }
__device__ __forceinline__ double ld_volatile(const double *p) { return *(const volatile double *)p; }

__device__ __forceinline__ void cp_async16(void *dst, const void *src, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(src_bytes)
                 : "memory");
}
template <int BYTES>
__device__ __forceinline__ void cp_async_small(void *dst, const void *src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src), "n"(BYTES), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Whole-system solve with 9-16 right-hand sides (the mixed Cholesky's
// correction solves).  Same chain as k_trsv_chain (ticket order, one CTA per
// block row, a flag per published block), but thread t owns row t / 16 and
// right-hand side t % 16 of its block, so a tile product needs no reduction.
// The off-diagonal tiles do not depend on the chain: they stream through
// CH16_STAGES shared-memory stages (cp.async) ahead of the flag waits, and the
// block's inverse is prefetched with them.  x_j is read once per tile into one
// of two buffers, so a tile costs two barriers.  Needs 16-byte rows (cs == 1)
// or columns (rs == 1) and n a multiple of the 16-byte vector.
constexpr int CH16_STAGES = 3;
constexpr int CH16_THREADS = TB * 16;
template <typename T>
constexpr size_t ch16_smem() {
    return sizeof(T) * ((size_t)(CH16_STAGES + 1) * TB * TB + 3 * TB * 16);
}

template <typename T>
__global__ void __launch_bounds__(CH16_THREADS)
    k_trsv_chain16(i64 n, int nblk, const T *__restrict__ A, i64 rs, i64 cs, int lower, int trans,
                   const T *__restrict__ inv, T *X, i64 ldx, int nr, int *flags, int *ticket, int *err) {
    extern __shared__ __align__(16) unsigned char ch_smem[];
    T *sA = reinterpret_cast<T *>(ch_smem);            // [CH16_STAGES][TB * TB]
    T *sInv = sA + (size_t)CH16_STAGES * TB * TB;       // [TB][TB]
    T *sx = sInv + TB * TB;                             // [2][TB][16]
    T *sacc = sx + 2 * TB * 16;                         // [TB][16]
    __shared__ int s_blk, s_abort;
    const int t = threadIdx.x, r = t >> 4, c = t & 15;
    if (t == 0) {
        s_blk = atomicAdd(ticket, 1);
        s_abort = 0;
    }
    __syncthreads();
    const int logical = s_blk;
    const int blk = lower ? logical : nblk - 1 - logical;
    const i64 r0 = (i64)blk * TB;
    const int rows = (int)(n - r0 < TB ? n - r0 : TB);
    constexpr int VEC = 16 / (int)sizeof(T);   // elements per 16-byte copy
    constexpr int NV = TB * TB / VEC;          // copies per tile
    // tile d (the d-th block before the diagonal in solve order) into stage
    // st: stored [i][k] (trans = 0, rows contiguous) or [k][i] (trans = 1)
    auto issue = [&](int d, int st) {
        const int j = lower ? d : nblk - 1 - d;
        const i64 c0 = (i64)j * TB;
        T *dst = sA + (size_t)st * TB * TB;
        for (int v = t; v < NV; v += CH16_THREADS) {
            const int a = v / (TB / VEC), b = (v % (TB / VEC)) * VEC;
            const i64 gi = trans ? r0 + b : r0 + a, gk = trans ? c0 + a : c0 + b;
            const bool in = gi < n && gk < n;
            cp_async16(dst + a * TB + b, in ? A + gi * rs + gk * cs : A, in ? 16 : 0);
        }
    };
    {
        const T *iv = inv + (i64)blk * TB * TB;
        for (int v = t; v < NV; v += CH16_THREADS) cp_async16(sInv + v * VEC, iv + v * VEC, 16);
    }
    cp_async_commit();
    for (int p = 0; p < CH16_STAGES - 1; p++) {
        if (p < logical) issue(p, p);
        cp_async_commit();
    }
    T acc = (r < rows && c < nr) ? X[(r0 + r) * ldx + c] : T(0);
    for (int d = 0; d < logical; d++) {
        const int j = lower ? d : nblk - 1 - d;
        const i64 c0 = (i64)j * TB;
        const int cols = (int)(n - c0 < TB ? n - c0 : TB);
        if (t == 0) {
            long long it = 0;
            while (ld_acquire(flags + j) == 0) {
                if (++it > SPIN_LIMIT) {
                    atomicExch(err, 1);
                    s_abort = 1;
                    break;
                }
                __nanosleep(64);
            }
        }
        // groups so far: inverse, tiles 0 .. d + CH16_STAGES - 2; tile d is
        // complete when at most CH16_STAGES - 2 groups are pending
        cp_async_wait<CH16_STAGES - 2>();
        __syncthreads();
        if (s_abort) break;
        // every thread is past tile d - 1: its stage takes tile d + CH16_STAGES - 1
        if (d + CH16_STAGES - 1 < logical) issue(d + CH16_STAGES - 1, (d + CH16_STAGES - 1) % CH16_STAGES);
        cp_async_commit();
        T *xb = sx + (d & 1) * TB * 16;
        xb[r * 16 + c] = (r < cols && c < nr) ? __ldcg(&X[(c0 + r) * ldx + c]) : T(0);
        __syncthreads();
        const T *tile = sA + (size_t)(d % CH16_STAGES) * TB * TB;
        if (!trans) {
            const T *arow = tile + r * TB;
#pragma unroll 16
            for (int k = 0; k < TB; k++) acc -= arow[k] * xb[k * 16 + c];
        } else {
#pragma unroll 16
            for (int k = 0; k < TB; k++) acc -= tile[k * TB + r] * xb[k * 16 + c];
        }
    }
    cp_async_wait<0>();
    if (s_abort) return;
    // x_blk = inv(A_blk,blk) * acc
    sacc[r * 16 + c] = acc;
    __syncthreads();
    T v = T(0);
    const T *irow = sInv + r * TB;
#pragma unroll 16
    for (int k = 0; k < TB; k++) v += irow[k] * sacc[k * 16 + c];
    if (r < rows && c < nr) X[(r0 + r) * ldx + c] = v;
    __syncthreads();
    if (t == 0) {
        __threadfence();
        st_release(flags + blk, 1);
    }
}

// Split mode (a grid of several clusters, W > 0).  The first cluster to start
// runs the chain above over the NEAR tiles of each block row only: for l > W,
// the W tiles A_lj with l - W <= j < l.  The other CTAs are helpers: each
// takes block rows l > W in increasing order (a counter) and forms the far
// sum F_l = sum_{j < l - W} A_lj x_j as the chain publishes each x_j (x_j in
// X, then a flag per block), streaming the tiles ahead of the flags.  The
// chain subtracts F_l from block l's right-hand side at its near tile
// j = l - PW, by when the helper has normally released it.  A row that no
// helper has taken when the chain reaches it is claimed by the chain and
// summed there, so no wait depends on a CTA that has not started: the roles
// and the rows are taken with atomics by whichever CTAs run first.  One
// right-hand side.
template <typename T>
struct SplitArgs {
    int *xflag;   // [nblk] logical block j's x is in X
    int *rowst;   // [nblk] 0 free, 1 chain-owned, 2 helper-owned, 3 far sum in part
    int *next;    // helpers' row counter
    int *role;    // id + 1 of the chain cluster
    T *part;      // [nblk][TB] far sums
    int W, PW;    // near tiles per block row (0: one cluster, no split); where F_l is added
};

// Helper shared memory: per warp, ClStages stages of its 8 tile rows and x_j.
template <typename T> __host__ __device__ constexpr int sp_stage() { return CL_WROWS * CL_TLD + TB; }
template <typename T> __host__ __device__ constexpr size_t sp_smem() {
    return sizeof(T) * (size_t)CL_WARPS * ClStages<T>::value * sp_stage<T>();
}

// Wait until at most k of this thread's cp.async groups are pending (k <= 7).
__device__ __forceinline__ void cp_async_wait_n(int k) {
    switch (k) {
        case 0: cp_async_wait<0>(); break;
        case 1: cp_async_wait<1>(); break;
        case 2: cp_async_wait<2>(); break;
        case 3: cp_async_wait<3>(); break;
        case 4: cp_async_wait<4>(); break;
        case 5: cp_async_wait<5>(); break;
        case 6: cp_async_wait<6>(); break;
        default: cp_async_wait<7>(); break;
    }
}

// A helper CTA: far sums of the block rows it takes.  Each warp owns 8 rows of
// the block row and streams its rows of the tiles A_lj (they do not depend on
// the chain) up to S - 1 ahead; x_j is read once its flag is seen, for every
// tile whose x has been published since the last look, so a helper that is
// level with the chain pays one flag round trip per batch, not per tile.
template <typename T>
__device__ void split_helper(i64 n, int nblk, const T *__restrict__ A, i64 rs, i64 cs, int lower, int vec,
                             const T *X, i64 ldx, int xvec, const SplitArgs<T> &sp, int *err, T *ring, int &s_row,
                             int &s_abort) {
    constexpr int S = ClStages<T>::value;
    constexpr int HS = sp_stage<T>();
    constexpr int CPR = TB * (int)sizeof(T) / 16, EPC = 16 / (int)sizeof(T);
    constexpr int CPL = CL_WROWS * CPR / 32;   // 16-byte chunks per lane of a warp's tile rows
    constexpr int XCH = TB / EPC;              // 16-byte chunks of x_j (<= 32)
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5, rr = lane >> 2, q = lane & 3;
    T *wring = ring + (size_t)warp * S * HS;
    auto phys = [&](int l) { return lower ? l : nblk - 1 - l; };
    int c_row[CPL], c_col[CPL];
#pragma unroll
    for (int i = 0; i < CPL; i++) {
        const int e = lane + 32 * i;
        c_row[i] = e / CPR;
        c_col[i] = (e % CPR) * EPC;
    }
    int ready = 0;   // x_0 .. x_{ready-1} are known to be published (warp-uniform)
    for (;;) {
        if (t == 0) {
            const int row = atomicAdd(sp.next, 1) + sp.W + 1;
            s_row = row >= nblk ? -2 : (atomicCAS(sp.rowst + row, 0, 2) == 0 ? row : -1);
        }
        __syncthreads();
        const int row = s_row;
        const bool quit = s_abort != 0;
        __syncthreads();   // s_row and s_abort are read before thread 0 writes them again
        if (row == -2 || quit) break;
        if (row < 0) continue;
        const int J = row - sp.W;   // far tiles j = 0 .. J - 1
        const i64 g0 = (i64)phys(row) * TB + warp * CL_WROWS;   // first row of this warp
        int produced = 0;
        auto issue = [&](int j) {
            T *dst = wring + (size_t)(j % S) * HS;
            const i64 c0 = (i64)phys(j) * TB;
            if (vec) {
#pragma unroll
                for (int i = 0; i < CPL; i++) {
                    const i64 gr = g0 + c_row[i], gc = c0 + c_col[i];
                    int bytes = 0;
                    const T *src = A;
                    if (gr < n && gc < n) {
                        const i64 left = n - gc;
                        bytes = (int)(left >= EPC ? 16 : left * (i64)sizeof(T));
                        src = A + gr * rs + gc;
                    }
                    cp_async16(dst + c_row[i] * CL_TLD + c_col[i], src, bytes);
                }
            } else {
                for (int e = lane; e < CL_WROWS * TB; e += 32) {
                    const int row_ = e / TB, col = e % TB;
                    const i64 gr = g0 + row_, gc = c0 + col;
                    const bool in = gr < n && gc < n;
                    cp_async_small<sizeof(T)>(dst + row_ * CL_TLD + col, in ? A + gr * rs + gc * cs : A,
                                              in ? (int)sizeof(T) : 0);
                }
            }
            cp_async_commit();
        };
        auto top_up = [&](int lim) {
            while (produced < lim) issue(produced++);
        };
        T f = T(0);
        bool bad = false;
        int j = 0;
        top_up(J < S ? J : S);
        while (j < J) {
            if (ready <= j) {
                long long it = 0;
                for (;;) {
                    const int idx = ready + lane;
                    const int v = idx < J ? ld_acquire(sp.xflag + idx) : 0;
                    const unsigned b = __ballot_sync(0xffffffffu, v != 0);
                    ready += b == 0xffffffffu ? 32 : __ffs(~b) - 1;
                    if (ready > j) break;
                    const bool stop = ++it > CL_SPIN || *(volatile int *)err != 0;
                    if (__any_sync(0xffffffffu, stop)) {
                        bad = true;
                        break;
                    }
                    if (it > 16) __nanosleep(64);
                }
                if (bad) break;
            }
            // the lanes' flag loads above come before every lane's reads of x
            __syncwarp();
            const int jend = (ready < J ? ready : J) < j + S ? (ready < J ? ready : J) : j + S;
            top_up(J < j + S ? J : j + S);
            for (int b = j; b < jend; b++) {
                T *xs = wring + (size_t)(b % S) * HS + CL_WROWS * CL_TLD;
                const i64 c0 = (i64)phys(b) * TB;
                if (xvec) {
                    if (lane < XCH) {
                        const i64 gc = c0 + lane * EPC;
                        if (gc + EPC <= n) {
                            *(uint4 *)(xs + lane * EPC) = __ldcg((const uint4 *)(X + gc));
                        } else {
#pragma unroll
                            for (int e = 0; e < EPC; e++) xs[lane * EPC + e] = gc + e < n ? __ldcg(X + gc + e) : T(0);
                        }
                    }
                } else {
                    for (int e = lane; e < TB; e += 32) xs[e] = c0 + e < n ? __ldcg(X + (c0 + e) * ldx) : T(0);
                }
            }
            cp_async_wait_n(produced - jend);   // the tiles of j .. jend - 1 have landed
            __syncwarp();
            for (int b = j; b < jend; b++) {
                const T *st = wring + (size_t)(b % S) * HS;
                const T *xs = st + CL_WROWS * CL_TLD;
#pragma unroll
                for (int i = 0; i < TB / 4; i++) f += st[rr * CL_TLD + q + 4 * i] * xs[q + 4 * i];
            }
            __syncwarp();   // stages j .. jend - 1 are free again
            j = jend;
            top_up(J < j + S ? J : j + S);
        }
        f += __shfl_xor_sync(0xffffffffu, f, 1);
        f += __shfl_xor_sync(0xffffffffu, f, 2);
        if (bad) {
            if (lane == 0) {
                atomicExch(err, 1);
                s_abort = 1;
            }
        } else if (q == 0) {
            sp.part[(size_t)row * TB + warp * CL_WROWS + rr] = f;
        }
        cp_async_wait<0>();
        __syncthreads();   // every warp's far sums are stored
        if (t == 0 && !s_abort) {
            __threadfence();
            st_release(sp.rowst + row, 3);
        }
    }
    cp_async_wait<0>();
}

template <typename T, int NR>
__global__ void __launch_bounds__(CL_THREADS)
    k_trsv_cluster(i64 n, int nblk, const T *__restrict__ A, i64 rs, i64 cs, int lower, int vec,
                   const T *__restrict__ inv, const T *__restrict__ mlast, T *X, i64 ldx, int nr, int *err,
                   SplitArgs<T> sp, int xvec) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    constexpr int S = ClStages<T>::value;
    const int CS = (int)cluster.num_blocks(), rank = (int)cluster.block_rank();
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5, r = t >> 2, q = t & 3;
    extern __shared__ __align__(128) unsigned char smem[];
    const ClLayout Ly = cl_layout<T, NR>(nblk);
    T *ring = (T *)(smem + Ly.ring);
    T *xall = (T *)(smem + Ly.xall);
    T *acc = (T *)(smem + Ly.acc);
    __shared__ int s_abort, s_role, s_own, s_row;
    const int W = sp.W;
    const bool fused = mlast != nullptr;
    const int cid = (int)(blockIdx.x / (unsigned)CS) + 1;
    auto phys = [&](int l) { return lower ? l : nblk - 1 - l; };
    // first tile of block row l that this chain streams
    auto jlo = [&](int l) { return W > 0 && l > W ? l - W : 0; };
    if (W > 0 && rank == 0 && t == 0) atomicCAS(sp.role, 0, cid);
    for (int e = t; e < nblk * TB * NR; e += CL_THREADS) xall[e] = cl_marker<T>();
    if (t == 0) s_abort = 0;
    cluster.sync();   // every CTA's copy holds markers before anyone writes x into it
    if (W > 0) {
        if (t == 0) s_role = ld_acquire(sp.role);
        __syncthreads();
        if (s_role != cid) {   // a helper cluster: no DSMEM from here on
            if constexpr (NR == 1)
                split_helper<T>(n, nblk, A, rs, cs, lower, vec, X, ldx, xvec, sp, err, ring, s_row, s_abort);
            return;
        }
    }
    // ring item (l, j): this warp's rows of tile A_lj (j < l) or of the
    // inverted diagonal block (j == l).  Each lane copies the same chunks
    // (row, 16-byte column chunk) of every item: their offsets are formed once.
    constexpr int CPR = TB * (int)sizeof(T) / 16, EPC = 16 / (int)sizeof(T);
    constexpr int CPL = CL_WROWS * CPR / 32;   // chunks per lane
    const int row0 = warp * CL_WROWS;
    int c_row[CPL], c_col[CPL];
    i64 c_goff[CPL];
#pragma unroll
    for (int i = 0; i < CPL; i++) {
        const int e = lane + 32 * i;
        c_row[i] = row0 + e / CPR;
        c_col[i] = (e % CPR) * EPC;
        c_goff[i] = (i64)c_row[i] * rs + c_col[i];
    }
    // item j of block row l: a tile (j below the last), the inverted diagonal
    // block, then (fused) M_l; contiguous TB x TB blocks are 16-byte aligned
    auto issue = [&](int l, int j, int stage) {
        T *dst = ring + (size_t)stage * TB * CL_TLD;
        const bool is_inv = fused && l > 0 ? j == l - 1 : j == l;
        if (is_inv || (fused && j == l)) {
            const T *src = (is_inv ? inv : mlast) + (i64)phys(l) * TB * TB;
#pragma unroll
            for (int i = 0; i < CPL; i++)
                cp_async16(dst + c_row[i] * CL_TLD + c_col[i], src + c_row[i] * TB + c_col[i], 16);
            return;
        }
        const i64 r0 = (i64)phys(l) * TB, c0 = (i64)phys(j) * TB;
        if (vec && r0 + TB <= n && c0 + TB <= n) {   // full tile
            const T *base = A + r0 * rs + c0;
#pragma unroll
            for (int i = 0; i < CPL; i++) cp_async16(dst + c_row[i] * CL_TLD + c_col[i], base + c_goff[i], 16);
        } else if (vec) {
#pragma unroll
            for (int i = 0; i < CPL; i++) {
                const i64 gr = r0 + c_row[i], gc = c0 + c_col[i];
                int bytes = 0;
                const T *src = A;
                if (gr < n && gc < n) {
                    const i64 left = n - gc;
                    bytes = (int)(left >= EPC ? 16 : left * (i64)sizeof(T));
                    src = A + gr * rs + gc;
                }
                cp_async16(dst + c_row[i] * CL_TLD + c_col[i], src, bytes);
            }
        } else {
            for (int e = lane; e < CL_WROWS * TB; e += 32) {
                const int row = row0 + e / TB, col = e % TB;
                const i64 gr = r0 + row, gc = c0 + col;
                const bool in = gr < n && gc < n;
                cp_async_small<sizeof(T)>(dst + row * CL_TLD + col, in ? A + gr * rs + gc * cs : A,
                                          in ? (int)sizeof(T) : 0);
            }
        }
    };
    // producer state: item (pl, pj) in consumption order
    int pl = rank, pj = jlo(rank);
    auto advance = [&]() {
        if (++pj > pl) {
            pl += CS;
            pj = jlo(pl);
        }
    };
    int produced = 0, consumed = 0;
    for (int i = 0; i < S - 1; i++) {
        if (pl < nblk) {
            issue(pl, pj, produced % S);
            advance();
        }
        produced++;
        cp_async_commit();
    }
    // this warp's row r of a tile times x (sum over the 4 lanes of the row)
    auto rowdot = [&](const T *tile, const T *xv, T *p) {
#pragma unroll
        for (int c = 0; c < NR; c++) p[c] = T(0);
#pragma unroll
        for (int i = 0; i < TB / 4; i++) {
            const int k = q + 4 * i;
            const T v = tile[r * CL_TLD + k];
#pragma unroll
            for (int c = 0; c < NR; c++) p[c] += v * xv[k * NR + c];
        }
#pragma unroll
        for (int c = 0; c < NR; c++) {
            p[c] += __shfl_xor_sync(0xffffffffu, p[c], 1);
            p[c] += __shfl_xor_sync(0xffffffffu, p[c], 2);
        }
    };
    auto next_item = [&]() {
        consumed++;
        if (pl < nblk) {
            issue(pl, pj, produced % S);
            advance();
        }
        produced++;
        cp_async_commit();
    };
    // this lane's entries of x_j (rows k = q + 4i) once none is the marker
    // (bounded; the decision to give up is warp-wide)
    auto wait_x = [&](int j, T (&xv)[TB / 4][NR]) -> bool {
        const T *xj = xall + (size_t)phys(j) * TB * NR;
        long long it = 0;
        for (;;) {
            bool pend = false;
#pragma unroll
            for (int i = 0; i < TB / 4; i++)
#pragma unroll
                for (int c = 0; c < NR; c++) {
                    xv[i][c] = ld_volatile(xj + (q + 4 * i) * NR + c);
                    pend |= cl_pending(xv[i][c]);
                }
            if (!__any_sync(0xffffffffu, pend)) return true;
            const bool stop = ++it > CL_SPIN || *(volatile int *)&s_abort;
            if (__any_sync(0xffffffffu, stop)) return false;
            if (it > 64) __nanosleep(20);
        }
    };
    for (int l = rank; l < nblk; l += CS) {
        const i64 r0 = (i64)phys(l) * TB;
        const bool helped = l > W && W > 0;
        bool own = false;
        if (helped) {
            if (t == 0) s_own = atomicCAS(sp.rowst + l, 0, 1) == 0;
            __syncthreads();
            own = s_own != 0;
        }
        if (q == 0)
#pragma unroll
            for (int c = 0; c < NR; c++) acc[r * NR + c] = (r0 + r < n && c < nr) ? X[(r0 + r) * ldx + c] : T(0);
        T p[NR], pr[NR];   // pr: far sum of row r, subtracted at the next acc update
#pragma unroll
        for (int c = 0; c < NR; c++) pr[c] = T(0);
        bool bad = false;
        if (helped && own) {   // no helper took this row: its far tiles, straight from A
            for (int j = 0; j < l - W; j++) {
                T xv[TB / 4][NR];
                if (!wait_x(j, xv)) {
                    bad = true;
                    break;
                }
                const i64 c0 = (i64)phys(j) * TB, gr = r0 + r;
#pragma unroll
                for (int i = 0; i < TB / 4; i++) {
                    const i64 gc = c0 + q + 4 * i;
                    const T v = gr < n && gc < n ? A[gr * rs + gc * cs] : T(0);
#pragma unroll
                    for (int c = 0; c < NR; c++) pr[c] += v * xv[i][c];
                }
            }
#pragma unroll
            for (int c = 0; c < NR; c++) {
                pr[c] += __shfl_xor_sync(0xffffffffu, pr[c], 1);
                pr[c] += __shfl_xor_sync(0xffffffffu, pr[c], 2);
            }
        }
        // tiles: all before the diagonal, or (fused) all but the last
        const int jend = fused && l > 0 ? l - 1 : l;
        for (int j = jlo(l); j < jend && !bad; j++) {
            cp_async_wait<S - 2>();
            T xv[TB / 4][NR];
            if (!wait_x(j, xv)) {
                bad = true;
                break;
            }
            __syncwarp();
            const T *tile = ring + (size_t)(consumed % S) * TB * CL_TLD;
#pragma unroll
            for (int c = 0; c < NR; c++) p[c] = T(0);
#pragma unroll
            for (int i = 0; i < TB / 4; i++) {
                const T v = tile[r * CL_TLD + q + 4 * i];
#pragma unroll
                for (int c = 0; c < NR; c++) p[c] += v * xv[i][c];
            }
#pragma unroll
            for (int c = 0; c < NR; c++) {
                p[c] += __shfl_xor_sync(0xffffffffu, p[c], 1);
                p[c] += __shfl_xor_sync(0xffffffffu, p[c], 2);
            }
            if (helped && !own && j == l - sp.PW) {
                // this warp's rows of F_l, once the helper has released them
                bool stop = false;
                if (lane == 0) {
                    long long it = 0;
                    while (ld_acquire(sp.rowst + l) != 3) {
                        if (++it > CL_SPIN || *(volatile int *)err != 0) {
                            stop = true;
                            break;
                        }
                        if (it > 16) __nanosleep(32);
                    }
                }
                if (__shfl_sync(0xffffffffu, stop, 0)) {
                    bad = true;
                    break;
                }
                __syncwarp();
                if (q == 0)
#pragma unroll
                    for (int c = 0; c < NR; c++) pr[c] += __ldcg(sp.part + ((size_t)l * TB + r) * NR + c);
            }
            next_item();
            if (q == 0)
#pragma unroll
                for (int c = 0; c < NR; c++) acc[r * NR + c] -= p[c] + pr[c];
#pragma unroll
            for (int c = 0; c < NR; c++) pr[c] = T(0);
        }
        if (bad && lane == 0) {
            atomicExch(err, 1);
            s_abort = 1;
        }
        __syncthreads();   // every row of acc is final (or some warp gave up)
        if (s_abort) break;
        cp_async_wait<S - 2>();
        __syncwarp();
        rowdot(ring + (size_t)(consumed % S) * TB * CL_TLD, acc, p);   // x_l = inv(A_ll) acc
        next_item();
        bool fail = false;
        if (fused && l > 0) {
            // x_l = inv(A_ll) acc - M_l x_{l-1}: each warp finishes its own rows
            // as soon as x_{l-1} is in, with no CTA barrier on the chain
            cp_async_wait<S - 2>();
            T xv[TB / 4][NR];
            if (!wait_x(l - 1, xv)) {
                fail = true;
                if (lane == 0) {
                    atomicExch(err, 1);
                    s_abort = 1;
                }
            } else {
                __syncwarp();
                const T *mt = ring + (size_t)(consumed % S) * TB * CL_TLD;
                T d[NR];
#pragma unroll
                for (int c = 0; c < NR; c++) d[c] = T(0);
#pragma unroll
                for (int i = 0; i < TB / 4; i++) {
                    const T v = mt[r * CL_TLD + q + 4 * i];
#pragma unroll
                    for (int c = 0; c < NR; c++) d[c] += v * xv[i][c];
                }
#pragma unroll
                for (int c = 0; c < NR; c++) {
                    d[c] += __shfl_xor_sync(0xffffffffu, d[c], 1);
                    d[c] += __shfl_xor_sync(0xffffffffu, d[c], 2);
                    p[c] -= d[c];
                }
            }
            next_item();
        }
        // publish x_l: the 4 lanes of row r each store it into a quarter of
        // the CTAs' copies (plain DSMEM stores; the values mark themselves)
        const int pb = phys(l);
        if (!fail) {
            for (int dst = q; dst < CS; dst += 4) {
                T *xd = cluster.map_shared_rank(xall, dst) + (size_t)pb * TB * NR + r * NR;
#pragma unroll
                for (int c = 0; c < NR; c++) xd[c] = p[c];
            }
            if (q == 0 && r0 + r < n)
                for (int c = 0; c < nr; c++) X[(r0 + r) * ldx + c] = p[c];
        }
        __syncthreads();   // acc is read above before the next block overwrites it
        if (s_abort) break;
        if (W > 0 && t == 0) {   // x_l is in X for the helpers
            __threadfence();
            st_release(sp.xflag + l, 1);
        }
    }
    cp_async_wait<0>();
    __syncthreads();
    cluster.sync();   // no CTA leaves while another may still write or read its shared memory
}

template <typename T, int NR>
struct ClusterCfg {
    static int cs;       // cluster size chosen (0 = not probed, -1 = unusable)
    static size_t avail;
};
template <typename T, int NR> int ClusterCfg<T, NR>::cs = 0;
template <typename T, int NR> size_t ClusterCfg<T, NR>::avail = 0;

// Cluster size for the cluster solve of nblk blocks (0 when it cannot run).
template <typename T, int NR>
int cluster_size(ddla_handle h, int nblk) {
    if (tune_get("trsv.cluster", 1) == 0) return 0;
    if (ClusterCfg<T, NR>::cs == 0) {
        ClusterCfg<T, NR>::cs = -1;
        if (cudaFuncSetAttribute(k_trsv_cluster<T, NR>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                cudaSuccess ||
            max_dyn_smem((const void *)k_trsv_cluster<T, NR>, h->smem_optin, &ClusterCfg<T, NR>::avail) != 0) {
            cudaGetLastError();
            return 0;
        }
        for (int c = CL_MAXCS; c >= 2; c /= 2) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(CL_THREADS);
            cfg.dynamicSmemBytes = cl_layout<T, NR>(1).total;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = c;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int nc = 0;
            if (cudaOccupancyMaxActiveClusters(&nc, (const void *)k_trsv_cluster<T, NR>, &cfg) == cudaSuccess &&
                nc > 0) {
                ClusterCfg<T, NR>::cs = c;
                break;
            }
            cudaGetLastError();
        }
    }
    int c = ClusterCfg<T, NR>::cs;
    if (c <= 0) return 0;
    const int want = (int)tune_get("trsv.cluster.size", 0);
    if (want >= 2 && want < c) c = want;
    if (cl_layout<T, NR>(nblk).total > ClusterCfg<T, NR>::avail) c = 0;
    return c;
}

// Clusters of cs CTAs with `smem` bytes each that fit on the GPU at once.
template <typename T, int NR>
int active_clusters(int cs, size_t smem) {
    static size_t last_smem = 0;
    static int last_cs = 0, last_nc = 0;
    if (smem == last_smem && cs == last_cs) return last_nc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, (const void *)k_trsv_cluster<T, NR>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        nc = 0;
    }
    last_smem = smem;
    last_cs = cs;
    last_nc = nc;
    return nc;
}

// One cluster, or (one right-hand side, a full cluster, far tiles to share)
// the split solve: the chain cluster plus helper clusters, as many as run at
// once and have block rows to take.  Tuning keys: trsv.split.w (near tiles
// per block row, 0 = no split), trsv.split.pw (where the chain adds a row's
// far sum), trsv.split.clusters (a cap on the clusters).
template <typename T, int NR>
int cluster_solve(ddla_handle h, int cs, i64 n, int nblk, View<const T> A, bool lower, const T *inv, const T *mlast,
                  T *X, i64 ldx, int nr) {
    const bool vec = A.cs == 1 && (A.rs * (i64)sizeof(T)) % 16 == 0 && (((uintptr_t)A.p) & 15) == 0;
    const int xvec = ldx == 1 && (((uintptr_t)X) & 15) == 0;
    size_t smem = cl_layout<T, NR>(nblk).total;
    SplitArgs<T> sp{};
    int G = 1;
    int W = NR == 1 && cs == CL_MAXCS ? (int)tune_get("trsv.split.w", 16) : 0;
    if (W < 2 || nblk <= W + 1) W = 0;
    if (W > 0) {
        const size_t need = smem > sp_smem<T>() ? smem : sp_smem<T>();
        const int rows = nblk - W - 1;   // block rows with far tiles
        const int nc = need <= ClusterCfg<T, NR>::avail ? active_clusters<T, NR>(cs, need) : 0;
        G = 1 + std::min(nc - 1, (rows + cs - 1) / cs);
        const int cap = (int)tune_get("trsv.split.clusters", 0);
        if (cap >= 1 && cap < G) G = cap;
        if (G >= 2) {
            int PW = (int)tune_get("trsv.split.pw", 6);
            const int pmin = mlast ? 2 : 1;   // fused: the last tile is not a tile step
            PW = PW < pmin ? pmin : (PW > W ? W : PW);
            const size_t ib = (sizeof(int) * (2 * (size_t)nblk + 2) + 15) & ~(size_t)15;
            char *w;
            DDLA_TRY(workspace(h, WS_TRSV, ib + sizeof(T) * (size_t)nblk * TB, (void **)&w));
            DDLA_CUDA(cudaMemsetAsync(w, 0, sizeof(int) * (2 * (size_t)nblk + 2), h->stream));
            int *ints = (int *)w;
            sp = SplitArgs<T>{ints, ints + nblk, ints + 2 * nblk, ints + 2 * nblk + 1, (T *)(w + ib), W, PW};
            smem = need;
        } else {
            G = 1;
        }
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs * G);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    DDLA_CUDA(cudaLaunchKernelEx(&cfg, k_trsv_cluster<T, NR>, n, nblk, A.p, A.rs, A.cs, lower ? 1 : 0, vec ? 1 : 0,
                                 inv, mlast, X, ldx, nr, h->d_info + INFO_TIMEOUT, sp, xvec));
    count_launch();
    return 0;
}

// The 16-wide chain applies when the tiles can move as 16-byte copies.
template <typename T>
bool chain16_fits(i64 n, View<const T> A, const T *inv) {
    constexpr i64 VEC = 16 / (i64)sizeof(T);
    const bool aligned = (((uintptr_t)A.p) & 15) == 0 && (((uintptr_t)inv) & 15) == 0 && n % VEC == 0;
    const bool rows = A.cs == 1 && (A.rs * (i64)sizeof(T)) % 16 == 0;
    const bool cols = A.rs == 1 && (A.cs * (i64)sizeof(T)) % 16 == 0;
    return aligned && (rows || cols) && tune_get("trsv.chain16", 1) != 0;
}

template <typename T>
int chain16(ddla_handle h, i64 n, int nblk, View<const T> A, bool lower, const T *inv, T *X, i64 ldx, int nr,
            int *flags) {
    static bool attr = false;
    if (!attr) {
        DDLA_CUDA(cudaFuncSetAttribute(k_trsv_chain16<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)ch16_smem<T>()));
        attr = true;
    }
    const int trans = A.cs == 1 ? 0 : 1;
    k_trsv_chain16<T><<<nblk, CH16_THREADS, ch16_smem<T>(), h->stream>>>(
        n, nblk, A.p, A.rs, A.cs, lower ? 1 : 0, trans, inv, X, ldx, nr, flags, flags + nblk,
        h->d_info + INFO_TIMEOUT);
    DDLA_LAUNCHED();
    return 0;
}

template <typename T, int NR>
int chain(ddla_handle h, i64 n, int nblk, View<const T> A, bool lower, const T *inv, T *X, i64 ldx, int nr,
          int *flags) {
    constexpr int G = NR >= 16 ? 4 : 1;
    k_trsv_chain<T, NR, G><<<nblk, CHAIN_THREADS * G, 0, h->stream>>>(n, nblk, A.p, A.rs, A.cs, lower ? 1 : 0, inv, X,
                                                                      ldx, nr, flags, flags + nblk,
                                                                      h->d_info + INFO_TIMEOUT);
    DDLA_LAUNCHED();
    return 0;
}

}  // namespace

template <typename T>
int gemm_any(ddla_handle h, int prec, i64 m, i64 n, i64 k, T alpha, View<const T> A, View<const T> B, T beta,
             View<T> C, int uplo);

// Inverses of the diagonal blocks of tri(A) (n x n) into inv (ceil(n/TB) *
// TB * TB elements).
template <typename T>
int tri_inverse_on(cudaStream_t s, bool lower, bool unit, View<const T> A, i64 n, T *inv) {
    int nblk = (int)((n + TB - 1) / TB);
    k_tri_inv<T><<<nblk, TI_THREADS, 0, s>>>(A.p, A.rs, A.cs, n, lower ? 1 : 0, unit ? 1 : 0, inv);
    DDLA_LAUNCHED();
    return 0;
}
template int tri_inverse_on<double>(cudaStream_t, bool, bool, View<const double>, i64, double *);
template int tri_inverse_on<float>(cudaStream_t, bool, bool, View<const float>, i64, float *);

template <typename T>
int tri_inverse(ddla_handle h, bool lower, bool unit, View<const T> A, i64 n, T *inv) {
    return tri_inverse_on<T>(h->stream, lower, unit, A, n, inv);
}

namespace {
// M_p = inv(A_pp) A_{p,p-1} (lower) or inv(A_pp) A_{p,p+1} (upper) for every
// block row p with that neighbour, TB x TB row-major at M + p TB^2: the last
// tile before a block's diagonal premultiplied by the block's inverse, so the
// cluster solve ends each block with one product once the previous block's x
// is in (x_l = inv(A_ll) acc - M_l x_{l-1}).  One CTA per block row; thread t
// forms row t / 4, columns t % 4 + 4 c.
template <typename T>
__global__ void __launch_bounds__(256) k_tri_mlast(const T *A, i64 rs, i64 cs, i64 n, int lower, const T *inv, T *M) {
    __shared__ T sA[TB][TB];
    const int p = lower ? blockIdx.x + 1 : blockIdx.x;
    const i64 r0 = (i64)p * TB, c0 = (i64)(lower ? p - 1 : p + 1) * TB;
    for (int e = threadIdx.x; e < TB * TB; e += 256) {
        const int i = e / TB, k = e % TB;
        const i64 gr = r0 + i, gc = c0 + k;
        sA[i][k] = gr < n && gc < n ? A[gr * rs + gc * cs] : T(0);
    }
    __syncthreads();
    const int i = threadIdx.x >> 2, k0 = threadIdx.x & 3;
    const T *iv = inv + (i64)p * TB * TB + (i64)i * TB;
    T out[TB / 4];
#pragma unroll
    for (int c = 0; c < TB / 4; c++) out[c] = T(0);
    for (int m = 0; m < TB; m++) {
        const T a = __ldg(iv + m);
#pragma unroll
        for (int c = 0; c < TB / 4; c++) out[c] += a * sA[m][k0 + 4 * c];
    }
    T *dst = M + (i64)p * TB * TB + (i64)i * TB;
#pragma unroll
    for (int c = 0; c < TB / 4; c++) dst[k0 + 4 * c] = out[c];
}
}  // namespace

template <typename T>
int tri_mlast(ddla_handle h, bool lower, View<const T> A, i64 n, const T *inv, T *M) {
    const int nblk = (int)((n + TB - 1) / TB);
    if (nblk < 2) return 0;
    k_tri_mlast<T><<<nblk - 1, 256, 0, h->stream>>>(A.p, A.rs, A.cs, n, lower ? 1 : 0, inv, M);
    DDLA_LAUNCHED();
    return 0;
}
template int tri_mlast<double>(ddla_handle, bool, View<const double>, i64, const double *, double *);
template int tri_mlast<float>(ddla_handle, bool, View<const float>, i64, const float *, float *);

// Solve tri(A) X = X in place for X row-major (n x nr, leading dim ldx),
// nr <= 16, with the precomputed diagonal-block inverses (and, for one
// right-hand side, the products tri_mlast forms: made here when not given;
// tuning key trsv.fused = 0 solves without them).
template <typename T>
int trsv_apply(ddla_handle h, bool lower, View<const T> A, i64 n, const T *inv, T *X, i64 ldx, int nr,
               const T *mlast) {
    int nblk = (int)((n + TB - 1) / TB);
    if (nr <= 1) {
        // FP64 on 16 SMs is bounded by their FP64 units: past ~96 blocks the
        // chained solve over one CTA per block is faster
        const int cs = (sizeof(T) == 8 && nblk > 96) ? 0 : cluster_size<T, 1>(h, nblk);
        if (cs > 1 && nblk > 1) {
            if (tune_get("trsv.fused", 1) == 0) {
                mlast = nullptr;
            } else if (!mlast) {
                T *m;
                DDLA_TRY(workspace(h, WS_TRSVM, sizeof(T) * (size_t)nblk * TB * TB, (void **)&m));
                DDLA_TRY(tri_mlast<T>(h, lower, A, n, inv, m));
                mlast = m;
            }
            return cluster_solve<T, 1>(h, cs, n, nblk, A, lower, inv, mlast, X, ldx, nr);
        }
    }
    int *flags;
    DDLA_TRY(workspace(h, WS_MISC, sizeof(int) * (size_t)(nblk + 1), (void **)&flags));
    DDLA_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)(nblk + 1), h->stream));
    if (nr <= 1) return chain<T, 1>(h, n, nblk, A, lower, inv, X, ldx, nr, flags);
    if (nr <= 2) return chain<T, 2>(h, n, nblk, A, lower, inv, X, ldx, nr, flags);
    if (nr <= 4) return chain<T, 4>(h, n, nblk, A, lower, inv, X, ldx, nr, flags);
    if (nr <= 8) return chain<T, 8>(h, n, nblk, A, lower, inv, X, ldx, nr, flags);
    if (nr <= 16) {
        if (chain16_fits<T>(n, A, inv)) return chain16<T>(h, n, nblk, A, lower, inv, X, ldx, nr, flags);
        return chain<T, 16>(h, n, nblk, A, lower, inv, X, ldx, nr, flags);
    }
    set_error("trsv_apply: more than 16 right-hand sides");
    return DDLA_ERR_UNSUPPORTED;
}

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
    const bool lower = (uplo == DDLA_LOWER), unit = (diag == DDLA_UNIT_DIAG);
    const int prec = sizeof(T) == 8 ? DDLA_PREC_FP64 : DDLA_PREC_FP32;
    const int nblk = (int)((m + TB - 1) / TB);
    T *inv, *tmp;
    DDLA_TRY(workspace(h, WS_TRI, sizeof(T) * (size_t)nblk * TB * TB, (void **)&inv));
    DDLA_TRY(tri_inverse<T>(h, lower, unit, A, m, inv));
    if (n <= 16) {
        // few right-hand sides: one chained kernel over a contiguous copy
        DDLA_TRY(workspace(h, WS_TMP, sizeof(T) * (size_t)m * n, (void **)&tmp));
        View<T> X{tmp, m, n, n, 1};
        DDLA_TRY(copy2d<T>(s, View<const T>{B.p, m, n, B.rs, B.cs}, X));
        DDLA_TRY(trsv_apply<T>(h, lower, A, m, inv, tmp, n, (int)n));
        return copy2d<T>(s, View<const T>{tmp, m, n, n, 1}, B);
    }
    DDLA_TRY(workspace(h, WS_TMP, sizeof(T) * (size_t)TB * n, (void **)&tmp));
    View<T> Tm{tmp, TB, n, n, 1};
    for (int bi = 0; bi < nblk; bi++) {
        const int b = lower ? bi : nblk - 1 - bi;
        const i64 i0 = (i64)b * TB;
        const int bs = (int)(m - i0 < TB ? m - i0 : TB);
        View<T> B1 = B.sub(i0, bs, 0, n);
        View<T> T1 = Tm.sub(0, bs, 0, n);
        DDLA_TRY(copy2d<T>(s, View<const T>{B1.p, bs, n, B1.rs, B1.cs}, T1));
        View<const T> IV{inv + (i64)b * TB * TB, bs, bs, TB, 1};
        DDLA_TRY(gemm_any<T>(h, prec, bs, n, bs, T(1), IV, View<const T>{tmp, bs, n, n, 1}, T(0), B1, DDLA_DENSE));
        View<const T> X1{B1.p, bs, n, B1.rs, B1.cs};
        if (lower) {
            i64 r = m - i0 - bs;
            if (r > 0)
                DDLA_TRY(gemm_any<T>(h, prec, r, n, bs, T(-1), A.sub(i0 + bs, r, i0, bs), X1, T(1),
                                     B.sub(i0 + bs, r, 0, n), DDLA_DENSE));
        } else if (i0 > 0) {
            DDLA_TRY(gemm_any<T>(h, prec, i0, n, bs, T(-1), A.sub(0, i0, i0, bs), X1, T(1), B.sub(0, i0, 0, n),
                                 DDLA_DENSE));
        }
    }
    return 0;
}

template int trsm<double>(ddla_handle, int, int, int, int, i64, i64, double, View<const double>, View<double>);
template int trsm<float>(ddla_handle, int, int, int, int, i64, i64, float, View<const float>, View<float>);
template int tri_inverse<double>(ddla_handle, bool, bool, View<const double>, i64, double *);
template int tri_inverse<float>(ddla_handle, bool, bool, View<const float>, i64, float *);
template int trsv_apply<double>(ddla_handle, bool, View<const double>, i64, const double *, double *, i64, int,
                                const double *);
template int trsv_apply<float>(ddla_handle, bool, View<const float>, i64, const float *, float *, i64, int,
                               const float *);

}  // namespace ddla

// ------------------------------------------------------------------ allocation-free solve
//
// ddla_dev_dtrsv_noalloc: the chained triangular solve above for callers that
// cannot allocate device memory (for example code that must not call
// cudaMalloc while other work is in flight, or that runs under an allocator it
// does not own).  All of its scratch -- the inverted 64 x 64 diagonal blocks
// and the per-block flags -- lives in ONE file-scope device array of fixed
// size, which every GPU that loads this library keeps for the life of the
// process.  That caps n at DDLA_NOALLOC_MAX_N and the right-hand sides at 16.
namespace ddla {
namespace {

constexpr int NOALLOC_MAX_N = 2048;
constexpr int NOALLOC_MAX_RHS = 16;
constexpr int NOALLOC_NBLK = NOALLOC_MAX_N / TB;
constexpr size_t NOALLOC_INV_BYTES = sizeof(double) * (size_t)NOALLOC_NBLK * TB * TB;   // 1 MiB
constexpr size_t NOALLOC_WORDS = NOALLOC_NBLK + 2;   // flags[nblk], ticket, error
constexpr size_t NOALLOC_BYTES = NOALLOC_INV_BYTES + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {};   // device address of g_noalloc_scratch, per device ordinal

}  // namespace

}  // namespace ddla

using namespace ddla;

extern "C" int ddla_dev_dtrsv_noalloc(void *stream, int32_t uplo, int32_t trans, int32_t diag, int64_t n,
                                      int64_t nrhs, const double *a, int64_t rsa, int64_t csa, double *x,
                                      int64_t ldx) {
    if (uplo != DDLA_LOWER && uplo != DDLA_UPPER) { set_error("uplo must be DDLA_LOWER or DDLA_UPPER"); return -2; }
    if (trans != DDLA_NO_TRANSPOSE && trans != DDLA_TRANSPOSE) { set_error("trans must be 0 or 8"); return -3; }
    if (diag != DDLA_UNIT_DIAG && diag != DDLA_NONUNIT_DIAG) { set_error("diag must be 0 or 0x100"); return -4; }
    if (n < 0 || n > NOALLOC_MAX_N) {
        set_error("ddla_dev_dtrsv_noalloc: n = " + std::to_string(n) + " exceeds the fixed scratch limit of " +
                  std::to_string(NOALLOC_MAX_N));
        return -5;
    }
    if (nrhs < 0 || nrhs > NOALLOC_MAX_RHS) {
        set_error("ddla_dev_dtrsv_noalloc: nrhs = " + std::to_string(nrhs) + " exceeds the limit of " +
                  std::to_string(NOALLOC_MAX_RHS));
        return -6;
    }
    if (ldx < (nrhs > 0 ? nrhs : 1)) { set_error("ldx must be >= nrhs"); return -11; }
    if (n == 0 || nrhs == 0) return 0;
    int dev = 0;
    DDLA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return DDLA_ERR_UNSUPPORTED; }
    void *base;
    {
        // one-time set-up per device, with that device current: the host-side
        // name g_noalloc_scratch is not a device address; ask the runtime for it
        std::lock_guard<std::mutex> g(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) DDLA_CUDA(cudaGetSymbolAddress(&g_noalloc_ptr[dev], g_noalloc_scratch));
        base = g_noalloc_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    double *inv = (double *)base;
    int *words = (int *)((unsigned char *)base + NOALLOC_INV_BYTES);
    const int nblk = (int)((n + TB - 1) / TB);
    int *flags = words, *ticket = words + nblk, *err = words + NOALLOC_NBLK + 1;
    // the array keeps the previous call's contents: the flags, the ticket and
    // the error word must start at zero
    DDLA_CUDA(cudaMemsetAsync(words, 0, sizeof(int) * NOALLOC_WORDS, s));
    View<const double> A{a, n, n, rsa, csa};
    bool lower = (uplo == DDLA_LOWER);
    if (trans == DDLA_TRANSPOSE) {
        A = A.t();
        lower = !lower;
    }
    k_tri_inv<double><<<nblk, TI_THREADS, 0, s>>>(A.p, A.rs, A.cs, n, lower ? 1 : 0, diag == DDLA_UNIT_DIAG ? 1 : 0, inv);
    DDLA_LAUNCHED();
    const int nr = (int)nrhs;
#define NOALLOC_CHAIN(NRV)                                                                                  \
    k_trsv_chain<double, NRV, 1><<<nblk, CHAIN_THREADS, 0, s>>>(n, nblk, A.p, A.rs, A.cs, lower ? 1 : 0, inv, x, \
                                                                ldx, nr, flags, ticket, err)
    if (nr <= 1) NOALLOC_CHAIN(1);
    else if (nr <= 2) NOALLOC_CHAIN(2);
    else if (nr <= 4) NOALLOC_CHAIN(4);
    else if (nr <= 8) NOALLOC_CHAIN(8);
    else NOALLOC_CHAIN(16);
#undef NOALLOC_CHAIN
    DDLA_LAUNCHED();
    int herr = 0;
    DDLA_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    DDLA_CUDA(cudaStreamSynchronize(s));
    if (herr) {
        set_error("ddla_dev_dtrsv_noalloc: a bounded wait of the chained solve gave up");
        return DDLA_ERR_TIMEOUT;
    }
    return 0;
}
