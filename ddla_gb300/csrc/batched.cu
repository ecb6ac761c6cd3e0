// Batched factorizations and solves of many small matrices of uneven size in
// ONE persistent launch (replayed from a CUDA graph).
//
// Each item is a square row-major matrix (n <= 1024) with one right-hand side:
//   kind 0  LU with partial pivoting   (DDLA LU.PLUDecompose, LU.cs:251-342)
//   kind 1  LU without pivoting        (LU.LUDecompose, LU.cs:133-203)
//   kind 2  Cholesky, lower            (Cholesky.CholDecompose, Cholesky.cs:52-160)
// Modes:
//   plain  FP64 factorization in place of A, then the FP64 solve x = A \ b;
//   mixed  FP32 factorization into a workspace, FP32 solves, FP64 residual
//          r = b - A x and update x += d until the item's backward error
//          ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol.
// CTAs of a persistent grid take items from a queue ordered by decreasing n
// (longest-first balancing).  One CTA factors one item with a blocked
// right-looking algorithm: the panel (m x nb) and the U12 / L21^T block live in
// shared memory, the trailing matrix stays in global memory, which L2 holds
// (a 256 x 256 FP64 item is 512 KB; 152 in flight fit in the 129 MB L2).
// Triangular solves go in 32-row blocks: one warp solves the diagonal block
// with shuffles, all threads update the rows below.
#include <algorithm>
#include <climits>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "timing.cuh"

namespace ddla {
namespace {

constexpr int BT = 256;            // threads per CTA
constexpr int BMAXN = 1024;        // largest item
constexpr int NBMAX = 32;          // largest panel width

struct BItem {
    int n, kind, nb, pad;
    i64 a, w, v;                   // element offsets: matrix (A), factor workspace, vectors (b, x, piv)
};

__device__ __forceinline__ unsigned long long bkey(double v) {
    unsigned long long u = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return u > 0x7ff0000000000000ull ? 0ull : u + 1ull;
}
__device__ __forceinline__ unsigned long long bkey(float v) {
    unsigned u = __float_as_uint(v) & 0x7fffffffu;
    return u > 0x7f800000u ? 0ull : (unsigned long long)u + 1ull;
}

constexpr int BMV = 2 * NBMAX;     // rows a panel's interchanges can move

struct BScratch {
    unsigned long long key[BT / 32];
    int idx[BT / 32];
    int fail;   // the pivot row and the row it displaces (LU), the scaled column (Cholesky)
    int nmv;            // rows moved by the current panel's interchanges
    int mv[BMV];        // those rows (relative to the panel's first row) ...
    int src[BMV];       // ... and the row each receives
};

// Calls f(r, c) for r in [0, rows), c in [0, cols) over the CTA: threads
// take columns in groups of the smallest power of two >= cols (at most 32),
// rows by the remaining thread index bits -- no division per element.
template <typename F>
__device__ __forceinline__ void for_rc(int rows, int cols, F f) {
    if (rows <= 0 || cols <= 0) return;
    int lg = 5;
    while (lg > 0 && (1 << (lg - 1)) >= cols) lg--;
    const int tid = threadIdx.x, tpr = 1 << lg, rpp = BT >> lg;
    for (int c = tid & (tpr - 1); c < cols; c += tpr)
        for (int r = tid >> lg; r < rows; r += rpp) f(r, c);
}

// Block-wide first-max over rows of column j of the panel.
template <typename T>
__device__ int panel_argmax(const T *Ps, int ld, int m, int j, BScratch &S) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned long long bv = 0;
    int bi = INT_MAX;
    for (int r = j + tid; r < m; r += BT) {
        unsigned long long v = bkey(Ps[r * ld + j]);
        if (bi == INT_MAX || v > bv) { bv = v; bi = r; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        unsigned long long ov = __shfl_down_sync(0xffffffffu, bv, off);
        int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (oi != INT_MAX && (bi == INT_MAX || ov > bv || (ov == bv && oi < bi))) { bv = ov; bi = oi; }
    }
    if (lane == 0) { S.key[warp] = bv; S.idx[warp] = bi; }
    __syncthreads();
    // every warp reduces the per-warp results itself (no second barrier)
    bv = lane < BT / 32 ? S.key[lane] : 0ull;
    bi = lane < BT / 32 ? S.idx[lane] : INT_MAX;
#pragma unroll
    for (int off = 4; off > 0; off >>= 1) {
        unsigned long long ov = __shfl_down_sync(0xffffffffu, bv, off);
        int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (oi != INT_MAX && (bi == INT_MAX || ov > bv || (ov == bv && oi < bi))) { bv = ov; bi = oi; }
    }
    bi = __shfl_sync(0xffffffffu, bi, 0);
    return bi == INT_MAX ? j : bi;
}

// In-place blocked factorization of one n x n row-major matrix W (ld = n).
// piv receives relative pivots (kind 0).  Returns 0 or the 1-based failing
// pivot.  Shared memory: panel Ps (n x (nb+1)) and block Us (nb x n).
template <typename T>
__device__ int factor_item(T *W, int n, int kind, int nb, int *piv, T *Ps, T *Us, BScratch &S) {
    const int tid = threadIdx.x;
    const int LDP = nb + 1;
    if (tid == 0) S.fail = 0;
    __syncthreads();
    for (int j0 = 0; j0 < n; j0 += nb) {
        const int jb = min(nb, n - j0), m = n - j0, r2 = n - j0 - jb;
        // 1. panel rows j0..n, cols j0..j0+jb
        for_rc(m, jb, [&](int r, int c) { Ps[r * LDP + c] = W[(i64)(j0 + r) * n + j0 + c]; });
        __syncthreads();
        // 2. unblocked factorization of the panel
        if (kind == 2) {
            // Cholesky of the diagonal block, then L21 = A21 L11^-T row by row
            for (int j = 0; j < jb; j++) {
                T d = Ps[j * LDP + j];
                bool bad = (isfinite(d) && d <= T(0));
                if (!bad) {
                    d = sqrt(d);
                    bad = !isfinite(d) || d == T(0);
                }
                if (bad) {
                    if (tid == 0) S.fail = j0 + j + 1;
                    break;
                }
                __syncthreads();
                if (tid == 0) Ps[j * LDP + j] = d;
                const T rinv = T(1) / d;
                for (int r = j + 1 + tid; r < m; r += BT) Ps[r * LDP + j] *= rinv;
                __syncthreads();
                for_rc(m - j - 1, jb - j - 1, [&](int rr, int cc) {
                    const int r = j + 1 + rr, c = j + 1 + cc;
                    if (r < jb && c > r) return;   // diagonal block: lower triangle only
                    Ps[r * LDP + c] = fma(Ps[c * LDP + j], -Ps[r * LDP + j], Ps[r * LDP + c]);
                });
                __syncthreads();
            }
        } else {
            for (int j = 0; j < jb; j++) {
                int p = j;
                if (kind == 0) {
                    p = panel_argmax<T>(Ps, LDP, m, j, S);
                    if (tid == 0) piv[j0 + j] = p - j;
                    if (p != j)
                        for (int c = tid; c < jb; c += BT) {
                            T t = Ps[j * LDP + c];
                            Ps[j * LDP + c] = Ps[p * LDP + c];
                            Ps[p * LDP + c] = t;
                        }
                    __syncthreads();
                } else if (j + 1 == m) {
                    break;   // LU without pivoting leaves the last pivot unchecked (LU.cs:191)
                }
                const T d = Ps[j * LDP + j];
                if (d == T(0)) {
                    if (tid == 0) S.fail = j0 + j + 1;
                    break;
                }
                const T rinv = T(1) / d;
                for (int r = j + 1 + tid; r < m; r += BT) Ps[r * LDP + j] *= rinv;
                __syncthreads();
                for_rc(m - j - 1, jb - j - 1, [&](int rr, int cc) {
                    const int r = j + 1 + rr, c = j + 1 + cc;
                    Ps[r * LDP + c] = fma(Ps[r * LDP + j], -Ps[j * LDP + c], Ps[r * LDP + c]);
                });
                __syncthreads();
            }
        }
        __syncthreads();
        if (S.fail) return S.fail;
        // 3. write the panel back (Cholesky: only the lower part of the diagonal block)
        for_rc(m, jb, [&](int r, int c) {
            if (kind == 2 && r < jb && c > r) return;
            W[(i64)(j0 + r) * n + j0 + c] = Ps[r * LDP + c];
        });
        __syncthreads();
        if (kind == 0) {
            // 4. the panel's interchanges on the other columns of rows j0..n,
            //    as one gather: the panel's permutation (thread 0 composes
            //    its jb swaps), the rows it moves (at most 2 jb), then those
            //    rows' elements in chunks of 32 columns, all loads before all
            //    stores of a chunk
            if (tid == 0) {
                // mv[k]: a position (relative to j0) whose content changes,
                // src[k]: the row whose original content ends there; the
                // first jb entries are positions 0 .. jb-1
                int cnt = 0;
                for (int j = 0; j < jb; j++) { S.mv[j] = j; S.src[j] = j; }
                for (int j = 0; j < jb; j++) {
                    const int p = piv[j0 + j] + j;
                    if (p == j) continue;
                    int kp = -1;   // slot of position p
                    if (p < jb) kp = p;
                    else
                        for (int k = jb; k < jb + cnt; k++)
                            if (S.mv[k] == p) { kp = k; break; }
                    if (kp < 0) { kp = jb + cnt++; S.mv[kp] = p; S.src[kp] = p; }
                    const int t = S.src[j];
                    S.src[j] = S.src[kp];
                    S.src[kp] = t;
                }
                S.nmv = jb + cnt;
            }
            __syncthreads();
            const int nmv = S.nmv;
            for (int cb = 0; cb < n; cb += 32) {
                T v[BMV / (BT / 32)];
#pragma unroll
                for (int t = 0; t < BMV / (BT / 32); t++) {
                    const int e = tid + BT * t, ri = e >> 5, c = cb + (e & 31);
                    if (ri < nmv && c < n && (c < j0 || c >= j0 + jb)) v[t] = W[(i64)(j0 + S.src[ri]) * n + c];
                }
                __syncthreads();
#pragma unroll
                for (int t = 0; t < BMV / (BT / 32); t++) {
                    const int e = tid + BT * t, ri = e >> 5, c = cb + (e & 31);
                    if (ri < nmv && c < n && (c < j0 || c >= j0 + jb)) W[(i64)(j0 + S.mv[ri]) * n + c] = v[t];
                }
                __syncthreads();
            }
        }
        if (r2 == 0) break;
        // 5. U12 = L11^-1 A12 (LU) or Us = L21^T (Cholesky), into shared memory
        if (kind == 2) {
            for_rc(jb, r2, [&](int i, int c) { Us[i * n + c] = Ps[(jb + c) * LDP + i]; });
        } else {
            // one thread per column c of U12, which it builds in Us (its own
            // column only: no barrier), forward substitution with unit L11
            for (int c = tid; c < r2; c += BT) {
                for (int i = 0; i < jb; i++) {
                    T s = W[(i64)(j0 + i) * n + j0 + jb + c];
                    for (int k = 0; k < i; k++) s = fma(-Ps[i * LDP + k], Us[k * n + c], s);
                    Us[i * n + c] = s;
                    W[(i64)(j0 + i) * n + j0 + jb + c] = s;
                }
            }
        }
        __syncthreads();
        // 6. trailing update A22 -= L21 * Us (Cholesky: lower triangle only),
        //    4 x 4 register tiles
        const int tr = (r2 + 3) / 4, tc = (r2 + 3) / 4;
        for (int t = tid; t < tr * tc; t += BT) {
            const int i0 = (t / tc) * 4, c0 = (t % tc) * 4;
            if (kind == 2 && c0 > i0 + 3) continue;
            T acc[4][4];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = T(0);
            for (int k = 0; k < jb; k++) {
                T l[4], u[4];
#pragma unroll
                for (int a = 0; a < 4; a++) l[a] = (i0 + a < r2) ? Ps[(jb + i0 + a) * LDP + k] : T(0);
#pragma unroll
                for (int b = 0; b < 4; b++) u[b] = (c0 + b < r2) ? Us[k * n + c0 + b] : T(0);
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) acc[a][b] = fma(l[a], u[b], acc[a][b]);
            }
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const int ii = i0 + a, cc = c0 + b;
                    if (ii < r2 && cc < r2 && !(kind == 2 && cc > ii)) {
                        T *p = &W[(i64)(j0 + jb + ii) * n + j0 + jb + cc];
                        *p -= acc[a][b];
                    }
                }
        }
        __syncthreads();
    }
    return 0;
}

// Triangular solve with one right-hand side x (shared memory, length n) and
// the factor in W (row-major).  lower: L (unit if `unit`) forward; else upper
// backward.  `trans` reads the triangle transposed (Cholesky's L^T).  Blocks
// of 32 rows: warp 0 loads its lanes' rows of the 32 x 32 diagonal block into
// registers first (independent loads, one L2 latency), then solves the block
// with shuffles; then every thread updates its rows outside the block.
template <typename T, typename X>
__device__ void trsv_item(const T *W, int n, bool lower, bool unit, bool trans, X *x) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    auto L = [&](int i, int k) -> X { return (X)(trans ? W[(i64)k * n + i] : W[(i64)i * n + k]); };
    const int nblk = (n + 31) / 32;
    for (int bi = 0; bi < nblk; bi++) {
        const int b = lower ? bi : nblk - 1 - bi;
        const int i0 = b * 32, bs = min(32, n - i0);
        if (warp == 0) {
            X lr[32];
#pragma unroll
            for (int k = 0; k < 32; k++) lr[k] = (lane < bs && k < bs) ? L(i0 + lane, i0 + k) : X(0);
            X xi = lane < bs ? x[i0 + lane] : X(0);
            if (lower) {
#pragma unroll
                for (int k = 0; k < 32; k++) {
                    if (k >= bs) break;
                    if (lane == k && !unit) xi /= lr[k];
                    const X xk = __shfl_sync(0xffffffffu, xi, k);
                    if (lane > k && lane < bs) xi = fma(-lr[k], xk, xi);
                }
            } else {
#pragma unroll
                for (int k = 31; k >= 0; k--) {
                    if (k >= bs) continue;
                    if (lane == k && !unit) xi /= lr[k];
                    const X xk = __shfl_sync(0xffffffffu, xi, k);
                    if (lane < k) xi = fma(-lr[k], xk, xi);
                }
            }
            if (lane < bs) x[i0 + lane] = xi;
        }
        __syncthreads();
        // rows outside the block
        const int r0 = lower ? i0 + bs : 0, r1 = lower ? n : i0;
        for (int r = r0 + tid; r < r1; r += BT) {
            X s = x[r];
#pragma unroll 8
            for (int k = 0; k < 32; k++)
                if (k < bs) s = fma(-L(r, i0 + k), x[i0 + k], s);
            x[r] = s;
        }
        __syncthreads();
    }
}

// The relative pivots of an LU item as one permutation: x_perm[i] =
// x[perm[i]] applies the interchanges i <-> i + piv[i] in increasing i
// (LU.cs:431-440) in one gather.  One thread, once per item.
__device__ void pivots_to_perm(const int *piv, int n, int kind, int *perm) {
    if (threadIdx.x == 0) {
        for (int i = 0; i < n; i++) perm[i] = i;
        if (kind == 0)
            for (int i = 0; i < n; i++) {
                const int p = piv[i];
                if (p) {
                    const int t = perm[i];
                    perm[i] = perm[i + p];
                    perm[i + p] = t;
                }
            }
    }
    __syncthreads();
}

// Mixed mode keeps its FP32 factor only for the correction solves, so each
// 32 x 32 diagonal block of it is replaced by its inverse once after the
// factorization (LU: strict lower part inv(L_kk), unit; upper part with the
// diagonal inv(U_kk); Cholesky: lower part with the diagonal inv(L_kk)).
// Every later block solve is then a product with the inverse (a lane per
// row, no sequential chain).  Warp w inverts the blocks w, w + 8, ..: the
// block goes through a 32 x 33 shared tile (tiles[w]), lane c forms column c
// of the inverse in registers (static indices).
__device__ void invert_diag_blocks(float *W, int n, int kind, float *tiles) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *Tl = tiles + warp * 32 * 33;
    const int nblk = (n + 31) / 32;
    for (int b = warp; b < nblk; b += BT / 32) {
        const int i0 = b * 32, bs = min(32, n - i0);
        // the block, padded with the identity
        for (int r = 0; r < 32; r++)
            Tl[r * 33 + lane] = (r < bs && lane < bs) ? W[(i64)(i0 + r) * n + i0 + lane] : (r == lane ? 1.f : 0.f);
        __syncwarp();
        const int c = lane;
        {
            // lower triangle: unit (LU) or with the diagonal (Cholesky)
            float x[32];
#pragma unroll
            for (int i = 0; i < 32; i++) {
                float s = (i == c) ? 1.f : 0.f;
#pragma unroll
                for (int k = 0; k < i; k++) s = fmaf(-Tl[i * 33 + k], x[k], s);
                x[i] = kind == 2 ? s / Tl[i * 33 + i] : s;
            }
            // column c below (Cholesky: and on) the diagonal
#pragma unroll
            for (int r = 0; r < 32; r++)
                if (r < bs && c < bs && (kind == 2 ? r >= c : r > c)) W[(i64)(i0 + r) * n + i0 + c] = x[r];
        }
        if (kind != 2) {
            // upper triangle with the diagonal (LU's U)
            float y[32];
#pragma unroll
            for (int i = 31; i >= 0; i--) {
                float s = (i == c) ? 1.f : 0.f;
#pragma unroll
                for (int k = i + 1; k < 32; k++) s = fmaf(-Tl[i * 33 + k], y[k], s);
                y[i] = s / Tl[i * 33 + i];
            }
#pragma unroll
            for (int r = 0; r < 32; r++)
                if (r < bs && c < bs && r <= c) W[(i64)(i0 + r) * n + i0 + c] = y[r];
        }
        __syncwarp();
    }
    __syncthreads();
}

// Triangular solve with the inverted diagonal blocks (invert_diag_blocks):
// per 32-row block, warp 0 forms x_blk = inv(T_kk) x_blk (lane i: one row or,
// transposed, one column of the inverse), then every thread updates its rows
// outside the block with the off-diagonal part of the factor.
__device__ void trsv_item_inv(const float *W, int n, bool lower, bool unit, bool trans, float *x) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    auto L = [&](int i, int k) -> float { return trans ? W[(i64)k * n + i] : W[(i64)i * n + k]; };
    const int nblk = (n + 31) / 32;
    for (int bi = 0; bi < nblk; bi++) {
        const int b = lower ? bi : nblk - 1 - bi;
        const int i0 = b * 32, bs = min(32, n - i0);
        if (warp == 0) {
            float li[32];
#pragma unroll
            for (int k = 0; k < 32; k++) {
                const bool in = lane < bs && k < bs && (lower ? k <= lane : k >= lane);
                li[k] = in ? L(i0 + lane, i0 + k) : 0.f;
            }
            float xv[32];
#pragma unroll
            for (int k = 0; k < 32; k++) xv[k] = k < bs ? x[i0 + k] : 0.f;
            __syncwarp();
            float y = 0.f;   // a unit diagonal is implicit: 1 in place of the stored entry
#pragma unroll
            for (int k = 0; k < 32; k++) y = fmaf((unit && k == lane) ? 1.f : li[k], xv[k], y);
            if (lane < bs) x[i0 + lane] = y;
        }
        __syncthreads();
        const int r0 = lower ? i0 + bs : 0, r1 = lower ? n : i0;
        for (int r = r0 + tid; r < r1; r += BT) {
            float s = x[r];
#pragma unroll 8
            for (int k = 0; k < 32; k++)
                if (k < bs) s = fmaf(-L(r, i0 + k), x[i0 + k], s);
            x[r] = s;
        }
        __syncthreads();
    }
}

// x holds the right-hand side already permuted (pivots_to_perm)
template <typename T, typename X>
__device__ void solve_item(const T *W, int n, int kind, X *x) {
    if (kind == 2) {
        trsv_item<T, X>(W, n, true, false, false, x);
        trsv_item<T, X>(W, n, false, false, true, x);
    } else {
        trsv_item<T, X>(W, n, true, true, false, x);
        trsv_item<T, X>(W, n, false, false, false, x);
    }
}

__device__ double block_max(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    v = red[0];
    for (int q = 1; q < BT / 32; q++) v = fmax(v, red[q]);
    return v;
}

struct BArgs {
    const BItem *items;
    const int *order;
    int count;
    double *A;        // inputs (plain: factored in place)
    const double *B;  // right-hand sides
    double *X;        // solutions
    int *piv;
    float *W32;       // FP32 factors (mixed)
    int *info;        // per item: failing pivot, 0 ok
    int *iters;       // per item: refinement steps (-1 = not converged)
    int *counter;
    int mixed, max_iter;
    double tol;
};

// MIXED: FP32 factor + FP64 refinement (two CTAs per SM); plain: FP64 (its
// shared memory allows one CTA per SM, so it may use more registers)
template <bool MIXED>
__global__ void __launch_bounds__(BT, MIXED ? 2 : 1) k_batched(BArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ BScratch S;
    __shared__ int s_item;
    __shared__ double red[BT / 32];
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
        __syncthreads();
        const int q = s_item;
        __syncthreads();
        if (q >= a.count) break;
        const BItem it = a.items[a.order[q]];
        const int n = it.n, tid = threadIdx.x;
        double *A = a.A + it.a;
        const double *b = a.B + it.v;
        double *x = a.X + it.v;
        int *piv = a.piv + it.v;
        int rc;
        if constexpr (!MIXED) {
            double *Ps = (double *)smem;
            double *Us = Ps + (size_t)n * (it.nb + 1);
            double *xs = Us + (size_t)it.nb * n;
            int *perm = (int *)(xs + n);
            rc = factor_item<double>(A, n, it.kind, it.nb, piv, Ps, Us, S);
            if (tid == 0) a.info[a.order[q]] = rc;
            if (rc == 0) {
                pivots_to_perm(piv, n, it.kind, perm);
                for (int i = tid; i < n; i += BT) xs[i] = b[perm[i]];
                __syncthreads();
                solve_item<double, double>(A, n, it.kind, xs);
                for (int i = tid; i < n; i += BT) x[i] = xs[i];
            }
            if (tid == 0) a.iters[a.order[q]] = 0;
        } else {
            float *Wf = a.W32 + it.w;
            float *Ps = (float *)smem;
            float *Us = Ps + (size_t)n * (it.nb + 1);
            float *ds = Us + (size_t)it.nb * n;
            double *xs = (double *)(((uintptr_t)(ds + n) + 15) & ~(uintptr_t)15);
            double *rs = xs + n;
            int *perm = (int *)(rs + n);
            for (int e = tid; e < n * n; e += BT) Wf[e] = (float)A[e];
            __syncthreads();
            // ||A||_inf of the FP64 matrix and ||b||_inf, before the copy is
            // factored
            double an = 0, bn = 0;
            for (int r = tid; r < n; r += BT) {
                double s = 0.0;
                for (int c = 0; c < n; c++) s += fabs(A[(i64)r * n + c]);
                an = fmax(an, s);
                bn = fmax(bn, fabs(b[r]));
            }
            an = block_max(an, red);
            bn = block_max(bn, red);
            __syncthreads();
            rc = factor_item<float>(Wf, n, it.kind, it.nb, piv, Ps, Us, S);
            if (tid == 0) a.info[a.order[q]] = rc;
            int iters = -1;
            if (rc == 0) {
                invert_diag_blocks(Wf, n, it.kind, Ps);   // the panel buffer is free now
                pivots_to_perm(piv, n, it.kind, perm);
                for (int i = tid; i < n; i += BT) { xs[i] = 0.0; rs[i] = b[i]; }
                __syncthreads();
                for (int k = 0; k <= a.max_iter; k++) {
                    // d = LU \ P r in FP32, x += d in FP64
                    for (int i = tid; i < n; i += BT) ds[i] = (float)rs[perm[i]];
                    __syncthreads();
                    if (it.kind == 2) {
                        trsv_item_inv(Wf, n, true, false, false, ds);
                        trsv_item_inv(Wf, n, false, false, true, ds);
                    } else {
                        trsv_item_inv(Wf, n, true, true, false, ds);
                        trsv_item_inv(Wf, n, false, false, false, ds);
                    }
                    for (int i = tid; i < n; i += BT) xs[i] += (double)ds[i];
                    __syncthreads();
                    // r = b - A x in FP64
                    double rn = 0, xn = 0;
                    for (int r = tid; r < n; r += BT) {
                        double s = b[r];
                        const double *ar = A + (i64)r * n;
                        for (int c = 0; c < n; c++) s = fma(-ar[c], xs[c], s);
                        rs[r] = s;
                        rn = fmax(rn, fabs(s));
                        xn = fmax(xn, fabs(xs[r]));
                    }
                    rn = block_max(rn, red);
                    xn = block_max(xn, red);
                    // stop at half the target: a recomputation of the
                    // backward error with another summation order differs by
                    // a few 1e-15 at these sizes, and must still meet tol
                    const double den = an * xn + bn;
                    if (den > 0 ? rn / den <= 0.5 * a.tol : rn == 0) { iters = k; break; }
                }
                for (int i = tid; i < n; i += BT) x[i] = xs[i];
            }
            if (tid == 0) a.iters[a.order[q]] = iters;
        }
        __syncthreads();
    }
}

}  // namespace

// ------------------------------------------------------------------ plan

struct BatchedPlan {
    ddla_handle h = nullptr;
    int count = 0;
    int mixed = 0;
    int max_n = 0;
    int grid = 0;
    size_t smem = 0;
    BItem *d_items = nullptr;
    int *d_order = nullptr;
    int *d_counter = nullptr;
    float *d_w32 = nullptr;
    BArgs args{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double flops = 0;
    std::vector<int> n_host;
};

static int nb_for(int n, int kind) {
    // panel width per size bucket (tuning keys batched.nb.<bucket>)
    const char *key = n <= 32 ? "batched.nb.32" : n <= 64 ? "batched.nb.64" : n <= 128 ? "batched.nb.128" : "batched.nb.big";
    int64_t v = tune_get(key, 0);
    if (v > 0) return (int)std::min<int64_t>(v, NBMAX);
    (void)kind;
    return n <= 32 ? 8 : (n <= 64 ? 16 : 32);
}

}  // namespace ddla

using namespace ddla;

extern "C" {

/* see include/ddla_gb300.h */
int ddla_batched_plan_create(ddla_handle h, int64_t count, const int32_t *n, const int32_t *kind, int32_t mixed,
                             double *d_a, const double *d_b, double *d_x, int32_t *d_piv, int32_t *d_info,
                             int32_t *d_iters, const ddla_opts *opts, void **plan_out) {
    if (!h) return -1;
    if (count < 0) return -2;
    if (!n && count) return -3;
    if (!kind && count) return -4;
    if (!plan_out) return -13;
    BatchedPlan *P = new BatchedPlan();
    P->h = h;
    P->count = (int)count;
    P->mixed = mixed ? 1 : 0;
    std::vector<BItem> items((size_t)count);
    i64 ao = 0, wo = 0, vo = 0;
    size_t smem = 0;
    for (i64 i = 0; i < count; i++) {
        int ni = n[i], ki = kind[i];
        if (ni < 1 || ni > BMAXN || ki < 0 || ki > 2) {
            delete P;
            set_error("batched item " + std::to_string(i) + ": n must be in [1, 1024] and kind in {0,1,2}");
            return -3;
        }
        int nb = nb_for(ni, ki);
        items[i] = BItem{ni, ki, nb, 0, ao, wo, vo};
        ao += (i64)ni * ni;
        wo += (i64)ni * ni;
        vo += ni;
        P->max_n = std::max(P->max_n, ni);
        // plain: Ps, Us, x in FP64; mixed: Ps, Us, d in FP32 + x, r in FP64
        // + the item's permutation (n ints)
        size_t sm = mixed ? sizeof(float) * ((size_t)ni * (nb + 1) + (size_t)nb * ni + ni) + 16 + sizeof(double) * 2 * ni
                          : sizeof(double) * ((size_t)ni * (nb + 1) + (size_t)nb * ni + ni);
        sm += sizeof(int) * (size_t)ni;
        // mixed: the panel buffer also holds one 32 x 33 tile per warp while
        // the diagonal blocks are inverted
        if (mixed) sm = std::max(sm, sizeof(float) * (BT / 32) * 32 * 33);
        smem = std::max(smem, sm);
        P->flops += (ki == 2 ? 1.0 / 3.0 : 2.0 / 3.0) * (double)ni * ni * ni + 2.0 * ni * ni;
        P->n_host.push_back(ni);
    }
    // longest items first
    std::vector<int> order((size_t)count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return items[x].n > items[y].n; });
    int rc = 0;
    auto fail = [&](int code) {
        if (P->d_items) cudaFree(P->d_items);
        if (P->d_order) cudaFree(P->d_order);
        if (P->d_counter) cudaFree(P->d_counter);
        if (P->d_w32) cudaFree(P->d_w32);
        delete P;
        return code;
    };
    if (cudaMalloc(&P->d_items, sizeof(BItem) * std::max<i64>(count, 1)) != cudaSuccess ||
        cudaMalloc(&P->d_order, sizeof(int) * std::max<i64>(count, 1)) != cudaSuccess ||
        cudaMalloc(&P->d_counter, sizeof(int)) != cudaSuccess ||
        (mixed && cudaMalloc(&P->d_w32, sizeof(float) * std::max<i64>(wo, 1)) != cudaSuccess)) {
        cudaGetLastError();
        set_error("batched plan: device allocation failed");
        return fail(DDLA_ERR_NOMEM);
    }
    if (cudaMemcpy(P->d_items, items.data(), sizeof(BItem) * count, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(P->d_order, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("batched plan: upload failed");
        return fail(DDLA_ERR_CUDA);
    }
    size_t avail = 0;
    const void *kfn = mixed ? (const void *)k_batched<true> : (const void *)k_batched<false>;
    rc = max_dyn_smem(kfn, h->smem_optin, &avail);
    if (rc) return fail(rc);
    if (smem > avail) {
        set_error("batched plan: items too large for shared memory");
        return fail(DDLA_ERR_UNSUPPORTED);
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, BT, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int64_t want = tune_get("batched.ctas_per_sm", 0);
    if (want > 0 && want < per_sm) per_sm = (int)want;
    P->grid = std::max(1, std::min<int>(h->sm_count * per_sm, (int)std::max<i64>(count, 1)));
    P->smem = smem;
    P->args = BArgs{P->d_items, P->d_order, (int)count, d_a, d_b, d_x, d_piv, P->d_w32, d_info, d_iters,
                    P->d_counter, P->mixed, (opts && opts->max_iter > 0) ? opts->max_iter : 30,
                    (opts && opts->tol > 0) ? opts->tol : 1e-14};
    // capture: reset the queue counter, run the persistent kernel
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return fail(DDLA_ERR_CUDA);
    bool ok = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        cudaMemsetAsync(P->d_counter, 0, sizeof(int), cap);
        if (mixed) k_batched<true><<<P->grid, BT, smem, cap>>>(P->args);
        else k_batched<false><<<P->grid, BT, smem, cap>>>(P->args);
        count_launch();
        ok = cudaStreamEndCapture(cap, &P->graph) == cudaSuccess;
    }
    if (ok) ok = cudaGraphInstantiate(&P->exec, P->graph, 0) == cudaSuccess;
    cudaStreamDestroy(cap);
    if (!ok) {
        cudaGetLastError();
        set_error("batched plan: CUDA graph capture failed");
        return fail(DDLA_ERR_CUDA);
    }
    *plan_out = P;
    return 0;
}

int ddla_batched_plan_exec(void *plan) {
    if (!plan) return -1;
    BatchedPlan *P = (BatchedPlan *)plan;
    Timed t(P->h->stream, TC_BATCHED, P->flops, 0.0);
    DDLA_CUDA(cudaGraphLaunch(P->exec, P->h->stream));
    count_launch();
    return 0;
}

int ddla_batched_plan_info(void *plan, double *flops, int32_t *grid, int64_t *smem_bytes) {
    if (!plan) return -1;
    BatchedPlan *P = (BatchedPlan *)plan;
    if (flops) *flops = P->flops;
    if (grid) *grid = P->grid;
    if (smem_bytes) *smem_bytes = (int64_t)P->smem;
    return 0;
}

int ddla_batched_plan_destroy(void *plan) {
    if (!plan) return 0;
    BatchedPlan *P = (BatchedPlan *)plan;
    cudaStreamSynchronize(P->h->stream);
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    cudaFree(P->d_items);
    cudaFree(P->d_order);
    cudaFree(P->d_counter);
    if (P->d_w32) cudaFree(P->d_w32);
    delete P;
    return 0;
}

}  // extern "C"
