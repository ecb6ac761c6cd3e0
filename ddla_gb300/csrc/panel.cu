// LU panel factorization with partial pivoting and the row interchanges.
//
// The panel (m rows x w <= 64 columns) is factored by ONE thread-block cluster
// (up to 16 CTAs).  Each CTA keeps a contiguous slice of the panel rows in
// shared memory for the whole factorization, so no panel data goes back to
// HBM between columns.  Per column j:
//   1. each CTA finds the first largest |a(r,j)| among its rows r >= j
//      (NaN compares smaller than everything, like bli_damaxv as DDLA
//      documents it, DDLA/BLAS/1v.cs:29-42);
//   2. it pushes a package -- (value, row, origin) and a finished copy of the
//      candidate row -- into an inbox slot of every CTA of the cluster with
//      st.async stores that complete on the receiver's mbarrier; the owner of
//      row j pushes row j as well;
//   3. every CTA waits on its own mbarrier until all packages of column j have
//      landed (no cluster barrier, no remote loads), picks the same winner
//      (largest value, lowest row on ties) from its local inbox, and the owners
//      of rows j and p swap them (whole panel rows, LU.cs:367-374);
//   4. rows below j are scaled by 1/pivot (InvScal, a zero pivot stops the
//      factorization and reports it, DDLA/BLAS/1v.cs:97-103) and rank-1
//      updated (GeR(-1), LU.cs:357-360).
// The inboxes are double-buffered on the column parity.  A CTA pushes the
// packages of column j+1 only after it has read its inbox of column j, and no
// CTA can send packages of column j+2 before it received those of column j+1
// from every CTA, so a slot is never overwritten while it is being read.
//
// Every row carries its origin (row index at panel start), so the interchange
// of the rest of the matrix is a gather of the touched rows (at most 2w),
// applied by k_laswp_list in parallel over columns.
#include <cooperative_groups.h>

#include <climits>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace ddla {

constexpr int PANEL_WMAX = 64;
constexpr int PANEL_THREADS = 512;
constexpr int PANEL_MAXCS = 16;

template <typename T>
struct PanelArgs {
    T *P;
    i64 rs, cs;
    int m, w, rows_per;
    int32_t *piv;
    int *info;
    i64 row_base;
    int *touch_count, *touch_rows, *touch_src;
    T *inv;   // optional: inverse of the unit-lower w x w block L11 (row-major, ld TRI_TB)
    int *calu;   // tournament-pivoting scratch (k_panel_calu)
    int *err;    // set to 1 when a bounded wait of the cluster panel gives up
    // optional (k_panel_lu): load the panel from ld (strides ld_rs, ld_cs)
    // instead of P, and copy u12_rows x w finished U12 rows from u12_src
    // (ld w) to u12_dst before the first exchange
    const T *ld;
    i64 ld_rs, ld_cs;
    const T *u12_src;
    T *u12_dst;
    int u12_rows;
};

// Pivot search keys: |x| as an unsigned integer bit pattern plus one, NaN as
// 0.  For non-negative IEEE values the integer order is the value order, so
// "largest key, lowest row on ties" is bli_damaxv's first-max rule with NaN
// below every number -- and it runs on the integer pipe (on GB300 even a
// double compare goes through the 1/64-rate FP64 pipe).
template <typename T> struct KeyT;
template <> struct KeyT<float> { typedef unsigned int type; };
template <> struct KeyT<double> { typedef unsigned long long type; };
__device__ __forceinline__ unsigned int amax_key(float v) {
    unsigned int u = __float_as_uint(v) & 0x7fffffffu;
    return u > 0x7f800000u ? 0u : u + 1u;
}
__device__ __forceinline__ unsigned long long amax_key(double v) {
    unsigned long long u = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return u > 0x7ff0000000000000ull ? 0ull : u + 1ull;
}

constexpr int PANEL_SUB = 8;   // sub-panel width (deferred updates)

// A package: 16-byte header (key at byte 0, row at 8, origin at 12), then
// the row's w values; slots are sized for PANEL_WMAX values.
constexpr int PKG_HDR = 16;
template <typename T> constexpr int pkg_stride() { return PKG_HDR + PANEL_WMAX * (int)sizeof(T); }
constexpr long long PANEL_SPIN = 1LL << 22;   // bounded waits (try_wait rounds)

struct PanelSmem {
    size_t rows, origin, u8, inbox, outbox, red, total;
};

template <typename T>
__host__ __device__ inline PanelSmem panel_smem_layout(int rows_per, int w) {
    PanelSmem L;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = (o + bytes + 15) & ~(size_t)15;
        return at;
    };
    L.rows = take(sizeof(T) * (size_t)rows_per * (w + 1));
    L.origin = take(sizeof(int) * (size_t)rows_per);
    L.u8 = take(sizeof(T) * (size_t)w * PANEL_SUB);
    L.inbox = take((size_t)2 * (PANEL_MAXCS + 1) * pkg_stride<T>());   // [parity][sender | row j][package]
    L.outbox = take((size_t)2 * pkg_stride<T>());                        // [candidate | row j+1]
    L.red = take((sizeof(typename KeyT<T>::type) + sizeof(int)) * (PANEL_THREADS / 32) + 16);
    L.total = o;
    return L;
}

// Block-wide first-max reduction of (key, row) pairs.  Every warp reduces
// the per-warp results itself, so all threads return the block's winner after
// a single barrier.
// Warp-wide first max of (key, row): the largest key, the lowest row among
// equal keys (rows INT_MAX stand for "no candidate").  32-bit keys use the
// warp reduction instructions.
template <typename K>
__device__ __forceinline__ void warp_argmax(K &bv, int &bi) {
    if constexpr (sizeof(K) == 4) {
        const unsigned m = __reduce_max_sync(0xffffffffu, (unsigned)bv);
        bi = __reduce_min_sync(0xffffffffu, (unsigned)bv == m ? bi : INT_MAX);
        bv = (K)m;
    } else {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            K ov = __shfl_xor_sync(0xffffffffu, bv, off);
            int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
        }
    }
}

// Block-wide first-max reduction of (key, row) pairs.  Every warp reduces
// the per-warp results itself, so all threads return the block's winner after
// a single barrier.
template <typename K>
__device__ __forceinline__ void block_argmax(K &bv, int &bi, K *red_v, int *red_i) {
    constexpr int NW = PANEL_THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    warp_argmax<K>(bv, bi);
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
    __syncthreads();
    bv = lane < NW ? red_v[lane] : K(0);
    bi = lane < NW ? red_i[lane] : INT_MAX;
    warp_argmax<K>(bv, bi);
}

// 8 consecutive U8 entries (one column of the sub-panel's pivot rows);
// 16-byte aligned
__device__ __forceinline__ void ld8(const float *p, float *v) {
    const float4 a = *reinterpret_cast<const float4 *>(p), b = *reinterpret_cast<const float4 *>(p + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void ld8(const double *p, double *v) {
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
        const double2 a = *reinterpret_cast<const double2 *>(p + i);
        v[i] = a.x; v[i + 1] = a.y;
    }
}

__device__ __forceinline__ unsigned su32p(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
// Shared-memory address of the same variable in CTA `rank` of the cluster.
__device__ __forceinline__ unsigned cluster_addr(const void *p, int rank) {
    unsigned out;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"((unsigned)__cvta_generic_to_shared(p)),
                 "r"(rank));
    return out;
}
// 16 bytes into another CTA's shared memory; the store completes 16 bytes of
// the transaction count of that CTA's mbarrier
__device__ __forceinline__ void st_async16(unsigned addr, uint4 v, unsigned mbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
                     addr),
                 "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "r"(mbar)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_cluster(unsigned mbar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void mbar_expect(unsigned mbar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// Panel factorization, one cluster (see the file comment).  The columns are
// processed in sub-panels of PANEL_SUB: within a sub-panel the rank-1 updates
// touch only the sub-panel's columns; the columns to its right receive the
// sub-panel's pivot rows (kept in U8) as one rank-PANEL_SUB update after its
// last column, which divides the shared-memory traffic of the updates by
// about PANEL_SUB.  Rows that leave their CTA (pivot candidates, row j+1) are
// packaged with every pending update applied to the copy.  Per column the
// critical path is: wait for the packages -> winner -> swap -> scale + update
// of the next column and its local argmax -> packages of the next column ->
// push to every CTA; the remaining updates run while the other CTAs' packages
// are in flight.  Every wait is bounded: on timeout the CTA records the error
// in a.err, stops factoring and meets the others at the final cluster barrier
// (they time out the same way, waiting for its packages).
template <typename T>
__global__ void __launch_bounds__(PANEL_THREADS, 1) k_panel_lu(PanelArgs<T> a) {
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = a.w, WP = w + 1, rp = a.rows_per;
    const PanelSmem L = panel_smem_layout<T>(rp, w);
    T *rows = (T *)(smem + L.rows);
    int *origin = (int *)(smem + L.origin);
    typedef typename KeyT<T>::type K;
    T *U8 = (T *)(smem + L.u8);   // [c][k]: pivot rows of the current sub-panel, column-major by k
    unsigned char *inbox = smem + L.inbox;
    unsigned char *outbox = smem + L.outbox;
    K *red_v = (K *)(smem + L.red);
    int *red_i = (int *)(red_v + PANEL_THREADS / 32);
    constexpr int STRIDE = pkg_stride<T>();
    // bytes pushed per package (header + w values, whole 16-byte chunks)
    const int PKG = PKG_HDR + (((int)sizeof(T) * w + 15) & ~15);
    auto slot = [&](int parity, int src) { return inbox + (parity * (PANEL_MAXCS + 1) + src) * STRIDE; };

    __shared__ int spiv[PANEL_WMAX];   // relative pivots, stored to global memory at the end
    __shared__ __align__(8) unsigned long long full[2];   // inbox mbarriers, by column parity
    for (int c = tid; c < PANEL_WMAX; c += PANEL_THREADS) spiv[c] = 0;
    const int base = rank * rp;
    int nloc = a.m - base;
    nloc = nloc < 0 ? 0 : (nloc > rp ? rp : nloc);
    auto owns = [&](int g) { return g >= base && g < base + nloc; };
    const int kmax = a.m < w ? a.m : w;
    const unsigned col_bytes = (unsigned)((CS + 1) * PKG);   // every CTA's candidate + row j

    if (rank == 0 && tid == 0) *a.touch_count = 0;
    {
        const T *src = a.ld ? a.ld : a.P;
        const i64 srs = a.ld ? a.ld_rs : a.rs, scs = a.ld ? a.ld_cs : a.cs;
        for (int e = tid; e < nloc * w; e += PANEL_THREADS) {
            int l = e / w, c = e % w;
            rows[l * WP + c] = src[(i64)(base + l) * srs + (i64)c * scs];
        }
    }
    if (a.u12_dst && rank == 0)
        for (int e = tid; e < a.u12_rows * w; e += PANEL_THREADS)
            a.u12_dst[(i64)(e / w) * a.rs + (i64)(e % w) * a.cs] = a.u12_src[e];
    for (int l = tid; l < nloc; l += PANEL_THREADS) origin[l] = base + l;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32p(&full[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32p(&full[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (kmax > 0) mbar_expect(su32p(&full[0]), col_bytes);
        if (kmax > 1) mbar_expect(su32p(&full[1]), col_bytes);
    }
    // every CTA's mbarriers are armed before anyone pushes
    cluster.sync();

    // Stage the packages of column c in the outbox (candidate cb with key cv;
    // row c if this CTA owns it; `val(row, col)` gives a row's finished
    // value) and push them: warp d sends to CTA d, the candidate into slot
    // `rank`, row c into slot PANEL_MAXCS.
    auto stage_push = [&](int c, K cv, int cb, auto val) {
        const bool with_row = owns(c);
        unsigned char *ob_c = outbox, *ob_r = outbox + STRIDE;
        if (tid < w) {
            if (cb != INT_MAX) ((T *)(ob_c + PKG_HDR))[tid] = val(rows + (cb - base) * WP, tid, false);
        } else if (tid >= 64 && tid < 64 + w && with_row) {
            ((T *)(ob_r + PKG_HDR))[tid - 64] = val(rows + (c - base) * WP, tid - 64, true);
        }
        if (tid == PANEL_THREADS - 1) {
            *(K *)ob_c = cv;
            *(int *)(ob_c + 8) = cb;
            *(int *)(ob_c + 12) = cb != INT_MAX ? origin[cb - base] : 0;
        } else if (tid == PANEL_THREADS - 2 && with_row) {
            *(K *)ob_r = K(0);
            *(int *)(ob_r + 8) = c;
            *(int *)(ob_r + 12) = origin[c - base];
        }
        __syncthreads();
        if (warp < CS) {
            const int par = c & 1;
            const unsigned mb = cluster_addr(&full[par], warp);
            const unsigned dc = cluster_addr(slot(par, rank), warp);
            const int chunks = PKG / 16;
            for (int q = lane; q < chunks; q += 32)
                st_async16(dc + 16 * q, *reinterpret_cast<const uint4 *>(ob_c + 16 * q), mb);
            if (with_row) {
                const unsigned dr = cluster_addr(slot(par, PANEL_MAXCS), warp);
                for (int q = lane; q < chunks; q += 32)
                    st_async16(dr + 16 * q, *reinterpret_cast<const uint4 *>(ob_r + 16 * q), mb);
            }
        }
    };

    bool failed = false;
    if (kmax > 0) {
        K bv = 0;
        int bi = INT_MAX;
        for (int l = tid; l < nloc; l += PANEL_THREADS) {
            K v = amax_key(rows[l * WP]);
            if (v > bv || bi == INT_MAX) { bv = v; bi = base + l; }
        }
        block_argmax<K>(bv, bi, red_v, red_i);
        // nothing is pending before column 0: the packages are the rows
        stage_push(0, bv, bi, [&](const T *row, int c, bool) { return row[c]; });
    }

    for (int j = 0; j < kmax; j++) {
        const int buf = j & 1;
        const int s0 = j - j % PANEL_SUB, s1 = s0 + PANEL_SUB < w ? s0 + PANEL_SUB : w;
        bool ok = false;
        {
            const unsigned mb = su32p(&full[buf]), par = (unsigned)((j >> 1) & 1);
            for (long long it = 0; it < PANEL_SPIN && !ok; it++) ok = mbar_try_cluster(mb, par);
        }
        // (also orders the previous column's row updates before the swap below)
        if (__syncthreads_or(!ok)) { failed = true; break; }
        if (tid == 0 && j + 2 < kmax) mbar_expect(su32p(&full[buf]), col_bytes);   // re-arm for column j+2
        // winner (identical in every CTA, from the local inbox): lanes
        // 0..CS-1 each read one candidate, then a butterfly over the warp
        K wv = lane < CS ? *(const K *)slot(buf, lane) : K(0);
        int wi = lane < CS ? *(const int *)(slot(buf, lane) + 8) : INT_MAX;
        const int myi = wi;
        warp_argmax<K>(wv, wi);
        // the winning row is unique: its CTA is the lane that proposed it
        const unsigned hit = __ballot_sync(0xffffffffu, myi == wi && wi != INT_MAX);
        const int wr = hit ? __ffs(hit) - 1 : 0;
        const bool none = (wi == INT_MAX);
        const int p = none ? j : wi;
        const unsigned char *upkg = slot(buf, none ? PANEL_MAXCS : wr), *rpkg = slot(buf, PANEL_MAXCS);
        const T *U = (const T *)(upkg + PKG_HDR);   // the finished pivot row (valid until column j+2)
        if (tid < w) {
            const T u = U[tid];
            U8[tid * PANEL_SUB + (j - s0)] = u;
            if (owns(j)) rows[(j - base) * WP + tid] = u;   // row j becomes the pivot row
        } else if (p != j && owns(p) && tid >= 64 && tid < 64 + w) {
            // row p receives the old row j, in the same pending-update state as the stored rows
            rows[(p - base) * WP + (tid - 64)] = ((const T *)(rpkg + PKG_HDR))[tid - 64];
        }
        if (tid == PANEL_THREADS - 1) {
            spiv[j] = p - j;
            if (owns(j)) origin[j - base] = *(const int *)(upkg + 12);
            if (p != j && owns(p)) origin[p - base] = *(const int *)(rpkg + 12);
        }
        __syncthreads();
        const T ujj = U[j];
        if (ujj == T(0)) {
            if (rank == 0 && tid == 0) atomicMin(a.info, (int)(a.row_base + j + 1));
            break;
        }
        const T rinv = T(1) / ujj;
        const bool more = j + 1 < kmax;
        const bool edge = (j + 1 == s1);   // j is the last column of its sub-panel
        int ls = j + 1 - base;
        if (ls < 0) ls = 0;
        // scale column j; bring column j+1 up to date (rank-1 inside the
        // sub-panel, the whole sub-panel at its edge) and find its local max
        K bv = 0;
        int bi = INT_MAX;
        const T uj1 = j + 1 < w ? U[j + 1] : T(0);
        for (int l = ls + tid; l < nloc; l += PANEL_THREADS) {
            T *row = rows + l * WP;
            T lv = row[j] * rinv;
            row[j] = lv;
            if (j + 1 < w) {
                T v = row[j + 1];
                if (!edge) {
                    v = fma(lv, -uj1, v);
                } else {
                    for (int k = s0; k <= j; k++) v = fma(row[k], -U8[(j + 1) * PANEL_SUB + (k - s0)], v);
                }
                row[j + 1] = v;
                K av = amax_key(v);
                if (av > bv || bi == INT_MAX) { bv = av; bi = base + l; }
            }
        }
        // pending update of row values for columns c >= j+2 after column j:
        // inside the sub-panel the rank-1 from column j; at or beyond its edge
        // the sub-panel's rank-(j-s0+1) product (applied to the stored rows
        // only at the edge)
        auto pend = [&](const T *row, int c) -> T {
            if (c < s1) return fma(row[j], -U8[c * PANEL_SUB + (j - s0)], row[c]);
            T v = row[c];
            for (int k = s0; k <= j; k++) v = fma(row[k], -U8[c * PANEL_SUB + (k - s0)], v);
            return v;
        };
        if (more) {
            block_argmax<K>(bv, bi, red_v, red_i);
            // packages of column j+1: the candidate with every pending update;
            // row j+1 with the updates every stored row receives below
            stage_push(j + 1, bv, bi, [&](const T *row, int c, bool is_row) -> T {
                if (c <= j + 1) return row[c];
                if (is_row && !edge && c >= s1) return row[c];
                return pend(row, c);
            });
        }
        // updates of the stored rows (overlap the other CTAs' pushes): rank-1
        // on the sub-panel's remaining columns, or at the edge the whole
        // sub-panel on every column to its right
        const int c_lo = j + 2, c_hi = edge ? w : s1;
        if (c_lo < c_hi) {
            for (int l = ls + tid; l < nloc; l += PANEL_THREADS) {
                const int g = base + l;
                if (g == j + 1) continue;   // replaced by the next pivot row or the old row j+1
                T *row = rows + l * WP;
                if (!edge) {
                    const T lv = row[j];
                    for (int c = c_lo; c < c_hi; c++) row[c] = fma(lv, -U8[c * PANEL_SUB + (j - s0)], row[c]);
                } else {
                    T lk[PANEL_SUB];
#pragma unroll
                    for (int k = 0; k < PANEL_SUB; k++) lk[k] = (s0 + k <= j) ? row[s0 + k] : T(0);
                    for (int c = c_lo; c < c_hi; c++) {
                        T u[PANEL_SUB];
                        ld8(U8 + c * PANEL_SUB, u);
                        T v = row[c];
#pragma unroll
                        for (int k = 0; k < PANEL_SUB; k++) v = fma(lk[k], -u[k], v);
                        row[c] = v;
                    }
                }
            }
        }
    }
    if (failed && tid == 0) atomicExch(a.err, 1);
    // every package sent to this CTA has landed (it waited for all of them),
    // and no CTA leaves before all have
    cluster.sync();
    if (rank == 0)
        for (int c = tid; c < kmax; c += PANEL_THREADS) a.piv[c] = spiv[c];
    if (a.inv && rank == 0) {
        // inverse of the unit-lower L11 (rows 0..kmax-1 are this CTA's first
        // rows): warp v forms columns v, v+16, .. by forward substitution, the
        // lanes owning rows lane and lane+32; the column's solved entry y_k is
        // broadcast with a shuffle
        const int wv = tid >> 5;
        for (int c0 = wv; c0 < TRI_TB; c0 += PANEL_THREADS / 32) {
            T y0 = (lane == c0) ? T(1) : T(0), y1 = (lane + 32 == c0) ? T(1) : T(0);
            if (c0 < kmax) {
                for (int k = c0; k < kmax - 1; k++) {
                    const T yk = __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, k & 31);
                    if (lane > k && lane < kmax) y0 = fma(-rows[lane * WP + k], yk, y0);
                    if (lane + 32 > k && lane + 32 < kmax) y1 = fma(-rows[(lane + 32) * WP + k], yk, y1);
                }
            } else {
                y0 = y1 = T(0);
            }
            a.inv[lane * TRI_TB + c0] = lane < kmax ? y0 : T(0);
            a.inv[(lane + 32) * TRI_TB + c0] = lane + 32 < kmax ? y1 : T(0);
        }
    }
    for (int e = tid; e < nloc * w; e += PANEL_THREADS) {
        int l = e / w, c = e % w;
        a.P[(i64)(base + l) * a.rs + (i64)c * a.cs] = rows[l * WP + c];
    }
    for (int l = tid; l < nloc; l += PANEL_THREADS) {
        if (origin[l] != base + l) {
            int k = atomicAdd(a.touch_count, 1);
            a.touch_rows[k] = base + l;
            a.touch_src[k] = origin[l];
        }
    }
}

// ------------------------------------------------------------------ tournament pivoting
//
// k_panel_calu: the same panel with communication-avoiding pivoting (CALU,
// tournament pivoting), for the FP32 factorizations of the mixed-precision
// solvers, whose pivots only have to be good, not DDLA's (FP64 refinement
// makes the solution FP64-accurate; the solve report gives the agreement with
// partial pivoting).  Each CTA selects w candidate rows by partial pivoting on
// its own rows, with no cluster traffic per column; groups of 4 CTAs then
// merge their candidates (partial pivoting on the candidates' original rows)
// until one set of w winners remains, in pivot order, with the LU of their
// block.  The panel is then the no-pivot LU of the permuted rows: every other
// row becomes a row of L21 = A21 U11^-1.  A cluster barrier separates the
// levels, so a panel costs a few barriers instead of one per column.

constexpr int CALU_LEVELS = 3;   // local, groups of 4, groups of 16 (16 CTAs at most)
constexpr int CALU_INTS = CALU_LEVELS * PANEL_MAXCS * PANEL_WMAX + CALU_LEVELS * PANEL_MAXCS + 64;

struct CaluSmem {
    size_t rows, org, merge, morg, ut, dinv, red, win, dtop, isw, total;
};

__host__ __device__ inline CaluSmem calu_smem_layout(int rp, int w) {
    CaluSmem L;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = (o + bytes + 15) & ~(size_t)15;
        return at;
    };
    L.rows = take(sizeof(float) * (size_t)rp * (w + 1));
    L.org = take(sizeof(int) * (size_t)rp);
    L.merge = take(sizeof(float) * (size_t)4 * w * (w + 1));
    L.morg = take(sizeof(int) * (size_t)4 * w);
    L.ut = take(sizeof(float) * (size_t)w * (w + 1));
    L.dinv = take(sizeof(float) * (size_t)w);
    L.red = take((sizeof(unsigned) + sizeof(int)) * (PANEL_THREADS / 32) + 16);
    L.win = take(sizeof(int) * (size_t)w);
    L.dtop = take(sizeof(int) * (size_t)w);
    L.isw = take((size_t)rp);
    L.total = o;
    return L;
}

// Partial-pivoting LU of the nr x w matrix M (row stride WP) in place; the
// rows carry their origins in org.  Pivot: the largest |x| (amax_key: NaN
// lowest), the lower row on ties.  A zero column keeps its first row as the
// pivot and is not scaled.
__device__ void calu_lu(float *M, int *org, int nr, int w, int WP, unsigned *red_v, int *red_i) {
    const int tid = threadIdx.x;
    const int kk = nr < w ? nr : w;
    for (int j = 0; j < kk; j++) {
        unsigned bv = 0;
        int bi = INT_MAX;
        for (int r = j + tid; r < nr; r += PANEL_THREADS) {
            const unsigned v = amax_key(M[r * WP + j]);
            if (v > bv || bi == INT_MAX) {
                bv = v;
                bi = r;
            }
        }
        block_argmax<unsigned>(bv, bi, red_v, red_i);
        const int p = bi == INT_MAX ? j : bi;
        if (p != j) {
            for (int c = tid; c < w; c += PANEL_THREADS) {
                const float t = M[j * WP + c];
                M[j * WP + c] = M[p * WP + c];
                M[p * WP + c] = t;
            }
            if (tid == 0) {
                const int t = org[j];
                org[j] = org[p];
                org[p] = t;
            }
        }
        __syncthreads();
        const float pv = M[j * WP + j];
        if (pv != 0.0f) {
            const float rinv = 1.0f / pv;
            for (int r = j + 1 + tid; r < nr; r += PANEL_THREADS) {
                float *row = M + r * WP;
                const float l = row[j] * rinv;
                row[j] = l;
                for (int c = j + 1; c < w; c++) row[c] = fmaf(-l, M[j * WP + c], row[c]);
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(PANEL_THREADS, 1) k_panel_calu(PanelArgs<float> a) {
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = a.w, WP = w + 1, rp = a.rows_per;
    const CaluSmem L = calu_smem_layout(rp, w);
    float *rows = (float *)(smem + L.rows), *merge = (float *)(smem + L.merge), *ut = (float *)(smem + L.ut);
    float *dinv = (float *)(smem + L.dinv);
    int *org = (int *)(smem + L.org), *morg = (int *)(smem + L.morg);
    int *win = (int *)(smem + L.win), *dtop = (int *)(smem + L.dtop);
    unsigned char *isw = smem + L.isw;
    unsigned *red_v = (unsigned *)(smem + L.red);
    int *red_i = (int *)(red_v + PANEL_THREADS / 32);
    int *cand = a.calu;                                            // [level][rank][64]
    int *ccnt = cand + CALU_LEVELS * PANEL_MAXCS * PANEL_WMAX;     // [level][rank]
    const int base = rank * rp;
    int nloc = a.m - base;
    nloc = nloc < 0 ? 0 : (nloc > rp ? rp : nloc);
    const int kmax = a.m < w ? a.m : w;
    auto ld = [&](int r, int c) { return a.P[(i64)r * a.rs + (i64)c * a.cs]; };

    // 1. local candidates
    for (int e = tid; e < nloc * w; e += PANEL_THREADS) rows[(e / w) * WP + e % w] = ld(base + e / w, e % w);
    for (int l = tid; l < nloc; l += PANEL_THREADS) org[l] = base + l;
    __syncthreads();
    calu_lu(rows, org, nloc, w, WP, red_v, red_i);
    {
        const int k0 = nloc < w ? nloc : w;
        for (int i = tid; i < k0; i += PANEL_THREADS) cand[rank * PANEL_WMAX + i] = org[i];
        if (tid == 0) ccnt[rank] = k0;
    }
    // 2. merges in groups of 4 until one CTA holds the winners
    const float *fin = rows;
    const int *finorg = org;
    int level = 0;
    for (int span = 1; span < CS; span *= 4, level++) {
        __threadfence();
        cluster.sync();
        if (rank % (4 * span) == 0) {
            int nr = 0;
            for (int q = 0; q < 4; q++) {
                const int src = rank + q * span;
                if (src >= CS) break;
                const int cnt = ((volatile int *)ccnt)[level * PANEL_MAXCS + src];
                const int *cl = cand + (level * PANEL_MAXCS + src) * PANEL_WMAX;
                for (int e = tid; e < cnt * w; e += PANEL_THREADS) {
                    const int r = e / w, c = e % w;
                    merge[(nr + r) * WP + c] = ld(((volatile int *)cl)[r], c);
                }
                for (int i = tid; i < cnt; i += PANEL_THREADS) morg[nr + i] = ((volatile int *)cl)[i];
                nr += cnt;
            }
            __syncthreads();
            calu_lu(merge, morg, nr, w, WP, red_v, red_i);
            const int kk = nr < w ? nr : w;
            for (int i = tid; i < kk; i += PANEL_THREADS)
                cand[((level + 1) * PANEL_MAXCS + rank) * PANEL_WMAX + i] = morg[i];
            if (tid == 0) ccnt[(level + 1) * PANEL_MAXCS + rank] = kk;
        }
        fin = merge;
        finorg = morg;
    }
    // 3. CTA 0: the winners' block, the interchanges as LAPACK-style swaps
    if (rank == 0) {
        for (int e = tid; e < kmax * w; e += PANEL_THREADS) ut[(e / w) * WP + e % w] = fin[(e / w) * WP + e % w];
        for (int j = tid; j < kmax; j += PANEL_THREADS) {
            win[j] = finorg[j];
            dtop[j] = -1;
        }
        __syncthreads();
        if (tid < kmax) {
            const float d = ut[tid * WP + tid];
            if (d == 0.0f) atomicMin(a.info, (int)(a.row_base + tid + 1));
            dinv[tid] = 1.0f / d;
        }
        if (warp == 0) {
            // slots 0..kmax-1 hold origins cur[]; rows moved below hold
            // (dorg, dpos); lane l owns slots / entries l and l + 32
            int cur0 = lane, cur1 = lane + 32;
            int dorg0 = -1, dorg1 = -1, dpos0 = 0, dpos1 = 0;
            int nd = 0;
            for (int j = 0; j < kmax; j++) {
                const int o = win[j];
                const unsigned hc0 = __ballot_sync(0xffffffffu, lane >= j && lane < kmax && cur0 == o);
                const unsigned hc1 = __ballot_sync(0xffffffffu, lane + 32 >= j && lane + 32 < kmax && cur1 == o);
                const unsigned hd0 = __ballot_sync(0xffffffffu, lane < nd && dorg0 == o);
                const unsigned hd1 = __ballot_sync(0xffffffffu, lane + 32 < nd && dorg1 == o);
                const int cj = __shfl_sync(0xffffffffu, j < 32 ? cur0 : cur1, j & 31);   // origin now in slot j
                int p;
                if (hc0) p = __ffs(hc0) - 1;
                else if (hc1) p = __ffs(hc1) - 1 + 32;
                else if (hd0) p = __shfl_sync(0xffffffffu, dpos0, __ffs(hd0) - 1);
                else if (hd1) p = __shfl_sync(0xffffffffu, dpos1, __ffs(hd1) - 1);
                else p = o;
                if (lane == 0) a.piv[j] = p - j;
                if (p != j) {
                    if (p < kmax) {
                        if (p < 32) { if (lane == p) cur0 = cj; }
                        else { if (lane == p - 32) cur1 = cj; }
                    } else if (hd0 | hd1) {
                        const int di = hd0 ? __ffs(hd0) - 1 : __ffs(hd1) - 1 + 32;
                        if (di < 32) { if (lane == di) dorg0 = cj; }
                        else { if (lane == di - 32) dorg1 = cj; }
                    } else {
                        if (nd < 32) { if (lane == nd) { dorg0 = cj; dpos0 = p; } }
                        else { if (lane == nd - 32) { dorg1 = cj; dpos1 = p; } }
                        nd++;
                    }
                    if (j < 32) { if (lane == j) cur0 = o; }
                    else { if (lane == j - 32) cur1 = o; }
                }
            }
            // displaced top rows: final positions; the touched-row list
            if (lane < nd) dtop[dorg0] = dpos0;
            if (lane + 32 < nd) dtop[dorg1] = dpos1;
            int tc = 0;
            for (int j = 0; j < kmax; j++)
                if (win[j] != j) {
                    if (lane == 0) {
                        a.touch_rows[tc] = j;
                        a.touch_src[tc] = win[j];
                    }
                    tc++;
                }
            for (int i = 0; i < nd; i++) {
                const int dor = __shfl_sync(0xffffffffu, i < 32 ? dorg0 : dorg1, i & 31);
                const int dps = __shfl_sync(0xffffffffu, i < 32 ? dpos0 : dpos1, i & 31);
                if (lane == 0) {
                    a.touch_rows[tc] = dps;
                    a.touch_src[tc] = dor;
                }
                tc++;
            }
            if (lane == 0) *a.touch_count = tc;
        }
        __syncthreads();
        if (a.inv) {
            // inverse of the unit-lower L11 (forward substitution per column)
            for (int c0 = warp; c0 < TRI_TB; c0 += PANEL_THREADS / 32) {
                float y0 = (lane == c0) ? 1.0f : 0.0f, y1 = (lane + 32 == c0) ? 1.0f : 0.0f;
                if (c0 < kmax) {
                    for (int k = c0; k < kmax - 1; k++) {
                        const float yk = __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, k & 31);
                        if (lane > k && lane < kmax) y0 = fmaf(-ut[lane * WP + k], yk, y0);
                        if (lane + 32 > k && lane + 32 < kmax) y1 = fmaf(-ut[(lane + 32) * WP + k], yk, y1);
                    }
                } else {
                    y0 = y1 = 0.0f;
                }
                a.inv[lane * TRI_TB + c0] = lane < kmax ? y0 : 0.0f;
                a.inv[(lane + 32) * TRI_TB + c0] = lane + 32 < kmax ? y1 : 0.0f;
            }
        }
    }
    cluster.sync();
    // 4. every CTA: the winners, the displaced rows' positions and U11 from
    // CTA 0; the original rows again (nothing of the panel is written before
    // the barrier below)
    if (rank != 0) {
        const float *ut0 = cluster.map_shared_rank(ut, 0);
        for (int e = tid; e < kmax * w; e += PANEL_THREADS) ut[(e / w) * WP + e % w] = ut0[(e / w) * WP + e % w];
        for (int j = tid; j < kmax; j += PANEL_THREADS) {
            win[j] = cluster.map_shared_rank(win, 0)[j];
            dtop[j] = cluster.map_shared_rank(dtop, 0)[j];
            dinv[j] = cluster.map_shared_rank(dinv, 0)[j];
        }
    }
    for (int e = tid; e < nloc * w; e += PANEL_THREADS) rows[(e / w) * WP + e % w] = ld(base + e / w, e % w);
    for (int l = tid; l < nloc; l += PANEL_THREADS) isw[l] = 0;
    __syncthreads();
    for (int j = tid; j < kmax; j += PANEL_THREADS) {
        const int o = win[j];
        if (o >= base && o < base + nloc) isw[o - base] = 1;
    }
    cluster.sync();
    // 5. L21 = A21 U11^-1 for the other rows, written to their final rows;
    // CTA 0 writes the winners' block
    for (int l = tid; l < nloc; l += PANEL_THREADS) {
        if (isw[l]) continue;
        const int o = base + l;
        const int dest = o < kmax ? dtop[o] : o;
        if (dest < kmax || dest >= a.m) continue;   // cannot happen: every displaced top row has a place
        float *x = rows + l * WP;
        for (int j = 0; j < kmax; j++) {
            const float lj = x[j] * dinv[j];
            x[j] = lj;
            for (int c = j + 1; c < w; c++) x[c] = fmaf(-lj, ut[j * WP + c], x[c]);
        }
        for (int c = 0; c < w; c++) a.P[(i64)dest * a.rs + (i64)c * a.cs] = x[c];
    }
    if (rank == 0)
        for (int e = tid; e < kmax * w; e += PANEL_THREADS)
            a.P[(i64)(e / w) * a.rs + (i64)(e % w) * a.cs] = ut[(e / w) * WP + e % w];
    // all DSMEM reads done before any CTA exits
    cluster.sync();
}

// Fallback for panels that do not fit in one cluster's shared memory: one CTA
// factors the panel in global memory (same arithmetic, same pivot rule).
template <typename T>
__global__ void __launch_bounds__(1024) k_panel_lu_global(PanelArgs<T> a, int *origin) {
    typedef typename KeyT<T>::type K;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ K red_v[32];
    __shared__ int red_i[32];
    __shared__ int s_p;
    for (int g = tid; g < a.m; g += 1024) origin[g] = g;
    if (tid == 0) *a.touch_count = 0;
    __syncthreads();
    auto at = [&](i64 r, i64 c) -> T & { return a.P[r * a.rs + c * a.cs]; };
    const int kmax = a.m < a.w ? a.m : a.w;
    for (int j = 0; j < kmax; j++) {
        K bv = 0;
        int bi = INT_MAX;
        for (int g = j + tid; g < a.m; g += 1024) {
            K v = amax_key(at(g, j));
            if (v > bv || bi == INT_MAX) { bv = v; bi = g; }
        }
        for (int off = 16; off > 0; off >>= 1) {
            K ov = __shfl_down_sync(0xffffffffu, bv, off);
            int oi = __shfl_down_sync(0xffffffffu, bi, off);
            if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
        }
        if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
        __syncthreads();
        if (tid == 0) {
            for (int q = 1; q < 32; q++)
                if (red_v[q] > bv || (red_v[q] == bv && red_i[q] < bi)) { bv = red_v[q]; bi = red_i[q]; }
            int p = bi == INT_MAX ? j : bi;
            s_p = p;
            a.piv[j] = p - j;
            if (p != j) { int t = origin[j]; origin[j] = origin[p]; origin[p] = t; }
        }
        __syncthreads();
        const int p = s_p;
        if (p != j)
            for (int c = tid; c < a.w; c += 1024) { T t = at(j, c); at(j, c) = at(p, c); at(p, c) = t; }
        __syncthreads();
        const T ujj = at(j, j);
        if (ujj == T(0)) {
            if (tid == 0) atomicMin(a.info, (int)(a.row_base + j + 1));
            break;
        }
        const T rinv = T(1) / ujj;
        for (int g = j + 1 + tid; g < a.m; g += 1024) {
            T lv = at(g, j) * rinv;
            at(g, j) = lv;
            for (int c = j + 1; c < a.w; c++) at(g, c) = fma(lv, -at(j, c), at(g, c));
        }
        __syncthreads();
    }
    __syncthreads();
    for (int g = tid; g < a.m; g += 1024)
        if (origin[g] != g) {
            int k = atomicAdd(a.touch_count, 1);
            a.touch_rows[k] = g;
            a.touch_src[k] = origin[g];
        }
}

// Gather-then-scatter of the touched rows for the columns outside the panel:
// columns c' in [0, ncols) map to c' (c' < skip0) or c' + skipw.
constexpr int LASWP_MAXT = 2 * PANEL_WMAX;
// With perm given, the last block applies the same interchanges to the
// permutation vector.
template <typename T>
__global__ void __launch_bounds__(256)
    k_laswp_list(T *X, i64 rs, i64 cs, i64 ncols, i64 skip0, i64 skipw, const int *count, const int *rows,
                 const int *src, int *perm) {
    __shared__ T tmp[LASWP_MAXT][32];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    if (perm && blockIdx.x == gridDim.x - 1) {
        __shared__ int tp[LASWP_MAXT];
        const int cnt = *count;
        for (int t = threadIdx.x; t < cnt; t += 256) tp[t] = perm[src[t]];
        __syncthreads();
        for (int t = threadIdx.x; t < cnt; t += 256) perm[rows[t]] = tp[t];
        return;
    }
    i64 cc = (i64)blockIdx.x * 32 + lane;
    const int cnt = *count;
    const bool ok = cc < ncols;
    i64 c = cc < skip0 ? cc : cc + skipw;
    for (int t = wp; t < cnt; t += 8)
        if (ok) tmp[t][lane] = X[(i64)src[t] * rs + c * cs];
    __syncthreads();
    for (int t = wp; t < cnt; t += 8)
        if (ok) X[(i64)rows[t] * rs + c * cs] = tmp[t][lane];
}

// Relative pivots -> permutation (perm[k] = source row of row k after the
// forward interchanges), one thread, permutation held in shared memory.
__global__ void k_piv_to_perm_smem(const int32_t *piv, i64 n, int *perm) {
    extern __shared__ int sp[];
    for (i64 i = threadIdx.x; i < n; i += blockDim.x) sp[i] = (int)i;
    __syncthreads();
    if (threadIdx.x == 0)
        for (i64 i = 0; i < n; i++) {
            i64 t = i + piv[i];
            if (t != i) { int x = sp[i]; sp[i] = sp[t]; sp[t] = x; }
        }
    __syncthreads();
    for (i64 i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}
__global__ void k_piv_to_perm_global(const int32_t *piv, i64 n, int *perm) {
    for (i64 i = 0; i < n; i++) perm[i] = (int)i;
    for (i64 i = 0; i < n; i++) {
        i64 t = i + piv[i];
        if (t != i) { int x = perm[i]; perm[i] = perm[t]; perm[t] = x; }
    }
}

// forward: Y[k] = X[perm[k]];  backward: Y[perm[k]] = X[k].  Y contiguous.
template <typename T>
__global__ void k_permute_rows(const T *X, i64 rs, i64 cs, i64 n, i64 ncol, const int *perm, bool forward, T *Y) {
    i64 tot = n * ncol;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        i64 k = e / ncol, c = e % ncol;
        if (forward) Y[k * ncol + c] = X[(i64)perm[k] * rs + c * cs];
        else Y[(i64)perm[k] * ncol + c] = X[k * rs + c * cs];
    }
}
template <typename T>
__global__ void k_copy_back(const T *Y, i64 n, i64 ncol, T *X, i64 rs, i64 cs) {
    i64 tot = n * ncol;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        i64 k = e / ncol, c = e % ncol;
        X[k * rs + c * cs] = Y[e];
    }
}

// ------------------------------------------------------------------ host side

namespace {
int g_max_cluster[2] = {0, 0};      // [double, float]
size_t g_panel_smem[2] = {0, 0};    // dynamic shared memory available to k_panel_lu<T>

template <typename T>
int max_cluster(ddla_handle h) {
    int &mc = g_max_cluster[sizeof(T) == 8 ? 0 : 1];
    if (mc) return mc;
    DDLA_CUDA(cudaFuncSetAttribute(k_panel_lu<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    size_t avail = 0;
    DDLA_TRY(max_dyn_smem((const void *)k_panel_lu<T>, h->smem_optin, &avail));
    g_panel_smem[sizeof(T) == 8 ? 0 : 1] = avail;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(PANEL_MAXCS);
    cfg.blockDim = dim3(PANEL_THREADS);
    cfg.dynamicSmemBytes = avail;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = PANEL_MAXCS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int cs = 0;
    if (cudaOccupancyMaxPotentialClusterSize(&cs, (const void *)k_panel_lu<T>, &cfg) != cudaSuccess || cs < 1) {
        cudaGetLastError();
        cs = 8;
    }
    int p2 = 1;
    while (p2 * 2 <= cs && p2 * 2 <= PANEL_MAXCS) p2 *= 2;
    mc = p2;
    return mc;
}
template <typename T>
size_t panel_smem_avail() { return g_panel_smem[sizeof(T) == 8 ? 0 : 1]; }

}  // namespace

// Widest panel (power of two, <= 64) whose m rows fit in one cluster.
template <typename T>
int panel_width_for(ddla_handle h, i64 m) {
    int cs = max_cluster<T>(h);
    if (cs <= 0) return 0;
    for (int w = PANEL_WMAX; w >= 8; w /= 2) {
        i64 rp = (m + cs - 1) / cs;
        if (panel_smem_layout<T>((int)rp, w).total <= panel_smem_avail<T>()) return w;
    }
    return 0;
}

// Factor the m x w panel at column pc of X (the m-row block of full rows) on
// stream s: relative pivots into d_piv[0..w) and the touched-row list into
// the WS_PIV scratch, which panel_swap_rest consumes.
template <typename T>
int tri_inverse_on(cudaStream_t s, bool lower, bool unit, View<const T> A, i64 n, T *inv);

// inv (optional, TRI_TB x TRI_TB): receives the inverse of the panel's
// unit-lower diagonal block L11 (zeros outside it), for the row-block solve.
// WS_PIV layout: two touched-row lists (count, rows, sources), selected by
// `slot`, so that the interchanges of panel k can still be applied while
// panel k+1 is being factored; then the origin scratch of the fallback kernel.
constexpr int TOUCH_INTS = 1 + 2 * LASWP_MAXT;

// The work between two panels of the look-ahead LU, for the columns of
// panel k+1, in one launch: panel k's row interchanges (its touched-row
// list), U12 = inv(L11) A12 and the rank-w0 update A22 -= L21 U12
// (LU.cs:334-360 for this block column).  F is panel k's top-left corner;
// its frame rows [0, m0) and frame columns [w0, w0 + w1) are the next
// panel's columns.  Nothing is written to F: the result (U12 in rows
// [0, w0), the updated rows below) goes to Tb (m0 x w1, row-major), from
// which panel k+1 loads its rows and copies U12 back.  So CTAs may gather
// any source row without racing each other's writes.  Every CTA forms U12
// itself (64^3 FMA) and updates 64 rows.
constexpr int NP_ROWS = 64, NP_LD = 68;   // 16-byte rows for float4 operand loads

// C (4 x 4 per thread, rows 4 ty.., columns 4 tx..) = sum_k AT[k][rows] B[k][cols]
__device__ __forceinline__ void np_tile(const float *AT, const float *B, int kn, int ty, int tx, float acc[4][4]) {
#pragma unroll 4
    for (int k = 0; k < kn; k++) {
        const float4 a = *reinterpret_cast<const float4 *>(AT + k * NP_LD + 4 * ty);
        const float4 b = *reinterpret_cast<const float4 *>(B + k * NP_LD + 4 * tx);
        const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
}

__global__ void __launch_bounds__(256) k_next_prep(const float *F, i64 rs, i64 cs, i64 m0, int w0, int w1,
                                                   const int *tcount, const int *trows, const int *tsrc,
                                                   const float *inv, float *Tb, int vec) {
    extern __shared__ __align__(16) unsigned char np_smem[];
    // A12[k][c], IvT[k][i] = inv(L11)[i][k], U12[k][c], L21T[k][l]; all ld NP_LD
    float *A12 = (float *)np_smem, *IvT = A12 + PANEL_WMAX * NP_LD, *U12 = IvT + PANEL_WMAX * NP_LD,
          *L21T = U12 + PANEL_WMAX * NP_LD;
    __shared__ i64 srcA[PANEL_WMAX], srcOwn[NP_ROWS];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const i64 r0 = w0 + (i64)blockIdx.x * NP_ROWS;
    const int nr = (int)(m0 - r0 < NP_ROWS ? (m0 - r0 > 0 ? m0 - r0 : 0) : NP_ROWS);
    if (tid < PANEL_WMAX) srcA[tid] = tid;
    if (tid >= 64 && tid < 64 + NP_ROWS) srcOwn[tid - 64] = r0 + (tid - 64);
    __syncthreads();
    const int cnt = *tcount;
    for (int t = tid; t < cnt; t += 256) {
        const i64 r = trows[t];
        if (r < w0) srcA[r] = tsrc[t];
        if (r >= r0 && r < r0 + NP_ROWS) srcOwn[r - r0] = tsrc[t];
    }
    __syncthreads();
    // operands (entries outside w0 / w1 / nr are zero), and the rows this
    // thread's 4 x 4 result is subtracted from, all loaded before any use:
    // with contiguous 16-byte aligned rows as float4 (4 chunks of each kind
    // per thread), else element by element
    float4 own[4];
    if (vec) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = tid + 256 * q, k = e >> 4, c4 = (e & 15) * 4;   // row k, columns c4 .. c4 + 3
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 a12 = k < w0 && c4 < w1 ? *reinterpret_cast<const float4 *>(F + srcA[k] * rs + w0 + c4) : z;
            const float4 iv = k < w0 ? *reinterpret_cast<const float4 *>(inv + k * TRI_TB + c4) : z;
            const float4 l21 = k < nr ? *reinterpret_cast<const float4 *>(F + (r0 + k) * rs + c4) : z;
            const int l = 4 * ty + q;
            own[q] = l < nr && 4 * tx < w1 ? *reinterpret_cast<const float4 *>(F + srcOwn[l] * rs + w0 + 4 * tx) : z;
            *reinterpret_cast<float4 *>(A12 + k * NP_LD + c4) = a12;
            const float ivv[4] = {iv.x, iv.y, iv.z, iv.w}, lv[4] = {l21.x, l21.y, l21.z, l21.w};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                IvT[(c4 + j) * NP_LD + k] = c4 + j < w0 ? ivv[j] : 0.f;   // IvT[c][k] = inv[k][c]
                L21T[(c4 + j) * NP_LD + k] = c4 + j < w0 ? lv[j] : 0.f;   // L21T[c][l = k]
            }
        }
    } else {
        for (int e = tid; e < PANEL_WMAX * PANEL_WMAX; e += 256) {
            const int k = e >> 6, c = e & 63;
            A12[k * NP_LD + c] = k < w0 && c < w1 ? F[srcA[k] * rs + (i64)(w0 + c) * cs] : 0.f;
            IvT[c * NP_LD + k] = k < w0 && c < w0 ? inv[k * TRI_TB + c] : 0.f;
            L21T[c * NP_LD + k] = k < nr && c < w0 ? F[(r0 + k) * rs + (i64)c * cs] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int l = 4 * ty + q;
            float o[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int c = 4 * tx + j;
                o[j] = l < nr && c < w1 ? F[srcOwn[l] * rs + (i64)(w0 + c) * cs] : 0.f;
            }
            own[q] = make_float4(o[0], o[1], o[2], o[3]);
        }
    }
    __syncthreads();
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
    np_tile(IvT, A12, w0, ty, tx, acc);   // U12 = inv(L11) A12
#pragma unroll
    for (int i = 0; i < 4; i++)
        *reinterpret_cast<float4 *>(U12 + (4 * ty + i) * NP_LD + 4 * tx) =
            make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    __syncthreads();
    if (blockIdx.x == 0)
        for (int e = tid; e < w0 * w1; e += 256) Tb[e] = U12[(e / w1) * NP_LD + e % w1];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
    np_tile(L21T, U12, w0, ty, tx, acc);   // L21 U12 for this CTA's rows
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int l = 4 * ty + i;
        if (l >= nr) continue;
        const float ov[4] = {own[i].x, own[i].y, own[i].z, own[i].w};
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = 4 * tx + j;
            if (c < w1) Tb[(r0 + l) * w1 + c] = ov[j] - acc[i][j];
        }
    }
}

int next_prep(ddla_handle h, cudaStream_t s, View<const float> F, i64 w0, i64 w1, int slot, const float *inv,
              float *Tb) {
    const i64 m0 = F.rows;
    int *tbuf;
    DDLA_TRY(workspace(h, WS_PIV, sizeof(int) * (size_t)(2 * TOUCH_INTS + m0 + CALU_INTS), (void **)&tbuf));
    tbuf += slot * TOUCH_INTS;
    const size_t smem = sizeof(float) * 4 * PANEL_WMAX * NP_LD;
    // float4 loads: unit column stride, 16-byte aligned rows (the next
    // panel's first column w0 and the row stride multiples of 4 elements)
    const bool vec = F.cs == 1 && F.rs % 4 == 0 && w0 % 4 == 0 && w1 % 4 == 0 && (((uintptr_t)F.p) & 15) == 0 &&
                     (((uintptr_t)inv) & 15) == 0;
    static bool attr = false;
    if (!attr) {
        DDLA_CUDA(cudaFuncSetAttribute(k_next_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    const i64 blocks = (m0 - w0 + NP_ROWS - 1) / NP_ROWS;
    k_next_prep<<<(unsigned)(blocks > 0 ? blocks : 1), 256, smem, s>>>(F.p, F.rs, F.cs, m0, (int)w0, (int)w1,
                                                                          tbuf, tbuf + 1, tbuf + 1 + LASWP_MAXT,
                                                                          inv, Tb, vec ? 1 : 0);
    DDLA_LAUNCHED();
    return 0;
}

// True when an m-row panel of width w runs on the cluster kernel k_panel_lu
// (the only panel kernel that takes a PanelLoad).
template <typename T>
bool panel_fused_ok(ddla_handle h, i64 m, int w) {
    int cs = max_cluster<T>(h);
    if (cs <= 0 || w > PANEL_WMAX) return false;
    if (sizeof(T) == 4 && tune_get("panel.calu", 0) != 0) return false;
    const int64_t want = tune_get("panel.cluster", 0);
    if (want > 0 && want < cs) cs = (int)want;
    const size_t avail = panel_smem_avail<T>();
    int use = 1;
    while (use < cs && ((m + use - 1) / use > 512 || panel_smem_layout<T>((int)((m + use - 1) / use), w).total > avail))
        use *= 2;
    return panel_smem_layout<T>((int)((m + use - 1) / use), w).total <= avail;
}

template <typename T>
int panel_factor(ddla_handle h, cudaStream_t s, View<T> X, i64 pc, int w, int32_t *d_piv, i64 row_base,
                 int *d_info, T *inv, int slot, const PanelLoad<T> *pl) {
    const i64 m = X.rows;
    int *tbuf;
    DDLA_TRY(workspace(h, WS_PIV, sizeof(int) * (size_t)(2 * TOUCH_INTS + m + CALU_INTS), (void **)&tbuf));
    int *origin = tbuf + 2 * TOUCH_INTS;
    int *calu = origin + m;
    tbuf += slot * TOUCH_INTS;
    int *tcount = tbuf, *trows = tbuf + 1, *tsrc = tbuf + 1 + LASWP_MAXT;
    PanelArgs<T> a;
    a.P = X.p + pc * X.cs;
    a.rs = X.rs;
    a.cs = X.cs;
    a.m = (int)m;
    a.w = w;
    a.piv = d_piv;
    a.info = d_info;
    a.row_base = row_base;
    a.touch_count = tcount;
    a.touch_rows = trows;
    a.touch_src = tsrc;
    a.inv = inv;
    a.calu = calu;
    a.err = h->d_info + INFO_TIMEOUT;
    a.ld = pl ? pl->ld : nullptr;
    a.ld_rs = pl ? pl->ld_rs : 0;
    a.ld_cs = pl ? pl->ld_cs : 0;
    a.u12_src = pl ? pl->u12_src : nullptr;
    a.u12_dst = pl ? pl->u12_dst : nullptr;
    a.u12_rows = pl ? pl->u12_rows : 0;
    if (pl && !panel_fused_ok<T>(h, m, w)) {
        set_error("panel_lu: an out-of-place panel load needs the cluster panel");
        return DDLA_ERR_UNSUPPORTED;
    }
    int cs = max_cluster<T>(h);
    if (cs <= 0) return cs < 0 ? cs : DDLA_ERR_UNSUPPORTED;
    const int64_t want = tune_get("panel.cluster", 0);
    if (want > 0 && want < cs) cs = (int)want;
    const size_t avail = panel_smem_avail<T>();
    if constexpr (sizeof(T) == 4) {
        // tournament pivoting for the FP32 factorizations (tuning key panel.calu)
        if (tune_get("panel.calu", 0) != 0 && w <= PANEL_WMAX) {
            int use = 1;
            while (use < cs && ((m + use - 1) / use > 512 || calu_smem_layout((int)((m + use - 1) / use), w).total > avail))
                use *= 2;
            const i64 rp = (m + use - 1) / use;
            const size_t smem = calu_smem_layout((int)rp, w).total;
            if (smem <= avail) {
                static bool attr = false;
                if (!attr) {
                    DDLA_CUDA(cudaFuncSetAttribute(k_panel_calu, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
                    DDLA_CUDA(cudaFuncSetAttribute(k_panel_calu, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)avail));
                    attr = true;
                }
                a.rows_per = (int)rp;
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(use);
                cfg.blockDim = dim3(PANEL_THREADS);
                cfg.dynamicSmemBytes = smem;
                cfg.stream = s;
                cudaLaunchAttribute attr1[1];
                attr1[0].id = cudaLaunchAttributeClusterDimension;
                attr1[0].val.clusterDim.x = use;
                attr1[0].val.clusterDim.y = 1;
                attr1[0].val.clusterDim.z = 1;
                cfg.attrs = attr1;
                cfg.numAttrs = 1;
                DDLA_CUDA(cudaLaunchKernelEx(&cfg, k_panel_calu, a));
                DDLA_LAUNCHED();
                return 0;
            }
        }
    }
    // smallest cluster that holds the rows with at most 512 rows per CTA
    int use = 1;
    while (use < cs && ((m + use - 1) / use > 512 ||
                        panel_smem_layout<T>((int)((m + use - 1) / use), w).total > avail))
        use *= 2;
    i64 rp = (m + use - 1) / use;
    size_t smem = panel_smem_layout<T>((int)rp, w).total;
    if (w <= PANEL_WMAX && smem <= avail) {
        a.rows_per = (int)rp;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(use);
        cfg.blockDim = dim3(PANEL_THREADS);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = use;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        DDLA_CUDA(cudaLaunchKernelEx(&cfg, k_panel_lu<T>, a));
        DDLA_LAUNCHED();
    } else {
        if (w > PANEL_WMAX) { set_error("panel_lu: panel wider than 64"); return DDLA_ERR_UNSUPPORTED; }
        a.rows_per = (int)m;
        k_panel_lu_global<T><<<1, 1024, 0, s>>>(a, origin);
        DDLA_LAUNCHED();
        if (inv) {
            const i64 k = m < w ? m : w;
            DDLA_TRY(tri_inverse_on<T>(s, true, true, View<const T>{X.p + pc * X.cs, k, k, X.rs, X.cs}, k, inv));
        }
    }
    return 0;
}

// Apply the interchanges of the panel factored with `slot` to the columns
// c' of the rows of X, for c' in [0, ncols) mapped to c' (c' < skip0) or
// c' + skipw, and to the permutation vector (if given), on the handle's stream.
template <typename T>
int panel_swap_cols(ddla_handle h, View<T> X, i64 ncols, i64 skip0, i64 skipw, int *perm, int slot) {
    cudaStream_t s = h->stream;
    int *tbuf;
    DDLA_TRY(workspace(h, WS_PIV, sizeof(int) * (size_t)(2 * TOUCH_INTS + X.rows), (void **)&tbuf));
    tbuf += slot * TOUCH_INTS;
    int *tcount = tbuf, *trows = tbuf + 1, *tsrc = tbuf + 1 + LASWP_MAXT;
    unsigned grid = (unsigned)((ncols > 0 ? ncols + 31 : 0) / 32) + (perm ? 1u : 0u);
    if (grid > 0) {
        // the permutation vector, when given, rides along in one more block
        k_laswp_list<T><<<grid, 256, 0, s>>>(X.p, X.rs, X.cs, ncols > 0 ? ncols : 0, skip0, skipw, tcount, trows,
                                             tsrc, perm);
        DDLA_LAUNCHED();
    }
    return 0;
}

// All columns of X outside the panel at pc (width w).
template <typename T>
int panel_swap_rest(ddla_handle h, View<T> X, i64 pc, int w, int *perm, int slot) {
    return panel_swap_cols<T>(h, X, X.cols - w, pc, w, perm, slot);
}

// Y[k] = X[perm[k]] for the rows of B (forward) using a precomputed
// permutation.
template <typename T>
int permute_rows(ddla_handle h, View<T> B, const int *perm, i64 n, bool forward) {
    if (n == 0 || B.cols == 0) return 0;
    cudaStream_t s = h->stream;
    T *tmp;
    DDLA_TRY(workspace(h, WS_TMP, sizeof(T) * (size_t)n * B.cols, (void **)&tmp));
    i64 tot = n * B.cols;
    int blocks = (int)((tot + 255) / 256 < 8192 ? (tot + 255) / 256 : 8192);
    k_permute_rows<T><<<blocks, 256, 0, s>>>(B.p, B.rs, B.cs, n, B.cols, perm, forward, tmp);
    DDLA_LAUNCHED();
    k_copy_back<T><<<blocks, 256, 0, s>>>(tmp, n, B.cols, B.p, B.rs, B.cs);
    DDLA_LAUNCHED();
    return 0;
}

template <typename T>
int apply_perm(ddla_handle h, View<T> B, const int32_t *d_piv, i64 n, bool forward) {
    if (n == 0 || B.cols == 0) return 0;
    cudaStream_t s = h->stream;
    int *perm;
    T *tmp;
    DDLA_TRY(workspace(h, WS_MISC, sizeof(int) * (size_t)n, (void **)&perm));
    DDLA_TRY(workspace(h, WS_TMP, sizeof(T) * (size_t)n * B.cols, (void **)&tmp));
    size_t sm = sizeof(int) * (size_t)n;
    size_t avail = 0;
    DDLA_TRY(max_dyn_smem((const void *)k_piv_to_perm_smem, h->smem_optin, &avail));
    if (sm <= avail) {
        k_piv_to_perm_smem<<<1, 256, sm, s>>>(d_piv, n, perm);
    } else {
        k_piv_to_perm_global<<<1, 1, 0, s>>>(d_piv, n, perm);
    }
    DDLA_LAUNCHED();
    i64 tot = n * B.cols;
    int blocks = (int)((tot + 255) / 256 < 8192 ? (tot + 255) / 256 : 8192);
    k_permute_rows<T><<<blocks, 256, 0, s>>>(B.p, B.rs, B.cs, n, B.cols, perm, forward, tmp);
    DDLA_LAUNCHED();
    k_copy_back<T><<<blocks, 256, 0, s>>>(tmp, n, B.cols, B.p, B.rs, B.cs);
    DDLA_LAUNCHED();
    return 0;
}

template int panel_width_for<double>(ddla_handle, i64);
template int panel_width_for<float>(ddla_handle, i64);
template int panel_factor<double>(ddla_handle, cudaStream_t, View<double>, i64, int, int32_t *, i64, int *,
                                  double *, int, const PanelLoad<double> *);
template int panel_factor<float>(ddla_handle, cudaStream_t, View<float>, i64, int, int32_t *, i64, int *, float *,
                                 int, const PanelLoad<float> *);
template bool panel_fused_ok<float>(ddla_handle, i64, int);
template bool panel_fused_ok<double>(ddla_handle, i64, int);
template int panel_swap_rest<double>(ddla_handle, View<double>, i64, int, int *, int);
template int panel_swap_rest<float>(ddla_handle, View<float>, i64, int, int *, int);
template int panel_swap_cols<double>(ddla_handle, View<double>, i64, i64, i64, int *, int);
template int panel_swap_cols<float>(ddla_handle, View<float>, i64, i64, i64, int *, int);
template int permute_rows<double>(ddla_handle, View<double>, const int *, i64, bool);
template int permute_rows<float>(ddla_handle, View<float>, const int *, i64, bool);
template int apply_perm<double>(ddla_handle, View<double>, const int32_t *, i64, bool);
template int apply_perm<float>(ddla_handle, View<float>, const int32_t *, i64, bool);

}  // namespace ddla
