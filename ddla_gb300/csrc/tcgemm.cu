// Tensor-core (tcgen05) GEMMs with FP32 accumulation in TMEM.
//
// gemm_tc: C = alpha * A * B + beta * C for FP32 operands with FP32-level
// accuracy from split products on the 5th-generation tensor cores:
//   3xTF32  x = hi + lo with hi = tf32(x), lo = tf32(x - hi);
//           A*B ~ hi*hi + hi*lo + lo*hi   (kind::tf32)
// The split is done on the fly while the operand tiles are staged into shared
// memory in the canonical K-major core-matrix layout (8 rows x 16 bytes per
// core matrix, no swizzle).  One elected thread issues the tcgen05.mma chain
// for a 128 x 64 output tile; the FP32 accumulator lives in TMEM (64 columns)
// and is read back with tcgen05.ld for the alpha/beta epilogue.  Every
// mbarrier wait is bounded: on timeout the kernel records the error, waits
// (bounded) for its own MMAs and frees its TMEM.
//
// gemm_ozaki: FP64 GEMM with FP64-level accuracy from BF16 slice products on
// the same kind of kernel (see the comment at its definition).
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>

#include "common.cuh"

namespace ddla {
namespace {

constexpr int TM = 128;          // tile rows (TMEM lanes)
constexpr int TN = 64;           // tile columns (TMEM columns)
constexpr int TK = 64;           // K elements staged per chunk
constexpr int TC_THREADS = 256;
constexpr long long TC_SPIN = 1LL << 24;

// bytes of one staged operand tile (rows x TK fp32)
constexpr int A_BYTES = TM * TK * 4;
constexpr int B_BYTES = TN * TK * 4;
constexpr int LBO = 128;                 // next 16-byte K chunk: next core matrix
constexpr int SBO = (TK / 4) * 128;      // next 8-row group

__device__ __forceinline__ unsigned su32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) of a K-major fp32 tile in core-matrix layout
__device__ __forceinline__ int cm_off(int r, int k) {
    return (r >> 3) * SBO + (k >> 2) * LBO + (r & 7) * 16 + (k & 3) * 4;
}

__device__ __forceinline__ float tf32_round(float x) {
    unsigned u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;   // inf / nan unchanged
    u = (u + 0x1000u) & 0xffffe000u;
    return __uint_as_float(u);
}

// smem matrix descriptor: start, LBO, SBO (16-byte units), version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(unsigned addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3ffff) >> 4);
    d |= (uint64_t)(LBO >> 4) << 16;
    d |= (uint64_t)(SBO >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor: D f32, A/B format `fmt` (tf32 = 2, bf16 = 1), both
// K-major, N = TN, M = TM
__host__ __device__ constexpr uint32_t idesc(uint32_t fmt) {
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(unsigned tmem, uint64_t a, uint64_t b, uint32_t id, int acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned mbar, unsigned phase) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(phase)
        : "memory");
    return ok != 0;
}

struct TcArgs {
    int64_t m, n, k;
    float alpha, beta;
    const float *A;
    int64_t rsa, csa;
    const float *B;
    int64_t rsb, csb;
    float *C;
    int64_t rsc, csc;
    int uplo;
    int *err;
};

__global__ void __launch_bounds__(TC_THREADS) k_tc_tf32x3(TcArgs g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *Ah = smem, *Al = smem + A_BYTES, *Bh = smem + 2 * A_BYTES, *Bl = Bh + B_BYTES;
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ unsigned tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t m0 = (int64_t)blockIdx.y * TM, n0 = (int64_t)blockIdx.x * TN;
    if (g.uplo == DDLA_LOWER && n0 > m0 + TM - 1) return;
    if (g.uplo == DDLA_UPPER && m0 > n0 + TN - 1) return;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_slot)),
                     "r"(TN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_slot;
    const uint32_t id = idesc(2);
    unsigned phase = 0;
    bool failed = false;
    const bool a_vec = (g.csa == 1) && ((g.rsa & 3) == 0) && ((((uintptr_t)g.A) & 15) == 0);

    for (int64_t k0 = 0; k0 < g.k; k0 += TK) {
        // stage A (TM x TK): 16-byte chunks of a row
        for (int e = tid; e < TM * (TK / 4); e += TC_THREADS) {
            const int r = e / (TK / 4), c = e % (TK / 4);
            const int64_t gr = m0 + r, gk = k0 + 4 * c;
            float v[4];
            if (a_vec && gr < g.m && gk + 3 < g.k) {
                float4 q = *reinterpret_cast<const float4 *>(g.A + gr * g.rsa + gk);
                v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
            } else {
#pragma unroll
                for (int t = 0; t < 4; t++)
                    v[t] = (gr < g.m && gk + t < g.k) ? g.A[gr * g.rsa + (gk + t) * g.csa] : 0.f;
            }
            float4 hi, lo;
            float *ph = &hi.x, *pl = &lo.x;
#pragma unroll
            for (int t = 0; t < 4; t++) {
                ph[t] = tf32_round(v[t]);
                pl[t] = tf32_round(v[t] - ph[t]);
            }
            *reinterpret_cast<float4 *>(Ah + cm_off(r, 4 * c)) = hi;
            *reinterpret_cast<float4 *>(Al + cm_off(r, 4 * c)) = lo;
        }
        // stage B as N-rows x K (B is K x N in memory): element (n, k) = B[k][n]
        for (int e = tid; e < TN * TK; e += TC_THREADS) {
            const int kk = e / TN, nn = e % TN;
            const int64_t gk = k0 + kk, gn = n0 + nn;
            const float v = (gk < g.k && gn < g.n) ? g.B[gk * g.rsb + gn * g.csb] : 0.f;
            const float h = tf32_round(v);
            *reinterpret_cast<float *>(Bh + cm_off(nn, kk)) = h;
            *reinterpret_cast<float *>(Bl + cm_off(nn, kk)) = tf32_round(v - h);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int s = 0; s < TK / 8; s++) {
                const unsigned off_a = s * 2 * LBO, off_b = s * 2 * LBO;
                const uint64_t ah = sdesc(su32(Ah) + off_a), al = sdesc(su32(Al) + off_a);
                const uint64_t bh = sdesc(su32(Bh) + off_b), bl = sdesc(su32(Bl) + off_b);
                const int first = (k0 == 0 && s == 0) ? 0 : 1;
                mma_tf32(tmem, ah, bh, id, first);
                mma_tf32(tmem, ah, bl, id, 1);
                mma_tf32(tmem, al, bh, id, 1);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             su32(&mbar))
                         : "memory");
        }
        // wait for the MMAs (bounded) before the tiles are overwritten / read
        bool ok = false;
        for (long long it = 0; it < TC_SPIN; it++)
            if (mbar_try(su32(&mbar), phase)) { ok = true; break; }
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {   // uniform across the CTA
            failed = true;
            if (tid == 0) atomicExch(g.err, 1);
            break;
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!failed && g.k > 0) {
        // epilogue: warp w reads TMEM lanes 32*(w%4).., columns 32*(w/4)..
        const int q = warp & 3, h = warp >> 2;
        uint32_t d[32];
        const unsigned taddr = tmem + ((unsigned)(32 * q) << 16) + (unsigned)(32 * h);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]),
              "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]),
              "=r"(d[15]), "=r"(d[16]), "=r"(d[17]), "=r"(d[18]), "=r"(d[19]), "=r"(d[20]), "=r"(d[21]),
              "=r"(d[22]), "=r"(d[23]), "=r"(d[24]), "=r"(d[25]), "=r"(d[26]), "=r"(d[27]), "=r"(d[28]),
              "=r"(d[29]), "=r"(d[30]), "=r"(d[31])
            : "r"(taddr)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        // stage the tile row-major in the (now idle) operand buffer, then update
        // C with coalesced accesses: a warp covers 128 consecutive bytes of a row
        constexpr int SLD = TN + 4;
        float *stage = reinterpret_cast<float *>(smem);
        {
            float *row = stage + (32 * q + lane) * SLD + 32 * h;
#pragma unroll
            for (int j = 0; j < 32; j += 4)
                *reinterpret_cast<float4 *>(row + j) =
                    make_float4(__uint_as_float(d[j]), __uint_as_float(d[j + 1]), __uint_as_float(d[j + 2]),
                                __uint_as_float(d[j + 3]));
        }
        __syncthreads();
        const bool c_vec = (g.csc == 1) && ((g.rsc & 3) == 0) && ((((uintptr_t)g.C) & 15) == 0) &&
                           (n0 + TN <= g.n) && g.uplo == DDLA_DENSE;
        if (c_vec) {
            for (int e = tid; e < TM * (TN / 4); e += TC_THREADS) {
                const int r = e / (TN / 4), c4 = (e % (TN / 4)) * 4;
                const int64_t gr = m0 + r;
                if (gr >= g.m) continue;
                float4 acc = *reinterpret_cast<const float4 *>(stage + r * SLD + c4);
                float4 *cp = reinterpret_cast<float4 *>(g.C + gr * g.rsc + n0 + c4);
                float4 o;
                if (g.beta == 0.f) {
                    o = make_float4(g.alpha * acc.x, g.alpha * acc.y, g.alpha * acc.z, g.alpha * acc.w);
                } else {
                    float4 cv = *cp;
                    o = make_float4(fmaf(g.beta, cv.x, g.alpha * acc.x), fmaf(g.beta, cv.y, g.alpha * acc.y),
                                    fmaf(g.beta, cv.z, g.alpha * acc.z), fmaf(g.beta, cv.w, g.alpha * acc.w));
                }
                *cp = o;
            }
        } else {
            for (int e = tid; e < TM * TN; e += TC_THREADS) {
                const int r = e / TN, c = e % TN;
                const int64_t gr = m0 + r, gc = n0 + c;
                if (gr >= g.m || gc >= g.n) continue;
                if (g.uplo == DDLA_LOWER && gc > gr) continue;
                if (g.uplo == DDLA_UPPER && gc < gr) continue;
                float *cp = g.C + gr * g.rsc + gc * g.csc;
                const float v = g.alpha * stage[r * SLD + c];
                *cp = (g.beta == 0.f) ? v : fmaf(g.beta, *cp, v);
            }
        }
    } else if (g.k <= 0) {
        // C = beta * C
        for (int e = tid; e < TM * TN; e += TC_THREADS) {
            const int64_t gr = m0 + e / TN, gc = n0 + e % TN;
            if (gr >= g.m || gc >= g.n) continue;
            if (g.uplo == DDLA_LOWER && gc > gr) continue;
            if (g.uplo == DDLA_UPPER && gc < gr) continue;
            float *cp = g.C + gr * g.rsc + gc * g.csc;
            *cp = (g.beta == 0.f) ? 0.f : g.beta * *cp;
        }
    }
    if (failed) {
        // our MMAs may still run: wait (bounded) before giving TMEM back
        for (long long it = 0; it < TC_SPIN; it++)
            if (mbar_try(su32(&mbar), phase ^ 1u)) break;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TN) : "memory");
    }
}

constexpr size_t TC_SMEM = 2 * A_BYTES + 2 * B_BYTES;

// ------------------------------------------------------------------ rank-64 update, split products
//
// C += alpha * A * B for K <= 64 (the trailing updates of the FP32
// factorizations) on the tensor cores, with FP32 operands split once into two
// parts x = hi + lo packed per 128-row (128-column) tile in the core-matrix
// layout the MMA reads (k_tc_pack):
//   3xTF32  hi = tf32(x), lo = tf32(x - hi); 8 k-steps of kind::tf32 (K = 8)
//   3xBF16  hi = bf16(x), lo = bf16(x - hi); 4 k-steps of kind::f16 (K = 16)
// and A*B ~ hi*hi + hi*lo + lo*hi accumulated in FP32 in TMEM.  Both splits
// move 32 bytes of K per k-step, so the shared-memory descriptors differ only
// in the distance between 8-row core-matrix groups (TK * element size * 8).
// A persistent kernel walks the 128 x 128 tiles of C with every data movement
// asynchronous:
//   * the four operand tiles arrive by bulk copy on one mbarrier, and the next
//     tile's copies start as soon as the current MMAs are done;
//   * the C tile is loaded with coalesced float4 loads (a warp per 512-byte
//     row) before the MMAs are issued and parked in a shared staging tile S
//     while they run;
//   * one thread issues the k-steps x 3 MMAs into a 128-column TMEM
//     accumulator;
//   * each thread adds alpha * (its TMEM row) into S, and S goes back to C
//     with coalesced float4 stores.
// C views that are not 16-byte aligned (or have a column stride) take scalar
// loads and stores.  Every mbarrier wait is bounded as in k_tc_tf32x3.
constexpr int UT = 128;                       // tile rows = tile columns
constexpr int UT_SLD = UT + 4;                // staging tile row (floats)

template <bool BF> struct UtSplit {
    static constexpr int ESZ = BF ? 2 : 4;                       // bytes per packed element
    static constexpr int PART = UT * TK * ESZ;                   // bytes of one packed operand part
    static constexpr int SBO = (TK / (16 / ESZ)) * 128;          // next 8-row core-matrix group
    static constexpr int KSTEPS = TK * ESZ / 32;                 // MMAs of 32 bytes of K each
    static constexpr size_t OPS = 4 * (size_t)PART;
    static constexpr size_t SMEM = OPS + (size_t)UT * UT_SLD * 4;
    // D f32, A / B tf32 (2) or bf16 (1), both K-major, N = M = 128
    static constexpr uint32_t IDESC =
        (1u << 4) | ((BF ? 1u : 2u) << 7) | ((BF ? 1u : 2u) << 10) | ((uint32_t)(UT >> 3) << 17) |
        ((uint32_t)(UT >> 4) << 24);
};

__device__ __forceinline__ uint64_t sdesc_sbo(unsigned addr, int sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3ffff) >> 4);
    d |= (uint64_t)(LBO >> 4) << 16;
    d |= (uint64_t)(sbo >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

template <bool BF>
__device__ __forceinline__ void mma_split(unsigned tmem, uint64_t a, uint64_t b, uint32_t id, int acc) {
    if constexpr (BF) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(a), "l"(b), "r"(id), "r"(acc)
            : "memory");
    } else {
        mma_tf32(tmem, a, b, id, acc);
    }
}

// rows r of X (rows x kdim, strides rs / cs) -> packed [tile][hi | lo][UT x TK]
// in the core-matrix layout (16-byte rows of 4 tf32 or 8 bf16 values); rows
// beyond `rows` and k beyond kdim are zero
template <bool BF>
__global__ void k_tc_pack(const float *X, i64 rs, i64 cs, i64 rows, int kdim, unsigned char *out, i64 tiles) {
    typedef UtSplit<BF> S;
    constexpr int PER = 16 / S::ESZ;   // elements per 16-byte core-matrix row
    const i64 tot = tiles * UT * (TK / PER);
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        const i64 tile = e / (UT * (TK / PER));
        const int rem = (int)(e % (UT * (TK / PER))), r = rem / (TK / PER), k0 = (rem % (TK / PER)) * PER;
        const i64 gr = tile * UT + r;
        unsigned char *base = out + tile * 2 * S::PART;
        const int off = (r >> 3) * S::SBO + (k0 / PER) * LBO + (r & 7) * 16;
        if constexpr (BF) {
            unsigned short hi[8], lo[8];
#pragma unroll
            for (int x = 0; x < 8; x++) {
                const float v = (gr < rows && k0 + x < kdim) ? X[gr * rs + (i64)(k0 + x) * cs] : 0.f;
                const __nv_bfloat16 h = __float2bfloat16_rn(v);
                hi[x] = __bfloat16_as_ushort(h);
                lo[x] = __bfloat16_as_ushort(__float2bfloat16_rn(v - __bfloat162float(h)));
            }
            uint4 qh, ql;
            qh.x = hi[0] | ((unsigned)hi[1] << 16); qh.y = hi[2] | ((unsigned)hi[3] << 16);
            qh.z = hi[4] | ((unsigned)hi[5] << 16); qh.w = hi[6] | ((unsigned)hi[7] << 16);
            ql.x = lo[0] | ((unsigned)lo[1] << 16); ql.y = lo[2] | ((unsigned)lo[3] << 16);
            ql.z = lo[4] | ((unsigned)lo[5] << 16); ql.w = lo[6] | ((unsigned)lo[7] << 16);
            *reinterpret_cast<uint4 *>(base + off) = qh;
            *reinterpret_cast<uint4 *>(base + S::PART + off) = ql;
        } else {
            float hi[4], lo[4];
#pragma unroll
            for (int x = 0; x < 4; x++) {
                const float v = (gr < rows && k0 + x < kdim) ? X[gr * rs + (i64)(k0 + x) * cs] : 0.f;
                hi[x] = tf32_round(v);
                lo[x] = tf32_round(v - hi[x]);
            }
            *reinterpret_cast<float4 *>(base + off) = make_float4(hi[0], hi[1], hi[2], hi[3]);
            *reinterpret_cast<float4 *>(base + S::PART + off) = make_float4(lo[0], lo[1], lo[2], lo[3]);
        }
    }
}

struct TuArgs {
    int64_t m, n;
    int ntm, ntn;
    const unsigned char *Ap, *Bp;   // packed operands
    float alpha;
    float *C;
    int64_t rsc, csc;
    int uplo;               // DDLA_DENSE, or the triangle of C that is updated (m == n)
    int *err;
};

// Tile t of the enumeration: row-major over all tiles (dense), or over the
// tiles on and below (DDLA_LOWER) / on and above (DDLA_UPPER) the diagonal.
__device__ __forceinline__ void tu_tile(const TuArgs &g, int t, int *mt, int *nt) {
    if (g.uplo == DDLA_DENSE) {
        *mt = t / g.ntn;
        *nt = t % g.ntn;
        return;
    }
    // triangular numbering: row i holds tiles i*(i+1)/2 .. i*(i+1)/2 + i
    int i = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
    while ((i + 1) * (i + 2) / 2 <= t) i++;
    while (i * (i + 1) / 2 > t) i--;
    const int j = t - i * (i + 1) / 2;
    if (g.uplo == DDLA_LOWER) { *mt = i; *nt = j; } else { *mt = j; *nt = i; }
}

__device__ __forceinline__ void bulk_g2s(unsigned dst, const void *src, unsigned bytes, unsigned mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

template <bool BF, bool VEC>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc_update(TuArgs g) {
    typedef UtSplit<BF> SP;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *Ahi = smem, *Alo = smem + SP::PART, *Bhi = smem + 2 * SP::PART, *Blo = smem + 3 * SP::PART;
    float *S = reinterpret_cast<float *>(smem + SP::OPS);
    __shared__ __align__(8) unsigned long long mb_ld, mb_mma;
    __shared__ unsigned tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int total = g.uplo == DDLA_DENSE ? g.ntm * g.ntn : g.ntm * (g.ntm + 1) / 2;
    if ((int)blockIdx.x >= total) return;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_slot)),
                     "r"(UT)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&mb_ld)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&mb_mma)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_slot;
    constexpr uint32_t id = SP::IDESC;
    auto issue_ops = [&](int t) {   // thread 0: the four operand tiles of tile t
        int mt, nt;
        tu_tile(g, t, &mt, &nt);
        const unsigned char *a = g.Ap + (size_t)mt * 2 * SP::PART, *b = g.Bp + (size_t)nt * 2 * SP::PART;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(&mb_ld)),
                     "r"((unsigned)SP::OPS)
                     : "memory");
        bulk_g2s(su32(Ahi), a, SP::PART, su32(&mb_ld));
        bulk_g2s(su32(Alo), a + SP::PART, SP::PART, su32(&mb_ld));
        bulk_g2s(su32(Bhi), b, SP::PART, su32(&mb_ld));
        bulk_g2s(su32(Blo), b + SP::PART, SP::PART, su32(&mb_ld));
    };
    // rows and columns of tile t
    auto tile_rc = [&](int t, int *rows, int *cols) {
        int mt, nt;
        tu_tile(g, t, &mt, &nt);
        const int64_t r_left = g.m - (int64_t)mt * UT, c_left = g.n - (int64_t)nt * UT;
        *rows = (int)(r_left < UT ? r_left : UT);
        *cols = (int)(c_left < UT ? c_left : UT);
    };
    auto wait_mb = [&](unsigned long long *mb, unsigned ph) -> bool {
        for (long long it = 0; it < TC_SPIN; it++)
            if (mbar_try(su32(mb), ph)) return true;
        return false;
    };
    unsigned ph_ld = 0, ph_mma = 0;
    bool failed = false, ops_out = false, mma_out = false;
    if (tid == 0) issue_ops(blockIdx.x);
    ops_out = true;
    const int q = warp & 3, h = warp >> 2;   // TMEM lanes 32q.., columns 64h..
    // coalesced view of a tile: item e = tid + 256 i is row e / 32, columns
    // 4 (e % 32) .. +3 (a warp covers one 512-byte row).  The C tile of the
    // next tile is loaded into registers while the current one finishes.
    float4 creg[16];
    auto load_c = [&](int t) {
        int rows, cols;
        tile_rc(t, &rows, &cols);
        int tm, tn;
        tu_tile(g, t, &tm, &tn);
        const float *ct = g.C + (int64_t)tm * UT * g.rsc + (int64_t)tn * UT * g.csc;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const int e = tid + 256 * i, r = e >> 5, c4 = (e & 31) * 4;
            if constexpr (VEC) {
                creg[i] = (r < rows && c4 < cols) ? *reinterpret_cast<const float4 *>(ct + (int64_t)r * g.rsc + c4)
                                                  : make_float4(0.f, 0.f, 0.f, 0.f);
            } else {
                float v[4];
#pragma unroll
                for (int x = 0; x < 4; x++)
                    v[x] = (r < rows && c4 + x < cols) ? ct[(int64_t)r * g.rsc + (int64_t)(c4 + x) * g.csc] : 0.f;
                creg[i] = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
    };
    load_c(blockIdx.x);
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        int rows, cols;
        tile_rc(t, &rows, &cols);
        int mt, nt;
        tu_tile(g, t, &mt, &nt);
        float *ctile = g.C + (int64_t)mt * UT * g.rsc + (int64_t)nt * UT * g.csc;
        const bool diag = g.uplo != DDLA_DENSE && mt == nt;
        const bool more = t + (int)gridDim.x < total;
        if (__syncthreads_or(!wait_mb(&mb_ld, ph_ld))) { failed = true; break; }
        ph_ld ^= 1u;
        ops_out = false;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int s = 0; s < SP::KSTEPS; s++) {
                const unsigned off = s * 2 * LBO;
                const uint64_t ah = sdesc_sbo(su32(Ahi) + off, SP::SBO), al = sdesc_sbo(su32(Alo) + off, SP::SBO);
                const uint64_t bh = sdesc_sbo(su32(Bhi) + off, SP::SBO), bl = sdesc_sbo(su32(Blo) + off, SP::SBO);
                mma_split<BF>(tmem, ah, bh, id, s == 0 ? 0 : 1);
                mma_split<BF>(tmem, ah, bl, id, 1);
                mma_split<BF>(tmem, al, bh, id, 1);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             su32(&mb_mma))
                         : "memory");
        }
        mma_out = true;
        // C into the staging tile while the MMAs run, then the next tile's C
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const int e = tid + 256 * i, r = e >> 5, c4 = (e & 31) * 4;
            *reinterpret_cast<float4 *>(S + r * UT_SLD + c4) = creg[i];
        }
        if (more) load_c(t + gridDim.x);
        if (__syncthreads_or(!wait_mb(&mb_mma, ph_mma))) { failed = true; break; }
        ph_mma ^= 1u;
        mma_out = false;
        if (more && tid == 0) issue_ops(t + gridDim.x);   // operands are free
        ops_out = more;
        // S[row][64h + j] += alpha * acc(row, 64h + j), row = 32q + lane
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        float *srow = S + (32 * q + lane) * UT_SLD + 64 * h;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            uint32_t d[32];
            const unsigned taddr = tmem + ((unsigned)(32 * q) << 16) + (unsigned)(64 * h + 32 * half);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]),
                  "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]),
                  "=r"(d[15]), "=r"(d[16]), "=r"(d[17]), "=r"(d[18]), "=r"(d[19]), "=r"(d[20]), "=r"(d[21]),
                  "=r"(d[22]), "=r"(d[23]), "=r"(d[24]), "=r"(d[25]), "=r"(d[26]), "=r"(d[27]), "=r"(d[28]),
                  "=r"(d[29]), "=r"(d[30]), "=r"(d[31])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
                float4 v = *reinterpret_cast<float4 *>(srow + 32 * half + j);
                v.x = fmaf(g.alpha, __uint_as_float(d[j]), v.x);
                v.y = fmaf(g.alpha, __uint_as_float(d[j + 1]), v.y);
                v.z = fmaf(g.alpha, __uint_as_float(d[j + 2]), v.z);
                v.w = fmaf(g.alpha, __uint_as_float(d[j + 3]), v.w);
                *reinterpret_cast<float4 *>(srow + 32 * half + j) = v;
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();   // S complete; TMEM read out before the next tile's MMAs
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const int e = tid + 256 * i, r = e >> 5, c4 = (e & 31) * 4;
            if (r < rows && c4 < cols) {
                if (VEC && !diag) {
                    *reinterpret_cast<float4 *>(ctile + (int64_t)r * g.rsc + c4) =
                        *reinterpret_cast<const float4 *>(S + r * UT_SLD + c4);
                } else {   // scalar: unaligned C, or the diagonal tile of a triangular update
#pragma unroll
                    for (int x = 0; x < 4; x++) {
                        const int c = c4 + x;
                        if (c >= cols) break;
                        if (diag && !(g.uplo == DDLA_LOWER ? c <= r : c >= r)) continue;
                        ctile[(int64_t)r * g.rsc + (int64_t)c * g.csc] = S[r * UT_SLD + c];
                    }
                }
            }
        }
        __syncthreads();   // S is read out before the next tile refills it
    }
    if (failed) {
        if (tid == 0) atomicExch(g.err, 1);
        // our copies / MMAs may still be in flight: wait (bounded) before leaving
        if (ops_out) wait_mb(&mb_ld, ph_ld);
        if (mma_out) wait_mb(&mb_mma, ph_mma);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UT) : "memory");
    }
}

template <bool BF>
int tc_update(ddla_handle h, i64 m, i64 n, i64 k, float alpha, View<const float> A, View<const float> B,
              View<float> C, int uplo) {
    typedef UtSplit<BF> SP;
    static size_t uavail = 0;
    if (!uavail) {
        DDLA_TRY(max_dyn_smem((const void *)k_tc_update<BF, true>, h->smem_optin, &uavail));
        size_t u2 = 0;
        DDLA_TRY(max_dyn_smem((const void *)k_tc_update<BF, false>, h->smem_optin, &u2));
        uavail = std::min(uavail, u2);
    }
    if (SP::SMEM > uavail) {
        set_error("gemm_tc: not enough shared memory for the rank-64 update");
        return DDLA_ERR_UNSUPPORTED;
    }
    const i64 ntm = (m + UT - 1) / UT, ntn = (n + UT - 1) / UT;
    unsigned char *pa, *pb;
    DDLA_TRY(workspace(h, WS_TC, 2 * (size_t)SP::PART * (ntm + ntn), (void **)&pa));
    pb = pa + 2 * (size_t)SP::PART * ntm;
    constexpr int PER = 16 / SP::ESZ;
    auto grid_of = [](i64 tot) { return (unsigned)((tot + 255) / 256 < 4096 ? (tot + 255) / 256 : 4096); };
    k_tc_pack<BF><<<grid_of(ntm * UT * (TK / PER)), 256, 0, h->stream>>>(A.p, A.rs, A.cs, m, (int)k, pa, ntm);
    DDLA_LAUNCHED();
    View<const float> Bt = B.t();   // n x k: columns of B as rows
    k_tc_pack<BF><<<grid_of(ntn * UT * (TK / PER)), 256, 0, h->stream>>>(Bt.p, Bt.rs, Bt.cs, n, (int)k, pb, ntn);
    DDLA_LAUNCHED();
    // a few tiles per CTA rather than one CTA per SM for the whole update:
    // CTAs retire often, so the look-ahead panel (a 16-CTA cluster on a
    // high-priority stream) finds free SMs while the update runs
    const i64 tiles = uplo == DDLA_DENSE ? ntm * ntn : ntm * (ntm + 1) / 2;
    const i64 per = std::max<int64_t>(1, tune_get("update.tiles_per_cta", 4));
    const i64 want = (tiles + per - 1) / per;
    const int grid = (int)(want < 65535 ? want : 65535);
    // float4 accesses to C when its rows are 16-byte aligned with a unit column stride
    const bool vec = C.cs == 1 && (C.rs & 3) == 0 && (((uintptr_t)C.p) & 15) == 0 && (n & 3) == 0;
    TuArgs a{m, n, (int)ntm, (int)ntn, pa, pb, alpha, C.p, C.rs, C.cs, uplo, h->d_info + INFO_TIMEOUT};
    if (vec) k_tc_update<BF, true><<<grid, TC_THREADS, SP::SMEM, h->stream>>>(a);
    else k_tc_update<BF, false><<<grid, TC_THREADS, SP::SMEM, h->stream>>>(a);
    DDLA_LAUNCHED();
    return 0;
}

}  // namespace

int gemm_tc(ddla_handle h, int prec, i64 m, i64 n, i64 k, float alpha, View<const float> A, View<const float> B,
            float beta, View<float> C, int uplo) {
    if (m <= 0 || n <= 0) return 0;
    const bool update = beta == 1.f && k > 0 && k <= TK && (uplo == DDLA_DENSE || m == n) &&
                        tune_get("update.tc", 1) != 0;
    if (prec == DDLA_PREC_BF16X3) {
        // 3xBF16 runs only as the rank-<=64 update (the trailing updates of the
        // FP32 factorizations)
        if (!update) {
            set_error("gemm_tc: 3xBF16 products cover the rank-64 update C += alpha A B (beta = 1, k <= 64) only");
            return DDLA_ERR_UNSUPPORTED;
        }
        return tc_update<true>(h, m, n, k, alpha, A, B, C, uplo);
    }
    if (prec != DDLA_PREC_TF32X3) {
        set_error("gemm_tc: precision must be DDLA_PREC_TF32X3 or DDLA_PREC_BF16X3");
        return DDLA_ERR_UNSUPPORTED;
    }
    if (update && C.cs == 1 && (n & 3) == 0 && (C.rs & 3) == 0 && (((uintptr_t)C.p) & 15) == 0) {
        // rank-<=64 update: packed operands + persistent tensor-core kernel
        const int rc = tc_update<false>(h, m, n, k, alpha, A, B, C, uplo);
        if (rc != DDLA_ERR_UNSUPPORTED) return rc;
    }
    static size_t avail = 0;
    if (!avail) DDLA_TRY(max_dyn_smem((const void *)k_tc_tf32x3, h->smem_optin, &avail));
    if (TC_SMEM > avail) {
        set_error("gemm_tc: not enough shared memory");
        return DDLA_ERR_UNSUPPORTED;
    }
    i64 gx = (n + TN - 1) / TN, gy = (m + TM - 1) / TM;
    if (gy > 65535) { set_error("gemm_tc: m too large"); return DDLA_ERR_UNSUPPORTED; }
    TcArgs a{m, n, alpha == 0.f ? 0 : k, alpha, beta, A.p, A.rs, A.cs, B.p, B.rs, B.cs, C.p, C.rs, C.cs, uplo,
             h->d_info + INFO_TIMEOUT};
    k_tc_tf32x3<<<dim3((unsigned)gx, (unsigned)gy), TC_THREADS, TC_SMEM, h->stream>>>(a);
    DDLA_LAUNCHED();
    return 0;
}

// ------------------------------------------------------------------ Ozaki split FP64 GEMM
//
// C = alpha*A*B + beta*C with FP64-level accuracy from BF16 tensor-core
// products (Ozaki scheme, error-free splitting):
//   * row i of A is scaled by sigma_i = 2^e_i (the smallest power of two above
//     max_k |a_ik|) and cut into OZ_S slices of OZ_BETA bits, taken from the
//     integer mantissa: a_ik = sigma_i sum_t q_t 2^(-beta (t+1)), 0 <= |q_t| <=
//     2^beta - 1, all slices carrying the sign of a_ik; the remainder below
//     2^(-beta OZ_S) sigma_i is dropped.  Columns of B likewise (tau_j).
//   * slices are stored pre-scaled, A_t = q_t 2^(-beta t), which is exact in
//     BF16 (8-bit integers times a power of two);
//   * A*B = 2^(-2 beta) diag(sigma) [sum_{t+u < OZ_S} A_t B_u] diag(tau).
//     Products of one level t+u = l are multiples of 2^(-beta l) below
//     2^(2 beta - beta l), so a level accumulates EXACTLY in FP32 (TMEM) while
//     its partial sum stays below 2^24 ulps: the levels l < OZ_EXACT each get
//     their own accumulator, flushed into FP64 registers after at most
//     oz_period(l) of K; the small levels l >= OZ_EXACT share one rounded FP32
//     accumulator (their rounding is below 2^-(beta OZ_EXACT + 24) of the
//     result scale).
// The error is bounded by a small multiple of 2^-53 K sigma_i tau_j, i.e.
// relative to max_k |a_ik| max_k |b_kj|.  Non-finite inputs make the affected
// rows / columns of C non-finite.
//
// Operand slices are packed by the split kernels directly in the shared-memory
// tile layout ([slice][row tile][K chunk][core matrices]) so that staging a
// K chunk is a contiguous copy.
namespace {

constexpr int OZ_S = 8, OZ_BETA = 7;
constexpr int OZ_EXACT = 5;               // levels with their own exact accumulator
constexpr int OZ_NACC = OZ_EXACT + 1;     // + one shared accumulator for the small levels
constexpr int OZ_TN = 64;                 // tile columns
constexpr int OZ_KC = 32;                 // K staged per chunk (bf16)
constexpr int OZ_NS = 2;                  // shared-memory stages (chunks in flight)
constexpr int OZ_SBO = (OZ_KC / 8) * 128; // bf16 core-matrix layout: 8 elements per 16-byte chunk
constexpr int OZ_A_TILE = TM * OZ_KC * 2, OZ_B_TILE = OZ_TN * OZ_KC * 2;
constexpr int OZ_STAGE = OZ_S * (OZ_A_TILE + OZ_B_TILE);   // every slice of one K chunk
constexpr size_t OZ_SMEM = (size_t)OZ_NS * OZ_STAGE;
// OZ_NACC live accumulators plus two spare slots of OZ_TN columns: a period
// that ends hands its slot to the flush and continues in the oldest spare
constexpr int OZ_SLOTS = OZ_NACC + 2;
constexpr int OZ_TMEM_COLS = 512;
static_assert(OZ_SLOTS * OZ_TN <= OZ_TMEM_COLS, "TMEM columns");

// Flush period of accumulator a in K chunks: level l sums (l+1) slice pairs of
// products below (2^beta - 1)^2 ulps, exact while (l+1) * period * OZ_KC *
// 127^2 < 2^24.  The shared small-level accumulator (a = OZ_EXACT) rounds
// anyway; its period bounds that rounding.
__host__ __device__ constexpr int oz_period(int a) {
    return a == 0 ? 32 : a == 1 ? 16 : a == 2 ? 8 : a == 3 ? 8 : a == 4 ? 4 : 32;
}
// Phase of each accumulator's flush periods: a period of accumulator a ends
// before chunk c when (c + oz_phase(a)) % oz_period(a) == 0.  The phases put
// at most one flush on any chunk (a = 4 on c = 0 mod 4, a = 3 / 2 on c = 2 / 6
// mod 8, a = 1 on c = 1 mod 16, a = 0 / 5 on c = 3 / 19 mod 32), so the FP64
// flush work spreads evenly under the MMAs.  The first period of an
// accumulator is shorter than oz_period, never longer.
__host__ __device__ constexpr int oz_phase(int a) {
    return a == 0 ? 29 : a == 1 ? 15 : a == 2 ? 2 : a == 3 ? 6 : a == 4 ? 0 : 13;
}
static_assert(1 * 32 * OZ_KC * 127 * 127 < (1 << 24) && 2 * 16 * OZ_KC * 127 * 127 < (1 << 24) &&
                  3 * 8 * OZ_KC * 127 * 127 < (1 << 24) && 4 * 8 * OZ_KC * 127 * 127 < (1 << 24) &&
                  5 * 4 * OZ_KC * 127 * 127 < (1 << 24),
              "exact accumulation periods");

// FP32 -> FP64 by the IEEE field layout (exponent rebias 1023 - 127 = 896,
// mantissa shifted by 52 - 23 = 29) on the integer pipe.  Only for zeros and
// normal values, which is all the level sums hold: they are multiples of
// 2^-(beta (OZ_S - 1)) far above the FP32 subnormal range, and finite.
__device__ __forceinline__ double oz_f2d(uint32_t u) {
    const uint32_t mag = u & 0x7fffffffu;
    const uint32_t hi = (u & 0x80000000u) | (mag ? (mag >> 3) + (896u << 20) : 0u);
    return __hiloint2double((int)hi, (int)(u << 29));
}

__device__ __forceinline__ int oz_off(int r, int k) {   // byte offset of bf16 element (r, k) in a tile
    return (r >> 3) * OZ_SBO + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint64_t oz_desc(unsigned addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3ffff) >> 4);
    d |= (uint64_t)(128 >> 4) << 16;
    d |= (uint64_t)(OZ_SBO >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// D f32, A and B bf16 (format 1), K-major, N = OZ_TN, M = TM
__host__ __device__ constexpr uint32_t oz_idesc() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

// Splits the rows of a strided FP64 matrix X (rows x cols) into OZ_S packed
// BF16 slices.  One block per padded row (row tiles of `tr` rows); the scale
// 2^e of each row goes to scale[r] (non-finite rows store their max, which
// makes the row of the result non-finite).
// Batched: blockIdx.y selects the product; X is offset by offs[3 y + which]
// (when offs is given) and pack / scale by whole items.
__global__ void k_oz_split(const double *X, i64 rs, i64 cs, i64 rows, i64 cols, int tr, i64 row_tiles,
                           i64 kchunks, __nv_bfloat16 *pack, double *scale, const i64 *offs, int which,
                           i64 pack_item, i64 scale_item) {
    const i64 r = blockIdx.x;
    if (offs) X += offs[3 * (i64)blockIdx.y + which];
    pack += (i64)blockIdx.y * pack_item;
    scale += (i64)blockIdx.y * scale_item;
    __shared__ unsigned long long red[32];
    const bool live = r < rows;
    // row max of |x| on the integer pipe: for non-negative doubles the bit
    // pattern orders like the value (NaN above +inf)
    unsigned long long mx = 0;
    if (live)
        for (i64 c = threadIdx.x; c < cols; c += blockDim.x)
            mx = max(mx, (unsigned long long)__double_as_longlong(X[r * rs + c * cs]) & 0x7fffffffffffffffULL);
    for (int off = 16; off > 0; off >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned long long v = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0ULL;
        for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
        if (threadIdx.x == 0) red[0] = v;
    }
    __syncthreads();
    mx = red[0];
    const int bexp = (int)(mx >> 52);   // biased exponent of the row max
    int e = 0;                          // row scale 2^e > max |x|
    bool finite = bexp < 2047;
    if (mx != 0 && finite) {
        if (bexp == 0) {                // subnormal max: 2^e above its leading bit
            e = -1074 + (64 - __clzll(mx));
        } else {
            e = bexp - 1022;
        }
    }
    if (threadIdx.x == 0) scale[r] = finite ? ldexp(1.0, e) : __longlong_as_double((long long)mx);
    const i64 rt = r / tr, rr = r % tr;
    for (i64 c8 = threadIdx.x; c8 < kchunks * (OZ_KC / 8); c8 += blockDim.x) {
        unsigned q[OZ_S][4];
#pragma unroll
        for (int t = 0; t < OZ_S; t++) q[t][0] = q[t][1] = q[t][2] = q[t][3] = 0;
#pragma unroll
        for (int x = 0; x < 8; x++) {
            const i64 c = 8 * c8 + x;
            long long bits = 0;
            if (live && finite && c < cols) bits = __double_as_longlong(X[r * rs + c * cs]);
            const unsigned long long ab = (unsigned long long)bits & 0x7fffffffffffffffULL;
            const int ex = (int)(ab >> 52);
            const unsigned long long man = (ab & ((1ULL << 52) - 1)) | (ex ? (1ULL << 52) : 0ULL);
            // |x| / 2^e as a fixed-point fraction with beta*S bits (truncated)
            const int sh = (ex ? ex - 1075 : -1074) - e + OZ_BETA * OZ_S;
            unsigned long long F = 0;
            if (sh >= 0) F = man << sh;   // sh <= 3 since |x| < 2^e
            else if (sh > -64) F = man >> (-sh);
            const unsigned sgn = bits < 0 ? 0x8000u : 0u;
#pragma unroll
            for (int t = 0; t < OZ_S; t++) {
                const unsigned qt = (unsigned)(F >> (OZ_BETA * (OZ_S - 1 - t))) & ((1u << OZ_BETA) - 1);
                // bf16 of qt * 2^(-beta t): exact (qt < 2^8), built from the float
                const float f = __int_as_float(__float_as_int((float)qt) - ((OZ_BETA * t) << 23) * (qt != 0));
                const unsigned hb = (__float_as_uint(f) >> 16) | (qt ? sgn : 0u);
                q[t][x >> 1] |= hb << (16 * (x & 1));
            }
        }
        const i64 kc = c8 / (OZ_KC / 8), kq = 8 * (c8 % (OZ_KC / 8));
#pragma unroll
        for (int t = 0; t < OZ_S; t++) {
            const i64 tile = ((t * row_tiles + rt) * kchunks + kc);
            unsigned char *dst = reinterpret_cast<unsigned char *>(pack) + tile * (i64)tr * OZ_KC * 2 +
                                 oz_off((int)rr, (int)kq);
            *reinterpret_cast<uint4 *>(dst) = make_uint4(q[t][0], q[t][1], q[t][2], q[t][3]);
        }
    }
}

struct OzArgs {
    int64_t m, n, kchunks, mtiles, ntiles;
    const __nv_bfloat16 *Ap, *Bp;   // packed slices
    const double *sa, *sb;          // row / column scales
    double alpha, beta;
    double *C;
    int64_t rsc, csc;
    const int64_t *offs;            // batched: C offset of product z at offs[3 z + 2]
    int64_t a_item, b_item, s_item_a, s_item_b;   // element strides between products
    int uplo;   // DDLA_DENSE, or the triangle of C that is written (GEMMT)
    int *err;
};

// One CTA per 128 x OZ_TN tile of C, OZ_THREADS threads.  Warp 8 (lane 0) is
// the issuer: it moves each K chunk's slices (OZ_S A tiles + OZ_S B tiles,
// contiguous in the packed layout) with bulk asynchronous copies into one of
// OZ_NS shared-memory stages and issues the chunk's slice-pair MMAs into the
// accumulators of the running flush periods.  Warps 0-7 are the flushers: for
// every chunk f they wait for its MMAs and add the accumulator whose period
// ended with f into FP64 registers, while the issuer runs ahead.  TMEM holds
// OZ_SLOTS slots: when a period of accumulator a ends, a continues in the
// oldest spare slot and its old slot, once flushed, becomes the newest spare
// (OzSlots; issuer and flushers replay the same sequence).  With at most one
// period end per chunk, a spare taken at chunk c was released at a chunk
// <= c - 2 and flushed by flush c - 3.  Warp w < 8 reads TMEM lanes
// 32 (w % 4).. and columns 32 (w / 4).. of each slot, so it owns 32 columns of
// one row of C.
// Barriers (all waits bounded):
//   full[st]   copies of a stage landed        (issuer waits)
//   mdone[st]  MMAs that read a stage retired  (issuer waits, then reloads it)
//   mready[f % 4]  MMAs of chunk f retired      (flushers wait)
//   fdone[f % 4]   flush of chunk f done, one arrival per flusher warp
//                                              (issuer waits)
// The issuer starts chunk c only after flush c - 3, so each ring slot
// completes again only after its previous phase was awaited.
constexpr int OZ_THREADS = 288;
constexpr int OZ_RING = 4;

// TMEM slot of each accumulator: OZ_NACC live slots and a FIFO of two spares.
struct OzSlots {
    int slot[OZ_NACC], spare0, spare1;
    __device__ __forceinline__ void init() {
#pragma unroll
        for (int a = 0; a < OZ_NACC; a++) slot[a] = a;
        spare0 = OZ_NACC;
        spare1 = OZ_NACC + 1;
    }
    // a period of accumulator a ends before chunk c: a moves to the oldest
    // spare, its old slot (to be flushed) becomes the newest; returns the old slot
    __device__ __forceinline__ int turn(int a) {
        const int old = slot[a];
        slot[a] = spare0;
        spare0 = spare1;
        spare1 = old;
        return old;
    }
};

constexpr int OZ_GROUP = 8;   // row tiles per raster group

__global__ void __launch_bounds__(OZ_THREADS, 1) k_oz_gemm(OzArgs g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) unsigned long long full[OZ_NS], mdone[OZ_NS], mready[OZ_RING], fdone[OZ_RING];
    __shared__ unsigned tmem_slot;
    __shared__ volatile int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // grouped raster: the CTAs launched together walk OZ_GROUP row tiles
    // before moving to the next column tile, so a wave shares A's and B's
    // slice panels in L2 instead of streaming all of B once per wave
    const int64_t NT = gridDim.x, MT = gridDim.y, bz = blockIdx.z;
    const int64_t lin = (int64_t)blockIdx.y * NT + blockIdx.x, span = (int64_t)OZ_GROUP * NT;
    const int64_t first = (lin / span) * OZ_GROUP, gm = MT - first < OZ_GROUP ? MT - first : OZ_GROUP;
    const int64_t mt = first + (lin % span) % gm, nt = (lin % span) / gm;
    const __nv_bfloat16 *Ap = g.Ap + bz * g.a_item, *Bp = g.Bp + bz * g.b_item;
    const double *sa = g.sa + bz * g.s_item_a, *sb = g.sb + bz * g.s_item_b;
    double *Cz = g.C + (g.offs ? g.offs[3 * bz + 2] : 0);
    const int64_t m0 = mt * TM, n0 = nt * OZ_TN;
    if (g.uplo == DDLA_LOWER && n0 > m0 + TM - 1) return;
    if (g.uplo == DDLA_UPPER && m0 > n0 + OZ_TN - 1) return;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_slot)),
                     "r"(OZ_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int st = 0; st < OZ_NS; st++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&full[st])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&mdone[st])) : "memory");
        }
        for (int r = 0; r < OZ_RING; r++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&mready[r])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 8;" ::"r"(su32(&fdone[r])) : "memory");
        }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_slot;
    const int K = (int)g.kchunks;
    // bounded wait; flushers also give up once the issuer has aborted
    auto wait_mb = [&](unsigned long long *mb, unsigned ph, bool watch) -> bool {
        for (long long it = 0; it < TC_SPIN; it++) {
            if (mbar_try(su32(mb), ph)) return true;
            if (watch && abort_flag) return false;
        }
        return false;
    };
    bool failed = false;
    if (warp == 8) {
        if (lane == 0) {
            const uint32_t id = oz_idesc();
            const size_t a_stride = (size_t)g.mtiles * K * (TM * OZ_KC);     // elements between slices
            const size_t b_stride = (size_t)g.ntiles * K * (OZ_TN * OZ_KC);
            auto load = [&](int c, int st) {   // every slice of chunk c into stage st
                unsigned char *base = smem + (size_t)st * OZ_STAGE;
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(&full[st])),
                             "r"((unsigned)OZ_STAGE)
                             : "memory");
                const __nv_bfloat16 *a = Ap + ((size_t)mt * K + c) * (TM * OZ_KC);
                const __nv_bfloat16 *b = Bp + ((size_t)nt * K + c) * (OZ_TN * OZ_KC);
                for (int t = 0; t < OZ_S; t++)
                    bulk_g2s(su32(base + (size_t)t * OZ_A_TILE), a + t * a_stride, OZ_A_TILE, su32(&full[st]));
                for (int u = 0; u < OZ_S; u++)
                    bulk_g2s(su32(base + (size_t)OZ_S * OZ_A_TILE + (size_t)u * OZ_B_TILE), b + u * b_stride,
                             OZ_B_TILE, su32(&full[st]));
            };
            OzSlots slots;
            slots.init();
            // chunk of the copy / MMA batch in flight per stage (-1: none), for the drain
            int ld_c[OZ_NS], mm_last = -1;
            for (int st = 0; st < OZ_NS; st++) ld_c[st] = -1;
            for (int st = 0; st < OZ_NS && st < K; st++) {
                load(st, st);
                ld_c[st] = st;
            }
            for (int c = 0; c < K; c++) {
                const int s = c % OZ_NS;
                if (!wait_mb(&full[s], (unsigned)(c / OZ_NS) & 1u, false)) { failed = true; break; }
                ld_c[s] = -1;
                if (c >= 3 && !wait_mb(&fdone[(c - 3) % OZ_RING], (unsigned)((c - 3) / OZ_RING) & 1u, false)) {
                    failed = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // per accumulator: its TMEM slot and whether this chunk starts a period
                unsigned dcol[OZ_NACC], fresh = c == 0 ? (1u << OZ_NACC) - 1u : 0u;
#pragma unroll
                for (int a = 0; a < OZ_NACC; a++) {
                    if (c > 0 && (c + oz_phase(a)) % oz_period(a) == 0) {
                        slots.turn(a);
                        fresh |= 1u << a;
                    }
                    dcol[a] = tmem + (unsigned)(slots.slot[a] * OZ_TN);
                }
                const unsigned char *At = smem + (size_t)s * OZ_STAGE;
                const uint64_t ad0 = oz_desc(su32(At)), bd0 = oz_desc(su32(At + (size_t)OZ_S * OZ_A_TILE));
                // slice pairs (t, u), t + u < OZ_S; the first pair of level a is (0, a)
#pragma unroll
                for (int t = 0; t < OZ_S; t++)
#pragma unroll
                    for (int u = 0; u < OZ_S - t; u++) {
                        const int a = (t + u < OZ_EXACT) ? t + u : OZ_EXACT;
                        const bool first = t == 0 && u == a;
#pragma unroll
                        for (int ks = 0; ks < OZ_KC / 16; ks++) {
                            // descriptor start addresses are in 16-byte units
                            const uint64_t ad = ad0 + (uint64_t)((t * OZ_A_TILE + ks * 256) >> 4);
                            const uint64_t bd = bd0 + (uint64_t)((u * OZ_B_TILE + ks * 256) >> 4);
                            const int accum = (first && ks == 0 && ((fresh >> a) & 1u)) ? 0 : 1;
                            asm volatile(
                                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dcol[a]),
                                "l"(ad), "l"(bd), "r"(id), "r"(accum)
                                : "memory");
                        }
                    }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 su32(&mdone[s]))
                             : "memory");
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 su32(&mready[c % OZ_RING]))
                             : "memory");
                mm_last = c;
                // chunk c - 1's stage is free once its MMAs retired: refill it
                if (c >= 1) {
                    const int sp = (c - 1) % OZ_NS;
                    if (!wait_mb(&mdone[sp], (unsigned)((c - 1) / OZ_NS) & 1u, false)) { failed = true; break; }
                    if (c - 1 + OZ_NS < K) {
                        load(c - 1 + OZ_NS, sp);
                        ld_c[sp] = c - 1 + OZ_NS;
                    }
                }
            }
            if (failed) {
                atomicExch(g.err, 1);
                abort_flag = 1;
                // copies and MMAs of this CTA still in flight (bounded waits)
                for (int st = 0; st < OZ_NS; st++)
                    if (ld_c[st] >= 0) wait_mb(&full[st], (unsigned)(ld_c[st] / OZ_NS) & 1u, false);
                if (mm_last >= 0) wait_mb(&mdone[mm_last % OZ_NS], (unsigned)(mm_last / OZ_NS) & 1u, false);
            }
        }
    } else {
        const int q = warp & 3, hcol = 32 * (warp >> 2);
        double acc[32];
#pragma unroll
        for (int j = 0; j < 32; j++) acc[j] = 0.0;
        OzSlots slots;
        slots.init();
        auto flush = [&](int sl) {   // add this warp's 32 x 32 block of TMEM slot sl
            uint32_t d[32];
            const unsigned taddr = tmem + ((unsigned)(32 * q) << 16) + (unsigned)(sl * OZ_TN + hcol);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]),
                  "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]),
                  "=r"(d[15]), "=r"(d[16]), "=r"(d[17]), "=r"(d[18]), "=r"(d[19]), "=r"(d[20]), "=r"(d[21]),
                  "=r"(d[22]), "=r"(d[23]), "=r"(d[24]), "=r"(d[25]), "=r"(d[26]), "=r"(d[27]), "=r"(d[28]),
                  "=r"(d[29]), "=r"(d[30]), "=r"(d[31])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 32; j++) acc[j] += oz_f2d(d[j]);
        };
        for (int f = 0; f < K; f++) {
            const bool ok = wait_mb(&mready[f % OZ_RING], (unsigned)(f / OZ_RING) & 1u, true);
            if (!__all_sync(0xffffffffu, ok)) {
                failed = true;
                if (lane == 0) atomicExch(g.err, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (f + 1 < K) {
                // the accumulator whose period ends with chunk f (the issuer
                // turns the same slot before chunk f + 1)
#pragma unroll
                for (int a = 0; a < OZ_NACC; a++)
                    if ((f + 1 + oz_phase(a)) % oz_period(a) == 0) flush(slots.turn(a));
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&fdone[f % OZ_RING]))
                                 : "memory");
            } else {
#pragma unroll
                for (int a = 0; a < OZ_NACC; a++) flush(slots.slot[a]);
            }
        }
        if (!failed) {
            // scales 2^(-2 beta) sigma_i tau_j and the alpha / beta epilogue
            const int64_t gr = m0 + 32 * q + lane;
            if (gr < g.m) {
                const double sr = sa[gr] * g.alpha * 0x1p-14;
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const int64_t gc = n0 + hcol + j;
                    if (gc >= g.n) continue;
                    if (g.uplo == DDLA_LOWER && gc > gr) continue;
                    if (g.uplo == DDLA_UPPER && gc < gr) continue;
                    const double v = (acc[j] * sr) * sb[gc];
                    double *cp = Cz + gr * g.rsc + gc * g.csc;
                    *cp = (g.beta == 0.0) ? v : fma(g.beta, *cp, v);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(OZ_TMEM_COLS)
                     : "memory");
    }
}

}  // namespace

int gemm_ozaki(ddla_handle h, i64 m, i64 n, i64 k, double alpha, View<const double> A, View<const double> B,
               double beta, View<double> C, int uplo, i64 batch, const i64 *d_offsets) {
    if (m <= 0 || n <= 0 || batch <= 0) return 0;
    cudaStream_t s = h->stream;
    if (k <= 0 || alpha == 0.0) {
        if (batch == 1 && !d_offsets) return gemm_f64(s, m, n, 0, 0.0, A, B, beta, C, uplo);
        if (beta == 1.0) return 0;
        set_error("gemm_ozaki: batched beta scaling with k = 0 is not supported");
        return DDLA_ERR_UNSUPPORTED;
    }
    static size_t avail = 0;
    if (!avail) DDLA_TRY(max_dyn_smem((const void *)k_oz_gemm, h->smem_optin, &avail));
    if (OZ_SMEM > avail) {
        set_error("gemm_ozaki: not enough shared memory");
        return DDLA_ERR_UNSUPPORTED;
    }
    const i64 mtiles = (m + TM - 1) / TM, ntiles = (n + OZ_TN - 1) / OZ_TN, kchunks = (k + OZ_KC - 1) / OZ_KC;
    if (mtiles > 65535) { set_error("gemm_ozaki: m too large"); return DDLA_ERR_UNSUPPORTED; }
    if (kchunks > (i64)INT32_MAX) { set_error("gemm_ozaki: k too large"); return DDLA_ERR_UNSUPPORTED; }
    const i64 a_item = (i64)OZ_S * mtiles * TM * kchunks * OZ_KC, b_item = (i64)OZ_S * ntiles * OZ_TN * kchunks * OZ_KC;
    const i64 sa_item = mtiles * TM, sb_item = ntiles * OZ_TN;
    // products in groups of at most 65535 (grid y / z limit), packed slices of one group at a time
    const i64 group = batch < 65535 ? batch : 65535;
    void *wa, *wb;
    DDLA_TRY(workspace(h, WS_TC, (size_t)group * (a_item * 2 + sa_item * 8), &wa));
    DDLA_TRY(workspace(h, WS_TC2, (size_t)group * (b_item * 2 + sb_item * 8), &wb));
    __nv_bfloat16 *ap = (__nv_bfloat16 *)wa, *bp = (__nv_bfloat16 *)wb;
    double *sa = (double *)((char *)wa + (size_t)group * a_item * 2);
    double *sb = (double *)((char *)wb + (size_t)group * b_item * 2);
    View<const double> Bt = B.t();   // columns of B as rows
    for (i64 z0 = 0; z0 < batch; z0 += group) {
        const i64 nz = batch - z0 < group ? batch - z0 : group;
        const i64 *offs = d_offsets ? d_offsets + 3 * z0 : nullptr;
        k_oz_split<<<dim3((unsigned)(mtiles * TM), (unsigned)nz), 256, 0, s>>>(A.p, A.rs, A.cs, m, k, TM, mtiles,
                                                                              kchunks, ap, sa, offs, 0, a_item,
                                                                              sa_item);
        DDLA_LAUNCHED();
        k_oz_split<<<dim3((unsigned)(ntiles * OZ_TN), (unsigned)nz), 256, 0, s>>>(
            Bt.p, Bt.rs, Bt.cs, n, k, OZ_TN, ntiles, kchunks, bp, sb, offs, 1, b_item, sb_item);
        DDLA_LAUNCHED();
        OzArgs a{m, n, kchunks, mtiles, ntiles, ap, bp, sa, sb, alpha, beta, C.p, C.rs, C.cs, offs,
                 a_item, b_item, sa_item, sb_item, uplo, h->d_info + INFO_TIMEOUT};
        k_oz_gemm<<<dim3((unsigned)ntiles, (unsigned)mtiles, (unsigned)nz), OZ_THREADS, OZ_SMEM, s>>>(a);
        DDLA_LAUNCHED();
    }
    return 0;
}

}  // namespace ddla

using namespace ddla;

// FP32 GEMM through the tensor-core path on device data (testing and tuning
// entry point; the mixed factorizations call the same kernel internally).
extern "C" int ddla_dev_sgemm_tc(ddla_handle h, int32_t precision, int64_t m, int64_t n, int64_t k, float alpha,
                                 const float *a, int64_t rsa, int64_t csa, const float *b, int64_t rsb, int64_t csb,
                                 float beta, float *c, int64_t rsc, int64_t csc) {
    if (!h) return -1;
    if (m < 0) return -3;
    if (n < 0) return -4;
    if (k < 0) return -5;
    if (precision == DDLA_PREC_FP32)
        return gemm_f32(h->stream, m, n, k, alpha, View<const float>{a, m, k, rsa, csa},
                        View<const float>{b, k, n, rsb, csb}, beta, View<float>{c, m, n, rsc, csc});
    return gemm_tc(h, precision, m, n, k, alpha, View<const float>{a, m, k, rsa, csa},
                   View<const float>{b, k, n, rsb, csb}, beta, View<float>{c, m, n, rsc, csc}, DDLA_DENSE);
}
