// GEMM kernels of libddla_gb300.
//
// FP64: DMMA (mma.sync.aligned.m8n8k4 .f64) on shared-memory tiles.  On GB300
// FP64 runs at ~1/70 of the FP32 CUDA-core rate (DMMA and DFMA both measure
// ~1.05 TFLOP/s), so an FP64 GEMM is compute-bound at any reasonable tile; the
// kernel reads operands through arbitrary element strides (DDLA views) and
// spends its effort on keeping every SM's DMMA pipe busy (tile shape chosen
// for an even split of tiles over the 152 SMs).
//
// FP32: CUDA-core FFMA, 128x128 tiles, 8x8 outputs per thread, double-buffered
// shared memory.  Used by the FP32-factorization (mixed) paths when the
// tensor-core variant is not selected.
//
// Both compute C = alpha*A*B + beta*C (BLIS semantics: beta == 0 never reads C)
// and optionally only the lower or upper triangle of C (GEMMT / SYRK), skipping
// tiles that do not intersect it (DDLA's GEMMTMacroKernel computes and masks
// them, DDLA/BLAS/Managed/3m/MacroKernel.cs:158-216).
//
// The FP64 kernel also reads structured operands (SYMM, TRMM, TRMM3): a
// symmetric operand stored in one triangle is mirrored on load, a triangular
// one reads zeros outside its triangle (ones on a unit diagonal) and its CTA's
// k loop is cut to the k range the triangle covers.  This is what DDLA's
// structured packing does (SYPack / TRPack, DDLA/BLAS/Managed/3m/Packing.cs:
// 105-374) before its ordinary macro kernel, without the packed copy.
#include "common.cuh"

namespace ddla {

// ------------------------------------------------------------------ FP64
namespace {

constexpr int BK64 = 16;

// Element (i, j) of a structured operand (mode: OP_* bits, see gemm_f64_struct).
template <bool STRUCT>
__device__ __forceinline__ double ld_op(const double *__restrict__ P, i64 rs, i64 cs, i64 i, i64 j, int mode) {
    if (STRUCT) {
        const bool outside = (mode & OP_LOWER) ? (j > i) : (j < i);
        if ((mode & 3) == OP_SYM) {
            if (outside) {
                i64 t = i;
                i = j;
                j = t;
            }
        } else if ((mode & 3) == OP_TRI) {
            if (outside) return 0.0;
            if (i == j && (mode & OP_UNIT)) return 1.0;
        }
    }
    return P[i * rs + j * cs];
}

template <int BM, int BN, int WM, int WN, bool STRUCT>
__global__ void __launch_bounds__(WM *WN * 32)
    k_gemm_f64(i64 m, i64 n, i64 k, double alpha, const double *__restrict__ A, i64 rsa, i64 csa,
               const double *__restrict__ B, i64 rsb, i64 csb, double beta, double *C, i64 rsc, i64 csc,
               int uplo, i64 sa, i64 sb, i64 sc, const i64 *__restrict__ boff, int amode, int bmode, i64 kslice) {
    constexpr int NT = WM * WN * 32;
    constexpr int TWM = BM / WM, TWN = BN / WN;  // warp tile
    constexpr int FM = TWM / 8, FN = TWN / 8;   // 8x8 fragments per warp
    constexpr int PAD = 8;
    __shared__ double As[BK64][BM + PAD];
    __shared__ double Bs[BK64][BN + PAD];

    const i64 bz = blockIdx.z;
    if (boff) {
        A += boff[3 * bz];
        B += boff[3 * bz + 1];
        C += boff[3 * bz + 2];
    } else {
        A += bz * sa;
        B += bz * sb;
        C += bz * sc;
    }
    const i64 m0 = (i64)blockIdx.y * BM, n0 = (i64)blockIdx.x * BN;
    if (uplo == DDLA_LOWER && n0 > m0 + BM - 1) return;
    if (uplo == DDLA_UPPER && m0 > n0 + BN - 1) return;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp / WN, wn = warp % WN;
    double acc[FM][FN][2];
#pragma unroll
    for (int i = 0; i < FM; i++)
#pragma unroll
        for (int j = 0; j < FN; j++) acc[i][j][0] = acc[i][j][1] = 0.0;

    const bool a_kfast = (csa == 1);  // K contiguous in A
    const bool b_nfast = (csb == 1);  // N contiguous in B
    // k range of this tile: a triangular A is zero right of its diagonal when
    // lower (left of it when upper); a triangular B is zero above its diagonal
    // when lower (below it when upper).
    i64 kb = 0, ke = k;
    if (kslice > 0) {   // split k: problem z sums k in [z*kslice, (z+1)*kslice)
        kb = bz * kslice;
        ke = min(k, kb + kslice);
    }
    if (STRUCT) {
        if ((amode & 3) == OP_TRI) {
            if (amode & OP_LOWER) ke = min(ke, m0 + BM);
            else kb = max(kb, m0);
        }
        if ((bmode & 3) == OP_TRI) {
            if (bmode & OP_LOWER) kb = max(kb, n0);
            else ke = min(ke, n0 + BN);
        }
    }
    for (i64 k0 = kb; k0 < ke; k0 += BK64) {
        // A tile BM x BK
        for (int e = tid; e < BM * BK64; e += NT) {
            int r, kk;
            if (a_kfast) { kk = e % BK64; r = e / BK64; } else { r = e % BM; kk = e / BM; }
            i64 gr = m0 + r, gk = k0 + kk;
            As[kk][r] = (gr < m && gk < ke) ? ld_op<STRUCT>(A, rsa, csa, gr, gk, amode) : 0.0;
        }
        // B tile BK x BN
        for (int e = tid; e < BN * BK64; e += NT) {
            int c, kk;
            if (b_nfast) { c = e % BN; kk = e / BN; } else { kk = e % BK64; c = e / BK64; }
            i64 gc = n0 + c, gk = k0 + kk;
            Bs[kk][c] = (gc < n && gk < ke) ? ld_op<STRUCT>(B, rsb, csb, gk, gc, bmode) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK64; ks += 4) {
            double af[FM], bf[FN];
#pragma unroll
            for (int i = 0; i < FM; i++) af[i] = As[ks + (lane & 3)][wm * TWM + i * 8 + (lane >> 2)];
#pragma unroll
            for (int j = 0; j < FN; j++) bf[j] = Bs[ks + (lane & 3)][wn * TWN + j * 8 + (lane >> 2)];
#pragma unroll
            for (int i = 0; i < FM; i++)
#pragma unroll
                for (int j = 0; j < FN; j++)
                    asm volatile(
                        "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                        : "+d"(acc[i][j][0]), "+d"(acc[i][j][1])
                        : "d"(af[i]), "d"(bf[j]));
        }
        __syncthreads();
    }
    // Epilogue: fragment element (row lane/4, cols 2*(lane%4)+{0,1}).
#pragma unroll
    for (int i = 0; i < FM; i++)
#pragma unroll
        for (int j = 0; j < FN; j++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                i64 gr = m0 + wm * TWM + i * 8 + (lane >> 2);
                i64 gc = n0 + wn * TWN + j * 8 + 2 * (lane & 3) + h;
                if (gr >= m || gc >= n) continue;
                if (uplo == DDLA_LOWER && gc > gr) continue;
                if (uplo == DDLA_UPPER && gc < gr) continue;
                double *cp = C + gr * rsc + gc * csc;
                double v = alpha * acc[i][j][h];
                *cp = (beta == 0.0) ? v : fma(beta, *cp, v);
            }
}

template <int BM, int BN, int WM, int WN>
int launch_f64(cudaStream_t s, i64 m, i64 n, i64 k, double alpha, View<const double> A, View<const double> B,
               double beta, View<double> C, int uplo, i64 batch, i64 sa, i64 sb, i64 sc, const i64 *boff,
               int amode, int bmode, i64 kslice = 0) {
    i64 gx = (n + BN - 1) / BN, gy = (m + BM - 1) / BM;
    if (gy > 65535) { set_error("gemm_f64: m too large for one launch"); return DDLA_ERR_UNSUPPORTED; }
    for (i64 b0 = 0; b0 < batch; b0 += 65535) {
        i64 nb = batch - b0 < 65535 ? batch - b0 : 65535;
        dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)nb);
        if (amode | bmode)
            k_gemm_f64<BM, BN, WM, WN, true><<<grid, WM * WN * 32, 0, s>>>(
                m, n, k, alpha, A.p + (boff ? 0 : b0 * sa), A.rs, A.cs, B.p + (boff ? 0 : b0 * sb), B.rs, B.cs,
                beta, C.p + (boff ? 0 : b0 * sc), C.rs, C.cs, uplo, sa, sb, sc, boff ? boff + 3 * b0 : nullptr,
                amode, bmode, kslice);
        else
            k_gemm_f64<BM, BN, WM, WN, false><<<grid, WM * WN * 32, 0, s>>>(
                m, n, k, alpha, A.p + (boff ? 0 : b0 * sa), A.rs, A.cs, B.p + (boff ? 0 : b0 * sb), B.rs, B.cs,
                beta, C.p + (boff ? 0 : b0 * sc), C.rs, C.cs, uplo, sa, sb, sc, boff ? boff + 3 * b0 : nullptr, 0, 0,
                kslice);
        DDLA_LAUNCHED();
    }
    return 0;
}

int g_sms = 0;
int sm_count() {
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 152;
    }
    return g_sms;
}

// Fraction of SM slots busy in the last wave when `tiles` equal tiles are
// spread over the SMs.
double balance(i64 tiles, int sms) {
    i64 waves = (tiles + sms - 1) / sms;
    return (double)tiles / (double)(waves * sms);
}

}  // namespace

static int gemm_f64_any(cudaStream_t s, i64 m, i64 n, i64 k, double alpha, View<const double> A,
                        View<const double> B, double beta, View<double> C, int uplo, i64 batch, i64 sa, i64 sb, i64 sc,
                        const i64 *boff, int amode = 0, int bmode = 0, i64 kslice = 0) {
    if (m <= 0 || n <= 0 || batch <= 0) return 0;
    if (k <= 0 || alpha == 0.0) {
        // C = beta*C on the requested part: reuse the kernel with k = 0.
        k = 0;
    }
    if (n <= 16)
        return launch_f64<128, 16, 4, 1>(s, m, n, k, alpha, A, B, beta, C, uplo, batch, sa, sb, sc, boff, amode, bmode, kslice);
    int sms = sm_count();
    i64 t64 = ((m + 63) / 64) * ((n + 63) / 64) * batch;
    i64 t32 = ((m + 31) / 32) * ((n + 63) / 64) * batch;
    i64 t3232 = ((m + 31) / 32) * ((n + 31) / 32) * batch;
    double b64 = balance(t64, sms), b32 = balance(t32, sms), b3232 = balance(t3232, sms);
    if (t64 >= 8 * sms || (b64 >= 0.9 && b64 >= b32 - 0.02))
        return launch_f64<64, 64, 2, 2>(s, m, n, k, alpha, A, B, beta, C, uplo, batch, sa, sb, sc, boff, amode, bmode, kslice);
    if (b32 >= 0.9 || b32 >= b3232 - 0.02)
        return launch_f64<32, 64, 2, 2>(s, m, n, k, alpha, A, B, beta, C, uplo, batch, sa, sb, sc, boff, amode, bmode, kslice);
    return launch_f64<32, 32, 2, 2>(s, m, n, k, alpha, A, B, beta, C, uplo, batch, sa, sb, sc, boff, amode, bmode, kslice);
}

int gemm_f64(cudaStream_t s, i64 m, i64 n, i64 k, double alpha, View<const double> A, View<const double> B,
             double beta, View<double> C, int uplo, i64 batch, i64 sa, i64 sb, i64 sc) {
    return gemm_f64_any(s, m, n, k, alpha, A, B, beta, C, uplo, batch, sa, sb, sc, nullptr);
}

// C = alpha*A*B + beta*C where A and / or B is structured (amode / bmode: OP_SYM
// or OP_TRI, plus OP_LOWER for the stored / nonzero triangle and OP_UNIT for an
// implicit unit diagonal that is never read).  A symmetric operand is square; a
// triangular one may be trapezoidal (the block of Householder vectors of a QR
// panel is unit-lower trapezoidal), the triangle being the one of element
// (i, j) with j <= i (lower) or j >= i (upper).
int gemm_f64_struct(cudaStream_t s, i64 m, i64 n, i64 k, double alpha, View<const double> A, int amode,
                    View<const double> B, int bmode, double beta, View<double> C, int uplo) {
    if (((amode & 3) == OP_SYM && k != m) || ((bmode & 3) == OP_SYM && k != n)) {
        set_error("gemm_f64_struct: symmetric operand must be square");
        return DDLA_ERR_UNSUPPORTED;
    }
    return gemm_f64_any(s, m, n, k, alpha, A, B, beta, C, uplo, 1, 0, 0, 0, nullptr, amode, bmode);
}

namespace {
// C = alpha * sum_z P_z + beta * C on C's triangle (the partials P_z are m x n
// row-major, z ascending).
__global__ void k_splitk_reduce(i64 m, i64 n, int parts, const double *__restrict__ P, double alpha, double beta,
                                double *C, i64 rsc, i64 csc, int uplo) {
    const i64 tot = m * n;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        const i64 i = e / n, j = e % n;
        if (uplo == DDLA_LOWER && j > i) continue;
        if (uplo == DDLA_UPPER && j < i) continue;
        double acc = 0.0;
        for (int z = 0; z < parts; z++) acc += P[z * tot + e];
        double *cp = C + i * rsc + j * csc;
        const double v = alpha * acc;
        *cp = (beta == 0.0) ? v : fma(beta, *cp, v);
    }
}
}  // namespace

int gemm_f64_struct_h(ddla_handle h, i64 m, i64 n, i64 k, double alpha, View<const double> A, int amode,
                      View<const double> B, int bmode, double beta, View<double> C, int uplo) {
    if (m <= 0 || n <= 0) return 0;
    const int sms = sm_count();
    // tiles of the configuration gemm_f64_any picks for this shape (an upper
    // bound for a triangular C)
    const i64 tiles = n <= 16 ? (m + 127) / 128 : ((m + 31) / 32) * ((n + 63) / 64);
    // k-slices: at least ~2 CTAs per SM, at most ~6 (every configuration keeps
    // 7 or more resident, so all slices run in one wave); among those, the
    // count whose CTAs spread most evenly over the SMs (tiles * parts close to
    // a multiple of the SM count), the smallest on ties
    i64 parts = 1;
    if (alpha != 0.0 && k >= 1024 && tiles < sms) {
        i64 lo = (2 * sms + tiles - 1) / tiles, hi = (6 * sms) / tiles;
        const i64 cap = k / 128 < 64 ? k / 128 : 64;
        if (hi > cap) hi = cap;
        if (lo > hi) lo = hi;
        double best = -1.0;
        for (i64 p = lo; p <= hi; p++) {
            const i64 ctas = tiles * p, per = (ctas + sms - 1) / sms;
            const double balance = (double)ctas / (double)(per * sms);
            if (balance > best + 1e-9) {
                best = balance;
                parts = p;
            }
        }
    }
    if (parts < 2) return gemm_f64_struct(h->stream, m, n, k, alpha, A, amode, B, bmode, beta, C, uplo);
    if ((amode & 3) == OP_SYM || (bmode & 3) == OP_SYM) {
        if (k != ((amode & 3) == OP_SYM ? m : n)) {
            set_error("gemm_f64_struct: symmetric operand must be square");
            return DDLA_ERR_UNSUPPORTED;
        }
    }
    i64 kslice = (k + parts - 1) / parts;
    kslice = (kslice + 15) / 16 * 16;
    parts = (k + kslice - 1) / kslice;
    void *ws;
    DDLA_TRY(workspace(h, WS_SPLIT, sizeof(double) * (size_t)(parts * m * n), &ws));
    double *P = (double *)ws;
    DDLA_TRY(gemm_f64_any(h->stream, m, n, k, 1.0, A, B, 0.0, View<double>{P, m, n, n, 1}, uplo, parts, 0, 0, m * n,
                          nullptr, amode, bmode, kslice));
    const i64 tot = m * n;
    const i64 blocks = (tot + 255) / 256 < 2048 ? (tot + 255) / 256 : 2048;
    k_splitk_reduce<<<(unsigned)blocks, 256, 0, h->stream>>>(m, n, (int)parts, P, alpha, beta, C.p, C.rs, C.cs,
                                                               uplo);
    DDLA_LAUNCHED();
    return 0;
}

// Batched GEMM whose problem z starts at element offsets d_offsets[3z..3z+2]
// of A, B and C (batch index tables of an einsum).
int gemm_f64_offsets(cudaStream_t s, i64 m, i64 n, i64 k, double alpha, View<const double> A,
                     View<const double> B, double beta, View<double> C, i64 batch, const i64 *d_offsets) {
    return gemm_f64_any(s, m, n, k, alpha, A, B, beta, C, DDLA_DENSE, batch, 0, 0, 0, d_offsets);
}

// ------------------------------------------------------------------ FP32
namespace {

constexpr int SBM = 128, SBN = 128, SBK = 8;

// C = alpha*A*B + beta*C, 256 threads, each thread an 8x8 block split in two
// 4-row and two 4-column halves (rows ty*4 and 64+ty*4, cols tx*4 and 64+tx*4)
// so shared-memory reads are conflict-free float4 broadcasts.
__global__ void __launch_bounds__(256)
    k_sgemm(i64 m, i64 n, i64 k, float alpha, const float *__restrict__ A, i64 rsa, i64 csa,
            const float *__restrict__ B, i64 rsb, i64 csb, float beta, float *C, i64 rsc, i64 csc, int uplo) {
    __shared__ __align__(16) float As[2][SBK][SBM];
    __shared__ __align__(16) float Bs[2][SBK][SBN];
    const i64 m0 = (i64)blockIdx.y * SBM, n0 = (i64)blockIdx.x * SBN;
    if (uplo == DDLA_LOWER && n0 > m0 + SBM - 1) return;
    if (uplo == DDLA_UPPER && m0 > n0 + SBN - 1) return;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;

    // Loader mapping: A tile 128x8 = 1024 elements, 4 per thread.
    //   K-contiguous A: thread -> row tid/2, k (tid&1)*4 .. +3
    //   otherwise:      thread -> k tid/32, rows (tid&31)*4 .. +3
    // B tile 8x128: N-contiguous: k tid/32, cols (tid&31)*4..+3; else col tid/2, k (tid&1)*4..
    const bool a_k = (csa == 1), b_n = (csb == 1);
    float ra[4], rb[4];
    auto load = [&](i64 k0) {
#pragma unroll
        for (int e = 0; e < 4; e++) {
            int r, kk;
            if (a_k) { r = tid >> 1; kk = (tid & 1) * 4 + e; } else { kk = tid >> 5; r = (tid & 31) * 4 + e; }
            i64 gr = m0 + r, gk = k0 + kk;
            ra[e] = (gr < m && gk < k) ? A[gr * rsa + gk * csa] : 0.f;
            int c;
            if (b_n) { kk = tid >> 5; c = (tid & 31) * 4 + e; } else { c = tid >> 1; kk = (tid & 1) * 4 + e; }
            i64 gc = n0 + c;
            gk = k0 + kk;
            rb[e] = (gc < n && gk < k) ? B[gk * rsb + gc * csb] : 0.f;
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int e = 0; e < 4; e++) {
            int r, kk;
            if (a_k) { r = tid >> 1; kk = (tid & 1) * 4 + e; } else { kk = tid >> 5; r = (tid & 31) * 4 + e; }
            As[buf][kk][r] = ra[e];
            int c;
            if (b_n) { kk = tid >> 5; c = (tid & 31) * 4 + e; } else { c = tid >> 1; kk = (tid & 1) * 4 + e; }
            Bs[buf][kk][c] = rb[e];
        }
    };

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = 0.f;

    int buf = 0;
    if (k > 0) {
        load(0);
        store(0);
    }
    __syncthreads();
    for (i64 k0 = 0; k0 < k; k0 += SBK) {
        bool more = k0 + SBK < k;
        if (more) load(k0 + SBK);
#pragma unroll
        for (int kk = 0; kk < SBK; kk++) {
            float4 a0 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4]);
            float4 a1 = *reinterpret_cast<const float4 *>(&As[buf][kk][64 + ty * 4]);
            float4 b0 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4]);
            float4 b1 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][64 + tx * 4]);
            float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        if (more) {
            store(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        i64 gr = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
        if (gr >= m) continue;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            i64 gc = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
            if (gc >= n) continue;
            if (uplo == DDLA_LOWER && gc > gr) continue;
            if (uplo == DDLA_UPPER && gc < gr) continue;
            float *cp = C + gr * rsc + gc * csc;
            float v = alpha * acc[i][j];
            *cp = (beta == 0.f) ? v : fmaf(beta, *cp, v);
        }
    }
}

// Rank-k update C += alpha * A * B for k <= 64 (the trailing updates of the
// FP32 factorizations): the 128 x 128 tile of C is loaded straight into the
// accumulators at the start (16 float4 loads per thread, in flight together
// with the A and B tiles), the whole K range of A and B is staged once, and
// the tile goes back with float4 stores.  Needs row-major C, A and B with
// 16-byte aligned rows.
constexpr int UK = 64;
// TN = 128 (256 threads) or 64 (128 threads, four CTAs per SM): the thread's
// 8 x 8 block is rows ty*4..+3 and 64+ty*4..+3, columns tx*4..+3 and
// TN/2+tx*4..+3
template <int TN>
__global__ void __launch_bounds__(TN * 2, TN == 128 ? 2 : 4)
    k_supdate(i64 m, i64 n, int k, float alpha, const float *__restrict__ A, i64 rsa, const float *__restrict__ B,
              i64 rsb, float *C, i64 rsc, int uplo) {
    constexpr int NT = TN * 2, TXN = TN / 8, HN = TN / 2;
    extern __shared__ __align__(16) float upd_smem[];
    float (*As)[SBM] = reinterpret_cast<float (*)[SBM]>(upd_smem);
    float (*Bs)[TN] = reinterpret_cast<float (*)[TN]>(upd_smem + UK * SBM);
    const i64 m0 = (i64)blockIdx.y * SBM, n0 = (i64)blockIdx.x * TN;
    if (uplo == DDLA_LOWER && n0 > m0 + SBM - 1) return;
    if (uplo == DDLA_UPPER && m0 > n0 + TN - 1) return;
    const int tid = threadIdx.x, tx = tid % TXN, ty = tid / TXN;
    float acc[8][8];
    // C tile into the accumulators
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const i64 gr = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const i64 gc = n0 + h * HN + tx * 4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (gr < m) {
                const float *cp = C + gr * rsc + gc;
                if (gc + 3 < n) {
                    v = *reinterpret_cast<const float4 *>(cp);
                } else {
                    float t[4] = {0.f, 0.f, 0.f, 0.f};
                    for (int e = 0; e < 4; e++)
                        if (gc + e < n) t[e] = cp[e];
                    v = make_float4(t[0], t[1], t[2], t[3]);
                }
            }
            acc[i][h * 4 + 0] = v.x;
            acc[i][h * 4 + 1] = v.y;
            acc[i][h * 4 + 2] = v.z;
            acc[i][h * 4 + 3] = v.w;
        }
    }
    // A tile (128 x k, K-contiguous rows) transposed into As[k][row], scaled
    // by alpha; consecutive threads take consecutive rows, so the transposed
    // stores hit different banks.  B tile (k x TN) into Bs[k][col].
    for (int e = tid; e < SBM * (UK / 4); e += NT) {
        const int r = e % SBM, kq = (e / SBM) * 4;
        const i64 gr = m0 + r;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gr < m && kq < k) {
            const float *ap = A + gr * rsa + kq;
            if (kq + 3 < k) {
                v = *reinterpret_cast<const float4 *>(ap);
            } else {
                float t[4] = {0.f, 0.f, 0.f, 0.f};
                for (int x = 0; x < 4; x++)
                    if (kq + x < k) t[x] = ap[x];
                v = make_float4(t[0], t[1], t[2], t[3]);
            }
        }
        As[kq + 0][r] = alpha * v.x;
        As[kq + 1][r] = alpha * v.y;
        As[kq + 2][r] = alpha * v.z;
        As[kq + 3][r] = alpha * v.w;
    }
    for (int e = tid; e < UK * (TN / 4); e += NT) {
        const int kk = e / (TN / 4), c = (e % (TN / 4)) * 4;
        const i64 gc = n0 + c;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (kk < k && gc < n) {
            const float *bp = B + (i64)kk * rsb + gc;
            if (gc + 3 < n) {
                v = *reinterpret_cast<const float4 *>(bp);
            } else {
                float t[4] = {0.f, 0.f, 0.f, 0.f};
                for (int x = 0; x < 4; x++)
                    if (gc + x < n) t[x] = bp[x];
                v = make_float4(t[0], t[1], t[2], t[3]);
            }
        }
        *reinterpret_cast<float4 *>(&Bs[kk][c]) = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < UK; kk++) {
        const float4 a0 = *reinterpret_cast<const float4 *>(&As[kk][ty * 4]);
        const float4 a1 = *reinterpret_cast<const float4 *>(&As[kk][64 + ty * 4]);
        const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[kk][tx * 4]);
        const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[kk][HN + tx * 4]);
        const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const i64 gr = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
        if (gr >= m) continue;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const i64 gc = n0 + h * HN + tx * 4;
            float *cp = C + gr * rsc + gc;
            if (uplo == DDLA_DENSE && gc + 3 < n) {
                *reinterpret_cast<float4 *>(cp) =
                    make_float4(acc[i][h * 4], acc[i][h * 4 + 1], acc[i][h * 4 + 2], acc[i][h * 4 + 3]);
            } else {
                for (int e = 0; e < 4; e++) {
                    if (gc + e >= n) break;
                    if (uplo == DDLA_LOWER && gc + e > gr) continue;
                    if (uplo == DDLA_UPPER && gc + e < gr) continue;
                    cp[e] = acc[i][h * 4 + e];
                }
            }
        }
    }
}

template <int TN>
int launch_supdate(cudaStream_t s, i64 m, i64 n, int k, float alpha, View<const float> A, View<const float> B,
                   View<float> C, int uplo) {
    constexpr size_t sm = sizeof(float) * UK * (SBM + TN);
    static bool attr = false;
    if (!attr) {
        DDLA_CUDA(cudaFuncSetAttribute(k_supdate<TN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        attr = true;
    }
    const i64 gx = (n + TN - 1) / TN, gy = (m + SBM - 1) / SBM;
    k_supdate<TN><<<dim3((unsigned)gx, (unsigned)gy), TN * 2, sm, s>>>(m, n, k, alpha, A.p, A.rs, B.p, B.rs, C.p,
                                                                      C.rs, uplo);
    DDLA_LAUNCHED();
    return 0;
}

}  // namespace

int gemm_f32(cudaStream_t s, i64 m, i64 n, i64 k, float alpha, View<const float> A, View<const float> B,
             float beta, View<float> C, int uplo) {
    if (m <= 0 || n <= 0) return 0;
    if (k < 0 || alpha == 0.f) k = 0;
    i64 gx = (n + SBN - 1) / SBN, gy = (m + SBM - 1) / SBM;
    if (gy > 65535) { set_error("gemm_f32: m too large"); return DDLA_ERR_UNSUPPORTED; }
    auto al16 = [](const void *p, i64 rs) { return ((((uintptr_t)p) & 15) == 0) && (rs & 3) == 0; };
    if (beta == 1.f && k > 0 && k <= UK && C.cs == 1 && A.cs == 1 && B.cs == 1 && al16(C.p, C.rs) &&
        al16(A.p, A.rs) && al16(B.p, B.rs)) {
        if (tune_get("update.tn", 128) == 64) return launch_supdate<64>(s, m, n, (int)k, alpha, A, B, C, uplo);
        return launch_supdate<128>(s, m, n, (int)k, alpha, A, B, C, uplo);
        return 0;
    }
    k_sgemm<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(m, n, k, alpha, A.p, A.rs, A.cs, B.p, B.rs, B.cs,
                                                            beta, C.p, C.rs, C.cs, uplo);
    DDLA_LAUNCHED();
    return 0;
}

}  // namespace ddla
