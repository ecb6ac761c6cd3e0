// Mixed-precision solves: LU / Cholesky in FP32 storage (trailing updates on
// FP32 CUDA cores or 3xTF32 / 3xBF16 tcgen05 tensor cores), then classical
// iterative refinement with everything that decides accuracy in FP64 on the
// GPU: the residual r = b - A x, the solution update x += d, and the
// backward-error test
//     max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf) <= tol.
// Only the correction solve (A d = r with the FP32 factors) runs in FP32.
#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "convert.cuh"
#include "timing.cuh"

namespace ddla {


namespace {

constexpr int MAX_RHS = 16;

__global__ void k_d2s(const double *X, i64 n, float *Y) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
        Y[e] = (float)X[e];
}
__global__ void k_s2d_add(const float *D, i64 n, double *X) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
        X[e] += (double)D[e];
}
__global__ void k_s2d(const float *D, i64 n, double *X) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
        X[e] = (double)D[e];
}

// r = b - A x for row-major A (n x n, lda), X/B/R n x nrhs row-major; one warp
// per row.  Also writes |r| row maxima per column into rowmax (for the norm).
template <int NR>
__global__ void __launch_bounds__(256)
    k_residual(i64 n, const double *__restrict__ A, i64 lda, const double *__restrict__ X,
               const double *__restrict__ B, double *R) {
    const int lane = threadIdx.x & 31;
    const i64 row = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
    if (row >= n) return;
    double acc[NR];
#pragma unroll
    for (int c = 0; c < NR; c++) acc[c] = 0.0;
    const double *ar = A + row * lda;
    for (i64 j = lane; j < n; j += 32) {
        double a = ar[j];
#pragma unroll
        for (int c = 0; c < NR; c++) acc[c] = fma(a, X[j * NR + c], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < NR; c++) {
        double v = acc[c];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        acc[c] = v;
    }
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < NR; c++) R[row * NR + c] = B[row * NR + c] - acc[c];
}

// Column-wise max |X[:, c]| over rows (atomicMax on the bit pattern of the
// non-negative double).
__global__ void k_colmax_abs(const double *X, i64 n, int nr, unsigned long long *out) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n * nr; e += (i64)gridDim.x * blockDim.x) {
        double v = fabs(X[e]);
        if (v == v) atomicMax(&out[e % nr], (unsigned long long)__double_as_longlong(v));
    }
}

// The FP32 copy of A (row-major n x n) and, in the same pass over A,
// ||A||_inf (out[0]) and max |a_ij| (out[1], NaN ignored), as bit patterns of
// non-negative doubles.  One warp per row.  No FP64 arithmetic per entry (it
// runs at 1/64 of the FP32 rate on GB300): the copy is rounded on the integer
// pipes (d2f_bits), max |a_ij| is an integer max of the FP64 bit patterns
// (exact), and the row sums add FP32 partial sums of 16 magnitudes of the
// FP32 copy into FP64 (relative error below 1e-6).  A row with an entry beyond
// the FP32 range (an infinite copy) is summed again in FP64.
__global__ void k_d2s_norms(i64 n, const double *A, i64 lda, float *A32, unsigned long long *out) {
    const int lane = threadIdx.x & 31;
    const i64 row = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
    if (row >= n) return;
    double s = 0.0;
    float fs = 0.f;   // partial sum of up to 16 magnitudes
    int cnt = 0;
    unsigned long long mx = 0;
    bool wide = false;
    const double *a = A + row * lda;
    float *y = A32 + row * n;
    // the FP32 copy of one entry; its magnitude goes to the partial sum
    auto conv = [&](double v) -> float {
        const unsigned long long b = (unsigned long long)__double_as_longlong(v), ab = b & 0x7FFFFFFFFFFFFFFFull;
        const unsigned f = d2f_bits(b);
        if (ab <= 0x7FF0000000000000ull) mx = ab > mx ? ab : mx;
        wide |= ab < 0x7FF0000000000000ull && (f & 0x7FFFFFFFu) == 0x7F800000u;
        return __uint_as_float(f);
    };
    if ((n & 3) == 0 && (lda & 3) == 0 && ((((uintptr_t)A) | ((uintptr_t)A32)) & 31) == 0) {
        // 4 consecutive entries per lane: two 16-byte loads, one 16-byte store
#pragma unroll 2
        for (i64 j = 4 * lane; j < n; j += 128) {
            const double2 v0 = *reinterpret_cast<const double2 *>(a + j);
            const double2 v1 = *reinterpret_cast<const double2 *>(a + j + 2);
            const float f0 = conv(v0.x), f1 = conv(v0.y), f2 = conv(v1.x), f3 = conv(v1.y);
            *reinterpret_cast<float4 *>(y + j) = make_float4(f0, f1, f2, f3);
            fs += (fabsf(f0) + fabsf(f1)) + (fabsf(f2) + fabsf(f3));
            if (++cnt == 4) {
                s += (double)fs;
                fs = 0.f;
                cnt = 0;
            }
        }
    } else {
#pragma unroll 4
        for (i64 j = lane; j < n; j += 32) {
            const float f = conv(a[j]);
            y[j] = f;
            fs += fabsf(f);
            if (++cnt == 16) {
                s += (double)fs;
                fs = 0.f;
                cnt = 0;
            }
        }
    }
    s += (double)fs;
    if (__any_sync(0xffffffffu, wide)) {
        s = 0.0;
        for (i64 j = lane; j < n; j += 32) s += fabs(a[j]);
    }
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, off);
        const unsigned long long o = __shfl_down_sync(0xffffffffu, mx, off);
        mx = o > mx ? o : mx;
    }
    if (lane == 0) {
        atomicMax(&out[0], (unsigned long long)__double_as_longlong(s));
        atomicMax(&out[1], mx);
    }
}

// ||A||_inf = max_i sum_j |a_ij| (row-major), one warp per row.
__global__ void k_norm_inf(i64 n, const double *A, i64 lda, unsigned long long *out) {
    const int lane = threadIdx.x & 31;
    const i64 row = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
    if (row >= n) return;
    double s = 0.0;
    for (i64 j = lane; j < n; j += 32) s += fabs(A[row * lda + j]);
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) atomicMax(out, (unsigned long long)__double_as_longlong(s));
}

// Pivot agreement of the mixed LU with a reference pivot vector (both in
// DDLA's relative convention, LU.cs:367-374): out[0] counts the equal
// entries, out[1] is the first index where they differ (INT_MAX if none).
__global__ void k_piv_cmp(const int32_t *piv, const int32_t *ref, i64 n, int *out) {
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        if (piv[i] == ref[i]) atomicAdd(&out[0], 1);
        else atomicMin(&out[1], (int)i);
    }
}

// Max |x - xr| and |xr| per column.
__global__ void k_fwd_err(const double *X, const double *XR, i64 n, int nr, unsigned long long *out) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n * nr; e += (i64)gridDim.x * blockDim.x) {
        double d = fabs(X[e] - XR[e]), r = fabs(XR[e]);
        atomicMax(&out[0], (unsigned long long)__double_as_longlong(d));
        atomicMax(&out[1], (unsigned long long)__double_as_longlong(r));
    }
}

// ---- GMRES building blocks (FP64, one right-hand side)
// y = A x, row-major A (n x n), one warp per row
__global__ void __launch_bounds__(256) k_matvec(i64 n, const double *__restrict__ A, const double *__restrict__ x,
                                               double *y) {
    const int lane = threadIdx.x & 31;
    const i64 row = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
    if (row >= n) return;
    const double *ar = A + row * n;
    double acc = 0.0;
    for (i64 j = lane; j < n; j += 32) acc = fma(ar[j], x[j], acc);
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (lane == 0) y[row] = acc;
}
__device__ __forceinline__ double block_sum(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
    return t;
}
// h[i] = V_i . w for the first kk columns of V (ld n), one block per column
__global__ void __launch_bounds__(512) k_dots(const double *V, const double *w, i64 n, double *h) {
    __shared__ double red[16];
    const double *v = V + (i64)blockIdx.x * n;
    double s = 0.0;
    for (i64 e = threadIdx.x; e < n; e += blockDim.x) s = fma(v[e], w[e], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) h[blockIdx.x] = s;
}
// w -= V h (kk columns)
__global__ void k_sub_vh(double *w, const double *V, const double *h, int kk, i64 n) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x) {
        double v = w[e];
        for (int i = 0; i < kk; i++) v = fma(-h[i], V[(i64)i * n + e], v);
        w[e] = v;
    }
}
// out = ||w||_2 (one block)
__global__ void __launch_bounds__(1024) k_nrm2(const double *w, i64 n, double *out) {
    __shared__ double red[32];
    double s = 0.0;
    for (i64 e = threadIdx.x; e < n; e += blockDim.x) s = fma(w[e], w[e], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) *out = sqrt(s);
}
// v = w / *nrm
__global__ void k_scale_by(const double *w, const double *nrm, i64 n, double *v) {
    const double inv = 1.0 / *nrm;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x)
        v[e] = w[e] * inv;
}
// x += V y (kk columns)
__global__ void k_add_vy(double *x, const double *V, const double *y, int kk, i64 n) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x) {
        double v = x[e];
        for (int i = 0; i < kk; i++) v = fma(y[i], V[(i64)i * n + e], v);
        x[e] = v;
    }
}

int grid1(i64 tot) {
    i64 g = (tot + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 16384 ? 16384 : g));
}

template <int NR>
int residual_nr(cudaStream_t s, i64 n, const double *A, const double *X, const double *B, double *R) {
    unsigned grid = (unsigned)((n * 32 + 255) / 256);
    k_residual<NR><<<grid, 256, 0, s>>>(n, A, n, X, B, R);
    DDLA_LAUNCHED();
    return 0;
}

int residual(ddla_handle h, i64 n, int nr, const double *A, const double *X, const double *B, double *R) {
    cudaStream_t s = h->stream;
    switch (nr) {
        case 1: return residual_nr<1>(s, n, A, X, B, R);
        case 2: return residual_nr<2>(s, n, A, X, B, R);
        default: break;
    }
    // 3 or more right-hand sides: FP64 GEMM on the DMMA path (R = B - A X),
    // k split over extra CTAs when the n x nr result has few tiles (the
    // row-sum kernel above reaches ~0.55 of the FP64 peak at 16 columns)
    DDLA_CUDA(cudaMemcpyAsync(R, B, sizeof(double) * n * nr, cudaMemcpyDeviceToDevice, s));
    return gemm_f64_struct_h(h, n, nr, n, -1.0, View<const double>{A, n, n, n, 1}, OP_DENSE,
                             View<const double>{X, n, nr, nr, 1}, OP_DENSE, 1.0, View<double>{R, n, nr, nr, 1});
}

double u64d(unsigned long long v) { return __builtin_bit_cast(double, v); }

}  // namespace

constexpr int GM_MAX = 30;

// One cycle of flexible GMRES(m) on A x = b, right-preconditioned by the
// FP32 factors (z = M^-1 v = solve32(FP32(v))): starting from r = b - A x (in
// R), it builds V (orthonormal, FP64, classical Gram-Schmidt applied twice)
// and Z = M^-1 V, minimises ||b - A (x + Z y)||_2 with Givens rotations on the
// host and adds Z y to x.  A z is formed in FP64, so the FP32 preconditioner
// limits only the speed, not the attainable accuracy.  Stops when the
// residual estimate is below `target` (2-norm, which bounds the inf-norm) or
// after m steps.  *used = preconditioner applications made.
template <typename F>
int gmres_cycle(ddla_handle h, i64 n, const double *A, const double *R, double *X, F &solve32, float *d32,
                double *V, double *Z, double *W, double *hd, int m, double target, int *used) {
    cudaStream_t s = h->stream;
    const unsigned gv = (unsigned)((n * 32 + 255) / 256);
    *used = 0;
    k_nrm2<<<1, 1024, 0, s>>>(R, n, hd);
    DDLA_LAUNCHED();
    double beta = 0.0;
    DDLA_CUDA(cudaMemcpyAsync(&beta, hd, sizeof(double), cudaMemcpyDeviceToHost, s));
    DDLA_CUDA(cudaStreamSynchronize(s));
    if (!(beta > 0.0) || !std::isfinite(beta)) return 0;
    k_scale_by<<<grid1(n), 256, 0, s>>>(R, hd, n, V);
    DDLA_LAUNCHED();
    std::vector<double> H((size_t)(m + 1) * m, 0.0), g(m + 1, 0.0), cs(m, 0.0), sn(m, 0.0), col(2 * (m + 1) + 2);
    g[0] = beta;
    int kk = 0;
    for (int k = 0; k < m; k++) {
        double *vk = V + (size_t)k * n, *vn = V + (size_t)(k + 1) * n, *zk = Z + (size_t)k * n;
        // z_k = M^-1 v_k, w = A z_k
        k_d2s<<<grid1(n), 256, 0, s>>>(vk, n, d32);
        DDLA_LAUNCHED();
        DDLA_TRY(solve32(d32));
        k_s2d<<<grid1(n), 256, 0, s>>>(d32, n, zk);
        DDLA_LAUNCHED();
        (*used)++;
        k_matvec<<<gv, 256, 0, s>>>(n, A, zk, W);
        DDLA_LAUNCHED();
        for (int pass = 0; pass < 2; pass++) {
            k_dots<<<k + 1, 512, 0, s>>>(V, W, n, hd + pass * (m + 1));
            DDLA_LAUNCHED();
            k_sub_vh<<<grid1(n), 256, 0, s>>>(W, V, hd + pass * (m + 1), k + 1, n);
            DDLA_LAUNCHED();
        }
        k_nrm2<<<1, 1024, 0, s>>>(W, n, hd + 2 * (m + 1));
        DDLA_LAUNCHED();
        DDLA_CUDA(cudaMemcpyAsync(col.data(), hd, sizeof(double) * (2 * (m + 1) + 1), cudaMemcpyDeviceToHost, s));
        DDLA_CUDA(cudaStreamSynchronize(s));
        double *hc = &H[(size_t)k * (m + 1)];   // column k of H, m+1 entries
        for (int i = 0; i <= k; i++) hc[i] = col[i] + col[(m + 1) + i];
        const double hn = col[2 * (m + 1)];
        hc[k + 1] = hn;
        kk = k + 1;
        for (int i = 0; i < k; i++) {
            const double t = cs[i] * hc[i] + sn[i] * hc[i + 1];
            hc[i + 1] = -sn[i] * hc[i] + cs[i] * hc[i + 1];
            hc[i] = t;
        }
        const double rr = std::hypot(hc[k], hc[k + 1]);
        cs[k] = rr > 0 ? hc[k] / rr : 1.0;
        sn[k] = rr > 0 ? hc[k + 1] / rr : 0.0;
        hc[k] = rr;
        hc[k + 1] = 0.0;
        g[k + 1] = -sn[k] * g[k];
        g[k] = cs[k] * g[k];
        if (!(hn > 0.0) || !std::isfinite(hn) || std::fabs(g[k + 1]) <= target) break;
        k_scale_by<<<grid1(n), 256, 0, s>>>(W, hd + 2 * (m + 1), n, vn);
        DDLA_LAUNCHED();
    }
    std::vector<double> y(kk, 0.0);
    for (int i = kk - 1; i >= 0; i--) {
        double t = g[i];
        for (int j = i + 1; j < kk; j++) t -= H[(size_t)j * (m + 1) + i] * y[j];
        const double d = H[(size_t)i * (m + 1) + i];
        y[i] = d != 0.0 ? t / d : 0.0;
    }
    DDLA_CUDA(cudaMemcpyAsync(hd, y.data(), sizeof(double) * kk, cudaMemcpyHostToDevice, s));
    k_add_vy<<<grid1(n), 256, 0, s>>>(X, Z, hd, kk, n);
    DDLA_LAUNCHED();
    DDLA_CUDA(cudaStreamSynchronize(s));   // y lives on this stack frame
    return 0;
}

// Shared refinement loop.  `solve32(d)` overwrites the FP32 right-hand side d
// (n x nr) with the correction.
template <typename F>
int refine(ddla_handle h, i64 n, int nr, const double *A, const double *B, double *X, const double *x_ref,
           const ddla_opts *opts, ddla_solve_report *rep, F solve32, float *d32, double *R,
           unsigned long long *norms, const unsigned long long *anorm = nullptr) {
    cudaStream_t s = h->stream;
    const int max_iter = (opts && opts->max_iter) ? opts->max_iter : 30;
    const double tol = (opts && opts->tol > 0) ? opts->tol : 1e-14;
    const i64 tot = n * nr;
    // norms[0] = ||A||_inf, [1..nr] = ||b_j||, [1+nr .. 1+2nr) = ||x_j||, [1+2nr .. 1+3nr) = ||r_j||
    DDLA_CUDA(cudaMemsetAsync(norms, 0, sizeof(unsigned long long) * (1 + 3 * MAX_RHS + 2), s));
    if (anorm) {   // formed with the FP32 copy of A
        DDLA_CUDA(cudaMemcpyAsync(norms, anorm, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s));
    } else {
        k_norm_inf<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(n, A, n, norms);
        DDLA_LAUNCHED();
    }
    k_colmax_abs<<<grid1(tot), 256, 0, s>>>(B, n, nr, norms + 1);
    DDLA_LAUNCHED();
    // x0 = LU \ b
    k_d2s<<<grid1(tot), 256, 0, s>>>(B, tot, d32);
    DDLA_LAUNCHED();
    DDLA_TRY(solve32(d32));
    k_s2d<<<grid1(tot), 256, 0, s>>>(d32, tot, X);
    DDLA_LAUNCHED();
    int it = 0;
    double berr = INFINITY;
    const int iters = max_iter < 0 ? 0 : max_iter;
    // flexible GMRES for one right-hand side (tuning key refine.gmres, on by
    // default); classical refinement otherwise
    const bool gm = nr == 1 && tune_get("refine.gmres", 1) != 0;
    const int gm_m = (int)std::max<int64_t>(2, std::min<int64_t>(GM_MAX, tune_get("refine.gmres.m", 10)));
    double *gV = nullptr, *gZ = nullptr, *gW = nullptr, *gh = nullptr;
    if (gm) {
        DDLA_TRY(workspace(h, WS_Y, sizeof(double) * ((size_t)(2 * GM_MAX + 2) * n + 4 * GM_MAX + 8), (void **)&gV));
        gZ = gV + (size_t)(GM_MAX + 1) * n;
        gW = gZ + (size_t)GM_MAX * n;
        gh = gW + n;
    }
    std::vector<unsigned long long> hn(1 + 3 * MAX_RHS);
    for (;;) {
        {
            Timed t(s, TC_REFINE, 2.0 * n * n * nr, 8.0 * n * n);
            DDLA_TRY(residual(h, n, nr, A, X, B, R));
        }
        DDLA_CUDA(cudaMemsetAsync(norms + 1 + nr, 0, sizeof(unsigned long long) * 2 * nr, s));
        k_colmax_abs<<<grid1(tot), 256, 0, s>>>(X, n, nr, norms + 1 + nr);
        DDLA_LAUNCHED();
        k_colmax_abs<<<grid1(tot), 256, 0, s>>>(R, n, nr, norms + 1 + 2 * nr);
        DDLA_LAUNCHED();
        DDLA_CUDA(cudaMemcpyAsync(hn.data(), norms, sizeof(unsigned long long) * (1 + 3 * nr),
                                  cudaMemcpyDeviceToHost, s));
        DDLA_CUDA(cudaStreamSynchronize(s));
        double an = u64d(hn[0]);
        berr = 0.0;
        for (int c = 0; c < nr; c++) {
            double bn = u64d(hn[1 + c]), xn = u64d(hn[1 + nr + c]), rn = u64d(hn[1 + 2 * nr + c]);
            double den = an * xn + bn;
            double e = den > 0 ? rn / den : (rn > 0 ? INFINITY : 0.0);
            if (!(e <= berr)) berr = e;  // NaN propagates
        }
        if (berr <= tol || it >= iters) break;
        if (gm) {
            // one restart cycle of flexible GMRES from the current x, aiming
            // straight at the backward-error target
            int used = 0;
            double an = u64d(hn[0]), xn = u64d(hn[1 + nr]), bn = u64d(hn[1]);
            // the cycle stops on the residual's 2-norm, which bounds the
            // inf-norm of the backward error from above by up to sqrt(n); the
            // target is relaxed by min(16, sqrt(n) / 4) (tuning key
            // refine.gmres.relax), and the loop re-checks the true backward
            // error, so a residual that is not spread out only costs a cycle
            const int64_t rk = tune_get("refine.gmres.relax", 0);
            const double relax = rk > 0 ? (double)rk : std::min(16.0, std::max(1.0, std::sqrt((double)n) / 4.0));
            const double target = 0.5 * tol * (an * xn + bn) * relax;
            DDLA_TRY(gmres_cycle(h, n, A, R, X, solve32, d32, gV, gZ, gW, gh, gm_m, target, &used));
            it += used;
        } else {
            k_d2s<<<grid1(tot), 256, 0, s>>>(R, tot, d32);
            DDLA_LAUNCHED();
            DDLA_TRY(solve32(d32));
            k_s2d_add<<<grid1(tot), 256, 0, s>>>(d32, tot, X);
            DDLA_LAUNCHED();
            it++;
        }
    }
    rep->iterations = it;
    rep->backward_error = berr;
    rep->converged = berr <= tol;
    rep->forward_error = -1.0;
    if (x_ref) {
        DDLA_CUDA(cudaMemsetAsync(norms + 1 + 3 * MAX_RHS, 0, 2 * sizeof(unsigned long long), s));
        k_fwd_err<<<grid1(tot), 256, 0, s>>>(X, x_ref, n, nr, norms + 1 + 3 * MAX_RHS);
        DDLA_LAUNCHED();
        unsigned long long fe[2];
        DDLA_CUDA(cudaMemcpyAsync(fe, norms + 1 + 3 * MAX_RHS, sizeof(fe), cudaMemcpyDeviceToHost, s));
        DDLA_CUDA(cudaStreamSynchronize(s));
        double rn = u64d(fe[1]);
        rep->forward_error = rn > 0 ? u64d(fe[0]) / rn : u64d(fe[0]);
    }
    if (!rep->converged) {
        set_error("iterative refinement did not reach the backward-error tolerance");
        return DDLA_ERR_NOT_CONVERGED;
    }
    return 0;
}

// ---- growth monitor: FP64 figures of the low-precision factors
//
// kind 0 (LU, U on and above the diagonal): row value max_j>=i |u_ij|,
// diagonal |u_ii|; kind 1 (Cholesky, L): sum_k<=i l_ik^2 (= a_ii for an exact
// factor), diagonal l_ii^2; kind 2 (LDL^T, unit L and D on the diagonal):
// sum_k<i l_ik^2 |d_k| + |d_i|, diagonal |d_i|.  For Cholesky and LDL^T the
// row value bounds the entries of |L||D||L^T|, which bounds the backward error
// of the factorization (so a value far above max|a_ij| signals instability).
// out[0] max row value, out[1] max diagonal, out[2] min diagonal (bit patterns
// of non-negative doubles, which order like the values).  One warp per row.
__global__ void k_growth(const float *F, i64 rs, i64 cs, i64 n, int kind, unsigned long long *out) {
    const int lane = threadIdx.x & 31;
    const i64 i = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
    if (i >= n) return;
    double v = 0.0;
    if (kind == 0) {
        // the largest magnitude of FP32 values, taken in FP32: exact
        float w = 0.f;
        const float *fr = F + i * rs;
        i64 j = i + lane;
        if (cs == 1 && ((((uintptr_t)fr) & 15) == 0)) {
            const i64 j4 = (i + 3) & ~(i64)3;   // first 16-byte-aligned column at or after i
            if (j < j4 && j < n) w = fabsf(fr[j]);
            for (i64 q = j4 + 4 * lane; q < n; q += 128) {
                if (q + 4 <= n) {
                    const float4 u = *reinterpret_cast<const float4 *>(fr + q);
                    w = fmaxf(fmaxf(w, fmaxf(fabsf(u.x), fabsf(u.y))), fmaxf(fabsf(u.z), fabsf(u.w)));
                } else {
                    for (i64 t = q; t < n; t++) w = fmaxf(w, fabsf(fr[t]));
                }
            }
        } else {
            for (; j < n; j += 32) w = fmaxf(w, fabsf(fr[j * cs]));
        }
        for (int off = 16; off > 0; off >>= 1) w = fmaxf(w, __shfl_down_sync(0xffffffffu, w, off));
        v = (double)w;
    } else {
        const i64 kend = kind == 1 ? i + 1 : i;
        for (i64 k = lane; k < kend; k += 32) {
            const double l = (double)F[i * rs + k * cs];
            v = fma(l, kind == 1 ? l : l * fabs((double)F[k * rs + k * cs]), v);
        }
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (kind == 2) v += fabs((double)F[i * rs + i * cs]);
    }
    if (lane == 0) {
        double d = fabs((double)F[i * rs + i * cs]);
        if (kind == 1) d *= d;
        if (v == v) atomicMax(&out[0], (unsigned long long)__double_as_longlong(v));
        if (d == d) {
            atomicMax(&out[1], (unsigned long long)__double_as_longlong(d));
            atomicMin(&out[2], (unsigned long long)__double_as_longlong(d));
        }
    }
}
// D z = y for the LDL^T correction solve: row i of Y (n x nr) divided by d_i
__global__ void k_rows_by_diag(float *Y, i64 n, int nr, const float *F, i64 dstride) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n * nr; e += (i64)gridDim.x * blockDim.x)
        Y[e] /= F[(e / nr) * dstride];
}
// columns c0 .. c0+nr of X (n x ld) <-> a dense n x nr block
__global__ void k_cols_copy(const double *S, i64 lds, double *D, i64 ldd, i64 n, int nr) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n * nr; e += (i64)gridDim.x * blockDim.x)
        D[(e / nr) * ldd + e % nr] = S[(e / nr) * lds + e % nr];
}

enum MixedKind { MIX_LU = 0, MIX_CHOL = 1, MIX_LDLT = 2 };

// Mixed-precision solve of A X = B: factor a FP32 copy of A (LU with partial
// pivoting, Cholesky or unpivoted LDL^T, trailing updates in opts->precision),
// measure the factor's growth in FP64, then refine every block of up to
// MAX_RHS right-hand sides in FP64 (refine above) with the same factors.
int mixed_solve(ddla_handle h, int kind, int uplo, i64 n, i64 nrhs, const double *A, const double *B, double *X,
                const double *x_ref, const ddla_opts *opts, ddla_solve_report *rep, const int32_t *piv_ref = nullptr,
                int32_t *piv_out = nullptr) {
    cudaStream_t s = h->stream;
    const int prec = (opts && opts->precision) ? opts->precision : DDLA_PREC_FP32;
    const int nb = opts ? opts->nb : 0;
    *rep = ddla_solve_report{};
    rep->precision = prec;
    rep->pivots_agree = -1;
    rep->pivots_first_diff = -1;
    const int nr0 = (int)std::min<i64>(nrhs, MAX_RHS);
    float *A32, *d32;
    double *R;
    int32_t *piv = nullptr;
    int *perm = nullptr;
    unsigned long long *norms;
    if (kind == MIX_LU) {
        DDLA_TRY(workspace(h, WS_PERM, sizeof(int) * (size_t)n, (void **)&perm));
        DDLA_TRY(workspace(h, WS_X, sizeof(int32_t) * (size_t)n, (void **)&piv));
    }
    DDLA_TRY(workspace(h, WS_F32, sizeof(float) * (size_t)n * n, (void **)&A32));
    DDLA_TRY(workspace(h, WS_B, sizeof(float) * (size_t)n * nr0 + 256, (void **)&d32));
    DDLA_TRY(workspace(h, WS_C, sizeof(double) * (size_t)n * nr0, (void **)&R));
    // norms: [0] ||A||, [1 .. 3 MAX_RHS] column norms, then the forward-error
    // pair, the pivot comparison, the three growth figures of the factor,
    // and ||A||_inf, max |a_ij| from the pass that forms the FP32 copy
    constexpr int NORMS = 1 + 3 * MAX_RHS + 2 + 1 + 3 + 2;
    DDLA_TRY(workspace(h, WS_A, sizeof(unsigned long long) * NORMS, (void **)&norms));
    unsigned long long *astat = norms + NORMS - 2;
    DDLA_TRY(reset_info(h));
    DDLA_CUDA(cudaEventRecord(h->ev0, s));
    DDLA_CUDA(cudaMemsetAsync(astat, 0, 2 * sizeof(unsigned long long), s));
    k_d2s_norms<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(n, A, n, A32, astat);
    DDLA_LAUNCHED();
    const View<float> F{A32, n, n, n, 1};
    if (kind == MIX_LU) DDLA_TRY(getrf<float>(h, n, F, piv, prec, nb, perm));
    // FP32 blocks of 64, so the trailing updates are rank-64 (the tensor-core update's shape)
    else if (kind == MIX_CHOL) DDLA_TRY(potrf<float>(h, uplo, n, F, prec, nb));
    else DDLA_TRY(ldlt<float>(h, uplo, n, F, prec, nb > 0 ? nb : 64));
    DDLA_CUDA(cudaEventRecord(h->ev1, s));
    int info;
    DDLA_TRY(read_info(h, &info));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    rep->factor_ms = ms;
    rep->info = info;
    if (piv_out && piv) DDLA_CUDA(cudaMemcpyAsync(piv_out, piv, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
    unsigned long long *grow = norms + 1 + 3 * MAX_RHS + 2 + 1;
    {
        // pivot agreement (LU) and growth, one read-back
        if (piv_ref && piv) {
            int *cmp = (int *)(norms + 1 + 3 * MAX_RHS + 2);
            const int init[2] = {0, INT_MAX};
            DDLA_CUDA(cudaMemcpyAsync(cmp, init, sizeof(init), cudaMemcpyHostToDevice, s));
            k_piv_cmp<<<grid1(n), 256, 0, s>>>(piv, piv_ref, n, cmp);
            DDLA_LAUNCHED();
        }
        const unsigned long long ginit[3] = {0ull, 0ull, 0x7ff0000000000000ull};
        DDLA_CUDA(cudaMemcpyAsync(grow, ginit, sizeof(ginit), cudaMemcpyHostToDevice, s));
        if (!info) {
            // the factor as the lower triangle L (Cholesky / LDL^T upper: the transpose)
            const View<const float> Fg = (kind != MIX_LU && uplo == DDLA_UPPER) ? View<const float>{A32, n, n, 1, n}
                                                                                 : View<const float>{A32, n, n, n, 1};
            k_growth<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(Fg.p, Fg.rs, Fg.cs, n, kind, grow);
            DDLA_LAUNCHED();
        }
        // pivot comparison, growth of the factor, ||A||_inf, max |a_ij|
        unsigned long long got[6];
        DDLA_CUDA(cudaMemcpyAsync(got, norms + 1 + 3 * MAX_RHS + 2, sizeof(got), cudaMemcpyDeviceToHost, s));
        DDLA_CUDA(cudaStreamSynchronize(s));
        if (piv_ref && piv) {
            const int *cmp = (const int *)&got[0];
            rep->pivots_agree = cmp[0];
            rep->pivots_first_diff = cmp[1] == INT_MAX ? -1 : cmp[1];
        }
        if (!info) {
            const double gmax = u64d(got[1]), dmax = u64d(got[2]), dmin = u64d(got[3]), amax = u64d(got[5]);
            rep->growth = amax > 0 ? gmax / amax : gmax;
            rep->diag_ratio = dmin > 0 ? dmax / dmin : INFINITY;
        }
    }
    if (info) return info;
    // the inverted 64 x 64 diagonal blocks of the two triangular factors are
    // formed once and serve every correction solve
    const View<const float> Fc{A32, n, n, n, 1};
    const View<const float> Lv = (kind == MIX_LU || uplo == DDLA_LOWER) ? Fc : Fc.t();
    const View<const float> Uv = kind == MIX_LU ? Fc : Lv.t();
    const bool unit_l = kind != MIX_CHOL, unit_u = kind == MIX_LDLT;
    const i64 nblk = (n + TRI_TB - 1) / TRI_TB;
    float *invL, *invU, *mL = nullptr, *mU = nullptr;
    const size_t blk = (size_t)nblk * TRI_TB * TRI_TB;
    DDLA_TRY(workspace(h, WS_INV, sizeof(float) * (nr0 <= 1 ? 4 : 2) * blk, (void **)&invL));
    invU = invL + blk;
    DDLA_TRY(tri_inverse<float>(h, true, unit_l, Lv, n, invL));
    DDLA_TRY(tri_inverse<float>(h, false, unit_u, Uv, n, invU));
    if (nr0 <= 1) {   // one right-hand side: the cluster solves' last-tile products, formed once
        mL = invU + blk;
        mU = mL + blk;
        DDLA_TRY(tri_mlast<float>(h, true, Lv, n, invL, mL));
        DDLA_TRY(tri_mlast<float>(h, false, Uv, n, invU, mU));
    }
    int nr = nr0;
    // d <- U^-1 (D^-1) L^-1 (P) d with the FP32 factors, nr columns
    auto solve32 = [&](float *d) -> int {
        Timed t(s, TC_SOLVE, 2.0 * n * n * nr, 4.0 * n * n);
        if (kind == MIX_LU) DDLA_TRY(permute_rows<float>(h, View<float>{d, n, nr, nr, 1}, perm, n, true));
        DDLA_TRY(trsv_apply<float>(h, true, Lv, n, invL, d, nr, nr, nr <= 1 ? mL : nullptr));
        if (kind == MIX_LDLT) {
            k_rows_by_diag<<<grid1(n * nr), 256, 0, s>>>(d, n, nr, A32, n + 1);
            DDLA_LAUNCHED();
        }
        return trsv_apply<float>(h, false, Uv, n, invU, d, nr, nr, nr <= 1 ? mU : nullptr);
    };
    DDLA_CUDA(cudaEventRecord(h->ev0, s));
    int rc = 0;
    if (nrhs <= MAX_RHS) {
        rc = refine(h, n, nr, A, B, X, x_ref, opts, rep, solve32, d32, R, norms, astat);
    } else {
        // blocks of MAX_RHS columns, copied into dense n x nr blocks and back
        double *blk;
        DDLA_TRY(workspace(h, WS_RHS, sizeof(double) * 3 * (size_t)n * MAX_RHS, (void **)&blk));
        double *Bc = blk, *Xc = blk + (size_t)n * MAX_RHS, *XRc = Xc + (size_t)n * MAX_RHS;
        int iters = 0;
        double berr = 0.0, ferr = x_ref ? 0.0 : -1.0;
        bool conv = true;
        for (i64 c0 = 0; c0 < nrhs; c0 += MAX_RHS) {
            nr = (int)std::min<i64>(MAX_RHS, nrhs - c0);
            k_cols_copy<<<grid1(n * nr), 256, 0, s>>>(B + c0, nrhs, Bc, nr, n, nr);
            DDLA_LAUNCHED();
            if (x_ref) {
                k_cols_copy<<<grid1(n * nr), 256, 0, s>>>(x_ref + c0, nrhs, XRc, nr, n, nr);
                DDLA_LAUNCHED();
            }
            ddla_solve_report part = *rep;
            const int prc = refine(h, n, nr, A, Bc, Xc, x_ref ? XRc : nullptr, opts, &part, solve32, d32, R, norms,
                                   astat);
            if (prc != 0 && prc != DDLA_ERR_NOT_CONVERGED) return prc;
            k_cols_copy<<<grid1(n * nr), 256, 0, s>>>(Xc, nr, X + c0, nrhs, n, nr);
            DDLA_LAUNCHED();
            iters = std::max(iters, part.iterations);
            if (!(part.backward_error <= berr)) berr = part.backward_error;
            if (x_ref && !(part.forward_error <= ferr)) ferr = part.forward_error;
            conv = conv && part.converged;
        }
        rep->iterations = iters;
        rep->backward_error = berr;
        rep->forward_error = ferr;
        rep->converged = conv;
        if (!conv) {
            set_error("iterative refinement did not reach the backward-error tolerance");
            rc = DDLA_ERR_NOT_CONVERGED;
        }
    }
    DDLA_CUDA(cudaEventRecord(h->ev1, s));
    DDLA_CUDA(cudaEventSynchronize(h->ev1));
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    rep->refine_ms = ms;
    return rc;
}

int mixed_lu(ddla_handle h, i64 n, i64 nrhs, const double *A, const double *B, double *X, const double *x_ref,
             const ddla_opts *opts, ddla_solve_report *rep, const int32_t *piv_ref = nullptr,
             int32_t *piv_out = nullptr) {
    return mixed_solve(h, MIX_LU, 0, n, nrhs, A, B, X, x_ref, opts, rep, piv_ref, piv_out);
}

int mixed_chol(ddla_handle h, int uplo, i64 n, i64 nrhs, const double *A, const double *B, double *X,
               const double *x_ref, const ddla_opts *opts, ddla_solve_report *rep) {
    return mixed_solve(h, MIX_CHOL, uplo, n, nrhs, A, B, X, x_ref, opts, rep);
}

int mixed_ldlt(ddla_handle h, int uplo, i64 n, i64 nrhs, const double *A, const double *B, double *X,
               const double *x_ref, const ddla_opts *opts, ddla_solve_report *rep) {
    return mixed_solve(h, MIX_LDLT, uplo, n, nrhs, A, B, X, x_ref, opts, rep);
}

}  // namespace ddla

using namespace ddla;

extern "C" {

int ddla_dev_dgesv_mixed(ddla_handle h, ddla_dim_t n, ddla_dim_t nrhs, const double *a, const double *b, double *x,
                         const double *x_ref, const ddla_opts *opts, ddla_solve_report *report) {
    if (n < 0) return -2;
    if (nrhs < 0) return -3;
    if (!report) return -9;
    if (n == 0 || nrhs == 0) { *report = ddla_solve_report{}; return 0; }
    return mixed_lu(h, n, nrhs, a, b, x, x_ref, opts, report);
}

int ddla_dev_dgesv_mixed_piv(ddla_handle h, ddla_dim_t n, ddla_dim_t nrhs, const double *a, const double *b,
                             double *x, const double *x_ref, const int32_t *piv_ref, int32_t *piv_out,
                             const ddla_opts *opts, ddla_solve_report *report) {
    if (n < 0) return -2;
    if (nrhs < 0) return -3;
    if (!report) return -11;
    if (n == 0 || nrhs == 0) { *report = ddla_solve_report{}; return 0; }
    return mixed_lu(h, n, nrhs, a, b, x, x_ref, opts, report, piv_ref, piv_out);
}

int ddla_dev_dsysv_mixed(ddla_handle h, int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a,
                         const double *b, double *x, const double *x_ref, const ddla_opts *opts,
                         ddla_solve_report *report) {
    if (uplo != DDLA_LOWER && uplo != DDLA_UPPER) return -2;
    if (n < 0) return -3;
    if (nrhs < 0) return -4;
    if (!report) return -10;
    if (n == 0 || nrhs == 0) { *report = ddla_solve_report{}; return 0; }
    return mixed_ldlt(h, uplo, n, nrhs, a, b, x, x_ref, opts, report);
}

int ddla_dev_dposv_mixed(ddla_handle h, int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a,
                         const double *b, double *x, const double *x_ref, const ddla_opts *opts,
                         ddla_solve_report *report) {
    if (uplo != DDLA_LOWER && uplo != DDLA_UPPER) return -2;
    if (n < 0) return -3;
    if (nrhs < 0) return -4;
    if (!report) return -10;
    if (n == 0 || nrhs == 0) { *report = ddla_solve_report{}; return 0; }
    return mixed_chol(h, uplo, n, nrhs, a, b, x, x_ref, opts, report);
}

// Host-pointer variants: A (n x n) and B (n x nrhs) are arbitrary strided host
// views; X receives the solution.
static int host_mixed(int kind, int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa,
                      ddla_inc_t csa, const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx,
                      ddla_inc_t csx, const double *x_ref, const ddla_opts *opts, ddla_solve_report *report) {
    if (n < 0) return -1;
    if (nrhs < 0) return -2;
    if (!report) return -15;
    if (n == 0 || nrhs == 0) { *report = ddla_solve_report{}; return 0; }
    ddla_handle h;
    DDLA_TRY(default_handle(&h));
    cudaStream_t s = h->stream;
    // dense row-major device copies (the mixed kernels assume them)
    double *dA, *dB, *dX, *dR = nullptr;
    size_t nn = (size_t)n * n, nb = (size_t)n * nrhs;
    DDLA_CUDA(cudaMallocAsync(&dA, nn * 8, s));
    DDLA_CUDA(cudaMallocAsync(&dB, nb * 8, s));
    DDLA_CUDA(cudaMallocAsync(&dX, nb * 8, s));
    if (x_ref) DDLA_CUDA(cudaMallocAsync(&dR, nb * 8, s));
    auto pack_in = [&](const double *hp, i64 r, i64 c, i64 rs, i64 cs, double *d) -> int {
        if (cs == 1 && (r <= 1 || rs >= c)) {
            DDLA_CUDA(cudaMemcpy2DAsync(d, c * 8, hp, (r > 1 ? rs : c) * 8, c * 8, r, cudaMemcpyHostToDevice, s));
        } else {
            std::vector<double> tmp((size_t)(r * c));
            for (i64 i = 0; i < r; i++)
                for (i64 j = 0; j < c; j++) tmp[i * c + j] = hp[i * rs + j * cs];
            DDLA_CUDA(cudaMemcpyAsync(d, tmp.data(), tmp.size() * 8, cudaMemcpyHostToDevice, s));
            DDLA_CUDA(cudaStreamSynchronize(s));
        }
        return 0;
    };
    int rc = pack_in(a, n, n, rsa, csa, dA);
    if (!rc) rc = pack_in(b, n, nrhs, rsb, csb, dB);
    if (!rc && x_ref) rc = pack_in(x_ref, n, nrhs, nrhs, 1, dR);
    if (!rc) rc = mixed_solve(h, kind, uplo, n, nrhs, dA, dB, dX, dR, opts, report);
    if (rc == 0 || rc == DDLA_ERR_NOT_CONVERGED) {
        std::vector<double> tmp(nb);
        if (cudaMemcpyAsync(tmp.data(), dX, nb * 8, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
            cudaStreamSynchronize(s) == cudaSuccess) {
            for (i64 i = 0; i < n; i++)
                for (i64 j = 0; j < nrhs; j++) x[i * rsx + j * csx] = tmp[i * nrhs + j];
        }
    }
    cudaFreeAsync(dA, s);
    cudaFreeAsync(dB, s);
    cudaFreeAsync(dX, s);
    if (dR) cudaFreeAsync(dR, s);
    cudaStreamSynchronize(s);
    return rc;
}

int ddla_dgesv_mixed(ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                     const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx,
                     const double *x_ref, const ddla_opts *opts, ddla_solve_report *report) {
    return host_mixed(MIX_LU, 0, n, nrhs, a, rsa, csa, b, rsb, csb, x, rsx, csx, x_ref, opts, report);
}

int ddla_dposv_mixed(int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                     const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx,
                     const double *x_ref, const ddla_opts *opts, ddla_solve_report *report) {
    if (uplo != DDLA_LOWER && uplo != DDLA_UPPER) return -1;
    return host_mixed(MIX_CHOL, uplo, n, nrhs, a, rsa, csa, b, rsb, csb, x, rsx, csx, x_ref, opts, report);
}

int ddla_dsysv_mixed(int32_t uplo, ddla_dim_t n, ddla_dim_t nrhs, const double *a, ddla_inc_t rsa, ddla_inc_t csa,
                     const double *b, ddla_inc_t rsb, ddla_inc_t csb, double *x, ddla_inc_t rsx, ddla_inc_t csx,
                     const double *x_ref, const ddla_opts *opts, ddla_solve_report *report) {
    if (uplo != DDLA_LOWER && uplo != DDLA_UPPER) return -1;
    return host_mixed(MIX_LDLT, uplo, n, nrhs, a, rsa, csa, b, rsb, csb, x, rsx, csx, x_ref, opts, report);
}

}  // extern "C"
