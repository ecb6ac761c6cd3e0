// Live measurement of this GPU's FP64 (DMMA) and FP32 (FFMA) peak throughput,
// the denominators of the FP64 / FP32 rooflines.  Register-resident bounded
// loops; no memory traffic besides one store per thread.
#include "common.cuh"

namespace ddla {
namespace {

constexpr int PROBE_ITERS = 2048;

__global__ void k_probe_dmma(double *out, double s) {
    double d[4][2];
    for (int i = 0; i < 4; i++) d[i][0] = d[i][1] = 0.0;
    double a0 = s * threadIdx.x, b0 = s * (threadIdx.x + 1);
    for (int it = 0; it < PROBE_ITERS; it++) {
#pragma unroll
        for (int i = 0; i < 4; i++)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                         : "+d"(d[i][0]), "+d"(d[i][1])
                         : "d"(a0), "d"(b0));
    }
    double r = 0;
    for (int i = 0; i < 4; i++) r += d[i][0] + d[i][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

__global__ void k_probe_ffma(float *out, float s) {
    float a[8];
    for (int i = 0; i < 8; i++) a[i] = s * (threadIdx.x + i);
    const float m = 1.0000001f, c = 1e-9f * s;
    for (int it = 0; it < PROBE_ITERS * 8; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) a[i] = fmaf(a[i], m, c);
    }
    float r = 0;
    for (int i = 0; i < 8; i++) r += a[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

}  // namespace
}  // namespace ddla

using namespace ddla;

extern "C" int ddla_measure_peaks(double *fp64_tflops, double *fp32_tflops) {
    int dev, sms;
    DDLA_CUDA(cudaGetDevice(&dev));
    DDLA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;
    void *buf;
    DDLA_CUDA(cudaMalloc(&buf, sizeof(double) * blocks * threads));
    cudaEvent_t e0, e1;
    DDLA_CUDA(cudaEventCreate(&e0));
    DDLA_CUDA(cudaEventCreate(&e1));
    float ms = 0;
    const double warps = (double)blocks * threads / 32.0;
    for (int w = 0; w < 2; w++) { k_probe_dmma<<<blocks, threads>>>((double *)buf, 1.0); DDLA_LAUNCHED(); }
    DDLA_CUDA(cudaEventRecord(e0));
    for (int r = 0; r < 3; r++) { k_probe_dmma<<<blocks, threads>>>((double *)buf, 1.0); DDLA_LAUNCHED(); }
    DDLA_CUDA(cudaEventRecord(e1));
    DDLA_CUDA(cudaEventSynchronize(e1));
    DDLA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (fp64_tflops) *fp64_tflops = warps * PROBE_ITERS * 4 * (2.0 * 8 * 8 * 4) * 3 / (ms * 1e-3) / 1e12;
    for (int w = 0; w < 2; w++) { k_probe_ffma<<<blocks, threads>>>((float *)buf, 1.0f); DDLA_LAUNCHED(); }
    DDLA_CUDA(cudaEventRecord(e0));
    for (int r = 0; r < 3; r++) { k_probe_ffma<<<blocks, threads>>>((float *)buf, 1.0f); DDLA_LAUNCHED(); }
    DDLA_CUDA(cudaEventRecord(e1));
    DDLA_CUDA(cudaEventSynchronize(e1));
    DDLA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (fp32_tflops) *fp32_tflops = (double)blocks * threads * PROBE_ITERS * 8 * 8 * 2.0 * 3 / (ms * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    return 0;
}
