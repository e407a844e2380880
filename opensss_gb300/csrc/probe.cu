// Throughput probe for the SFU 2^x instruction (ex2.approx.ftz.f32), the
// instruction the pair kernel is bound by.  bench.py uses the measured rate
// as the roofline denominator of that kernel.
#include "common.cuh"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) ex2_probe_kernel(int iters, float* sink)
{
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 0.1f * (threadIdx.x & 7) + 0.01f * c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = sss::ex2(fmaf(x[c], -0.5f, 0.25f));
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 123.456f) sink[0] = s;  // keeps the chains alive
}

}  // namespace

extern "C" int sss_probe_ex2_rate(double* gex2_per_s, void* stream)
{
    if (!gex2_per_s) return sss_set_error(SSS_ERR_INVALID, "sss_probe_ex2_rate: null output");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    float* sink = nullptr;
    if (cudaMallocAsync(&sink, sizeof(float), st) != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_probe_ex2_rate: allocation failed");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    ex2_probe_kernel<<<blocks, threads, 0, st>>>(iters / 8, sink);  // warm-up
    cudaEventRecord(a, st);
    ex2_probe_kernel<<<blocks, threads, 0, st>>>(iters, sink);
    cudaEventRecord(b, st);
    int rc = sss_check_launch("ex2_probe_kernel");
    float ms = 0.f;
    if (!rc && (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess))
        rc = sss_set_error(SSS_ERR_CUDA, "sss_probe_ex2_rate: timing failed");
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFreeAsync(sink, st);
    if (rc) return rc;
    double n = (double)blocks * threads * iters * kChains;
    *gex2_per_s = n / (ms * 1e-3) / 1e9;
    return SSS_OK;
}
