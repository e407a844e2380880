// Throughput probes for the roofline denominators of the pair stage, measured
// on the device the engine runs on: the SFU 2^x instruction
// (ex2.approx.ftz.f32), the shared-memory load bandwidth (the pair kernel
// reads its TOF factors from shared memory) and the L2 load bandwidth (where
// a TOF-table gather, as the reference does it, would read them from).
//
// Measurement only: built into its own library (libsss300_probe.so), which
// the benchmark loads; the engine library does not contain these kernels.
// Each entry point returns 0 or the failing cudaError_t, synchronises
// `stream` and writes its rate (GB/s, 1e9 results/s for 2^x, DADD and
// DDIV, GFLOP/s for FFMA2).
#include <cuda_runtime.h>

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

// FP32 FMA pipe: independent chains of packed FFMA2 (two FMAs per lane and
// instruction, the form the pair kernel's bin loop issues).
__global__ void __launch_bounds__(256) ffma2_probe_kernel(int iters, float* sink)
{
    float2 x[kChains];
    const float2 a = make_float2(0.999f, 0.998f), b = make_float2(1e-3f, 2e-3f);
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = make_float2(0.1f * (threadIdx.x & 7) + 0.01f * c, 0.5f);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = __ffma2_rn(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c].x + x[c].y;
    if (s == 123.456f) sink[0] = s;  // keeps the chains alive
}

// FP64 adds: independent chains of DADD (the ray walk's step before it moved
// to the integer pipe).
__global__ void __launch_bounds__(256) dadd_probe_kernel(int iters, double* sink)
{
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 0.1 * (threadIdx.x & 7) + 0.01 * c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = __dadd_rn(x[c], 1e-3);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 123.456) sink[0] = s;
}

// FP64 divisions: independent chains of IEEE round-to-nearest DDIV (the
// per-ray set-up of the ray walk holds fifteen of them).
__global__ void __launch_bounds__(256) ddiv_probe_kernel(int iters, double* sink)
{
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 1.5 + 0.1 * (threadIdx.x & 7) + 0.01 * c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = __ddiv_rn(x[c], 0.9999999);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 123.456) sink[0] = s;
}

// Shared-memory loads: every warp reads 512 contiguous bytes per LDS.128
// (no bank conflicts), eight independent loads per iteration, from a 32 KB
// buffer; the loaded words are folded with XOR so that no load is dead.
constexpr int kSmemVec = 2048;  // float4 entries (32 KB)
__global__ void __launch_bounds__(256) smem_probe_kernel(int iters, unsigned* sink)
{
    __shared__ float4 buf[kSmemVec];
    for (int i = threadIdx.x; i < kSmemVec; i += blockDim.x)
        buf[i] = make_float4((float)i, (float)(i + 1), (float)(i + 2), (float)(i + 3));
    __syncthreads();
    unsigned acc = 0;
    int idx = threadIdx.x & 1023;  // idx + 7 * 128 < kSmemVec
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const float4 v = buf[idx + c * 128];
            acc ^= __float_as_uint(v.x) ^ __float_as_uint(v.y) ^ __float_as_uint(v.z) ^ __float_as_uint(v.w);
        }
        idx = (idx + 32) & 1023;
    }
    if (acc == 0x9e3779b9u) sink[0] = acc;
}

// L2 loads: a buffer that fits in L2 is read with ld.global.cg (L2 only, no
// L1), four independent 16-byte loads in flight per thread.
__global__ void __launch_bounds__(256) l2_probe_kernel(const float4* __restrict__ buf, long long n4, int reps,
                                                       unsigned* sink)
{
    unsigned acc = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long first = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (int r = 0; r < reps; ++r) {
        long long i = first;
        for (; i + 3 * stride < n4; i += 4 * stride) {
            const float4 a = __ldcg(buf + i), b = __ldcg(buf + i + stride);
            const float4 c = __ldcg(buf + i + 2 * stride), d = __ldcg(buf + i + 3 * stride);
            acc ^= __float_as_uint(a.x) ^ __float_as_uint(a.w) ^ __float_as_uint(b.x) ^ __float_as_uint(b.w) ^
                   __float_as_uint(c.x) ^ __float_as_uint(c.w) ^ __float_as_uint(d.x) ^ __float_as_uint(d.w);
        }
        for (; i < n4; i += stride) {
            const float4 a = __ldcg(buf + i);
            acc ^= __float_as_uint(a.x) ^ __float_as_uint(a.w);
        }
    }
    if (acc == 0x9e3779b9u) sink[0] = acc;
}

// Times one launch of a probe between two events on st (after one warm-up
// launch); returns 0 and the milliseconds, or the failing cudaError_t.
template <typename Launch>
int time_probe(cudaStream_t st, Launch launch, float* ms)
{
    cudaEvent_t a, b;
    cudaError_t e = cudaEventCreate(&a);
    if (e != cudaSuccess) return (int)e;
    if ((e = cudaEventCreate(&b)) != cudaSuccess) {
        cudaEventDestroy(a);
        return (int)e;
    }
    launch(true);
    cudaEventRecord(a, st);
    launch(false);
    cudaEventRecord(b, st);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return (int)e;
}

}  // namespace

extern "C" int sss_probe_smem_rate(double* gb_per_s, void* stream)
{
    if (!gb_per_s) return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 4, threads = 256, iters = 4096;
    unsigned* sink = nullptr;
    cudaError_t e = cudaMallocAsync(&sink, sizeof(unsigned), st);
    if (e != cudaSuccess) return (int)e;
    float ms = 0.f;
    int rc = time_probe(st, [&](bool warm) {
        smem_probe_kernel<<<blocks, threads, 0, st>>>(warm ? iters / 8 : iters, sink);
    }, &ms);
    cudaFreeAsync(sink, st);
    if (rc) return rc;
    *gb_per_s = (double)blocks * threads * iters * 8 * 16 / (ms * 1e-3) / 1e9;
    return 0;
}

extern "C" int sss_probe_l2_rate(double* gb_per_s, void* stream)
{
    if (!gb_per_s) return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long n4 = (32ll << 20) / 16;  // 32 MB, L2-resident
    const int blocks = sms * 8, threads = 256, reps = 256;
    float4* buf = nullptr;
    unsigned* sink = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, n4 * 16 + 256, st);
    if (e != cudaSuccess) return (int)e;
    sink = reinterpret_cast<unsigned*>(buf + n4);
    cudaMemsetAsync(buf, 0, n4 * 16, st);
    float ms = 0.f;
    int rc = time_probe(st, [&](bool warm) {
        l2_probe_kernel<<<blocks, threads, 0, st>>>(buf, n4, warm ? 2 : reps, sink);
    }, &ms);
    cudaFreeAsync(buf, st);
    if (rc) return rc;
    *gb_per_s = (double)n4 * 16 * reps / (ms * 1e-3) / 1e9;
    return 0;
}

extern "C" int sss_probe_ex2_rate(double* gex2_per_s, void* stream)
{
    if (!gex2_per_s) return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    float* sink = nullptr;
    cudaError_t e = cudaMallocAsync(&sink, sizeof(float), st);
    if (e != cudaSuccess) return (int)e;
    float ms = 0.f;
    int rc = time_probe(st, [&](bool warm) {
        ex2_probe_kernel<<<blocks, threads, 0, st>>>(warm ? iters / 8 : iters, sink);
    }, &ms);
    cudaFreeAsync(sink, st);
    if (rc) return rc;
    *gex2_per_s = (double)blocks * threads * iters * kChains / (ms * 1e-3) / 1e9;
    return 0;
}

extern "C" int sss_probe_ffma_rate(double* gflop_per_s, void* stream)
{
    if (!gflop_per_s) return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 8192;
    float* sink = nullptr;
    cudaError_t e = cudaMallocAsync(&sink, sizeof(float), st);
    if (e != cudaSuccess) return (int)e;
    float ms = 0.f;
    int rc = time_probe(st, [&](bool warm) {
        ffma2_probe_kernel<<<blocks, threads, 0, st>>>(warm ? iters / 8 : iters, sink);
    }, &ms);
    cudaFreeAsync(sink, st);
    if (rc) return rc;
    // two FMAs (four flops) per FFMA2
    *gflop_per_s = (double)blocks * threads * iters * kChains * 4 / (ms * 1e-3) / 1e9;
    return 0;
}

extern "C" int sss_probe_dadd_rate(double* gadd_per_s, void* stream)
{
    if (!gadd_per_s) return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 1024;
    double* sink = nullptr;
    cudaError_t e = cudaMallocAsync(&sink, sizeof(double), st);
    if (e != cudaSuccess) return (int)e;
    float ms = 0.f;
    int rc = time_probe(st, [&](bool warm) {
        dadd_probe_kernel<<<blocks, threads, 0, st>>>(warm ? iters / 8 : iters, sink);
    }, &ms);
    cudaFreeAsync(sink, st);
    if (rc) return rc;
    *gadd_per_s = (double)blocks * threads * iters * kChains / (ms * 1e-3) / 1e9;
    return 0;
}

extern "C" int sss_probe_ddiv_rate(double* gdiv_per_s, void* stream)
{
    if (!gdiv_per_s) return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 128;
    double* sink = nullptr;
    cudaError_t e = cudaMallocAsync(&sink, sizeof(double), st);
    if (e != cudaSuccess) return (int)e;
    float ms = 0.f;
    int rc = time_probe(st, [&](bool warm) {
        ddiv_probe_kernel<<<blocks, threads, 0, st>>>(warm ? iters / 8 : iters, sink);
    }, &ms);
    cudaFreeAsync(sink, st);
    if (rc) return rc;
    *gdiv_per_s = (double)blocks * threads * iters * kChains / (ms * 1e-3) / 1e9;
    return 0;
}
