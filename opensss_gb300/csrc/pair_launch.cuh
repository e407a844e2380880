// The single-problem pair stage of sss_tof_run: kernel, launch and dispatch
// over the bin count.  Shared by sss.cu (plain FP32 reduction over the
// scatter points) and kahan.cu (Kahan-compensated reduction), which
// instantiate disjoint sets of kernels so that the two compile in parallel.
#pragma once

#include <algorithm>

#include "common.cuh"
#include "pair.cuh"

namespace sss {

constexpr int kMaxWaveSlices = 256;

struct PairParams {
    PairCtx ctx;            // the problem (legs of the wave's first point at index 0)
    TofConst T;             // TOF bin centres and Gaussian constants
    const float* tof_log2w; // [8001][2]
    int nchunks;            // 32-partner chunks per walking leg
    int nslices;
    int slice_first[kMaxWaveSlices];   // first point of slice j within the wave
    int slice_count[kMaxWaveSlices];
    unsigned int* counter;
    unsigned long long* work;  // [0] voxel lists walked per pair, [1] pairs evaluated
    int32_t* status;
    int warps;                 // warps per block, 0 = pair_block_warps (the compiled bound)
};

template <int NP, bool SINGLE, bool ODD, bool KAHAN, int MINB>
__global__ void __launch_bounds__(pair_block_warps(NP, KAHAN) * 32, MINB) pair_kernel(const __grid_constant__ PairParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float2* sAR = reinterpret_cast<float2*>(smem);
    unsigned char* sN = smem + kSmemNOff;
    float2* vbuf = reinterpret_cast<float2*>(smem + kSmemVbufOff) + (threadIdx.x >> 5) * 32;
    float* sG = reinterpret_cast<float*>(smem + kSmemGOff);
    float* vlo = KAHAN ? reinterpret_cast<float*>(smem + kSmemVloOff) + (threadIdx.x >> 5) * 32 : nullptr;
    float2* kahan = reinterpret_cast<float2*>(smem + pair_smem_kahan_off(P.ctx.nbins)) + threadIdx.x;
    load_pair_tables(P.tof_log2w, P.T, sAR, sN, sG);
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const long long per_slice = (long long)P.ctx.nl * P.nchunks;
    const long long ntasks = (long long)P.nslices * per_slice;
    bool tof_bad = false, energy_bad = false, nonfinite = false;
    unsigned long long walked = 0, npairs = 0;
    for (;;) {
        long long task = 0;
        if (lane == 0) task = atomicAdd(P.counter, 1u);
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= ntasks) break;
        const int slice = (int)(task / per_slice);
        const int rem = (int)(task % per_slice);
        walk_task<NP, SINGLE, ODD, KAHAN>(P.ctx, P.T, P.slice_first[slice], P.slice_count[slice],
                                          rem / P.nchunks, rem % P.nchunks, lane, sAR, sN, sG, vbuf, vlo, kahan,
                                          tof_bad, energy_bad, nonfinite, walked, npairs);
    }
    finish_pairs(lane, tof_bad, energy_bad, nonfinite, walked, npairs, P.status, P.work);
}

template <int NP, bool SINGLE, bool ODD, bool KAHAN>
int launch_pairs(const PairParams& P, cudaStream_t st)
{
    constexpr int MINB = KAHAN ? 1 : 2;
    constexpr int kBound = pair_block_warps(NP, KAHAN);
    const int kWarps = P.warps > 0 && P.warps < kBound ? P.warps : kBound;
    auto kern = pair_kernel<NP, SINGLE, ODD, KAHAN, MINB>;
    const size_t smem = pair_smem_bytes(P.ctx.nbins, KAHAN ? NP : 0);
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, smem);
    if (per_sm < 1) per_sm = 1;
    long long ntasks = (long long)P.nslices * P.ctx.nl * P.nchunks;
    long long blocks = std::min<long long>((long long)sms * per_sm, (ntasks + kWarps - 1) / kWarps);
    if (blocks < 1) blocks = 1;
    kern<<<(unsigned)blocks, kWarps * 32, smem, st>>>(P);
    return sss_check_launch("pair_kernel");
}

template <bool KAHAN>
int dispatch_pairs(const PairParams& P, cudaStream_t st)
{
    if (P.ctx.nbins == 1) return launch_pairs<1, true, false, KAHAN>(P, st);
    const bool odd = P.ctx.nbins & 1;
    switch ((P.ctx.nbins + 1) / 2) {
#define SSS_NP(k)                                                                  \
    case k:                                                                        \
        return odd ? launch_pairs<k, false, true, KAHAN>(P, st)                    \
                   : launch_pairs<k, false, false, KAHAN>(P, st);
        SSS_NP(1) SSS_NP(2) SSS_NP(3) SSS_NP(4) SSS_NP(5) SSS_NP(6) SSS_NP(7) SSS_NP(8)
        SSS_NP(9) SSS_NP(10) SSS_NP(11) SSS_NP(12) SSS_NP(13) SSS_NP(14) SSS_NP(15) SSS_NP(16)
        SSS_NP(17) SSS_NP(18) SSS_NP(19) SSS_NP(20) SSS_NP(21) SSS_NP(22) SSS_NP(23) SSS_NP(24)
        SSS_NP(25) SSS_NP(26) SSS_NP(27) SSS_NP(28) SSS_NP(29) SSS_NP(30) SSS_NP(31) SSS_NP(32)
#undef SSS_NP
    }
    return sss_set_error(SSS_ERR_INVALID, "nbins out of range");
}

// Defined in sss.cu (plain) and kahan.cu (compensated).
int dispatch_pairs_plain(const PairParams& P, cudaStream_t st);
int dispatch_pairs_kahan(const PairParams& P, cudaStream_t st);

}  // namespace sss
