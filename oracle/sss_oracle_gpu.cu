// ORACLE — test infrastructure, not product code.
//
// The FP64 GPU oracle: the C restatement's SingleScatterSimulationTOF
// (orc_sss, sss_oracle.c) evaluated on a GPU, so that the engine's error
// against FP64 can be stated on workloads that the host cores cannot finish
// in a test's or a benchmark's time (the 128x128x96, 33-bin instance has
// 11,362 scatter points).  It runs the same code as the C restatement: the ray
// walk, the per-leg integrals and the per-pair term come from orc_core.h,
// every operation in FP64 with no multiply-add contraction (-fmad=false), and
// every sum in the C restatement's order:
//   - a voxel's TOF weights are added into a pair's bins in walk order;
//   - one thread owns each (leg 1, leg 2) cell and adds the slice's scatter
//     points into it in lattice order, as the C restatement's loop over the
//     slice's points does;
//   - the slice's normalised sums are added to the result slice by slice.
// The two oracles differ only where the device's exp, pow, acos, cos and sin
// round differently from the host's libm (an ulp or two).  Only the tests and
// the benchmark's error study load it; the engine never links or calls it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "orc_core.h"

namespace {

constexpr int kMaxBins = 64;        // the pair kernel's per-thread bin scratch
constexpr int kThreads = 128;
constexpr int kErrCuda = -100;      // a CUDA call failed (message on stderr)

// One scatter point's legs, [point][voxel][leg] with the leg fastest, so that
// the threads of a warp (neighbouring legs) touch neighbouring words.
__global__ void orc_gpu_leg_kernel(orc_sss_problem P, const double* __restrict__ pts, int64_t npts, int cap,
                                   double* A, double* R, int32_t* IX, orc_leg_stats* S, int* status)
{
    const int64_t NL = P.nru * P.ndu;
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= npts * NL) return;
    const int64_t w = id / NL, l = id % NL;
    const int64_t base = w * (int64_t)cap * NL + l;
    const int st = orc_leg_trace(&P, l / P.ndu, l % P.ndu, pts[3 * w], pts[3 * w + 1], pts[3 * w + 2], cap,
                                 A + base, R + base, IX + base, NL, S + w * NL + l);
    if (st) atomicExch(status, st);
}

// One thread per ordered leg pair (l1, l2) = one result cell; the points of
// the launch are added in order (SingleScatterSimulationTOF.py:433-553).
__global__ void orc_gpu_pair_kernel(orc_sss_problem P, orc_pair_consts c, int64_t npts, int cap,
                                    const double* __restrict__ A, const double* __restrict__ R,
                                    const orc_leg_stats* __restrict__ S, double* slice_sum, double* slice_cnt,
                                    int* status)
{
    const int64_t NRU = P.nru, NDU = P.ndu, NL = NRU * NDU;
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= NL * NL) return;
    const int64_t l1 = id / NL, l2 = id % NL;
    const int64_t ri1 = l1 / NDU, di1 = l1 % NDU, ri2 = l2 / NDU, di2 = l2 % NDU;
    const int64_t ring1 = P.rings[ri1], det1 = P.dets[di1];
    const int64_t ring2 = P.rings[ri2], det2 = P.dets[di2];
    if ((det1 == det2 && ri2 == ri1) || det1 > det2) return;
    const double* d1p = P.geom + 3 * (ring1 * P.nd + det1);
    const double zD1 = P.geom[3 * (ring1 * P.nd) + 2];
    const double* d2p = P.geom + 3 * (ring2 * P.nd + det2);
    const double zD2 = P.geom[3 * (ring2 * P.nd) + 2];
    const double lor = (d1p[0] - d2p[0]) * (d1p[0] - d2p[0]) + (d1p[1] - d2p[1]) * (d1p[1] - d2p[1]) +
                       (zD1 - zD2) * (zD1 - zD2);
    const int64_t ncell = NL * NL;
    const int64_t cell = ((ri1 * NRU + ri2) * NDU + di1) * NDU + di2;
    double ab1[kMaxBins], ab2[kMaxBins];
    double cnt = slice_cnt[cell];
    int st = 0;
    for (int64_t w = 0; w < npts; ++w) {
        const orc_leg_stats* L1 = S + w * NL + l1;
        if (L1->att == 0) continue;
        const int64_t base = w * (int64_t)cap * NL;
        cnt += orc_pair(&c, L1, A + base + l1, R + base + l1, S + w * NL + l2, A + base + l2, R + base + l2, NL,
                        lor, ab1, ab2, slice_sum + cell, ncell, &st);
    }
    slice_cnt[cell] = cnt;
    if (st) atomicExch(status, st);
}

// Per-slice normalisation, NaN -> 0 (SingleScatterSimulationTOF.py:555-557),
// then the slice accumulators are cleared for the next slice.
__global__ void orc_gpu_normalise_kernel(int64_t ncell, int64_t nbins, double* slice_sum, double* slice_cnt,
                                         double* out)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const double cn = slice_cnt[c];
    for (int64_t b = 0; b < nbins; ++b) {
        if (cn != 0) out[b * ncell + c] += slice_sum[b * ncell + c] / cn;
        slice_sum[b * ncell + c] = 0;
    }
    slice_cnt[c] = 0;
}

unsigned blocks(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// Device copies of the problem's arrays; freed on scope exit.
struct DeviceArrays {
    std::vector<void*> held;
    ~DeviceArrays()
    {
        for (void* p : held) cudaFree(p);
    }
    template <class T>
    T* alloc(size_t n)
    {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        held.push_back(p);
        return (T*)p;
    }
    template <class T>
    T* copy(const T* h, size_t n)
    {
        T* d = alloc<T>(n);
        if (d && n && cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
        return d;
    }
};

int cuda_failed(const char* what)
{
    const cudaError_t e = cudaGetLastError();
    fprintf(stderr, "orc_sss_gpu: %s: %s\n", what, cudaGetErrorString(e));
    return kErrCuda;
}

}  // namespace

// Same problem, result layout and status codes as orc_sss (host arrays in,
// out[b][(ri1*nru + ri2)][di1][di2] on the host), plus -7 for more than 64
// bins and -100 for a failed CUDA call.  Runs on the current device.
// leg_bytes bounds the device memory of the voxel lists held at once (0: 4 GB);
// a slice whose points need more is taken in several launches of whole points.
extern "C" int orc_sss_gpu(const orc_sss_problem* p, double* out, int64_t leg_bytes)
{
    const int64_t NRU = p->nru, NDU = p->ndu, B = p->nbins, NL = NRU * NDU;
    const int64_t ncell = NL * NL;
    const int cap = (int)(p->nx + p->ny + p->nz);
    if (B < 1 || B > kMaxBins) return -7;

    const int64_t nsp = orc_scatter_points_of(p, nullptr, nullptr);
    std::vector<double> sxyz(3 * std::max<int64_t>(nsp, 1));
    std::vector<int64_t> sz(std::max<int64_t>(nsp, 1));
    orc_scatter_points_of(p, sxyz.data(), sz.data());
    const int64_t sb = p->sp_begin < 0 ? 0 : p->sp_begin;
    const int64_t se = (p->sp_end < 0 || p->sp_end > nsp) ? nsp : p->sp_end;
    const int64_t nsel = p->sp_list ? p->sp_count : (se > sb ? se - sb : 0);
    std::vector<int64_t> sel(std::max<int64_t>(nsel, 1));
    for (int64_t k = 0; k < nsel; ++k) {
        sel[k] = p->sp_list ? p->sp_list[k] : sb + k;
        if (sel[k] < 0 || sel[k] >= nsp || (k > 0 && sel[k] <= sel[k - 1])) return -5;
    }
    std::vector<double> tof_rows((size_t)ORC_TOF_ENTRIES * B);
    for (int64_t b = 0; b < B; ++b)
        for (int64_t t = 0; t < ORC_TOF_ENTRIES; ++t) tof_rows[t * B + b] = p->tof_table[b * ORC_TOF_ENTRIES + t];

    DeviceArrays D;
    const size_t nvox = (size_t)(p->nx * p->ny * p->nz);
    orc_sss_problem P = *p;
    P.act = D.copy(p->act, nvox);
    P.mu = D.copy(p->mu, nvox);
    P.image_size = D.copy(p->image_size, 6);
    P.geom = D.copy(p->geom, (size_t)(3 * p->nr * p->nd));
    P.normals = D.copy(p->normals, (size_t)(3 * p->nr * p->nd));
    P.det_size = D.copy(p->det_size, 2);
    P.rings = D.copy(p->rings, (size_t)NRU);
    P.dets = D.copy(p->dets, (size_t)NDU);
    P.eff = D.copy(p->eff, 2000);
    P.ratio = D.copy(p->ratio, 2000);
    P.tof_table = nullptr;
    P.sp_list = nullptr;
    const double* tof_d = D.copy(tof_rows.data(), tof_rows.size());
    if (!P.act || !P.mu || !P.image_size || !P.geom || !P.normals || !P.det_size || !P.rings || !P.dets ||
        !P.eff || !P.ratio || !tof_d)
        return cuda_failed("copying the problem");
    const orc_pair_consts c = orc_pair_consts_of(p, tof_d);
    // orc_pair_consts_of read eff_ref from the host's table; the rest are device pointers
    const orc_pair_consts cd = {c.eref, c.eref_j, c.eff_ref, c.ds, c.light, c.nbins, tof_d, P.eff, P.ratio};

    const int64_t per_point = NL * (int64_t)cap * (2 * (int64_t)sizeof(double) + (int64_t)sizeof(int32_t)) +
                              NL * (int64_t)sizeof(orc_leg_stats);
    const int64_t budget = leg_bytes > 0 ? leg_bytes : (int64_t)4 << 30;
    const int64_t wmax = std::max<int64_t>(1, budget / per_point);
    double* A = D.alloc<double>((size_t)(wmax * cap * NL));
    double* R = D.alloc<double>((size_t)(wmax * cap * NL));
    int32_t* IX = D.alloc<int32_t>((size_t)(wmax * cap * NL));
    orc_leg_stats* S = D.alloc<orc_leg_stats>((size_t)(wmax * NL));
    double* pts = D.alloc<double>((size_t)(3 * wmax));
    double* slice_sum = D.alloc<double>((size_t)(B * ncell));
    double* slice_cnt = D.alloc<double>((size_t)ncell);
    double* out_d = D.alloc<double>((size_t)(B * ncell));
    int* status_d = D.alloc<int>(1);
    if (!A || !R || !IX || !S || !pts || !slice_sum || !slice_cnt || !out_d || !status_d)
        return cuda_failed("allocating the work arrays");
    if (cudaMemset(slice_sum, 0, sizeof(double) * B * ncell) != cudaSuccess ||
        cudaMemset(slice_cnt, 0, sizeof(double) * ncell) != cudaSuccess ||
        cudaMemset(out_d, 0, sizeof(double) * B * ncell) != cudaSuccess ||
        cudaMemset(status_d, 0, sizeof(int)) != cudaSuccess)
        return cuda_failed("clearing the work arrays");

    std::vector<double> chunk(3 * wmax);
    int status = 0;
    int64_t k = 0;
    while (k < nsel && status == 0) {
        const int64_t zcur = sz[sel[k]];
        while (k < nsel && sz[sel[k]] == zcur) {
            int64_t n = 0;
            for (; k < nsel && sz[sel[k]] == zcur && n < wmax; ++k, ++n)
                for (int i = 0; i < 3; ++i) chunk[3 * n + i] = sxyz[3 * sel[k] + i];
            if (cudaMemcpy(pts, chunk.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice) != cudaSuccess)
                return cuda_failed("copying the scatter points");
            orc_gpu_leg_kernel<<<blocks(n * NL), kThreads>>>(P, pts, n, cap, A, R, IX, S, status_d);
            orc_gpu_pair_kernel<<<blocks(NL * NL), kThreads>>>(P, cd, n, cap, A, R, S, slice_sum, slice_cnt,
                                                                status_d);
            if (cudaGetLastError() != cudaSuccess) return cuda_failed("launching the slice's kernels");
        }
        orc_gpu_normalise_kernel<<<blocks(ncell), kThreads>>>(ncell, B, slice_sum, slice_cnt, out_d);
        if (cudaMemcpy(&status, status_d, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            return cuda_failed("running the slice");
    }
    if (cudaMemcpy(out, out_d, sizeof(double) * B * ncell, cudaMemcpyDeviceToHost) != cudaSuccess)
        return cuda_failed("copying the result");
    return status;
}
