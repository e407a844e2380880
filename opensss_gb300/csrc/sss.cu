// Fused TOF single scatter simulation on sm_103a.
//
// Pipeline per wave of whole z-slices (reference: SingleScatterSimulationTOF.py
// :82-208 and bodySSS :301-559):
//   1. scatter_points_kernel — ordered lattice compaction of mu > 0 points.
//   2. leg_kernel   — one thread per (scatter point, sampled crystal): FP64
//      Amanatides-Woo walk (bit-identical voxel sequence), FP32 integrals of
//      mu and activity, incidence term, and the list of the leg's non-zero
//      activity voxels (act*len, TOF sample offset), one list per leg.
//   3. pair_kernel  — persistent warps pull (slice, walking leg, 32-partner
//      chunk) tasks; each lane owns one detector pair, loops over the slice's
//      scatter points, evaluates the Klein-Nishina x efficiency x attenuation
//      factors once per pair, and for each voxel of the walking leg (staged in
//      shared memory, read as broadcasts) adds the factored TOF weights
//      [A r^b] G[n][b] of every bin from shared-memory tables; the slice
//      numerator and count stay in registers and numerator/count is added to
//      the output (per-slice normalisation, :555-557).
// Nothing per voxel or per pair reaches HBM except the leg lists themselves.
#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "legs.cuh"
#include "pair.cuh"
#include "pair_launch.cuh"
#include "trace.cuh"

namespace {

using namespace sss;

struct LatticeDims {
    int lx, ly, lz;     // lattice points per axis
    int sx, sy, sz;     // steps
};

LatticeDims lattice(const sss_tof_problem& p)
{
    LatticeDims L;
    L.sx = p.sample_step[0];
    L.sy = p.sample_step[1];
    L.sz = p.sample_step[2];
    L.lx = (p.nx + L.sx - 1) / L.sx;
    L.ly = (p.ny + L.sy - 1) / L.sy;
    L.lz = (p.nz + L.sz - 1) / L.sz;
    return L;
}

// ---------------------------------------------------------------- 1. points

// Single block, 1024 threads: walks the lattice in the reference's order
// (z, then y, then x: :182, :387, :391) in chunks of 1024, block-scans the
// mu > 0 flags and writes the points in order.  Coordinates follow :176-179,
// :381, :389, :394 in FP64.
__global__ void __launch_bounds__(1024) scatter_points_kernel(
    const float* __restrict__ mu, int nx, int ny, int nz, LatticeDims L, double radius,
    double zstart, double zvox, double* __restrict__ out, int64_t capacity,
    unsigned long long* __restrict__ total, unsigned long long* __restrict__ slice_counts)
{
    __shared__ int warp_sums[32];
    __shared__ unsigned long long base;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) base = 0;
    __syncthreads();
    const long long npts = (long long)L.lx * L.ly * L.lz;
    for (long long c0 = 0; c0 < npts; c0 += 1024) {
        long long i = c0 + tid;
        int flag = 0, ix = 0, iy = 0, iz = 0;
        if (i < npts) {
            ix = (int)(i % L.lx);
            iy = (int)((i / L.lx) % L.ly);
            iz = (int)(i / ((long long)L.lx * L.ly));
            int x = ix * L.sx, y = iy * L.sy, z = iz * L.sz;
            flag = mu[x + (long long)nx * (y + (long long)ny * z)] > 0.0f;
        }
        unsigned ball = __ballot_sync(0xffffffffu, flag);
        int pre = __popc(ball & ((1u << lane) - 1u));
        if (lane == 0) warp_sums[warp] = __popc(ball);
        __syncthreads();
        if (warp == 0) {
            int v = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            warp_sums[lane] = v;  // inclusive
        }
        __syncthreads();
        int wbase = warp ? warp_sums[warp - 1] : 0;
        if (flag) {
            unsigned long long pos = base + wbase + pre;
            int x = ix * L.sx, y = iy * L.sy, z = iz * L.sz;
            if ((long long)pos < capacity) {
                double xs = sub64(div64(mul64((double)((x + 1) * 2), radius), (double)nx), radius);
                double ys = sub64(div64(mul64((double)((y + 1) * 2), radius), (double)ny), radius);
                double zs = add64(zstart, mul64((double)z, zvox));
                out[4 * pos + 0] = xs;
                out[4 * pos + 1] = ys;
                out[4 * pos + 2] = zs;
                out[4 * pos + 3] = (double)z;
            }
            atomicAdd(&slice_counts[iz], 1ull);
        }
        __syncthreads();
        if (tid == 0) base += warp_sums[31];
        __syncthreads();
    }
    if (tid == 0) *total = base;
}

// ---------------------------------------------------------------- 2. legs

__global__ void __launch_bounds__(kLegThreadsMax) leg_kernel(LegParams P)
{
    long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)P.npts * P.nl) return;
    leg_one(P, (int)(gid / P.nl), (int)(gid % P.nl));
}

// ---------------------------------------------------------------- 3. pairs

// ---------------------------------------------------------------- densify

__global__ void densify_kernel(const float* __restrict__ cmp, int nbins, int nru, int ndu, int nd,
                               const int16_t* __restrict__ lor, const int32_t* __restrict__ dets,
                               float* __restrict__ dense, int32_t* status)
{
    const int nl = nru * ndu;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)nbins * nl * nl;
    if (i >= total) return;
    const int l2 = (int)(i % nl);
    const int l1 = (int)((i / nl) % nl);
    const int b = (int)(i / ((long long)nl * nl));
    const int di1 = l1 / nru, ri1 = l1 % nru, di2 = l2 / nru, ri2 = l2 % nru;
    if (di1 > di2 || (di1 == di2 && ri1 == ri2)) return;
    const int d1 = dets[di1], d2 = dets[di2];
    if ((unsigned)d1 >= (unsigned)nd || (unsigned)d2 >= (unsigned)nd) {  // the caller's crystal table
        raise_error(status, kErrTable);
        return;
    }
    const int ang = lor[2 * ((long long)d1 * nd + d2)];
    const int rad = lor[2 * ((long long)d1 * nd + d2) + 1];
    const int nang = nd / 2, nsino = nru * nru;
    if (rad < 0 || rad > nd || ang < 0 || ang >= nang) {  // the caller's LOR table
        raise_error(status, kErrTable);
        return;
    }
    dense[(((long long)b * (nd + 1) + rad) * nang + ang) * nsino + ri2 + ri1 * nru] = cmp[i];
}

// Every element of the dense layout in one pass, zeros included, four
// slices (one 16-byte store) a thread: cell (rad, ang) holds sampled pair
// cell_pair[cell] = di1 * ndu + di2 (di1 <= di2) or -1.  The destination
// may be page-locked host memory, which the GPU writes over its host link.
__global__ void densify_full_kernel(const float* __restrict__ cmp, int nbins, int nru, int ndu, long long ncell,
                                    const int32_t* __restrict__ cell_pair, float* __restrict__ dense,
                                    int32_t* status)
{
    const int nl = nru * ndu, nsino = nru * nru;
    const long long plane = (long long)nl * nl;
    const long long total4 = (long long)nbins * ncell * nsino / 4;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total4;
         q += (long long)gridDim.x * blockDim.x) {
        const long long e = 4 * q;
        const int sino = (int)(e % nsino);
        const long long cell = (e / nsino) % ncell;
        const int b = (int)(e / ((long long)nsino * ncell));
        const int pair = __ldg(cell_pair + cell);
        float v[4] = {0.f, 0.f, 0.f, 0.f};
        const int di1 = pair / ndu, di2 = pair % ndu;
        if (pair < -1 || pair >= ndu * ndu || (pair >= 0 && di1 > di2)) {  // the caller's cell table
            raise_error(status, kErrTable);
        } else if (pair >= 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int s = sino + k, ri1 = s / nru, ri2 = s % nru;
                if (di1 < di2 || ri1 != ri2)
                    v[k] = __ldg(cmp + b * plane + (long long)(di1 * nru + ri1) * nl + di2 * nru + ri2);
            }
        }
        reinterpret_cast<float4*>(dense)[q] = make_float4(v[0], v[1], v[2], v[3]);
    }
}

// The cells of sampled pairs alone, for a destination whose other cells
// already hold zeros: one warp a cell (the cell's entry read as a broadcast);
// a sampled cell's nru^2 slices of every bin go out as 16-byte stores, one a
// lane.  Under 1% of the cells are sampled, so the scan is most of the work
// and the writes are 0.4% of the layout's bytes.
__global__ void densify_cells_kernel(const float* __restrict__ cmp, int nbins, int nru, int ndu, long long ncell,
                                     const int32_t* __restrict__ cell_pair, float* __restrict__ dense,
                                     int32_t* status)
{
    const int nl = nru * ndu, nsino = nru * nru, nq = nsino / 4;
    const long long plane = (long long)nl * nl;
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long cell = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; cell < ncell; cell += warps) {
        const int pair = __ldg(cell_pair + cell);
        if (pair == -1) continue;
        const int di1 = pair / ndu, di2 = pair % ndu;
        if (pair < -1 || pair >= ndu * ndu || di1 > di2) {  // the caller's cell table
            if (lane == 0) raise_error(status, kErrTable);
            continue;
        }
        for (int b = 0; b < nbins; ++b) {
            float4* dst = reinterpret_cast<float4*>(dense + ((long long)b * ncell + cell) * nsino);
            const float* src = cmp + b * plane + (long long)di1 * nru * nl + di2 * nru;  // + ri1 * nl + ri2
            for (int q = lane; q < nq; q += 32) {
                float v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int sl = 4 * q + k, ri1 = sl / nru, ri2 = sl % nru;
                    v[k] = (di1 < di2 || ri1 != ri2) ? __ldg(src + (long long)ri1 * nl + ri2) : 0.f;
                }
                dst[q] = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
    }
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Optional stage timing (events recorded on the caller's stream).
struct StageTimer {
    bool on = false;
    std::vector<cudaEvent_t> ev;  // pairs: leg start/end, pair start/end per wave
    int launches = 0, waves = 0, nbins = 0;
    const unsigned long long* work = nullptr;  // device counters of the last run
    cudaEvent_t get()
    {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ev.push_back(e);
        return e;
    }
    void clear()
    {
        for (auto e : ev) cudaEventDestroy(e);
        ev.clear();
        launches = waves = 0;
    }
};
thread_local StageTimer g_timer;

struct WsLayout {
    size_t legA, legB, legC, vox, vox_lo, counter, total;
};

WsLayout ws_layout(const sss_tof_problem& p, long long wave_points)
{
    const long long nl = (long long)p.nru * p.ndu;
    const long long cap = (long long)p.nx + p.ny + p.nz;
    WsLayout w;
    size_t off = 0;
    w.legA = off;
    off = align_up(off + sizeof(float4) * wave_points * nl);
    w.legB = off;
    off = align_up(off + sizeof(float4) * wave_points * nl);
    w.legC = off;
    off = align_up(off + sizeof(float4) * wave_points * nl);
    w.vox = off;  // no voxel lists when every TOF weight is 1
    const bool lists = !(p.flags & SSS_FLAG_UNIT_TOF);
    if (lists) off = align_up(off + sizeof(float2) * wave_points * cap * nl);
    w.vox_lo = off;  // the samples' low floats: the precision (Kahan) launch only
    if (lists && (p.flags & SSS_FLAG_KAHAN)) off = align_up(off + sizeof(float) * wave_points * cap * nl);
    w.counter = off;
    off = align_up(off + 256);
    w.total = off;
    return w;
}


int validate(const sss_tof_problem* p)
{
    if (!p) return sss_set_error(SSS_ERR_INVALID, "null problem");
    if (p->nx < 1 || p->ny < 1 || p->nz < 1) return sss_set_error(SSS_ERR_INVALID, "bad volume shape");
    if (!p->activity || !p->attenuation || !p->geometry || !p->normals || !p->rings ||
        !p->detectors || !p->tof_log2w || !p->efficiency || !p->atten_ratio)
        return sss_set_error(SSS_ERR_INVALID, "null array in problem");
    if (p->nr < 1 || p->nd < 2 || p->nru < 1 || p->ndu < 1 || p->nru > p->nr || p->ndu > p->nd)
        return sss_set_error(SSS_ERR_INVALID, "bad scanner / sampling sizes");
    if (p->sample_step[0] < 1 || p->sample_step[1] < 1 || p->sample_step[2] < 1)
        return sss_set_error(SSS_ERR_INVALID, "sample_step must be >= 1");
    if (p->nbins < 1 || p->nbins > 64) return sss_set_error(SSS_ERR_INVALID, "nbins must be 1..64");
    if ((p->flags & SSS_FLAG_UNIT_TOF) && p->nbins != 1)
        return sss_set_error(SSS_ERR_INVALID, "SSS_FLAG_UNIT_TOF needs nbins == 1");
    if (!(p->image_size[3] > p->image_size[0] && p->image_size[4] > p->image_size[1] &&
          p->image_size[5] > p->image_size[2]))
        return sss_set_error(SSS_ERR_INVALID, "image_size must satisfy max > min");
    long long nl = (long long)p->nru * p->ndu;
    if (nl * nl * p->nbins > (1ll << 40)) return sss_set_error(SSS_ERR_INVALID, "output too large");
    const int wmax = sss_pair_warps_max(p->nbins, p->flags);
    if (p->pair_warps < 0 || p->pair_warps > wmax)
        return sss_set_error(SSS_ERR_INVALID, "pair_warps %d outside 0..%d", p->pair_warps, wmax);
    if (p->leg_threads < 0 || p->leg_threads > kLegThreadsMax || p->leg_threads % 32)
        return sss_set_error(SSS_ERR_INVALID, "leg_threads %d: 0 or a multiple of 32 up to %d", p->leg_threads,
                             kLegThreadsMax);
    return SSS_OK;
}

}  // namespace

// The pair kernels of the plain reduction (the compensated ones are in kahan.cu).
int sss::dispatch_pairs_plain(const PairParams& P, cudaStream_t st) { return dispatch_pairs<false>(P, st); }

int sss_internal_validate(const sss_tof_problem* p) { return validate(p); }

extern "C" int sss_pair_warps_max(int32_t nbins, int32_t flags)
{
    if (nbins < 1 || nbins > 64) return 0;
    return sss::pair_block_warps((nbins + 1) / 2, (flags & SSS_FLAG_KAHAN) != 0);
}

int sss_internal_scatter_points(const sss_tof_problem* p, double* points, long long capacity,
                                unsigned long long* counts, cudaStream_t st)
{
    LatticeDims L = lattice(*p);
    const double* IS = p->image_size;
    const double zvox = (IS[5] - IS[2]) / p->nz;  // :87
    const double zstart = zvox / 2 - (-IS[2]);    // :176, :179
    const double radius = -IS[0];                 // :177
    scatter_points_kernel<<<1, 1024, 0, st>>>(p->attenuation, p->nx, p->ny, p->nz, L, radius, zstart,
                                               zvox, points, capacity, counts, counts + 1);
    return sss_check_launch("scatter_points_kernel");
}

extern "C" int sss_scatter_points(const sss_tof_problem* p, double* points, int64_t capacity,
                                  int64_t* count, int64_t* slice_counts, void* stream)
{
    int rc = validate(p);
    if (rc) return rc;
    if (!count) return sss_set_error(SSS_ERR_INVALID, "sss_scatter_points: null count");
    if (capacity > 0 && !points) return sss_set_error(SSS_ERR_INVALID, "sss_scatter_points: null points");
    cudaStream_t st = (cudaStream_t)stream;
    LatticeDims L = lattice(*p);
    const double* IS = p->image_size;
    double zvox = (IS[5] - IS[2]) / p->nz;  // :87
    double zstart = zvox / 2 - (-IS[2]);    // :176, :179
    double radius = -IS[0];                 // :177
    unsigned long long* dbuf = nullptr;
    size_t nbuf = 1 + (size_t)L.lz;
    if (cudaMallocAsync(&dbuf, nbuf * sizeof(unsigned long long), st) != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_scatter_points: allocation failed");
    cudaMemsetAsync(dbuf, 0, nbuf * sizeof(unsigned long long), st);
    scatter_points_kernel<<<1, 1024, 0, st>>>(p->attenuation, p->nx, p->ny, p->nz, L, radius,
                                               zstart, zvox, points, capacity, dbuf, dbuf + 1);
    rc = sss_check_launch("scatter_points_kernel");
    std::vector<unsigned long long> h(nbuf);
    if (!rc && cudaMemcpyAsync(h.data(), dbuf, nbuf * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = sss_set_error(SSS_ERR_CUDA, "sss_scatter_points: copy failed");
    cudaFreeAsync(dbuf, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc)
        rc = sss_set_error(SSS_ERR_CUDA, "sss_scatter_points: %s", cudaGetErrorString(cudaGetLastError()));
    if (rc) return rc;
    *count = (int64_t)h[0];
    if (slice_counts)
        for (int i = 0; i < L.lz; ++i) slice_counts[i] = (int64_t)h[1 + i];
    if ((int64_t)h[0] > capacity)
        return sss_set_error(SSS_ERR_CAPACITY, "sss_scatter_points: %lld points > capacity %lld",
                             (long long)h[0], (long long)capacity);
    return SSS_OK;
}

extern "C" size_t sss_tof_workspace_size(const sss_tof_problem* p, int64_t wave_points)
{
    if (validate(p)) return 0;
    return ws_layout(*p, wave_points).total;
}

extern "C" int sss_tof_run(const sss_tof_problem* p, const double* points, int64_t n_points,
                           const int64_t* slice_counts, int64_t n_slices, int64_t wave_points,
                           void* workspace, size_t workspace_bytes, float* out, int32_t* status,
                           void* stream)
{
    int rc = validate(p);
    if (rc) return rc;
    if (!out || (n_points > 0 && (!points || !slice_counts)) || n_slices < 0 || (n_slices > 0 && !slice_counts))
        return sss_set_error(SSS_ERR_INVALID, "sss_tof_run: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    const long long nl = (long long)p->nru * p->ndu;
    const long long cap = (long long)p->nx + p->ny + p->nz;
    long long maxslice = 0, tot = 0;
    for (int64_t i = 0; i < n_slices; ++i) {
        if (slice_counts[i] < 0)
            return sss_set_error(SSS_ERR_INVALID, "sss_tof_run: slice_counts[%lld] is negative", (long long)i);
        maxslice = std::max<long long>(maxslice, slice_counts[i]);
        tot += slice_counts[i];
    }
    if (tot != n_points) return sss_set_error(SSS_ERR_INVALID, "slice_counts do not sum to n_points");
    if (wave_points < maxslice)
        return sss_set_error(SSS_ERR_INVALID, "wave_points %lld < largest slice %lld",
                             (long long)wave_points, maxslice);
    WsLayout w = ws_layout(*p, wave_points);
    if (!workspace || workspace_bytes < w.total)
        return sss_set_error(SSS_ERR_WORKSPACE, "sss_tof_run: workspace %zu < %zu bytes",
                             workspace_bytes, w.total);
    char* ws = (char*)workspace;
    if (cudaMemsetAsync(out, 0, sizeof(float) * p->nbins * nl * nl, st) != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_tof_run: memset failed");
    if (n_points == 0) return SSS_OK;


    LegParams LP;
    LP.g = grid_of(p->nx, p->ny, p->nz, p->image_size);
    LP.act = p->activity;
    LP.mu = p->attenuation;
    LP.geom = p->geometry;
    LP.normals = p->normals;
    LP.rings = p->rings;
    LP.dets = p->detectors;
    LP.nr = p->nr;
    LP.nd = p->nd;
    LP.nru = p->nru;
    LP.ndu = p->ndu;
    LP.nl = (int)nl;
    LP.cap = (int)cap;
    LP.nvox = (long long)p->nx * p->ny * p->nz;
    LP.legA = (float4*)(ws + w.legA);
    LP.legB = (float4*)(ws + w.legB);
    LP.legC = (float4*)(ws + w.legC);
    LP.vox = (p->flags & SSS_FLAG_UNIT_TOF) ? nullptr : (float2*)(ws + w.vox);
    LP.vox_lo = (LP.vox && (p->flags & SSS_FLAG_KAHAN)) ? (float*)(ws + w.vox_lo) : nullptr;
    LP.status = status;

    PairParams PP;
    PairCtx& C = PP.ctx;
    C.nru = p->nru;
    C.ndu = p->ndu;
    C.nl = (int)nl;
    C.nd = p->nd;
    C.cap = (int)cap;
    C.nbins = p->nbins;
    C.geo_c = geo_const(*p);
    C.gamma_kn = gamma_kn_const();
    C.eff = p->efficiency;
    C.ratio = p->atten_ratio;
    C.geom = p->geometry;
    C.rings = p->rings;
    C.dets = p->detectors;
    C.legA = LP.legA;
    C.legB = LP.legB;
    C.legC = LP.legC;
    C.vox = LP.vox;
    C.vox_lo = LP.vox_lo;
    C.unit_tof = (p->flags & SSS_FLAG_UNIT_TOF) != 0;
    C.out = out;
    PP.T = tof_const(*p);
    PP.tof_log2w = p->tof_log2w;
    PP.nchunks = pair_chunks(p->nru, p->ndu);
    PP.counter = (unsigned int*)(ws + w.counter);
    PP.work = (unsigned long long*)(ws + w.counter + 8);
    cudaMemsetAsync(ws + w.counter, 0, 256, st);
    PP.status = status;
    PP.warps = p->pair_warps;

    g_timer.clear();
    g_timer.work = PP.work;
    g_timer.nbins = p->nbins;
    // waves of whole slices
    long long first = 0;
    int64_t si = 0;
    while (si < n_slices) {
        long long npts = 0;
        int nsl = 0;
        PP.nslices = 0;
        while (si < n_slices && nsl < kMaxWaveSlices && npts + slice_counts[si] <= wave_points) {
            if (slice_counts[si] > 0) {
                PP.slice_first[PP.nslices] = (int)npts;
                PP.slice_count[PP.nslices] = (int)slice_counts[si];
                PP.nslices++;
            }
            npts += slice_counts[si];
            ++nsl;
            ++si;
        }
        if (npts > 0) {
            LP.points = points + 4 * first;
            LP.npts = (int)npts;
            long long threads = npts * nl;
            if (g_timer.on) cudaEventRecord(g_timer.get(), st);
            const int lt = p->leg_threads ? p->leg_threads : kLegThreadsDefault;
            leg_kernel<<<(unsigned)((threads + lt - 1) / lt), lt, 0, st>>>(LP);
            if ((rc = sss_check_launch("leg_kernel"))) return rc;
            if (g_timer.on) cudaEventRecord(g_timer.get(), st);
            PP.ctx.points = LP.points;
            cudaMemsetAsync(PP.counter, 0, sizeof(unsigned int), st);
            if (g_timer.on) cudaEventRecord(g_timer.get(), st);
            if ((rc = (p->flags & SSS_FLAG_KAHAN) ? dispatch_pairs_kahan(PP, st) : dispatch_pairs_plain(PP, st)))
                return rc;
            if (g_timer.on) cudaEventRecord(g_timer.get(), st);
            g_timer.launches += 2;
            g_timer.waves += 1;
        }
        first += npts;
    }
    return SSS_OK;
}

extern "C" void sss_set_timing(int enable)
{
    g_timer.clear();
    g_timer.work = nullptr;
    g_timer.on = enable != 0;
}

extern "C" int sss_get_timing(double out[6])
{
    if (!out) return sss_set_error(SSS_ERR_INVALID, "sss_get_timing: null output");
    double leg = 0, pair = 0;
    for (size_t i = 0; i + 3 < g_timer.ev.size(); i += 4) {
        float a = 0, b = 0;
        if (cudaEventSynchronize(g_timer.ev[i + 3]) != cudaSuccess ||
            cudaEventElapsedTime(&a, g_timer.ev[i], g_timer.ev[i + 1]) != cudaSuccess ||
            cudaEventElapsedTime(&b, g_timer.ev[i + 2], g_timer.ev[i + 3]) != cudaSuccess)
            return sss_set_error(SSS_ERR_CUDA, "sss_get_timing: event query failed");
        leg += a;
        pair += b;
    }
    out[0] = leg;
    out[1] = pair;
    out[2] = g_timer.launches;
    out[3] = g_timer.waves;
    unsigned long long h[2] = {0, 0};
    if (g_timer.work && g_timer.on) {
        if (cudaMemcpy(h, g_timer.work, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
            return sss_set_error(SSS_ERR_CUDA, "sss_get_timing: counter copy failed");
    }
    out[4] = (double)h[0] * g_timer.nbins;  // 2^x evaluations (voxel x bin)
    out[5] = (double)h[1];                  // detector-pair evaluations
    return SSS_OK;
}

extern "C" int sss_tof_densify(const float* compact, int32_t nbins, int32_t nru, int32_t ndu,
                               int32_t nd, const int16_t* lor, const int32_t* detectors,
                               float* dense, int32_t* status, void* stream)
{
    if (!compact || !lor || !detectors || !dense || !status || nbins < 1 || nru < 1 || ndu < 1 || nd < 2)
        return sss_set_error(SSS_ERR_INVALID, "sss_tof_densify: bad argument");
    long long nl = (long long)nru * ndu;
    long long total = (long long)nbins * nl * nl;
    densify_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        compact, nbins, nru, ndu, nd, lor, detectors, dense, status);
    return sss_check_launch("densify_kernel");
}

namespace {

int densify_full(const float* compact, int32_t nbins, int32_t nru, int32_t ndu, int32_t nd, const int32_t* cell_pair,
                 float* dense, int32_t* status, void* stream, bool sampled_only, const char* who)
{
    if (!compact || !cell_pair || !dense || !status || nbins < 1 || nru < 1 || ndu < 1 || nd < 2)
        return sss_set_error(SSS_ERR_INVALID, "%s: bad argument", who);
    if ((nru * nru) % 4 != 0 || (uintptr_t)dense % 16 != 0)
        return sss_set_error(SSS_ERR_INVALID, "%s: needs nru*nru a multiple of 4 and a 16-byte aligned output", who);
    // the destination must be memory the device can address: device memory,
    // or host memory page-locked through CUDA (written at its device address)
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, dense) != cudaSuccess) {
        cudaGetLastError();
        return sss_set_error(SSS_ERR_INVALID, "%s: output pointer unknown to CUDA", who);
    }
    float* dst = nullptr;
    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged)
        dst = dense;
    else if (attr.type == cudaMemoryTypeHost && attr.devicePointer)
        dst = (float*)attr.devicePointer;
    else
        return sss_set_error(SSS_ERR_INVALID, "%s: output must be device memory or page-locked host memory", who);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long ncell = (long long)(nd + 1) * (nd / 2);
    const long long total4 = (long long)nbins * ncell * nru * nru / 4;
    const long long want = (total4 + 255) / 256;
    const unsigned blocks = (unsigned)std::max<long long>(1, std::min<long long>(want, (long long)sms * 8));
    if (sampled_only) {
        const long long cw = (ncell * 32 + 255) / 256;  // one warp a cell
        const unsigned cb = (unsigned)std::max<long long>(1, std::min<long long>(cw, (long long)sms * 16));
        densify_cells_kernel<<<cb, 256, 0, (cudaStream_t)stream>>>(compact, nbins, nru, ndu, ncell, cell_pair, dst,
                                                                   status);
        return sss_check_launch("densify_cells_kernel");
    }
    densify_full_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(compact, nbins, nru, ndu, ncell, cell_pair, dst,
                                                                  status);
    return sss_check_launch("densify_full_kernel");
}

}  // namespace

extern "C" int sss_tof_densify_full(const float* compact, int32_t nbins, int32_t nru, int32_t ndu, int32_t nd,
                                    const int32_t* cell_pair, float* dense, int32_t* status, void* stream)
{
    return densify_full(compact, nbins, nru, ndu, nd, cell_pair, dense, status, stream, false,
                        "sss_tof_densify_full");
}

extern "C" int sss_tof_densify_cells(const float* compact, int32_t nbins, int32_t nru, int32_t ndu, int32_t nd,
                                     const int32_t* cell_pair, float* dense, int32_t* status, void* stream)
{
    return densify_full(compact, nbins, nru, ndu, nd, cell_pair, dense, status, stream, true,
                        "sss_tof_densify_cells");
}

// ---------------------------------------------------------------- no-allocation scatter points
//
// sss_scatter_points_noalloc: the same scatter-point enumeration as
// sss_scatter_points for callers that must not allocate device memory —
// code that runs inside a fixed memory arena or pool it does not own, or in
// a process whose memory is capped so that a late allocation could fail
// mid-pipeline.  Its scratch (the running total and one counter per sampled
// z-slice) lives in the file-scope array below instead of a temporary
// buffer.  Like sss_scatter_points it copies the counts to the host and
// synchronises the stream.
namespace {

// At most this many sampled z-slices (ceil(nz / sample_step_z)).
constexpr int kNoAllocMaxSlices = 4096;
constexpr int kNoAllocMaxDevices = 64;

// [0] = total points, [1 + i] = points of sampled slice i.  32 KiB that every
// GPU which loads this library keeps until the process exits.  All calls
// share it: each call clears the part it uses before the kernel runs, and two
// calls whose work overlaps on the GPU race on it.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[1 + kNoAllocMaxSlices];

std::mutex g_noalloc_lock;
unsigned long long* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device (host code cannot use the symbol's name as an address) and kept: a
// device reset after the first call would leave it stale, which the header
// rules out.
int noalloc_scratch(unsigned long long** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_scatter_points_noalloc: no current device");
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return sss_set_error(SSS_ERR_INVALID, "sss_scatter_points_noalloc: device %d not supported", dev);
    std::lock_guard<std::mutex> guard(g_noalloc_lock);
    if (!g_noalloc_addr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return sss_set_error(SSS_ERR_CUDA, "sss_scatter_points_noalloc: cudaGetSymbolAddress: %s",
                                 cudaGetErrorString(e));
        g_noalloc_addr[dev] = (unsigned long long*)ptr;
    }
    *out = g_noalloc_addr[dev];
    return SSS_OK;
}

}  // namespace

extern "C" int sss_scatter_points_noalloc(const sss_tof_problem* p, double* points, int64_t capacity,
                                          int64_t* count, int64_t* slice_counts, void* stream)
{
    int rc = validate(p);
    if (rc) return rc;
    if (!count) return sss_set_error(SSS_ERR_INVALID, "sss_scatter_points_noalloc: null count");
    if (capacity > 0 && !points)
        return sss_set_error(SSS_ERR_INVALID, "sss_scatter_points_noalloc: null points");
    LatticeDims L = lattice(*p);
    if (L.lz > kNoAllocMaxSlices)
        return sss_set_error(SSS_ERR_INVALID,
                             "sss_scatter_points_noalloc: %d sampled z-slices exceed its limit of %d",
                             L.lz, kNoAllocMaxSlices);
    unsigned long long* scratch = nullptr;
    if ((rc = noalloc_scratch(&scratch))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const double* IS = p->image_size;
    double zvox = (IS[5] - IS[2]) / p->nz;  // :87
    double zstart = zvox / 2 - (-IS[2]);    // :176, :179
    double radius = -IS[0];                 // :177
    const size_t used = (1 + (size_t)L.lz) * sizeof(unsigned long long);
    if (cudaMemsetAsync(scratch, 0, used, st) != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_scatter_points_noalloc: clearing the scratch failed");
    scatter_points_kernel<<<1, 1024, 0, st>>>(p->attenuation, p->nx, p->ny, p->nz, L, radius, zstart,
                                               zvox, points, capacity, scratch, scratch + 1);
    if ((rc = sss_check_launch("scatter_points_kernel"))) return rc;
    unsigned long long total = 0;
    if (cudaMemcpyAsync(&total, scratch, sizeof(total), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        (slice_counts && cudaMemcpyAsync(slice_counts, scratch + 1, (size_t)L.lz * sizeof(int64_t),
                                         cudaMemcpyDeviceToHost, st) != cudaSuccess))
        return sss_set_error(SSS_ERR_CUDA, "sss_scatter_points_noalloc: copy failed");
    if (cudaStreamSynchronize(st) != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_scatter_points_noalloc: %s",
                             cudaGetErrorString(cudaGetLastError()));
    *count = (int64_t)total;
    if ((int64_t)total > capacity)
        return sss_set_error(SSS_ERR_CAPACITY, "sss_scatter_points_noalloc: %lld points > capacity %lld",
                             (long long)total, (long long)capacity);
    return SSS_OK;
}
