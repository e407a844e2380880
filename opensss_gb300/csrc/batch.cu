// Batched TOF-SSS: many problems of different sizes run as one schedule.
//
// A plan enumerates every problem's scatter points (one small kernel per
// problem, one synchronisation), cuts the work into (problem, z-slice) items
// and packs consecutive items into waves that fit the workspace.  A wave is
// one leg launch over all its items and one persistent pair launch per TOF
// class (bin count and TOF kernel; a launch shares one TOF table in shared
// memory).  Every item carries its own problem's geometry, sampling, tables
// and output, so problems of different sizes share a launch.  All device
// memory a plan uses is carved from the caller's workspace, and sss_batch_run
// is a fixed sequence of asynchronous launches: the same plan can be run
// again on new activity maps (the attenuation, and with it the scatter
// points, stays fixed) and captured in a CUDA graph.
#include <algorithm>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "legs.cuh"
#include "pair.cuh"
#include "trace.cuh"

namespace {

using namespace sss;

struct LegItem {
    LegParams p;              // points / legA / legB / vox already point at this item's data
    long long thread_begin;   // prefix over the wave's items of npts * nl
};

struct PairItem {
    PairCtx ctx;              // legs indexed from the item's first point
    int npts;                 // the item's points (one z-slice)
    int nchunks;
    long long task_begin;     // prefix over the launch's items of nl * nchunks
};

__global__ void __launch_bounds__(kLegThreadsMax) batch_leg_kernel(const LegItem* __restrict__ items, int nitems,
                                                        long long total)
{
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= total) return;
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (items[mid].thread_begin <= gid) lo = mid;
        else hi = mid - 1;
    }
    const LegItem& it = items[lo];
    const long long local = gid - it.thread_begin;
    leg_one(it.p, (int)(local / it.p.nl), (int)(local % it.p.nl));
}

template <int NP, bool SINGLE, bool ODD, int MINB>
__global__ void __launch_bounds__(pair_block_warps(NP, false) * 32, MINB)
    batch_pair_kernel(const PairItem* __restrict__ items, int nitems, long long ntasks, TofConst T,
                      const float* tof_log2w, unsigned int* counter, int32_t* status)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float2* sAR = reinterpret_cast<float2*>(smem);
    unsigned char* sN = smem + kSmemNOff;
    float2* vbuf = reinterpret_cast<float2*>(smem + kSmemVbufOff) + (threadIdx.x >> 5) * 32;
    float* sG = reinterpret_cast<float*>(smem + kSmemGOff);
    // each warp's current item, copied from global memory when the warp moves
    // to another item, so that the task reads its problem's constants and
    // pointers from shared memory
    __shared__ PairItem witem[pair_block_warps(NP, false)];
    static_assert(sizeof(PairItem) % 4 == 0, "items are copied as words");
    load_pair_tables(tof_log2w, T, sAR, sN, sG);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    PairItem& it = witem[threadIdx.x >> 5];
    int cur = -1;
    bool tof_bad = false, energy_bad = false, nonfinite = false;
    unsigned long long walked = 0, npairs = 0;
    for (;;) {
        long long task = 0;
        if (lane == 0) task = atomicAdd(counter, 1u);
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= ntasks) break;
        int lo = 0, hi = nitems - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].task_begin <= task) lo = mid;
            else hi = mid - 1;
        }
        if (lo != cur) {  // warp-uniform: every lane found the same item
            __syncwarp();
            const int* src = reinterpret_cast<const int*>(items + lo);
            int* dst = reinterpret_cast<int*>(&it);
            for (int w = lane; w < (int)(sizeof(PairItem) / 4); w += 32) dst[w] = __ldg(src + w);
            __syncwarp();
            cur = lo;
        }
        const int rem = (int)(task - it.task_begin);
        walk_task<NP, SINGLE, ODD, false>(it.ctx, T, 0, it.npts, rem / it.nchunks, rem % it.nchunks, lane, sAR,
                                          sN, sG, vbuf, nullptr, nullptr, tof_bad, energy_bad, nonfinite, walked,
                                          npairs);
    }
    finish_pairs(lane, tof_bad, energy_bad, nonfinite, walked, npairs, status, nullptr);
}

using BatchPairFn = void (*)(const PairItem*, int, long long, TofConst, const float*, unsigned int*,
                            int32_t*);

template <int NP, bool SINGLE, bool ODD>
BatchPairFn batch_pair_fn()
{
    return batch_pair_kernel<NP, SINGLE, ODD, 2>;
}

// The pair kernel of a bin count (same register / occupancy choices as sss_tof_run).
BatchPairFn pick_batch_pairs(int nbins)
{
    if (nbins == 1) return batch_pair_fn<1, true, false>();
    const bool odd = nbins & 1;
    switch ((nbins + 1) / 2) {
#define SSS_BNP(k) \
    case k: return odd ? batch_pair_fn<k, false, true>() : batch_pair_fn<k, false, false>();
        SSS_BNP(1) SSS_BNP(2) SSS_BNP(3) SSS_BNP(4) SSS_BNP(5) SSS_BNP(6) SSS_BNP(7) SSS_BNP(8)
        SSS_BNP(9) SSS_BNP(10) SSS_BNP(11) SSS_BNP(12) SSS_BNP(13) SSS_BNP(14) SSS_BNP(15) SSS_BNP(16)
        SSS_BNP(17) SSS_BNP(18) SSS_BNP(19) SSS_BNP(20) SSS_BNP(21) SSS_BNP(22) SSS_BNP(23) SSS_BNP(24)
        SSS_BNP(25) SSS_BNP(26) SSS_BNP(27) SSS_BNP(28) SSS_BNP(29) SSS_BNP(30) SSS_BNP(31) SSS_BNP(32)
#undef SSS_BNP
    }
    return nullptr;
}

// Shared-memory opt-in and persistent grid size of a pair launch, decided at
// plan time so that a run only enqueues launches (and can be captured).
int prepare_batch_pairs(BatchPairFn fn, int nbins, int warps, long long ntasks, long long* blocks)
{
    const size_t smem = pair_smem_bytes(nbins);
    if (cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_batch_plan: %s", cudaGetErrorString(cudaGetLastError()));
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, warps * 32, smem);
    if (per_sm < 1) per_sm = 1;
    *blocks = std::max<long long>(1, std::min<long long>((long long)sms * per_sm, (ntasks + warps - 1) / warps));
    return SSS_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct LatticeSize {
    long long lz, capacity;
};

LatticeSize lattice_size(const sss_tof_problem& p)
{
    const long long lx = (p.nx + p.sample_step[0] - 1) / p.sample_step[0];
    const long long ly = (p.ny + p.sample_step[1] - 1) / p.sample_step[1];
    const long long lz = (p.nz + p.sample_step[2] - 1) / p.sample_step[2];
    return {lz, lx * ly * lz};
}

// leg-record bytes of `npts` scatter points of problem p
size_t item_bytes(const sss_tof_problem& p, long long npts)
{
    const long long nl = (long long)p.nru * p.ndu;
    const long long cap = (long long)p.nx + p.ny + p.nz;
    const size_t lists = (p.flags & SSS_FLAG_UNIT_TOF) ? 0 : align256(sizeof(float2) * npts * nl * cap);
    return 3 * align256(sizeof(float4) * npts * nl) + lists;
}

}  // namespace

struct sss_batch {
    struct Launch {
        int nbins;
        TofConst T;
        const float* tof;
        const PairItem* items;  // device
        int nitems;
        long long ntasks;
        unsigned int* counter;  // device
        BatchPairFn fn;
        long long blocks;
        int warps;              // warps per block (the class's first problem's pair_warps)
    };
    struct Wave {
        const LegItem* legs;    // device
        int nlegs;
        long long threads;
        int ctr_first;          // the wave's launch counters: counters[ctr_first ..]
        std::vector<Launch> launches;
    };
    std::vector<sss_tof_problem> problems;
    std::vector<float*> outs;
    std::vector<long long> npoints;
    std::vector<Wave> waves;
    int leg_threads = 128;      // leg-kernel block (the first problem's leg_threads)
    unsigned int* counters = nullptr;
    int ncounters = 0;
    int32_t* status = nullptr;
    long long units = 0;
};

namespace {

// Checks shared by both planning entry points.
int check_plan_args(const sss_tof_problem* problems, int32_t n, float* const* outs, void* workspace,
                    sss_batch** plan)
{
    if (!problems || n < 1 || !outs || !workspace || !plan)
        return sss_set_error(SSS_ERR_INVALID, "sss_batch_plan: bad argument");
    *plan = nullptr;
    for (int i = 0; i < n; ++i) {
        int rc = sss_internal_validate(&problems[i]);
        if (rc) return rc;
        if (!outs[i]) return sss_set_error(SSS_ERR_INVALID, "sss_batch_plan: null output %d", i);
    }
    return SSS_OK;
}

// Items, waves and descriptors of a plan whose scatter points are known:
// points[i] (device, [count][4]) and counts[i][z] (points of sampled slice z)
// for every problem.  The descriptors go to the workspace from `off` on.
int plan_items(const sss_tof_problem* problems, int32_t n, float* const* outs,
               const std::vector<const double*>& points,
               const std::vector<std::vector<unsigned long long>>& counts, char* ws, size_t off,
               size_t workspace_bytes, int32_t* status, sss_batch** plan, cudaStream_t st);

}  // namespace

extern "C" int sss_batch_plan(const sss_tof_problem* problems, int32_t n, float* const* outs,
                              void* workspace, size_t workspace_bytes, int32_t* status,
                              sss_batch** plan, void* stream)
{
    int rc = check_plan_args(problems, n, outs, workspace, plan);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    char* ws = (char*)workspace;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    // 1. scatter points of every problem
    std::vector<size_t> pts_off(n), cnt_off(n);
    std::vector<LatticeSize> lat(n);
    for (int i = 0; i < n; ++i) {
        lat[i] = lattice_size(problems[i]);
        pts_off[i] = take(sizeof(double) * 4 * (size_t)std::max<long long>(lat[i].capacity, 1));
        cnt_off[i] = take(sizeof(unsigned long long) * (size_t)(1 + lat[i].lz));
    }
    if (off > workspace_bytes)
        return sss_set_error(SSS_ERR_WORKSPACE, "sss_batch_plan: workspace too small for the point lists");
    for (int i = 0; i < n; ++i) {
        unsigned long long* cnt = (unsigned long long*)(ws + cnt_off[i]);
        if (cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (size_t)(1 + lat[i].lz), st) != cudaSuccess)
            return sss_set_error(SSS_ERR_CUDA, "sss_batch_plan: memset failed");
        int rc = sss_internal_scatter_points(&problems[i], (double*)(ws + pts_off[i]), lat[i].capacity,
                                             cnt, st);
        if (rc) return rc;
    }
    std::vector<std::vector<unsigned long long>> counts(n);
    std::vector<std::vector<unsigned long long>> raw(n);
    for (int i = 0; i < n; ++i) {
        raw[i].resize((size_t)(1 + lat[i].lz));
        if (cudaMemcpyAsync(raw[i].data(), ws + cnt_off[i], raw[i].size() * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return sss_set_error(SSS_ERR_CUDA, "sss_batch_plan: count copy failed");
    }
    if (cudaStreamSynchronize(st) != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_batch_plan: %s", cudaGetErrorString(cudaGetLastError()));
    std::vector<const double*> points(n);
    for (int i = 0; i < n; ++i) {
        counts[i].assign(raw[i].begin() + 1, raw[i].end());
        points[i] = (const double*)(ws + pts_off[i]);
    }
    return plan_items(problems, n, outs, points, counts, ws, off, workspace_bytes, status, plan, st);
}

extern "C" int sss_batch_plan_points(const sss_tof_problem* problems, int32_t n, float* const* outs,
                                     const double* const* points, const int64_t* const* slice_counts,
                                     void* workspace, size_t workspace_bytes, int32_t* status,
                                     sss_batch** plan, void* stream)
{
    int rc = check_plan_args(problems, n, outs, workspace, plan);
    if (rc) return rc;
    if (!points || !slice_counts) return sss_set_error(SSS_ERR_INVALID, "sss_batch_plan_points: bad argument");
    std::vector<const double*> pts(n);
    std::vector<std::vector<unsigned long long>> counts(n);
    for (int i = 0; i < n; ++i) {
        const LatticeSize lat = lattice_size(problems[i]);
        if (!slice_counts[i] || (!points[i] && lat.capacity > 0))
            return sss_set_error(SSS_ERR_INVALID, "sss_batch_plan_points: null points of problem %d", i);
        counts[i].resize((size_t)lat.lz);
        const long long per_slice = lat.lz > 0 ? lat.capacity / lat.lz : 0;  // lattice points of one slice
        for (long long z = 0; z < lat.lz; ++z) {
            if (slice_counts[i][z] < 0 || slice_counts[i][z] > per_slice)
                return sss_set_error(SSS_ERR_INVALID,
                                     "sss_batch_plan_points: problem %d slice %lld has %lld points (0..%lld)", i, z,
                                     (long long)slice_counts[i][z], per_slice);
            counts[i][(size_t)z] = (unsigned long long)slice_counts[i][z];
        }
        pts[i] = points[i];
    }
    return plan_items(problems, n, outs, pts, counts, (char*)workspace, 0, workspace_bytes, status, plan,
                      (cudaStream_t)stream);
}

namespace {

int plan_items(const sss_tof_problem* problems, int32_t n, float* const* outs,
               const std::vector<const double*>& points,
               const std::vector<std::vector<unsigned long long>>& counts, char* ws, size_t off,
               size_t workspace_bytes, int32_t* status, sss_batch** plan, cudaStream_t st)
{
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    // 2. items = (problem, z-slice) with points
    struct Item {
        int prob;
        long long first, count;
    };
    std::vector<Item> items;
    std::unique_ptr<sss_batch> B(new sss_batch());
    B->problems.assign(problems, problems + n);
    if (problems[0].leg_threads) B->leg_threads = problems[0].leg_threads;
    B->outs.assign(outs, outs + n);
    B->status = status;
    for (int i = 0; i < n; ++i) {
        long long first = 0;
        for (size_t z = 0; z < counts[i].size(); ++z) {
            const long long c = (long long)counts[i][z];
            if (c > 0) items.push_back({i, first, c});
            first += c;
        }
        B->npoints.push_back(first);
        const long long nru = problems[i].nru, ndu = problems[i].ndu;
        const long long pairs = nru * nru * ndu * (ndu - 1) / 2 + ndu * nru * (nru - 1);
        B->units += first * pairs * problems[i].nbins;
    }
    // descriptors: one LegItem and one PairItem per item, counters per launch
    const size_t desc_off = take(sizeof(LegItem) * std::max<size_t>(items.size(), 1));
    const size_t pdesc_off = take(sizeof(PairItem) * std::max<size_t>(items.size(), 1));
    const int max_launches = (int)items.size() + 1;
    const size_t ctr_off = take(sizeof(unsigned int) * (size_t)max_launches);
    const size_t data_off = off;
    if (data_off >= workspace_bytes)
        return sss_set_error(SSS_ERR_WORKSPACE, "sss_batch_plan: no workspace left for leg records");
    const size_t data_bytes = workspace_bytes - data_off;

    // 3. waves of consecutive items that fit
    std::vector<LegItem> hleg(items.size());
    std::vector<PairItem> hpair(items.size());
    LegItem* dleg = (LegItem*)(ws + desc_off);
    PairItem* dpair = (PairItem*)(ws + pdesc_off);
    unsigned int* dctr = (unsigned int*)(ws + ctr_off);
    int nctr = 0;
    size_t k = 0;
    while (k < items.size()) {
        size_t used = 0, k_end = k;
        while (k_end < items.size()) {
            const size_t b = item_bytes(problems[items[k_end].prob], items[k_end].count);
            if (used + b > data_bytes) break;
            used += b;
            ++k_end;
        }
        if (k_end == k)
            return sss_set_error(SSS_ERR_WORKSPACE,
                                 "sss_batch_plan: a z-slice of problem %d needs %zu bytes of leg records, "
                                 "only %zu available", items[k].prob,
                                 item_bytes(problems[items[k].prob], items[k].count), data_bytes);
        sss_batch::Wave W;
        W.ctr_first = nctr;
        W.legs = dleg + k;
        W.nlegs = (int)(k_end - k);
        W.threads = 0;
        size_t doff = data_off;
        // group the wave's items by TOF class for the pair launches
        std::map<std::tuple<int, double, double>, std::vector<size_t>> classes;
        for (size_t j = k; j < k_end; ++j) {
            const Item& it = items[j];
            const sss_tof_problem& p = problems[it.prob];
            const long long nl = (long long)p.nru * p.ndu, cap = (long long)p.nx + p.ny + p.nz;
            LegItem& L = hleg[j];
            L.p.g = grid_of(p.nx, p.ny, p.nz, p.image_size);
            L.p.act = p.activity;
            L.p.mu = p.attenuation;
            L.p.geom = p.geometry;
            L.p.normals = p.normals;
            L.p.rings = p.rings;
            L.p.dets = p.detectors;
            L.p.nr = p.nr;
            L.p.nd = p.nd;
            L.p.nru = p.nru;
            L.p.ndu = p.ndu;
            L.p.nl = (int)nl;
            L.p.cap = (int)cap;
            L.p.nvox = (long long)p.nx * p.ny * p.nz;
            L.p.points = points[it.prob] + 4 * it.first;
            L.p.npts = (int)it.count;
            L.p.legA = (float4*)(ws + doff);
            doff += align256(sizeof(float4) * it.count * nl);
            L.p.legB = (float4*)(ws + doff);
            doff += align256(sizeof(float4) * it.count * nl);
            L.p.legC = (float4*)(ws + doff);
            doff += align256(sizeof(float4) * it.count * nl);
            if (p.flags & SSS_FLAG_UNIT_TOF) {
                L.p.vox = nullptr;  // every TOF weight is 1: the pairs use the leg integrals
            } else {
                L.p.vox = (float2*)(ws + doff);
                doff += align256(sizeof(float2) * it.count * nl * cap);
            }
            L.p.vox_lo = nullptr;
            L.p.status = status;
            L.thread_begin = W.threads;
            W.threads += it.count * nl;
            classes[std::make_tuple(p.nbins, p.tof_bin_width, p.tof_resolution)].push_back(j);
        }
        // pair items, contiguous per class
        size_t pk = k;
        for (auto& kv : classes) {
            sss_batch::Launch Lc;
            const sss_tof_problem& p0 = problems[items[kv.second[0]].prob];
            Lc.nbins = p0.nbins;
            Lc.T = tof_const(p0);
            Lc.tof = p0.tof_log2w;
            Lc.items = dpair + pk;
            Lc.nitems = (int)kv.second.size();
            Lc.ntasks = 0;
            Lc.counter = dctr + nctr++;
            Lc.fn = pick_batch_pairs(p0.nbins);
            Lc.warps = p0.pair_warps ? p0.pair_warps : pair_block_warps((p0.nbins + 1) / 2, false);
            if (!Lc.fn) return sss_set_error(SSS_ERR_INVALID, "sss_batch_plan: nbins out of range");
            for (size_t j : kv.second) {
                const Item& it = items[j];
                const sss_tof_problem& p = problems[it.prob];
                PairItem& P = hpair[pk++];
                PairCtx& C = P.ctx;
                C.nru = p.nru;
                C.ndu = p.ndu;
                C.nl = p.nru * p.ndu;
                C.nd = p.nd;
                C.cap = p.nx + p.ny + p.nz;
                C.nbins = p.nbins;
                C.geo_c = geo_const(p);
                C.gamma_kn = gamma_kn_const();
                C.eff = p.efficiency;
                C.ratio = p.atten_ratio;
                C.geom = p.geometry;
                C.rings = p.rings;
                C.dets = p.detectors;
                C.points = hleg[j].p.points;
                C.legA = hleg[j].p.legA;
                C.legB = hleg[j].p.legB;
                C.legC = hleg[j].p.legC;
                C.vox = hleg[j].p.vox;
                C.vox_lo = nullptr;  // the batched engine runs the plain pair kernel
                C.unit_tof = (p.flags & SSS_FLAG_UNIT_TOF) != 0;
                C.out = outs[it.prob];
                P.npts = (int)it.count;
                P.nchunks = pair_chunks(p.nru, p.ndu);
                P.task_begin = Lc.ntasks;
                Lc.ntasks += (long long)C.nl * P.nchunks;
            }
            int rc = prepare_batch_pairs(Lc.fn, Lc.nbins, Lc.warps, Lc.ntasks, &Lc.blocks);
            if (rc) return rc;
            W.launches.push_back(Lc);
        }
        B->waves.push_back(W);
        k = k_end;
    }
    if (!items.empty()) {
        if (cudaMemcpyAsync(dleg, hleg.data(), sizeof(LegItem) * hleg.size(), cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaMemcpyAsync(dpair, hpair.data(), sizeof(PairItem) * hpair.size(), cudaMemcpyHostToDevice,
                            st) != cudaSuccess)
            return sss_set_error(SSS_ERR_CUDA, "sss_batch_plan: descriptor upload failed");
        if (cudaStreamSynchronize(st) != cudaSuccess)
            return sss_set_error(SSS_ERR_CUDA, "sss_batch_plan: %s", cudaGetErrorString(cudaGetLastError()));
    }
    B->counters = dctr;
    B->ncounters = nctr;
    *plan = B.release();
    return SSS_OK;
}

}  // namespace

extern "C" int sss_batch_run_waves(const sss_batch* B, int32_t first, int32_t count, void* stream)
{
    if (!B) return sss_set_error(SSS_ERR_INVALID, "sss_batch_run: null plan");
    const int nw = (int)B->waves.size();
    if (first < 0 || count < 0 || first > nw || count > nw - first)
        return sss_set_error(SSS_ERR_INVALID, "sss_batch_run_waves: waves [%d, %d) outside [0, %d)", first,
                             first + count, nw);
    cudaStream_t st = (cudaStream_t)stream;
    if (first == 0) {
        for (size_t i = 0; i < B->problems.size(); ++i) {
            const sss_tof_problem& p = B->problems[i];
            const size_t nl = (size_t)p.nru * p.ndu;
            if (cudaMemsetAsync(B->outs[i], 0, sizeof(float) * p.nbins * nl * nl, st) != cudaSuccess)
                return sss_set_error(SSS_ERR_CUDA, "sss_batch_run: memset failed");
        }
    }
    for (int w = first; w < first + count; ++w) {
        const auto& W = B->waves[(size_t)w];
        if (!W.launches.empty() &&
            cudaMemsetAsync(B->counters + W.ctr_first, 0, sizeof(unsigned int) * W.launches.size(), st) !=
                cudaSuccess)
            return sss_set_error(SSS_ERR_CUDA, "sss_batch_run: memset failed");
        const int lt = B->leg_threads;
        batch_leg_kernel<<<(unsigned)((W.threads + lt - 1) / lt), lt, 0, st>>>(W.legs, W.nlegs, W.threads);
        int rc = sss_check_launch("batch_leg_kernel");
        if (rc) return rc;
        for (const auto& L : W.launches) {
            L.fn<<<(unsigned)L.blocks, L.warps * 32, pair_smem_bytes(L.nbins),
                   st>>>(
                L.items, L.nitems, L.ntasks, L.T, L.tof, L.counter, B->status);
            rc = sss_check_launch("batch_pair_kernel");
            if (rc) return rc;
        }
    }
    return SSS_OK;
}

extern "C" int sss_batch_run(const sss_batch* B, void* stream)
{
    if (!B) return sss_set_error(SSS_ERR_INVALID, "sss_batch_run: null plan");
    return sss_batch_run_waves(B, 0, (int32_t)B->waves.size(), stream);
}

extern "C" int sss_batch_info(const sss_batch* B, int64_t* info)
{
    if (!B || !info) return sss_set_error(SSS_ERR_INVALID, "sss_batch_info: bad argument");
    int64_t launches = 0;
    for (const auto& W : B->waves) launches += 1 + (int64_t)W.launches.size();
    info[0] = (int64_t)B->waves.size();
    info[1] = launches;
    info[2] = B->units;
    int64_t pts = 0;
    for (long long v : B->npoints) pts += v;
    info[3] = pts;
    return SSS_OK;
}

extern "C" void sss_batch_free(sss_batch* B) { delete B; }
