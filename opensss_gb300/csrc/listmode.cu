// CASToR list-mode events on the GPU: prompt histogramming and scatter
// injection (the reference's Timber package, Python/Timber/Datafile.py).
//
//  * histogram_kernel: one thread per event.  Crystal IDs -> (crystal, ring)
//    pairs and TOF sign as ParseCASToRIDs (Coincidence.py:97-159), sinogram
//    cell from the LOR and slice tables, TOF bin as ExportPrompts
//    (Datafile.py:86-113); counts are 32-bit atomics, reduced to the
//    reference's wrapping uint16 at the end.  The randoms and normalisation
//    sinograms keep the value of the last event (file order) of each cell,
//    as the reference's per-event assignment does: atomicMax of the event
//    number, then a pass over the cells writes the winners' values.
//  * inject_*: InjectScatters (Datafile.py:117-240): events outside the TOF
//    range or the tables are dropped, the others get a scatter rate inserted
//    after their correction factors; the kept events keep file order
//    (block counts, one scan, ordered writes).
#include "common.cuh"

namespace {

using namespace sss;

struct Parsed {
    int d1, r1, d2, r2;  // crystal (unshifted, d1 < d2) and ring of each side
    double tof;          // ps, sign for the (r1, r2) order
};

__device__ __forceinline__ uint32_t load_u32(const unsigned char* rec, int off)
{
    return *reinterpret_cast<const uint32_t*>(rec + off);
}

__device__ __forceinline__ float load_f32(const unsigned char* rec, int off)
{
    return *reinterpret_cast<const float*>(rec + off);
}

// ParseCASToRIDs (Coincidence.py:97-159) for the event at rec.
__device__ __forceinline__ Parsed parse_event(const unsigned char* rec, const sss_listmode_layout& L, int ncr,
                                              int shift)
{
    const long long a = load_u32(rec, L.id_offset), b = load_u32(rec, L.id_offset + 4);
    const double tof = (double)load_f32(rec, L.tof_offset);
    const long long id1 = a < b ? a : b, id2 = a < b ? b : a;
    const double tof_t = a < b ? tof : -tof;
    Parsed P;
    const int c1 = (int)(id1 % ncr), c2 = (int)(id2 % ncr);
    P.d1 = c1 < c2 ? c1 : c2;
    P.d2 = c1 < c2 ? c2 : c1;
    int s1 = c1 - shift, s2 = c2 - shift;
    if (s1 < 0) s1 += ncr;
    if (s2 < 0) s2 += ncr;
    if (s1 < s2) {
        P.r1 = (int)(id1 / ncr);
        P.r2 = (int)(id2 / ncr);
        P.tof = tof_t;
    } else {
        P.r1 = (int)(id2 / ncr);
        P.r2 = (int)(id1 / ncr);
        P.tof = -tof_t;
    }
    return P;
}

// Sinogram cell of an event: -1 = skipped as the reference skips it, -2 =
// outside the tables (the reference raises IndexError).
__device__ __forceinline__ long long event_cell(const Parsed& P, const sss_sino_map& M)
{
    const int i1 = P.d1 / M.mash, i2 = P.d2 / M.mash;
    if (i1 >= M.nd_lor || i2 >= M.nd_lor || P.r1 >= M.nr_table || P.r2 >= M.nr_table) return -2;
    const int ang = M.lor[2 * ((long long)i1 * M.nd_lor + i2)];
    const int rad = M.lor[2 * ((long long)i1 * M.nd_lor + i2) + 1];
    const int sino = M.slices[(long long)P.r1 * M.nr_table + P.r2];
    if (sino == -1 || rad == -1 || ang == -1) return -1;
    if (rad < 0 || rad >= M.nrad || ang < 0 || ang >= M.nang || sino < 0 || sino >= M.nslices) return -2;
    return ((long long)rad * M.nang + ang) * M.nslices + sino;
}

// TOF bin as the reference computes it (Datafile.py:103-110); -1 = outside.
__device__ __forceinline__ int tof_bin(double tof, const sss_sino_map& M)
{
    if (fabs(tof) > M.tof_range) return -1;
    const double w = (2.0 * M.tof_range) / M.tof_bins;
    const double t = (tof + M.tof_range) / w;
    if (t < 0.0 || t >= (double)M.tof_bins) return -1;
    return (int)t;
}

__global__ void histogram_kernel(const unsigned char* __restrict__ ev, long long n, sss_listmode_layout L,
                                 sss_sino_map M, unsigned int* __restrict__ counts,
                                 unsigned long long* __restrict__ last, int32_t* status)
{
    const int ncr = M.nd_lor * M.mash;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const Parsed P = parse_event(ev + e * L.record_bytes, L, ncr, M.shift);
        const long long cell = event_cell(P, M);
        if (cell == -2) {
            raise_error(status, kErrEvent);
            continue;
        }
        if (cell < 0) continue;
        if (last) atomicMax(last + cell, (unsigned long long)(e + 1));
        const int bin = tof_bin(P.tof, M);
        if (bin < 0) continue;
        atomicAdd(counts + cell * M.tof_bins + bin, 1u);
    }
}

__global__ void histogram_finish_kernel(const unsigned int* __restrict__ counts, long long n,
                                        uint16_t* __restrict__ prompts)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        prompts[i] = (uint16_t)(counts[i] & 0xffffu);  // numpy uint16 += 1 wraps
}

// One thread per cell: the cell's last event (numbered from 1 by the
// histogram pass, 0 = none) gives its randoms and normalisation values,
// event[0] * scan_duration / TOF_bins and event[1] (Datafile.py:95-99).  The
// cells are read in order and only the winning events at random: cheaper
// than parsing every event again to find the winners.
__global__ void last_values_kernel(const unsigned char* __restrict__ ev, long long n, sss_listmode_layout L,
                                   long long ncell, int tof_bins, const unsigned long long* __restrict__ last,
                                   double duration, float* __restrict__ randoms, float* __restrict__ norm)
{
    for (long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x; cell < ncell;
         cell += (long long)gridDim.x * blockDim.x) {
        const unsigned long long e1 = last[cell];
        if (e1 == 0 || e1 > (unsigned long long)n) continue;
        const unsigned char* rec = ev + (long long)(e1 - 1) * L.record_bytes;
        if (randoms) randoms[cell] = (float)(((double)load_u32(rec, 0) * duration) / tof_bins);
        if (norm) norm[cell] = load_f32(rec, 4);
    }
}

// ------------------------------------------------------------------ injection

constexpr int kInjectThreads = 256;

__device__ __forceinline__ bool inject_keep(const unsigned char* rec, const sss_listmode_layout& L,
                                            const sss_sino_map& M, const float* scat, const float* factor,
                                            float& rate, bool& bad)
{
    const Parsed P = parse_event(rec, L, M.nd_lor * M.mash, M.shift);
    if (fabs(P.tof) > M.tof_range) return false;  // :207-208, before the tables
    const long long cell = event_cell(P, M);
    if (cell == -2) {
        bad = true;
        return false;
    }
    if (cell < 0) return false;
    const int bin = tof_bin(P.tof, M);
    if (bin < 0) return false;
    const long long ncell = (long long)M.nrad * M.nang * M.nslices;
    rate = __fmul_rn(factor[bin], scat[bin * ncell + cell]);  // :229 in float32
    return true;
}

__global__ void __launch_bounds__(kInjectThreads) inject_count_kernel(
    const unsigned char* __restrict__ ev, long long n, sss_listmode_layout L, sss_sino_map M,
    const float* __restrict__ scat, const float* __restrict__ factor, unsigned int* __restrict__ block_counts,
    int32_t* status)
{
    const long long e = (long long)blockIdx.x * kInjectThreads + threadIdx.x;
    float rate;
    bool bad = false;
    const bool keep = e < n && inject_keep(ev + e * L.record_bytes, L, M, scat, factor, rate, bad);
    if (bad) raise_error(status, kErrEvent);
    const int c = __syncthreads_count(keep);
    if (threadIdx.x == 0) block_counts[blockIdx.x] = (unsigned int)c;
}

// Exclusive scan of the block counts in one block (counts are < 2^32 total
// per block; offsets are 64-bit).
__global__ void __launch_bounds__(1024) inject_scan_kernel(const unsigned int* __restrict__ counts, long long nb,
                                                           unsigned long long* __restrict__ offsets,
                                                           unsigned long long* __restrict__ total)
{
    __shared__ unsigned long long part[1024];
    const long long per = (nb + 1023) / 1024;
    const long long lo = threadIdx.x * per, hi = min(nb, lo + per);
    unsigned long long s = 0;
    for (long long i = lo; i < hi; ++i) s += counts[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned long long v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = part[threadIdx.x] - s;
    for (long long i = lo; i < hi; ++i) {
        offsets[i] = run;
        run += counts[i];
    }
    if (threadIdx.x == 1023) *total = part[1023];
}

__global__ void __launch_bounds__(kInjectThreads) inject_write_kernel(
    const unsigned char* __restrict__ ev, long long n, sss_listmode_layout L, sss_sino_map M,
    const float* __restrict__ scat, const float* __restrict__ factor,
    const unsigned long long* __restrict__ offsets, unsigned char* __restrict__ out, int out_bytes)
{
    __shared__ unsigned int warp_sums[kInjectThreads / 32];
    const long long e = (long long)blockIdx.x * kInjectThreads + threadIdx.x;
    float rate = 0.f;
    bool bad = false;
    const unsigned char* rec = ev + e * L.record_bytes;
    const bool keep = e < n && inject_keep(rec, L, M, scat, factor, rate, bad);
    // rank of this event among the block's kept events
    const unsigned int ballot = __ballot_sync(0xffffffffu, keep);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_sums[warp] = __popc(ballot);
    __syncthreads();
    unsigned int before = 0;
    for (int w = 0; w < warp; ++w) before += warp_sums[w];
    before += __popc(ballot & ((1u << lane) - 1u));
    if (!keep) return;
    unsigned char* dst = out + (offsets[blockIdx.x] + before) * (unsigned long long)out_bytes;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(rec);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    const int head = L.scatter_offset / 4, words = L.record_bytes / 4;
    for (int i = 0; i < head; ++i) d[i] = src[i];
    d[head] = __float_as_uint(rate);
    for (int i = head; i < words; ++i) d[i + 1] = src[i];
}

int check_layout(const sss_listmode_layout* L, const sss_sino_map* M, const char* who)
{
    if (!L || !M || !M->lor || !M->slices)
        return sss_set_error(SSS_ERR_INVALID, "%s: bad argument", who);
    if (L->record_bytes < 12 || L->record_bytes % 4 || L->id_offset % 4 || L->tof_offset % 4 ||
        L->id_offset < 0 || L->id_offset + 8 > L->record_bytes || L->tof_offset < 0 ||
        L->tof_offset + 4 > L->record_bytes || L->scatter_offset % 4 || L->scatter_offset < 0 ||
        L->scatter_offset > L->record_bytes)
        return sss_set_error(SSS_ERR_INVALID, "%s: event layout must be whole, 4-byte aligned fields", who);
    if (M->nd_lor < 1 || M->mash < 1 || M->nr_table < 1 || M->nrad < 1 || M->nang < 1 || M->nslices < 1 ||
        M->tof_bins < 1 || !(M->tof_range > 0.0))
        return sss_set_error(SSS_ERR_INVALID, "%s: bad sinogram map", who);
    return SSS_OK;
}

unsigned grid_for(long long n, int threads)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (n + threads - 1) / threads, cap = (long long)sms * 16;
    return (unsigned)(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace

extern "C" int sss_histogram_prompts(const void* events, int64_t n_events, const sss_listmode_layout* layout,
                                     const sss_sino_map* map, uint32_t* counts, unsigned long long* last,
                                     int32_t* status, void* stream)
{
    int rc = check_layout(layout, map, "sss_histogram_prompts");
    if (rc) return rc;
    if (n_events < 0 || (n_events > 0 && !events) || !counts)
        return sss_set_error(SSS_ERR_INVALID, "sss_histogram_prompts: bad argument");
    if (n_events == 0) return SSS_OK;
    histogram_kernel<<<grid_for(n_events, 256), 256, 0, (cudaStream_t)stream>>>(
        (const unsigned char*)events, n_events, *layout, *map, counts, last, status);
    return sss_check_launch("histogram_kernel");
}

extern "C" int sss_histogram_finish(const void* events, int64_t n_events, const sss_listmode_layout* layout,
                                    const sss_sino_map* map, const uint32_t* counts,
                                    const unsigned long long* last, double duration, uint16_t* prompts,
                                    float* randoms, float* norm, void* stream)
{
    int rc = check_layout(layout, map, "sss_histogram_finish");
    if (rc) return rc;
    if (!counts || !prompts || ((randoms || norm) && !last) || n_events < 0 || (n_events > 0 && !events))
        return sss_set_error(SSS_ERR_INVALID, "sss_histogram_finish: bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    const long long ncell = (long long)map->nrad * map->nang * map->nslices;
    const long long nbins = ncell * map->tof_bins;
    histogram_finish_kernel<<<grid_for(nbins, 256), 256, 0, st>>>(counts, nbins, prompts);
    if ((rc = sss_check_launch("histogram_finish_kernel"))) return rc;
    if ((randoms || norm) && n_events > 0) {
        last_values_kernel<<<grid_for(ncell, 256), 256, 0, st>>>((const unsigned char*)events, n_events, *layout,
                                                                  ncell, map->tof_bins, last, duration, randoms,
                                                                  norm);
        return sss_check_launch("last_values_kernel");
    }
    return SSS_OK;
}

extern "C" size_t sss_inject_workspace_size(int64_t n_events)
{
    const long long nb = (n_events + kInjectThreads - 1) / kInjectThreads;
    return (size_t)(((nb * 4 + 255) / 256) * 256 + ((nb * 8 + 255) / 256) * 256 + 256);
}

extern "C" int sss_inject_scatters(const void* events, int64_t n_events, const sss_listmode_layout* layout,
                                   const sss_sino_map* map, const float* scatters, const float* factor,
                                   void* out_events, unsigned long long* out_count, void* workspace,
                                   size_t workspace_bytes, int32_t* status, void* stream)
{
    int rc = check_layout(layout, map, "sss_inject_scatters");
    if (rc) return rc;
    if (n_events < 0 || (n_events > 0 && (!events || !out_events)) || !scatters || !factor || !out_count ||
        !workspace || workspace_bytes < sss_inject_workspace_size(n_events))
        return sss_set_error(SSS_ERR_INVALID, "sss_inject_scatters: bad argument or workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    if (n_events == 0) {
        if (cudaMemsetAsync(out_count, 0, sizeof(unsigned long long), st) != cudaSuccess)
            return sss_set_error(SSS_ERR_CUDA, "sss_inject_scatters: memset failed");
        return SSS_OK;
    }
    const long long nb = (n_events + kInjectThreads - 1) / kInjectThreads;
    if (nb > 0x7fffffffLL) return sss_set_error(SSS_ERR_INVALID, "sss_inject_scatters: too many events");
    char* ws = (char*)workspace;
    unsigned int* counts = (unsigned int*)ws;
    unsigned long long* offsets = (unsigned long long*)(ws + ((nb * 4 + 255) / 256) * 256);
    const unsigned char* ev = (const unsigned char*)events;
    inject_count_kernel<<<(unsigned)nb, kInjectThreads, 0, st>>>(ev, n_events, *layout, *map, scatters, factor,
                                                                  counts, status);
    if ((rc = sss_check_launch("inject_count_kernel"))) return rc;
    inject_scan_kernel<<<1, 1024, 0, st>>>(counts, nb, offsets, out_count);
    if ((rc = sss_check_launch("inject_scan_kernel"))) return rc;
    inject_write_kernel<<<(unsigned)nb, kInjectThreads, 0, st>>>(ev, n_events, *layout, *map, scatters, factor,
                                                                  offsets, (unsigned char*)out_events,
                                                                  layout->record_bytes + 4);
    return sss_check_launch("inject_write_kernel");
}
