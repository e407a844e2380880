// Upsampling, tail mask and back-projection fit on sm_103a.
//
//  * upsample_kernel: the reference's nearest-neighbour upsampling
//    (Python/openSSS/Interpolation.py:197-319) is a pure gather once the
//    geometry-time source tables exist: output (cell, slice) copies the
//    sampled value at cell_src[cell] + ring_off[ring_idx[slice]] (clamped at
//    0 like fill_with_interp1d, :163), optionally summed over TOF bins in bin
//    order (:317).  HBM-write bound.
//  * mask_kernel: MaskDetectors (Python/openSSS/TailsMask.py:84-163): one
//    thread per LOR on the AccelerationFactor lattice, FP64 walk and FP64
//    line integral, mask = (1/exp(-sum) == 1).
//  * bp_kernel + fit_reduce_kernel + fit_final_kernel: BackProjection and
//    BackProjectionScatterRandFit (Python/openSSS/BackProjection.py:31-215):
//    one thread per LOR, FP32 atomic scatter-add of P/n, S/n, R/n and 1 into
//    four images, then per voxel Sbp = S/sens, T = max(P/sens - R/sens, 0)
//    and the slope sum(x T)/sum(x^2) in FP64 with x = float(Sbp * 1e10).
#include "common.cuh"
#include "trace.cuh"

namespace {

using namespace sss;

// LOR number -> (ring1, ring2, crystal index 1, crystal index 2) with the
// ring pair fastest, so a warp handles one crystal pair on neighbouring ring
// pairs (same sinogram cell, nearby slices, similar voxel paths).
struct LorIndex {
    int r1, r2, i1, i2;
};

__device__ __forceinline__ LorIndex lor_of(long long id, int nr, int na)
{
    LorIndex L;
    L.r2 = (int)(id % nr);
    id /= nr;
    L.r1 = (int)(id % nr);
    id /= nr;
    L.i2 = (int)(id % na);
    L.i1 = (int)(id / na);
    return L;
}

// LOR number -> rings, crystal indices and sinogram slice.  Without a pair
// list every ring pair (r1, r2) of the geometry is used and `slice_of`
// ([nr][nr]) gives its slice; with one (span: the mashed sinograms on the
// expanded geometry) the LOR's ring pair is pairs[p] = (Ring1, Ring2, slice),
// p fastest.
struct LorRef {
    int r1, r2, i1, i2, slice;
};

__device__ __forceinline__ LorRef lor_ref(long long id, int nr, int na, const int16_t* slice_of,
                                          const int32_t* pairs, int npairs)
{
    LorRef R;
    if (pairs) {
        const int p = (int)(id % npairs);
        id /= npairs;
        R.i2 = (int)(id % na);
        R.i1 = (int)(id / na);
        R.r1 = pairs[3 * p];
        R.r2 = pairs[3 * p + 1];
        R.slice = pairs[3 * p + 2];
    } else {
        const LorIndex L = lor_of(id, nr, na);
        R.r1 = L.r1;
        R.r2 = L.r2;
        R.i1 = L.i1;
        R.i2 = L.i2;
        R.slice = slice_of[L.r1 * nr + L.r2];
    }
    return R;
}

// The caller-table parts of a LOR: its slice in 0..nslices-1 and (span
// pair lists) its rings in 0..nr-1.
__device__ __forceinline__ bool lor_ref_ok(const LorRef& L, int nr, int nslices)
{
    return (unsigned)L.slice < (unsigned)nslices && (unsigned)L.r1 < (unsigned)nr && (unsigned)L.r2 < (unsigned)nr;
}

__device__ __forceinline__ void lor_line(const double* geom, int nd, int r1, int d1, int r2, int d2,
                                         double* lc)
{
    const double* p1 = geom + 3 * ((long long)r1 * nd + d1);
    const double* p2 = geom + 3 * ((long long)r2 * nd + d2);
    lc[0] = p1[0];
    lc[1] = p1[1];
    lc[2] = geom[3 * ((long long)r1 * nd) + 2];  // the ring's z (TailsMask.py:118, :125)
    lc[3] = p2[0];
    lc[4] = p2[1];
    lc[5] = geom[3 * ((long long)r2 * nd) + 2];
}

// ---------------------------------------------------------------- upsampling

// One sinogram cell per block iteration: the cell's distinct sampled ring
// pairs (nring values, bins summed in bin order) go to shared memory, then
// the cell's nslices outputs are written from there with coalesced
// streaming stores.  Every sampled value a cell needs is read once per cell
// instead of once per output.
__global__ void __launch_bounds__(256) upsample_kernel(const float* __restrict__ in, long long bin_stride,
                                                       int nbins, const long long* __restrict__ cell_src,
                                                       long long ncell,
                                                       const long long* __restrict__ ring_off, int nring,
                                                       const int32_t* __restrict__ ring_idx, int nslices,
                                                       float* __restrict__ out)
{
    extern __shared__ float vals[];
    for (long long cell = blockIdx.x; cell < ncell; cell += gridDim.x) {
        const long long base = cell_src[cell];
        __syncthreads();  // the previous cell's stores have read vals
        for (int j = threadIdx.x; j < nring; j += blockDim.x) {
            const float* src = in + base + ring_off[j];
            float acc = 0.f;
            for (int b = 0; b < nbins; ++b) acc += fmaxf(__ldg(src + (long long)b * bin_stride), 0.f);
            vals[j] = acc;
        }
        __syncthreads();
        float* o = out + cell * nslices;
        if ((nslices & 3) == 0 && ((reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(ring_idx)) & 15) == 0) {
            // four slices per store: the row start is 16-byte aligned
            const int4* ri4 = reinterpret_cast<const int4*>(ring_idx);
            float4* o4 = reinterpret_cast<float4*>(o);
            for (int q = threadIdx.x; q < (nslices >> 2); q += blockDim.x) {
                const int4 r = __ldg(ri4 + q);
                __stcs(o4 + q, make_float4(vals[r.x], vals[r.y], vals[r.z], vals[r.w]));
            }
        } else {
            for (int sl = threadIdx.x; sl < nslices; sl += blockDim.x) __stcs(o + sl, vals[__ldg(ring_idx + sl)]);
        }
    }
}

// ---------------------------------------------------------------- tail mask

struct MaskParams {
    Grid g;
    const float* mu;            // attenuation, or activity when use_activity
    int use_activity;
    long long nvox;
    const double* geom;
    const int16_t* lor;
    const int16_t* sino;
    const int32_t* pairs;       // span: [npairs][3] (Ring1, Ring2, slice), else null
    int npairs, nslices;
    int nr, nd, na, af, cap;
    double acf_below;           // 0: the reference's rule ACF == 1; else mask where ACF < acf_below
    double decided;             // a line integral above this fixes the LOR as not masked
    uint8_t* out;
    int32_t* status;
};

constexpr double kDecided = 1e-6;  // far above the 2^-53 where 1/exp(-s) stops being 1

// Pre-pass of the tail mask: notes a negative or NaN map value in the status word.
__global__ void map_sign_kernel(const float* __restrict__ map, long long n, int32_t* status)
{
    bool signed_value = false;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float v = map[i];
        if (!(v >= 0.f)) signed_value = true;
    }
    if (__syncthreads_or(signed_value) && threadIdx.x == 0) atomicOr(status, kNoteMapSigned);
}

__global__ void __launch_bounds__(128) mask_kernel(MaskParams P)
{
    const long long n = (long long)(P.pairs ? P.npairs : P.nr * P.nr) * P.na * P.na;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const LorRef L = lor_ref(id, P.nr, P.na, P.sino, P.pairs, P.npairs);
    const int d1 = L.i1 * P.af, d2 = L.i2 * P.af;
    if ((d1 == d2 && L.r1 == L.r2) || d1 > d2) return;  // TailsMask.py:129, :273
    if (!lor_ref_ok(L, P.nr, P.nslices)) {  // the caller's slice or ring-pair table
        raise_error(P.status, kErrTable);
        return;
    }
    double lc[6];
    lor_line(P.geom, P.nd, L.r1, d1, L.r2, d2, lc);
    double acf = 1.0;  // a miss gives Attenuation = 1 (:146-148)
    Ray r;
    if (ray_setup(P.g, lc, 1e-20, r)) {
        double sum = 0.0;
        bool bad = false;
        // With a map of non-negative values the sum only grows: once it is
        // above P.decided the mask value is fixed (the factor is past the rule's
        // bound, or activity > 0) and the remaining lengths need not be
        // evaluated.  The walk itself always runs to the end, so an overrun is
        // still reported.
        const bool nonneg = !(*(volatile const int32_t*)P.status & kNoteMapSigned);
        int c = ray_walk(P.g, r, P.cap, [&](int, int64_t lin, double t0, double t1) {
            const long long v = lin - 1;
            if (v < 0 || v >= P.nvox) {
                bad = true;
                return;
            }
            // a zero voxel adds exactly +0 whatever its length, so the FP64
            // length (the walk's dominant cost) is evaluated only where it counts
            const float mu = __ldg(P.mu + v);
            if (mu != 0.f && !(nonneg && sum > P.decided)) sum = add64(sum, mul64((double)mu, ref_length(r, t0, t1)));
        });
        if (c < 0) raise_error(P.status, kErrOverrun);
        if (bad) raise_error(P.status, kErrVoxel);
        if (P.use_activity)
            acf = sum > 0.0 ? 0.0 : 1.0;  // :153-156
        else if (nonneg && sum == 0.0)
            acf = 1.0;  // 1 / exp(-0), exactly
        else if (nonneg && sum > P.decided)
            acf = INFINITY;  // past either rule's bound: not masked (the factor's value is not needed)
        else
            acf = div64(1.0, exp(-sum));  // :144-148
    }
    // :150-161 (ACF == 1), or the caller's bound on the factor; one LOR per (cell, slice)
    const bool tail = (P.acf_below > 0.0 && !P.use_activity) ? acf < P.acf_below : acf == 1.0;
    if (tail) {
        const int ang = P.lor[2 * ((long long)d1 * P.nd + d2)];
        const int rad = P.lor[2 * ((long long)d1 * P.nd + d2) + 1];
        if (rad < 0 || rad > P.nd || ang < 0 || ang >= P.nd / 2) {  // the caller's LOR table
            raise_error(P.status, kErrTable);
            return;
        }
        const long long cell = (long long)rad * (P.nd / 2) + ang;
        P.out[cell * P.nslices + L.slice] = 1;
    }
}

// ---------------------------------------------------------------- back-projection fit

struct FitParams {
    Grid g;
    long long nvox;
    const double* geom;
    const int16_t* lor;
    const int16_t* order;       // [nr][nr]: slice read by the LOR (Ring1, Ring2) (:157-176)
    const int32_t* pairs;       // span: [npairs][3] (Ring1, Ring2, slice), else null
    int npairs, nslices;
    int length_weighted;        // span: value * length / sum(lengths) (:294-297), else value / n
    int nr, nd, na, af, cap;
    int nbins;                  // bins fitted together (one walk per LOR serves all)
    long long prompt_stride;    // elements between the bins' prompt sinograms
    long long scat_stride;      // elements between the bins' scatter values
    const float* prompts;       // [bin][cell][slice]
    const float* randoms;       // [cell][slice], shared by the bins
    const float* mask_f32;      // either a float mask (multiplied, :157-167) ...
    const uint8_t* mask_u8;     // ... or a uint8 tail mask (mask >= 1, Scaling.py:76)
    const float* scat;          // scatter values, addressed through the tables below
    const long long* scat_cell; // [cell] offset of the scatter value's cell
    const long long* scat_ring; // [slice] offset of the scatter value's slice
    int scat_clamp;             // clamp the scatter value at 0 (upsampling's fill, :163)
    float* img;                 // [nbins + 1][4 * nvox]: bins 2q, 2q+1 share blocks 2q, 2q+1 as
                                // float4 (P, S, P, S) then (R, sens, R, sens); an odd last bin
                                // has float2 (P, S) then (R, sens); block nbins holds, as float2
                                // in its second half, the R and sensitivity of the LORs that every
                                // bin uses
    int32_t* status;
};

// Scatter value of bin b at (cell, slice), clamped as the upsampling fills it.
__device__ __forceinline__ float fit_scatter(const FitParams& P, int b, long long cell, int slice)
{
    const float sv = P.scat[b * P.scat_stride + P.scat_cell[cell] + P.scat_ring[slice]];
    return P.scat_clamp ? fmaxf(sv, 0.f) : sv;
}

// The fit's images, device float [nbins + 1][4 nvox].  Per voxel and bin:
// D, the sum over the LORs through the voxel of (prompts - randoms) / voxels,
// S, that of scatter / voxels, and the sensitivity, their count
// (BackProjection.py:99-110).  The reference keeps prompts and randoms apart
// and subtracts them after dividing by the sensitivity (:191-204); D is that
// difference summed once, so that it costs no atomic of its own.
//   bins 2q, 2q+1: block 2q float4 (D, S, D, S); block 2q+1 float4
//     (0, sens, 0, sens) of the LORs that use some of the bins only;
//   an odd last bin L: block L float4 (D, S, 0, common sens), the common
//     sensitivity counting the LORs every bin uses (one atomic with L's
//     values); block nbins float2 [0, nvox) (0, sens) of the LORs that use
//     some bins only;
//   even bin counts: the common sensitivity in block nbins, float2
//     [nvox, 2 nvox), (0, sens).
struct FitImages {
    float* img;
    long long nv;
    int nbins;
    __device__ float4* pair_ds(int b0) const { return reinterpret_cast<float4*>(img + (long long)b0 * 4 * nv); }
    __device__ float4* pair_sens(int b0) const
    {
        return reinterpret_cast<float4*>(img + (long long)(b0 + 1) * 4 * nv);
    }
    __device__ float4* last_ds(int lastb) const { return reinterpret_cast<float4*>(img + (long long)lastb * 4 * nv); }
    __device__ float2* last_sens() const { return reinterpret_cast<float2*>(img + (long long)nbins * 4 * nv); }
    __device__ float2* common_sens() const { return last_sens() + nv; }
};

// A 16-byte shared-memory load issued where it stands: the per-LOR values
// are re-read at every voxel instead of being held in registers across the
// walk, which keeps the kernel's register count (and so its occupancy) at that
// of the walk alone.
__device__ __forceinline__ float4 lds_v4(const float4* p)
{
    float4 v;
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
    return v;
}

constexpr int kBpThreads = 128;  // threads of a bp_kernel block

// One thread per lattice LOR; lattice order keeps a warp on one crystal pair
// over neighbouring ring pairs (similar voxel paths, similar walk lengths).
// NPB > 0: the plain (not length-weighted) back-projection of at most
// 2 NPB + 1 bins, whose per-voxel values are the same along the whole LOR
// (value / voxel count, :108-110): they are formed once per LOR and kept in
// the thread's own shared-memory column, and each voxel issues only its
// vector atomics.  With those values out of the registers the walk sets the
// register count; six blocks a multiprocessor (80 registers) hold it without
// spilling but the odd word.  NPB = 0: the general form, which forms the
// values per voxel (the length-weighted span fit, :294-297, and more than 17
// bins), with its own register count.
template <int NPB>
__global__ void __launch_bounds__(kBpThreads, NPB > 0 ? 6 : 0) bp_kernel(FitParams P)
{
    const long long n = (long long)(P.pairs ? P.npairs : P.nr * P.nr) * P.na * P.na;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const LorRef L = lor_ref(id, P.nr, P.na, P.order, P.pairs, P.npairs);
    const int d1 = L.i1 * P.af, d2 = L.i2 * P.af;
    if ((d1 == d2 && L.r1 == L.r2) || d1 > d2) return;  // BackProjection.py:88, :278
    const int ang = P.lor[2 * ((long long)d1 * P.nd + d2)];
    const int rad = P.lor[2 * ((long long)d1 * P.nd + d2) + 1];
    const int slice = L.slice;
    if (rad < 0 || rad > P.nd || ang < 0 || ang >= P.nd / 2 || !lor_ref_ok(L, P.nr, P.nslices)) {
        raise_error(P.status, kErrTable);  // the caller's LOR, slice-order or ring-pair table
        return;
    }
    const long long cell = (long long)rad * (P.nd / 2) + ang;
    const long long c = cell * (long long)P.nslices + slice;
    const float m = P.mask_u8 ? (P.mask_u8[c] >= 1 ? 1.f : 0.f) : P.mask_f32[c];
    // bins whose masked scatter is non-zero back-project this LOR (:99-100)
    unsigned long long bins = 0;
    for (int b = 0; b < P.nbins; ++b)
        if (m * fit_scatter(P, b, cell, slice) != 0.f) bins |= 1ull << b;
    if (!bins) return;
    const unsigned long long all = P.nbins == 64 ? ~0ull : (1ull << P.nbins) - 1;
    const float rv = m * P.randoms[c];
    const float s0 = m * fit_scatter(P, 0, cell, slice), p0 = m * P.prompts[c];
    double lc[6];
    lor_line(P.geom, P.nd, L.r1, d1, L.r2, d2, lc);
    Ray r;
    if (!ray_setup(P.g, lc, 1e-20, r)) return;
    // Voxel count (the reference divides by len(Lengths), :108-110).  Every
    // step of the walk moves one voxel along one axis towards the end voxel,
    // so a walk that ends crosses 1 + |dX| + |dY| + |dZ| voxels; one that would
    // overrun is caught by the walk below.  The length-weighted back-projection
    // needs the summed length first (:294-297), so it walks twice.
    double total = 0.0;
    int n_vox = 1 + abs(r.xe - r.X) + abs(r.ye - r.Y) + abs(r.ze - r.Z);
    if (P.length_weighted) {
        Ray r2 = r;
        n_vox = ray_walk(P.g, r2, P.cap, [&](int, int64_t, double t0, double t1) {
            total = add64(total, ref_length(r2, t0, t1));
        });
    }
    if (n_vox < 0 || n_vox > P.cap) {
        raise_error(P.status, kErrOverrun);
        return;
    }
    const float fn = (float)n_vox;
    const float ar = rv / fn;
    bool bad = false;
    if constexpr (NPB > 0) {
        // (D, S) of bin b from this LOR: prompts minus randoms, and scatter,
        // each divided by the voxel count, as below
        auto contrib = [&](int b) {
            const float s = P.nbins == 1 ? s0 : m * fit_scatter(P, b, cell, slice);
            const float pv = P.nbins == 1 ? p0 : m * P.prompts[b * P.prompt_stride + c];
            return make_float2(pv / fn - ar, s / fn);
        };
        const int paired = P.nbins & ~1;
        // this thread's (D, S, D, S) of each bin pair, in its own shared-memory column
        __shared__ float4 s_cps[NPB][kBpThreads];
        unsigned pm = 0;  // bin pairs with a bin this LOR contributes to
#pragma unroll
        for (int k = 0; k < NPB; ++k) {
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (2 * k < paired) {
                const bool in0 = (bins >> (2 * k)) & 1ull, in1 = (bins >> (2 * k + 1)) & 1ull;
                const float2 c0 = in0 ? contrib(2 * k) : make_float2(0.f, 0.f);
                const float2 c1 = in1 ? contrib(2 * k + 1) : make_float2(0.f, 0.f);
                v = make_float4(c0.x, c0.y, c1.x, c1.y);
                if (in0 || in1) pm |= 1u << k;
            }
            s_cps[k][threadIdx.x] = v;
        }
        const int lastb = P.nbins - 1;
        const bool odd = P.nbins & 1;
        const bool has_last = odd && ((bins >> lastb) & 1ull);
        const bool every = bins == all;
        // the odd last bin's (D, S) with, for LORs every bin uses, one count of
        // the common sensitivity: one vector atomic
        const float2 cl = has_last ? contrib(lastb) : make_float2(0.f, 0.f);
        const float4 clast = make_float4(cl.x, cl.y, 0.f, every ? 1.f : 0.f);
        const FitImages I{P.img, P.nvox, P.nbins};
        const int walked = ray_walk(P.g, r, P.cap, [&](int, int64_t lin, double, double) {
            const long long v = lin - 1;
            if (v < 0 || v >= P.nvox) {
                bad = true;
                return;
            }
#pragma unroll
            for (int k = 0; k < NPB; ++k) {
                if ((pm >> k) & 1u) {
                    atomicAdd(I.pair_ds(2 * k) + v, lds_v4(&s_cps[k][threadIdx.x]));
                    if (!every) {  // sensitivity of these bins alone
                        const bool in0 = (bins >> (2 * k)) & 1ull, in1 = (bins >> (2 * k + 1)) & 1ull;
                        atomicAdd(I.pair_sens(2 * k) + v, make_float4(0.f, in0 ? 1.f : 0.f, 0.f, in1 ? 1.f : 0.f));
                    }
                }
            }
            if (has_last) {
                atomicAdd(I.last_ds(lastb) + v, clast);
                if (!every) atomicAdd(I.last_sens() + v, make_float2(0.f, 1.0f));
            }
            if (every && !odd) atomicAdd(I.common_sens() + v, make_float2(0.f, 1.0f));  // shared by every bin
        });
        if (bad) raise_error(P.status, kErrVoxel);
        if (walked != n_vox) raise_error(P.status, kErrOverrun);
        return;
    }
    const int walked = ray_walk(P.g, r, P.cap, [&](int, int64_t lin, double t0, double t1) {
        const long long v = lin - 1;
        if (v < 0 || v >= P.nvox) {
            bad = true;
            return;
        }
        const double w = P.length_weighted ? div64(ref_length(r, t0, t1), total) : 0.0;
        const float rw = P.length_weighted ? (float)mul64((double)rv, w) : ar;
        // (D, S) of bin b from this LOR: prompts minus randoms, and scatter
        // (one bin: the LOR's values, else re-read per voxel, L1-resident)
        auto contrib = [&](int b) {
            const float s = P.nbins == 1 ? s0 : m * fit_scatter(P, b, cell, slice);
            const float pv = P.nbins == 1 ? p0 : m * P.prompts[b * P.prompt_stride + c];
            return P.length_weighted
                       ? make_float2((float)mul64((double)pv, w) - rw, (float)mul64((double)s, w))
                       : make_float2(pv / fn - rw, s / fn);
        };
        // Bins 2q and 2q+1 share float4 images, (D, S, D, S) then (0, sens, 0,
        // sens): one vector atomic each for the pair; an odd last bin has
        // (D, S, 0, common sens) and a float2 (0, sens) (FitImages).
        const FitImages I{P.img, P.nvox, P.nbins};
        const bool every = bins == all, odd = P.nbins & 1;
        const int paired = P.nbins & ~1;
        for (unsigned long long rest = bins; rest;) {
            const int b = __ffsll((long long)rest) - 1;
            if (b < paired) {
                const int b0 = b & ~1;
                const bool in0 = (bins >> b0) & 1ull, in1 = (bins >> (b0 + 1)) & 1ull;
                rest &= ~(3ull << b0);
                const float2 c0 = in0 ? contrib(b0) : make_float2(0.f, 0.f);
                const float2 c1 = in1 ? contrib(b0 + 1) : make_float2(0.f, 0.f);
                atomicAdd(I.pair_ds(b0) + v, make_float4(c0.x, c0.y, c1.x, c1.y));
                if (!every)  // sensitivity of these bins alone
                    atomicAdd(I.pair_sens(b0) + v, make_float4(0.f, in0 ? 1.f : 0.f, 0.f, in1 ? 1.f : 0.f));
            } else {
                rest &= rest - 1;
                const float2 cb = contrib(b);
                atomicAdd(I.last_ds(b) + v, make_float4(cb.x, cb.y, 0.f, every ? 1.f : 0.f));
                if (!every) atomicAdd(I.last_sens() + v, make_float2(0.f, 1.0f));
            }
        }
        if (every && !odd) atomicAdd(I.common_sens() + v, make_float2(0.f, 1.0f));  // shared by every bin
    });
    if (bad) raise_error(P.status, kErrVoxel);
    if (walked != n_vox) raise_error(P.status, kErrOverrun);
}

// per voxel: Sbp, T (BackProjection.py:191-204); sums of x*T and x*x in FP64;
// blockIdx.y = bin (images as FitImages lays them out, sums [bin][2]).  T is
// D / sens, the reference's ActivityImage / sens - RandomImage / sens.
__global__ void fit_reduce_kernel(const float* __restrict__ img_all, long long nvox, int nbins,
                                  double* sums_all)
{
    const int b = blockIdx.y;
    const FitImages I{const_cast<float*>(img_all), nvox, nbins};
    const bool odd = nbins & 1, pair = b < (nbins & ~1);  // float4 images shared with the neighbouring bin
    double* sums = sums_all + 2 * blockIdx.y;
    double sxt = 0.0, sxx = 0.0;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nvox;
         v += (long long)gridDim.x * blockDim.x) {
        float2 ds;
        float own;
        if (pair) {
            const float4 p4 = I.pair_ds(b & ~1)[v], s4 = I.pair_sens(b & ~1)[v];
            ds = (b & 1) ? make_float2(p4.z, p4.w) : make_float2(p4.x, p4.y);
            own = (b & 1) ? s4.w : s4.y;
        } else {
            const float4 l4 = I.last_ds(b)[v];
            ds = make_float2(l4.x, l4.y);
            own = I.last_sens()[v].y;
        }
        const float sens = own + (odd ? I.last_ds(nbins - 1)[v].w : I.common_sens()[v].y);
        float sb = ds.y / sens;
        float t = ds.x / sens;
        if (isnan(sb) || isinf(sb)) sb = 0.f;
        if (isnan(t) || isinf(t)) t = 0.f;
        if (t < 0.f) t = 0.f;
        const float x = (float)((double)sb * 1e10);  // float32 array * 1e10 (:207)
        sxt += (double)x * (double)t;
        sxx += (double)x * (double)x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sxt += __shfl_xor_sync(0xffffffffu, sxt, o);
        sxx += __shfl_xor_sync(0xffffffffu, sxx, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sums, sxt);
        atomicAdd(sums + 1, sxx);
    }
}

// lstsq of one column through the origin (:207-210): minimum-norm solution
// sum(xT)/sum(x^2) (0 when x is all zero), cast to float32, times 1e10.
__global__ void fit_final_kernel(const double* sums, float* scale, int nbins)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbins) return;
    const double a = sums[2 * b + 1] > 0.0 ? sums[2 * b] / sums[2 * b + 1] : 0.0;
    scale[b] = (float)((double)(float)a * 1e10);
}

int check_grid(const int32_t* grid, const double* bounds, const char* who)
{
    if (!grid || !bounds) return sss_set_error(SSS_ERR_INVALID, "%s: null grid", who);
    if (grid[0] < 1 || grid[1] < 1 || grid[2] < 1)
        return sss_set_error(SSS_ERR_INVALID, "%s: grid must be positive", who);
    if (!(bounds[3] > bounds[0] && bounds[4] > bounds[1] && bounds[5] > bounds[2]))
        return sss_set_error(SSS_ERR_INVALID, "%s: bounds must satisfy max > min", who);
    return SSS_OK;
}

Grid make_grid(const int32_t* grid, const double* bounds) { return grid_of(grid[0], grid[1], grid[2], bounds); }

unsigned blocks_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

extern "C" int sss_upsample(const float* sampled, int64_t bin_stride, int32_t nbins, const int64_t* cell_src,
                            int64_t ncell, const int64_t* ring_off, int32_t nring, const int32_t* ring_idx,
                            int32_t nslices, float* out, void* stream)
{
    if (!sampled || !cell_src || !ring_off || !ring_idx || !out || nbins < 1 || ncell < 1 || nslices < 1 ||
        nring < 1 || nring > 16384)
        return sss_set_error(SSS_ERR_INVALID, "sss_upsample: bad argument");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long cap = (long long)sms * 8;
    const unsigned blocks = (unsigned)(ncell < cap ? ncell : cap);
    const size_t smem = sizeof(float) * (size_t)nring;
    // more than 12288 ring pairs (over 110 sampled rings) need the opt-in past 48 KB
    if (smem > 48 * 1024 && cudaFuncSetAttribute((const void*)upsample_kernel,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_upsample: %zu bytes of shared memory refused", smem);
    upsample_kernel<<<blocks, 256, smem, (cudaStream_t)stream>>>(
        sampled, bin_stride, nbins, (const long long*)cell_src, ncell, (const long long*)ring_off, nring,
        ring_idx, nslices, out);
    return sss_check_launch("upsample_kernel");
}

namespace {

int tail_mask(const int32_t grid[3], const double bounds[6], const float* map, int32_t use_activity, int32_t nr,
              int32_t nd, const double* geometry, const int16_t* lor, const int16_t* sino_index,
              const int32_t* pairs, int32_t npairs, int32_t nslices, int32_t af, double acf_below, uint8_t* out,
              int32_t* status, void* stream)
{
    if (!(acf_below == 0.0 || acf_below > 1.0))
        return sss_set_error(SSS_ERR_INVALID, "sss_tail_mask: acf_below must be 0 (ACF == 1) or above 1");
    MaskParams P;
    P.acf_below = acf_below;
    // the factor 1/exp(-s) passes acf_below once s > log(acf_below), with a
    // margin far above FP64 rounding
    P.decided = acf_below > 0.0 ? log(acf_below) * (1.0 + 1e-9) + 1e-12 : kDecided;
    P.pairs = pairs;
    P.npairs = npairs;
    P.nslices = pairs ? nslices : nr * nr;
    P.g = make_grid(grid, bounds);
    P.mu = map;
    P.use_activity = use_activity;
    P.nvox = (long long)grid[0] * grid[1] * grid[2];
    P.geom = geometry;
    P.lor = lor;
    P.sino = sino_index;
    P.nr = nr;
    P.nd = nd;
    P.af = af;
    P.na = (nd + af - 1) / af;
    P.cap = grid[0] + grid[1] + grid[2];
    P.out = out;
    P.status = status;
    const long long n = (long long)(pairs ? npairs : nr * nr) * P.na * P.na;
    if (n == 0) return SSS_OK;
    if (!status) return sss_set_error(SSS_ERR_INVALID, "sss_tail_mask: status word required");
    const long long nb = (P.nvox + 255) / 256;
    map_sign_kernel<<<(unsigned)(nb < 1024 ? nb : 1024), 256, 0, (cudaStream_t)stream>>>(map, P.nvox, status);
    int rc = sss_check_launch("map_sign_kernel");
    if (rc) return rc;
    mask_kernel<<<blocks_for(n, 128), 128, 0, (cudaStream_t)stream>>>(P);
    return sss_check_launch("mask_kernel");
}

}  // namespace

extern "C" int sss_tail_mask(const int32_t grid[3], const double bounds[6], const float* map,
                             int32_t use_activity, int32_t nr, int32_t nd, const double* geometry,
                             const int16_t* lor, const int16_t* sino_index, int32_t af, double acf_below,
                             uint8_t* out, int32_t* status, void* stream)
{
    int rc = check_grid(grid, bounds, "sss_tail_mask");
    if (rc) return rc;
    if (!map || !geometry || !lor || !sino_index || !out || nr < 1 || nd < 2 || af < 1)
        return sss_set_error(SSS_ERR_INVALID, "sss_tail_mask: bad argument");
    return tail_mask(grid, bounds, map, use_activity, nr, nd, geometry, lor, sino_index, nullptr, 0, 0, af,
                     acf_below, out, status, stream);
}

extern "C" int sss_tail_mask_pairs(const int32_t grid[3], const double bounds[6], const float* map,
                                   int32_t use_activity, int32_t nr, int32_t nd, const double* geometry,
                                   const int16_t* lor, const int32_t* pairs, int32_t npairs, int32_t nslices,
                                   int32_t af, double acf_below, uint8_t* out, int32_t* status, void* stream)
{
    int rc = check_grid(grid, bounds, "sss_tail_mask_pairs");
    if (rc) return rc;
    if (!map || !geometry || !lor || !pairs || !out || nr < 1 || nd < 2 || af < 1 || npairs < 0 || nslices < 1)
        return sss_set_error(SSS_ERR_INVALID, "sss_tail_mask_pairs: bad argument");
    return tail_mask(grid, bounds, map, use_activity, nr, nd, geometry, lor, nullptr, pairs, npairs, nslices, af,
                     acf_below, out, status, stream);
}

namespace {

int backproject_fit(const int32_t grid[3], const double bounds[6], int32_t nr, int32_t nd, const double* geometry,
                    const int16_t* lor, const int16_t* sino_order, const int32_t* pairs, int32_t npairs,
                    int32_t nslices, int32_t length_weighted, int32_t af, int32_t nbins, const float* prompts,
                    int64_t prompt_stride, const float* randoms, const float* mask_f32, const uint8_t* mask_u8,
                    const float* scatters, int64_t scat_stride, const int64_t* scat_cell,
                    const int64_t* scat_ring, int32_t scat_clamp, float* images, double* sums, float* scale,
                    int32_t* status, void* stream)
{
    int rc;
    if (!geometry || !lor || !prompts || !randoms || (!mask_f32 && !mask_u8) || !scatters || !scat_cell ||
        !scat_ring || !images || !sums || !scale || nr < 1 || nd < 2 || af < 1 || nbins < 1 || nbins > 64)
        return sss_set_error(SSS_ERR_INVALID, "sss_backproject_fit: bad argument");
    if ((uintptr_t)images % 16 != 0)  // vector atomics on float4 / float2 image entries
        return sss_set_error(SSS_ERR_INVALID, "sss_backproject_fit: images must be 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    FitParams P;
    P.pairs = pairs;
    P.npairs = npairs;
    P.nslices = pairs ? nslices : nr * nr;
    P.length_weighted = length_weighted;
    P.nbins = nbins;
    P.prompt_stride = prompt_stride;
    P.scat_stride = scat_stride;
    P.g = make_grid(grid, bounds);
    P.nvox = (long long)grid[0] * grid[1] * grid[2];
    P.geom = geometry;
    P.lor = lor;
    P.order = sino_order;
    P.nr = nr;
    P.nd = nd;
    P.af = af;
    P.na = (nd + af - 1) / af;
    P.cap = grid[0] + grid[1] + grid[2];
    P.prompts = prompts;
    P.randoms = randoms;
    P.mask_f32 = mask_u8 ? nullptr : mask_f32;
    P.mask_u8 = mask_u8;
    P.scat = scatters;
    P.scat_cell = (const long long*)scat_cell;
    P.scat_ring = (const long long*)scat_ring;
    P.scat_clamp = scat_clamp;
    P.img = images;
    P.status = status;
    if (cudaMemsetAsync(images, 0, sizeof(float) * 4 * P.nvox * (nbins + 1), st) != cudaSuccess ||
        cudaMemsetAsync(sums, 0, 2 * sizeof(double) * nbins, st) != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "sss_backproject_fit: memset failed");
    const long long n = (long long)(pairs ? npairs : nr * nr) * P.na * P.na;
    if (n > 0) {
        const unsigned nb = blocks_for(n, kBpThreads);
        if (length_weighted || nbins > 17)
            bp_kernel<0><<<nb, kBpThreads, 0, st>>>(P);
        else if (nbins <= 3)
            bp_kernel<1><<<nb, kBpThreads, 0, st>>>(P);
        else if (nbins <= 5)
            bp_kernel<2><<<nb, kBpThreads, 0, st>>>(P);
        else if (nbins <= 9)
            bp_kernel<4><<<nb, kBpThreads, 0, st>>>(P);
        else if (nbins <= 13)
            bp_kernel<6><<<nb, kBpThreads, 0, st>>>(P);
        else
            bp_kernel<8><<<nb, kBpThreads, 0, st>>>(P);
        if ((rc = sss_check_launch("bp_kernel"))) return rc;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (P.nvox + 255) / 256;
    const dim3 rgrid((unsigned)(want < sms * 4 ? want : sms * 4), (unsigned)nbins);
    fit_reduce_kernel<<<rgrid, 256, 0, st>>>(images, P.nvox, nbins, sums);
    if ((rc = sss_check_launch("fit_reduce_kernel"))) return rc;
    fit_final_kernel<<<1, 64, 0, st>>>(sums, scale, nbins);
    return sss_check_launch("fit_final_kernel");
}

}  // namespace

extern "C" int sss_backproject_fit(const int32_t grid[3], const double bounds[6], int32_t nr,
                                   int32_t nd, const double* geometry, const int16_t* lor,
                                   const int16_t* sino_order, int32_t af, const float* prompts,
                                   const float* randoms, const float* mask_f32,
                                   const uint8_t* mask_u8, const float* scatters,
                                   const int64_t* scat_cell, const int64_t* scat_ring,
                                   int32_t scat_clamp, float* images, double* sums, float* scale,
                                   int32_t* status, void* stream)
{
    int rc = check_grid(grid, bounds, "sss_backproject_fit");
    if (rc) return rc;
    if (!sino_order) return sss_set_error(SSS_ERR_INVALID, "sss_backproject_fit: bad argument");
    return backproject_fit(grid, bounds, nr, nd, geometry, lor, sino_order, nullptr, 0, 0, 0, af, 1, prompts, 0,
                           randoms, mask_f32, mask_u8, scatters, 0, scat_cell, scat_ring, scat_clamp, images, sums,
                           scale, status, stream);
}

extern "C" int sss_backproject_fit_pairs(const int32_t grid[3], const double bounds[6], int32_t nr, int32_t nd,
                                         const double* geometry, const int16_t* lor, const int32_t* pairs,
                                         int32_t npairs, int32_t nslices, int32_t length_weighted, int32_t af,
                                         const float* prompts, const float* randoms, const float* mask_f32,
                                         const uint8_t* mask_u8, const float* scatters, const int64_t* scat_cell,
                                         const int64_t* scat_ring, int32_t scat_clamp, float* images,
                                         double* sums, float* scale, int32_t* status, void* stream)
{
    int rc = check_grid(grid, bounds, "sss_backproject_fit_pairs");
    if (rc) return rc;
    if (!pairs || npairs < 0 || nslices < 1)
        return sss_set_error(SSS_ERR_INVALID, "sss_backproject_fit_pairs: bad argument");
    return backproject_fit(grid, bounds, nr, nd, geometry, lor, nullptr, pairs, npairs, nslices, length_weighted,
                           af, 1, prompts, 0, randoms, mask_f32, mask_u8, scatters, 0, scat_cell, scat_ring,
                           scat_clamp, images, sums, scale, status, stream);
}

extern "C" int sss_backproject_fit_bins(const int32_t grid[3], const double bounds[6], int32_t nr, int32_t nd,
                                        const double* geometry, const int16_t* lor, const int16_t* sino_order,
                                        const int32_t* pairs, int32_t npairs, int32_t nslices,
                                        int32_t length_weighted, int32_t af, int32_t nbins, const float* prompts,
                                        int64_t prompt_stride, const float* randoms, const float* mask_f32,
                                        const uint8_t* mask_u8, const float* scatters, int64_t scat_stride,
                                        const int64_t* scat_cell, const int64_t* scat_ring, int32_t scat_clamp,
                                        float* images, double* sums, float* scales, int32_t* status,
                                        void* stream)
{
    int rc = check_grid(grid, bounds, "sss_backproject_fit_bins");
    if (rc) return rc;
    if ((!sino_order && !pairs) || (pairs && (npairs < 0 || nslices < 1)))
        return sss_set_error(SSS_ERR_INVALID, "sss_backproject_fit_bins: bad argument");
    return backproject_fit(grid, bounds, nr, nd, geometry, lor, pairs ? nullptr : sino_order, pairs,
                           pairs ? npairs : 0, pairs ? nslices : 0, length_weighted, af, nbins, prompts,
                           prompt_stride, randoms, mask_f32, mask_u8, scatters, scat_stride, scat_cell, scat_ring,
                           scat_clamp, images, sums, scales, status, stream);
}
