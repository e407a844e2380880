// The TOF-SSS pair stage: one warp task = (z-slice of one problem, walking
// leg lw, 32 partner legs).  Shared by the single-problem kernel (sss.cu)
// and the batched kernels (batch.cu).  Reference: bodySSS,
// Python/openSSS/SingleScatterSimulationTOF.py:433-557.
#pragma once

#include "common.cuh"
#include "trace.cuh"

namespace sss {

constexpr double kLightCmPerPs = 299792458.0 * 1e-10;  // :144
constexpr int kPairWarps = 12;  // most warps of a pair-kernel block
constexpr int kKahanWarps = 8;  // warps of a Kahan-compensated pair block

// Warps of a pair block of np bin pairs: 12 up to 8 pairs (two blocks a
// multiprocessor, 80 registers a thread); 8 above, where the accumulators want
// 128 registers (two blocks); kKahanWarps for Kahan-compensated launches (one
// block, the partial sums in shared memory).
__host__ __device__ constexpr int pair_block_warps(int np, bool kahan)
{
    return kahan ? kKahanWarps : (np <= 8 ? kPairWarps : 8);
}
// Gaussian factors 2^(-gamma (n-b)^2) of the factored weights: [n][b], rows of
// kGRow floats (at most 64 bins plus 4 of padding, so that lanes reading the
// same bins of different rows fall in different shared-memory banks)
constexpr int kGRow = 68;

// Shared memory of a pair block, in this order:
//   ar    float2 [8001]  (A, r) of each TOF offset (factored weights; A carries
//         the nearest bin n in its low mantissa bits) or (Y, 0), then one
//         entry (0, 0) at kZeroEntry (factored weights of exactly 0)
//   n     u8     [8001]  bin of the column's largest weight
//   vbuf  float2 [warps][32]  staged voxels of each warp's walk; a
//         Kahan-compensated launch (kKahanWarps warps) keeps the low floats of
//         its staged samples after them, float [kKahanWarps][32]
//   g     float  [nbins][kGRow]
//   kahan float2 [2 NP][32 kKahanWarps]  (Kahan-compensated launches only,
//         which run kKahanWarps warps so that 64 bins still fit)
constexpr int kZeroEntry = kTofEntries;  // the (0, 0) entry after the table
constexpr int kSmemNOff = (8 * (kZeroEntry + 1) + 15) & ~15;
constexpr int kSmemVbufOff = (kSmemNOff + kTofEntries + 15) & ~15;
constexpr int kSmemGOff = kSmemVbufOff + 8 * 32 * kPairWarps;
constexpr int kSmemVloOff = kSmemVbufOff + 8 * 32 * kKahanWarps;  // Kahan launches only
static_assert(kSmemGOff % 16 == 0, "shared-memory sections must be 16-byte aligned");
static_assert(kSmemVloOff + 4 * 32 * kKahanWarps <= kSmemGOff, "the low floats must fit in the vbuf section");

__host__ __device__ inline int pair_smem_kahan_off(int nbins) { return kSmemGOff + 4 * kGRow * nbins; }

// Dynamic shared memory of a pair launch; kahan_np = bin pairs of a
// Kahan-compensated launch, 0 otherwise.
inline size_t pair_smem_bytes(int nbins, int kahan_np = 0)
{
    return (size_t)pair_smem_kahan_off(nbins) + sizeof(float2) * 2 * kahan_np * 32 * kKahanWarps;
}

// TOF constants of one launch (every task of a launch shares one TOF table)
struct TofConst {
    float s0, w;           // first bin centre offset and bin width (ps)
    float kappa2w, gamma;  // 2 kappa w and kappa w^2, kappa = 4/FWHM^2 (log2 units)
    int factored;          // weights as 2^(Y - n beta) r^b G[n][b] (see accumulate_voxel)
    int tsafe;             // table entries below this index use the factored weights; entries
                           // from it on (offsets far past the last bin) hold (Y, 0) and take
                           // the per-bin 2^x evaluation (see far_voxel)
    int nbins;
    int nmask;             // low mantissa bits of the tabled A that carry the nearest bin n
};

// Everything one task needs about its problem and z-slice.
struct PairCtx {
    int nru, ndu, nl, nd, cap, nbins;
    float geo_c;             // (ds0*ds1*1e-2)^2 / (4 pi)
    float gamma_kn;          // E/(m_e c^2) of the reference's KleinNishina
    const float* eff;        // [2000]
    const float* ratio;      // [2000]
    const double* geom;      // [nr][nd][3]
    const int32_t* rings;
    const int32_t* dets;
    const double* points;    // scatter points the leg arrays are indexed by
    const float4* legA;      // [point][nl]
    const float4* legB;
    const float4* legC;      // low floats of legB's unit vectors, and of legA's distance
    const float2* vox;       // [point][nl][cap]
    const float* vox_lo;     // [point][nl][cap] low floats of the samples (Kahan launches), else null
    float* out;              // [nbins][nl][nl]
    int unit_tof;            // one bin, every TOF weight exactly 1: AB = the leg's activity integral
};

// Launch constants of a problem's TOF table (:98, :282) and Watson factors.
inline TofConst tof_const(const sss_tof_problem& p)
{
    const double w = p.tof_bin_width;
    const double kappa = 4.0 / (p.tof_resolution * p.tof_resolution);
    TofConst T;
    T.s0 = (float)((1.0 - (p.nbins + 1) / 2.0) * w);
    T.w = (float)w;
    T.kappa2w = (float)(2.0 * kappa * w);
    T.gamma = (float)(kappa * w * w);
    // The factored form multiplies powers of 2^beta: every product stays below
    // 2^127 when gamma (B-1) < 100 (in-span offsets, |beta| <= gamma) and
    // w / FWHM < 1.33 (offsets whose column is still above 2^-126 have
    // beta < 45 w / FWHM, so r^2 = 2^(2 beta) < 2^120).
    T.factored = p.nbins > 1 && (kappa * w * w) * (p.nbins - 1) < 100.0 && w / p.tof_resolution < 1.33;
    // Past the last bin centre s_{B-1} the nearest bin is B-1 and the chain
    // starts at ca 2^(Y - (B-1) beta), beta = 2 kappa w (t - s_{B-1}).  Up to
    // (B-1) beta = 62 that start stays a normal float for voxel terms ca down
    // to 2^-64 and r^2 = 2^(2 beta) stays below 2^124; offsets beyond take the
    // per-bin path.  Offsets below -4000 ps wrap into the table's top (numpy's
    // negative index), so the far entries are one suffix of the table.
    T.tsafe = kTofEntries;
    if (T.factored) {
        const double s_last = (1.0 - (p.nbins + 1) / 2.0) * w + (p.nbins - 1) * w;
        const double t_safe = s_last + 62.0 / ((p.nbins - 1) * 2.0 * kappa * w);
        const double idx = floor(t_safe) + kTimeRange + 1;  // first entry whose offset passes t_safe
        T.tsafe = idx >= kTofEntries ? kTofEntries : (int)idx;
    }
    T.nbins = p.nbins;
    int bits = 1;
    while ((1 << bits) < p.nbins) ++bits;
    T.nmask = (1 << bits) - 1;
    return T;
}
inline float geo_const(const sss_tof_problem& p)
{
    const double ds = p.detector_size[0] * p.detector_size[1] * 1e-2;
    return (float)(ds * ds / (4.0 * 3.141592653589793));
}
inline float gamma_kn_const()
{
    return (float)(511.0E3 * 1.6E-19 / (9.10938356E-31 * (299792458.0 * 299792458.0)));
}

// 32-partner chunks per walking leg: nl legs plus nru same-crystal entries
__host__ __device__ inline int pair_chunks(int nru, int ndu) { return (nru * ndu + nru + 31) / 32; }

// A with the bin n in its low mantissa bits: the representable value nearest
// to a whose bits & mask equal n (a >= 0; a == 0 stays 0, all weights zero).
__device__ __forceinline__ float pack_bin(float a, int n, int mask)
{
    const int ai = __float_as_int(a);
    if (ai == 0) return 0.f;
    int p = ai - ((ai - n) & mask);
    if (ai - p > (mask + 1) / 2 || p < 0) p += mask + 1;
    return __int_as_float(p);
}

// Block-wide set-up of the shared tables.  From the (log2 largest weight Y,
// bin n) table: for the factored weights, per TOF offset t below T.tsafe,
// beta(t) = 2 kappa w (t - 4000 - s_n) rounded to float once, r = 2^beta and
// A = 2^(Y - n beta) with the same beta (so that A r^n = 2^Y up to rounding),
// A rounded to the nearest value whose low bits hold n (relative change below
// 2^-(24 - bits), bits = ceil(log2 nbins)); otherwise (Y, 0).
// G[n][b] = 2^(-gamma (n - b)^2), 0 past the last bin and in the padding.
__device__ __forceinline__ void load_pair_tables(const float* g, const TofConst& T, float2* sAR,
                                                 unsigned char* sN, float* sG)
{
    for (int i = threadIdx.x; i < kTofEntries; i += blockDim.x) {
        const float Y = g[2 * i];
        const float n = g[2 * i + 1];
        sN[i] = (unsigned char)n;
        if (T.factored && i < T.tsafe) {
            const float off = (float)(i - kTimeRange);
            const float beta = T.kappa2w * (off - fmaf(n, T.w, T.s0));  // as the per-voxel form rounds it
            const double e = (double)Y - (double)n * (double)beta;     // -inf stays -inf
            float a = 0.f;
            if (e > -1000.0) {
                const double k = floor(e);
                a = ldexpf(exp2f((float)(e - k)), (int)k);
            }
            sAR[i] = make_float2(pack_bin(a, (int)n, T.nmask), exp2f(beta));
        } else {
            sAR[i] = make_float2(Y, 0.f);
        }
    }
    if (threadIdx.x == 0) sAR[kZeroEntry] = make_float2(0.f, 0.f);
    if (T.factored)
        for (int i = threadIdx.x; i < T.nbins * kGRow; i += blockDim.x) {
            const int n = i / kGRow, b = i % kGRow;
            const float d = (float)(n - b);
            sG[i] = b < T.nbins ? exp2f(-T.gamma * d * d) : 0.f;
        }
}

// Energy row of a pair in FP64, used when the FP32 estimate lies within 1e-3
// keV of a rounding boundary.  The law-of-cosines argument q is formed with the
// reference's FP64 operations (:442-444, :474-475, :216-235).  The reference
// then takes theta = 180 - degrees(acos(q)) and cos(deg2rad(theta)) (:498-499),
// which is -q up to that round trip's own rounding (~1e-16); -q is used
// directly, so the row can differ from the reference's only where 511/(2 + q)
// + 0.5 lies within ~1e-13 of an integer.  Symmetric in the two legs.
static __device__ __noinline__ int energy_row_fp64(const PairCtx& C, int s, int ri1, int di1, int ri2,
                                            int di2)
{
    const double xS = C.points[4 * s], yS = C.points[4 * s + 1], zS = C.points[4 * s + 2];
    const int r1 = C.rings[ri1], r2 = C.rings[ri2], d1 = C.dets[di1], d2 = C.dets[di2];
    const double* p1 = C.geom + 3 * ((long long)r1 * C.nd + d1);
    const double* p2 = C.geom + 3 * ((long long)r2 * C.nd + d2);
    const double z1 = C.geom[3 * ((long long)r1 * C.nd) + 2];
    const double z2 = C.geom[3 * ((long long)r2 * C.nd) + 2];
    double sv1 = __dsqrt_rn(add64(add64(mul64(sub64(p1[0], xS), sub64(p1[0], xS)),
                                        mul64(sub64(p1[1], yS), sub64(p1[1], yS))),
                                  mul64(sub64(z1, zS), sub64(z1, zS))));
    double sv2 = __dsqrt_rn(add64(add64(mul64(sub64(p2[0], xS), sub64(p2[0], xS)),
                                        mul64(sub64(p2[1], yS), sub64(p2[1], yS))),
                                  mul64(sub64(z2, zS), sub64(z2, zS))));
    double lor = add64(add64(mul64(sub64(p1[0], p2[0]), sub64(p1[0], p2[0])),
                             mul64(sub64(p1[1], p2[1]), sub64(p1[1], p2[1]))),
                       mul64(sub64(z1, z2), sub64(z1, z2)));
    double a = mul64(sv1, sv1), b = mul64(sv2, sv2);
    double q = div64(sub64(add64(a, b), lor), mul64(2.0, __dsqrt_rn(mul64(a, b))));
    if (!(q >= -1.0 && q <= 1.0)) return -1;  // outside acos' domain: the reference fails too
    // cos(deg2rad(180 - degrees(acos(q)))) is -q up to the round trip's rounding
    double es = floor(add64(div64(511.0, add64(1.0, add64(1.0, q))), 0.5));
    return (int)mul64(es, 2.0) - 1;
}

// Scattered-energy row of a pair from the two legs' unit vectors held as
// float pairs (b + c, about 48 bits each), all in FP32: the cosine q between
// the legs (= -cos of the scatter angle, :495, :498-499) as a float pair from
// exact products (FMA residuals) and two-sums, d = 2 + q, e = 511 / d with
// one residual correction, and the fraction of e + 0.5.  Its error is about
// 1e-11 keV, the FP64 evaluation's (energy_row_fp64) about 1e-12, so the row
// floor(e + 0.5) * 2 - 1 is decided here unless e + 0.5 lies within 1e-6 of
// an integer or the legs are within 1e-6 of collinear (where the reference's
// acos may leave its domain): then -2, and the FP64 evaluation decides.  qc:
// q in FP32 for the Klein-Nishina factor.
__device__ __forceinline__ int energy_row_pair(float4 bw, float4 cw, float4 bp, float4 cp, float& qc)
{
    const float p0 = bw.x * bp.x, p1 = bw.y * bp.y, p2 = bw.z * bp.z;
    const float r = fmaf(bw.x, bp.x, -p0) + fmaf(bw.y, bp.y, -p1) + fmaf(bw.z, bp.z, -p2);
    float s = p0 + p1, v = s - p0;
    float t = (p0 - (s - v)) + (p1 - v);
    const float s2 = s + p2;
    v = s2 - s;
    t += (s - (s2 - v)) + (p2 - v);
    const float cross = fmaf(bw.x, cp.x, fmaf(cw.x, bp.x, fmaf(bw.y, cp.y, fmaf(cw.y, bp.y, fmaf(bw.z, cp.z, cw.z * bp.z)))));
    const float ql = t + r + cross;  // q = s2 + ql
    qc = fminf(1.f, fmaxf(-1.f, s2 + ql));
    float dh = 2.f + s2;
    v = dh - 2.f;
    float dl = ((2.f - (dh - v)) + (s2 - v)) + ql;
    const float d1 = dh + dl;
    dl -= d1 - dh;
    dh = d1;
    const float y = __fdiv_rn(511.f, dh);
    const float el = __fdividef(fmaf(-y, dh, 511.f) - y * dl, dh);  // e = y + el
    const float n0 = floorf(y + 0.5f);
    const float f = (y - (n0 - 0.5f)) + el;  // fraction of e + 0.5 (y - (n0 - 0.5) is exact)
    if (!(f > 1e-6f && f < 1.f - 1e-6f) || fabsf(qc) > 1.f - 1e-6f) return -2;
    return 2 * (int)n0 - 1;
}

// Factored weights of one voxel whose table entry is loaded: w_b =
// 2^(Y - (n-b) beta - gamma (n-b)^2) = [A r^b] G[n][b], with ar = (A, r),
// A = 2^(Y - n beta), r = 2^beta tabled per offset and nb = n; ca times the
// power of r is carried along: one FFMA2 and one FMUL2 per bin pair.  Bins past
// the last one have G = 0.
template <int NP>
__device__ __forceinline__ void accumulate_loaded(float2 (&acc)[NP], float ca, float2 ar, int nb, const float* sG)
{
    float2 P2 = make_float2(ca * ar.x, 0.f);
    P2.y = P2.x * ar.y;
    const float r2 = ar.y * ar.y;
    const float2 R2 = make_float2(r2, r2);
    const float2* G2 = reinterpret_cast<const float2*>(sG + nb * kGRow);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        acc[k] = __ffma2_rn(P2, G2[k], acc[k]);
        if (k + 1 < NP) P2 = __fmul2_rn(P2, R2);
    }
}

// floor(x) for |x| < 2^22: a round-down add of 1.5 * 2^23 leaves it in the
// mantissa.
__device__ __forceinline__ int floor_small(float x)
{
    return __float_as_int(__fadd_rd(x, 12582912.0f)) - 0x4B400000;
}

// floor(uh + ul + sigma (rh + rl)), sigma = +-1, for |uh + sigma rh| < 2^22
// and low parts far below 1: the TOF offset of a voxel from float-pair
// distances (about 44 bits), which takes the reference's FP64 column (:520,
// :526) except within about 1e-9 ps of a column boundary.  s = uh + sigma rh
// and its rounding error e come from a two-sum; floor(s) moves by one when
// the low parts carry the sum across an integer.  With f = s - floor(s)
// (exact for s >= 0: s and floor(s) lie within a factor of two) that is
// low >= 1 - f or low < -f, both compared exactly (1 - f is exact too).
__device__ __forceinline__ int floor_pair(float uh, float ul, float sigma, float rh, float rl)
{
    const float b = sigma * rh;  // exact
    const float s = uh + b;
    const float bb = s - uh;
    const float e = (uh - (s - bb)) + (b - bb);
    const float low = e + fmaf(sigma, rl, ul);
    const float y = __fadd_rd(s, 12582912.0f);
    const int t = __float_as_int(y) - 0x4B400000;
    const float f = s - (y - 12582912.0f);  // s - floor(s)
    return t + (low >= 1.f - f ? 1 : 0) - (low < -f ? 1 : 0);
}

// numpy's wrap of a negative table index (:521, :527).  The result may still
// lie outside 0..8000 (the reference's IndexError); the caller compares it
// with its bound.
__device__ __forceinline__ int wrap_offset(int t) { return t < 0 ? t + kTofEntries : t; }

// Offset index of the factored path's hot loop: t (a raw floor) when it lies
// in 0..tsafe-1, else kZeroEntry (weights 0) with the miss noted in far.  A
// negative t counts as a miss here too; far_voxel then applies numpy's wrap
// to it.
__device__ __forceinline__ int lookup_offset(int t, int tsafe, bool& far)
{
    const bool ok = (unsigned)t < (unsigned)tsafe;
    far |= !ok;
    return ok ? t : kZeroEntry;
}

// Per-bin weights w_b = 2^(Y - d (beta + gamma d)), d = n - b, each on the
// SFU; ca * w_b is added to every bin.  Bins go two at a time through packed
// FP32x2 instructions; with an odd bin count the last pair's second bin does
// not exist.
template <int NP, bool ODD>
__device__ __forceinline__ void accumulate_per_bin(float2 (&acc)[NP], float ca, float Y, float n, float beta,
                                                   const TofConst& T)
{
    const float2 Y2 = make_float2(Y, Y), b2 = make_float2(beta, beta);
    const float2 ca2 = make_float2(ca, ca), mg2 = make_float2(-T.gamma, -T.gamma);
    const float2 two = make_float2(2.f, 2.f);
    float2 nd = make_float2(-n, 1.f - n);  // b - n for the pair (b, b+1)
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const float2 t2 = __ffma2_rn(mg2, nd, b2);  // beta + gamma d
        const float2 e2 = __ffma2_rn(nd, t2, Y2);   // Y - d (beta + gamma d)
        const float wy = (ODD && k + 1 == NP) ? 0.f : ex2(e2.y);
        acc[k] = __ffma2_rn(ca2, make_float2(ex2(e2.x), wy), acc[k]);
        if (k + 1 < NP) nd = __fadd2_rn(nd, two);
    }
}

// A voxel the factored path's hot loop left out (raw floor traw outside
// 0..T.tsafe-1): numpy's wrap of a negative index; a wrapped offset below
// T.tsafe takes the factored weights, one far past the last bin the per-bin
// weights from its (Y, 0) entry and its bin n, and one outside the table is
// flagged and adds nothing.  Runs only for such voxels.
template <int NP, bool ODD>
__device__ __forceinline__ void far_voxel(float2 (&acc)[NP], float ca, int traw, const float2* sAR,
                                          const unsigned char* sN, const float* sG, const TofConst& T,
                                          bool& tof_bad)
{
    const int t = wrap_offset(traw);
    if ((unsigned)t >= (unsigned)kTofEntries) {
        tof_bad = true;
        return;
    }
    if (t < T.tsafe) {
        const float2 ar = sAR[t];
        accumulate_loaded<NP>(acc, ca, ar, __float_as_int(ar.x) & T.nmask, sG);
        return;
    }
    const float n = (float)sN[t];
    const float beta = T.kappa2w * ((float)(t - kTimeRange) - fmaf(n, T.w, T.s0));
    accumulate_per_bin<NP, ODD>(acc, ca, sAR[t].x, n, beta, T);
}

// Adds ca * w_b(t) to every bin b, t = traw (a raw floor: an offset index
// into the reference's 8001-entry TOF table, :520-528), where the factored
// weights are not used (one bin, or bins too wide for them).  w_b is rebuilt
// from the largest weight of the column, 2^Y at bin n, and the Gaussian's
// exact ratio between bins: log2 w_b = Y - d (beta + gamma d), d = n - b;
// NP = number of bin pairs.
template <int NP, bool SINGLE, bool ODD>
__device__ __forceinline__ void accumulate_voxel(float2 (&acc)[NP], float ca, int traw,
                                                 const float2* sAR, const unsigned char* sN,
                                                 const TofConst& T, bool& tof_bad)
{
    int t = traw;
    if ((unsigned)t >= (unsigned)kTofEntries) {
        if (t < 0 && t + kTofEntries >= 0) {  // numpy negative index wraps (:521, :527)
            t += kTofEntries;
        } else {
            tof_bad = true;
            return;
        }
    }
    const float off = (float)(t - kTimeRange);  // exact
    const float Y = sAR[t].x;
    const float n = (float)sN[t];
    // beta = 2 kappa w (off - s_n), s_n = s0 + n w
    const float beta = T.kappa2w * (off - fmaf(n, T.w, T.s0));
    if constexpr (SINGLE) {
        acc[0].x = fmaf(ca, ex2(fmaf(-n, fmaf(T.gamma, n, beta), Y)), acc[0].x);
    } else {
        accumulate_per_bin<NP, ODD>(acc, ca, Y, n, beta, T);
    }
}

// One task.  Every lane pairs lw with its own partner leg lp; the pair
// (l1, l2) is ordered as the reference orders it (crystal of l1 < crystal of
// l2, :469).  The task adds the part of the pair's TOF sum that runs over
// lw's voxels (AB1 if lw is l1, AB2 if lw is l2, :519-530); the other part
// comes from the task that walks lp.  Both tasks see the same scatter points,
// so both divide by the same per-slice count (:555-557).  All lanes walk the
// same voxel list: 32 voxels at a time are staged in the warp's shared
// buffer and read back as broadcasts, so the trip count is uniform.
// KAHAN: the precision launch, which also forms each voxel's TOF offset from
// float-pair distances (floor_pair; the samples' low floats staged in vlo).
template <int NP, bool SINGLE, bool ODD, bool KAHAN>
__device__ __forceinline__ void walk_task(const PairCtx& C, const TofConst& T, int s_first, int s_count,
                                          int lw, int chunk, int lane, const float2* sAR,
                                          const unsigned char* sN, const float* sG, float2* vbuf, float* vlo,
                                          float2* kahan,
                                          bool& tof_bad, bool& energy_bad, bool& nonfinite,
                                          unsigned long long& walked, unsigned long long& npairs)
{
    const float inv_c = (float)(1.0 / kLightCmPerPs);
    const int dw = lw / C.nru, rw = lw % C.nru;  // legs are crystal-major

    // partner of this lane: legs 0..nl-1 (lw leads the pair unless its
    // crystal is the larger), then one more entry per other ring for the
    // same crystal in the opposite role (both orders are distinct pairs)
    const int q = chunk * 32 + lane;
    int lp = lw, rp = rw, dp = dw;
    bool w_first = true, lane_ok = false;
    if (q < C.nl) {
        lp = q;
        dp = q / C.nru;
        rp = q % C.nru;
        lane_ok = lp != lw;
        w_first = dp >= dw;
    } else if (q < C.nl + C.nru) {
        rp = q - C.nl;
        dp = dw;
        lp = dw * C.nru + rp;
        lane_ok = rp != rw;
        w_first = false;
    }
    const int l1 = w_first ? lw : lp, l2 = w_first ? lp : lw;
    // sv1 - sv2 = -sigma (sv_w - sv_p); the walked leg's samples enter the TOF
    // offset with sign sigma (:520 for leg 1, :526 for leg 2)
    const float sigma = w_first ? -1.f : 1.f;

    float2 acc[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) acc[k] = make_float2(0.f, 0.f);
    float cnt = 0.f;
    constexpr int kStride = 32 * kKahanWarps;  // this thread's Kahan column: [j * kStride]
    if constexpr (KAHAN) {
#pragma unroll
        for (int j = 0; j < 2 * NP; ++j) kahan[j * kStride] = make_float2(0.f, 0.f);
    }

    for (int s = s_first; s < s_first + s_count; ++s) {
        if constexpr (KAHAN) {
#pragma unroll
            for (int k = 0; k < NP; ++k) acc[k] = make_float2(0.f, 0.f);  // this point's partial
        }
        const long long lo = (long long)s * C.nl;
        const float4 Aw = C.legA[lo + lw], Bw = C.legB[lo + lw];
        const float4 Ap = C.legA[lo + lp], Bp = C.legB[lo + lp];
        // everything below but the TOF offset's sign is symmetric in the two legs
        bool ok = lane_ok && Aw.z != INFINITY && Ap.z != INFINITY && !(Aw.y == 0.f && Ap.y == 0.f);
        float c = 0.f;
        if (ok) {
            // cos of the angle between the legs = -cos(scatter angle) (:495, :498-499)
            // and the scattered energy's row.  In FP32 from the legs' high floats
            // the energy is within 3e-4 keV of the FP64 value, which decides the
            // row except within 1e-3 keV of a rounding boundary (one pair in 500):
            // there the float pairs decide it, and FP64 only within 1e-6 keV (about
            // one pair in a million).
            float qc = fmaf(Bw.x, Bp.x, fmaf(Bw.y, Bp.y, Bw.z * Bp.z));
            qc = fminf(1.f, fmaxf(-1.f, qc));
            const float e = __fdividef(511.0f, 2.0f + qc);
            const float eh = e + 0.5f;
            const float fr = eh - floorf(eh);
            int row;
            if (fr < 1e-3f || fr > 1.0f - 1e-3f || fabsf(qc) > 1.0f - 1e-5f) {
                row = energy_row_pair(Bw, C.legC[lo + lw], Bp, C.legC[lo + lp], qc);
                if (row == -2) row = energy_row_fp64(C, s, rw, dw, rp, dp);
            } else {
                row = 2 * (int)floorf(eh) - 1;
            }
            if (row < 0 || row >= 2000) {
                energy_bad = true;
            } else {
                const float effp = __ldg(C.eff + row);
                if (effp != 0.f) {  // :508-509 skips before the count is added
                    const float rr = __ldg(C.ratio + row);
                    // Klein-Nishina with cos(theta) = -qc (:239-258): Ratio = 1/den
                    const float den = fmaf(C.gamma_kn, 1.0f + qc, 1.0f);
                    const float ratio = __frcp_rn(den);
                    const float sin2 = fmaf(-qc, qc, 1.0f);
                    const float kn = ratio * ratio * (ratio + den - sin2);
                    // geometry (:533-536): (ds)^2 |cos a1||cos a2| / (4 pi sv1^2 sv2^2)
                    const float f = C.geo_c * (Aw.w * Ap.w) * (effp * kn);
                    // this task's part: M1 * M2^r * AB1 or M2 * M1^r * AB2 (:540)
                    const float mw = ex2(-Aw.z), mpr = ex2(-rr * Ap.z);
                    if (Aw.y != 0.f) c = f * mw * mpr;
                    cnt += (Aw.y != 0.f && Ap.y != 0.f) ? 2.f : 1.f;  // :485-488
                    npairs += 1;
                }
            }
        }
        // TOF offset index: floor(2((sv1-sv2)/2 -/+ r)/c + 0.5) + 4000 (:520, :526)
        float u = fmaf(-sigma * (Aw.x - Ap.x), inv_c, 4000.5f), ul = 0.f;
        if constexpr (KAHAN) {
            // u = 4000.5 - sigma (sv_w - sv_p) / c as a float pair from the
            // distances' float pairs (high in legA.x, low in legC.w)
            const float dw = C.legC[lo + lw].w, dp = C.legC[lo + lp].w;
            const float dh = Aw.x - Ap.x, dv = dh - Aw.x;
            const float dl = ((Aw.x - (dh - dv)) + (-Ap.x - dv)) + (dw - dp);  // sv_w - sv_p = dh + dl
            const float ich = (float)(1.0 / kLightCmPerPs);
            const float icl = (float)(1.0 / kLightCmPerPs - (double)ich);
            const float ph = dh * ich;
            const float pl = fmaf(dh, ich, -ph) + fmaf(dh, icl, dl * ich);  // (sv_w - sv_p) / c = ph + pl
            const float b = -sigma * ph;
            u = 4000.5f + b;
            const float bb = u - 4000.5f;
            ul = ((4000.5f - (u - bb)) + (b - bb)) - sigma * pl;
        }
        if (SINGLE && C.unit_tof) {
            // weights of exactly 1: sum(a_v * 1) is the walking leg's activity integral
            acc[0].x = fmaf(c, Aw.y, acc[0].x);
        } else if (__any_sync(0xffffffffu, c != 0.f)) {
            const int nw = __float_as_int(Bw.w);
            if (c != 0.f) walked += nw;
            const float2* vw = C.vox + (lo + lw) * C.cap;
            // raw floor of the TOF offset of staged voxel j, v = vbuf[j]
            auto offset_of = [&](const float2& v, int j) {
                if constexpr (KAHAN)
                    return floor_pair(u, ul, sigma, v.y, vlo[j]);
                else
                    return floor_small(fmaf(sigma, v.y, u));
            };
            for (int k0 = 0; k0 < nw; k0 += 32) {
                __syncwarp();
                if (k0 + lane < nw) {
                    vbuf[lane] = vw[k0 + lane];
                    if constexpr (KAHAN) vlo[lane] = C.vox_lo[(lo + lw) * C.cap + k0 + lane];
                }
                __syncwarp();
                const int jn = min(32, nw - k0);
                if (c != 0.f) {
                    if (!SINGLE && T.factored) {
                        // the table lookup of voxel j+1 overlaps the accumulation of voxel j
                        // (offsets outside 0..T.tsafe-1, far past the last bin, wrapped or
                        // outside the table, add nothing here; they are noted and taken
                        // afterwards)
                        bool anyfar = false;
                        const float2 v = vbuf[0];
                        int t = lookup_offset(offset_of(v, 0), T.tsafe, anyfar);
                        float2 ar = sAR[t];
                        int nb = __float_as_int(ar.x) & T.nmask;
                        float ca = c * v.x;
#pragma unroll 2
                        for (int j = 0; j < jn; ++j) {
                            const int j1 = j + 1 < jn ? j + 1 : j;
                            const float2 v1 = vbuf[j1];
                            const int t1 = lookup_offset(offset_of(v1, j1), T.tsafe, anyfar);
                            const float2 ar1 = sAR[t1];
                            const int nb1 = __float_as_int(ar1.x) & T.nmask;
                            accumulate_loaded<NP>(acc, ca, ar, nb, sG);
                            ar = ar1;
                            nb = nb1;
                            ca = c * v1.x;
                        }
                        if (anyfar) {  // rare: this batch's voxels outside the factored range
                            for (int j = 0; j < jn; ++j) {
                                const float2 vf = vbuf[j];
                                const int tf = offset_of(vf, j);
                                if ((unsigned)tf >= (unsigned)T.tsafe)
                                    far_voxel<NP, ODD>(acc, c * vf.x, tf, sAR, sN, sG, T, tof_bad);
                            }
                        }
                    } else {
#pragma unroll 2
                        for (int j = 0; j < jn; ++j) {
                            const float2 v = vbuf[j];
                            accumulate_voxel<NP, SINGLE, ODD>(acc, c * v.x, offset_of(v, j), sAR, sN, T, tof_bad);
                        }
                    }
                }
            }
        }
        if constexpr (KAHAN) {
            // sum += partial with Kahan's compensated addition (all terms >= 0)
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                float2 sum = kahan[k * kStride], cmp = kahan[(NP + k) * kStride];
                const float yx = __fsub_rn(acc[k].x, cmp.x), yy = __fsub_rn(acc[k].y, cmp.y);
                const float tx = __fadd_rn(sum.x, yx), ty = __fadd_rn(sum.y, yy);
                cmp = make_float2(__fsub_rn(__fsub_rn(tx, sum.x), yx), __fsub_rn(__fsub_rn(ty, sum.y), yy));
                kahan[k * kStride] = make_float2(tx, ty);
                kahan[(NP + k) * kStride] = cmp;
            }
        }
    }
    if constexpr (KAHAN) {
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            const float2 sum = kahan[k * kStride], cmp = kahan[(NP + k) * kStride];
            acc[k] = make_float2(__fsub_rn(sum.x, cmp.x), __fsub_rn(sum.y, cmp.y));
        }
    }
    if (lane_ok && cnt > 0.f) {
        float* o = C.out + (long long)l1 * C.nl + l2;
        const long long plane = (long long)C.nl * C.nl;
        const float inv = 1.0f / cnt;
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            const float vx = acc[k].x * inv, vy = acc[k].y * inv;
            if (2 * k < C.nbins) {
                nonfinite |= !isfinite(vx);
                atomicAdd(o + (2 * k) * plane, vx);
            }
            if (2 * k + 1 < C.nbins) {
                nonfinite |= !isfinite(vy);
                atomicAdd(o + (2 * k + 1) * plane, vy);
            }
        }
    }
}

// Block-end bookkeeping: error bits and the walked / evaluated counters.
__device__ __forceinline__ void finish_pairs(int lane, bool tof_bad, bool energy_bad, bool nonfinite,
                                             unsigned long long walked, unsigned long long npairs,
                                             int32_t* status, unsigned long long* work)
{
    if (tof_bad) raise_error(status, kErrTofRange);
    if (energy_bad) raise_error(status, kErrEnergy);
    if (nonfinite) raise_error(status, kErrNonFinite);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        walked += __shfl_xor_sync(0xffffffffu, walked, o);
        npairs += __shfl_xor_sync(0xffffffffu, npairs, o);
    }
    if (lane == 0 && work) {
        atomicAdd(work, walked);
        atomicAdd(work + 1, npairs);
    }
}

}  // namespace sss
