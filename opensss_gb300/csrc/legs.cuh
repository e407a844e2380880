// The TOF-SSS leg stage: one scatter point to one sampled crystal.  Shared
// by the single-problem kernel (sss.cu) and the batched kernels (batch.cu).
// Reference: bodySSS legs, Python/openSSS/SingleScatterSimulationTOF.py:400-430.
#pragma once

#include "common.cuh"
#include "pair.cuh"
#include "trace.cuh"

namespace sss {

constexpr int kLegThreadsDefault = 128;  // leg-kernel block (sss_tof_problem.leg_threads = 0)
constexpr int kLegThreadsMax = 256;      // the leg kernels are compiled for blocks up to this size

struct LegParams {
    Grid g;
    const float* act;
    const float* mu;
    const double* geom;
    const double* normals;
    const int32_t* rings;
    const int32_t* dets;
    int nr, nd, nru, ndu, nl, cap;
    long long nvox;
    const double* points;  // wave's first point, [n][4]
    int npts;
    float4* legA;   // [npts][nl]: sv, activity integral, mu integral * log2(e), |cos a|/sv^2
    float4* legB;   // [npts][nl]: unit vector to the crystal (high floats), voxel-list length (int bits)
    float4* legC;   // [npts][nl]: the unit vector's low floats (FP64 value = high + low), the
                    // distance's low float
    float2* vox;    // [npts][nl][cap]: act*len, 2*sample/c (ps), leg-major; null: no lists
    float* vox_lo;  // [npts][nl][cap]: the samples' low floats (2*sample/c = high + low), or null
    int32_t* status;
};

// A unit-vector component u (|u| <= 1) as a float pair hi + lo: hi is u
// truncated to 24 significant bits, lo the float nearest the remaining bits
// (about 48 bits together), formed from u's bit pattern with integer
// operations.  Components below 2^-74 in magnitude keep hi only.
__device__ __forceinline__ void split_float_pair(double u, float& hi, float& lo)
{
    const uint64_t b = dbits(u);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    const uint32_t sign = (uint32_t)(b >> 63) << 31;
    if (e < 1023 - 126) {  // |u| < 2^-126: below the float normal range, negligible here
        hi = 0.f;
        lo = 0.f;
        return;
    }
    const uint64_t m = b & ((1ull << 52) - 1);
    hi = __uint_as_float(sign | ((e - 1023 + 127) << 23) | (uint32_t)(m >> 29));
    const uint32_t low = (uint32_t)(m & ((1u << 29) - 1));  // value low * 2^(e - 1075)
    lo = e >= 949 ? __uint_as_float(sign | 0x3F800000u) * (float)low * __uint_as_float((e - 1075 + 127) << 23)
                  : 0.f;
}

// One leg: scatter point s to sampled crystal leg l.
__device__ __forceinline__ void leg_one(const LegParams& P, int s, int l)
{
    const int di = l / P.nru, ri = l % P.nru;  // legs are crystal-major
    const int ring = P.rings[ri], det = P.dets[di];
    const long long o = (long long)s * P.nl + l;
    if ((unsigned)ring >= (unsigned)P.nr || (unsigned)det >= (unsigned)P.nd) {
        // the caller's ring or crystal table: an empty leg (mu integral +inf,
        // so no pair uses it) and the error bit
        raise_error(P.status, kErrTable);
        P.legA[o] = make_float4(0.f, 0.f, INFINITY, 0.f);
        P.legB[o] = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
        P.legC[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const double* dp = P.geom + 3 * ((long long)ring * P.nd + det);
    const double zD = P.geom[3 * ((long long)ring * P.nd) + 2];  // :402 (crystal 0's z)
    const double xS = P.points[4 * s], yS = P.points[4 * s + 1], zS = P.points[4 * s + 2];
    double lc[6] = {xS, yS, zS, dp[0], dp[1], zD};

    // distance (:442-444) and the unit vector to the crystal in FP64; the
    // unit vector is kept as float pairs for the pair stage's energy row
    const double vx = dp[0] - xS, vy = dp[1] - yS, vz = zD - zS;
    const double vn = sqrt(vx * vx + vy * vy + vz * vz);
    const double inv = div64(1.0, vn);
    float hi[3], lo[3];
    split_float_pair(vx * inv, hi[0], lo[0]);
    split_float_pair(vy * inv, hi[1], lo[1]);
    split_float_pair(vz * inv, hi[2], lo[2]);
    // incidence term |cos a| / sv^2 (:424-430, :533-535), in FP32: it only
    // scales the pair's term (relative error ~1e-7)
    const double* nv = P.normals + 3 * ((long long)ring * P.nd + det);
    const float nx = (float)nv[0], ny = (float)nv[1], nz = (float)nv[2];
    const float cosa = fabsf(fmaf(hi[0], nx, fmaf(hi[1], ny, hi[2] * nz))) * rsqrtf(fmaf(nx, nx, fmaf(ny, ny, nz * nz)));
    const float sv = (float)vn;
    float asum = 0.f, musum = 0.f;
    int nlist = 0;
    Ray r;
    if (ray_setup(P.g, lc, 1e-20, r)) {
        const float vlen = sv;  // |end - start|: the ray's direction is the leg vector itself
        const float inv_c = (float)(1.0 / kLightCmPerPs);
        const double t0 = r.tmin;
        // parameter gaps in fixed point (exact differences, no FP64 subtraction)
        // while the parameters stay below 4 in magnitude, else in FP64
        const bool ok0 = fix61_ok(t0);
        const int64_t f0 = fix61(t0);
        int64_t fprev = f0;
        bool okprev = ok0;
        float2* out = P.vox ? P.vox + ((long long)s * P.nl + l) * P.cap : nullptr;
        float* out_lo = P.vox_lo ? P.vox_lo + ((long long)s * P.nl + l) * P.cap : nullptr;
        int c = ray_walk(P.g, r, P.cap, [&](int k, int64_t lin, double ta, double tb) {
            const bool okb = fix61_ok(tb);
            const int64_t fb = fix61(tb);
            const bool okab = okb && okprev, ok0b = okb && ok0;
            const int64_t fa = fprev;
            fprev = fb;
            okprev = okb;
            long long v = lin - 1;
            if (v < 0 || v >= P.nvox) {
                raise_error(P.status, kErrVoxel);
                return;
            }
            // |vec| * |dt|; for near-zero steps the reference's own FP64 length
            // expression decides whether a corner-grazing segment is zero or
            // not (that decides whether a leg carries activity, :483-488)
            const float adt = okab ? unfix61_abs(fb - fa) : (float)fabs(tb - ta);
            float len = adt < 1e-9f ? (float)ref_length(r, ta, tb) : vlen * adt;
            float a = __ldg(P.act + v) * len;
            musum = fmaf(__ldg(P.mu + v), len, musum);
            asum += a;
            if (a != 0.f && out) {
                // sample = half the distance walked to the voxel's exit (:155-156)
                if (out_lo) {
                    // the precision launch: 2 * sample / c in FP64, kept as a float pair
                    const double dt = ok0b ? unfix61_abs_d(fb - f0) : tb - t0;
                    const double rho = vn * dt * (1.0 / kLightCmPerPs);
                    const float rh = (float)rho;
                    out[nlist] = make_float2(a, rh);
                    out_lo[nlist] = (float)(rho - (double)rh);
                } else {
                    const float dt0 = ok0b ? unfix61_abs(fb - f0) : (float)(tb - t0);
                    out[nlist] = make_float2(a, vlen * dt0 * inv_c);
                }
                ++nlist;
            }
        });
        if (c < 0) raise_error(P.status, kErrOverrun);
    }
    // exp(-I) underflows to 0 in FP64 above ~745.13 (the skip at :451 / :483)
    const float ilog2 = musum > 745.13f ? INFINITY : musum * 1.4426950408889634f;
    P.legA[o] = make_float4(sv, asum, ilog2, cosa / (sv * sv));
    P.legB[o] = make_float4(hi[0], hi[1], hi[2], __int_as_float(nlist));
    P.legC[o] = make_float4(lo[0], lo[1], lo[2], (float)(vn - (double)sv));
}

}  // namespace sss
