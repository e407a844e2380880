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
    int nd, nru, ndu, nl, cap;
    long long nvox;
    const double* points;  // wave's first point, [n][4]
    int npts;
    float4* legA;   // [npts][nl]: sv, activity integral, mu integral * log2(e), |cos a|/sv^2
    float4* legB;   // [npts][nl]: unit vector to the crystal (high floats), voxel-list length (int bits)
    float4* legC;   // [npts][nl]: the unit vector's low floats (FP64 value = high + low), 0
    float2* vox;    // [npts][nl][cap]: act*len, 2*sample/c (ps), leg-major; null: no lists
    int32_t* status;
};

// One leg: scatter point s to sampled crystal leg l.
__device__ __forceinline__ void leg_one(const LegParams& P, int s, int l)
{
    const int di = l / P.nru, ri = l % P.nru;  // legs are crystal-major
    const int ring = P.rings[ri], det = P.dets[di];
    const double* dp = P.geom + 3 * ((long long)ring * P.nd + det);
    const double zD = P.geom[3 * ((long long)ring * P.nd) + 2];  // :402 (crystal 0's z)
    const double xS = P.points[4 * s], yS = P.points[4 * s + 1], zS = P.points[4 * s + 2];
    double lc[6] = {xS, yS, zS, dp[0], dp[1], zD};

    // incidence angle term |cos a| (:424-430, :533-535) and distance (:442-444)
    const double vx = dp[0] - xS, vy = dp[1] - yS, vz = zD - zS;
    const double* nv = P.normals + 3 * ((long long)ring * P.nd + det);
    const double vn = sqrt(vx * vx + vy * vy + vz * vz);
    const double nn = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
    const double cosa = fabs((vx * nv[0] + vy * nv[1] + vz * nv[2]) / (nn * vn));
    const float sv = (float)vn;

    float asum = 0.f, musum = 0.f;
    int nlist = 0;
    Ray r;
    if (ray_setup(P.g, lc, 1e-20, r)) {
        const float vlen = (float)sqrt(r.xv * r.xv + r.yv * r.yv + r.zv * r.zv);
        const float inv_c = (float)(1.0 / kLightCmPerPs);
        const double t0 = r.tmin;
        // parameter gaps in fixed point (exact differences, no FP64 subtraction)
        // while the parameters stay below 4 in magnitude, else in FP64
        const bool ok0 = fix61_ok(t0);
        const int64_t f0 = fix61(t0);
        int64_t fprev = f0;
        bool okprev = ok0;
        float2* out = P.vox ? P.vox + ((long long)s * P.nl + l) * P.cap : nullptr;
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
                const float dt0 = ok0b ? unfix61_abs(fb - f0) : (float)(tb - t0);
                float rho = vlen * dt0 * inv_c;
                out[nlist] = make_float2(a, rho);
                ++nlist;
            }
        });
        if (c < 0) raise_error(P.status, kErrOverrun);
    }
    const long long o = (long long)s * P.nl + l;
    // exp(-I) underflows to 0 in FP64 above ~745.13 (the skip at :451 / :483)
    const float ilog2 = musum > 745.13f ? INFINITY : musum * 1.4426950408889634f;
    P.legA[o] = make_float4(sv, asum, ilog2, (float)(cosa / (vn * vn)));
    // the unit vector in FP64, kept as float pairs (high + low, about 48 bits)
    // so that the pair stage can form the cosine between two legs to ~1e-14
    const double inv = 1.0 / vn;
    const double u[3] = {vx * inv, vy * inv, vz * inv};
    float hi[3], lo[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        hi[k] = (float)u[k];
        lo[k] = (float)(u[k] - (double)hi[k]);
    }
    P.legB[o] = make_float4(hi[0], hi[1], hi[2], __int_as_float(nlist));
    P.legC[o] = make_float4(lo[0], lo[1], lo[2], 0.f);
}

}  // namespace sss
