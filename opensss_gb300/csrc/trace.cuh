// Amanatides-Woo voxel traversal in IEEE FP64, operation for operation as in
// the reference tracer (Python/openSSS/RayTracing3DTOF.py:29-180 with
// BoxIntersectTest :204-269; Matlab/RayTracing3DTOF.cpp:51-341).  Every FP64
// operation is an explicit round-to-nearest intrinsic, so no multiply-add is
// fused whatever the compile flags, and the voxel sequence is bit-identical
// to the reference's.
#pragma once

#include <cstring>

#include "common.cuh"

namespace sss {

__device__ __forceinline__ double mul64(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add64(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub64(double a, double b) { return __dsub_rn(a, b); }
// FP64 division, round to nearest: on the integer pipe where div_bits takes
// the operands (normal values with a normal or zero quotient), else __ddiv_rn;
// the same IEEE result either way.
__device__ __forceinline__ double div64(double a, double b);
// Python's built-in min/max: the first argument wins unless the second
// compares strictly smaller / larger (RayTracing3DTOF.py:53-54, 77-78).
__device__ __forceinline__ double pymin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double pymax(double a, double b) { return (b > a) ? b : a; }

struct Grid {
    int nx, ny, nz;
    double b[6];   // xMin yMin zMin xMax yMax zMax
    double vs[3];  // voxel sizes (b[3+k] - b[k]) / n_k, set by grid_of (:80-82)
    double ivs[3]; // 1 / vs[k], for quotients whose ceiling alone is needed
};

// A grid with its voxel sizes, computed once per launch with the reference's
// IEEE operations (one subtraction and one division, no fused multiply-add).
__host__ __device__ inline Grid grid_of(int nx, int ny, int nz, const double* bounds)
{
    Grid g;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    for (int k = 0; k < 6; ++k) g.b[k] = bounds[k];
    const double n[3] = {(double)nx, (double)ny, (double)nz};
    for (int k = 0; k < 3; ++k) g.vs[k] = (bounds[3 + k] - bounds[k]) / n[k];
    for (int k = 0; k < 3; ++k) g.ivs[k] = 1.0 / g.vs[k];
    return g;
}

// ceil(RN(num / vs)) from q = RN(num * RN(1 / vs)) without the division:
// q lies within 2.5 ulps of RN(num / vs), so where q is more than 4 ulps
// from every integer the two have the same ceiling, read here from q's bits
// (integer operations only).  Returns false, and leaves c alone, where q is
// that close to an integer, above 2^52 in magnitude or not finite: the
// caller then divides.
__host__ __device__ inline bool ceil_clear(double q, long long& c)
{
    uint64_t b;
    memcpy(&b, &q, 8);
    const int ex = (int)((b >> 52) & 0x7FF);
    const bool neg = (b >> 63) != 0;
    if (ex >= 1023 + 52) return false;  // |q| >= 2^52, infinite or NaN
    if ((b << 1) == 0) {                // +-0: the quotient is 0 too (num == 0)
        c = 0;
        return true;
    }
    if (ex < 1022) {  // 0 < |q| < 0.5, the quotient has q's sign: ceil is 1 or 0
        c = neg ? 0 : 1;
        return true;
    }
    const int fb = 1023 + 52 - ex;  // fraction bits of q, 1..53
    if (fb < 4) return false;
    const uint64_t m = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const uint64_t ip = m >> fb, fr = m & ((1ull << fb) - 1);
    if (fr <= 4 || fr >= (1ull << fb) - 4) return false;
    c = neg ? -(long long)ip : (long long)ip + 1;
    return true;
}

// Parametric state of one ray after set-up.
struct Ray {
    double tmin, tmax;
    double xv, yv, zv;          // direction (end - start)
    double xt, yt, zt;          // next crossing parameter per axis
    double xd, yd, zd;          // parametric step per axis
    int X, Y, Z;                // current voxel, 1-based
    int xe, ye, ze;             // final voxel, 1-based
    int xs, ys, zs;             // step directions
};

// BoxIntersectTest; eps = 1e-20 (RayTracing3DTOF.py:225) or 1e-23 for the
// non-TOF MEX variant (Matlab/RayTracing3D.cpp:267).
__device__ __forceinline__ bool box_intersect(const Grid& g, const double* lc, double eps,
                                              double& rtmin, double& rtmax)
{
    double tmin, tmax, a, b;
    double xdiv = div64(1.0, add64(sub64(lc[3], lc[0]), eps));
    if (xdiv >= 0) {
        tmin = mul64(sub64(g.b[0], lc[0]), xdiv);
        tmax = mul64(sub64(g.b[3], lc[0]), xdiv);
    } else {
        tmin = mul64(sub64(g.b[3], lc[0]), xdiv);
        tmax = mul64(sub64(g.b[0], lc[0]), xdiv);
    }
    double ydiv = div64(1.0, add64(sub64(lc[4], lc[1]), eps));
    if (ydiv >= 0) {
        a = mul64(sub64(g.b[1], lc[1]), ydiv);
        b = mul64(sub64(g.b[4], lc[1]), ydiv);
    } else {
        a = mul64(sub64(g.b[4], lc[1]), ydiv);
        b = mul64(sub64(g.b[1], lc[1]), ydiv);
    }
    if (tmin > b || a > tmax) return false;
    if (a > tmin) tmin = a;
    if (b < tmax) tmax = b;
    double zdiv = div64(1.0, add64(sub64(lc[5], lc[2]), eps));
    if (zdiv >= 0) {
        a = mul64(sub64(g.b[2], lc[2]), zdiv);
        b = mul64(sub64(g.b[5], lc[2]), zdiv);
    } else {
        a = mul64(sub64(g.b[5], lc[2]), zdiv);
        b = mul64(sub64(g.b[2], lc[2]), zdiv);
    }
    if (tmin > b || a > tmax) return false;
    if (a > tmin) tmin = a;
    if (b < tmax) tmax = b;
    if ((tmin >= 1 && tmax >= 1) || (tmin <= 0 && tmax <= 0)) return false;
    rtmin = tmin;
    rtmax = tmax;
    return true;
}

// Per-axis set-up (RayTracing3DTOF.py:77-123).  `start`/`end` are the grid
// entry/exit coordinates, n the voxel count on the axis.
// The first and last voxel on an axis: ceil((c - lo) / vs) clamped to 1..n
// (:89-110).  The ceiling comes from a product with 1/vs where that decides
// it (ceil_clear), else from the division; the clamp is the reference's
// min/max pair (both orders give the same integer).
__device__ __forceinline__ double voxel_of(double c, double lo, double vs, double ivs, int n, bool int_first)
{
    const double num = sub64(c, lo);
    long long k;
    if (ceil_clear(mul64(num, ivs), k)) return (double)(k < 1 ? 1 : (k > n ? n : k));
    const double c0 = ceil(div64(num, vs)), nn = (double)n;
    // z: int() before the clamp (RayTracing3DTOF.py:109-110)
    return int_first ? pymin(pymax(1.0, c0), nn) : pymax(1.0, pymin(nn, c0));
}

__device__ __forceinline__ void axis_setup(double lo, double vs, double ivs, int n, double v,
                                           double start, double end, double tmin, double tmax,
                                           bool int_first, int& X, int& Xe, int& st, double& tn,
                                           double& td)
{
    const double x = voxel_of(start, lo, vs, ivs, n, int_first);
    const double xe = voxel_of(end, lo, vs, ivs, n, int_first);
    if (v > 0) {
        st = 1;
        td = div64(vs, v);
        tn = add64(tmin, div64(sub64(add64(lo, mul64(x, vs)), start), v));
    } else if (v < 0) {
        st = -1;
        td = div64(vs, -v);
        tn = add64(tmin, div64(sub64(add64(lo, mul64(sub64(x, 1.0), vs)), start), v));
    } else {
        st = 0;
        tn = tmax;
        td = tmax;
    }
    X = (int)x;
    Xe = (int)xe;
}

// Ray set-up; returns false on a miss (the reference returns empty arrays).
__device__ __forceinline__ bool ray_setup(const Grid& g, const double* lc, double eps, Ray& r)
{
    double tmin, tmax;
    if (!box_intersect(g, lc, eps, tmin, tmax)) return false;
    tmin = pymax(tmin, 0.0);
    tmax = pymin(tmax, 1.0);
    const double vx = g.vs[0], vy = g.vs[1], vz = g.vs[2];
    r.xv = sub64(lc[3], lc[0]);
    r.yv = sub64(lc[4], lc[1]);
    r.zv = sub64(lc[5], lc[2]);
    double xs = add64(lc[0], mul64(r.xv, tmin)), ys = add64(lc[1], mul64(r.yv, tmin)),
           zs = add64(lc[2], mul64(r.zv, tmin));
    double xe = add64(lc[0], mul64(r.xv, tmax)), ye = add64(lc[1], mul64(r.yv, tmax)),
           ze = add64(lc[2], mul64(r.zv, tmax));
    axis_setup(g.b[0], vx, g.ivs[0], g.nx, r.xv, xs, xe, tmin, tmax, false, r.X, r.xe, r.xs, r.xt, r.xd);
    axis_setup(g.b[1], vy, g.ivs[1], g.ny, r.yv, ys, ye, tmin, tmax, false, r.Y, r.ye, r.ys, r.yt, r.yd);
    axis_setup(g.b[2], vz, g.ivs[2], g.nz, r.zv, zs, ze, tmin, tmax, true, r.Z, r.ze, r.zs, r.zt, r.zd);
    r.tmin = tmin;
    r.tmax = tmax;
    return true;
}

// sub2ind (RayTracing3DTOF.py:182-202): X + (Y-1)*Ny + (Z-1)*Ny*Nx, 1-based.
// Ny is the x stride, as in the reference; this is the true Fortran index
// only when Nx == Ny.
__device__ __forceinline__ int64_t sub2ind(const Grid& g, int X, int Y, int Z)
{
    return (int64_t)X + (int64_t)(Y - 1) * g.ny + (int64_t)(Z - 1) * g.ny * g.nx;
}

// IEEE-754 binary64 addition, round to nearest even, of two non-negative
// finite values given as bit patterns, with integer operations only (on this
// GPU the FP64 pipe issues a small fraction of the integer rate).  Written
// from the format's definition: the larger operand's significand (hidden bit
// restored, 10 guard bits) plus the smaller one's shifted right by the
// exponent difference with a sticky bit; a carry out shifts right once
// (sticky kept); the 53-bit result is rounded to nearest, ties to even, and
// the exponent is added back so that a rounding carry or a subnormal sum that
// reaches the normal range moves the exponent field by itself.  The caller
// keeps the exact sum below 2^1023 (no overflow to infinity).
__host__ __device__ __forceinline__ uint64_t add_nonneg_bits(uint64_t a, uint64_t b)
{
    constexpr uint64_t kFrac = (1ull << 52) - 1;
    const uint64_t hi = a > b ? a : b, lo = a > b ? b : a;  // bit order = value order here
    const uint32_t eh = (uint32_t)(hi >> 52), el = (uint32_t)(lo >> 52);
    const uint32_t sh = eh ? eh : 1u, sl = el ? el : 1u;  // subnormals: exponent field 0 counts as 1
    const uint64_t mh = ((hi & kFrac) | ((uint64_t)(eh != 0) << 52)) << 10;
    const uint64_t ml = ((lo & kFrac) | ((uint64_t)(el != 0) << 52)) << 10;
    const uint32_t d = sh - sl;
    uint64_t al;
    if (d == 0)
        al = ml;
    else if (d < 63)
        al = (ml >> d) | (uint64_t)((ml & ((1ull << d) - 1)) != 0);
    else
        al = (uint64_t)(ml != 0);
    uint64_t sum = mh + al;  // below 2^64: mh < 2^63, al < 2^63
    uint32_t e = sh;
    if (sum >> 63) {
        sum = (sum >> 1) | (sum & 1);
        e += 1;
    }
    uint64_t m = sum >> 10;  // 53 bits with the hidden one at bit 52 (below it for a subnormal sum)
    const uint32_t rest = (uint32_t)sum & 0x3FFu;
    m += (uint64_t)(rest > 0x200u || (rest == 0x200u && (m & 1)));
    return ((uint64_t)(e - 1) << 52) + m;
}

// High 64 bits of a 64 x 64-bit product.
__host__ __device__ inline uint64_t mulhi64(uint64_t a, uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// IEEE-754 binary64 division, round to nearest even, with integer
// operations only, for normal (or zero) dividends and normal divisors whose
// quotient is a normal double or zero; returns false (leaving q alone) for any
// other operands, which the caller divides in FP64.  Written from the
// format's definition: with significands ma, mb (hidden bit restored, ma
// doubled when below mb so that ma/mb lies in [1, 2)), the quotient's 56
// leading bits are floor(ma 2^55 / mb).  They come from a reciprocal
// R ~ 2^116 / mb held below its true value: a float seed with a margin, then
// two Newton steps in 128-bit fixed point (each stays below and squares the
// error), then q = floor(ma R / 2^61), at most two short, and the exact
// remainder ma 2^55 - q mb corrects it.  The three extra bits and whether
// the remainder is zero give round to nearest, ties to even.
__host__ __device__ inline bool div_bits(uint64_t a, uint64_t b, uint64_t& q)
{
    constexpr uint64_t kFrac = (1ull << 52) - 1, kHid = 1ull << 52;
    const uint32_t ea = (uint32_t)(a >> 52) & 0x7FFu, eb = (uint32_t)(b >> 52) & 0x7FFu;
    const uint64_t sign = (a ^ b) & (1ull << 63);
    if (eb == 0 || eb == 0x7FFu || ea == 0x7FFu) return false;  // zero, subnormal, inf or NaN divisor
    if (ea == 0) {
        if ((a & ~(1ull << 63)) != 0) return false;  // subnormal dividend
        q = sign;                                    // zero: a signed zero
        return true;
    }
    uint64_t ma = (a & kFrac) | kHid;
    const uint64_t mb = (b & kFrac) | kHid;
    int e = (int)ea - (int)eb + 1023;
    if (ma < mb) {
        ma <<= 1;
        e -= 1;
    }
    if (e < 1 || e > 2046) return false;  // the quotient is not a normal double
    uint64_t quo, rem;
    if (mb == kHid) {  // a power of two: exact
        quo = ma << 3;
        rem = 0;
    } else {
        // seed: 2^87 / (mb >> 29) in float, as 2^64-scaled fixed point, minus a
        // margin above its relative error (< 2^-22.5)
        const float rf = 1.0f / (float)(uint32_t)(mb >> 29);  // in (2^-24, 2^-23]
        uint32_t rbits;
        memcpy(&rbits, &rf, 4);
        uint64_t R = ((rbits >> 23) & 0xFFu) >= 127u - 23u ? ~0ull : ((uint64_t)((rbits & 0x7FFFFFu) | 0x800000u) << 40);
        R -= 1ull << 42;
#pragma unroll
        for (int it = 0; it < 2; ++it) {
            // E = 2^116 - mb R > 0 (R is below 2^116 / mb); R += floor(R E / 2^116)
            const uint64_t plo = mb * R, phi = mulhi64(mb, R);
            const uint64_t elo = 0 - plo, ehi = (1ull << 52) - phi - (plo != 0 ? 1ull : 0ull);
            const uint64_t t_lo = R * ehi, t_hi = mulhi64(R, ehi);  // R ehi, below 2^96
            const uint64_t add = mulhi64(R, elo);
            const uint64_t s_lo = t_lo + add;
            const uint64_t s_hi = t_hi + (s_lo < t_lo ? 1ull : 0ull);
            R += (s_hi << 12) | (s_lo >> 52);
        }
        const uint64_t plo = ma * R, phi = mulhi64(ma, R);
        quo = (phi << 3) | (plo >> 61);
        rem = (ma << 55) - quo * mb;  // exact: the true remainder lies in [0, 3 mb)
#pragma unroll
        for (int it = 0; it < 2; ++it) {
            if (rem >= mb) {
                rem -= mb;
                quo += 1;
            }
        }
    }
    uint64_t m = quo >> 3;
    const uint32_t g = (uint32_t)(quo & 7u);
    m += (uint64_t)(g > 4u || (g == 4u && (rem != 0 || (m & 1))));
    q = sign | (((uint64_t)(e - 1) << 52) + m);
    return true;
}

__device__ __forceinline__ uint64_t dbits(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double bitsd(uint64_t b) { return __longlong_as_double((long long)b); }

__device__ __forceinline__ double div64(double a, double b)
{
    uint64_t q;
    return div_bits(dbits(a), dbits(b), q) ? bitsd(q) : __ddiv_rn(a, b);
}

// Fixed-point form of a walk parameter, in units of 2^-61, for |t| < 4
// (fix61_ok): exact for |t| >= 2^-8 and truncated below, an absolute error
// under 2^-61.  Differences of such values are exact, so parameter gaps need
// no FP64 subtraction.
__device__ __forceinline__ bool fix61_ok(double t) { return ((dbits(t) >> 52) & 0x7FF) <= 1024; }
__device__ __forceinline__ int64_t fix61(double t)
{
    const uint64_t b = dbits(t);
    const int ex = (int)((b >> 52) & 0x7FF);
    const uint64_t m = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = ex - 1023 + 9;  // value = m 2^(ex - 1075) = (m 2^sh) 2^-61
    uint64_t v = 0;
    if (ex != 0) v = sh >= 0 ? m << sh : (sh > -64 ? m >> -sh : 0);
    return (b >> 63) ? -(int64_t)v : (int64_t)v;
}
// |x| 2^-61 as a float, truncated to 24 significant bits.
__device__ __forceinline__ float unfix61_abs(int64_t x)
{
    const uint64_t u = x < 0 ? (uint64_t)(-x) : (uint64_t)x;
    if (u == 0) return 0.f;
    const int lz = __clzll((long long)u);
    const uint32_t man = (uint32_t)((u << lz) >> 40);  // 24 bits, the leading one at bit 23
    return __uint_as_float(((uint32_t)(129 - lz) << 23) | (man & 0x7FFFFFu));
}

// The same as a double (53 bits, truncated).
__device__ __forceinline__ double unfix61_abs_d(int64_t x)
{
    const uint64_t u = x < 0 ? (uint64_t)(-x) : (uint64_t)x;
    if (u == 0) return 0.0;
    const int lz = __clzll((long long)u);
    const uint64_t man = (u << lz) >> 11;  // 53 bits, the leading one at bit 52
    return __longlong_as_double((long long)(((uint64_t)(1025 - lz) << 52) | (man & ((1ull << 52) - 1))));
}

// Walk the voxels.  For voxel k (0-based) the visitor receives
// (k, 1-based linear index, t at entry, t at exit).  Returns the voxel
// count, or -1 if the reference would overrun its Nx+Ny+Nz storage
// (RayTracing3DTOF.py:71-75, 162) — the visitor has then seen `cap` voxels.
//
// The axis choice and the crossing updates are the reference's FP64 ones
// (:133-150).  They are evaluated on the integer pipe while every crossing
// parameter is a non-negative finite double and every step is below 2^1000:
// then `<` between parameters is `<` between their bit patterns, and
// add_nonneg_bits gives the FP64 sum bit for bit (the walk takes at most cap
// steps, so no sum comes near overflow).  A start point on a voxel face can
// put a first crossing a rounding error below 0 (or at -0); such values are
// the smallest, so the FP64 steps that consume them come first, and the walk
// continues on the integer pipe once all three are non-negative.  Rays with a
// step of 2^1000 or more stay in FP64.
template <class Visit>
__device__ __forceinline__ int ray_walk(const Grid& g, Ray& r, int cap, Visit&& visit)
{
    constexpr uint64_t kLimit = 0x7E70000000000000ull;  // bit pattern of 2^1000
    int64_t cur = sub2ind(g, r.X, r.Y, r.Z);
    double tprev = r.tmin;
    int n = 1;
    constexpr uint64_t kMag = ~(1ull << 63);  // magnitude bits; NaN and infinity lie above kLimit
    const bool steps_ok = dbits(r.xd) < kLimit && dbits(r.yd) < kLimit && dbits(r.zd) < kLimit &&
                          (dbits(r.xt) & kMag) < kLimit && (dbits(r.yt) & kMag) < kLimit &&
                          (dbits(r.zt) & kMag) < kLimit;
    bool fp64 = !steps_ok || ((dbits(r.xt) | dbits(r.yt) | dbits(r.zt)) >> 63);
    while (r.X != r.xe || r.Y != r.ye || r.Z != r.ze) {
        if (n >= cap) return -1;
        // The reference's choice (:133-150): x if xt < yt and xt < zt, y if
        // yt <= xt and yt < zt, else z; made with selects so that the lanes of a
        // warp stepping along different axes share one add.
        bool sx, sy, pa;
        double t, tn;
        if (fp64) {
            const bool xy = r.xt < r.yt;
            const double a = xy ? r.xt : r.yt;
            pa = a < r.zt;
            sx = pa && xy;
            sy = pa && !xy;
            t = pa ? a : r.zt;
            tn = add64(t, sx ? r.xd : (sy ? r.yd : r.zd));
        } else {
            const uint64_t xb = dbits(r.xt), yb = dbits(r.yt), zb = dbits(r.zt);
            const bool xy = xb < yb;
            const uint64_t ab = xy ? xb : yb;
            pa = ab < zb;
            sx = pa && xy;
            sy = pa && !xy;
            const uint64_t tb = pa ? ab : zb;
            t = bitsd(tb);
            tn = bitsd(add_nonneg_bits(tb, dbits(sx ? r.xd : (sy ? r.yd : r.zd))));
        }
        r.xt = sx ? tn : r.xt;
        r.yt = sy ? tn : r.yt;
        r.zt = pa ? r.zt : tn;
        r.X += sx ? r.xs : 0;
        r.Y += sy ? r.ys : 0;
        r.Z += pa ? 0 : r.zs;
        fp64 = fp64 && (!steps_ok || ((dbits(r.xt) | dbits(r.yt) | dbits(r.zt)) >> 63));
        visit(n - 1, cur, tprev, t);
        tprev = t;
        cur = sub2ind(g, r.X, r.Y, r.Z);
        n += 1;
    }
    visit(n - 1, cur, tprev, r.tmax);
    return n;
}

// Segment length exactly as the reference evaluates it:
// sqrt((xv*t0 - xv*t1)^2 + (yv*t0 - yv*t1)^2 + (zv*t0 - zv*t1)^2)
// (RayTracing3DTOF.py:152-154, with the grid start replaced by xv*tMin at :127).
__device__ __forceinline__ double ref_length(const Ray& r, double t0, double t1)
{
    double dx = sub64(mul64(r.xv, t0), mul64(r.xv, t1));
    double dy = sub64(mul64(r.yv, t0), mul64(r.yv, t1));
    double dz = sub64(mul64(r.zv, t0), mul64(r.zv, t1));
    return __dsqrt_rn(add64(add64(mul64(dx, dx), mul64(dy, dy)), mul64(dz, dz)));
}

}  // namespace sss
