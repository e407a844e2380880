/*
 * ORACLE — test infrastructure, not product code.
 *
 * The FP64 arithmetic that the C restatement (sss_oracle.c, host cores) and
 * the FP64 GPU oracle (sss_oracle_gpu.cu) share: the reference's ray walk,
 * the per-leg integrals and the per-pair scatter term of
 * SingleScatterSimulationTOF.  Written once, so that both oracles evaluate
 * the same operations in the same order; each is built without multiply-add
 * contraction (gcc -ffp-contract=off, nvcc -fmad=false), so they differ only
 * where the host's and the device's exp/pow/acos/cos/sin round differently
 * (an ulp or two).
 */
#ifndef ORC_CORE_H
#define ORC_CORE_H

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define ORC_FN static __host__ __device__ inline
#else
#define ORC_FN static inline
#endif

#define ORC_TIME_RANGE 4000
#define ORC_TOF_ENTRIES (2 * ORC_TIME_RANGE + 1)

/* Python's built-in min/max semantics (first argument wins unless the second
 * compares strictly smaller/larger), as used at RayTracing3DTOF.py:77-78. */
ORC_FN double py_min(double a, double b) { return (b < a) ? b : a; }
ORC_FN double py_max(double a, double b) { return (b > a) ? b : a; }

/* BoxIntersectTest, RayTracing3DTOF.py:204-269 (eps = 1e-20; the MEX
 * RayTracing3D.cpp:267 variant uses 1e-23).  Returns 1 on a hit. */
ORC_FN int orc_box_intersect(const double *gb, const double *lc, double eps, double *rtmin, double *rtmax)
{
    double tmin, tmax, ytmin, ytmax, ztmin, ztmax;
    double xdiv = 1.0 / (lc[3] - lc[0] + eps);
    if (xdiv >= 0) {
        tmin = (gb[0] - lc[0]) * xdiv;
        tmax = (gb[3] - lc[0]) * xdiv;
    } else {
        tmin = (gb[3] - lc[0]) * xdiv;
        tmax = (gb[0] - lc[0]) * xdiv;
    }
    double ydiv = 1.0 / (lc[4] - lc[1] + eps);
    if (ydiv >= 0) {
        ytmin = (gb[1] - lc[1]) * ydiv;
        ytmax = (gb[4] - lc[1]) * ydiv;
    } else {
        ytmin = (gb[4] - lc[1]) * ydiv;
        ytmax = (gb[1] - lc[1]) * ydiv;
    }
    if (tmin > ytmax || ytmin > tmax) return 0;
    if (ytmin > tmin) tmin = ytmin;
    if (ytmax < tmax) tmax = ytmax;
    double zdiv = 1.0 / (lc[5] - lc[2] + eps);
    if (zdiv >= 0) {
        ztmin = (gb[2] - lc[2]) * zdiv;
        ztmax = (gb[5] - lc[2]) * zdiv;
    } else {
        ztmin = (gb[5] - lc[2]) * zdiv;
        ztmax = (gb[2] - lc[2]) * zdiv;
    }
    if (tmin > ztmax || ztmin > tmax) return 0;
    if (ztmin > tmin) tmin = ztmin;
    if (ztmax < tmax) tmax = ztmax;
    if ((tmin >= 1 && tmax >= 1) || (tmin <= 0 && tmax <= 0)) return 0;
    *rtmin = tmin;
    *rtmax = tmax;
    return 1;
}

/* RayTracing3DTOF, RayTracing3DTOF.py:29-180.  grid = [Nx, Ny, Nz];
 * writes up to cap entries of (length, 1-based linear index, sample), entry k
 * at k * stride.  Returns the voxel count, 0 for a miss, -1 if the traversal
 * would exceed cap (the reference would write past its Nx+Ny+Nz storage). */
ORC_FN int orc_trace_strided(const int64_t *grid, const double *gb, const double *lc, double eps, double *len,
                             int32_t *idx, double *samp, int cap, int64_t stride)
{
    double tmin, tmax;
    if (!orc_box_intersect(gb, lc, eps, &tmin, &tmax)) return 0;
    tmin = py_max(tmin, 0.0);
    tmax = py_min(tmax, 1.0);
    const double n0 = (double)grid[0], n1 = (double)grid[1], n2 = (double)grid[2];
    double vx = (gb[3] - gb[0]) / n0;
    double vy = (gb[4] - gb[1]) / n1;
    double vz = (gb[5] - gb[2]) / n2;
    double xv = lc[3] - lc[0], yv = lc[4] - lc[1], zv = lc[5] - lc[2];
    double xs = lc[0] + xv * tmin, ys = lc[1] + yv * tmin, zs = lc[2] + zv * tmin;
    double xe = lc[0] + xv * tmax, ye = lc[1] + yv * tmax, ze = lc[2] + zv * tmax;

    double X = py_max(1.0, py_min(n0, ceil((xs - gb[0]) / vx)));
    double xend = py_max(1.0, py_min(n0, ceil((xe - gb[0]) / vx)));
    double xstep, xdelta, xtmax;
    if (xv > 0) { xstep = 1; xdelta = vx / xv; xtmax = tmin + (gb[0] + X * vx - xs) / xv; }
    else if (xv < 0) { xstep = -1; xdelta = vx / -xv; xtmax = tmin + (gb[0] + (X - 1) * vx - xs) / xv; }
    else { xstep = 0; xtmax = tmax; xdelta = tmax; }

    double Y = py_max(1.0, py_min(n1, ceil((ys - gb[1]) / vy)));
    double yend = py_max(1.0, py_min(n1, ceil((ye - gb[1]) / vy)));
    double ystep, ydelta, ytmax;
    if (yv > 0) { ystep = 1; ydelta = vy / yv; ytmax = tmin + (gb[1] + Y * vy - ys) / yv; }
    else if (yv < 0) { ystep = -1; ydelta = vy / -yv; ytmax = tmin + (gb[1] + (Y - 1) * vy - ys) / yv; }
    else { ystep = 0; ytmax = tmax; ydelta = tmax; }

    /* Z goes through int() first (RayTracing3DTOF.py:109-110) */
    double Z = (double)(int64_t)ceil((zs - gb[2]) / vz);
    Z = py_min(py_max(1.0, Z), n2);
    double zend = (double)(int64_t)ceil((ze - gb[2]) / vz);
    zend = py_min(py_max(1.0, zend), n2);
    double zstep, zdelta, ztmax;
    if (zv > 0) { zstep = 1; zdelta = vz / zv; ztmax = tmin + (gb[2] + Z * vz - zs) / zv; }
    else if (zv < 0) { zstep = -1; zdelta = vz / -zv; ztmax = tmin + (gb[2] + (Z - 1) * vz - zs) / zv; }
    else { zstep = 0; ztmax = tmax; zdelta = tmax; }

    /* sub2ind, RayTracing3DTOF.py:202: X + (Y-1)*Ny + (Z-1)*Ny*Nx */
#define ORC_SUB2IND(x, y, z) ((int32_t)((x) + ((y) - 1) * n1 + ((z) - 1) * n1 * n0))
    if (cap < 1) return -1;
    idx[0] = ORC_SUB2IND(X, Y, Z);
    int n = 1;
    xs = xv * tmin;
    ys = yv * tmin;
    zs = zv * tmin;
    double prev = 0.0, t;
    while (X != xend || Y != yend || Z != zend) {
        if (xtmax < ytmax) {
            if (xtmax < ztmax) { X += xstep; t = xtmax; xtmax += xdelta; }
            else { Z += zstep; t = ztmax; ztmax += zdelta; }
        } else {
            if (ytmax < ztmax) { Y += ystep; t = ytmax; ytmax += ydelta; }
            else { Z += zstep; t = ztmax; ztmax += zdelta; }
        }
        if (n >= cap) return -1;
        double dx = xs - xv * t, dy = ys - yv * t, dz = zs - zv * t;
        double d = sqrt(dx * dx + dy * dy + dz * dz);
        len[(n - 1) * stride] = d;
        samp[(n - 1) * stride] = prev + d / 2;
        prev = samp[(n - 1) * stride];
        xs = xv * t;
        ys = yv * t;
        zs = zv * t;
        n += 1;
        idx[(n - 1) * stride] = ORC_SUB2IND(X, Y, Z);
    }
    {
        double dx = xs - xv * tmax, dy = ys - yv * tmax, dz = zs - zv * tmax;
        double d = sqrt(dx * dx + dy * dy + dz * dz);
        len[(n - 1) * stride] = d;
        samp[(n - 1) * stride] = prev + d / 2;
    }
#undef ORC_SUB2IND
    return n;
}

ORC_FN int orc_trace(const int64_t *grid, const double *gb, const double *lc, double eps, double *len,
                     int32_t *idx, double *samp, int cap)
{
    return orc_trace_strided(grid, gb, lc, eps, len, idx, samp, cap, 1);
}

/* Linear indices past the volume (the reference's sub2ind uses Ny as the x
 * stride, so Nx != Ny volumes can produce them) make the reference's numpy
 * indexing raise IndexError; here they are status -6. */
ORC_FN int orc_indices_ok(const int32_t *ix, int n, int64_t nvox, int64_t stride)
{
    for (int k = 0; k < n; ++k)
        if (ix[k * stride] < 1 || (int64_t)ix[k * stride] > nvox) return 0;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* SingleScatterSimulationTOF (SingleScatterSimulationTOF.py:36-208, 301-559) */

typedef struct {
    int64_t nx, ny, nz;
    const float *act;          /* Fortran-order flat [nx*ny*nz] */
    const float *mu;
    const double *image_size;  /* [6] cm */
    int64_t nr, nd;
    const double *geom;        /* [nr][nd][3] cm */
    const double *normals;     /* [nr][nd][3] */
    const double *det_size;    /* [2] mm */
    int64_t nru, ndu;
    const int64_t *rings;      /* [nru] ring numbers */
    const int64_t *dets;       /* [ndu] detector numbers */
    int64_t step[3];
    int64_t nbins;
    const double *tof_table;   /* [nbins][8001] */
    const double *eff;         /* [2000] efficiency column */
    const double *ratio;       /* [2000] water mu(E)/mu(511) */
    int64_t energy_ref;        /* 511 */
    int64_t sp_begin, sp_end;  /* scatter-point range in lattice order; end<0: all */
    const int64_t *sp_list;    /* NULL, or sp_count ascending scatter-point numbers (lattice
                                  order) to use instead of the range */
    int64_t sp_count;
} orc_sss_problem;

/* Scatter points: z-major lattice, y then x, mu > 0
 * (SingleScatterSimulationTOF.py:182, 381, 387-394).  Host only. */
static inline int64_t orc_scatter_points_of(const orc_sss_problem *p, double *xyz, int64_t *slice)
{
    const double *IS = p->image_size;
    double zvox = (IS[5] - IS[2]) / (double)p->nz;
    double width = -IS[2], radius = -IS[0];
    double zstart = zvox / 2 - width;
    int64_t count = 0;
    for (int64_t z = 0; z < p->nz; z += p->step[2]) {
        double zs = zstart + z * zvox;
        for (int64_t y = 0; y < p->ny; y += p->step[1]) {
            double ys = ((y + 1) * 2 * radius / p->ny) - radius;
            for (int64_t x = 0; x < p->nx; x += p->step[0]) {
                if (p->mu[x + p->nx * (y + p->ny * z)] > 0) {
                    if (xyz) {
                        xyz[3 * count + 0] = ((x + 1) * 2 * radius / p->nx) - radius;
                        xyz[3 * count + 1] = ys;
                        xyz[3 * count + 2] = zs;
                        slice[count] = z;
                    }
                    count += 1;
                }
            }
        }
    }
    return count;
}

ORC_FN double orc_deg(double r) { return r * (180.0 / M_PI); }
ORC_FN double orc_rad(double d) { return d * (M_PI / 180.0); }

/* CalcAngleScatter, SingleScatterSimulationTOF.py:216-235 */
ORC_FN double orc_scatter_angle(double a, double b, double c)
{
    return 180 - orc_deg(acos((a + b - c) / (2 * sqrt(a * b))));
}

/* KleinNishina, SingleScatterSimulationTOF.py:239-258 */
ORC_FN double orc_klein_nishina(double energy_j, double angle)
{
    const double me = 9.10938356E-31, c = 299792458.0;
    double gamma = energy_j / (me * (c * c));
    double ratio = 1.0 / (1.0 + gamma * (1.0 - cos(orc_rad(angle))));
    double s = sin(orc_rad(angle));
    return ratio * ratio * (ratio + 1 / ratio - s * s);
}

ORC_FN int orc_tof_index(double v)
{
    /* SpatialOffset -> int32 then numpy fancy indexing (negative wraps) */
    int64_t i = (int64_t)v;
    if (i < 0) i += ORC_TOF_ENTRIES;
    if (i < 0 || i >= ORC_TOF_ENTRIES) return -1;
    return (int)i;
}

/* One leg's integrals. */
typedef struct {
    double att;   /* exp(-sum mu*len) */
    double actv;  /* sum act*len */
    double sv;    /* |detector - scatter point| */
    double angle; /* incidence angle in degrees */
    int n;        /* voxels */
} orc_leg_stats;

/* The leg from scatter point (xS, yS, zS) to sampled crystal (ri, di)
 * (SingleScatterSimulationTOF.py:400-430): a[k * stride] = activity x length
 * and r[k * stride] = sample distance of its k-th voxel (ix is scratch for
 * the voxel numbers), and the leg's integrals in *L.  Returns 0, or -3 for a
 * walk past cap voxels and -6 for a voxel number past the volume, the leg
 * then being empty. */
ORC_FN int orc_leg_trace(const orc_sss_problem *p, int64_t ri, int64_t di, double xS, double yS, double zS, int cap,
                   double *a, double *r, int32_t *ix, int64_t stride, orc_leg_stats *L)
{
    const int64_t ring = p->rings[ri], det = p->dets[di];
    const double *dp = p->geom + 3 * (ring * p->nd + det);
    const double zD = p->geom[3 * (ring * p->nd + 0) + 2];
    const double lc[6] = {xS, yS, zS, dp[0], dp[1], zD};
    const int64_t grid[3] = {p->nx, p->ny, p->nz};
    int st = 0;
    int n = orc_trace_strided(grid, p->image_size, lc, 1e-20, a, ix, r, cap, stride);
    if (n < 0) {
        st = -3;
        n = 0;
    } else if (!orc_indices_ok(ix, n, p->nx * p->ny * p->nz, stride)) {
        st = -6;
        n = 0;
    }
    double asum = 0, musum = 0;
    for (int k = 0; k < n; ++k) {
        const int64_t v = (int64_t)ix[k * stride] - 1;
        const double len = a[k * stride];
        const double av = (double)p->act[v] * len;
        a[k * stride] = av;
        asum += av;
        musum += (double)p->mu[v] * len;
    }
    L->n = n;
    L->actv = asum;
    L->att = exp(-musum);
    double v3[3] = {dp[0] - xS, dp[1] - yS, zD - zS};
    const double *nv = p->normals + 3 * (ring * p->nd + det);
    double dot = v3[0] * nv[0] + v3[1] * nv[1] + v3[2] * nv[2];
    double nn = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
    double vn = sqrt(v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2]);
    L->angle = fabs(orc_deg(acos(dot / (nn * vn))));
    L->sv = sqrt((dp[0] - xS) * (dp[0] - xS) + (dp[1] - yS) * (dp[1] - yS) + (zD - zS) * (zD - zS));
    return st;
}

/* Per-problem constants of the pair terms. */
typedef struct {
    double eref, eref_j, eff_ref, ds, light;
    int64_t nbins;
    const double *tof; /* [8001][nbins]: the TOF table transposed, a row per offset */
    const double *eff, *ratio;
} orc_pair_consts;

static inline orc_pair_consts orc_pair_consts_of(const orc_sss_problem *p, const double *tof_rows)
{
    orc_pair_consts c;
    c.eref = (double)p->energy_ref;
    c.eref_j = 511.0E3 * 1.6E-19;
    c.eff_ref = p->eff[p->energy_ref * 2 - 1];
    c.ds = p->det_size[0] * p->det_size[1] * 1e-2;
    c.light = 299792458.0 * 1e-10;
    c.nbins = p->nbins;
    c.tof = tof_rows;
    c.eff = p->eff;
    c.ratio = p->ratio;
    return c;
}

/* One detector pair at one scatter point (SingleScatterSimulationTOF.py:433-553):
 * legs L1 and L2 with their voxel values a and samples r (entry k at
 * k * stride) and the squared crystal distance lor.  Adds the pair's term of
 * every bin b to sum[b * bstride] and returns the pair's count (2, or 1 when
 * one leg carries no activity), or 0 for a pair the reference skips.  ab1 and
 * ab2 are nbins doubles of scratch.  An energy row outside the tables sets
 * *status = -4, a TOF index outside the table -2. */
ORC_FN double orc_pair(const orc_pair_consts *c, const orc_leg_stats *L1, const double *a1, const double *r1,
                       const orc_leg_stats *L2, const double *a2, const double *r2, int64_t stride, double lor,
                       double *ab1, double *ab2, double *sum, int64_t bstride, int *status)
{
    const double sv1 = L1->sv, sv2 = L2->sv;
    double cnt;
    if (L2->att == 0 || (L1->actv == 0 && L2->actv == 0)) return 0;
    else if (L1->actv != 0 && L2->actv != 0) cnt = 2;
    else cnt = 1;
    double th = orc_scatter_angle(sv1 * sv1, sv2 * sv2, lor);
    double es = floor(c->eref / (1 + (c->eref / 511.0) * (1 - cos(orc_rad(th)))) + 0.5);
    int64_t ei = (int64_t)(es * 2) - 1;
    if (ei < 0 || ei >= 2000) {
        *status = -4;
        return 0;
    }
    double effp = c->eff[ei] * c->eff_ref;
    if (effp == 0) return 0;
    double sc = c->ratio[ei];
    double as1 = pow(L1->att, sc), as2 = pow(L2->att, sc);
    const int64_t B = c->nbins;
    for (int64_t b = 0; b < B; ++b) ab1[b] = ab2[b] = 0;
    if (L1->actv != 0) {
        for (int k = 0; k < L1->n; ++k) {
            int ti = orc_tof_index(floor(2 * ((sv1 - sv2) / 2 - r1[k * stride]) / c->light + 0.5) + ORC_TIME_RANGE);
            if (ti < 0) {
                *status = -2;
                continue;
            }
            const double *w = c->tof + (int64_t)ti * B;
            for (int64_t b = 0; b < B; ++b) ab1[b] += a1[k * stride] * w[b];
        }
    }
    if (L2->actv != 0) {
        for (int k = 0; k < L2->n; ++k) {
            int ti = orc_tof_index(floor(2 * ((sv1 - sv2) / 2 + r2[k * stride]) / c->light + 0.5) + ORC_TIME_RANGE);
            if (ti < 0) {
                *status = -2;
                continue;
            }
            const double *w = c->tof + (int64_t)ti * B;
            for (int64_t b = 0; b < B; ++b) ab2[b] += a2[k * stride] * w[b];
        }
    }
    double geo = ((c->ds * c->ds) * fabs(cos(orc_rad(L1->angle)))) *
                 (fabs(cos(orc_rad(L2->angle))) / (4 * M_PI * (sv1 * sv1) * (sv2 * sv2)));
    double kn = orc_klein_nishina(c->eref_j, th);
    double f = geo * effp * kn;
    for (int64_t b = 0; b < B; ++b) {
        double pr = f * (L1->att * as2 * ab1[b] + L2->att * as1 * ab2[b]);
        sum[b * bstride] += pr;
    }
    return cnt;
}

#endif
