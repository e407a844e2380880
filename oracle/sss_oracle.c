/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C, FP64 restatement of the openSSS (v1.0, Python) algorithms on the
 * TOF-SSS path.  It is the test oracle for the CUDA engine and the CPU baseline
 * timed by bench.py; the engine never links or calls it.  Every function
 * follows the reference's arithmetic step by step (IEEE FP64, no FMA
 * contraction: build with -ffp-contract=off) and cites the reference lines it
 * restates.  Differences from the reference that are deliberate:
 *   - the per-slice scatter accumulators are FP64 (the reference uses FP32,
 *     SingleScatterSimulationTOF.py:383-385), so this is the FP64 truth that
 *     the engine's error is stated against;
 *   - sums are sequential (numpy uses pairwise summation); both only change
 *     rounding in the last bits.
 * Tables that the reference builds with SciPy/NumPy (erf efficiency table,
 * TOF table, attenuation ratios) are inputs, built by the Python layer with
 * the same library calls as the reference.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_TIME_RANGE 4000
#define ORC_TOF_ENTRIES (2 * ORC_TIME_RANGE + 1)

/* Python's built-in min/max semantics (first argument wins unless the second
 * compares strictly smaller/larger), as used at RayTracing3DTOF.py:77-78. */
static inline double py_min(double a, double b) { return (b < a) ? b : a; }
static inline double py_max(double a, double b) { return (b > a) ? b : a; }

/* BoxIntersectTest, RayTracing3DTOF.py:204-269 (eps = 1e-20; the MEX
 * RayTracing3D.cpp:267 variant uses 1e-23).  Returns 1 on a hit. */
static int orc_box_intersect(const double *gb, const double *lc, double eps,
                             double *rtmin, double *rtmax)
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
 * writes up to cap entries of (length, 1-based linear index, sample).
 * Returns the voxel count, 0 for a miss, -1 if the traversal would exceed
 * cap (the reference would write past its Nx+Ny+Nz storage). */
int orc_trace(const int64_t *grid, const double *gb, const double *lc, double eps,
              double *len, int32_t *idx, double *samp, int cap)
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
        len[n - 1] = d;
        samp[n - 1] = prev + d / 2;
        prev = samp[n - 1];
        xs = xv * t;
        ys = yv * t;
        zs = zv * t;
        n += 1;
        idx[n - 1] = ORC_SUB2IND(X, Y, Z);
    }
    {
        double dx = xs - xv * tmax, dy = ys - yv * tmax, dz = zs - zv * tmax;
        double d = sqrt(dx * dx + dy * dy + dz * dz);
        len[n - 1] = d;
        samp[n - 1] = prev + d / 2;
    }
#undef ORC_SUB2IND
    return n;
}

/* Batched wrapper: rays [n][6] -> fixed-stride outputs [n][cap]. */
/* Linear indices past the volume (the reference's sub2ind uses Ny as the x
 * stride, so Nx != Ny volumes can produce them) make the reference's numpy
 * indexing raise IndexError; here they are status -6. */
static int orc_indices_ok(const int32_t *ix, int n, int64_t nvox)
{
    for (int k = 0; k < n; ++k)
        if (ix[k] < 1 || (int64_t)ix[k] > nvox) return 0;
    return 1;
}

int orc_trace_batch(const int64_t *grid, const double *gb, const double *lines, int64_t nrays,
                    double eps, int cap, int32_t *counts, double *len, int32_t *idx,
                    double *samp, int nthreads)
{
    int bad = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : bad)
#endif
    for (int64_t r = 0; r < nrays; ++r) {
        int c = orc_trace(grid, gb, lines + 6 * r, eps, len + r * cap, idx + r * cap,
                          samp + r * cap, cap);
        if (c < 0) bad += 1;
        counts[r] = c;
    }
    return bad;
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

typedef struct {
    double att;   /* exp(-sum mu*len) */
    double actv;  /* sum act*len */
    double sv;    /* |detector - scatter point| */
    double angle; /* incidence angle in degrees */
    int n;        /* voxels */
    double *a;    /* act*len per voxel */
    double *r;    /* sample distance per voxel */
} orc_leg;

/* Scatter points: z-major lattice, y then x, mu > 0
 * (SingleScatterSimulationTOF.py:182, 381, 387-394). */
int64_t orc_scatter_points(const orc_sss_problem *p, double *xyz, int64_t *slice)
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

static double orc_deg(double r) { return r * (180.0 / M_PI); }
static double orc_rad(double d) { return d * (M_PI / 180.0); }

/* CalcAngleScatter, SingleScatterSimulationTOF.py:216-235 */
static double orc_scatter_angle(double a, double b, double c)
{
    return 180 - orc_deg(acos((a + b - c) / (2 * sqrt(a * b))));
}

/* KleinNishina, SingleScatterSimulationTOF.py:239-258 */
static double orc_klein_nishina(double energy_j, double angle)
{
    const double me = 9.10938356E-31, c = 299792458.0;
    double gamma = energy_j / (me * (c * c));
    double ratio = 1.0 / (1.0 + gamma * (1.0 - cos(orc_rad(angle))));
    double s = sin(orc_rad(angle));
    return ratio * ratio * (ratio + 1 / ratio - s * s);
}

static int orc_tof_index(double v)
{
    /* SpatialOffset -> int32 then numpy fancy indexing (negative wraps) */
    int64_t i = (int64_t)v;
    if (i < 0) i += ORC_TOF_ENTRIES;
    if (i < 0 || i >= ORC_TOF_ENTRIES) return -1;
    return (int)i;
}

/* Compact output layout: out[b][(ri1*nru + ri2)][di1][di2] (di1 <= di2 used).
 * Returns 0 ok, <0 error (-2: TOF index out of table, -3: trace overflow). */
int orc_sss(const orc_sss_problem *p, double *out, int nthreads)
{
    const int64_t NRU = p->nru, NDU = p->ndu, B = p->nbins;
    const int64_t NL = NRU * NDU;
    const int64_t cap = p->nx + p->ny + p->nz;
    const double light = 299792458.0 * 1e-10;
    const double eref = (double)p->energy_ref;
    const double eref_j = 511.0E3 * 1.6E-19;
    const int64_t ncell = NRU * NRU * NDU * NDU;
    const double *IS = p->image_size;
    int64_t grid[3] = {p->nx, p->ny, p->nz};
    int status = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif

    int64_t nsp = orc_scatter_points(p, NULL, NULL);
    double *sxyz = (double *)malloc(sizeof(double) * 3 * (nsp > 0 ? nsp : 1));
    int64_t *sz = (int64_t *)malloc(sizeof(int64_t) * (nsp > 0 ? nsp : 1));
    orc_scatter_points(p, sxyz, sz);
    int64_t sb = p->sp_begin < 0 ? 0 : p->sp_begin;
    int64_t se = (p->sp_end < 0 || p->sp_end > nsp) ? nsp : p->sp_end;
    /* the points to use, in lattice order: a list, or the range [sb, se) */
    int64_t nsel = p->sp_list ? p->sp_count : (se > sb ? se - sb : 0);
    int64_t *sel = (int64_t *)malloc(sizeof(int64_t) * (nsel > 0 ? nsel : 1));
    for (int64_t k = 0; k < nsel; ++k) {
        sel[k] = p->sp_list ? p->sp_list[k] : sb + k;
        if (sel[k] < 0 || sel[k] >= nsp || (k > 0 && sel[k] <= sel[k - 1])) {
            free(sel);
            free(sxyz);
            free(sz);
            return -5; /* the list must be ascending point numbers */
        }
    }

    /* TOF table transposed to [t][b] for locality */
    double *tof = (double *)malloc(sizeof(double) * ORC_TOF_ENTRIES * B);
    for (int64_t b = 0; b < B; ++b)
        for (int64_t t = 0; t < ORC_TOF_ENTRIES; ++t)
            tof[t * B + b] = p->tof_table[b * ORC_TOF_ENTRIES + t];

    double *slice_sum = (double *)calloc((size_t)ncell * B, sizeof(double));
    double *slice_cnt = (double *)calloc((size_t)ncell, sizeof(double));
    orc_leg *legs = (orc_leg *)calloc((size_t)NL, sizeof(orc_leg));
    for (int64_t l = 0; l < NL; ++l) {
        legs[l].a = (double *)malloc(sizeof(double) * cap);
        legs[l].r = (double *)malloc(sizeof(double) * cap);
    }
    memset(out, 0, sizeof(double) * (size_t)ncell * B);

    const double ds = p->det_size[0] * p->det_size[1] * 1e-2;
    const double eff_ref = p->eff[p->energy_ref * 2 - 1];

    int64_t k = 0;
    while (k < nsel && status == 0) {
        int64_t zcur = sz[sel[k]];
        /* the slice accumulators are large (cells x bins): cleared in parallel */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t c = 0; c < ncell; ++c) {
            slice_cnt[c] = 0;
            for (int64_t b = 0; b < B; ++b) slice_sum[b * ncell + c] = 0;
        }
        for (; k < nsel && sz[sel[k]] == zcur && status == 0; ++k) {
            const int64_t s = sel[k];
            const double xS = sxyz[3 * s], yS = sxyz[3 * s + 1], zS = sxyz[3 * s + 2];
            /* legs: SingleScatterSimulationTOF.py:400-430 */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
            for (int64_t l = 0; l < NL; ++l) {
                int64_t ri = l / NDU, di = l % NDU;
                int64_t ring = p->rings[ri], det = p->dets[di];
                const double *dp = p->geom + 3 * (ring * p->nd + det);
                double zD = p->geom[3 * (ring * p->nd + 0) + 2];
                double lc[6] = {xS, yS, zS, dp[0], dp[1], zD};
                double *len = (double *)malloc(sizeof(double) * cap);
                int32_t *ix = (int32_t *)malloc(sizeof(int32_t) * cap);
                double *sm = (double *)malloc(sizeof(double) * cap);
                int n = orc_trace(grid, IS, lc, 1e-20, len, ix, sm, (int)cap);
                orc_leg *L = &legs[l];
                if (n < 0) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                    status = -3;
                    n = 0;
                } else if (!orc_indices_ok(ix, n, p->nx * p->ny * p->nz)) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                    status = -6;
                    n = 0;
                }
                double asum = 0, musum = 0;
                for (int k = 0; k < n; ++k) {
                    int64_t v = (int64_t)ix[k] - 1;
                    double a = (double)p->act[v] * len[k];
                    L->a[k] = a;
                    L->r[k] = sm[k];
                    asum += a;
                    musum += (double)p->mu[v] * len[k];
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
                L->sv = sqrt((dp[0] - xS) * (dp[0] - xS) + (dp[1] - yS) * (dp[1] - yS) +
                             (zD - zS) * (zD - zS));
                free(len);
                free(ix);
                free(sm);
            }
            if (status) break;
            /* pairs: SingleScatterSimulationTOF.py:433-553.  Parallel over leg 1:
             * pairs (l1, *) write disjoint cells. */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
            for (int64_t l1 = 0; l1 < NL; ++l1) {
                int64_t ri1 = l1 / NDU, di1 = l1 % NDU;
                int64_t ring1 = p->rings[ri1], det1 = p->dets[di1];
                const orc_leg *L1 = &legs[l1];
                if (L1->att == 0) continue;
                const double *d1p = p->geom + 3 * (ring1 * p->nd + det1);
                double zD1 = p->geom[3 * (ring1 * p->nd) + 2];
                double sv1 = L1->sv;
                double *ab1 = (double *)malloc(sizeof(double) * B);
                double *ab2 = (double *)malloc(sizeof(double) * B);
                for (int64_t ri2 = 0; ri2 < NRU; ++ri2) {
                    int64_t ring2 = p->rings[ri2];
                    double zD2 = p->geom[3 * (ring2 * p->nd) + 2];
                    for (int64_t di2 = 0; di2 < NDU; ++di2) {
                        int64_t det2 = p->dets[di2];
                        if ((det1 == det2 && ri2 == ri1) || det1 > det2) continue;
                        const orc_leg *L2 = &legs[ri2 * NDU + di2];
                        const double *d2p = p->geom + 3 * (ring2 * p->nd + det2);
                        double sv2 = L2->sv;
                        double lor = (d1p[0] - d2p[0]) * (d1p[0] - d2p[0]) +
                                     (d1p[1] - d2p[1]) * (d1p[1] - d2p[1]) +
                                     (zD1 - zD2) * (zD1 - zD2);
                        double cnt;
                        if (L2->att == 0 || (L1->actv == 0 && L2->actv == 0)) continue;
                        else if (L1->actv != 0 && L2->actv != 0) cnt = 2;
                        else cnt = 1;
                        double th = orc_scatter_angle(sv1 * sv1, sv2 * sv2, lor);
                        double es = floor(eref / (1 + (eref / 511.0) * (1 - cos(orc_rad(th)))) + 0.5);
                        int64_t ei = (int64_t)(es * 2) - 1;
                        if (ei < 0 || ei >= 2000) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                            status = -4;
                            continue;
                        }
                        double effp = p->eff[ei] * eff_ref;
                        if (effp == 0) continue;
                        double sc = p->ratio[ei];
                        double as1 = pow(L1->att, sc), as2 = pow(L2->att, sc);
                        for (int64_t b = 0; b < B; ++b) ab1[b] = ab2[b] = 0;
                        if (L1->actv != 0) {
                            for (int k = 0; k < L1->n; ++k) {
                                int ti = orc_tof_index(floor(2 * ((sv1 - sv2) / 2 - L1->r[k]) / light + 0.5) +
                                                       ORC_TIME_RANGE);
                                if (ti < 0) { status = -2; continue; }
                                const double *w = tof + (int64_t)ti * B;
                                for (int64_t b = 0; b < B; ++b) ab1[b] += L1->a[k] * w[b];
                            }
                        }
                        if (L2->actv != 0) {
                            for (int k = 0; k < L2->n; ++k) {
                                int ti = orc_tof_index(floor(2 * ((sv1 - sv2) / 2 + L2->r[k]) / light + 0.5) +
                                                       ORC_TIME_RANGE);
                                if (ti < 0) { status = -2; continue; }
                                const double *w = tof + (int64_t)ti * B;
                                for (int64_t b = 0; b < B; ++b) ab2[b] += L2->a[k] * w[b];
                            }
                        }
                        double geo = ((ds * ds) * fabs(cos(orc_rad(L1->angle)))) *
                                     (fabs(cos(orc_rad(L2->angle))) / (4 * M_PI * (sv1 * sv1) * (sv2 * sv2)));
                        double kn = orc_klein_nishina(eref_j, th);
                        double f = geo * effp * kn;
                        int64_t cell = ((ri1 * NRU + ri2) * NDU + di1) * NDU + di2;
                        for (int64_t b = 0; b < B; ++b) {
                            double pr = f * (L1->att * as2 * ab1[b] + L2->att * as1 * ab2[b]);
                            slice_sum[b * ncell + cell] += pr;
                        }
                        slice_cnt[cell] += cnt;
                    }
                }
                free(ab1);
                free(ab2);
            }
        }
        /* per-slice normalisation, NaN -> 0 (SingleScatterSimulationTOF.py:555-557);
         * cells are independent */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t c = 0; c < ncell; ++c) {
            double cn = slice_cnt[c];
            if (cn == 0) continue;
            for (int64_t b = 0; b < B; ++b) out[b * ncell + c] += slice_sum[b * ncell + c] / cn;
        }
    }

    for (int64_t l = 0; l < NL; ++l) {
        free(legs[l].a);
        free(legs[l].r);
    }
    free(legs);
    free(slice_sum);
    free(slice_cnt);
    free(tof);
    free(sxyz);
    free(sz);
    free(sel);
    return status;
}

/* ------------------------------------------------------------------------ */
/* MaskDetectors / MaskGenerator (TailsMask.py:84-228); `mu` is the activity
 * map when use_activity (the UseAttenuation=False rule).
 * out: uint8 [(nd+1)][nd/2][nr*nr], slice SinogramIndex[Ring1, Ring2]. */
int orc_mask(const int64_t *grid, const float *mu, const double *gb, int64_t nr, int64_t nd,
             const double *geom, const int16_t *lor, const int16_t *sino_index, int64_t af,
             int use_activity, uint8_t *out, int nthreads, double acf_below)
{
    const int64_t nang = nd / 2, nsino = nr * nr;
    const int cap = (int)(grid[0] + grid[1] + grid[2]);
    int status = 0;
    memset(out, 0, (size_t)(nd + 1) * nang * nsino);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t ring1 = 0; ring1 < nr; ++ring1) {
        double *len = (double *)malloc(sizeof(double) * cap);
        int32_t *ix = (int32_t *)malloc(sizeof(int32_t) * cap);
        double *sm = (double *)malloc(sizeof(double) * cap);
        double z1 = geom[3 * (ring1 * nd) + 2];
        for (int64_t d1 = 0; d1 < nd; d1 += af) {
            const double *p1 = geom + 3 * (ring1 * nd + d1);
            for (int64_t ring2 = 0; ring2 < nr; ++ring2) {
                double z2 = geom[3 * (ring2 * nd) + 2];
                for (int64_t d2 = 0; d2 < nd; d2 += af) {
                    if ((d1 == d2 && ring2 == ring1) || d1 > d2) continue;
                    const double *p2 = geom + 3 * (ring2 * nd + d2);
                    int64_t ang = lor[(d1 * nd + d2) * 2 + 0];
                    int64_t rad = lor[(d1 * nd + d2) * 2 + 1];
                    double lc[6] = {p1[0], p1[1], z1, p2[0], p2[1], z2};
                    int n = orc_trace(grid, gb, lc, 1e-20, len, ix, sm, cap);
                    double att;
                    if (n < 0) { status = -3; continue; }
                    if (!orc_indices_ok(ix, n, grid[0] * grid[1] * grid[2])) { status = -6; continue; }
                    if (n != 0) {
                        double s = 0;
                        for (int k = 0; k < n; ++k) s += (double)mu[ix[k] - 1] * len[k];
                        /* attenuation rule :145, activity rule :144 and :153-156 */
                        att = use_activity ? (s > 0 ? 0.0 : 1.0) : 1 / exp(-s);
                    } else {
                        att = 1;
                    }
                    /* the reference's tails (factor exactly 1), or a bound on the factor */
                    if (acf_below > 0 && !use_activity) att = att < acf_below ? 1 : 0;
                    else if (att != 1) att = 0;
                    int64_t sidx = sino_index[ring1 * nr + ring2];
                    uint8_t *cell = out + ((rad * nang + ang) * nsino + sidx);
                    *cell = (uint8_t)(*cell + (uint8_t)att);
                }
            }
        }
        free(len);
        free(ix);
        free(sm);
    }
    return status;
}

/* ------------------------------------------------------------------------ */
/* BackProjection + BackProjectionScatterRandFit (BackProjection.py:31-215).
 * prompts/scatters/randoms/mask: float32 [(nd+1)][nd/2][nr*nr]; the LOR from
 * (Ring1,d1) to (Ring2,d2) reads slice SinogramIndex[Ring2, Ring1]
 * (BackProjection.py:157-176 index with SinogramIndex.T).  Images are FP32
 * per Ring1 and summed in Ring1 order like the reference; the slope is
 * sum(x*T)/sum(x*x) in FP64 with x = float32(Sbp*1e10).
 * images (optional): 4 x grid voxels (P, S, R, sensitivity). */
int orc_fit(const int64_t *grid, const double *gb, int64_t nr, int64_t nd, const double *geom,
            const int16_t *lor, const int16_t *sino_index, int64_t af, const float *prompts,
            const float *scatters, const float *randoms, const float *mask, float *scale_out,
            float *images, int nthreads)
{
    const int64_t nang = nd / 2, nsino = nr * nr;
    const int64_t nvox = grid[0] * grid[1] * grid[2];
    const int cap = (int)(grid[0] + grid[1] + grid[2]);
    int status = 0;
    float *part = (float *)calloc((size_t)nr * 4 * nvox, sizeof(float));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t ring1 = 0; ring1 < nr; ++ring1) {
        float *iP = part + (size_t)ring1 * 4 * nvox, *iS = iP + nvox, *iR = iS + nvox, *iN = iR + nvox;
        double *len = (double *)malloc(sizeof(double) * cap);
        int32_t *ix = (int32_t *)malloc(sizeof(int32_t) * cap);
        double *sm = (double *)malloc(sizeof(double) * cap);
        double z1 = geom[3 * (ring1 * nd) + 2];
        for (int64_t d1 = 0; d1 < nd; d1 += af) {
            const double *p1 = geom + 3 * (ring1 * nd + d1);
            for (int64_t ring2 = 0; ring2 < nr; ++ring2) {
                double z2 = geom[3 * (ring2 * nd) + 2];
                int64_t sidx = sino_index[ring2 * nr + ring1];
                for (int64_t d2 = 0; d2 < nd; d2 += af) {
                    if ((d1 == d2 && ring2 == ring1) || d1 > d2) continue;
                    int64_t ang = lor[(d1 * nd + d2) * 2 + 0];
                    int64_t rad = lor[(d1 * nd + d2) * 2 + 1];
                    size_t c = (size_t)((rad * nang + ang) * nsino + sidx);
                    float m = mask[c];
                    float sv = m * scatters[c];
                    if (sv == 0) continue;
                    float pv = m * prompts[c], rv = m * randoms[c];
                    const double *p2 = geom + 3 * (ring2 * nd + d2);
                    double lc[6] = {p1[0], p1[1], z1, p2[0], p2[1], z2};
                    int n = orc_trace(grid, gb, lc, 1e-20, len, ix, sm, cap);
                    if (n < 0) { status = -3; continue; }
                    if (!orc_indices_ok(ix, n, nvox)) { status = -6; continue; }
                    if (n > 0) {
                        float fn = (float)n;
                        float ap = pv / fn, as = sv / fn, ar = rv / fn;
                        for (int k = 0; k < n; ++k) {
                            int64_t v = ix[k] - 1;
                            iP[v] = iP[v] + ap;
                            iS[v] = iS[v] + as;
                            iR[v] = iR[v] + ar;
                            iN[v] = iN[v] + 1.0f;
                        }
                    }
                }
            }
        }
        free(len);
        free(ix);
        free(sm);
    }
    float *tot = (float *)calloc((size_t)4 * nvox, sizeof(float));
    for (int64_t ring1 = 0; ring1 < nr; ++ring1) {
        const float *src = part + (size_t)ring1 * 4 * nvox;
        for (int64_t i = 0; i < 4 * nvox; ++i) tot[i] = tot[i] + src[i];
    }
    double sxt = 0, sxx = 0;
    for (int64_t v = 0; v < nvox; ++v) {
        float sens = tot[3 * nvox + v];
        float sb = tot[nvox + v] / sens;
        float ab = tot[v] / sens;
        float rb = tot[2 * nvox + v] / sens;
        if (isnan(sb) || isinf(sb)) sb = 0;
        if (isnan(ab) || isinf(ab)) ab = 0;
        if (isnan(rb) || isinf(rb)) rb = 0;
        float tl = ab - rb;
        if (tl < 0) tl = 0;
        float x = (float)((double)sb * 1e10);
        sxt += (double)x * (double)tl;
        sxx += (double)x * (double)x;
    }
    double a = (sxx > 0) ? sxt / sxx : 0.0;
    *scale_out = (float)((double)(float)a * 1e10);
    if (images) memcpy(images, tot, sizeof(float) * 4 * nvox);
    free(tot);
    free(part);
    return status;
}

/* ------------------------------------------------------------------------ */
/* Span variants: MaskDetectorsMashing (TailsMask.py:230-309) and
 * BackProjectionMashing + BackProjectionScatterRandFitMashing
 * (BackProjection.py:217-393).  Each mashed sinogram i is traced at the ring
 * pair pairs[3i], pairs[3i+1] of the expanded geometry `geom` (nr rings) and
 * reads / writes slice pairs[3i+2] of [(nd+1)][nd/2][nslices] sinograms.  The
 * back-projection weights each voxel by len / sum(len) (:294-297) and the
 * per-sinogram images are summed in sinogram order (:381-385). */
int orc_mask_pairs(const int64_t *grid, const float *mu, const double *gb, int64_t nr, int64_t nd,
                   const double *geom, const int16_t *lor, const int32_t *pairs, int64_t npairs,
                   int64_t nslices, int64_t af, int use_activity, uint8_t *out, int nthreads,
                   double acf_below)
{
    const int64_t nang = nd / 2;
    const int cap = (int)(grid[0] + grid[1] + grid[2]);
    int status = 0;
    memset(out, 0, (size_t)(nd + 1) * nang * nslices);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t i = 0; i < npairs; ++i) {
        const int64_t ring1 = pairs[3 * i], ring2 = pairs[3 * i + 1], slice = pairs[3 * i + 2];
        double *len = (double *)malloc(sizeof(double) * cap);
        int32_t *ix = (int32_t *)malloc(sizeof(int32_t) * cap);
        double *sm = (double *)malloc(sizeof(double) * cap);
        const double z1 = geom[3 * (ring1 * nd) + 2], z2 = geom[3 * (ring2 * nd) + 2];
        for (int64_t d1 = 0; d1 < nd; d1 += af) {
            const double *p1 = geom + 3 * (ring1 * nd + d1);
            for (int64_t d2 = 0; d2 < nd; d2 += af) {
                if ((d1 == d2 && ring2 == ring1) || d1 > d2) continue;
                const double *p2 = geom + 3 * (ring2 * nd + d2);
                int64_t ang = lor[(d1 * nd + d2) * 2 + 0];
                int64_t rad = lor[(d1 * nd + d2) * 2 + 1];
                double lc[6] = {p1[0], p1[1], z1, p2[0], p2[1], z2};
                int n = orc_trace(grid, gb, lc, 1e-20, len, ix, sm, cap);
                if (n < 0) { status = -3; continue; }
                if (!orc_indices_ok(ix, n, grid[0] * grid[1] * grid[2])) { status = -6; continue; }
                double att = 1;
                if (n != 0) {
                    double s = 0;
                    for (int k = 0; k < n; ++k) s += (double)mu[ix[k] - 1] * len[k];
                    att = use_activity ? (s > 0 ? 0.0 : 1.0) : 1 / exp(-s);  /* :289-301 */
                }
                if (acf_below > 0 && !use_activity) att = att < acf_below ? 1 : 0;
                else if (att != 1) att = 0;
                uint8_t *cell = out + ((rad * nang + ang) * nslices + slice);
                *cell = (uint8_t)(*cell + (uint8_t)att);
            }
        }
        free(len);
        free(ix);
        free(sm);
    }
    return status;
}

int orc_fit_pairs(const int64_t *grid, const double *gb, int64_t nr, int64_t nd, const double *geom,
                  const int16_t *lor, const int32_t *pairs, int64_t npairs, int64_t nslices, int64_t af,
                  const float *prompts, const float *scatters, const float *randoms, const float *mask,
                  float *scale_out, int nthreads)
{
    const int64_t nang = nd / 2;
    const int64_t nvox = grid[0] * grid[1] * grid[2];
    const int cap = (int)(grid[0] + grid[1] + grid[2]);
    int status = 0;
    float *part = (float *)calloc((size_t)npairs * 4 * nvox, sizeof(float));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t i = 0; i < npairs; ++i) {
        const int64_t ring1 = pairs[3 * i], ring2 = pairs[3 * i + 1], slice = pairs[3 * i + 2];
        float *iP = part + (size_t)i * 4 * nvox, *iS = iP + nvox, *iR = iS + nvox, *iN = iR + nvox;
        double *len = (double *)malloc(sizeof(double) * cap);
        int32_t *ix = (int32_t *)malloc(sizeof(int32_t) * cap);
        double *sm = (double *)malloc(sizeof(double) * cap);
        const double z1 = geom[3 * (ring1 * nd) + 2], z2 = geom[3 * (ring2 * nd) + 2];
        for (int64_t d1 = 0; d1 < nd; d1 += af) {
            const double *p1 = geom + 3 * (ring1 * nd + d1);
            for (int64_t d2 = 0; d2 < nd; d2 += af) {
                if ((d1 == d2 && ring2 == ring1) || d1 > d2) continue;
                int64_t ang = lor[(d1 * nd + d2) * 2 + 0];
                int64_t rad = lor[(d1 * nd + d2) * 2 + 1];
                size_t c = (size_t)((rad * nang + ang) * nslices + slice);
                float m = mask[c];
                float sv = m * scatters[c];
                if (sv == 0) continue;
                float pv = m * prompts[c], rv = m * randoms[c];
                const double *p2 = geom + 3 * (ring2 * nd + d2);
                double lc[6] = {p1[0], p1[1], z1, p2[0], p2[1], z2};
                int n = orc_trace(grid, gb, lc, 1e-20, len, ix, sm, cap);
                if (n < 0) { status = -3; continue; }
                if (!orc_indices_ok(ix, n, nvox)) { status = -6; continue; }
                if (n > 0) {
                    /* value * Lengths / np.sum(Lengths) in FP64, added to the FP32
                     * image and rounded back (numpy sums pairwise; the sequential
                     * sum differs from it in the last bits only) */
                    double total = 0;
                    for (int k = 0; k < n; ++k) total += len[k];
                    for (int k = 0; k < n; ++k) {
                        int64_t v = ix[k] - 1;
                        iP[v] = (float)((double)iP[v] + (double)pv * len[k] / total);
                        iS[v] = (float)((double)iS[v] + (double)sv * len[k] / total);
                        iR[v] = (float)((double)iR[v] + (double)rv * len[k] / total);
                        iN[v] = iN[v] + 1.0f;
                    }
                }
            }
        }
        free(len);
        free(ix);
        free(sm);
    }
    float *tot = (float *)calloc((size_t)4 * nvox, sizeof(float));
    for (int64_t i = 0; i < npairs; ++i) {
        const float *src = part + (size_t)i * 4 * nvox;
        for (int64_t k = 0; k < 4 * nvox; ++k) tot[k] = tot[k] + src[k];
    }
    double sxt = 0, sxx = 0;
    for (int64_t v = 0; v < nvox; ++v) {
        /* S / (sens + 1e-15) in float32 (:358-369): the 1e-15 only matters where sens is 0 */
        float sens = tot[3 * nvox + v] + 1e-15f;
        float sb = tot[nvox + v] / sens;
        float ab = tot[v] / sens;
        float rb = tot[2 * nvox + v] / sens;
        if (isnan(sb) || isinf(sb)) sb = 0;
        if (isnan(ab) || isinf(ab)) ab = 0;
        if (isnan(rb) || isinf(rb)) rb = 0;
        float tl = ab - rb;
        if (tl < 0) tl = 0;
        float x = (float)((double)sb * 1e10);
        sxt += (double)x * (double)tl;
        sxx += (double)x * (double)x;
    }
    double a = (sxx > 0) ? sxt / sxx : 0.0;
    *scale_out = (float)((double)(float)a * 1e10);
    free(tot);
    free(part);
    return status;
}

/* InterpolateAllBins gather (Interpolation.py:197-319) given the nearest
 * source tables: lut[rad*nang+ang] = griddata point index p (p = a*ndu + b,
 * a/b indexing the sampled detectors of the two rings), ringmap[r] = nearest
 * sampled ring index.  sampled: compact [b][(ri1*nru+ri2)][di1][di2].
 * out (one bin): [(nd+1)][nd/2][nr*nr], slice s = SinogramIndex[r1, r2]. */
void orc_upsample_bin(const double *sampled_bin, int64_t nru, int64_t ndu, int64_t nr, int64_t nd,
                      const int32_t *lut, const int32_t *ringmap, const int16_t *sino_index,
                      float *out)
{
    const int64_t nang = nd / 2, nsino = nr * nr;
    for (int64_t rad = 0; rad <= nd; ++rad)
        for (int64_t ang = 0; ang < nang; ++ang) {
            int32_t pidx = lut[rad * nang + ang];
            int64_t a = pidx / ndu, b = pidx % ndu;
            int64_t lo = a < b ? a : b, hi = a < b ? b : a;
            for (int64_t r1 = 0; r1 < nr; ++r1)
                for (int64_t r2 = 0; r2 < nr; ++r2) {
                    int64_t src = ((ringmap[r1] * nru + ringmap[r2]) * ndu + lo) * ndu + hi;
                    int64_t s = sino_index[r1 * nr + r2];
                    out[(rad * nang + ang) * nsino + s] = (float)sampled_bin[src];
                }
        }
}
