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
 * the same library calls as the reference.  The ray walk, the per-leg
 * integrals and the per-pair term live in orc_core.h, which the FP64 GPU
 * oracle (sss_oracle_gpu.cu) compiles too.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "orc_core.h"

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

/* A leg of the slice being simulated: its integrals and per-voxel values. */
typedef struct {
    orc_leg_stats s;
    double *a; /* act*len per voxel */
    double *r; /* sample distance per voxel */
} orc_leg;

int64_t orc_scatter_points(const orc_sss_problem *p, double *xyz, int64_t *slice)
{
    return orc_scatter_points_of(p, xyz, slice);
}

/* Compact output layout: out[b][(ri1*nru + ri2)][di1][di2] (di1 <= di2 used).
 * Returns 0 ok, <0 error (-2: TOF index out of table, -3: trace overflow). */
int orc_sss(const orc_sss_problem *p, double *out, int nthreads)
{
    const int64_t NRU = p->nru, NDU = p->ndu, B = p->nbins;
    const int64_t NL = NRU * NDU;
    const int64_t cap = p->nx + p->ny + p->nz;
    const int64_t ncell = NRU * NRU * NDU * NDU;
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

    const orc_pair_consts pc = orc_pair_consts_of(p, tof);

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
                int32_t *ix = (int32_t *)malloc(sizeof(int32_t) * cap);
                int st = orc_leg_trace(p, l / NDU, l % NDU, xS, yS, zS, (int)cap, legs[l].a, legs[l].r, ix, 1,
                                 &legs[l].s);
                if (st) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                    status = st;
                }
                free(ix);
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
                if (L1->s.att == 0) continue;
                const double *d1p = p->geom + 3 * (ring1 * p->nd + det1);
                double zD1 = p->geom[3 * (ring1 * p->nd) + 2];
                double *ab1 = (double *)malloc(sizeof(double) * B);
                double *ab2 = (double *)malloc(sizeof(double) * B);
                int pst = 0;
                for (int64_t ri2 = 0; ri2 < NRU; ++ri2) {
                    int64_t ring2 = p->rings[ri2];
                    double zD2 = p->geom[3 * (ring2 * p->nd) + 2];
                    for (int64_t di2 = 0; di2 < NDU; ++di2) {
                        int64_t det2 = p->dets[di2];
                        if ((det1 == det2 && ri2 == ri1) || det1 > det2) continue;
                        const orc_leg *L2 = &legs[ri2 * NDU + di2];
                        const double *d2p = p->geom + 3 * (ring2 * p->nd + det2);
                        double lor = (d1p[0] - d2p[0]) * (d1p[0] - d2p[0]) +
                                     (d1p[1] - d2p[1]) * (d1p[1] - d2p[1]) +
                                     (zD1 - zD2) * (zD1 - zD2);
                        int64_t cell = ((ri1 * NRU + ri2) * NDU + di1) * NDU + di2;
                        slice_cnt[cell] += orc_pair(&pc, &L1->s, L1->a, L1->r, &L2->s, L2->a, L2->r, 1, lor, ab1,
                                                    ab2, slice_sum + cell, ncell, &pst);
                    }
                }
                if (pst) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                    status = pst;
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
                    if (!orc_indices_ok(ix, n, grid[0] * grid[1] * grid[2], 1)) { status = -6; continue; }
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
                    if (!orc_indices_ok(ix, n, nvox, 1)) { status = -6; continue; }
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
                if (!orc_indices_ok(ix, n, grid[0] * grid[1] * grid[2], 1)) { status = -6; continue; }
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
                if (!orc_indices_ok(ix, n, nvox, 1)) { status = -6; continue; }
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
