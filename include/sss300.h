/*
 * sss300 — C ABI of the GB300 (sm_103a) TOF single-scatter-simulation engine.
 *
 * Plain C: integers, doubles and raw pointers.  "device" pointers are CUDA
 * global-memory addresses on the current device (e.g. torch.Tensor.data_ptr()),
 * "host" pointers are ordinary process memory.  `stream` is a cudaStream_t
 * passed as void* (NULL = the legacy default stream).  Every call returns 0 on
 * success or an SSS_ERR_* code and never throws; sss_last_error() gives a
 * thread-local message.  Kernels report data-dependent failures by OR-ing bits
 * into a caller-owned device status word (int32, zeroed by the caller); map it
 * with sss_status_code() after synchronising the stream.
 *
 * Each entry point cites the reference interface it replaces
 * (openSSS v1.0, paths relative to the reference project root).
 */
#ifndef SSS300_H
#define SSS300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SSS300_ABI_VERSION 7

enum {
    SSS_OK = 0,
    SSS_ERR_INVALID = 1,    /* bad argument (shape, null pointer, range) */
    SSS_ERR_CUDA = 2,       /* a CUDA runtime call failed */
    SSS_ERR_OVERRUN = 3,    /* a ray walked past Nx+Ny+Nz voxels; the reference raises
                               IndexError there (Python/openSSS/RayTracing3DTOF.py:162) */
    SSS_ERR_TOF_RANGE = 4,  /* TOF offset beyond the 8001-entry table; the reference raises
                               IndexError (SingleScatterSimulationTOF.py:521,527) */
    SSS_ERR_ENERGY = 5,     /* scattered energy row outside the 2000-row tables */
    SSS_ERR_VOXEL = 6,      /* linear voxel index outside the volume (only if Nx != Ny) */
    SSS_ERR_WORKSPACE = 7,  /* workspace too small */
    SSS_ERR_CAPACITY = 8,   /* an output capacity was too small */
    SSS_ERR_EVENT = 9,      /* a list-mode event addresses a crystal or ring outside the sinogram
                               tables; the reference raises IndexError (Timber/Datafile.py:90-92) */
    SSS_ERR_NONFINITE = 10, /* a scatter term came out infinite or NaN; no reference counterpart
                               (the reference's nan_to_num, SingleScatterSimulationTOF.py:557, only
                               hides 0/0 of empty slices): the result must not be used */
    SSS_ERR_TABLE = 11      /* a device index table the caller passed (sampled rings or crystals,
                               LOR coordinates, cell table, slice table) holds an entry outside its
                               range; the kernels skip such entries, so the result is incomplete */
};

/* Thread-local text of the last error. */
const char *sss_last_error(void);
/* SSS300_ABI_VERSION of the loaded library. */
int sss_abi_version(void);
/* Map a device status word to an SSS_ERR_* code (and set the message). */
int sss_status_code(int32_t device_status);

/* ---------------------------------------------------------------------------
 * Ray tracing.  Replaces RayTracing3DTOF (Python/openSSS/RayTracing3DTOF.py:29-180)
 * and the MEX tracers Matlab/RayTracing3DTOF.cpp:51 (variant 0) and
 * Matlab/RayTracing3D.cpp:51 (variant 1: float lengths, eps 1e-23, no samples),
 * batched: ray i is lines[6*i .. 6*i+5] = x1 y1 z1 x2 y2 z2 (device, f64).
 * Outputs are [n_rays][capacity] (device), capacity >= Nx+Ny+Nz:
 *   counts[i]            voxels crossed (0 = miss, -1 = the reference would overrun)
 *   lengths / lengths_f32  segment lengths (variant 0 / 1; the other may be NULL)
 *   indices              1-based linear voxel indices, X + (Y-1)*Ny + (Z-1)*Ny*Nx
 *   samples              running half-length samples (variant 0; may be NULL)
 * A ray that overruns sets SSS_ERR_OVERRUN in *status. */
int sss_raytrace(const int32_t grid[3], const double bounds[6], const double *lines,
                 int64_t n_rays, int32_t variant, int32_t capacity, int32_t *counts,
                 double *lengths, float *lengths_f32, int32_t *indices, double *samples,
                 int32_t *status, void *stream);

/* ---------------------------------------------------------------------------
 * TOF single scatter simulation.  Replaces SingleScatterSimulationTOF
 * (Python/openSSS/SingleScatterSimulationTOF.py:36-208 with bodySSS :301-559).
 * The non-TOF SingleScatterSimulation (Matlab/SingleScatterSimulation.m:44) is
 * nbins = 1 with a TOF kernel wide enough that every weight is 1. */
typedef struct sss_tof_problem {
    int32_t nx, ny, nz;            /* volume shape */
    const float *activity;         /* device, [nx*ny*nz] Fortran order (x fastest) */
    const float *attenuation;      /* device, cm^-1, same layout */
    double image_size[6];          /* xMin yMin zMin xMax yMax zMax, cm */
    int32_t nr, nd;                /* scanner rings, crystals per ring */
    const double *geometry;        /* device, [nr][nd][3] crystal centres, cm */
    const double *normals;         /* device, [nr][nd][3] face normals */
    double detector_size[2];       /* crystal face, mm */
    int32_t nru, ndu;              /* sampled rings, sampled crystals per ring */
    const int32_t *rings;          /* device, [nru] ring numbers (:153), each in 0..nr-1 */
    const int32_t *detectors;      /* device, [ndu] crystal numbers (:159-167), each in 0..nd-1;
                                      a leg whose ring or crystal is outside is left empty and
                                      sets SSS_ERR_TABLE in the status word */
    int32_t sample_step[3];        /* scatter-point lattice step, voxels */
    int32_t nbins;                 /* TOF bins, 1..64 */
    double tof_bin_width;          /* ps, 2*TOFRange/NrBins */
    double tof_resolution;         /* ps FWHM */
    const float *tof_log2w;        /* device, [8001][2]: log2 of the largest normalised TOF
                                      weight at offset t-4000 ps and its bin (as float);
                                      -inf where the reference's column is all zero */
    const float *efficiency;       /* device, [2000]: eff(E)*eff(511 keV); exact 0 where the
                                      FP64 product is 0 (:505-509) */
    const float *atten_ratio;      /* device, [2000]: water mu(E)/mu(511) (:117-120) */
    int32_t flags;                 /* SSS_FLAG_*; 0 = the plain FP32 reduction */
    int32_t pair_warps;            /* launch shape (no reference counterpart): warps per pair-kernel
                                      block, 0 = sss_pair_warps_max(nbins, flags), else 1..that */
    int32_t leg_threads;           /* threads per leg-kernel block, 0 = 128, else a multiple of 32
                                      up to 256 */
} sss_tof_problem;

/* Largest (and default) pair-kernel block of a bin count, in warps: the
 * kernels are compiled for it; a smaller pair_warps launches fewer warps a
 * block (no reference counterpart: the bound of the launch-shape tuner). */
int sss_pair_warps_max(int32_t nbins, int32_t flags);

/* sss_tof_problem.flags.  SSS_FLAG_KAHAN: the precision launch.  Each
 * detector pair's per-point terms are summed over a z-slice's scatter points
 * with Kahan's compensated addition (the reference sums them in FP32 too,
 * :551), and each voxel's TOF offset is formed from float-pair distances and
 * samples (about 44 bits; the voxel lists carry a third float per entry), so
 * that it takes the reference's FP64 table column (:520, :526) except within
 * about 1e-9 ps of a column boundary; the plain launch's FP32 offset can take
 * the neighbouring column within about 1e-3 ps.  Honoured by sss_tof_run;
 * sss_batch_* always uses the plain launch. */
#define SSS_FLAG_KAHAN 1
/* sss_tof_problem.flags.  SSS_FLAG_UNIT_TOF: the caller asserts that every
 * tof_log2w entry is (0, 0), i.e. one bin whose normalised TOF weight is
 * exactly 1 at every offset (the non-TOF SingleScatterSimulation, a kernel
 * of 1e6 ps).  Each pair then takes its legs' activity integrals instead of
 * walking their voxels (the reference's dot product with a row of ones,
 * :521-522), and no voxel lists are built.  Honoured by sss_tof_run and
 * sss_batch_*; the Python engine sets it when its table has that form. */
#define SSS_FLAG_UNIT_TOF 2

/* Scatter points on the SampleStep lattice with mu > 0, z-slice major, in the
 * reference's order (:182, :381-394).  points (device) receives [count][4]
 * (x, y, z, lattice z index) for up to `capacity` points; slice_counts (host,
 * may be NULL) receives the number of points of each sampled z-slice
 * (ceil(nz/step_z) entries).  Synchronises `stream`; *count (host) is the
 * total even when it exceeds capacity (then SSS_ERR_CAPACITY). */
int sss_scatter_points(const sss_tof_problem *p, double *points, int64_t capacity,
                       int64_t *count, int64_t *slice_counts, void *stream);

/* No counterpart in the reference.  sss_scatter_points without any device
 * allocation, for callers that must not allocate: code running inside a
 * fixed memory arena or pool it does not own, or in a process whose device
 * memory is capped, where a late allocation could fail in mid-pipeline.
 * Same arguments, results and errors as sss_scatter_points; like it, the call
 * copies its counts to the host and synchronises `stream` before it returns.
 * Its scratch is a 32 KiB array inside the library that every GPU loading
 * the library holds until exit.  Limit: at most 4096 sampled z-slices
 * (ceil(nz / sample_step[2])); larger problems get SSS_ERR_INVALID.  The
 * first call on each device looks up that array's device address and keeps
 * it, so make that first call before any stream capture on the device; a
 * device reset (cudaDeviceReset) is not supported afterwards.  All calls
 * share the array: calls whose work overlaps on the GPU race, so serialise
 * them. */
int sss_scatter_points_noalloc(const sss_tof_problem *p, double *points, int64_t capacity,
                               int64_t *count, int64_t *slice_counts, void *stream);

/* Bytes of device workspace sss_tof_run needs for waves of at most
 * wave_points scatter points (a wave always holds whole z-slices). */
size_t sss_tof_workspace_size(const sss_tof_problem *p, int64_t wave_points);

/* Run the simulation for the points [0, n_points) (whole slices as given by
 * slice_counts, host, n_slices entries).  out (device) receives the sampled
 * scatter sinogram in leg-pair layout [nbins][NL][NL], NL = nru*ndu, leg
 * l = det_index*nru + ring_index (crystal-major): element [b][l1][l2] is the reference's
 * Scatters[b, Radial, Angular, ri2 + ri1*nru] for the crystal pair
 * (detectors[di1], detectors[di2]), defined for di1 < di2 and for di1 == di2
 * with ri1 != ri2, zero elsewhere.  Asynchronous on `stream`. */
int sss_tof_run(const sss_tof_problem *p, const double *points, int64_t n_points,
                const int64_t *slice_counts, int64_t n_slices, int64_t wave_points,
                void *workspace, size_t workspace_bytes, float *out, int32_t *status,
                void *stream);

/* Expand the leg-pair output to the reference's dense layout
 * [nbins][nd+1][nd/2][nru*nru] (SingleScatterSimulationTOF.py:171).  lor
 * (device) is LORCoordinates int16 [nd][nd][2] (Python/openSSS/Sinogram.py:121-122);
 * the entries of the sampled crystal pairs must lie in range (angular < nd/2,
 * radial <= nd), and detectors[] in 0..nd-1.  Entries outside are skipped and
 * set SSS_ERR_TABLE in *status (device int32, OR-ed).  dense must be zeroed by
 * the caller. */
int sss_tof_densify(const float *compact, int32_t nbins, int32_t nru, int32_t ndu, int32_t nd,
                    const int16_t *lor, const int32_t *detectors, float *dense, int32_t *status,
                    void *stream);

/* The same dense layout, every element written (zeros included), so dense
 * needs no clearing: for a fresh result array such as the one
 * SingleScatterSimulationTOF returns (SingleScatterSimulationTOF.py:201-208).
 * cell_pair (device int32 [(nd+1)*(nd/2)]) gives, per sinogram cell
 * rad*(nd/2) + ang, the sampled crystal pair di1*ndu + di2 (di1 <= di2) whose
 * LOR it is, or -1 (each pair in at most one cell).  An entry that is not -1
 * or such a pair writes zeros and sets SSS_ERR_TABLE in *status (device int32,
 * OR-ed).  dense may be device memory or page-locked host memory (written over
 * the host link at its device address); any other pointer is SSS_ERR_INVALID.
 * Needs nru*nru a multiple of 4 and a 16-byte aligned dense. */
int sss_tof_densify_full(const float *compact, int32_t nbins, int32_t nru, int32_t ndu, int32_t nd,
                         const int32_t *cell_pair, float *dense, int32_t *status, void *stream);

/* As sss_tof_densify_full, but only the cells of sampled pairs are written
 * (every element of them); the other cells of dense are left as they are.
 * For a destination whose other cells already hold zeros: the drop-in copies
 * zeros into its page-locked result while the simulation runs and then writes
 * the sampled cells (well under 1% of the array) with this call. */
int sss_tof_densify_cells(const float *compact, int32_t nbins, int32_t nru, int32_t ndu, int32_t nd,
                          const int32_t *cell_pair, float *dense, int32_t *status, void *stream);

/* ---------------------------------------------------------------------------
 * Batched simulation (no counterpart in the reference, which runs one
 * SingleScatterSimulationTOF call per problem).  sss_batch_plan enumerates the
 * scatter points of n problems (different volumes, scanners, samplings and
 * bin counts allowed), cuts them into (problem, sampled z-slice) items and
 * packs the items into waves that fit the workspace; each wave is one leg
 * launch over all its items and one pair launch per TOF class (bin count and
 * TOF kernel).  Everything lives in the caller's device workspace: the plan
 * itself allocates no device memory.  It synchronises `stream` once.  outs[i]
 * (device) receives problem i's output in the leg-pair layout of
 * sss_tof_run.  sss_batch_run zeroes the outputs and enqueues the waves on
 * `stream` without synchronising; it may run again after the activity maps
 * change in place (the attenuation maps, which decide the scatter points,
 * must not) and may be captured in a CUDA graph.  The problems' device
 * arrays, the outputs and the workspace must outlive the plan's last run.
 * sss_batch_info: info[0] waves, info[1] kernel launches per run, info[2]
 * detector-pair x bin evaluations per run, info[3] scatter points.  Launch
 * shapes: the leg launches use problem 0's leg_threads, and each TOF class's
 * pair launch uses the pair_warps of its first problem. */
typedef struct sss_batch sss_batch;
int sss_batch_plan(const sss_tof_problem *problems, int32_t n, float *const *outs, void *workspace,
                   size_t workspace_bytes, int32_t *status, sss_batch **plan, void *stream);
int sss_batch_run(const sss_batch *plan, void *stream);
/* sss_batch_plan for problems whose scatter points are already known (for
 * instance from sss_scatter_points, which depend on the attenuation map
 * only): points[i] (device, [count][4]) and slice_counts[i] (host,
 * ceil(nz/step_z) entries) for each problem.  Does not synchronise `stream`
 * except to upload the plan's descriptors; the point arrays must outlive the
 * plan's last run. */
int sss_batch_plan_points(const sss_tof_problem *problems, int32_t n, float *const *outs,
                          const double *const *points, const int64_t *const *slice_counts,
                          void *workspace, size_t workspace_bytes, int32_t *status, sss_batch **plan,
                          void *stream);
/* Run waves [first, first + count) of a plan (0 <= first, first + count <=
 * info[0]).  Waves must run in order, each once per run, and the outputs are
 * complete after the last; starting at wave 0 zeroes them.  A caller can
 * interleave other work between waves (continuous batching). */
int sss_batch_run_waves(const sss_batch *plan, int32_t first, int32_t count, void *stream);
int sss_batch_info(const sss_batch *plan, int64_t info[4]);
void sss_batch_free(sss_batch *plan);

/* ---------------------------------------------------------------------------
 * Upsampling.  Replaces InterpolateAllBins (Python/openSSS/Interpolation.py:197-319)
 * once its nearest-neighbour choices are known (geometry time, see
 * opensss_gb300/geometry.py): out[cell*nslices + s] = sum over the nbins bins
 * of max(sampled[b*bin_stride + cell_src[cell] + ring_off[ring_idx[s]]], 0),
 * in bin order (one bin: nbins = 1).  cell = rad*(ND/2) + ang over the full
 * (ND+1) x ND/2 sinogram, s = full-sinogram slice, ring_off = the nring
 * distinct sampled ring-pair offsets (nring <= 16384), ring_idx[s] in
 * [0, nring).  The offset tables (device) address either the reference's
 * dense sampled layout or the leg-pair layout of sss_tof_run.  out (device)
 * is [ncell][nslices]. */
int sss_upsample(const float *sampled, int64_t bin_stride, int32_t nbins, const int64_t *cell_src,
                 int64_t ncell, const int64_t *ring_off, int32_t nring, const int32_t *ring_idx,
                 int32_t nslices, float *out, void *stream);

/* Tail mask.  Replaces MaskGenerator / MaskDetectors (Python/openSSS/TailsMask.py:84-228):
 * every LOR (Ring1, d1, Ring2, d2) with d1, d2 multiples of af and d1 <= d2
 * (not the same crystal) is traced through map (device float32, Fortran
 * order; attenuation in cm^-1, or activity when use_activity) in FP64.
 * out[cell*nr*nr + sino_index[Ring1][Ring2]] = 1 where 1/exp(-sum mu*len) == 1
 * (attenuation) or sum act*len <= 0 (activity).  acf_below = 0 keeps that
 * rule (the reference's, :145-151); acf_below > 1 masks instead where the
 * attenuation factor 1/exp(-sum mu*len) is below acf_below (no reference
 * counterpart: a looser tail definition, e.g. 1.03).  out (device uint8,
 * [(nd+1)*(nd/2)][nr*nr]) must be zeroed by the caller.  A sino_index entry
 * outside 0..nr*nr-1, or LOR coordinates outside the sinogram, skip the LOR
 * and set SSS_ERR_TABLE in *status. */
int sss_tail_mask(const int32_t grid[3], const double bounds[6], const float *map, int32_t use_activity,
                  int32_t nr, int32_t nd, const double *geometry, const int16_t *lor,
                  const int16_t *sino_index, int32_t af, double acf_below, uint8_t *out, int32_t *status,
                  void *stream);

/* Tail mask with span.  Replaces MaskGeneratorMashing / MaskDetectorsMashing
 * (Python/openSSS/TailsMask.py:230-377): the LORs are those of the npairs ring
 * pairs pairs[p] = (Ring1, Ring2, slice) (device int32 [npairs][3]) on the
 * expanded geometry (nr = 2*rings - 1, Python/openSSS/Geometry.py:161-197),
 * crystal pairs and acf_below as in sss_tail_mask; LOR (p, d1, d2) marks
 * out[cell*nslices + slice].  out (device uint8 [(nd+1)*(nd/2)][nslices])
 * must be zeroed by the caller.  A pair with a ring outside 0..nr-1 or a slice
 * outside 0..nslices-1 is skipped and sets SSS_ERR_TABLE in *status. */
int sss_tail_mask_pairs(const int32_t grid[3], const double bounds[6], const float *map, int32_t use_activity,
                        int32_t nr, int32_t nd, const double *geometry, const int16_t *lor, const int32_t *pairs,
                        int32_t npairs, int32_t nslices, int32_t af, double acf_below, uint8_t *out,
                        int32_t *status, void *stream);

/* Back-projection scale fit.  Replaces BackProjectionScatterRandFit
 * (Python/openSSS/BackProjection.py:115-215) and BackProjection (:31-113).
 * The LOR (Ring1, d1, Ring2, d2) on the af lattice reads slice
 * sino_order[Ring1][Ring2] (the reference passes SinogramIndex.T) of the
 * full sinograms prompts / randoms (device float32 [cell][slice]) and of the
 * mask: mask_f32 (multiplied) or, if not NULL, mask_u8 (mask >= 1).  The
 * scatter value is scatters[scat_cell[cell] + scat_ring[slice]] (clamped at
 * 0 when scat_clamp), so an upsampled sinogram can be read straight from
 * the sampled one.  images: device workspace 8 * Nx*Ny*Nz floats, 16-byte
 * aligned, laid out as sss_backproject_fit_bins's for one bin; sums: device
 * 2 doubles; scale: device float, the fitted slope (reference: float32 array
 * of shape (1,)). */
int sss_backproject_fit(const int32_t grid[3], const double bounds[6], int32_t nr, int32_t nd,
                        const double *geometry, const int16_t *lor, const int16_t *sino_order,
                        int32_t af, const float *prompts, const float *randoms, const float *mask_f32,
                        const uint8_t *mask_u8, const float *scatters, const int64_t *scat_cell,
                        const int64_t *scat_ring, int32_t scat_clamp, float *images, double *sums,
                        float *scale, int32_t *status, void *stream);

/* Fit with span.  Replaces BackProjectionScatterRandFitMashing /
 * BackProjectionMashing (Python/openSSS/BackProjection.py:217-393): LORs of
 * the ring pairs pairs[p] = (Ring1, Ring2, slice) on the expanded geometry,
 * reading slice `slice` of the [cell][nslices] sinograms.  length_weighted:
 * each voxel gets value * length / sum(lengths) (:294-297) instead of
 * value / voxels.  Other arguments and outputs as sss_backproject_fit. */
int sss_backproject_fit_pairs(const int32_t grid[3], const double bounds[6], int32_t nr, int32_t nd,
                              const double *geometry, const int16_t *lor, const int32_t *pairs, int32_t npairs,
                              int32_t nslices, int32_t length_weighted, int32_t af, const float *prompts,
                              const float *randoms, const float *mask_f32, const uint8_t *mask_u8,
                              const float *scatters, const int64_t *scat_cell, const int64_t *scat_ring,
                              int32_t scat_clamp, float *images, double *sums, float *scale, int32_t *status,
                              void *stream);

/* All TOF bins of a scale fit in one pass.  Replaces the per-bin loop of
 * ScaleScattersToPrompts (Python/openSSS/Scaling.py:86-113): every LOR is
 * walked once and back-projected into the images of each bin whose masked
 * scatter is non-zero there; each bin gets the scale its own
 * sss_backproject_fit(_pairs) call would give.  Bin b reads
 * prompts[b*prompt_stride + cell*nslices + slice] and the scatter value
 * scatters[b*scat_stride + scat_cell[cell] + scat_ring[slice]]; randoms and
 * the mask are shared.  Either sino_order (all ring pairs) or pairs (span)
 * is given.  images: device float [nbins + 1][4 * Nx*Ny*Nz], 16-byte aligned.
 * Per voxel and bin they hold D, the back-projected (prompts - randoms) (the
 * reference's ActivityImage - RandomImage, summed once), S, the scatter, and
 * the sensitivity: bins 2q and 2q+1 share blocks 2q and 2q+1 as float4 per
 * voxel, (D, S, D, S) then (0, sensitivity, 0, sensitivity) of the LORs that
 * use some bins only; an odd last bin L has float4 (D, S, 0, common
 * sensitivity) in block L, the common sensitivity counting the LORs every
 * bin uses, and float2 (0, sensitivity) in the first half of block nbins;
 * with an even bin count the common sensitivity is float2 (0, sensitivity)
 * in the second half of block nbins; sums: device [nbins][2]; scales: device
 * float [nbins];
 * 1 <= nbins <= 64. */
int sss_backproject_fit_bins(const int32_t grid[3], const double bounds[6], int32_t nr, int32_t nd,
                             const double *geometry, const int16_t *lor, const int16_t *sino_order,
                             const int32_t *pairs, int32_t npairs, int32_t nslices, int32_t length_weighted,
                             int32_t af, int32_t nbins, const float *prompts, int64_t prompt_stride,
                             const float *randoms, const float *mask_f32, const uint8_t *mask_u8,
                             const float *scatters, int64_t scat_stride, const int64_t *scat_cell,
                             const int64_t *scat_ring, int32_t scat_clamp, float *images, double *sums,
                             float *scales, int32_t *status, void *stream);

/* ---------------------------------------------------------------------------
 * CASToR list-mode events.  Replaces ExportPrompts and InjectScatters
 * (Python/Timber/Datafile.py:29-240) with ParseCASToRIDs (Coincidence.py:97-159).
 * Events are fixed-size little-endian records (GenerateListEventInfo,
 * Coincidence.py:47-95) already in device memory. */
typedef struct sss_listmode_layout {
    int32_t record_bytes;    /* bytes per event, a multiple of 4 */
    int32_t id_offset;       /* byte offset of the two uint32 CASToR crystal IDs */
    int32_t tof_offset;      /* byte offset of the float32 TOF difference (ps) */
    int32_t scatter_offset;  /* injection: byte offset the scatter rate is inserted at */
} sss_listmode_layout;

typedef struct sss_sino_map {
    const int16_t *lor;      /* device [nd_lor][nd_lor][2] (angular, radial), -1 = no LOR */
    int32_t nd_lor;          /* crystals of the LOR table (crystals per ring / mash) */
    int32_t mash;            /* crystals per LOR-table crystal */
    int32_t shift;           /* crystal ID shift of the first module */
    const int16_t *slices;   /* device [nr_table][nr_table] slice of each ring pair, -1 = none
                                (SinogramIndex, or LookUpTable with span) */
    int32_t nr_table;
    int32_t nrad, nang, nslices;  /* sinogram shape */
    int32_t tof_bins;
    double tof_range;        /* ps */
} sss_sino_map;

/* Prompt histogram: counts (device uint32 [nrad][nang][nslices][tof_bins],
 * zeroed by the caller) += 1 per event in range.  last (device, zeroed,
 * [nrad*nang*nslices], or NULL when no randoms / normalisation sinogram is
 * wanted) records the last event of each cell for sss_histogram_finish. */
int sss_histogram_prompts(const void *events, int64_t n_events, const sss_listmode_layout *layout,
                          const sss_sino_map *map, uint32_t *counts, unsigned long long *last,
                          int32_t *status, void *stream);
/* prompts (device uint16, same shape as counts) = counts modulo 2^16, as the
 * reference's uint16 histogram wraps; randoms / norm (device float32 per
 * cell, each may be NULL) get the last event's event[0] * duration /
 * tof_bins and event[1] (Datafile.py:94-99; norm must start at 1). */
int sss_histogram_finish(const void *events, int64_t n_events, const sss_listmode_layout *layout,
                         const sss_sino_map *map, const uint32_t *counts, const unsigned long long *last,
                         double duration, uint16_t *prompts, float *randoms, float *norm, void *stream);
/* Scatter injection: keeps the events the reference keeps, in file order,
 * each with the float32 rate factor[bin] * scatters[bin][cell] inserted at
 * scatter_offset (out_events: record_bytes + 4 per event; *out_count
 * (device) = events written).  scatters: device float32
 * [tof_bins][nrad][nang][nslices]; factor: device float32 [tof_bins] =
 * Scale[b] * 2/c / duration as the reference rounds it.  workspace: at least
 * sss_inject_workspace_size(n_events) device bytes. */
size_t sss_inject_workspace_size(int64_t n_events);
int sss_inject_scatters(const void *events, int64_t n_events, const sss_listmode_layout *layout,
                        const sss_sino_map *map, const float *scatters, const float *factor, void *out_events,
                        unsigned long long *out_count, void *workspace, size_t workspace_bytes,
                        int32_t *status, void *stream);

/* ---------------------------------------------------------------------------
 * Image preparation.  Replaces CropAndDownscale (Python/openSSS/Utils.py:212-267,
 * used by PrepareImages :30-74): a crop or zero-pad window about the volume
 * centre, then skimage.transform.resize(order=3, mode='edge',
 * anti_aliasing=True, preserve_range=True) of that window.  Volumes are
 * C-ordered float32 [n0][n1][n2] on the device.  The window (computed by the
 * caller with the reference's slicing rules): crop[i] = image[i - before +
 * start] per axis where that lies inside the image, else 0, for i <
 * crop_dims.  sigma: the anti-aliasing Gaussian's sigma per axis in voxels
 * (0 = no filter on that axis).  clip != 0 clips the result to the window's
 * [min, max]; results below zero_below become 0 (-INFINITY: none).
 * workspace: at least sss_crop_downscale_workspace_size(crop_dims) device
 * bytes. */
size_t sss_crop_downscale_workspace_size(const int crop_dims[3]);
int sss_crop_downscale(const float *image, const int image_dims[3], const int crop_start[3],
                       const int crop_before[3], const int crop_dims[3], const int out_dims[3],
                       const double sigma[3], int clip, float zero_below, float *out, void *workspace,
                       size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Stage timing (no reference counterpart: instrumentation for benchmarks).
 * When enabled, sss_tof_run records CUDA events around its kernels on the
 * caller's stream; sss_get_timing waits for them and returns, for the last
 * run on this thread, out[0] = leg-stage ms, out[1] = pair-stage ms,
 * out[2] = kernel launches, out[3] = waves, out[4] = TOF weights evaluated
 * (voxel x bin), out[5] = detector pairs evaluated (all scatter points).
 * The workspace of that run must still be alive. */
void sss_set_timing(int enable);
int sss_get_timing(double out[6]);

#ifdef __cplusplus
}
#endif

#endif /* SSS300_H */
