// Error handling, version, and the batched ray tracer entry point.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.cuh"
#include "trace.cuh"

static thread_local char g_err[1024] = "";

int sss_set_error(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int sss_check_launch(const char* what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return sss_set_error(SSS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return SSS_OK;
}

extern "C" const char* sss_last_error(void) { return g_err; }

extern "C" int sss_abi_version(void) { return SSS300_ABI_VERSION; }

extern "C" int sss_status_code(int32_t s)
{
    using namespace sss;
    s &= ~kNoteMapSigned;
    if (s == 0) return SSS_OK;
    if (s & kErrOverrun)
        return sss_set_error(SSS_ERR_OVERRUN,
                             "a ray traversal would pass Nx+Ny+Nz voxels (the reference raises "
                             "IndexError here)");
    if (s & kErrVoxel)
        return sss_set_error(SSS_ERR_VOXEL, "a linear voxel index fell outside the volume");
    if (s & kErrTofRange)
        return sss_set_error(SSS_ERR_TOF_RANGE,
                             "a TOF offset fell beyond the 8001-entry table (reference: IndexError)");
    if (s & kErrEnergy)
        return sss_set_error(SSS_ERR_ENERGY, "a scattered energy row fell outside the tables");
    if (s & kErrCapacity)
        return sss_set_error(SSS_ERR_CAPACITY, "an internal capacity was exceeded");
    if (s & kErrNonFinite)
        return sss_set_error(SSS_ERR_NONFINITE,
                             "a detector pair's scatter term came out infinite or NaN (the result is not "
                             "usable)");
    if (s & kErrTable)
        return sss_set_error(SSS_ERR_TABLE,
                             "an index table (sampled rings or crystals, LOR coordinates, cell or slice "
                             "table) holds an entry outside its range");
    if (s & kErrEvent)
        return sss_set_error(SSS_ERR_EVENT,
                             "a list-mode event addresses a crystal or ring outside the sinogram tables "
                             "(the reference raises IndexError here)");
    return sss_set_error(SSS_ERR_INVALID, "unknown device status 0x%x", (unsigned)s);
}

namespace {

using namespace sss;

// One thread per ray.  Variant 0 = RayTracing3DTOF (f64 lengths + samples,
// eps 1e-20); variant 1 = RayTracing3D MEX (f32 lengths, eps 1e-23).
__global__ void __launch_bounds__(128) raytrace_kernel(Grid g, const double* __restrict__ lines,
                                                       int64_t n, int variant, int cap,
                                                       int32_t* __restrict__ counts,
                                                       double* __restrict__ len64,
                                                       float* __restrict__ len32,
                                                       int32_t* __restrict__ idx,
                                                       double* __restrict__ samples,
                                                       int32_t* status)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double lc[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) lc[k] = lines[6 * i + k];
    Ray r;
    const double eps = variant == 0 ? 1e-20 : 1e-23;
    if (!ray_setup(g, lc, eps, r)) {
        counts[i] = 0;
        return;
    }
    const int64_t base = i * (int64_t)cap;
    double prev = 0.0;
    int c = ray_walk(g, r, cap, [&](int k, int64_t lin, double t0, double t1) {
        double d = ref_length(r, t0, t1);
        idx[base + k] = (int32_t)lin;
        if (variant == 0) {
            if (len64) len64[base + k] = d;
            prev = add64(prev, d / 2);
            if (samples) samples[base + k] = prev;
        } else {
            if (len32) len32[base + k] = (float)d;
        }
    });
    if (c < 0) raise_error(status, kErrOverrun);
    counts[i] = c;
}

}  // namespace

extern "C" int sss_raytrace(const int32_t grid[3], const double bounds[6], const double* lines,
                            int64_t n_rays, int32_t variant, int32_t capacity, int32_t* counts,
                            double* lengths, float* lengths_f32, int32_t* indices,
                            double* samples, int32_t* status, void* stream)
{
    if (!grid || !bounds || (!lines && n_rays > 0) || !counts || !indices)
        return sss_set_error(SSS_ERR_INVALID, "sss_raytrace: null argument");
    if (variant != 0 && variant != 1)
        return sss_set_error(SSS_ERR_INVALID, "sss_raytrace: variant must be 0 or 1");
    if (grid[0] < 1 || grid[1] < 1 || grid[2] < 1)
        return sss_set_error(SSS_ERR_INVALID, "sss_raytrace: grid must be positive");
    if (!(bounds[3] > bounds[0] && bounds[4] > bounds[1] && bounds[5] > bounds[2]))
        return sss_set_error(SSS_ERR_INVALID, "sss_raytrace: bounds must satisfy max > min");
    int64_t need = (int64_t)grid[0] + grid[1] + grid[2];
    if (capacity < need)
        return sss_set_error(SSS_ERR_CAPACITY, "sss_raytrace: capacity %d < Nx+Ny+Nz = %lld",
                             capacity, (long long)need);
    if (n_rays <= 0) return SSS_OK;
    const Grid g = grid_of(grid[0], grid[1], grid[2], bounds);
    const int threads = 128;
    int64_t blocks = (n_rays + threads - 1) / threads;
    raytrace_kernel<<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(
        g, lines, n_rays, variant, capacity, counts, lengths, lengths_f32, indices, samples,
        status);
    return sss_check_launch("sss_raytrace");
}
