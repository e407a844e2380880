// Image preparation on the GPU: crop or zero-pad about the volume centre, then
// resize with the anti-aliasing Gaussian and cubic B-spline interpolation that
// the reference reaches through skimage.transform.resize (Python/openSSS/
// Utils.py:212-267, CropAndDownscale; :30-74, PrepareImages).  resize(order=3,
// mode='edge', anti_aliasing=True, preserve_range=True, clip=True) is, step by
// step:
//   1. a Gaussian filter per axis, sigma = max(0, (in/out - 1)/2), kernel
//      radius int(4 sigma + 0.5), edge samples repeated past the ends;
//   2. cubic B-spline coefficients of the result, computed on a copy padded by
//      12 edge samples per side (recursive filter, pole sqrt(3) - 2);
//   3. the coefficients sampled at x = (o + 0.5) in/out - 0.5 per axis;
//   4. the result clipped to the [min, max] of the cropped input.
// Volumes are C-ordered float32 [n0][n1][n2].
#include <math.h>

#include "common.cuh"

namespace {

constexpr int kPad = 12;        // edge samples added per side before the spline filter
constexpr int kMaxRadius = 512; // Gaussian kernel radius limit (weights in shared memory)

struct Dims {
    int n[3];
    __host__ __device__ long long count() const { return (long long)n[0] * n[1] * n[2]; }
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// out[i] = in[i - before + start] per axis where that lies inside the input, else 0.
__global__ void crop_kernel(const float* __restrict__ in, Dims din, float* __restrict__ out, Dims dout,
                            int3 start, int3 before)
{
    const long long total = dout.count();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i % dout.n[2]);
        const int j = (int)((i / dout.n[2]) % dout.n[1]);
        const int h = (int)(i / ((long long)dout.n[2] * dout.n[1]));
        const int a = h - before.x + start.x, b = j - before.y + start.y, c = k - before.z + start.z;
        float v = 0.f;
        if (a >= 0 && a < din.n[0] && b >= 0 && b < din.n[1] && c >= 0 && c < din.n[2])
            v = in[((long long)a * din.n[1] + b) * din.n[2] + c];
        out[i] = v;
    }
}

// Per-block minimum and maximum of x[0..n) into part[2 * block].
__global__ void __launch_bounds__(256) minmax_partial_kernel(const float* __restrict__ x, long long n,
                                                             float* __restrict__ part)
{
    float lo = INFINITY, hi = -INFINITY;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float v = x[i];
        lo = fminf(lo, v);
        hi = fmaxf(hi, v);
    }
    __shared__ float slo[256], shi[256];
    slo[threadIdx.x] = lo;
    shi[threadIdx.x] = hi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            slo[threadIdx.x] = fminf(slo[threadIdx.x], slo[threadIdx.x + s]);
            shi[threadIdx.x] = fmaxf(shi[threadIdx.x], shi[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = slo[0];
        part[2 * blockIdx.x + 1] = shi[0];
    }
}

// Reduces nb per-block pairs to part[0] = min, part[1] = max (one block).
__global__ void __launch_bounds__(256) minmax_final_kernel(float* __restrict__ part, int nb)
{
    float lo = INFINITY, hi = -INFINITY;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        lo = fminf(lo, part[2 * i]);
        hi = fmaxf(hi, part[2 * i + 1]);
    }
    __shared__ float slo[256], shi[256];
    slo[threadIdx.x] = lo;
    shi[threadIdx.x] = hi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            slo[threadIdx.x] = fminf(slo[threadIdx.x], slo[threadIdx.x + s]);
            shi[threadIdx.x] = fmaxf(shi[threadIdx.x], shi[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[0] = slo[0];
        part[1] = shi[0];
    }
}

// One axis of the Gaussian filter: out = sum_k w[k] in[clamp(i + k - r)] along
// `axis` (edge samples repeated).  Weights are FP32 copies of the normalised
// FP64 kernel, staged in shared memory.  I: the index type, 32-bit unsigned
// for volumes below 2^31 elements (the index arithmetic is most of the
// kernel's instructions), 64-bit above.
template <typename I>
__global__ void __launch_bounds__(256) gauss_axis_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                         Dims d, int axis, const float* __restrict__ w, int r)
{
    __shared__ float sw[2 * kMaxRadius + 1];
    for (int i = threadIdx.x; i <= 2 * r; i += blockDim.x) sw[i] = w[i];
    __syncthreads();
    const I total = (I)d.count();
    const I stride = axis == 2 ? (I)1 : (axis == 1 ? (I)d.n[2] : (I)d.n[1] * (I)d.n[2]);
    const int len = d.n[axis];
    for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (I)gridDim.x * blockDim.x) {
        const int p = (int)((i / stride) % (I)len);  // position along the axis
        const I base = i - (I)p * stride;
        float acc = 0.f;
        if (p >= r && p + r < len) {  // no sample past an end: a running offset
            I q = base + (I)(p - r) * stride;
            for (int k = 0; k <= 2 * r; ++k, q += stride) acc = fmaf(sw[k], in[q], acc);
        } else {
            for (int k = -r; k <= r; ++k) acc = fmaf(sw[k + r], in[base + (I)clampi(p + k, 0, len - 1) * stride], acc);
        }
        out[i] = acc;
    }
}

// Edge padding by kPad samples on every side: P[p] = F[clamp(p - kPad)].
__global__ void pad_edge_kernel(const float* __restrict__ f, Dims d, float* __restrict__ P, Dims dp)
{
    const long long total = dp.count();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i % dp.n[2]);
        const int j = (int)((i / dp.n[2]) % dp.n[1]);
        const int h = (int)(i / ((long long)dp.n[2] * dp.n[1]));
        const int a = clampi(h - kPad, 0, d.n[0] - 1), b = clampi(j - kPad, 0, d.n[1] - 1),
                  c = clampi(k - kPad, 0, d.n[2] - 1);
        P[i] = f[((long long)a * d.n[1] + b) * d.n[2] + c];
    }
}

// Cubic B-spline coefficients along `axis`, in place, one thread per line
// (Unser's recursive filter: gain 6, causal and anti-causal passes with pole
// z = sqrt(3) - 2, mirror-symmetric start values).  The 12 edge samples in
// front of the data make the start values' effect on the data below z^12.
constexpr int kSplineAhead = 8;  // values loaded ahead of the in-place recursion

__global__ void spline_axis_kernel(float* __restrict__ P, Dims d, int axis)
{
    const float z = -0.26794919243112270f;  // sqrt(3) - 2
    const long long stride = axis == 2 ? 1 : (axis == 1 ? d.n[2] : (long long)d.n[1] * d.n[2]);
    const int len = d.n[axis];
    const long long lines = d.count() / len;
    for (long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x; l < lines;
         l += (long long)gridDim.x * blockDim.x) {
        // line l: the other two indices in C order
        long long base;
        if (axis == 2) {
            base = l * len;
        } else if (axis == 1) {
            const long long h = l / d.n[2], k = l % d.n[2];
            base = h * (long long)d.n[1] * d.n[2] + k;
        } else {
            base = l;  // l = j * n2 + k
        }
        float* x = P + base;
        // causal start: sum_k z^k c[k] over the first terms (z^28 < 1e-16)
        const int kmax = len < 28 ? len : 28;
        float zk = 1.f, c0 = 0.f;
        for (int k = 0; k < kmax; ++k) {
            c0 = fmaf(zk, 6.f * x[k * stride], c0);
            zk *= z;
        }
        x[0] = c0;
        float prev = c0;
        // The recursion runs in place, so each load would otherwise wait for
        // the store before it: kSplineAhead values are loaded together first
        // (none of them written yet), then filtered and stored.
        int k = 1;
        for (; k + kSplineAhead <= len; k += kSplineAhead) {
            float v[kSplineAhead];
#pragma unroll
            for (int j = 0; j < kSplineAhead; ++j) v[j] = x[(long long)(k + j) * stride];
#pragma unroll
            for (int j = 0; j < kSplineAhead; ++j) {
                prev = fmaf(z, prev, 6.f * v[j]);
                x[(long long)(k + j) * stride] = prev;
            }
        }
        for (; k < len; ++k) {
            prev = fmaf(z, prev, 6.f * x[(long long)k * stride]);
            x[(long long)k * stride] = prev;
        }
        // anti-causal start from the last two causal values
        float next = (z / (z * z - 1.f)) * fmaf(z, len > 1 ? x[(long long)(len - 2) * stride] : prev, prev);
        x[(long long)(len - 1) * stride] = next;
        k = len - 2;
        for (; k - kSplineAhead + 1 >= 0; k -= kSplineAhead) {
            float v[kSplineAhead];
#pragma unroll
            for (int j = 0; j < kSplineAhead; ++j) v[j] = x[(long long)(k - j) * stride];
#pragma unroll
            for (int j = 0; j < kSplineAhead; ++j) {
                next = z * (next - v[j]);
                x[(long long)(k - j) * stride] = next;
            }
        }
        for (; k >= 0; --k) {
            next = z * (next - x[(long long)k * stride]);
            x[(long long)k * stride] = next;
        }
    }
}

__device__ __forceinline__ void cubic_weights(double x, int& i0, float w[4])
{
    const double f = floor(x);
    const float t = (float)(x - f);
    const float t2 = t * t, t3 = t2 * t, u = 1.f - t;
    w[0] = u * u * u * (1.f / 6.f);
    w[1] = (3.f * t3 - 6.f * t2 + 4.f) * (1.f / 6.f);
    w[2] = (-3.f * t3 + 3.f * t2 + 3.f * t + 1.f) * (1.f / 6.f);
    w[3] = t3 * (1.f / 6.f);
    i0 = (int)f - 1 + kPad;
}

// Output voxel o: the coefficients sampled at x_d = (o_d + 0.5) in_d/out_d - 0.5,
// clipped to [lim[0], lim[1]] when clip is set; values below zero_below become 0.
__global__ void zoom_kernel(const float* __restrict__ P, Dims dp, Dims din, float* __restrict__ out, Dims dout,
                            const float* __restrict__ lim, int clip, float zero_below)
{
    const long long total = dout.count();
    const float lo = clip ? lim[0] : -INFINITY, hi = clip ? lim[1] : INFINITY;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int o2 = (int)(i % dout.n[2]);
        const int o1 = (int)((i / dout.n[2]) % dout.n[1]);
        const int o0 = (int)(i / ((long long)dout.n[2] * dout.n[1]));
        int a0, a1, a2;
        float w0[4], w1[4], w2[4];
        cubic_weights((o0 + 0.5) * ((double)din.n[0] / dout.n[0]) - 0.5, a0, w0);
        cubic_weights((o1 + 0.5) * ((double)din.n[1] / dout.n[1]) - 0.5, a1, w1);
        cubic_weights((o2 + 0.5) * ((double)din.n[2] / dout.n[2]) - 0.5, a2, w2);
        float acc = 0.f;
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            float accp = 0.f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float* row = P + ((long long)(a0 + p) * dp.n[1] + (a1 + q)) * dp.n[2] + a2;
                const float s = fmaf(w2[0], row[0], fmaf(w2[1], row[1], fmaf(w2[2], row[2], w2[3] * row[3])));
                accp = fmaf(w1[q], s, accp);
            }
            acc = fmaf(w0[p], accp, acc);
        }
        acc = fminf(fmaxf(acc, lo), hi);
        out[i] = acc < zero_below ? 0.f : acc;
    }
}

int grid_for(long long n, int threads = 256)
{
    long long b = (n + threads - 1) / threads;
    return (int)(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

constexpr int kMinmaxBlocks = 1024;

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct PrepLayout {
    size_t crop, tmp, padded, part, weights, total;
};

PrepLayout prep_layout(const int crop[3])
{
    const long long c = (long long)crop[0] * crop[1] * crop[2];
    const long long p = (long long)(crop[0] + 2 * kPad) * (crop[1] + 2 * kPad) * (crop[2] + 2 * kPad);
    PrepLayout L;
    L.crop = 0;
    L.tmp = L.crop + align256(c * sizeof(float));
    L.padded = L.tmp + align256(c * sizeof(float));
    L.part = L.padded + align256(p * sizeof(float));
    L.weights = L.part + align256(2 * kMinmaxBlocks * sizeof(float));
    L.total = L.weights + align256(3 * (2 * kMaxRadius + 1) * sizeof(float));
    return L;
}

}  // namespace

extern "C" size_t sss_crop_downscale_workspace_size(const int crop_dims[3])
{
    if (!crop_dims || crop_dims[0] < 1 || crop_dims[1] < 1 || crop_dims[2] < 1) return 0;
    return prep_layout(crop_dims).total;
}

extern "C" int sss_crop_downscale(const float* image, const int image_dims[3], const int crop_start[3],
                                  const int crop_before[3], const int crop_dims[3], const int out_dims[3],
                                  const double sigma[3], int clip, float zero_below, float* out, void* workspace,
                                  size_t workspace_bytes, void* stream)
{
    if (!image || !image_dims || !crop_start || !crop_before || !crop_dims || !out_dims || !sigma || !out)
        return sss_set_error(SSS_ERR_INVALID, "sss_crop_downscale: null argument");
    for (int d = 0; d < 3; ++d) {
        if (image_dims[d] < 1 || crop_dims[d] < 1 || out_dims[d] < 1)
            return sss_set_error(SSS_ERR_INVALID, "sss_crop_downscale: empty dimension %d", d);
        if (!(sigma[d] >= 0.0) || sigma[d] > 100.0)
            return sss_set_error(SSS_ERR_INVALID, "sss_crop_downscale: sigma[%d] = %g outside [0, 100]", d, sigma[d]);
        if ((long long)crop_dims[d] + 2 * kPad > (1ll << 30))
            return sss_set_error(SSS_ERR_INVALID, "sss_crop_downscale: crop dimension %d too large", d);
    }
    const PrepLayout L = prep_layout(crop_dims);
    if (!workspace || workspace_bytes < L.total)
        return sss_set_error(SSS_ERR_WORKSPACE, "sss_crop_downscale: workspace of %zu bytes, %zu needed",
                             workspace_bytes, L.total);
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char* ws = (unsigned char*)workspace;
    float* crop = (float*)(ws + L.crop);
    float* tmp = (float*)(ws + L.tmp);
    float* padded = (float*)(ws + L.padded);
    float* part = (float*)(ws + L.part);
    float* wdev = (float*)(ws + L.weights);

    const Dims din = {{image_dims[0], image_dims[1], image_dims[2]}};
    const Dims dc = {{crop_dims[0], crop_dims[1], crop_dims[2]}};
    const Dims dp = {{crop_dims[0] + 2 * kPad, crop_dims[1] + 2 * kPad, crop_dims[2] + 2 * kPad}};
    const Dims dout = {{out_dims[0], out_dims[1], out_dims[2]}};

    // Gaussian weights (FP64, normalised, then rounded to FP32) for every axis filtered
    float hw[3][2 * kMaxRadius + 1];
    int radius[3];
    for (int d = 0; d < 3; ++d) {
        radius[d] = -1;
        if (sigma[d] <= 1e-15) continue;  // axes with a zero sigma are left unfiltered
        const int r = (int)(4.0 * sigma[d] + 0.5);
        if (r > kMaxRadius) return sss_set_error(SSS_ERR_INVALID, "sss_crop_downscale: kernel radius %d", r);
        double sum = 0.0, tmpw[2 * kMaxRadius + 1];
        for (int k = -r; k <= r; ++k) sum += (tmpw[k + r] = exp(-0.5 / (sigma[d] * sigma[d]) * k * k));
        for (int k = 0; k <= 2 * r; ++k) hw[d][k] = (float)(tmpw[k] / sum);
        radius[d] = r;
    }
    for (int d = 0; d < 3; ++d)
        if (radius[d] >= 0 &&
            cudaMemcpyAsync(wdev + d * (2 * kMaxRadius + 1), hw[d], (2 * radius[d] + 1) * sizeof(float),
                            cudaMemcpyHostToDevice, st) != cudaSuccess)
            return sss_set_error(SSS_ERR_CUDA, "sss_crop_downscale: weight upload failed");

    const long long nc = dc.count();
    crop_kernel<<<grid_for(nc), 256, 0, st>>>(image, din, crop, dc,
                                              make_int3(crop_start[0], crop_start[1], crop_start[2]),
                                              make_int3(crop_before[0], crop_before[1], crop_before[2]));
    const int nb = (int)(nc / 256 + 1 < kMinmaxBlocks ? nc / 256 + 1 : kMinmaxBlocks);
    minmax_partial_kernel<<<nb, 256, 0, st>>>(crop, nc, part);
    minmax_final_kernel<<<1, 256, 0, st>>>(part, nb);
    // Gaussian per axis, ping-pong between crop and tmp (the cropped input is kept for nothing else)
    float* cur = crop;
    float* other = tmp;
    for (int d = 0; d < 3; ++d) {
        if (radius[d] < 0) continue;
        if (nc < (1ll << 31))
            gauss_axis_kernel<unsigned><<<grid_for(nc), 256, 0, st>>>(cur, other, dc, d,
                                                                      wdev + d * (2 * kMaxRadius + 1), radius[d]);
        else
            gauss_axis_kernel<long long><<<grid_for(nc), 256, 0, st>>>(cur, other, dc, d,
                                                                       wdev + d * (2 * kMaxRadius + 1), radius[d]);
        float* t = cur;
        cur = other;
        other = t;
    }
    const long long np = dp.count();
    pad_edge_kernel<<<grid_for(np), 256, 0, st>>>(cur, dc, padded, dp);
    for (int d = 0; d < 3; ++d) {
        const long long lines = np / dp.n[d];
        spline_axis_kernel<<<grid_for(lines, 128), 128, 0, st>>>(padded, dp, d);
    }
    zoom_kernel<<<grid_for(dout.count()), 256, 0, st>>>(padded, dp, dc, out, dout, part, clip, zero_below);
    return sss_check_launch("sss_crop_downscale");
}
